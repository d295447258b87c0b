"""The checkpointed GPU adjoint of the deposit -> decay -> diffuse chain
against the binary64 oracle adjoint and binary64 central finite differences
on the frozen-trajectory forward (the deposit counts of every step are taken
from the oracle's bit-identical replay of the same agents)."""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from test_oracle import fd4

pytestmark = pytest.mark.gpu

# Parameter gradients: within 1e-6 relative of the binary64 references (the
# target for this adjoint; measured up to 5.3e-7).  A reference of exactly 0
# (a deposition on the clamp kink) must come out 0.
REL = 1e-6


def assert_rel(got, ref, what, tol=REL):
    if ref == 0.0:
        assert got == 0.0, (what, got, ref)
    else:
        assert abs(got - ref) <= tol * abs(ref), (what, got, ref, abs(got - ref) / abs(ref))


def run_case(W, H, n, steps, K, dm, bm, dep, seed=0, radius=1.0, t_lo=0.0, decay=None):
    import slime_gb300 as sg
    p = config0_params(W, H, decay_mode=dm, blur_mode=bm, pheromone_deposition_amount=dep,
                       decay_factor=decay if decay is not None else (0.97 if dm else 10.0), agent_speed_min=30.0,
                       agent_speed_max=50.0, blur_radius=radius)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=seed)
    rng = np.random.default_rng(seed + 1)
    t0 = (t_lo + rng.random((H, W)) * (0.5 - t_lo)).astype(np.float32)
    target = rng.random((H, W)).astype(np.float32)
    with sg.Simulation(W, H, n, p) as sim:
        sim.upload_agents(agents)
        sim.upload_trail(t0)
        sim.forward_record(steps, K)
        tn = sim.download_trail()
        g = tn - target
        grads, d0 = sim.backward(g)
        # the live state is untouched by the backward
        assert np.array_equal(sim.download_trail(), tn)
    a, t = agents.copy(), t0.copy()
    counts = oracle.run(p, W, H, a, t, steps, record_counts=True)
    assert np.array_equal(t, tn), "forward differs from the oracle"
    theta = [float(np.float32(p.decay_factor)), float(np.float32(p.diffusion_rate)),
             float(np.float32(p.pheromone_deposition_amount))]
    loss, ref, d0_ref = oracle.chain_adjoint_f64(p, W, H, *theta, t0, counts, g_final=g.astype(np.float64))
    return p, t0, counts, theta, grads, d0, ref, d0_ref, g


@pytest.mark.parametrize("dm,bm,dep", [(1, 1, 0.3), (0, 0, 0.3), (1, 0, 0.05), (0, 1, 1.0)])
def test_adjoint_matches_binary64_adjoint(gpu, dm, bm, dep):
    W, H = 96, 80
    p, t0, counts, theta, grads, d0, ref, d0_ref, g = run_case(W, H, 2000, 37, 10, dm, bm, dep)
    got = [grads.d_decay_factor, grads.d_diffusion_rate, grads.d_deposition_amount]
    for i in range(3):
        assert_rel(got[i], ref[i], f"parameter {i}")
    # the initial-trail gradient, relative to its largest entry
    assert np.abs(d0 - d0_ref).max() <= REL * np.abs(d0_ref).max()


def test_adjoint_matches_finite_differences(gpu):
    W, H = 64, 64
    # off the kinks: small deposition, trail away from 0 and 1
    p, t0, counts, theta, grads, d0, ref, d0_ref, g = run_case(W, H, 1500, 25, 7, 1, 1, 0.02, seed=3, t_lo=0.1)
    assert counts.max() * 0.02 + 0.5 < 1.0
    target = None
    # loss L = <g_fixed, T_n>: linear in T_n, so its FD needs no target
    got = [grads.d_decay_factor, grads.d_diffusion_rate, grads.d_deposition_amount]
    h = 1e-4
    gf = g.astype(np.float64)

    def lin_loss(th):
        _, fin = oracle.chain_loss_f64(p, W, H, *th, t0, counts, np.zeros((H, W)))
        return (fin * gf).sum()

    for i in range(3):
        fd = fd4(lin_loss, theta, i, h)
        assert_rel(got[i], fd, f"parameter {i} vs finite differences")
    assert target is None


def test_adjoint_at_the_1024_configuration_size(gpu):
    """The adjoint at the size of the 1024^2 gradient configuration:
    1,048,576 agents on a 1024x1024 trail, 200 steps recorded with
    checkpoints every 50 (four segments replayed), multiplicative decay and
    the 3-tap Gaussian, off the clamp kinks (deposition 2e-4, decay 0.95,
    trail in [0.1, 0.5]: the agents gather into networks with up to ~350 of
    them on a cell, yet no fold input comes near the clamp at 1), loss
    L = 0.5 ||T_200 - target||^2.

    Two references, two tolerances:
      * the binary64 adjoint run along the binary32 trajectory the GPU ran
        (its trails replayed bit for bit by the oracle): the backward's own
        arithmetic, within 1e-6 relative (measured 2.5e-7 for the rate);
      * the binary64 adjoint of the binary64 forward, and binary64
        fourth-order central differences (h = 1e-4) of the frozen-trajectory
        forward: within 2e-6 relative.  Over 200 steps the binary32 forward
        itself departs from the binary64 one enough to move the gradients by
        up to 8.8e-7 relative (the rate's B(u) - u is a small difference of
        nearly equal trails); with the backward's share the GPU measured
        1.13e-6 there.
    The initial-trail gradient: within 1e-6 of its largest entry against
    the first reference."""
    import slime_gb300 as sg
    W = H = 1024
    n, steps, K, dep = 1_048_576, 200, 50, 2e-4
    p = config0_params(W, H, decay_mode=1, blur_mode=1, pheromone_deposition_amount=dep, decay_factor=0.95,
                       agent_speed_min=30.0, agent_speed_max=50.0)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=11)
    rng = np.random.default_rng(12)
    t0 = (0.1 + rng.random((H, W)) * 0.4).astype(np.float32)
    target = rng.random((H, W)).astype(np.float32)
    with sg.Simulation(W, H, n, p) as sim:
        sim.upload_agents(agents)
        sim.upload_trail(t0)
        sim.forward_record(steps, K)
        tn = sim.download_trail()
        g = tn - target
        grads, d0 = sim.backward(g)
    # the oracle's replay of the same binary32 forward, step by step
    a, t = agents.copy(), t0.copy()
    trails = np.empty((steps + 1, H, W), np.float32)
    counts = np.empty((steps, H, W), np.uint32)
    trails[0] = t
    for s in range(steps):
        counts[s] = oracle.agents_pass(p, W, H, a, t)
        t = oracle.trail_pass(p, W, H, t, counts[s])
        trails[s + 1] = t
    assert np.array_equal(t, tn), "forward differs from the oracle"
    theta = [float(np.float32(0.95)), float(np.float32(p.diffusion_rate)), float(np.float32(dep))]
    # every fold input t + dep k stays below 0.9: the differences (which move
    # the trail by a few per cent) see no kink
    assert float((trails[:-1] + np.float32(dep) * counts).max()) < 0.9
    got = [grads.d_decay_factor, grads.d_diffusion_rate, grads.d_deposition_amount]
    gf = g.astype(np.float64)
    along, d0_along = oracle.chain_adjoint_f64_along(p, W, H, *theta, trails, counts, gf)
    for i in range(3):
        assert_rel(got[i], along[i], f"parameter {i} vs the binary64 adjoint along the binary32 forward")
    assert np.abs(d0 - d0_along).max() <= REL * np.abs(d0_along).max()
    del trails
    _, ref, _ = oracle.chain_adjoint_f64(p, W, H, *theta, t0, counts, g_final=gf)

    def lin_loss(th):
        # <g, T_n> has the same gradient as the loss at the forward the GPU ran
        _, fin = oracle.chain_loss_f64(p, W, H, *th, t0, counts, np.zeros((H, W)))
        return (fin * gf).sum()

    for i in range(3):
        assert_rel(got[i], ref[i], f"parameter {i} vs the binary64 adjoint", tol=2 * REL)
        assert_rel(got[i], fd4(lin_loss, theta, i, 1e-4), f"parameter {i} vs finite differences", tol=2 * REL)


def test_adjoint_radius2_and_ragged_segments(gpu):
    W, H = 70, 45
    p, t0, counts, theta, grads, d0, ref, d0_ref, g = run_case(W, H, 900, 23, 5, 1, 1, 0.2, seed=5, radius=2.0)
    got = [grads.d_decay_factor, grads.d_diffusion_rate, grads.d_deposition_amount]
    for i in range(3):
        assert_rel(got[i], ref[i], f"parameter {i} (radius 2)")


def test_backward_without_record_is_an_error(gpu):
    import slime_gb300 as sg
    with sg.Simulation(16, 16, 8) as sim:
        with pytest.raises(sg.SlimeError) as e:
            sim.backward(np.zeros((16, 16), np.float32))
        assert e.value.status == -4


def test_autograd_function_role(gpu):
    """TrailChain wires the C ABI backward into torch.autograd."""
    import torch
    import slime_gb300 as sg
    from slime_gb300.autograd import trail_chain
    W, H, n, steps = 64, 48, 1200, 20
    p = config0_params(W, H, pheromone_deposition_amount=0.05, agent_speed_min=30.0, agent_speed_max=50.0)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=8)
    rng = np.random.default_rng(8)
    t0 = torch.tensor((0.2 + 0.3 * rng.random((H, W))).astype(np.float32), requires_grad=True)
    target = torch.tensor(rng.random((H, W)).astype(np.float32))
    decay = torch.tensor(0.97, dtype=torch.float64, requires_grad=True)
    rate = torch.tensor(0.5, dtype=torch.float64, requires_grad=True)
    dep = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    with sg.Simulation(W, H, n, p) as sim:
        out = trail_chain(t0, decay, rate, dep, sim, steps, 6, agents)
        loss = 0.5 * ((out - target) ** 2).sum()
        loss.backward()
    counts = oracle.run(p, W, H, agents.copy(), t0.detach().numpy().copy(), steps, record_counts=True)
    theta = [float(np.float32(0.97)), float(np.float32(0.5)), float(np.float32(0.05))]
    # dL/dT_n of the loss at the binary32 forward the GPU ran (the adjoint's
    # input), carried back by the binary64 adjoint
    g_final = (out.detach() - target).numpy().astype(np.float64)
    _, ref, d0_ref = oracle.chain_adjoint_f64(p, W, H, *theta, t0.detach().numpy(), counts, g_final=g_final)
    for i, (got, want) in enumerate(zip((decay.grad, rate.grad, dep.grad), ref)):
        assert_rel(float(got), want, f"parameter {i}")
    assert np.abs(t0.grad.numpy() - d0_ref).max() <= REL * np.abs(d0_ref).max()
