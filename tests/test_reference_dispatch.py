"""SLIME_DISPATCH_REFERENCE: the reference's own agent dispatch.

The reference dispatches ceil(n / 64) workgroups of 64 as wx x wy with
wx = min(ceil(n / 64), 65535) (src/main.rs:1174-1178), and invocation
(gx, gy) updates agent gx + 65535 gy (compute.wgsl:60).  Above 4,194,240
agents the highest agents are never visited and some are visited several
times.  The tests check the closed-form visit count against an enumeration
of the dispatch grid, the oracle's pass in this mode, and (where the
reference's source tree is present) the oracle against the translated
shader run over that very grid.
"""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from wgsl import wgslref

SIZES = [1, 63, 64, 65, 65536, 4194240, 4194241, 4264240, 5000000, 16777216]


def enumerate_visits(n):
    groups = -(-n // 64)
    wx = min(groups, 65535)
    wy = -(-groups // wx)
    visits = np.zeros(n, np.uint32)
    for gy in range(wy):
        idx = np.arange(64 * wx, dtype=np.int64) + gy * 65535
        idx = idx[idx < n]
        visits[idx] += 1  # indices within one row of the grid are distinct
    return visits


@pytest.mark.parametrize("n", SIZES)
def test_visit_count_matches_the_dispatch_grid(n):
    want = enumerate_visits(n)
    got = oracle.dispatch_visits(n, np.arange(n, dtype=np.uint64))
    assert np.array_equal(got, want)
    assert oracle.dispatch_visits(n, [n, n + 5, 2**40]).tolist() == [0, 0, 0]


def test_visit_count_at_the_headline_size():
    """16,777,216 agents (4096^2 at one agent per cell): 12,320,836 are never
    updated; the first 65,535 once, agents 65,535 .. 4,194,239 up to 5 times."""
    v = oracle.dispatch_visits(16777216, np.arange(16777216, dtype=np.uint64))
    assert int((v == 0).sum()) == 12320836
    assert int(np.flatnonzero(v)[-1]) == 4 * 65535 + 64 * 65535 - 1
    assert v.max() == 5 and v[:65535].max() == 1


def test_reference_dispatch_is_every_agent_below_4194241():
    W, H, n = 128, 96, 65536
    trail = np.random.default_rng(1).random((H, W), dtype=np.float32)
    a0 = agents_uniform(n, W, H, 30.0, 50.0, seed=2)
    outs = []
    for mode in (0, 1):
        p = config0_params(W, H, dispatch_mode=mode)
        a = a0.copy()
        c = oracle.agents_pass(p, W, H, a, trail)
        outs.append((a, c))
    assert np.array_equal(outs[0][0].view(np.uint32), outs[1][0].view(np.uint32))
    assert np.array_equal(outs[0][1], outs[1][1])


def test_oracle_pass_in_reference_dispatch():
    """Unvisited agents keep their state bit for bit (speed unclamped); a
    visited agent moves as in the every-agent pass and deposits once per
    visit."""
    W, H, n = 64, 48, 4264240
    trail = np.random.default_rng(3).random((H, W), dtype=np.float32)
    a0 = agents_uniform(n, W, H, 0.5, 80.0, seed=4)  # speeds outside 30..50 show the clamp
    p_ref = config0_params(W, H, dispatch_mode=1, agent_speed_min=30.0, agent_speed_max=50.0)
    p_all = config0_params(W, H, dispatch_mode=0, agent_speed_min=30.0, agent_speed_max=50.0)
    a_ref, a_all = a0.copy(), a0.copy()
    c_ref = oracle.agents_pass(p_ref, W, H, a_ref, trail)
    oracle.agents_pass(p_all, W, H, a_all, trail)
    v = oracle.dispatch_visits(n, np.arange(n, dtype=np.uint64))
    frozen = v == 0
    assert int(frozen.sum()) == 4465
    assert np.array_equal(a_ref[frozen].view(np.uint32), a0[frozen].view(np.uint32))
    assert np.array_equal(a_ref[~frozen].view(np.uint32), a_all[~frozen].view(np.uint32))
    # deposits: each visited agent's cell gets its visit count
    cells = a_all[~frozen, 1].astype(np.int64) * W + a_all[~frozen, 0].astype(np.int64)
    want = np.bincount(cells, weights=v[~frozen], minlength=W * H).astype(np.uint32)
    assert np.array_equal(c_ref.reshape(-1), want)


@pytest.mark.skipif(not wgslref.available(), reason="the reference's source tree is not present")
@pytest.mark.parametrize("n", [70000, 4264240])
def test_reference_dispatch_matches_the_shader_over_its_dispatch_grid(n):
    """The translated shader run invocation by invocation over the reference's
    wx x wy grid, agents and trail read as the pass found them: at sensor
    angle 0 and deposition 1.0 (every deposit leaves its cell at 1) the
    oracle's pass in this mode, then decay and diffuse, is the reference's
    frame bit for bit, frozen agents included; two frames."""
    W, H = 64, 48
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, diffusion_rate=1.0,
                       agent_sensor_angle=0.0, pheromone_deposition_amount=1.0, dispatch_mode=1,
                       agent_speed_min=30.0, agent_speed_max=50.0)
    a0 = agents_uniform(n, W, H, 0.5, 80.0, seed=5)
    t0 = np.random.default_rng(6).random((H, W), dtype=np.float32)
    ref_a, ref_t = a0, t0
    for _ in range(2):
        ref_a, ref_t = wgslref.agents_pass_dispatch(p, ref_a, ref_t)
        ref_t = wgslref.diffuse(p, wgslref.decay(p, ref_t))
    got_a, got_t = a0.copy(), t0.copy()
    oracle.run(p, W, H, got_a, got_t, 2)
    assert np.array_equal(got_a.view(np.uint32), ref_a.view(np.uint32))
    assert np.array_equal(got_t.view(np.uint32), ref_t.view(np.uint32))
    if n > 4194240:
        frozen = oracle.dispatch_visits(n, np.arange(n, dtype=np.uint64)) == 0
        assert np.array_equal(ref_a[frozen].view(np.uint32), a0[frozen].view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("reorder,marks", [(0, False), (1, True)])
def test_gpu_reference_dispatch_at_4096(gpu, reorder, marks):
    """16,777,216 agents on 4096^2 in the reference's dispatch: the library
    against the oracle, bit for bit, two steps; with Morton reordering (the
    visit count follows the agent's original index) and with deposit marks
    (visits beyond the first change nothing once a deposit saturates)."""
    from test_parity_gpu import assert_bitexact, make_sim
    W, H, n = 4096, 4096, 16_777_216
    p = config0_params(W, H, decay_mode=1, blur_mode=1, agent_speed_min=1.0, agent_speed_max=2.0,
                       dispatch_mode=1)
    agents = agents_uniform(n, W, H, 0.5, 3.0, seed=21)
    trail = np.random.default_rng(22).random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p, agents, trail)
    sim.set_options(reorder_every=reorder, exact_counts=0 if marks else 1, trail_tile=8)
    ca, ct = agents.copy(), trail.copy()
    for step in range(2):
        sim.step(1)
        counts = oracle.run(p, W, H, ca, ct, 1, record_counts=True)
        if not marks:
            assert_bitexact(sim.download_deposit_counts(), counts[0], f"counts step {step}")
        assert_bitexact(sim.download_agents(), ca, f"agents step {step}")
        assert_bitexact(sim.download_trail(), ct, f"trail step {step}")
    sim.close()
    frozen = oracle.dispatch_visits(n, np.arange(n, dtype=np.uint64)) == 0
    assert int(frozen.sum()) == 12320836
    assert np.array_equal(ca[frozen].view(np.uint32), agents[frozen].view(np.uint32))


@pytest.mark.gpu
def test_gpu_reference_dispatch_small_is_every_agent(gpu):
    from test_parity_gpu import assert_bitexact, make_sim
    W, H, n = 512, 512, 65536
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=23)
    out = []
    for mode in (0, 1):
        sim = make_sim(W, H, n, config0_params(W, H, dispatch_mode=mode), agents)
        sim.step(5)
        out.append((sim.download_agents(), sim.download_trail()))
        sim.close()
    assert_bitexact(out[1][0], out[0][0], "agents")
    assert_bitexact(out[1][1], out[0][1], "trail")


@pytest.mark.gpu
def test_gpu_rejects_unknown_dispatch_and_ensemble_reference_dispatch(gpu):
    import slime_gb300 as sg
    with pytest.raises(sg.SlimeError):
        sg.Simulation(64, 64, 10, config0_params(64, 64, dispatch_mode=2))
    with pytest.raises(sg.SlimeError):
        sg.Ensemble([64], [64], [10], [config0_params(64, 64, dispatch_mode=1)])


@pytest.mark.gpu
def test_gpu_reference_dispatch_after_reordered_steps(gpu):
    """Morton reordering in the every-agent mode scatters the agent ids over
    the slots; switching to the reference's dispatch (reordering off) must
    first put the agents it updates back in the leading slots.  Then back to
    every agent.  Against the oracle at each switch, exact counts."""
    from test_parity_gpu import assert_bitexact, make_sim
    W, H, n = 256, 192, 4_264_240
    p_each = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, pheromone_deposition_amount=0.3,
                            agent_speed_min=30.0, agent_speed_max=50.0)
    p_ref = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, pheromone_deposition_amount=0.3,
                           agent_speed_min=30.0, agent_speed_max=50.0, dispatch_mode=1)
    agents = agents_uniform(n, W, H, 0.5, 80.0, seed=31)
    trail = np.random.default_rng(32).random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p_each, agents, trail)
    sim.set_options(reorder_every=1, exact_counts=1)
    ca, ct = agents.copy(), trail.copy()
    for p, steps, reorder in ((p_each, 2, 1), (p_ref, 2, 0), (p_each, 1, 0), (p_ref, 1, 1)):
        sim.set_params(p)
        sim.set_options(reorder_every=reorder, exact_counts=1)
        sim.step(steps)
        counts = oracle.run(p, W, H, ca, ct, steps, record_counts=True)
        assert_bitexact(sim.download_deposit_counts(), counts[-1], f"counts mode {p.dispatch_mode}")
        assert_bitexact(sim.download_agents(), ca, f"agents mode {p.dispatch_mode}")
        assert_bitexact(sim.download_trail(), ct, f"trail mode {p.dispatch_mode}")
    sim.close()
