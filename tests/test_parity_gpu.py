"""Parity of the CUDA step (through the C ABI) with the CPU oracle.

Integer and index work (deposit cells, counts, floor/wrap) and, because the
shared builtins are evaluated identically on both sides, every binary32 value
of the agent state and the trail are compared bit for bit.  Sizes are the
512x512 reference-size configuration and small edge cases the oracle finishes
in seconds; the full-size configurations are covered by property tests in
test_properties_gpu.py.
"""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def assert_bitexact(gpu_arr, cpu_arr, what):
    """Bit-for-bit equality; two NaNs match whatever their payloads (the GPU
    produces the canonical NaN, a CPU propagates the operand's payload)."""
    g, c = bits(gpu_arr).reshape(-1), bits(cpu_arr).reshape(-1)
    both_nan = np.isnan(np.asarray(gpu_arr, np.float32).reshape(-1)) & np.isnan(np.asarray(cpu_arr, np.float32).reshape(-1))
    bad = np.flatnonzero((g != c) & ~both_nan)
    assert bad.size == 0, (f"{what}: {bad.size} mismatches, first at {bad[:5]}: "
                           f"gpu={np.asarray(gpu_arr).reshape(-1)[bad[:5]]} cpu={np.asarray(cpu_arr).reshape(-1)[bad[:5]]}")


def make_sim(W, H, n, params, agents, trail=None):
    import slime_gb300 as sg
    sim = sg.Simulation(W, H, n, params)
    sim.upload_agents(agents)
    if trail is not None:
        sim.upload_trail(trail)
    return sim


@pytest.mark.parametrize("decay_mode,blur_mode", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_one_step_bitexact_random_trail(gpu, decay_mode, blur_mode):
    W = H = 512
    n = 65536
    p = config0_params(W, H, decay_mode=decay_mode, blur_mode=blur_mode, agent_speed_min=30.0,
                       agent_speed_max=50.0)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=1)
    trail = np.random.default_rng(2).random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p, agents, trail)
    sim.set_options(exact_counts=1)
    sim.step(1)
    ga, gt, gc = sim.download_agents(), sim.download_trail(), sim.download_deposit_counts()
    ca = agents.copy()
    cc = oracle.agents_pass(p, W, H, ca, trail)
    ct = oracle.trail_pass(p, W, H, trail, cc)
    assert np.array_equal(gc, cc), "deposit counts differ"
    assert_bitexact(ga, ca, "agents")
    assert_bitexact(gt, ct, "trail")
    # the random trail makes every turn branch occur
    turned = np.abs(ga[:, 2] - np.mod(agents[:, 2], np.float32(2 * np.pi)))
    assert (turned > 0.1).mean() > 0.3


def test_config0_100_steps_every_step_bitexact(gpu):
    """The 512x512 / 65,536-agent configuration from a zero trail, 100 steps,
    agent state and trail compared after every step."""
    W = H = 512
    n = 65536
    p = config0_params(W, H)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=0)
    trail = np.zeros((H, W), np.float32)
    sim = make_sim(W, H, n, p, agents)
    ca, ct = agents.copy(), trail.copy()
    for s in range(100):
        sim.step(1)
        oracle.run(p, W, H, ca, ct, 1)
        if s % 10 == 9 or s < 3:
            assert_bitexact(sim.download_agents(), ca, f"agents after step {s + 1}")
            assert_bitexact(sim.download_trail(), ct, f"trail after step {s + 1}")
    assert_bitexact(sim.download_agents(), ca, "agents after 100 steps")
    assert_bitexact(sim.download_trail(), ct, "trail after 100 steps")
    assert ct.sum() > 0


def test_graph_chunks_match_single_steps(gpu):
    W, H, n = 300, 200, 20000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, agent_speed_min=30.0,
                       agent_speed_max=50.0, agent_jitter=0.3)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=3)
    a = make_sim(W, H, n, p, agents)
    b = make_sim(W, H, n, p, agents)
    a.set_options(use_graphs=1, graph_chunk=7)
    b.set_options(use_graphs=0)
    a.step(23)
    for _ in range(23):
        b.step(1)
    assert_bitexact(a.download_agents(), b.download_agents(), "agents")
    assert_bitexact(a.download_trail(), b.download_trail(), "trail")
    ca, ct = agents.copy(), np.zeros((H, W), np.float32)
    oracle.run(p, W, H, ca, ct, 23)
    assert_bitexact(a.download_agents(), ca, "agents vs oracle")
    assert_bitexact(a.download_trail(), ct, "trail vs oracle")
    assert a.info().steps_done == 23


def test_prepare_steps_captures_without_stepping(gpu):
    """slime_prepare_steps captures the chunk graphs (graph_chunk 7, a reorder
    every 10 steps cutting chunks) without stepping; the steps after it replay
    them with the same result as an unprepared run."""
    W, H, n = 256, 96, 9000
    p = config0_params(W, H, agent_speed_min=20.0, agent_speed_max=40.0, agent_jitter=0.2)
    agents = agents_uniform(n, W, H, 20.0, 40.0, seed=5)
    a = make_sim(W, H, n, p, agents)
    b = make_sim(W, H, n, p, agents)
    for s in (a, b):
        s.set_options(use_graphs=1, graph_chunk=7, reorder_every=10)
    a.step(3)
    b.step(3)
    t0, g0 = a.download_trail(), a.download_agents()
    a.prepare_steps(31)
    assert a.info().steps_done == 3
    assert_bitexact(a.download_trail(), t0, "trail after prepare")
    assert_bitexact(a.download_agents(), g0, "agents after prepare")
    a.step(31)
    b.step(31)
    assert_bitexact(a.download_agents(), b.download_agents(), "agents")
    assert_bitexact(a.download_trail(), b.download_trail(), "trail")
    assert a.info().steps_done == 34


@pytest.mark.parametrize("tile", range(1, 12))
@pytest.mark.parametrize("W,H", [(333, 77), (336, 77), (256, 40), (8, 9)])
def test_every_trail_tile_is_bitexact(gpu, tile, W, H):
    # sizes ragged against every tile shape; the streaming tiles need W % 4 == 0,
    # the tensor-copy tile (11) W % 16 == 0 and has interior tiles at 336 x 77
    n = 5000
    for blur_mode, radius in ((0, 1.0), (1, 1.0), (1, 2.0), (1, 3.0)):
        p = config0_params(W, H, decay_mode=1, blur_mode=blur_mode, blur_radius=radius, blur_sigma=1.5)
        agents = agents_uniform(n, W, H, 1.0, 2.0, seed=4)
        trail = np.random.default_rng(5).random((H, W), dtype=np.float32)
        sim = make_sim(W, H, n, p, agents, trail)
        sim.set_options(trail_tile=tile)
        sim.step(2)
        ca, ct = agents.copy(), trail.copy()
        oracle.run(p, W, H, ca, ct, 2)
        assert_bitexact(sim.download_trail(), ct, f"trail tile {tile} blur {blur_mode} r {radius}")
        assert_bitexact(sim.download_agents(), ca, "agents")


@pytest.mark.parametrize("sensor_mode", [0, 1])
@pytest.mark.parametrize("shape", range(1, 17))
@pytest.mark.parametrize("W,H", [(256, 150), (201, 150)])
def test_every_agent_shape_is_bitexact(gpu, shape, W, H, sensor_mode):
    # 256 wide: the trail has gather textures; 201 wide: its rows are not
    # aligned for one, and the texture shapes (13..15) run their pointer
    # twins.  The largest case runs Morton-reordered (slot -> id map).
    sim0 = make_sim(W, H, 1, config0_params(W, H), agents_uniform(1, W, H, 1.0, 2.0, seed=0),
                    np.zeros((H, W), np.float32))
    assert sim0.info().trail_texture == (1 if W == 256 else 0)
    for n in (1, 3, 4097, 20001):
        p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, agent_speed_min=30.0,
                           agent_speed_max=50.0, agent_jitter=0.3, sensor_mode=sensor_mode)
        agents = agents_uniform(n, W, H, 30.0, 50.0, seed=n)
        trail = np.random.default_rng(n).random((H, W), dtype=np.float32)
        sim = make_sim(W, H, n, p, agents, trail)
        sim.set_options(agent_shape=shape, reorder_every=1 if n == 20001 else 0)
        assert sim.info().agent_shape == shape - 1
        sim.step(3)
        ca, ct = agents.copy(), trail.copy()
        oracle.run(p, W, H, ca, ct, 3)
        assert_bitexact(sim.download_agents(), ca, f"agents shape {shape} n {n} sensor mode {sensor_mode}")
        assert_bitexact(sim.download_trail(), ct, f"trail shape {shape} n {n} sensor mode {sensor_mode}")


def test_autotune_keeps_state(gpu):
    W, H, n = 512, 256, 40000
    p = config0_params(W, H)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=21)
    trail = np.random.default_rng(21).random((H, W), dtype=np.float32)
    a = make_sim(W, H, n, p, agents, trail)
    a.autotune(2)
    a.step(5)
    ca, ct = agents.copy(), trail.copy()
    oracle.run(p, W, H, ca, ct, 5)
    assert_bitexact(a.download_agents(), ca, "agents after autotune")
    assert_bitexact(a.download_trail(), ct, "trail after autotune")


@pytest.mark.parametrize("shape", [0, 14])
@pytest.mark.parametrize("W,H", [(1, 1), (2, 3), (3, 2), (5, 3), (4, 4), (17, 1), (1, 19), (8, 2), (16, 3)])
def test_tiny_toroidal_grids(gpu, W, H, shape):
    n = 64
    for blur_mode, radius in ((0, 1.0), (1, 2.0)):
        p = config0_params(W, H, decay_mode=0, blur_mode=blur_mode, blur_radius=radius,
                           decay_factor=5.0, agent_sensor_distance=1.5, agent_speed_min=30.0, agent_speed_max=90.0,
                           pheromone_deposition_amount=0.3)
        agents = agents_uniform(n, W, H, 30.0, 90.0, seed=6)
        trail = np.random.default_rng(7).random((H, W), dtype=np.float32)
        sim = make_sim(W, H, n, p, agents, trail)
        sim.set_options(agent_shape=shape)
        sim.step(3)
        ca, ct = agents.copy(), trail.copy()
        oracle.run(p, W, H, ca, ct, 3)
        assert_bitexact(sim.download_agents(), ca, f"agents {W}x{H}")
        assert_bitexact(sim.download_trail(), ct, f"trail {W}x{H}")


@pytest.mark.parametrize("shape", [0, 14])
def test_edge_positions_and_sensor_bounds(gpu, shape):
    """Agents on the last row/column, at x rounding up to W after the wrap,
    sensors off the grid (the sampler returns 0 there, it does not wrap),
    negative and huge angles."""
    W, H = 64, 48
    Wf, Hf = np.float32(W), np.float32(H)
    eps = np.float32(1e-6)
    rows = [
        (Wf - eps, 10.0, 0.0, 1.0), (0.0, 0.0, np.pi, 1.0), (Wf - 1, Hf - 1, 0.3, 1.0),
        (-1e-8, 5.0, np.pi, 1.0), (5.0, -1e-8, 1.5 * np.pi, 1.0), (W - 0.5, H - 0.5, 0.785, 60.0),
        (31.5, 23.5, -7.0, 40.0), (10.0, 10.0, 1e6, 40.0), (10.0, 10.0, -1e7, 40.0), (0.0, 0.0, 0.0, 0.0),
        (Wf - np.float32(2e-6), Hf - np.float32(2e-6), 0.01, 1.0),
        (3.0, 3.0, -0.0, -0.0), (4.0, 4.0, 0.0, -0.0), (5.0, 5.0, np.nan, 40.0), (6.0, np.nan, 1.0, 40.0),
        (np.inf, 7.0, 1.0, 40.0), (8.0, 8.0, 1.0, np.nan),
    ]
    agents = np.array(rows, np.float32)
    n = agents.shape[0]
    trail = np.random.default_rng(8).random((H, W), dtype=np.float32)
    for smin in (0.5, 0.0):
        p = config0_params(W, H, decay_mode=0, blur_mode=0, agent_sensor_distance=20.0, agent_speed_min=smin,
                           agent_speed_max=100.0, agent_jitter=1.0, agent_turn_speed=0.43)
        _edge_case(W, H, agents, trail, p, shape)


def _edge_case(W, H, agents, trail, p, shape=0):
    n = agents.shape[0]
    sim = make_sim(W, H, n, p, agents, trail)
    sim.set_options(agent_shape=shape)
    for s in range(5):
        sim.step(1)
    ca, ct = agents.copy(), trail.copy()
    oracle.run(p, W, H, ca, ct, 5)
    assert_bitexact(sim.download_agents(), ca, "edge agents")
    assert_bitexact(sim.download_trail(), ct, "edge trail")


def test_deposit_fold_many_agents_one_cell(gpu):
    """Thousands of agents landing in one cell in one step: the sequential
    clamp fold is reproduced exactly (small deposition so it does not
    saturate at once)."""
    W, H, n = 32, 32, 4096
    agents = np.zeros((n, 4), np.float32)
    agents[:, 0] = 16.25
    agents[:, 1] = 16.25
    agents[:, 2] = 0.0
    agents[:, 3] = 0.0
    trail = np.zeros((H, W), np.float32)
    for dep in (1.0e-4, 0.37, 3.0, 0.0):
        p = config0_params(W, H, decay_mode=1, blur_mode=0, agent_jitter=0.0, agent_speed_min=0.0,
                           agent_speed_max=0.0, pheromone_deposition_amount=dep, decay_factor=1.0)
        sim = make_sim(W, H, n, p, agents, trail)
        sim.step(1)
        gc = sim.download_deposit_counts()
        assert gc[16, 16] == n and gc.sum() == n
        ca, ct = agents.copy(), trail.copy()
        oracle.run(p, W, H, ca, ct, 1)
        assert_bitexact(sim.download_trail(), ct, f"fold dep={dep}")


def test_zero_agents_and_odd_counts(gpu):
    W, H = 40, 30
    p = config0_params(W, H)
    trail = np.random.default_rng(9).random((H, W), dtype=np.float32)
    for n in (0, 1, 3, 5, 129):
        agents = agents_uniform(n, W, H, 1.0, 2.0, seed=n)
        sim = make_sim(W, H, n, p, agents, trail)
        sim.step(4)
        ca, ct = agents.copy(), trail.copy()
        oracle.run(p, W, H, ca, ct, 4)
        assert_bitexact(sim.download_trail(), ct, f"trail n={n}")
        if n:
            assert_bitexact(sim.download_agents(), ca, f"agents n={n}")


def test_morton_reorder_changes_nothing(gpu):
    W, H, n = 256, 256, 30000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, agent_speed_min=30.0, agent_speed_max=50.0,
                       agent_jitter=0.2)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=10)
    a = make_sim(W, H, n, p, agents)
    b = make_sim(W, H, n, p, agents)
    a.set_options(reorder_every=5, reorder_cell_log2=1)
    a.step(17)
    b.step(17)
    assert a.info().reordered == 1
    assert_bitexact(a.download_agents(), b.download_agents(), "agents (reordered vs not)")
    assert_bitexact(a.download_trail(), b.download_trail(), "trail (reordered vs not)")
    ca, ct = agents.copy(), np.zeros((H, W), np.float32)
    oracle.run(p, W, H, ca, ct, 17)
    assert_bitexact(a.download_agents(), ca, "agents vs oracle")


def test_seed_agents_matches_generator(gpu):
    import slime_gb300 as sg
    W, H, n = 1600, 900, 1000
    sim = sg.Simulation(W, H, n, config0_params(W, H, agent_speed_min=30.0, agent_speed_max=50.0))
    sim.seed_agents(1234, 0.0, 6.28318530718)
    a = sim.download_agents()
    u = [oracle.uniform01(1234, n, f) for f in range(4)]
    x = (u[0] * np.float32(W)).astype(np.float32)
    assert np.array_equal(a[:, 0], np.minimum(x, np.nextafter(np.float32(W), np.float32(0))))
    assert np.array_equal(a[:, 2], np.float32(0.0) + u[2] * np.float32(6.28318530718))
    assert np.array_equal(a[:, 3], np.float32(30.0) + u[3] * np.float32(20.0))
    assert (a[:, 1] < H).all() and (a[:, 1] >= 0).all()


def test_resize_and_clear_follow_reference(gpu):
    """Resize scales x, y by new/old and drops the trail (src/main.rs:954-1015);
    clear zeroes the trail (src/main.rs:909-913)."""
    import slime_gb300 as sg
    W, H, n = 200, 100, 500
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=11)
    sim = make_sim(W, H, n, config0_params(W, H), agents, np.ones((H, W), np.float32))
    sim.resize(300, 50)
    a = sim.download_agents()
    assert np.array_equal(a[:, 0], agents[:, 0] * (np.float32(300) / np.float32(200)))
    assert np.array_equal(a[:, 1], agents[:, 1] * (np.float32(50) / np.float32(100)))
    assert sim.download_trail().shape == (50, 300) and not sim.download_trail().any()
    sim.upload_trail(np.ones((50, 300), np.float32))
    sim.clear_trail()
    assert not sim.download_trail().any()
    p = sim.params()
    assert (p.width, p.height) == (300, 50)
    sim.set_agent_count(77, seed=5)
    assert sim.download_agents().shape == (77, 4)
    with pytest.raises(sg.SlimeError):
        sim.upload_agents(np.zeros((5, 4), np.float32))


def test_nan_parameters_rejected(gpu):
    import slime_gb300 as sg
    sim = sg.Simulation(16, 16, 4)
    p = config0_params(16, 16)
    p.diffusion_rate = float("nan")
    with pytest.raises(sg.SlimeError) as e:
        sim.set_params(p)
    assert e.value.status == -1
    p = config0_params(16, 16, blur_mode=1, blur_sigma=0.0)
    with pytest.raises(sg.SlimeError):
        sim.set_params(p)
    p = config0_params(32, 16)
    with pytest.raises(sg.SlimeError):
        sim.set_params(p)
    with pytest.raises(sg.SlimeError) as e:
        sim.seed_agents(1, 0.0, float("inf"))
    assert e.value.status == -1


def test_colorize_matches_display_pass(gpu):
    W, H = 160, 90
    trail = np.random.default_rng(12).random((H, W), dtype=np.float32) * 1.2 - 0.1
    lut = np.random.default_rng(13).integers(0, 256, 768).astype(np.uint8)
    sim = make_sim(W, H, 4, config0_params(W, H), agents_uniform(4, W, H, 1, 2), trail)
    for tw, th in ((160, 90), (200, 90), (160, 200), (37, 11)):
        assert np.array_equal(sim.colorize(lut, tw, th), oracle.colorize(W, H, trail, lut, tw, th)), (tw, th)


def test_colorize_async_frames(gpu):
    """slime_colorize_async between steps, as a frame loop calls it: each
    frame is the oracle's colourise of the trail of its step, across a LUT
    change, a new image size, and page-locked as well as pageable images."""
    import torch
    W, H, n = 300, 170, 20000
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=41)
    sim = make_sim(W, H, n, config0_params(W, H), agents)
    rng = np.random.default_rng(42)
    luts = [rng.integers(0, 256, 768, dtype=np.uint8) for _ in range(2)]
    for frame, (tw, th, lut, pinned) in enumerate([(160, 90, luts[0], True), (160, 90, luts[0], True),
                                                   (160, 90, luts[1], False), (90, 160, luts[1], True)]):
        sim.step(3)
        trail = sim.download_trail()
        if pinned:
            out = torch.empty((th, tw, 4), dtype=torch.uint8, pin_memory=True).numpy()
        else:
            out = np.empty((th, tw, 4), np.uint8)
        sim.colorize_async(lut, out)
        sim.step(2)  # steps enqueued after the frame do not change it
        sim.wait_download()
        assert np.array_equal(out, oracle.colorize(W, H, trail, lut, tw, th)), f"frame {frame}"
    sim.close()


def test_async_display_feed_snapshots_the_current_trail(gpu):
    """slime_download_trail_async copies the trail as it was at the call,
    while later steps proceed."""
    import torch
    W, H, n = 256, 128, 20000
    p = config0_params(W, H)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=31)
    sim = make_sim(W, H, n, p, agents, np.random.default_rng(31).random((H, W), dtype=np.float32))
    sim.step(3)
    want = sim.download_trail()
    host = torch.empty((H, W), dtype=torch.float32, pin_memory=True).numpy()
    sim.download_trail_async(host)
    sim.step(5)  # the copy must still deliver the step-3 trail
    sim.wait_download()
    assert_bitexact(host, want, "async snapshot")
    later = sim.download_trail()
    assert not np.array_equal(later, want)
    pageable = np.empty((H, W), np.float32)
    sim.download_trail_async(pageable)
    sim.download_trail_async(host)
    sim.wait_download()
    assert_bitexact(pageable, later, "pageable copy")
    assert_bitexact(host, later, "second pinned copy")


def test_async_display_feed_back_to_back(gpu):
    """Downloads issued one after another with steps in between and no wait,
    as a frame loop does: the two device snapshots are used in turn, and each
    host buffer receives the trail of its own step."""
    import torch
    W, H, n = 256, 128, 20000
    p = config0_params(W, H)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=33)
    trail = np.random.default_rng(34).random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p, agents, trail)
    hosts = [torch.empty((H, W), dtype=torch.float32, pin_memory=True).numpy() for _ in range(5)]
    for h in hosts:
        sim.step(2)
        sim.download_trail_async(h)
    sim.wait_download()
    ca, ct = agents.copy(), trail.copy()
    for k, h in enumerate(hosts):
        oracle.run(p, W, H, ca, ct, 2)
        assert_bitexact(h, ct, f"frame {k}")
    # a resize while a copy is in flight, then downloads at the new size (new snapshots)
    pending = torch.empty((H, W), dtype=torch.float32, pin_memory=True).numpy()
    sim.step(1)
    oracle.run(p, W, H, ca, ct, 1)
    sim.download_trail_async(pending)
    W2 = W + 64
    sim.resize(W2, H)
    sim.wait_download()
    assert_bitexact(pending, ct, "copy in flight across a resize")
    ca[:, 0] = ca[:, 0] * (np.float32(W2) / np.float32(W))  # src/main.rs:987-993
    ct = np.zeros((H, W2), np.float32)
    p2 = config0_params(W2, H)
    hosts2 = [torch.empty((H, W2), dtype=torch.float32, pin_memory=True).numpy() for _ in range(3)]
    for h in hosts2:
        sim.step(1)
        sim.download_trail_async(h)
    sim.wait_download()
    for k, h in enumerate(hosts2):
        oracle.run(p2, W2, H, ca, ct, 1)
        assert_bitexact(h, ct, f"frame {k} after the resize")
    sim.close()


def test_checkpoint_resume_continues_bit_identically(gpu, tmp_path):
    import slime_gb300 as sg
    W, H, n = 200, 120, 15000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, agent_speed_min=30.0,
                       agent_speed_max=50.0, agent_jitter=0.2)
    a = make_sim(W, H, n, p, agents_uniform(n, W, H, 30.0, 50.0, seed=41))
    a.set_options(reorder_every=4)
    a.step(6)
    path = str(tmp_path / "run.slmstate")
    a.save_state(path)
    b = sg.Simulation.load_state(path)
    b.set_options(reorder_every=4)
    # the step counter comes back, so the reorders fall on the same steps
    assert b.info().steps_done == a.info().steps_done == 6
    ra, rb = a.info().reorders_done, b.info().reorders_done
    a.step(5)
    b.step(5)
    assert a.info().reorders_done - ra == b.info().reorders_done - rb == 1  # at step 8
    assert b.info().steps_done == 11
    assert_bitexact(a.download_agents(), b.download_agents(), "agents after resume")
    assert_bitexact(a.download_trail(), b.download_trail(), "trail after resume")
    assert bytes(a.params()) == bytes(b.params())
    # a state of another size or agent count is refused, the context unchanged
    c = make_sim(W, H, n + 1, p, agents_uniform(n + 1, W, H, 30.0, 50.0, seed=42))
    before = c.download_agents()
    with pytest.raises(sg.SlimeError):
        c.restore_state(path)
    assert_bitexact(c.download_agents(), before, "agents after a refused load")
    with open(path, "r+b") as f:
        f.write(b"NOTSTATE")
    with pytest.raises(sg.SlimeError):
        b.restore_state(path)


def seeded_agents(seed, n, W, H, hmin, hmax, smin, smax):
    """slime_seed_agents' draws restated on the host: x ~ U[0,W), y ~ U[0,H),
    angle ~ hmin + U[0,1) (hmax - hmin), speed ~ smin + U[0,1) (smax - smin),
    each U[0,1) the seeded generator's draw for (seed, id, field), binary32."""
    u = [oracle.uniform01(seed, n, f) for f in range(4)]
    a = np.empty((n, 4), np.float32)
    a[:, 0] = np.minimum(u[0] * np.float32(W), np.nextafter(np.float32(W), np.float32(0)))
    a[:, 1] = np.minimum(u[1] * np.float32(H), np.nextafter(np.float32(H), np.float32(0)))
    a[:, 2] = np.float32(hmin) + u[2] * (np.float32(hmax) - np.float32(hmin))
    a[:, 3] = np.float32(smin) + u[3] * (np.float32(smax) - np.float32(smin))
    return a


def test_reassign_speeds_matches_generator(gpu):
    """reassign_agent_speeds (src/main.rs:101-145) on the device: every
    agent's speed is redrawn from the seeded generator (field 3 of its id) in
    [speed_min, speed_max], bit for bit the host restatement; positions and
    headings are untouched, also when the agents sit in Morton order."""
    W, H, n = 300, 200, 20001
    p = config0_params(W, H, agent_speed_min=12.5, agent_speed_max=47.0)
    agents = agents_uniform(n, W, H, 30.0, 50.0, seed=51)
    sim = make_sim(W, H, n, p, agents)
    for reorder in (False, True):
        if reorder:
            sim.reorder_agents()
            assert sim.info().reordered == 1
        sim.reassign_speeds(777 + reorder)
        got = sim.download_agents()
        want = seeded_agents(777 + reorder, n, W, H, 0.0, 1.0, 12.5, 47.0)[:, 3]
        assert_bitexact(got[:, 3], want, f"speeds (reordered={reorder})")
        assert_bitexact(got[:, :3], agents[:, :3], "positions and headings")


def test_set_agent_count_matches_seed_generator(gpu):
    """An agent-count change (src/main.rs:682-791) reseeds every agent: the
    new agents are exactly slime_seed_agents' draws for the seed, with
    headings in [0, 2pi) and the current speed bounds."""
    import slime_gb300 as sg
    W, H = 320, 180
    p = config0_params(W, H, agent_speed_min=30.0, agent_speed_max=50.0)
    sim = make_sim(W, H, 1000, p, agents_uniform(1000, W, H, 30.0, 50.0, seed=52))
    sim.set_options(reorder_every=1)
    sim.step(2)
    for n, seed in ((5000, 9), (777, 10)):
        sim.set_agent_count(n, seed=seed)
        assert sim.info().reordered == 0
        want = seeded_agents(seed, n, W, H, 0.0, 6.28318530718, 30.0, 50.0)
        assert_bitexact(sim.download_agents(), want, f"agents after set_agent_count({n})")
        other = sg.Simulation(W, H, n, p)
        other.seed_agents(seed, 0.0, 6.28318530718)
        assert_bitexact(other.download_agents(), want, "slime_seed_agents")
        other.close()
        sim.step(1)  # the new buffer steps


def test_memory_cap_reports_out_of_memory(gpu):
    """Out-of-memory paths through a capped allocator (SLIME_DEVICE_MEMORY_CAP):
    the failing call returns SLIME_ERR_OUT_OF_MEMORY and nothing leaks into
    later calls.  A resize or an agent-count change that runs out of memory
    leaves the context as it was: same size, same agents, same trail, and
    its next steps match a context that never tried."""
    import os
    import subprocess
    import sys
    from conftest import ROOT
    code = (
        "import sys; sys.path.insert(0, %r); import numpy as np; import slime_gb300 as sg\n"
        "try:\n"
        "    sg.Simulation(1024, 1024, 1000)\n"
        "    print('created')\n"
        "except sg.SlimeError as e:\n"
        "    print('status', e.status)\n"
        "s = sg.Simulation(64, 64, 100)\n"
        "s.step(2); print('small ok')\n"
        "s.seed_agents(5); s.step(3)\n"
        "a0, t0 = s.download_agents(), s.download_trail()\n"
        "for call in (lambda: s.resize(1024, 1024), lambda: s.set_agent_count(1_000_000)):\n"
        "    try:\n"
        "        call(); print('grew')\n"
        "    except sg.SlimeError as e:\n"
        "        print('status', e.status)\n"
        "i = s.info()\n"
        "same = (i.width, i.height, i.n_agents) == (64, 64, 100)\n"
        "same = same and np.array_equal(s.download_agents().view(np.uint32), a0.view(np.uint32))\n"
        "same = same and np.array_equal(s.download_trail().view(np.uint32), t0.view(np.uint32))\n"
        "print('unchanged', same)\n"
        "r = sg.Simulation(64, 64, 100, s.params())\n"
        "r.upload_agents(a0); r.upload_trail(t0); r.step(4); s.step(4)\n"
        "same = np.array_equal(s.download_agents().view(np.uint32), r.download_agents().view(np.uint32))\n"
        "same = same and np.array_equal(s.download_trail().view(np.uint32), r.download_trail().view(np.uint32))\n"
        "print('steps after failure', same)\n" % os.path.join(ROOT, "slime-mold_gb300"))
    env = dict(os.environ, SLIME_DEVICE_MEMORY_CAP=str(2 * 1024 * 1024))
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    text = out.stdout + out.stderr
    assert out.stdout.count("status -2") == 3 and "small ok" in out.stdout, text
    assert "unchanged True" in out.stdout and "steps after failure True" in out.stdout, text


def test_l2_carveout_only_for_trails_that_fit(gpu):
    """The trail persists in L2 only when all of it fits the carve-out; a
    larger trail, or persistence switched off, reserves nothing."""
    import slime_gb300 as sg
    small = sg.Simulation(1024, 1024, 1000, config0_params(1024, 1024))
    assert small.info().l2_persist_bytes == 1024 * 1024 * 4
    small.set_options(l2_persist=0)
    assert small.info().l2_persist_bytes == 0
    small.set_options(l2_persist=1)
    assert small.info().l2_persist_bytes == 1024 * 1024 * 4
    big = sg.Simulation(8192, 8192, 1000, config0_params(8192, 8192))
    assert big.info().l2_persist_bytes == 0  # 256 MiB: more than any carve-out
    big.close()
    small.close()


STREAM8 = 8  # 1 + the tile-table index of the 8-row streaming trail kernel


TMA_TILE = 11  # 1 + the tile-table index of the tensor-copy trail tile


@pytest.mark.parametrize("tile", [STREAM8, 9, 10, TMA_TILE])
@pytest.mark.parametrize("decay_mode,decay,dep", [(0, 10.0, 1.0), (1, 0.97, 1.0), (1, 0.9, 2.5), (0, 0.0, 1.0)])
def test_deposit_marks_match_counts(gpu, decay_mode, decay, dep, tile):
    """Steps that record deposit marks (deposition >= 1 on a non-negative
    trail) give the same bits as steps that count, and as the oracle."""
    W, H, n = 512, 384, 150_000  # ~0.8 agents per cell: many cells with 2+ deposits
    p = config0_params(W, H, decay_mode=decay_mode, blur_mode=1, decay_factor=decay,
                       pheromone_deposition_amount=dep)
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=31)
    trail = np.random.default_rng(32).random((H, W), dtype=np.float32)
    a = make_sim(W, H, n, p, agents, trail)
    a.set_options(trail_tile=tile, exact_counts=1)
    b = make_sim(W, H, n, p, agents, trail)
    b.set_options(trail_tile=tile)
    for chunk in (1, 7, 12):
        a.step(chunk)
        b.step(chunk)
        assert_bitexact(b.download_trail(), a.download_trail(), f"trail, marks vs counts ({chunk})")
        assert_bitexact(b.download_agents(), a.download_agents(), f"agents, marks vs counts ({chunk})")
    a.download_deposit_counts()  # counting steps keep their counts
    with pytest.raises(RuntimeError):
        b.download_deposit_counts()  # marking steps have none
    ca, ct = agents.copy(), trail.copy()
    oracle.run(p, W, H, ca, ct, 20)
    assert_bitexact(b.download_trail(), ct, "trail vs oracle")
    assert_bitexact(b.download_agents(), ca, "agents vs oracle")


def test_deposit_marks_only_when_every_deposit_saturates(gpu):
    """Marks are used only while they cannot change a result: a trail with
    negative or NaN values, a deposition below 1, or a growing multiplicative
    decay keep the counts; a cleared trail brings the marks back."""
    W, H, n = 256, 128, 30_000
    agents = agents_uniform(n, W, H, 1.0, 2.0, seed=41)
    rng = np.random.default_rng(42)
    dirty = rng.random((H, W), dtype=np.float32) - np.float32(0.3)  # some cells negative
    dirty[5, 7] = np.nan
    cases = [
        (config0_params(W, H), dirty, False),
        (config0_params(W, H, pheromone_deposition_amount=0.5), np.abs(dirty), False),
        (config0_params(W, H, decay_mode=1, decay_factor=1.5), np.abs(dirty[:, :]).clip(0, 1), False),
        (config0_params(W, H), np.nan_to_num(np.abs(dirty)), True),
    ]
    for p, tr, marks in cases:
        tr = np.ascontiguousarray(tr, np.float32)
        sim = make_sim(W, H, n, p, agents, tr)
        sim.set_options(trail_tile=STREAM8)
        sim.step(3)
        if marks:
            with pytest.raises(RuntimeError):
                sim.download_deposit_counts()
        else:
            sim.download_deposit_counts()
        ca, ct = agents.copy(), tr.copy()
        oracle.run(p, W, H, ca, ct, 3)
        assert_bitexact(sim.download_trail(), ct, f"trail (marks={marks})")
        assert_bitexact(sim.download_agents(), ca, f"agents (marks={marks})")
    # clearing a dirty trail makes it clean again
    sim = make_sim(W, H, n, config0_params(W, H), agents, np.ascontiguousarray(dirty))
    sim.set_options(trail_tile=STREAM8)
    sim.step(1)
    sim.download_deposit_counts()
    sim.clear_trail()
    sim.step(1)
    with pytest.raises(RuntimeError):
        sim.download_deposit_counts()


@pytest.mark.parametrize("W,H", [(1024, 512), (4096, 64), (528, 97), (272, 66)])
def test_tensor_copy_trail_tile(gpu, W, H):
    """The trail pass whose input window arrives by 2-D tensor copies (one
    box of trail and one of deposit record per 128 x 32 tile, the border tiles
    by wrapped loads): bit for bit the oracle over several steps, with byte
    marks and with 32-bit counts, box blur and Gaussian radius 1 and 2, both
    decays.  272 x 66 is the smallest grid with an interior tile (a 16-column
    margin of byte marks on each side of a 128-column tile, and its halo rows);
    4096 x 64 has border tiles only."""
    n = W * H // 2
    for blur_mode, radius, decay_mode, decay in ((0, 1.0, 0, 10.0), (1, 1.0, 1, 0.97), (1, 2.0, 1, 0.9),
                                                 (1, 1.0, 0, 3.0)):
        for exact_counts in (0, 1):
            p = config0_params(W, H, decay_mode=decay_mode, blur_mode=blur_mode, blur_radius=radius, blur_sigma=1.2,
                               decay_factor=decay)
            agents = agents_uniform(n, W, H, 1.0, 2.0, seed=W + H)
            trail = np.random.default_rng(H).random((H, W), dtype=np.float32)
            sim = make_sim(W, H, n, p, agents, trail)
            sim.set_options(trail_tile=TMA_TILE, exact_counts=exact_counts)
            assert sim.info().trail_tile == TMA_TILE - 1
            sim.step(3)
            sim.sync()
            ca, ct = agents.copy(), trail.copy()
            oracle.run(p, W, H, ca, ct, 3)
            what = f"{W}x{H} blur {blur_mode} r {radius} decay {decay_mode} counts {exact_counts}"
            assert_bitexact(sim.download_trail(), ct, "trail " + what)
            assert_bitexact(sim.download_agents(), ca, "agents " + what)
            sim.close()

