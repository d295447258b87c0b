"""The batched ensemble (both engines: per-colony kernel chains on capture
lanes, and one cooperative persistent launch per step, over colonies of
uneven sizes and parameters) against one plain Simulation per colony and the
CPU oracle, bit for bit."""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from test_parity_gpu import assert_bitexact

pytestmark = pytest.mark.gpu


def colony_setup(seed, blur_mode, radius=1.0):
    rng = np.random.default_rng(seed)
    sizes = [(256, 256), (128, 64), (512, 200), (8, 8), (300, 120), (64, 333)]
    cols = []
    for j, (W, H) in enumerate(sizes):
        n = int(W * H * rng.uniform(0.25, 4.0))
        p = config0_params(W, H, decay_mode=int(rng.integers(0, 2)), blur_mode=blur_mode, blur_radius=radius,
                           blur_sigma=float(rng.uniform(0.7, 1.5)),
                           agent_sensor_angle=float(rng.uniform(0.2, 0.8)),
                           agent_sensor_distance=float(rng.uniform(4, 20)),
                           agent_turn_speed=float(rng.uniform(0.1, 0.6)), agent_jitter=float(rng.uniform(0, 0.1)),
                           decay_factor=float(rng.uniform(0.9, 0.995)), diffusion_rate=float(rng.uniform(0.1, 0.9)),
                           pheromone_deposition_amount=float(rng.uniform(0.5, 2.0)),
                           agent_speed_min=30.0, agent_speed_max=60.0)
        if p.decay_mode == 0:
            p.decay_factor = float(rng.uniform(1, 20))
        agents = agents_uniform(n, W, H, 30.0, 60.0, seed=seed * 100 + j)
        trail = rng.random((H, W), dtype=np.float32)
        cols.append((W, H, n, p, agents, trail))
    return cols


@pytest.mark.parametrize("engine", [0, 1])
@pytest.mark.parametrize("blur_mode,radius,reorder", [(1, 1.0, 0), (0, 1.0, 3), (1, 2.0, 2)])
def test_ensemble_matches_plain_runs(gpu, blur_mode, radius, reorder, engine):
    import slime_gb300 as sg
    cols = colony_setup(7, blur_mode, radius)
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    ens.set_engine(engine)
    ens.set_reorder(reorder, 1)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    assert ens.info().graphs_in_use == 0  # no step yet
    ens.step(7)
    ens.sync()
    assert ens.launch_count() >= 7
    info = ens.info()
    # the step launches were captured and replayed as graphs
    assert info.graphs_in_use == 1, "capture of the step launches fell back to direct launches"
    assert info.engine == engine and info.lanes == (len(cols) if engine == sg.ENSEMBLE_LANES else 0)
    if engine == sg.ENSEMBLE_COOPERATIVE:
        assert info.marks_colonies == 0
    assert (info.n_colonies, info.steps_done) == (len(cols), 7)
    assert info.total_agents == sum(c[2] for c in cols) and info.total_cells == sum(c[0] * c[1] for c in cols)
    assert info.grid_blocks > 0 and info.strip_rows in (8, 16, 32)
    assert info.agents_per_thread in (2, 4)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        with sg.Simulation(W, H, n, p) as sim:
            sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(7)
            assert_bitexact(ens.download_agents(j), sim.download_agents(), f"colony {j} agents")
            assert_bitexact(ens.download_trail(j), sim.download_trail(), f"colony {j} trail")
        if W * H <= 40000:
            ca, ct = agents.copy(), trail.copy()
            oracle.run(p, W, H, ca, ct, 7)
            assert_bitexact(ens.download_trail(j), ct, f"colony {j} trail vs oracle")


@pytest.mark.parametrize("rows,bps,apt", [(8, 0, 2), (32, 2, 2), (16, 1, 2), (8, 4, 4), (32, 0, 4)])
def test_every_launch_shape_gives_the_same_result(gpu, rows, bps, apt):
    """Strip height, residency and agents per thread (four alone or two as a
    pair; colonies with agent counts that leave a ragged last group) change
    the launch only: every colony matches a plain run bit for bit."""
    import slime_gb300 as sg
    cols = colony_setup(17, 1)
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    ens.set_shape(rows, bps, apt)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    ens.step(5)
    ens.sync()
    info = ens.info()
    assert (info.strip_rows, info.agents_per_thread) == (rows, apt)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        with sg.Simulation(W, H, n, p) as sim:
            sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(5)
            assert_bitexact(ens.download_agents(j), sim.download_agents(), f"colony {j} agents")
            assert_bitexact(ens.download_trail(j), sim.download_trail(), f"colony {j} trail")
    with pytest.raises(sg.SlimeError):
        ens.set_shape(12, 0, 4)
    with pytest.raises(sg.SlimeError):
        ens.set_shape(16, 0, 3)
    ens.close()


@pytest.mark.parametrize("shape,tile", [(13, 8), (9, 7), (15, 9), (0, 3), (12, 4)])
def test_lanes_engine_shapes_and_params_update(gpu, shape, tile):
    """The lanes engine (each colony a chain of the single-colony kernels on
    its own capture lane) with persistent and regular agent shapes, streaming
    and shared-memory trail tiles, and a parameter change between chunks
    (the captured graphs hold parameters as kernel arguments): bit for bit
    the plain runs."""
    import slime_gb300 as sg
    cols = colony_setup(19, 1)
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    ens.set_engine(sg.ENSEMBLE_LANES, shape, tile)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    assert ens.profile_reorder(2) > 0  # reorders change only the slot order: results below still match
    ens.prepare_steps(3)
    assert ens.info().steps_done == 0
    ens.step(3)
    marks_before = ens.info().marks_colonies
    streams = tile in (7, 8, 9)
    assert (marks_before > 0) == streams  # deposition >= 1 on a streaming tile: byte marks
    # colony 1: new decay and turn; colonies 2 and 4: deposition moved across 1,
    # so that their deposit records switch between counts and marks mid-run
    changed = {}
    for j in (1, 2, 4):
        q = cols[j][3].copy()
        if j == 1:
            q.agent_turn_speed = 0.05
            q.decay_factor = 0.5
        else:
            q.pheromone_deposition_amount = 0.6 if q.pheromone_deposition_amount >= 1.0 else 1.5
        ens.set_params(j, q)
        changed[j] = q
    ens.step(4)
    ens.sync()
    info = ens.info()
    assert (info.engine, info.lane_agent_shape, info.lane_trail_tile) == (sg.ENSEMBLE_LANES, shape, tile)
    assert info.kernel_launches > 0 and info.steps_done == 7
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        with sg.Simulation(W, H, n, p) as sim:
            sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(3)
            if j in changed:
                sim.set_params(changed[j])
            sim.step(4)
            assert_bitexact(ens.download_agents(j), sim.download_agents(), f"colony {j} agents")
            assert_bitexact(ens.download_trail(j), sim.download_trail(), f"colony {j} trail")
    with pytest.raises(sg.SlimeError):
        ens.set_engine(2)
    with pytest.raises(sg.SlimeError):
        ens.set_engine(sg.ENSEMBLE_LANES, 99, 8)
    with pytest.raises(sg.SlimeError):
        ens.set_engine(sg.ENSEMBLE_LANES, 13, 10)  # the tensor-copy tile needs per-colony maps
    ens.close()


@pytest.mark.parametrize("lanes", [0, 3])
def test_lanes_engine_many_small_colonies(gpu, lanes):
    """70 small colonies (some without agents): more colonies than lanes, so
    a lane chains several colonies' kernels one after another (programmatic
    dependent launches across colonies); every colony matches its plain run."""
    import slime_gb300 as sg
    rng = np.random.default_rng(23)
    cols = []
    for j in range(70):
        W, H = 4 * int(rng.integers(2, 17)), int(rng.integers(4, 41))
        n = 0 if j % 11 == 5 else int(rng.integers(1, 2000))
        p = config0_params(W, H, blur_mode=1, agent_speed_min=20.0, agent_speed_max=60.0,
                           agent_jitter=float(rng.uniform(0, 0.2)),
                           pheromone_deposition_amount=float(rng.uniform(0.5, 2.0)))
        agents = agents_uniform(n, W, H, 20.0, 60.0, seed=500 + j) if n else np.zeros((0, 4), np.float32)
        cols.append((W, H, n, p, agents, rng.random((H, W), dtype=np.float32)))
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    ens.set_engine(sg.ENSEMBLE_LANES, 13, 8, lanes)
    ens.set_reorder(2, 1)
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        if n:
            ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    ens.step(5)
    ens.sync()
    info = ens.info()
    assert info.lanes == (lanes if lanes else 64) and info.graphs_in_use == 1
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        with sg.Simulation(W, H, n, p) as sim:
            if n:
                sim.upload_agents(agents)
            sim.upload_trail(trail)
            sim.step(5)
            if n:
                assert_bitexact(ens.download_agents(j), sim.download_agents(), f"colony {j} agents")
            assert_bitexact(ens.download_trail(j), sim.download_trail(), f"colony {j} trail")
    ens.close()


def test_ensemble_autotune_and_params_update(gpu):
    import slime_gb300 as sg
    cols = colony_setup(11, 1)
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    ens.set_reorder(2)
    ens.autotune(1)
    q = cols[2][3].copy()
    q.agent_jitter = 0.5
    ens.set_params(2, q)
    ens.step(4)
    ens.sync()
    W, H, n, p, agents, trail = cols[2]
    ca, ct = agents.copy(), trail.copy()
    oracle.run(q, W, H, ca, ct, 4)
    assert_bitexact(ens.download_trail(2), ct, "colony 2 after set_params")
    assert_bitexact(ens.download_agents(2), ca, "colony 2 agents after set_params")


def test_ensemble_rejects_mixed_blur_and_bad_widths(gpu):
    import slime_gb300 as sg
    p1 = config0_params(64, 64, blur_mode=1)
    p2 = config0_params(64, 64, blur_mode=0)
    with pytest.raises(sg.SlimeError):
        sg.Ensemble([64, 64], [64, 64], [10, 10], [p1, p2])
    with pytest.raises(sg.SlimeError):
        sg.Ensemble([66], [64], [10], [config0_params(66, 64)])
    ens = sg.Ensemble([64], [64], [10], [config0_params(64, 64)])
    with pytest.raises(sg.SlimeError) as e:
        ens.seed_agents(0, 1, float("nan"), 1.0)
    assert e.value.status == -1
    with pytest.raises(sg.SlimeError):
        ens.seed_agents(1, 1)  # colony index out of range
    ens.close()


def test_bounded_barrier_times_out_and_recovers(gpu):
    """The grid barrier's wait is bounded: a barrier that can never be
    released gives SLIME_ERR_DEVICE_TIMEOUT (no hang, no trap), and the
    ensemble keeps stepping correctly afterwards."""
    import slime_gb300 as sg
    cols = colony_setup(13, 1)[:2]
    ens = sg.Ensemble([c[0] for c in cols], [c[1] for c in cols], [c[2] for c in cols], [c[3] for c in cols])
    for j, (W, H, n, p, agents, trail) in enumerate(cols):
        ens.upload_agents(j, agents)
        ens.upload_trail(j, trail)
    assert ens.selftest_barrier_timeout() == -5
    ens.step(2)
    ens.sync()
    W, H, n, p, agents, trail = cols[0]
    ca, ct = agents.copy(), trail.copy()
    oracle.run(p, W, H, ca, ct, 2)
    assert_bitexact(ens.download_trail(0), ct, "colony 0 after the timeout self-test")
