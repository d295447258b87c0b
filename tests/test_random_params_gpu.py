"""A seeded sweep of random parameter sets: the CUDA path against the oracle,
bit for bit (agents, trail, and the last step's deposit counts).

Each case draws a trail size, an agent count and every SlimeParams field
from wide ranges, including values no preset uses (negative rates, zero
sensor distance, turn speeds beyond pi, deposition above and below 1, speeds
above the clamp, decay factors beyond 1), both decay and blur modes and both
dispatch modes, plus the engine options (Morton reordering every step,
graphs off, exact counts or deposit marks).  Parameters are drawn as binary32
values, so the oracle and the library see the same bits.
"""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params
from test_parity_gpu import assert_bitexact, make_sim

pytestmark = pytest.mark.gpu

CASES = 40


def draw(rng):
    W = int(rng.integers(2, 300))
    H = int(rng.integers(2, 200))
    n = int(rng.integers(1, 30000))
    f = lambda lo, hi: float(np.float32(rng.uniform(lo, hi)))  # noqa: E731
    decay_mode = int(rng.integers(0, 2))
    blur_mode = int(rng.integers(0, 2))
    p = config0_params(
        W, H, decay_mode=decay_mode, blur_mode=blur_mode,
        decay_factor=f(0.0, 1.2) if decay_mode == 1 else f(-5.0, 400.0),
        agent_jitter=f(-1.0, 3.0), agent_speed_min=f(-10.0, 60.0), agent_speed_max=f(0.0, 150.0),
        agent_turn_speed=f(-0.5, 4.0), agent_sensor_angle=f(-3.5, 3.5), agent_sensor_distance=f(0.0, 40.0),
        diffusion_rate=f(-0.3, 1.3), pheromone_deposition_amount=f(0.0, 2.5),
        blur_radius=f(0.0, 2.99) if blur_mode == 1 else 1.0, blur_sigma=f(0.3, 3.0),
        time_step=f(0.0, 0.05), dispatch_mode=int(rng.integers(0, 2)), sensor_mode=int(rng.integers(0, 2)))
    options = dict(reorder_every=int(rng.choice([0, 1, 3])), use_graphs=int(rng.integers(0, 2)),
                   exact_counts=int(rng.integers(0, 2)))
    return W, H, n, p, options


@pytest.mark.parametrize("case", range(CASES))
def test_random_parameters_bitexact(gpu, case):
    rng = np.random.default_rng(1000 + case)
    W, H, n, p, options = draw(rng)
    agents = agents_uniform(n, W, H, 0.0, 100.0, seed=case)
    trail = rng.random((H, W), dtype=np.float32)
    sim = make_sim(W, H, n, p, agents, trail)
    sim.set_options(**options)
    steps = int(rng.integers(1, 6))
    sim.step(steps)
    ca, ct = agents.copy(), trail.copy()
    counts = oracle.run(p, W, H, ca, ct, steps, record_counts=True)
    what = f"case {case}: {W}x{H}, {n} agents, {steps} steps, {options}"
    assert_bitexact(sim.download_agents(), ca, "agents " + what)
    assert_bitexact(sim.download_trail(), ct, "trail " + what)
    if options["exact_counts"]:
        assert_bitexact(sim.download_deposit_counts(), counts[-1], "counts " + what)
    sim.close()
