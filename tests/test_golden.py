"""Golden fixtures from the independent pure-Python restatement
(tests/golden/restate.py, generated by tests/golden/make_golden.py): the CPU
oracle (always) and the CUDA path (gpu) must reproduce every step bit for
bit."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT

FIXTURES = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "*.npz")))
KEYS = ["decay_factor", "agent_jitter", "agent_speed_min", "agent_speed_max", "agent_turn_speed",
        "agent_sensor_angle", "agent_sensor_distance", "diffusion_rate", "pheromone_deposition_amount",
        "blur_radius", "blur_sigma", "time_step", "decay_mode", "blur_mode"]


def load(path):
    from slime_gb300 import SlimeParams
    d = dict(np.load(path))
    p = SlimeParams()
    p.width, p.height = int(d["W"]), int(d["H"])
    for k in KEYS:
        setattr(p, k, d["p_" + k].item())
    # the side-sensor evaluation (0, the shader's, unless the case says otherwise)
    p.sensor_mode = int(d["p_sensor_mode"]) if "p_sensor_mode" in d else 0
    return d, p


def test_fixtures_present():
    assert len(FIXTURES) >= 4


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_oracle_reproduces_golden(path):
    d, p = load(path)
    W, H = int(d["W"]), int(d["H"])
    a, t = d["agents0"].copy(), d["trail0"].copy()
    for s in range(1, int(d["steps"]) + 1):
        c = oracle.agents_pass(p, W, H, a, t)
        t = oracle.trail_pass(p, W, H, t, c)
        assert np.array_equal(c, d[f"counts{s}"]), f"counts step {s}"
        assert np.array_equal(a.view(np.uint32), d[f"agents{s}"].view(np.uint32)), f"agents step {s}"
        assert np.array_equal(t.view(np.uint32), d[f"trail{s}"].view(np.uint32)), f"trail step {s}"


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_gpu_reproduces_golden(gpu, path):
    import slime_gb300 as sg
    d, p = load(path)
    W, H = int(d["W"]), int(d["H"])
    n = d["agents0"].shape[0]
    with sg.Simulation(W, H, n, p) as sim:
        sim.upload_agents(d["agents0"])
        sim.upload_trail(d["trail0"])
        for s in range(1, int(d["steps"]) + 1):
            sim.step(1)
            assert np.array_equal(sim.download_deposit_counts(), d[f"counts{s}"]), f"counts step {s}"
            assert np.array_equal(sim.download_agents().view(np.uint32), d[f"agents{s}"].view(np.uint32))
            assert np.array_equal(sim.download_trail().view(np.uint32), d[f"trail{s}"].view(np.uint32))
