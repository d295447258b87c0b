"""Golden frames from the reference's own shaders (tests/golden/wgsl/, made by
tests/golden/make_reference_golden.py from mechanical C++ translations of
src/compute.wgsl and src/display.wgsl run invocation by invocation): the CPU
oracle (always) and the CUDA path (gpu) must reproduce each saved frame bit
for bit, agents and trail; in `single_deposit_cells` cases the trail is
compared on the cells at most one agent landed on, the only cells whose
value the shader's non-atomic deposit defines.  The display images must be
reproduced byte for byte."""
import glob
import os

import numpy as np
import pytest

import oracle
from conftest import ROOT

FIXTURES = sorted(p for p in glob.glob(os.path.join(ROOT, "tests", "golden", "wgsl", "*.npz"))
                  if not os.path.basename(p).startswith("display_"))
DISPLAY = os.path.join(ROOT, "tests", "golden", "wgsl", "display_fit.npz")
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


def check(d, s, agents, trail, counts):
    assert np.array_equal(agents.view(np.uint32), d[f"agents{s}"].view(np.uint32)), f"agents frame {s}"
    ref = d[f"trail{s}"]
    if str(d["compare"]) == "all":
        assert np.array_equal(trail.view(np.uint32), ref.view(np.uint32)), f"trail frame {s}"
    else:
        single = counts <= 1
        assert np.count_nonzero(single) > single.size // 2
        assert np.array_equal(trail[single].view(np.uint32), ref[single].view(np.uint32)), f"trail frame {s}"


def test_fixtures_present():
    assert len(FIXTURES) == 5


@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_oracle_reproduces_reference_frames(path):
    d, p = load(path)
    W, H = int(d["W"]), int(d["H"])
    a, t = d["agents0"].copy(), d["trail0"].copy()
    done = 0
    for s in d["frames"].tolist():
        while done < s:
            c = oracle.agents_pass(p, W, H, a, t)
            t = oracle.trail_pass(p, W, H, t, c)
            done += 1
        check(d, s, a, t, c)


def test_rotated_mode_departs_from_the_reference_frames():
    """The fixtures discriminate: with the opt-in rotated sensor directions
    the oracle leaves the reference's run on at least one of them (a flipped
    near-tie turn, then chaotic divergence), while the default mode
    reproduces all of them."""
    departed = []
    for path in FIXTURES:
        d, p = load(path)
        p.sensor_mode = 1
        W, H = int(d["W"]), int(d["H"])
        a, t = d["agents0"].copy(), d["trail0"].copy()
        last = d["frames"].tolist()[-1]
        oracle.run(p, W, H, a, t, last)
        departed.append(not np.array_equal(a.view(np.uint32), d[f"agents{last}"].view(np.uint32)))
    assert any(departed)


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=lambda p: os.path.basename(p))
def test_gpu_reproduces_reference_frames(gpu, path):
    import slime_gb300 as sg
    d, p = load(path)
    W, H = int(d["W"]), int(d["H"])
    with sg.Simulation(W, H, d["agents0"].shape[0], p) as sim:
        sim.set_options(exact_counts=1)
        sim.upload_agents(d["agents0"])
        sim.upload_trail(d["trail0"])
        done = 0
        for s in d["frames"].tolist():
            if s - 1 > done:
                sim.step(s - 1 - done)
            sim.step(1)  # the counts of the saved frame's own step
            done = s
            check(d, s, sim.download_agents(), sim.download_trail(), sim.download_deposit_counts())


def display_cases():
    d = dict(np.load(DISPLAY))
    for key in sorted(k for k in d if k.startswith("image")):
        tw, th = (int(v) for v in key[5:].split("x"))
        yield d["trail"], d["lut"], tw, th, d[key]


def test_oracle_reproduces_reference_display():
    for trail, lut, tw, th, image in display_cases():
        H, W = trail.shape
        assert np.array_equal(oracle.colorize(W, H, trail, lut, tw, th), image), (tw, th)


@pytest.mark.gpu
def test_gpu_reproduces_reference_display(gpu):
    import slime_gb300 as sg
    for trail, lut, tw, th, image in display_cases():
        H, W = trail.shape
        with sg.Simulation(W, H, 1, None) as sim:
            sim.upload_trail(trail)
            assert np.array_equal(sim.colorize(lut, tw, th), image), (tw, th)
