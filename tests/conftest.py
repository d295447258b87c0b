import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "slime-mold_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def built_lib():
    """Build libslime_gb300.so if it is missing or stale, then load it."""
    import build  # slime-mold_gb300/build.py
    build.build()
    import slime_gb300
    return slime_gb300.lib()


@pytest.fixture(scope="session")
def gpu(built_lib):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test ran without a CUDA device")
    torch.cuda.init()
    return built_lib


def agents_uniform(n, W, H, speed_lo, speed_hi, seed=0):
    """Agents as in the benchmark configurations: x ~ U[0,W), y ~ U[0,H),
    heading ~ U[0, 2pi), speed ~ U[lo, hi], binary32 (AoS x, y, angle, speed)."""
    rng = np.random.default_rng(seed)
    a = np.empty((n, 4), np.float32)
    a[:, 0] = rng.uniform(0, W, n).astype(np.float32)
    a[:, 1] = rng.uniform(0, H, n).astype(np.float32)
    a[:, 2] = rng.uniform(0, 2 * np.pi, n).astype(np.float32)
    a[:, 3] = rng.uniform(speed_lo, speed_hi, n).astype(np.float32)
    a[:, 0] = np.minimum(a[:, 0], np.nextafter(np.float32(W), np.float32(0)))
    a[:, 1] = np.minimum(a[:, 1], np.nextafter(np.float32(H), np.float32(0)))
    return a


def config0_params(W=512, H=512, decay_mode=1, blur_mode=1, **kw):
    """The 512x512 reference-size configuration: sensor angle 0.4 rad,
    distance 9 px, turn 0.3, jitter 0.05, deposition 1.0, decay 0.97,
    diffusion 0.5 through a 3-tap sigma=1 Gaussian, speed 1..2."""
    from slime_gb300 import SlimeParams
    p = SlimeParams()
    p.width, p.height = W, H
    p.decay_factor = 0.97
    p.agent_jitter = 0.05
    p.agent_speed_min, p.agent_speed_max = 1.0, 2.0
    p.agent_turn_speed = 0.3
    p.agent_sensor_angle = 0.4
    p.agent_sensor_distance = 9.0
    p.diffusion_rate = 0.5
    p.pheromone_deposition_amount = 1.0
    p.blur_radius = 1.0
    p.blur_sigma = 1.0
    p.time_step = 0.016
    p.decay_mode = decay_mode
    p.blur_mode = blur_mode
    for k, v in kw.items():
        setattr(p, k, v)
    return p
