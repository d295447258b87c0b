"""Generate the golden fixtures (tests/golden/*.npz) from the pure-Python
restatement in restate.py.

Each case stores the parameters, the initial agents (AoS x, y, angle, speed)
and trail, and after every step the agents, the trail and the deposit counts.
Run: python tests/golden/make_golden.py
"""
import os
import sys

import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import restate  # noqa: E402

PARAM_KEYS = ["decay_factor", "agent_jitter", "agent_speed_min", "agent_speed_max", "agent_turn_speed",
              "agent_sensor_angle", "agent_sensor_distance", "diffusion_rate", "pheromone_deposition_amount",
              "blur_radius", "blur_sigma", "time_step"]


def base_params(**kw):
    p = dict(decay_factor=0.97, agent_jitter=0.05, agent_speed_min=30.0, agent_speed_max=50.0,
             agent_turn_speed=0.3, agent_sensor_angle=0.4, agent_sensor_distance=9.0, diffusion_rate=0.5,
             pheromone_deposition_amount=1.0, blur_radius=1.0, blur_sigma=1.0, time_step=0.016,
             decay_mode=1, blur_mode=1, sensor_mode=0)
    p.update(kw)
    return {k: (np.float32(v) if k in PARAM_KEYS else int(v)) for k, v in p.items()}


def agents(n, W, H, lo, hi, seed):
    rng = np.random.default_rng(seed)
    a = np.stack([rng.uniform(0, W, n), rng.uniform(0, H, n), rng.uniform(0, 2 * np.pi, n),
                  rng.uniform(lo, hi, n)], axis=1).astype(np.float32)
    a[:, 0] = np.minimum(a[:, 0], np.nextafter(np.float32(W), np.float32(0)))
    a[:, 1] = np.minimum(a[:, 1], np.nextafter(np.float32(H), np.float32(0)))
    return a


def cases():
    W, H = 40, 30
    yield "ref_box", W, H, base_params(decay_mode=0, blur_mode=0, decay_factor=10.0, agent_jitter=0.3,
                                       agent_turn_speed=0.43), agents(300, W, H, 30, 50, 1), 3
    yield "mult_gauss_r1", W, H, base_params(), agents(300, W, H, 30, 50, 2), 3
    # the opt-in rotated side-sensor directions (SLIME_SENSOR_ROTATED)
    yield "mult_gauss_r1_rotated", W, H, base_params(sensor_mode=1), agents(300, W, H, 30, 50, 2), 3
    yield "gauss_r2_subtract", W, H, base_params(decay_mode=0, blur_radius=2.0, blur_sigma=1.5,
                                                 decay_factor=20.0, pheromone_deposition_amount=0.3,
                                                 agent_jitter=2.0), agents(300, W, H, 60, 120, 3), 3
    e = np.float32(1e-6)
    edge = np.array([[W - e, 10.0, 0.0, 40.0], [0.0, 0.0, np.pi, 40.0], [W - 1, H - 1, 0.3, 40.0],
                     [-1e-8, 5.0, np.pi, 40.0], [5.0, -1e-8, 1.5 * np.pi, 40.0], [W - 0.5, H - 0.5, 0.785, 60.0],
                     [20.5, 15.5, -7.0, 40.0], [10.0, 10.0, 1e6, 40.0], [10.0, 10.0, -1e7, 40.0],
                     [3.0, 3.0, 1e9, 40.0], [0.0, 0.0, 0.0, 0.0]], np.float32)
    yield "edges", W, H, base_params(decay_mode=0, blur_mode=0, agent_sensor_distance=20.0, agent_speed_min=0.5,
                                     agent_speed_max=100.0, agent_jitter=1.0, agent_turn_speed=0.43), edge, 4


def main():
    for name, W, H, p, a0, steps in cases():
        trail0 = np.random.default_rng(zlib.crc32(name.encode())).random((H, W), dtype=np.float32)
        a, t = a0.copy(), trail0.copy()
        out = {"W": W, "H": H, "agents0": a0, "trail0": trail0}
        for k, v in p.items():
            out["p_" + k] = v
        for s in range(steps):
            a, t, c = restate.step(p, W, H, a, t)
            out[f"agents{s + 1}"], out[f"trail{s + 1}"], out[f"counts{s + 1}"] = a, t, c
        out["steps"] = steps
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        print(name, "done")


if __name__ == "__main__":
    main()
