"""Generate tests/golden/wgsl/*.npz from the reference's own compute shader.

The reference's src/compute.wgsl, translated to C++ and run invocation by
invocation (oracle/wgsl/: translate.py, prelude.h, harness.cpp, wgslref.py),
advances small colonies frame by frame: `main` over every agent sensing the
trail as the frame found it, then decay_trail, then diffuse_trail.  Each
case keeps to where the shader's frame is deterministic and where the oracle
follows it exactly:

  frames_axis_dep1     the reference's default settings (deposition 1.0:
                       on a trail in [0, 1] every racing deposit leaves its
                       cell at 1) with jitter 0.05 and sensor angle 0, 12
                       frames; the saved frames compare whole.
  frames_shader_angle  the default settings as they are (sensor angle
                       0.3 rad), 3,000 agents on 64x64, 60 frames.
  frames_angle04       config 0's agent parameters (sensor angle 0.4 rad,
                       distance 9 px, turn 0.3, jitter 0.05) with deposition
                       1.0 in the reference's own decay and blur, 5,000
                       agents on 96x96, 60 frames.
  frames_angle0785     sensor angle pi/4 (0.7854 rad), distance 20 px,
                       jitter 0.3, 3,000 agents on 80x60, 60 frames.
                       These three use the seeds they are given, no others;
                       the oracle (default sensor mode, cos/sin of the
                       rounded angle -/+ a as the shader writes it) must
                       equal every saved frame, or the script fails.  At
                       about 5 flipped turns in 100,000 agent-steps the
                       opt-in rotated mode is expected to depart from each
                       of them (tests/test_golden_reference.py checks that
                       it does).
  pass_dep03           one frame at deposition 0.3 with decay and diffusion
                       0 (the frame is then the agent pass alone); the trail
                       compares on cells at most one agent lands on, where
                       the shader's non-atomic update loses nothing.
  display_fit          src/display.wgsl's colourise of a 97x61 trail (values
                       outside [0, 1] and NaN included) through a random LUT
                       into a wide (160x90) and a tall (90x160) image.

Each frames file holds W, H, the parameters (p_*), agents0 and trail0, the
list of saved frames, agents<s> and trail<s> for each, and `compare` ("all"
or "single_deposit_cells"); display_fit holds trail, lut and image<w>x<h>.
Needs the reference's source tree.
Run: python tests/golden/make_reference_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "slime-mold_gb300"))
sys.path.insert(0, HERE)
import oracle  # noqa: E402
from make_golden import PARAM_KEYS, agents  # noqa: E402
from slime_gb300 import SlimeParams  # noqa: E402
from wgsl import wgslref  # noqa: E402

OUT = os.path.join(HERE, "wgsl")


def params(W, H, **kw):
    """The reference's default settings (src/settings.rs:10-27, 49-70) in its
    own decay and blur (subtractive decay, 3x3 box)."""
    d = dict(decay_factor=10.0, agent_jitter=0.0, agent_speed_min=30.0, agent_speed_max=50.0,
             agent_turn_speed=0.43, agent_sensor_angle=0.3, agent_sensor_distance=20.0, diffusion_rate=1.0,
             pheromone_deposition_amount=1.0, blur_radius=2.0, blur_sigma=1.0, time_step=0.016,
             decay_mode=0, blur_mode=0)
    d.update(kw)
    p = SlimeParams()
    p.width, p.height = W, H
    for k, v in d.items():
        setattr(p, k, v)
    return p, d


def oracle_frames(p, W, H, a0, t0, saved):
    a, t = a0.copy(), t0.copy()
    out, done = {}, 0
    for s in saved:
        oracle.run(p, W, H, a, t, s - done)
        done = s
        out[s] = (a.copy(), t.copy())
    return out


def bits_equal(x, y):
    return np.array_equal(np.ascontiguousarray(x, np.float32).view(np.uint32),
                          np.ascontiguousarray(y, np.float32).view(np.uint32))


def write_case(name, W, H, p, d, a0, t0, saved, compare):
    a, t = a0.copy(), t0.copy()
    out = {"W": W, "H": H, "agents0": a0, "trail0": t0, "frames": np.array(saved, np.int32),
           "compare": np.array(compare)}
    for k, v in d.items():
        out["p_" + k] = np.float32(v) if k in PARAM_KEYS else np.int32(v)
    for s in range(1, max(saved) + 1):
        a, t = wgslref.frame(p, a, t)
        if s in saved:
            out[f"agents{s}"], out[f"trail{s}"] = a, t
    if compare == "all":
        ours = oracle_frames(p, W, H, a0, t0, saved)
        for s in saved:
            if not (bits_equal(ours[s][0], out[f"agents{s}"]) and bits_equal(ours[s][1], out[f"trail{s}"])):
                raise SystemExit(f"{name}: the oracle departs from the reference at frame {s}")
    os.makedirs(OUT, exist_ok=True)
    np.savez_compressed(os.path.join(OUT, f"{name}.npz"), **out)
    print(name, "written")


def main():
    if not wgslref.available():
        raise SystemExit("the reference's source tree is not present")
    W, H = 64, 48
    p, d = params(W, H, agent_sensor_angle=0.0, agent_jitter=0.05)
    write_case("frames_axis_dep1", W, H, p, d, agents(1500, W, H, 30, 50, 21),
               np.random.default_rng(22).random((H, W), dtype=np.float32), [1, 3, 12], "all")
    W, H = 64, 64
    p, d = params(W, H)
    write_case("frames_shader_angle", W, H, p, d, agents(3000, W, H, 30, 50, 23),
               np.random.default_rng(24).random((H, W), dtype=np.float32), [1, 8, 60], "all")
    W, H = 96, 96
    p, d = params(W, H, agent_sensor_angle=0.4, agent_sensor_distance=9.0, agent_turn_speed=0.3, agent_jitter=0.05)
    write_case("frames_angle04", W, H, p, d, agents(5000, W, H, 30, 50, 31),
               np.random.default_rng(32).random((H, W), dtype=np.float32), [1, 10, 60], "all")
    W, H = 80, 60
    p, d = params(W, H, agent_sensor_angle=0.7854, agent_jitter=0.3)
    write_case("frames_angle0785", W, H, p, d, agents(3000, W, H, 30, 50, 33),
               np.random.default_rng(34).random((H, W), dtype=np.float32), [1, 10, 60], "all")
    W, H = 64, 48
    p, d = params(W, H, agent_sensor_angle=0.0, agent_jitter=0.05, pheromone_deposition_amount=0.3,
                  decay_factor=0.0, diffusion_rate=0.0)
    write_case("pass_dep03", W, H, p, d, agents(2000, W, H, 30, 50, 25),
               np.random.default_rng(26).random((H, W), dtype=np.float32), [1], "single_deposit_cells")
    rng = np.random.default_rng(27)
    trail = rng.uniform(-0.2, 1.2, (61, 97)).astype(np.float32)
    trail.flat[:6] = [0.0, 1.0, np.nan, -0.0, 0.5 / 255, 254.5 / 255]
    lut = rng.integers(0, 256, 768, dtype=np.uint8)
    out = {"trail": trail, "lut": lut}
    for tw, th in ((160, 90), (90, 160)):
        out[f"image{tw}x{th}"] = wgslref.colorize(trail, lut, tw, th)
    np.savez_compressed(os.path.join(OUT, "display_fit.npz"), **out)
    print("display_fit written")


if __name__ == "__main__":
    main()
