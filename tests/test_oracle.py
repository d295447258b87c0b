"""Known-answer tests of the CPU oracle (hand-derived single-agent cases for
each turn branch, wraps, sampler bounds, the deposit fold, decay and the 3x3
stencil), its thread-count invariance, the binary32-vs-binary64 error of the
trail pass, and its binary64 adjoint against central finite differences."""
import numpy as np
import pytest

import oracle
from conftest import agents_uniform, config0_params

f32 = np.float32


def one_agent(x, y, angle, speed):
    return np.array([[x, y, angle, speed]], np.float32)


def ref_params(W, H, **kw):
    base = dict(decay_mode=0, blur_mode=0, agent_jitter=0.0, agent_speed_min=30.0, agent_speed_max=50.0,
                agent_turn_speed=0.3, agent_sensor_angle=0.4, agent_sensor_distance=9.0, decay_factor=10.0,
                diffusion_rate=1.0)
    base.update(kw)
    return config0_params(W, H, **base)


def test_straight_move_and_deposit_zero_trail():
    W, H = 64, 48
    p = ref_params(W, H)
    a = one_agent(10.5, 20.5, 0.0, 40.0)
    c = oracle.agents_pass(p, W, H, a, np.zeros((H, W), np.float32))
    # angle 0: cos = 1, sin = 0 exactly; move = 40 * 0.016 in binary32
    move = f32(40.0) * f32(0.016)
    assert a[0, 0] == f32(10.5) + move and a[0, 1] == f32(20.5)
    assert a[0, 2] == 0.0 and a[0, 3] == 40.0
    assert c[20, int(a[0, 0])] == 1 and c.sum() == 1


def test_speed_is_clamped_and_stored():
    W, H = 16, 16
    p = ref_params(W, H)
    a = np.array([[5.0, 5.0, 0.0, 100.0], [5.0, 5.0, 0.0, 1.0]], np.float32)
    oracle.agents_pass(p, W, H, a, np.zeros((H, W), np.float32))
    assert a[0, 3] == 50.0 and a[1, 3] == 30.0  # compute.wgsl:72, :144


def _sensor_trail(W, H, x, y, angle, p, which):
    """A trail that is bright only around one sensor's position."""
    t = np.zeros((H, W), np.float32)
    off = {"left": -p.agent_sensor_angle, "right": p.agent_sensor_angle, "center": 0.0}[which]
    sx = x + p.agent_sensor_distance * np.cos(angle + off)
    sy = y + p.agent_sensor_distance * np.sin(angle + off)
    t[int(np.floor(sy)):int(np.floor(sy)) + 2, int(np.floor(sx)):int(np.floor(sx)) + 2] = 1.0
    return t


@pytest.mark.parametrize("which,expected", [("left", -0.3), ("right", 0.3), ("center", 0.0)])
def test_turn_branches(which, expected):
    W, H = 64, 64
    p = ref_params(W, H)
    x, y, angle = 30.0, 30.0, 1.0
    t = _sensor_trail(W, H, x, y, angle, p, which)
    a = one_agent(x, y, angle, 40.0)
    oracle.agents_pass(p, W, H, a, t)
    # compute.wgsl:98-112: angle += min(turn, |diff|) * sign(diff), diff = (angle -/+ TAU) - angle
    tau = f32(6.28318530718)
    if which == "left":
        diff = (f32(angle) - tau) - f32(angle)
        want = f32(angle) + np.minimum(f32(0.3), np.abs(diff)) * np.sign(diff)
    elif which == "right":
        diff = (f32(angle) + tau) - f32(angle)
        want = f32(angle) + np.minimum(f32(0.3), np.abs(diff)) * np.sign(diff)
    else:
        want = f32(angle)
    assert a[0, 2] == f32(want)
    assert abs(float(a[0, 2]) - (1.0 + expected)) < 1e-6


def test_equal_sensors_do_not_turn():
    W, H = 64, 64
    p = ref_params(W, H)
    a = one_agent(30.0, 30.0, 2.0, 40.0)
    oracle.agents_pass(p, W, H, a, np.full((H, W), 0.5, np.float32))
    assert a[0, 2] == f32(2.0)


def test_angle_normalised_into_0_2pi():
    W, H = 64, 64
    p = ref_params(W, H, agent_turn_speed=0.3)
    t = _sensor_trail(W, H, 30.0, 30.0, 0.1, p, "left")
    a = one_agent(30.0, 30.0, 0.1, 40.0)
    oracle.agents_pass(p, W, H, a, t)
    # 0.1 - 0.3 < 0, so fmod keeps the sign and 2*pi is added (compute.wgsl:121-122)
    assert a[0, 2] == (f32(0.1) - f32(0.3)) + f32(6.28318530718)


def test_position_wraps_toroidally():
    W, H = 64, 48
    p = ref_params(W, H)
    a = one_agent(W - 0.25, 10.0, 0.0, 40.0)
    c = oracle.agents_pass(p, W, H, a, np.zeros((H, W), np.float32))
    want = np.fmod(f32(W - 0.25) + f32(40.0) * f32(0.016), f32(W))
    assert a[0, 0] == want and 0 <= a[0, 0] < 1
    assert c[10, 0] == 1
    # moving left past x = 0 wraps to W - something; pi is not exact, so the
    # sine term leaves y nearly unchanged
    b = one_agent(0.1, 10.0, np.pi, 40.0)
    oracle.agents_pass(p, W, H, b, np.zeros((H, W), np.float32))
    assert W - 1 < b[0, 0] < W


def test_sensor_outside_grid_reads_zero_not_wrapped():
    """sample_trail_map returns 0 when a tap leaves the grid (compute.wgsl:14-16)."""
    W, H = 32, 32
    p = ref_params(W, H, agent_sensor_distance=9.0)
    t = np.zeros((H, W), np.float32)
    t[:, :4] = 1.0  # bright on the left edge: a wrapped sampler would see it
    a = one_agent(30.0, 16.0, 0.0, 40.0)  # all three sensors past the right edge
    oracle.agents_pass(p, W, H, a, t)
    assert a[0, 2] == 0.0  # all samples 0: no turn


def test_deposit_fold_sequence():
    W, H = 4, 4
    p = ref_params(W, H, decay_factor=0.0, diffusion_rate=0.0, pheromone_deposition_amount=0.3)
    t = np.full((H, W), 0.2, np.float32)
    counts = np.zeros((H, W), np.uint32)
    counts[1, 2] = 4
    counts[3, 3] = 1
    out = oracle.trail_pass(p, W, H, t, counts)
    seq = f32(0.2)
    for _ in range(4):
        seq = np.clip(seq + f32(0.3), f32(0.0), f32(1.0))
    assert out[1, 2] == seq == 1.0
    assert out[3, 3] == f32(0.2) + f32(0.3)
    assert out[0, 0] == f32(0.2)


def test_decay_modes():
    W, H = 3, 3
    t = np.full((H, W), 0.5, np.float32)
    z = np.zeros((H, W), np.uint32)
    p = ref_params(W, H, decay_factor=10.0, diffusion_rate=0.0)
    assert (oracle.trail_pass(p, W, H, t, z) == f32(0.5) - f32(10.0) * f32(0.001)).all()
    p = ref_params(W, H, decay_factor=1000.0, diffusion_rate=0.0)
    assert (oracle.trail_pass(p, W, H, t, z) == 0.0).all()  # max(t - 1, 0)
    p = ref_params(W, H, decay_mode=1, decay_factor=0.97, diffusion_rate=0.0)
    assert (oracle.trail_pass(p, W, H, t, z) == f32(0.5) * f32(0.97)).all()


def test_box_diffuse_hand_computed():
    """3x3 toroidal box, summed dy-outer dx-inner from 0.0, /9, then
    mix(t, avg, rate) (compute.wgsl:176-194)."""
    W, H = 4, 3
    t = np.arange(12, dtype=np.float32).reshape(H, W) / f32(16)
    z = np.zeros((H, W), np.uint32)
    p = ref_params(W, H, decay_factor=0.0, diffusion_rate=0.25)
    out = oracle.trail_pass(p, W, H, t, z)
    for y in range(H):
        for x in range(W):
            s = f32(0.0)
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    s = f32(s + t[(y + dy) % H, (x + dx) % W])
            avg = f32(s / f32(9.0))
            want = f32(f32(t[y, x] * f32(0.75)) + f32(avg * f32(0.25)))
            assert out[y, x] == want, (y, x)


def test_gauss_weights_symmetric_and_normalised():
    w = oracle.gauss_weights(1.0, 1.0)
    e = np.exp(-0.5)
    assert np.allclose(w, [e / (1 + 2 * e), 1 / (1 + 2 * e), e / (1 + 2 * e)], rtol=1e-7)
    w = oracle.gauss_weights(3.7, 1.5)
    assert w.size == 7 and np.array_equal(w, w[::-1]) and abs(w.sum() - 1) < 1e-6
    assert oracle.gauss_weights(1.0, 0.0) is None


def test_thread_count_invariance():
    W, H, n = 96, 80, 5000
    p = config0_params(W, H, decay_mode=0, blur_mode=0, decay_factor=10.0, agent_speed_min=30.0,
                       agent_speed_max=50.0, agent_jitter=0.4)
    a0 = agents_uniform(n, W, H, 30.0, 50.0, seed=1)
    t0 = np.random.default_rng(1).random((H, W), dtype=np.float32)
    res = []
    for threads in (1, 3, 8):
        a, t = a0.copy(), t0.copy()
        oracle.run(p, W, H, a, t, 5, threads=threads)
        res.append((a.view(np.uint32).copy(), t.view(np.uint32).copy()))
    for a, t in res[1:]:
        assert np.array_equal(a, res[0][0]) and np.array_equal(t, res[0][1])


def test_trail_pass_binary32_error_vs_binary64():
    """The binary32 decay+diffuse step against the binary64 twin: a few ulp."""
    W, H = 128, 96
    rng = np.random.default_rng(3)
    t = rng.random((H, W), dtype=np.float32)
    c = rng.integers(0, 3, (H, W)).astype(np.uint32)
    for dm, bm, r in ((0, 0, 1.0), (1, 1, 1.0), (1, 1, 4.0)):
        p = config0_params(W, H, decay_mode=dm, blur_mode=bm, blur_radius=r, pheromone_deposition_amount=0.2,
                           decay_factor=0.97 if dm else 10.0)
        o32 = oracle.trail_pass(p, W, H, t, c).astype(np.float64)
        o64 = oracle.trail_pass_f64(p, W, H, t.astype(np.float64), c)
        rel = np.abs(o32 - o64).max() / np.abs(o64).max()
        assert rel < 1e-6, (dm, bm, r, rel)


def _chain_setup(W=48, H=40, n=600, steps=12, dm=1, bm=1, dep=0.05, seed=0):
    p = config0_params(W, H, decay_mode=dm, blur_mode=bm, pheromone_deposition_amount=dep,
                       decay_factor=0.97 if dm else 10.0, agent_speed_min=30.0, agent_speed_max=50.0)
    a = agents_uniform(n, W, H, 30.0, 50.0, seed=seed)
    rng = np.random.default_rng(seed + 1)
    # Away from the kinks: trail in [0.2, 0.5] stays above the subtractive
    # decay's floor and, with a small deposition, below the fold's clamp at 1.
    t0 = (0.2 + rng.random((H, W)) * 0.3).astype(np.float32)
    counts = oracle.run(p, W, H, a, t0.copy(), steps, record_counts=True)
    target = rng.random((H, W))
    return p, t0.astype(np.float64), counts, target


@pytest.mark.parametrize("dm,bm", [(1, 1), (0, 0)])
def test_chain_adjoint_matches_finite_differences(dm, bm):
    W, H = 48, 40
    p, t0, counts, target = _chain_setup(W, H, dm=dm, bm=bm)
    theta = [float(np.float32(p.decay_factor)), float(np.float32(p.diffusion_rate)),
             float(np.float32(p.pheromone_deposition_amount))]
    loss, grads, d0 = oracle.chain_adjoint_f64(p, W, H, *theta, t0, counts, target=target)
    _, fin = oracle.chain_loss_f64(p, W, H, *theta, t0, counts, target)
    assert fin.max() < 1.0 and (counts.max() * 0.05 + 0.5) < 1.0
    # h = 1e-4, except for the subtractive decay, which enters as decay * 0.001
    hs = [1e-4 if dm == 1 else 1e-2, 1e-4, 1e-4]

    def loss_at(th):
        return oracle.chain_loss_f64(p, W, H, *th, t0, counts, target)[0]

    for i in range(3):
        fd = fd4(loss_at, theta, i, hs[i])
        assert abs(fd - grads[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, grads[i])
    # directional derivative along a random trail direction
    v = np.random.default_rng(9).standard_normal(t0.shape)
    eps = 1e-5
    lp, _ = oracle.chain_loss_f64(p, W, H, *theta, t0 + eps * v, counts, target)
    lm, _ = oracle.chain_loss_f64(p, W, H, *theta, t0 - eps * v, counts, target)
    assert abs((lp - lm) / (2 * eps) - (d0 * v).sum()) <= 1e-6 * max(1.0, abs((d0 * v).sum()))


def fd4(f, theta, i, h):
    """Fourth-order central finite difference of f along coordinate i."""
    def at(k):
        t = list(theta)
        t[i] += k * h
        return f(t)
    return (-at(2) + 8 * at(1) - 8 * at(-1) + at(-2)) / (12 * h)
