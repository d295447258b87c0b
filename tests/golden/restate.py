"""Independent pure-Python restatement of the reference step, used only to
generate the golden fixtures in this folder (make_golden.py).

It is written separately from the C++ oracle (oracle/slime_oracle.cpp) and
from the CUDA kernels: binary32 arithmetic is numpy float32 scalar arithmetic,
fused multiply-adds and integer-to-float conversions are rounded exactly from
rationals, and the sin/cos reductions are redone with Python integers.  The
algorithm is src/compute.wgsl (sample_trail_map :7-29, main :57-145,
decay_trail :148-161, diffuse_trail :164-195) with the builtins defined in
include/slime_math.h (Cody-Waite / Payne-Hanek reduction, Taylor polynomials).
Slow by design: only for small cases.
"""
from fractions import Fraction

import numpy as np

f32 = np.float32
MAXF = float(np.finfo(np.float32).max)


def round_f32(q):
    """Round a rational (Fraction or int) to binary32, ties to even."""
    q = Fraction(q)
    if q == 0:
        return f32(0.0)
    neg = q < 0
    q = -q if neg else q
    e = q.numerator.bit_length() - q.denominator.bit_length()
    while q >= Fraction(2) ** (e + 1):
        e += 1
    while q < Fraction(2) ** e:
        e -= 1
    e = max(e, -126)
    sh = e - 23
    scaled = q / (Fraction(2) ** sh)
    m = scaled.numerator // scaled.denominator
    r = scaled - m
    if r > Fraction(1, 2) or (r == Fraction(1, 2) and (m & 1)):
        m += 1
    val = float(m) * 2.0 ** sh
    if val > MAXF:
        val = float("inf")
    return f32(-val if neg else val)


def fma(a, b, c):
    return round_f32(Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c)))


def add(a, b):
    return f32(f32(a) + f32(b))


def sub(a, b):
    return f32(f32(a) - f32(b))


def mul(a, b):
    return f32(f32(a) * f32(b))


def div(a, b):
    return f32(f32(a) / f32(b))


def isnan(x):
    return x != x


def fmin(a, b):
    """minimumNumber: NaN ignored, -0 below +0."""
    if isnan(a):
        return f32(b)
    if isnan(b):
        return f32(a)
    if a == b:
        return f32(a) if np.signbit(a) else f32(b)
    return f32(b) if b < a else f32(a)


def fmax(a, b):
    """maximumNumber: NaN ignored, +0 above -0."""
    if isnan(a):
        return f32(b)
    if isnan(b):
        return f32(a)
    if a == b:
        return f32(b) if np.signbit(a) else f32(a)
    return f32(b) if b > a else f32(a)


def clamp(e, lo, hi):
    return fmin(fmax(e, lo), hi)


def sign(x):
    return f32(1.0) if x > 0 else (f32(-1.0) if x < 0 else f32(0.0))


def floor(x):
    return f32(np.floor(f32(x)))


def fract(x):
    return sub(x, floor(x))


def mix(a, b, t):
    return add(mul(a, sub(f32(1.0), t)), mul(b, t))


def fmod(x, y):
    import math
    return f32(math.fmod(float(x), float(y)))


def f2i(x):
    if isnan(x):
        return 0
    if x >= 2147483648.0:
        return 2147483647
    if x <= -2147483648.0:
        return -2147483648
    return int(float(x))  # truncation toward zero


def i2f(i):
    return round_f32(int(i))


# -- constants (same derivation as include/gen_slime_math_constants.py)
def _hex(s):
    return f32(float.fromhex(s))


TWO_OVER_PI_F = _hex("0x1.45f306p-1")
PIO2 = [_hex("0x1.921fb6p+0"), _hex("-0x1.777a5cp-25"), _hex("-0x1.ee59dap-50")]
S = [_hex("-0x1.555556p-3"), _hex("0x1.111112p-7"), _hex("-0x1.a01a02p-13"), _hex("0x1.71de3ap-19")]
CC = [_hex("-0x1p-1"), _hex("0x1.555556p-5"), _hex("-0x1.6c16c2p-10"), _hex("0x1.a01a02p-16"),
      _hex("-0x1.27e4fcp-22")]
TWO_OVER_PI_WORDS = [0x00000000, 0xa2f9836e, 0x4e441529, 0xfc2757d1, 0xf534ddc0, 0xdb629599, 0x3c439041,
                     0xfe5163ab, 0xdebbc561, 0xb7246e3a]
TAU = f32(6.28318530718)
M64 = (1 << 64) - 1


def reduce_pio2(x):
    x = f32(x)
    if abs(float(x)) < 4096.0:
        j = f32(np.rint(mul(x, TWO_OVER_PI_F)))
        r = fma(-j, PIO2[0], x)
        r = fma(-j, PIO2[1], r)
        r = fma(-j, PIO2[2], r)
        return r, int(j) & 3
    ix = int(np.array(x).view(np.uint32))
    E = (ix >> 23) & 0xFF
    if E == 0xFF:
        return sub(x, x), 0
    m = (ix & 0x7FFFFF) | 0x800000
    e = E - 150
    u = e - 2 + 32
    wi, sh = u >> 5, u & 31
    T = TWO_OVER_PI_WORDS

    def win(k):
        return (((T[k] << 32) | T[k + 1]) >> (32 - sh)) & 0xFFFFFFFF

    w0, w1, w2 = win(wi), win(wi + 1), win(wi + 2)
    p2, p1, p0 = m * w2, m * w1, m * w0
    limb0 = p2 & 0xFFFFFFFF
    b = p1 + (p2 >> 32)
    limb1 = b & 0xFFFFFFFF
    c = p0 + (b >> 32)
    ipart = (c >> 30) & 3
    frac64 = (((c & 0x3FFFFFFF) << 34) | (limb1 << 2) | (limb0 >> 30)) & M64
    q = (ipart + (frac64 >> 63)) & 3
    neg = frac64 >> 63
    a = ((1 << 64) - frac64) & M64 if neg else frac64
    r = f32(0.0)
    if a != 0:
        lz = 64 - a.bit_length()
        t = ((a << lz) & M64) >> 34
        hi = round_f32(t)
        lo = round_f32(t - int(float(hi)))
        scale = f32(2.0 ** (-30 - lz))
        rh, rl = mul(hi, scale), mul(lo, scale)
        r = fma(rh, PIO2[0], fma(rh, PIO2[1], mul(rl, PIO2[0])))
        if neg:
            r = f32(-r)
    if ix >> 31:
        r = -r
        q = (4 - q) & 3
    return f32(r), q


def sincos(x):
    r, q = reduce_pio2(x)
    z = mul(r, r)
    ps = fma(z, S[3], S[2])
    ps = fma(z, ps, S[1])
    ps = fma(z, ps, S[0])
    s = fma(mul(r, z), ps, r)
    pc = fma(z, CC[4], CC[3])
    pc = fma(z, pc, CC[2])
    pc = fma(z, pc, CC[1])
    pc = fma(z, pc, CC[0])
    c = fma(z, pc, f32(1.0))
    return [(s, c), (c, f32(-s)), (f32(-s), f32(-c)), (f32(-c), s)][q]


def jitter_hash(index, x, y):
    a = mul(i2f(index), f32(12.9898))
    a = add(a, mul(x, f32(78.233)))
    a = add(a, mul(y, f32(37.719)))
    s, _ = sincos(a)
    return fract(mul(s, f32(43758.5453)))


def sample(trail, W, H, px, py):
    x0, y0 = f2i(floor(px)), f2i(floor(py))
    if x0 < 0 or x0 >= W - 1 or y0 < 0 or y0 >= H - 1:
        return f32(0.0)
    dx, dy = sub(px, i2f(x0)), sub(py, i2f(y0))
    v00, v10 = trail[y0, x0], trail[y0, x0 + 1]
    v01, v11 = trail[y0 + 1, x0], trail[y0 + 1, x0 + 1]
    return mix(mix(v00, v10, dx), mix(v01, v11, dx), dy)


def agent_update(p, W, H, index, a, trail):
    x, y, angle, speed = (f32(v) for v in a)
    speed = clamp(speed, p["agent_speed_min"], p["agent_speed_max"])
    dist = p["agent_sensor_distance"]
    sc, cc = sincos(angle)
    if p.get("sensor_mode", 0) == 1:
        # rotated mode: (cos angle, sin angle) rotated by -/+ a
        sa, ca = sincos(p["agent_sensor_angle"])
        cca, sca = mul(cc, ca), mul(sc, ca)
        cl, sl = fma(sc, sa, cca), fma(f32(-cc), sa, sca)
        cr, sr = fma(f32(-sc), sa, cca), fma(cc, sa, sca)
    else:
        # compute.wgsl:75-90: cos/sin of the binary32 angles angle -/+ a
        sl, cl = sincos(sub(angle, p["agent_sensor_angle"]))
        sr, cr = sincos(add(angle, p["agent_sensor_angle"]))
    left = sample(trail, W, H, add(x, mul(dist, cl)), add(y, mul(dist, sl)))
    right = sample(trail, W, H, add(x, mul(dist, cr)), add(y, mul(dist, sr)))
    center = sample(trail, W, H, add(x, mul(dist, cc)), add(y, mul(dist, sc)))
    if center > left and center > right:
        pass
    elif left > right:
        diff = sub(sub(angle, TAU), angle)
        angle = add(angle, mul(fmin(p["agent_turn_speed"], f32(abs(diff))), sign(diff)))
    elif right > left:
        diff = sub(add(angle, TAU), angle)
        angle = add(angle, mul(fmin(p["agent_turn_speed"], f32(abs(diff))), sign(diff)))
    rv = jitter_hash(index, x, y)
    angle = add(angle, mul(sub(mul(rv, f32(2.0)), f32(1.0)), p["agent_jitter"]))
    angle = fmod(angle, TAU)
    if angle < 0:
        angle = add(angle, TAU)
    move = mul(speed, p["time_step"])
    sm, cm = sincos(angle)
    x = add(x, mul(move, cm))
    y = add(y, mul(move, sm))
    Wf, Hf = f32(W), f32(H)
    x = fmod(x, Wf)
    if x < 0:
        x = add(x, Wf)
    y = fmod(y, Hf)
    if y < 0:
        y = add(y, Hf)
    dx, dy = f2i(x), f2i(y)
    cell = dy * W + dx if (0 <= dx < W and 0 <= dy < H) else -1
    return (x, y, angle, speed), cell


def fold(t, k, dep):
    t = f32(t)
    for _ in range(int(k)):
        nt = clamp(add(t, dep), f32(0.0), f32(1.0))
        if np.array(nt).view(np.uint32) == np.array(t).view(np.uint32):
            break
        t = nt
    return t


def exp_neg(a):
    y = a / 1024.0
    term, tot = 1.0, 1.0
    for k in range(1, 19):
        term = term * (-y) / float(k)
        tot = tot + term
    for _ in range(10):
        tot = tot * tot
    return tot


def gauss_weights(radius, sigma, max_radius=8):
    R = min(max(f2i(f32(radius)), 0), max_radius)
    s2 = 2.0 * float(f32(sigma)) * float(f32(sigma))
    vals = [exp_neg(float(i * i) / s2) for i in range(-R, R + 1)]
    tot = 0.0
    for v in vals:
        tot = tot + v
    return R, [f32(v / tot) for v in vals]


def trail_pass(p, W, H, trail, counts):
    d = np.empty((H, W), np.float32)
    dk = mul(p["decay_factor"], f32(0.001))
    rate = clamp(p["diffusion_rate"], f32(0.0), f32(1.0))
    for yy in range(H):
        for xx in range(W):
            v = fold(trail[yy, xx], counts[yy, xx], p["pheromone_deposition_amount"])
            v = mul(v, p["decay_factor"]) if p["decay_mode"] == 1 else fmax(sub(v, dk), f32(0.0))
            d[yy, xx] = v
    out = np.empty((H, W), np.float32)
    if p["blur_mode"] == 1:
        R, w = gauss_weights(p["blur_radius"], p["blur_sigma"])
        h = np.empty((H, W), np.float32)
        for yy in range(H):
            for xx in range(W):
                acc = f32(0.0)
                for i in range(-R, R + 1):
                    acc = fma(w[i + R], d[yy, (xx + i) % W], acc)
                h[yy, xx] = acc
        for yy in range(H):
            for xx in range(W):
                acc = f32(0.0)
                for j in range(-R, R + 1):
                    acc = fma(w[j + R], h[(yy + j) % H, xx], acc)
                out[yy, xx] = mix(d[yy, xx], acc, rate)
    else:
        for yy in range(H):
            for xx in range(W):
                s = f32(0.0)
                for dy in (-1, 0, 1):
                    for dx in (-1, 0, 1):
                        s = add(s, d[(yy + dy + H) % H, (xx + dx + W) % W])
                out[yy, xx] = mix(d[yy, xx], div(s, f32(9.0)), rate)
    return out


def step(p, W, H, agents, trail):
    """One step; returns (agents, trail, counts)."""
    n = agents.shape[0]
    na = np.empty_like(agents)
    counts = np.zeros((H, W), np.uint32)
    for i in range(n):
        vals, cell = agent_update(p, W, H, i, agents[i], trail)
        na[i] = vals
        if cell >= 0:
            counts[cell // W, cell % W] += 1
    return na, trail_pass(p, W, H, trail, counts), counts
