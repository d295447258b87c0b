/*
 * slime_math.h - deterministic binary32 builtins shared by the CUDA kernels and
 * the CPU oracle.
 *
 * The reference shader (src/compute.wgsl) uses the WGSL builtins sin, cos,
 * floor, fract, mix, clamp, min, abs, sign, i32(f32) and the f32 `%`
 * operator.  WGSL leaves the precision of sin/cos implementation-defined and
 * does not forbid fusing a*b+c, so the reference is not bit-reproducible even
 * between two GPUs.  This header pins one definition of every builtin that both
 * sides of a parity test evaluate identically:
 *
 *   - every + - * / is an explicitly rounded IEEE binary32 operation
 *     (__fadd_rn & co. on the device; plain operators on the host, which must
 *     be compiled with -ffp-contract=off so nothing is fused);
 *   - fused multiply-adds appear only where written as slm_fma, which is
 *     correctly rounded on both sides (fmaf / __fmaf_rn);
 *   - sin and cos are computed here from published methods:
 *       * |x| < 4096: Cody-Waite reduction by pi/2 split into three binary32
 *         parts (W. J. Cody and W. Waite, "Software Manual for the Elementary
 *         Functions", 1980), evaluated with fused multiply-adds, the nearest
 *         multiple found by the 1.5 * 2^23 rounding addition;
 *       * otherwise: Payne-Hanek reduction (M. Payne and R. Hanek, "Radian
 *         reduction for trigonometric functions", SIGNUM Newsletter 18(1),
 *         1983) with a 96-bit window of 2/pi and 32x32->64 integer products;
 *         below 2^44 the window comes from four fixed words of 2/pi by funnel
 *         shifts instead of table reads (same bits, fewer instructions);
 *       * the reduced argument |r| <= pi/4 is fed to the Taylor polynomials of
 *         sin (to r^9) and cos (to r^10) in Horner form.
 *     The accuracy is a few ulp; what matters for parity is that the host and
 *     the device produce the same bits.
 *
 * All constants come from include/gen_slime_math_constants.py (mpmath, 400 bits).
 */
#ifndef SLIME_MATH_H
#define SLIME_MATH_H

#include <stdint.h>
#include <string.h>
#include <math.h>

#if defined(__CUDACC__)
#define SLM_FN static __host__ __device__ __forceinline__
#else
#define SLM_FN static inline
#endif

/* BEGIN GENERATED CONSTANTS (include/gen_slime_math_constants.py) */
#define SLM_TWO_OVER_PI_F (0x1.45f3060000000p-1f)
#define SLM_PIO2_1 (0x1.921fb60000000p+0f)
#define SLM_PIO2_2 (-0x1.777a5c0000000p-25f)
#define SLM_PIO2_3 (-0x1.ee59da0000000p-50f)
#define SLM_S1 (-0x1.5555560000000p-3f)
#define SLM_S2 (0x1.1111120000000p-7f)
#define SLM_S3 (-0x1.a01a020000000p-13f)
#define SLM_S4 (0x1.71de3a0000000p-19f)
#define SLM_C1 (-0x1.0000000000000p-1f)
#define SLM_C2 (0x1.5555560000000p-5f)
#define SLM_C3 (-0x1.6c16c20000000p-10f)
#define SLM_C4 (0x1.a01a020000000p-16f)
#define SLM_C5 (-0x1.27e4fc0000000p-22f)
#define SLM_TWO_OVER_PI_NWORDS 10
#define SLM_TWO_OVER_PI_INIT { 0x00000000u, 0xa2f9836eu, 0x4e441529u, 0xfc2757d1u, 0xf534ddc0u, 0xdb629599u, 0x3c439041u, 0xfe5163abu, 0xdebbc561u, 0xb7246e3au }
#define SLM_PH_WIN_INIT { 0x000517ccu, 0x1b727220u, 0xa94fe13au, 0xbe8fa9a6u }
/* END GENERATED CONSTANTS */

/* Word 0 is zero: the bits of 2/pi "before" the binary point.  Word i >= 1
 * holds bits 32(i-1)+1 .. 32i of the fraction, most significant first. */
#if defined(__CUDACC__)
static __device__ const uint32_t slm_two_over_pi_dev[SLM_TWO_OVER_PI_NWORDS] = SLM_TWO_OVER_PI_INIT;
#endif
static const uint32_t slm_two_over_pi_host[SLM_TWO_OVER_PI_NWORDS] = SLM_TWO_OVER_PI_INIT;

/* WGSL's f32 constants, rounded to binary32 exactly as the shader's
 * abstract-float constant expressions are (compute.wgsl:4, :55, :121). */
#define SLM_WGSL_TAU (6.28318530718f)           /* TAU, compute.wgsl:4 */
#define SLM_WGSL_TWO_PI (6.28318530718f)        /* 2.0 * 3.14159265359, compute.wgsl:121 */
#define SLM_WGSL_TIME_STEP (0.016f)             /* TIME_STEP, compute.wgsl:55 */

/* ---------------------------------------------------------------- basic ops */
SLM_FN float slm_add(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
SLM_FN float slm_sub(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
SLM_FN float slm_mul(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
SLM_FN float slm_div(float a, float b) {
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
SLM_FN float slm_fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}

SLM_FN uint32_t slm_f2u_bits(float x) { uint32_t u; memcpy(&u, &x, 4); return u; }
SLM_FN float slm_u2f_bits(uint32_t u) { float x; memcpy(&x, &u, 4); return x; }
SLM_FN int slm_isnan(float x) { return x != x; }

/* WGSL min/max, pinned as IEEE 754-2019 minimumNumber/maximumNumber: a NaN
 * operand is ignored, and -0 orders below +0.  The device's fminf/fmaxf
 * (min.f32/max.f32) implement exactly this; the host spells it out. */
SLM_FN float slm_min(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fminf(a, b);
#else
    if (slm_isnan(a)) return b;
    if (slm_isnan(b)) return a;
    if (a == b) return (slm_f2u_bits(a) >> 31) ? a : b; /* -0 before +0 */
    return (b < a) ? b : a;
#endif
}
SLM_FN float slm_max(float a, float b) {
#if defined(__CUDA_ARCH__)
    return fmaxf(a, b);
#else
    if (slm_isnan(a)) return b;
    if (slm_isnan(b)) return a;
    if (a == b) return (slm_f2u_bits(a) >> 31) ? b : a; /* +0 after -0 */
    return (b > a) ? b : a;
#endif
}
/* WGSL clamp(e, low, high) = min(max(e, low), high). */
SLM_FN float slm_clamp(float e, float lo, float hi) { return slm_min(slm_max(e, lo), hi); }
/* WGSL sign: 1, -1 or 0 (NaN maps to 0). */
SLM_FN float slm_sign(float x) { return (x > 0.0f) ? 1.0f : ((x < 0.0f) ? -1.0f : 0.0f); }
SLM_FN float slm_abs(float x) { return slm_u2f_bits(slm_f2u_bits(x) & 0x7fffffffu); }
SLM_FN float slm_floor(float x) { return floorf(x); }
/* WGSL fract(e) = e - floor(e). */
SLM_FN float slm_fract(float x) { return slm_sub(x, slm_floor(x)); }
/* WGSL mix(e1, e2, e3) = e1 * (1 - e3) + e2 * e3, unfused. */
SLM_FN float slm_mix(float a, float b, float t) {
    return slm_add(slm_mul(a, slm_sub(1.0f, t)), slm_mul(b, t));
}
/* The f32 `%` operator: remainder with the sign of the dividend.  fmodf is
 * exact on every conforming implementation, so host and device agree. */
SLM_FN float slm_fmod(float x, float y) {
    /* For y > 0 and |x| < 2y the remainder is one of x, x - y, x + y, each
     * exact (Sterbenz), which is what every exact fmodf returns; the
     * remainder of -y is -0.  Written as selects; everything else goes to
     * fmodf. */
    float y2 = slm_add(y, y);
    int in0 = slm_abs(x) < y;
    int in1 = (x >= y) && (x < y2);
    int in2 = (x <= -y) && (x > -y2);
    if (!(y > 0.0f) || !(in0 || in1 || in2)) return fmodf(x, y);
    float r1 = slm_sub(x, y);
    float r2 = slm_add(x, y);
    r2 = (r2 == 0.0f) ? -0.0f : r2;
    return in0 ? x : (in1 ? r1 : r2);
}

/* The shader's toroidal wrap, `v = v % n; if (v < 0.0) { v = v + n; }`
 * (compute.wgsl:121-122, :130-133), for n > 0.  Values within one period of
 * [0, n) take the exact short paths; -n and -0 give -0 as the remainder does. */
SLM_FN float slm_wrap(float v, float n) {
    if (v >= 0.0f && v < n) return v;
    if (v >= n && v < slm_add(n, n)) return slm_sub(v, n);
    if (v < 0.0f && v > -n) return slm_add(v, n);
    float r = slm_fmod(v, n);
    if (r < 0.0f) r = slm_add(r, n);
    return r;
}

/* WGSL i32(f32): truncate toward zero, saturate to the i32 range, NaN -> 0.
 * (Matches the device's cvt.rzi.sat; spelled out so the host has no UB.) */
SLM_FN int32_t slm_f2i(float x) {
#if defined(__CUDA_ARCH__)
    return __float2int_rz(x); /* cvt.rzi.s32.f32: truncates, saturates, NaN -> 0 */
#else
    if (slm_isnan(x)) return 0;
    if (x >= 2147483648.0f) return 2147483647;
    if (x <= -2147483648.0f) return (int32_t)(-2147483647 - 1);
    return (int32_t)x;
#endif
}
/* WGSL f32(i32): round to nearest even. */
SLM_FN float slm_i2f(int32_t i) { return (float)i; }

/* ---------------------------------------------------------- sin and cos */
/* Leading zero bits of a nonzero 64-bit value. */
SLM_FN int slm_clz64(uint64_t a) {
#if defined(__CUDA_ARCH__)
    return __clzll((long long)a);
#else
    return __builtin_clzll(a);
#endif
}

/* (hi:lo) << d, upper 32 bits, for 0 <= d <= 31. */
SLM_FN uint32_t slm_funnel_l(uint32_t lo, uint32_t hi, int d) {
#if defined(__CUDA_ARCH__)
    return __funnelshift_l(lo, hi, (unsigned)d);
#else
    return d == 0 ? hi : ((hi << d) | (lo >> (32 - d)));
#endif
}

/* Second half of the Payne-Hanek reduction: from the mantissa m of |x|
 * (2^23 <= m < 2^24), the 96 bits w0:w1:w2 of 2/pi that follow the bits
 * dropped as multiples of 4, and the sign of x, the reduced argument and the
 * quadrant. */
SLM_FN void slm_ph_finish(uint32_t m, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t sign, float* r_out,
                          int* q_out) {
    /* Q = m * (w0:w1:w2), a 120-bit integer; |x| * 2/pi = Q * 2^-94 (mod 4). */
    uint64_t p2 = (uint64_t)m * w2;
    uint64_t p1 = (uint64_t)m * w1;
    uint64_t p0 = (uint64_t)m * w0;
    uint32_t limb0 = (uint32_t)p2;
    uint64_t b = p1 + (p2 >> 32);
    uint32_t limb1 = (uint32_t)b;
    uint64_t c = p0 + (b >> 32); /* bits 64.. of Q */
    uint32_t ipart = (uint32_t)(c >> 30) & 3u;
    uint64_t frac64 = ((c & 0x3fffffffull) << 34) | ((uint64_t)limb1 << 2) | (limb0 >> 30);
    /* Round to the nearest quadrant: a fraction >= 1/2 becomes negative. */
    uint32_t q = (ipart + (uint32_t)(frac64 >> 63)) & 3u;
    int neg = (int)(frac64 >> 63);
    uint64_t a = neg ? (0ull - frac64) : frac64; /* |fraction| * 2^64 */
    float r = 0.0f;
    if (a != 0) {
        /* 30 leading bits as a 24-bit head plus an exact correction, both
         * scaled by a power of two built in the exponent field: only 32-bit
         * conversions. */
        int lz = slm_clz64(a);
        uint32_t t = (uint32_t)((a << lz) >> 34); /* in [2^29, 2^30) */
        float hi = (float)(int32_t)t;
        float lo = (float)((int32_t)t - (int32_t)hi);
        float scale = slm_u2f_bits((uint32_t)(127 - 30 - lz) << 23); /* 2^(-30-lz) */
        float rh = slm_mul(hi, scale);
        float rl = slm_mul(lo, scale);
        r = slm_fma(rh, SLM_PIO2_1, slm_fma(rh, SLM_PIO2_2, slm_mul(rl, SLM_PIO2_1)));
        if (neg) r = -r;
    }
    if (sign) {
        r = -r;
        q = (4u - q) & 3u;
    }
    *r_out = r;
    *q_out = (int)q;
}

/* Payne-Hanek for finite |x| >= 4096, window read from the table of 2/pi. */
SLM_FN void slm_reduce_pio2_ph(float x, float* r_out, int* q_out) {
    uint32_t ix = slm_f2u_bits(x);
    uint32_t E = (ix >> 23) & 0xffu;
    /* |x| = m * 2^e with 2^23 <= m < 2^24 and e >= -11. */
    uint32_t m = (ix & 0x7fffffu) | 0x800000u;
    int e = (int)E - 150;
    /* Bits of 2/pi with index <= s = e - 2 contribute multiples of 4 to
     * |x| * 2/pi and are dropped; take the 96 bits s+1 .. s+96. */
    int u = e - 2 + 32; /* table position of bit s, >= 19 */
#if defined(__CUDA_ARCH__)
    const uint32_t* T = slm_two_over_pi_dev;
#else
    const uint32_t* T = slm_two_over_pi_host;
#endif
    int wi = u >> 5;
    int sh = u & 31;
    uint32_t w0 = (uint32_t)(((((uint64_t)T[wi]) << 32) | T[wi + 1]) >> (32 - sh));
    uint32_t w1 = (uint32_t)(((((uint64_t)T[wi + 1]) << 32) | T[wi + 2]) >> (32 - sh));
    uint32_t w2 = (uint32_t)(((((uint64_t)T[wi + 2]) << 32) | T[wi + 3]) >> (32 - sh));
    slm_ph_finish(m, w0, w1, w2, ix >> 31, r_out, q_out);
}

/* The same for 4096 <= |x| < 2^44 (biased exponent 139..170): there the
 * window starts at table position u = e + 30 in [19, 50], so its 96 bits lie
 * inside the fixed 128 bits 19..146 of the table (SLM_PH_WIN_INIT), and each
 * window word is one funnel shift of two of them by u - 19 <= 31.  Equal to
 * slm_reduce_pio2_ph bit for bit on that range (the oracle's self-test
 * compares all 2^29 inputs). */
SLM_FN void slm_reduce_pio2_win(float x, float* r_out, int* q_out) {
    const uint32_t K[4] = SLM_PH_WIN_INIT;
    uint32_t ix = slm_f2u_bits(x);
    uint32_t E = (ix >> 23) & 0xffu;
    uint32_t m = (ix & 0x7fffffu) | 0x800000u;
    int d = (int)E - 139;
    uint32_t w0 = slm_funnel_l(K[1], K[0], d);
    uint32_t w1 = slm_funnel_l(K[2], K[1], d);
    uint32_t w2 = slm_funnel_l(K[3], K[2], d);
    slm_ph_finish(m, w0, w1, w2, ix >> 31, r_out, q_out);
}

/* Reduce x to r in about [-pi/4, pi/4] and quadrant q in 0..3 with
 * x = (4k + q) * pi/2 + r. */
SLM_FN void slm_reduce_pio2(float x, float* r_out, int* q_out) {
    if (slm_abs(x) < 4096.0f) {
        /* Cody-Waite.  j = rint(x * 2/pi) by adding and removing 1.5 * 2^23
         * (exact round-to-nearest-even for |j| < 2^22); the low bits of the
         * biased sum are j mod 4.  SLM_PIO2_1 has its last bit at 2^-23, so
         * the first fma is exact for every |x| < 4096; the two later parts
         * restore the lost bits. */
        float biased = slm_add(slm_mul(x, SLM_TWO_OVER_PI_F), 12582912.0f);
        float j = slm_sub(biased, 12582912.0f);
        float r = slm_fma(-j, SLM_PIO2_1, x);
        r = slm_fma(-j, SLM_PIO2_2, r);
        r = slm_fma(-j, SLM_PIO2_3, r);
        *r_out = r;
        *q_out = (int)(slm_f2u_bits(biased) & 3u);
        return;
    }
    uint32_t E = (slm_f2u_bits(x) >> 23) & 0xffu;
    if (E == 0xffu) { /* inf or NaN */
        *r_out = slm_sub(x, x);
        *q_out = 0;
        return;
    }
    if (E <= 170u)
        slm_reduce_pio2_win(x, r_out, q_out);
    else
        slm_reduce_pio2_ph(x, r_out, q_out);
}

SLM_FN void slm_sincos(float x, float* s_out, float* c_out) {
    float r;
    int q;
    slm_reduce_pio2(x, &r, &q);
    float z = slm_mul(r, r);
    float ps = slm_fma(z, SLM_S4, SLM_S3);
    ps = slm_fma(z, ps, SLM_S2);
    ps = slm_fma(z, ps, SLM_S1);
    float s = slm_fma(slm_mul(r, z), ps, r);
    float pc = slm_fma(z, SLM_C5, SLM_C4);
    pc = slm_fma(z, pc, SLM_C3);
    pc = slm_fma(z, pc, SLM_C2);
    pc = slm_fma(z, pc, SLM_C1);
    float c = slm_fma(z, pc, 1.0f);
    /* quadrant q: (sin, cos) = (s, c), (c, -s), (-s, -c), (-c, s) */
    float a = (q & 1) ? c : s;
    float bb = (q & 1) ? s : c;
    *s_out = (q & 2) ? -a : a;
    *c_out = ((q + 1) & 2) ? -bb : bb;
}

SLM_FN float slm_sin(float x) { float s, c; slm_sincos(x, &s, &c); return s; }
SLM_FN float slm_cos(float x) { float s, c; slm_sincos(x, &s, &c); return c; }

/* ---------------------------------------------- composite shader pieces */
/* How many invocations of the reference's agent dispatch update agent
 * `index` of `n` (compute.wgsl:60 with src/main.rs:1174-1178): wx x wy
 * workgroups of 64, wx = min(ceil(n / 64), 65535), wy = ceil(ceil(n / 64) / wx);
 * invocation (gx, gy), gx < 64 wx, gy < wy, updates agent gx + 65535 gy, so
 * agent i is visited once for each gy < wy with gy 65535 <= i < gy 65535 + 64 wx.
 * Every agent once for n <= 4,194,240; for n < 2^31 the shader's u32 index
 * neither wraps nor turns negative as an i32. */
/* The dispatch's rows wy and row span 64 wx for n agents, 0 < n < 2^31. */
SLM_FN void slm_dispatch_geometry(uint64_t n, uint32_t* wy, uint32_t* span) {
    const uint64_t groups = (n + 63) / 64;
    const uint64_t wx = groups < 65535 ? groups : 65535;
    *wy = (uint32_t)((groups + wx - 1) / wx);
    *span = (uint32_t)(64 * wx);
}
/* Visits of agent `index` < n from that geometry (32-bit arithmetic). */
SLM_FN uint32_t slm_dispatch_visits_in(uint32_t index, uint32_t wy, uint32_t span) {
    const uint32_t hi = index / 65535u < wy - 1u ? index / 65535u : wy - 1u; /* gy 65535 <= index */
    const uint32_t lo = index >= span ? (index - span) / 65535u + 1u : 0u;  /* index < gy 65535 + span */
    return hi >= lo ? hi - lo + 1u : 0u;
}
SLM_FN uint32_t slm_dispatch_visits(uint64_t n, uint64_t index) {
    if (index >= n || n >= (1ull << 31)) return 0;
    uint32_t wy, span;
    slm_dispatch_geometry(n, &wy, &span);
    return slm_dispatch_visits_in((uint32_t)index, wy, span);
}

/* Sensor directions of compute.wgsl:75-90 as the shader writes them: the
 * sensor angles angle - a and angle + a are binary32 differences and sums
 * (:75-76), and each of the three directions is slm_sincos of its own angle. */
SLM_FN void slm_sensor_dirs_shader(float angle, float a, float* cl, float* sl, float* cc, float* sc, float* cr,
                                   float* sr) {
    slm_sincos(slm_sub(angle, a), sl, cl);
    slm_sincos(slm_add(angle, a), sr, cr);
    slm_sincos(angle, sc, cc);
}

/* The rotated form (SLIME_SENSOR_ROTATED): the centre direction is
 * slm_sincos(angle); the side directions are that vector rotated by -a and +a
 * with (sin a, cos a) = slm_sincos(sensor_angle), a fixed sequence of
 * binary32 products and fused multiply-adds.  Within a few 1e-8 of cos/sin of
 * the rounded angle -/+ a, but not equal to it: near-ties of the turn
 * decision can go the other way than the shader's. */
SLM_FN void slm_sensor_dirs(float angle, float sa, float ca, float* cl, float* sl, float* cc, float* sc, float* cr,
                            float* sr) {
    float s, c;
    slm_sincos(angle, &s, &c);
    *cc = c;
    *sc = s;
    /* rotate (c, s) by -a: (c ca + s sa, s ca - c sa); by +a: (c ca - s sa, s ca + c sa) */
    float cca = slm_mul(c, ca), sca = slm_mul(s, ca);
    *cl = slm_fma(s, sa, cca);
    *sl = slm_fma(-c, sa, sca);
    *cr = slm_fma(-s, sa, cca);
    *sr = slm_fma(c, sa, sca);
}

/* The shader's per-agent jitter hash (compute.wgsl:117):
 *   fract(sin(f32(agent_index) * 12.9898 + x * 78.233 + y * 37.719) * 43758.5453)
 * evaluated left to right, unfused. */
SLM_FN float slm_jitter_hash(int32_t agent_index, float x, float y) {
    float a = slm_mul(slm_i2f(agent_index), 12.9898f);
    a = slm_add(a, slm_mul(x, 78.233f));
    a = slm_add(a, slm_mul(y, 37.719f));
    return slm_fract(slm_mul(slm_sin(a), 43758.5453f));
}

/* Counter-based generator for seeded initial agent states: SplitMix64
 * (G. Steele, D. Lea, C. Flood, "Fast splittable pseudorandom number
 * generators", OOPSLA 2014) of seed, agent index and field. */
SLM_FN uint64_t slm_splitmix64(uint64_t z) {
    z += 0x9e3779b97f4a7c15ull;
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
/* Uniform binary32 in [0, 1) with 24 random bits. */
SLM_FN float slm_uniform01(uint64_t seed, uint64_t index, uint32_t field) {
    uint64_t h = slm_splitmix64(seed ^ slm_splitmix64(index * 4ull + field));
    return (float)(h >> 40) * 0x1.0p-24f;
}

/* ------------------------------------------ Gaussian blur weights (host) */
/* exp(-a) for a >= 0 in binary64 from + - * / only (Taylor series of
 * exp(-a/1024), then ten squarings), so every host computes the same bits. */
static inline double slm_exp_neg_host(double a) {
    double y = a / 1024.0;
    double term = 1.0, sum = 1.0;
    for (int k = 1; k <= 18; k++) {
        term = term * (-y) / (double)k;
        sum = sum + term;
    }
    for (int i = 0; i < 10; i++) sum = sum * sum;
    return sum;
}

/* Number of taps on each side of the Gaussian blur: i32(blur_radius)
 * clamped to [0, max_radius]. */
static inline int slm_gauss_radius(float blur_radius, int max_radius) {
    int r = slm_f2i(blur_radius);
    if (r < 0) r = 0;
    if (r > max_radius) r = max_radius;
    return r;
}

/* Normalised 1-D weights w[0..2R] of exp(-i^2 / (2 sigma^2)), i = -R..R,
 * computed in binary64 and rounded once to binary32.  Returns 0, or -1 if
 * sigma is not a positive finite number. */
static inline int slm_gauss_weights(int radius, float sigma, float* w) {
    if (!(sigma > 0.0f) || !(sigma < 3.0e38f)) return -1;
    double s2 = 2.0 * (double)sigma * (double)sigma;
    double tmp[2 * 64 + 1];
    double total = 0.0;
    for (int i = -radius; i <= radius; i++) {
        double v = slm_exp_neg_host((double)(i * i) / s2);
        tmp[i + radius] = v;
        total = total + v;
    }
    for (int i = 0; i <= 2 * radius; i++) w[i] = (float)(tmp[i] / total);
    return 0;
}

#endif /* SLIME_MATH_H */
