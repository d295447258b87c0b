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
/* Rarely taken paths (huge or non-finite arguments, remainders outside one
 * period) are compiled once, out of line, so that the kernels' hot loops stay
 * small enough for the instruction cache. */
#define SLM_COLD_FN static __host__ __device__ __noinline__
#else
#define SLM_FN static inline
#define SLM_COLD_FN static
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
/* |x|: the sign bit cleared.  On the device abs.f32, which folds into the
 * instruction that uses it as an operand modifier; its result for a NaN is
 * some NaN, and every use here (compares, minimumNumber) treats all NaNs
 * alike. */
SLM_FN float slm_abs(float x) {
#if defined(__CUDA_ARCH__)
    return fabsf(x);
#else
    return slm_u2f_bits(slm_f2u_bits(x) & 0x7fffffffu);
#endif
}
SLM_FN float slm_floor(float x) { return floorf(x); }
/* WGSL fract(e) = e - floor(e). */
SLM_FN float slm_fract(float x) { return slm_sub(x, slm_floor(x)); }
/* WGSL mix(e1, e2, e3) = e1 * (1 - e3) + e2 * e3, unfused. */
SLM_FN float slm_mix(float a, float b, float t) {
    return slm_add(slm_mul(a, slm_sub(1.0f, t)), slm_mul(b, t));
}
/* fmodf, out of line: exact on every conforming implementation. */
SLM_COLD_FN float slm_fmod_exact(float x, float y) { return fmodf(x, y); }

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
    if (!(y > 0.0f) || !(in0 || in1 || in2)) return slm_fmod_exact(x, y);
    float r1 = slm_sub(x, y);
    float r2 = slm_add(x, y);
    r2 = (r2 == 0.0f) ? -0.0f : r2;
    return in0 ? x : (in1 ? r1 : r2);
}

/* The general case of slm_wrap, out of line (values more than a period
 * outside [0, n), -n, -0, NaN, infinities, n <= 0). */
SLM_COLD_FN float slm_wrap_general(float v, float n) {
    float r = slm_fmod(v, n);
    if (r < 0.0f) r = slm_add(r, n);
    return r;
}

/* The shader's toroidal wrap, `v = v % n; if (v < 0.0) { v = v + n; }`
 * (compute.wgsl:121-122, :130-133), for n > 0.  Values within one period of
 * [0, n) take the exact short paths; -n and -0 give -0 as the remainder does. */
SLM_FN float slm_wrap(float v, float n) {
    if (v >= 0.0f && v < n) return v;
    if (v >= n && v < slm_add(n, n)) return slm_sub(v, n);
    if (v < 0.0f && v > -n) return slm_add(v, n);
    return slm_wrap_general(v, n);
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

/* High 32 bits of a 32x32-bit product. */
SLM_FN uint32_t slm_umulhi(uint32_t a, uint32_t b) {
#if defined(__CUDA_ARCH__)
    return __umulhi(a, b);
#else
    return (uint32_t)(((uint64_t)a * b) >> 32);
#endif
}
/* Leading zero bits of a nonzero 32-bit value. */
SLM_FN int slm_clz32(uint32_t a) {
#if defined(__CUDA_ARCH__)
    return __clz((int)a);
#else
    return __builtin_clz(a);
#endif
}

/* |r| = |fraction| * pi/2 from the fraction's magnitude a = a_hi:a_lo
 * (times 2^64, a_hi nonzero): its 30 leading bits as a 24-bit head plus an
 * exact correction, both scaled by a power of two built in the exponent
 * field, so only 32-bit conversions are needed. */
SLM_FN float slm_ph_abs_r(uint32_t a_lo, uint32_t a_hi) {
    const int lz = slm_clz32(a_hi);
    const uint32_t t = slm_funnel_l(a_lo, a_hi, lz) >> 2; /* in [2^29, 2^30) */
    float hi = (float)(int32_t)t;
    float lo = (float)((int32_t)t - (int32_t)hi);
    float scale = slm_u2f_bits((uint32_t)(127 - 30 - lz) << 23); /* 2^(-30-lz) */
    float rh = slm_mul(hi, scale);
    float rl = slm_mul(lo, scale);
    return slm_fma(rh, SLM_PIO2_1, slm_fma(rh, SLM_PIO2_2, slm_mul(rl, SLM_PIO2_1)));
}
/* The same for a_hi == 0 (|fraction| < 2^-32, or zero), out of line. */
SLM_COLD_FN float slm_ph_abs_r_small(uint32_t a_lo) {
    if (a_lo == 0u) return 0.0f;
    const int lzh = slm_clz32(a_lo);
    const int lz = lzh + 32;
    const uint32_t t = (a_lo << lzh) >> 2;
    float hi = (float)(int32_t)t;
    float lo = (float)((int32_t)t - (int32_t)hi);
    float scale = slm_u2f_bits((uint32_t)(127 - 30 - lz) << 23);
    float rh = slm_mul(hi, scale);
    float rl = slm_mul(lo, scale);
    return slm_fma(rh, SLM_PIO2_1, slm_fma(rh, SLM_PIO2_2, slm_mul(rl, SLM_PIO2_1)));
}

/* Second half of the Payne-Hanek reduction: from the mantissa m of |x|
 * (2^23 <= m < 2^24), the 96 bits w0:w1:w2 of 2/pi that follow the bits
 * dropped as multiples of 4, and the sign of x, the reduced argument and the
 * quadrant.  Written in 32-bit words (the products' low and high halves,
 * add-with-carry, funnel shifts, one 32-bit leading-zero count); the same bits
 * as the 64-bit statement slm_ph_finish_u64 below for every input, which the
 * oracle's self-test checks over every binary32 with |x| >= 4096. */
SLM_FN void slm_ph_finish(uint32_t m, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t sign, float* r_out,
                          int* q_out) {
    /* Q = m * (w0:w1:w2), a 120-bit integer; |x| * 2/pi = Q * 2^-94 (mod 4).
     * Its low word is limb0, then limb1, then c_lo (bits 64..95); the bits
     * above do not matter (multiples of 4 after the scaling). */
    const uint32_t limb0 = m * w2;
    const uint32_t p2hi = slm_umulhi(m, w2);
    const uint32_t p1lo = m * w1;
    const uint32_t limb1 = p1lo + p2hi;
    const uint32_t b_hi = slm_umulhi(m, w1) + (limb1 < p1lo ? 1u : 0u);
    const uint32_t c_lo = m * w0 + b_hi;
    const uint32_t ipart = c_lo >> 30;
    /* the 64-bit fraction (bits 29..0 of c_lo, limb1, top 2 bits of limb0) */
    const uint32_t f_hi = slm_funnel_l(limb1, c_lo, 2);
    const uint32_t f_lo = slm_funnel_l(limb0, limb1, 2);
    /* Round to the nearest quadrant: a fraction >= 1/2 becomes negative. */
    const uint32_t neg = f_hi >> 31;
    uint32_t q = (ipart + neg) & 3u;
    const uint32_t mask = 0u - neg;
    const uint32_t a_lo = (f_lo ^ mask) + neg;
    const uint32_t a_hi = (f_hi ^ mask) + (a_lo < neg ? 1u : 0u); /* |fraction| * 2^64 */
    /* |r| from |fraction|; a fraction below 2^-32 (or zero) out of line */
    const float r_abs = a_hi != 0u ? slm_ph_abs_r(a_lo, a_hi) : slm_ph_abs_r_small(a_lo);
    /* r takes the sign of the fraction times that of x (bit 31 of f_hi and of
     * x); the quadrant of -x is -q (mod 4) */
    *r_out = slm_u2f_bits(slm_f2u_bits(r_abs) ^ ((f_hi ^ (sign << 31)) & 0x80000000u));
    const uint32_t smask = 0u - sign;
    *q_out = (int)(((q ^ smask) - smask) & 3u);
}

/* The same in 64-bit integer arithmetic (the statement slm_ph_finish was
 * derived from; kept for the self-test). */
SLM_FN void slm_ph_finish_u64(uint32_t m, uint32_t w0, uint32_t w1, uint32_t w2, uint32_t sign, float* r_out,
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

/* The mantissa of finite |x| >= 4096 and the 96-bit window of 2/pi that
 * slm_reduce_pio2_ph multiplies it by, from the table. */
SLM_FN void slm_ph_window_table(float x, uint32_t* m_out, uint32_t* w) {
    uint32_t ix = slm_f2u_bits(x);
    uint32_t E = (ix >> 23) & 0xffu;
    int u = (int)E - 150 - 2 + 32;
#if defined(__CUDA_ARCH__)
    const uint32_t* T = slm_two_over_pi_dev;
#else
    const uint32_t* T = slm_two_over_pi_host;
#endif
    int wi = u >> 5;
    int sh = u & 31;
    for (int k = 0; k < 3; k++)
        w[k] = (uint32_t)(((((uint64_t)T[wi + k]) << 32) | T[wi + k + 1]) >> (32 - sh));
    *m_out = (ix & 0x7fffffu) | 0x800000u;
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

/* Reduced argument and quadrant. */
typedef struct SlmRQ {
    float r;
    int q;
} SlmRQ;

/* Cody-Waite for |x| < 4096.  j = rint(x * 2/pi) by adding and removing
 * 1.5 * 2^23 (exact round-to-nearest-even for |j| < 2^22); the low bits of
 * the biased sum are j mod 4.  SLM_PIO2_1 has its last bit at 2^-23, so the
 * first fma is exact for every |x| < 4096; the two later parts restore the
 * lost bits. */
SLM_FN SlmRQ slm_reduce_pio2_cw(float x) {
    float biased = slm_add(slm_mul(x, SLM_TWO_OVER_PI_F), 12582912.0f);
    float j = slm_sub(biased, 12582912.0f);
    float r = slm_fma(-j, SLM_PIO2_1, x);
    r = slm_fma(-j, SLM_PIO2_2, r);
    r = slm_fma(-j, SLM_PIO2_3, r);
    SlmRQ o;
    o.r = r;
    o.q = (int)(slm_f2u_bits(biased) & 3u);
    return o;
}

/* |x| >= 4096, inf or NaN. */
SLM_FN SlmRQ slm_reduce_pio2_large(float x) {
    SlmRQ o;
    uint32_t E = (slm_f2u_bits(x) >> 23) & 0xffu;
    if (E == 0xffu) { /* inf or NaN */
        o.r = slm_sub(x, x);
        o.q = 0;
    } else if (E <= 170u) {
        slm_reduce_pio2_win(x, &o.r, &o.q);
    } else {
        slm_reduce_pio2_ph(x, &o.r, &o.q);
    }
    return o;
}
SLM_COLD_FN SlmRQ slm_reduce_pio2_large_cold(float x) { return slm_reduce_pio2_large(x); }
SLM_COLD_FN SlmRQ slm_reduce_pio2_cw_cold(float x) { return slm_reduce_pio2_cw(x); }

/* Reduce x to r in about [-pi/4, pi/4] and quadrant q in 0..3 with
 * x = (4k + q) * pi/2 + r: Cody-Waite inline for |x| < 4096 (every heading
 * the shader produces), the rest out of line. */
SLM_FN void slm_reduce_pio2(float x, float* r_out, int* q_out) {
    SlmRQ o = slm_abs(x) < 4096.0f ? slm_reduce_pio2_cw(x) : slm_reduce_pio2_large_cold(x);
    *r_out = o.r;
    *q_out = o.q;
}

/* The same split for arguments that are mostly in 4096 <= |x| < 2^44 (the
 * jitter hash's, whose agent-index term alone exceeds 4096 for every index
 * above 315): the fixed-window Payne-Hanek inline, the rest out of line.
 * The same bits as slm_reduce_pio2 for every x. */
SLM_FN void slm_reduce_pio2_hash(float x, float* r_out, int* q_out) {
    const uint32_t E = (slm_f2u_bits(x) >> 23) & 0xffu;
    SlmRQ o;
    if (E >= 139u && E <= 170u) {
        slm_reduce_pio2_win(x, &o.r, &o.q);
    } else {
        o = slm_abs(x) < 4096.0f ? slm_reduce_pio2_cw_cold(x) : slm_reduce_pio2_large_cold(x);
    }
    *r_out = o.r;
    *q_out = o.q;
}

/* The quadrant step of slm_sincos: (sin, cos) from the polynomials s, c and
 * the quadrant q. */
SLM_FN void slm_sincos_quadrant(float s, float c, int q, float* s_out, float* c_out) {
    const float a = (q & 1) ? c : s;
    const float bb = (q & 1) ? s : c;
    /* negation as a flip of the sign bit: bit 1 of q for the sine, of q + 1
     * for the cosine, shifted to bit 31 */
    *s_out = slm_u2f_bits(slm_f2u_bits(a) ^ (((uint32_t)q << 30) & 0x80000000u));
    *c_out = slm_u2f_bits(slm_f2u_bits(bb) ^ (((uint32_t)q + 1u) << 30 & 0x80000000u));
}

/* sin and cos from the reduced argument r and the quadrant q. */
SLM_FN void slm_sincos_rq(float r, int q, float* s_out, float* c_out) {
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
    slm_sincos_quadrant(s, c, q, s_out, c_out);
}

SLM_FN void slm_sincos(float x, float* s_out, float* c_out) {
    float r;
    int q;
    slm_reduce_pio2(x, &r, &q);
    slm_sincos_rq(r, q, s_out, c_out);
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

#if defined(__CUDACC__)
/* slm_sincos of two arguments with |x0|, |x1| < 4096 at once, bit for bit.
 * Each lane's reduction starts with a binary32 product and sum (a packed
 * product followed by a packed sum may be contracted into one fused
 * operation, which would round once instead of twice, so these stay
 * scalar); every later step is a fused multiply-add, or a product that feeds
 * one as a multiplicand, evaluated for both lanes by one packed instruction
 * (fma.rn.f32x2, mul.rn.f32x2: each lane rounded as its scalar form). */
static __device__ __forceinline__ void slm_sincos2_cw(float x0, float x1, float* s0, float* c0, float* s1,
                                                      float* c1) {
    const float b0 = slm_add(slm_mul(x0, SLM_TWO_OVER_PI_F), 12582912.0f);
    const float b1 = slm_add(slm_mul(x1, SLM_TWO_OVER_PI_F), 12582912.0f);
    /* -j, exactly: 1.5 * 2^23 - biased, as one packed sum (a packed sum of
     * operands that no packed product produced rounds per lane) */
    const float2 nj = __fadd2_rn(make_float2(12582912.0f, 12582912.0f), make_float2(-b0, -b1));
    float2 r = __ffma2_rn(nj, make_float2(SLM_PIO2_1, SLM_PIO2_1), make_float2(x0, x1));
    r = __ffma2_rn(nj, make_float2(SLM_PIO2_2, SLM_PIO2_2), r);
    r = __ffma2_rn(nj, make_float2(SLM_PIO2_3, SLM_PIO2_3), r);
    const float2 z = __fmul2_rn(r, r);
    float2 ps = __ffma2_rn(z, make_float2(SLM_S4, SLM_S4), make_float2(SLM_S3, SLM_S3));
    ps = __ffma2_rn(z, ps, make_float2(SLM_S2, SLM_S2));
    ps = __ffma2_rn(z, ps, make_float2(SLM_S1, SLM_S1));
    const float2 s = __ffma2_rn(__fmul2_rn(r, z), ps, r);
    float2 pc = __ffma2_rn(z, make_float2(SLM_C5, SLM_C5), make_float2(SLM_C4, SLM_C4));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C3, SLM_C3));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C2, SLM_C2));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C1, SLM_C1));
    const float2 c = __ffma2_rn(z, pc, make_float2(1.0f, 1.0f));
    slm_sincos_quadrant(s.x, c.x, (int)(slm_f2u_bits(b0) & 3u), s0, c0);
    slm_sincos_quadrant(s.y, c.y, (int)(slm_f2u_bits(b1) & 3u), s1, c1);
}

/* Two general slm_sincos evaluations, out of line. */
typedef struct SlmSinCos2 {
    float s0, c0, s1, c1;
} SlmSinCos2;
static __device__ __noinline__ SlmSinCos2 slm_sincos2_cold(float x0, float x1) {
    SlmSinCos2 o;
    slm_sincos(x0, &o.s0, &o.c0);
    slm_sincos(x1, &o.s1, &o.c1);
    return o;
}

/* slm_sincos of two arguments, bit for bit: the packed pair when both are
 * below 4096 in magnitude, the general form out of line otherwise. */
static __device__ __forceinline__ void slm_sincos2(float x0, float x1, float* s0, float* c0, float* s1, float* c1) {
    if (slm_abs(x0) < 4096.0f && slm_abs(x1) < 4096.0f) {
        slm_sincos2_cw(x0, x1, s0, c0, s1, c1);
    } else {
        const SlmSinCos2 o = slm_sincos2_cold(x0, x1);
        *s0 = o.s0;
        *c0 = o.c0;
        *s1 = o.s1;
        *c1 = o.c1;
    }
}

/* slm_sincos_rq of two reduced arguments: the polynomials as packed fused
 * multiply-adds (products only as their multiplicands), the same bits. */
static __device__ __forceinline__ void slm_sincos_rq2(float r0, int q0, float r1, int q1, float* s0, float* c0,
                                                      float* s1, float* c1) {
    const float2 r = make_float2(r0, r1);
    const float2 z = __fmul2_rn(r, r);
    float2 ps = __ffma2_rn(z, make_float2(SLM_S4, SLM_S4), make_float2(SLM_S3, SLM_S3));
    ps = __ffma2_rn(z, ps, make_float2(SLM_S2, SLM_S2));
    ps = __ffma2_rn(z, ps, make_float2(SLM_S1, SLM_S1));
    const float2 s = __ffma2_rn(__fmul2_rn(r, z), ps, r);
    float2 pc = __ffma2_rn(z, make_float2(SLM_C5, SLM_C5), make_float2(SLM_C4, SLM_C4));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C3, SLM_C3));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C2, SLM_C2));
    pc = __ffma2_rn(z, pc, make_float2(SLM_C1, SLM_C1));
    const float2 c = __ffma2_rn(z, pc, make_float2(1.0f, 1.0f));
    slm_sincos_quadrant(s.x, c.x, q0, s0, c0);
    slm_sincos_quadrant(s.y, c.y, q1, s1, c1);
}
#endif

/* The rotated form (SLIME_SENSOR_ROTATED): the centre direction (c, s) =
 * slm_sincos(angle); the side directions are that vector rotated by -a and +a
 * with (sin a, cos a) = slm_sincos(sensor_angle), a fixed sequence of
 * binary32 products and fused multiply-adds.  Within a few 1e-8 of cos/sin of
 * the rounded angle -/+ a, but not equal to it: near-ties of the turn
 * decision can go the other way than the shader's. */
SLM_FN void slm_rotate_dirs(float c, float s, float sa, float ca, float* cl, float* sl, float* cr, float* sr) {
    /* rotate (c, s) by -a: (c ca + s sa, s ca - c sa); by +a: (c ca - s sa, s ca + c sa) */
    float cca = slm_mul(c, ca), sca = slm_mul(s, ca);
    *cl = slm_fma(s, sa, cca);
    *sl = slm_fma(-c, sa, sca);
    *cr = slm_fma(-s, sa, cca);
    *sr = slm_fma(c, sa, sca);
}
SLM_FN void slm_sensor_dirs(float angle, float sa, float ca, float* cl, float* sl, float* cc, float* sc, float* cr,
                            float* sr) {
    float s, c;
    slm_sincos(angle, &s, &c);
    *cc = c;
    *sc = s;
    slm_rotate_dirs(c, s, sa, ca, cl, sl, cr, sr);
}

/* The two side directions alone, in the shader's form (the first half of
 * slm_sensor_dirs_shader). */
SLM_FN void slm_side_dirs_shader(float angle, float a, float* cl, float* sl, float* cr, float* sr) {
    const float xl = slm_sub(angle, a), xr = slm_add(angle, a);
#if defined(__CUDA_ARCH__)
    slm_sincos2(xl, xr, sl, cl, sr, cr);
#else
    slm_sincos(xl, sl, cl);
    slm_sincos(xr, sr, cr);
#endif
}

/* Sensor directions of compute.wgsl:75-90 as the shader writes them: the
 * sensor angles angle - a and angle + a are binary32 differences and sums
 * (:75-76), and each of the three directions is slm_sincos of its own angle.
 * On the device the two side directions are evaluated as one packed pair
 * when both angles are below 4096 in magnitude (every heading the shader
 * produces), with the same bits. */
SLM_FN void slm_sensor_dirs_shader(float angle, float a, float* cl, float* sl, float* cc, float* sc, float* cr,
                                   float* sr) {
    slm_side_dirs_shader(angle, a, cl, sl, cr, sr);
    slm_sincos(angle, sc, cc);
}

/* The shader's per-agent jitter hash (compute.wgsl:117):
 *   fract(sin(f32(agent_index) * 12.9898 + x * 78.233 + y * 37.719) * 43758.5453)
 * evaluated left to right, unfused. */
SLM_FN float slm_jitter_arg(int32_t agent_index, float x, float y) {
    float a = slm_mul(slm_i2f(agent_index), 12.9898f);
    a = slm_add(a, slm_mul(x, 78.233f));
    return slm_add(a, slm_mul(y, 37.719f));
}
SLM_FN float slm_jitter_hash(int32_t agent_index, float x, float y) {
    float r, s, c;
    int q;
    slm_reduce_pio2_hash(slm_jitter_arg(agent_index, x, y), &r, &q);
    slm_sincos_rq(r, q, &s, &c);
    return slm_fract(slm_mul(s, 43758.5453f));
}
#if defined(__CUDACC__)
/* The reductions of two hash arguments that are not both in the fixed
 * window, each with its own range test, out of line. */
typedef struct SlmRQ2 {
    SlmRQ a, b;
} SlmRQ2;
static __device__ __noinline__ SlmRQ2 slm_reduce_pio2_hash2_cold(float x0, float x1) {
    SlmRQ2 o;
    slm_reduce_pio2_hash(x0, &o.a.r, &o.a.q);
    slm_reduce_pio2_hash(x1, &o.b.r, &o.b.q);
    return o;
}

/* Two jitter hashes, the same bits as slm_jitter_hash for each: one range
 * test for both arguments (the fixed-window reduction inline when both are
 * in it, the rest out of line), their sin polynomials as one packed pair. */
static __device__ __forceinline__ void slm_jitter_hash2(int32_t i0, float x0, float y0, int32_t i1, float x1,
                                                        float y1, float* h0, float* h1) {
    float r0, r1, s0, c0, s1, c1;
    int q0, q1;
    const float a0 = slm_jitter_arg(i0, x0, y0), a1 = slm_jitter_arg(i1, x1, y1);
    const uint32_t e0 = ((slm_f2u_bits(a0) >> 23) & 0xffu) - 139u, e1 = ((slm_f2u_bits(a1) >> 23) & 0xffu) - 139u;
    if (e0 <= 31u && e1 <= 31u) {
        slm_reduce_pio2_win(a0, &r0, &q0);
        slm_reduce_pio2_win(a1, &r1, &q1);
    } else {
        const SlmRQ2 o = slm_reduce_pio2_hash2_cold(a0, a1);
        r0 = o.a.r, q0 = o.a.q, r1 = o.b.r, q1 = o.b.q;
    }
    slm_sincos_rq2(r0, q0, r1, q1, &s0, &c0, &s1, &c1);
    *h0 = slm_fract(slm_mul(s0, 43758.5453f));
    *h1 = slm_fract(slm_mul(s1, 43758.5453f));
}
#endif

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
