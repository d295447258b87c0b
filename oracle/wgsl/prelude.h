/*
 * prelude.h - WGSL types and builtins for C++ translations of the reference's
 * compute shader (test infrastructure: only the parity tests use it).
 *
 * oracle/wgsl/translate.py turns src/compute.wgsl into C++ that reads almost
 * token for token like the shader; this header gives that C++ the shader's
 * meaning:
 *   - f32 is a binary32 value type whose + - * / round once each (compiled
 *     with -ffp-contract=off, nothing fuses) and whose % is the WGSL float
 *     remainder (fmod: sign of the dividend);
 *   - i32 / u32 are the 32-bit integers, with the WGSL conversions i32(f32)
 *     (truncate, saturate, NaN -> 0), f32(i32) (round to nearest) and
 *     i32(u32) (same bits);
 *   - vec2/vec3/vec4 are plain component structs;
 *   - floor, fract, mix, clamp, min, max, abs, sign are the WGSL definitions
 *     (fract(e) = e - floor(e), mix(a, b, t) = a * (1 - t) + b * t,
 *     clamp(e, lo, hi) = min(max(e, lo), hi)) on the pinned binary32
 *     operations of include/slime_math.h; sin and cos, whose precision WGSL
 *     leaves to the implementation, are that header's;
 *   - storage buffers are Buffer<T>: arrays the harness binds, read and
 *     written through operator[] either in place (the shader's own binding)
 *     or Jacobi-style (reads from one array, writes to another), which is how
 *     a race-free execution of an in-place pass is defined for comparison.
 *     An index outside the array reads 0 and drops the write, one of the
 *     outcomes WGSL's robust buffer access allows;
 *   - i32 arithmetic wraps as in WGSL (the harness is compiled with -fwrapv);
 *   - the display's texture_storage_2d<rgba8unorm, write> is StorageTexRGBA8,
 *     an RGBA8 image the harness binds: textureDimensions gives its size,
 *     textureStore converts each channel as a unorm8 store does,
 *     round(clamp(c, 0, 1) * 255) (to nearest; NaN stores 0), and drops
 *     stores outside the image.
 */
#ifndef SLIME_WGSL_PRELUDE_H
#define SLIME_WGSL_PRELUDE_H

#include <stdint.h>

#include "../../include/slime_math.h"

namespace wgsl {

struct f32 {
    float v;
    f32() : v(0.0f) {}
    explicit f32(float x) : v(x) {}
    f32& operator+=(f32 o) { v = slm_add(v, o.v); return *this; }
    f32& operator-=(f32 o) { v = slm_sub(v, o.v); return *this; }
    f32& operator*=(f32 o) { v = slm_mul(v, o.v); return *this; }
    f32& operator/=(f32 o) { v = slm_div(v, o.v); return *this; }
};
inline f32 operator+(f32 a, f32 b) { return f32(slm_add(a.v, b.v)); }
inline f32 operator-(f32 a, f32 b) { return f32(slm_sub(a.v, b.v)); }
inline f32 operator*(f32 a, f32 b) { return f32(slm_mul(a.v, b.v)); }
inline f32 operator/(f32 a, f32 b) { return f32(slm_div(a.v, b.v)); }
inline f32 operator%(f32 a, f32 b) { return f32(fmodf(a.v, b.v)); }
inline f32 operator-(f32 a) { return f32(-a.v); }
inline bool operator<(f32 a, f32 b) { return a.v < b.v; }
inline bool operator>(f32 a, f32 b) { return a.v > b.v; }
inline bool operator<=(f32 a, f32 b) { return a.v <= b.v; }
inline bool operator>=(f32 a, f32 b) { return a.v >= b.v; }
inline bool operator==(f32 a, f32 b) { return a.v == b.v; }
inline bool operator!=(f32 a, f32 b) { return a.v != b.v; }

typedef int32_t i32;
typedef uint32_t u32;

struct vec2f {
    f32 x, y;
};
struct vec2i {
    int32_t x, y;
};
struct vec2u {
    uint32_t x, y;
};
struct vec4f {
    f32 x, y, z, w;
};
struct vec3u {
    u32 x, y, z;
};

/* conversions */
inline i32 to_i32(f32 e) { return slm_f2i(e.v); }
inline i32 to_i32(u32 e) { return (i32)e; }
inline i32 to_i32(i32 e) { return e; }
inline u32 to_u32(f32 e) { /* truncate, saturate to [0, 2^32 - 1], NaN -> 0 */
    if (!(e.v > 0.0f)) return 0u;
    if (e.v >= 4294967296.0f) return 0xffffffffu;
    return (u32)e.v;
}
inline u32 to_u32(i32 e) { return (u32)e; }
inline u32 to_u32(u32 e) { return e; }
inline f32 to_f32(i32 e) { return f32(slm_i2f(e)); }
inline f32 to_f32(u32 e) { return f32((float)e); }
inline f32 to_f32(f32 e) { return e; }

/* builtins */
inline f32 floor(f32 e) { return f32(slm_floor(e.v)); }
inline f32 fract(f32 e) { return f32(slm_fract(e.v)); }
inline f32 mix(f32 a, f32 b, f32 t) { return f32(slm_mix(a.v, b.v, t.v)); }
inline f32 min(f32 a, f32 b) { return f32(slm_min(a.v, b.v)); }
inline f32 max(f32 a, f32 b) { return f32(slm_max(a.v, b.v)); }
inline f32 clamp(f32 e, f32 lo, f32 hi) { return f32(slm_clamp(e.v, lo.v, hi.v)); }
inline f32 abs(f32 e) { return f32(slm_abs(e.v)); }
inline f32 sign(f32 e) { return f32(slm_sign(e.v)); }
inline f32 sin(f32 e) { return f32(slm_sin(e.v)); }
inline f32 cos(f32 e) { return f32(slm_cos(e.v)); }

/* storage buffers */
template <class T>
struct Buffer;
template <class T>
struct BufRef {
    Buffer<T>* b;
    int32_t i;
    operator T() const;
    BufRef& operator=(const T& v);
    BufRef& operator=(const BufRef& o) { return *this = (T)o; }
};
template <class T>
struct Buffer {
    T* data = nullptr;      // the binding (reads, and writes in place)
    const T* src = nullptr; // Jacobi binding: reads come from here, writes go to data
    uint32_t length = 0;
    BufRef<T> operator[](int32_t i) { return BufRef<T>{this, i}; }
};
template <class T>
BufRef<T>::operator T() const {
    if (i < 0 || (uint32_t)i >= b->length) return T();
    return b->src ? b->src[i] : b->data[i];
}
template <class T>
BufRef<T>& BufRef<T>::operator=(const T& v) {
    if (i >= 0 && (uint32_t)i < b->length) b->data[i] = v;
    return *this;
}
template <class T>
inline u32 arrayLength(const Buffer<T>& b) {
    return b.length;
}
/* write-only rgba8unorm storage texture */
struct StorageTexRGBA8 {
    uint8_t* data = nullptr; /* width * height RGBA8 texels, row-major */
    uint32_t width = 0, height = 0;
};
inline vec2u textureDimensions(const StorageTexRGBA8& t) { return vec2u{t.width, t.height}; }
inline uint8_t unorm8(f32 c) {
    if (!(c.v > 0.0f)) return 0;
    if (c.v >= 1.0f) return 255;
    return (uint8_t)(double)((double)c.v * 255.0 + 0.5); /* c * 255 is exact in binary64 */
}
inline void textureStore(StorageTexRGBA8& t, vec2i at, vec4f c) {
    if (at.x < 0 || at.y < 0 || (uint32_t)at.x >= t.width || (uint32_t)at.y >= t.height) return;
    uint8_t* o = t.data + 4 * ((size_t)at.y * t.width + (uint32_t)at.x);
    o[0] = unorm8(c.x);
    o[1] = unorm8(c.y);
    o[2] = unorm8(c.z);
    o[3] = unorm8(c.w);
}

/* `let x = e;` takes e's value (a buffer element is read, not referenced) */
template <class T>
inline T value(const T& v) {
    return v;
}
template <class T>
inline T value(const BufRef<T>& r) {
    return (T)r;
}

} // namespace wgsl

#endif
