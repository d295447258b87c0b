// trail_stream.cuh - the streaming form of the fused deposit-fold + decay +
// diffuse pass (decay_trail, compute.wgsl:148-161, and diffuse_trail,
// compute.wgsl:164-195), shared by the plain and the ensemble kernels.
#pragma once

#include "common.cuh"

namespace slime {

// ---------------------------------------------------------------------------
// Streaming variant for W % 4 == 0 and radius <= 2: one thread owns four
// adjacent columns (16-byte loads of trail and counts, 16-byte stores of the
// new trail and of the zeroed counts) and walks a strip of ROWS output rows
// with a rolling window of 2R+1 input rows in registers.  Horizontal halos
// come from the neighbouring lanes by warp shuffle; the first lane and the
// last active lane of a warp load theirs (wrapped) directly.  Every output
// is produced by the same operations in the same order as the tiled kernels.
template <int R>
struct ExtRow {
    float v[4 + 2 * R]; // columns c0-R .. c0+3+R after fold + decay
};

// Counts written earlier in the same launch (the ensemble's persistent
// kernel) must not be read through the non-coherent read-only path.
template <bool kCoherent>
__device__ __forceinline__ uint32_t load_count(const uint32_t* p) {
    return kCoherent ? __ldcg(p) : __ldg(p);
}
template <bool kCoherent>
__device__ __forceinline__ uint4 load_count4(const uint4* p) {
    return kCoherent ? __ldcg(p) : __ldg(p);
}

// The step's deposit record is either per-cell 32-bit counts or, when every
// deposit saturates the fold, per-cell byte marks (0 or 1).  A lane's four
// cells come as a uint4 of counts or as one 32-bit word of four marks (one
// register per row in flight instead of four); dep_at reads cell j of either
// as a count k, and a mark of 1 folds exactly as any k >= 1 does then.
template <class D>
struct DepVec {
    typedef uint4 type;
};
template <>
struct DepVec<uint8_t> {
    typedef uint32_t type;
};
__device__ __forceinline__ uint32_t dep_at(const uint4& k, int j) {
    return j == 0 ? k.x : (j == 1 ? k.y : (j == 2 ? k.z : k.w));
}
__device__ __forceinline__ uint32_t dep_at(uint32_t k, int j) { return (k >> (8 * j)) & 0xffu; }
template <bool kCoherent>
__device__ __forceinline__ uint4 load_dep4(const uint32_t* p) {
    return load_count4<kCoherent>(reinterpret_cast<const uint4*>(p));
}
template <bool kCoherent>
__device__ __forceinline__ uint32_t load_dep4(const uint8_t* p) {
    return __ldg(reinterpret_cast<const unsigned int*>(p));
}
template <bool kCoherent>
__device__ __forceinline__ uint32_t load_dep(const uint32_t* p) {
    return load_count<kCoherent>(p);
}
template <bool kCoherent>
__device__ __forceinline__ uint32_t load_dep(const uint8_t* p) {
    return __ldg(p);
}
__device__ __forceinline__ void zero_dep4(uint32_t* p) { *reinterpret_cast<uint4*>(p) = make_uint4(0u, 0u, 0u, 0u); }
__device__ __forceinline__ void zero_dep4(uint8_t* p) { *reinterpret_cast<uchar4*>(p) = make_uchar4(0, 0, 0, 0); }

// One input row as a lane sees it: its four cells and, for the first lane and
// the last active lane of the warp, the R wrapped halo cells on its open side.
template <int R, class D>
struct RowFetch {
    float4 t;
    typename DepVec<D>::type k;
    float ht[R];
    uint32_t hk[R];
};

// L2 prefetch of a row's trail cells and deposit record (a hint: no registers
// held, no result), so a later fetch_row of it is served from L2.
template <class D>
__device__ __forceinline__ void prefetch_row(const DevParams& p, const float* __restrict__ in,
                                             const D* __restrict__ cin, int row, int cl) {
    const size_t base = (size_t)row * p.W + cl;
    asm volatile("prefetch.global.L2 [%0];" ::"l"(in + base));
    asm volatile("prefetch.global.L2 [%0];" ::"l"(cin + base));
}

template <int R, bool kCoherent, class D>
__device__ __forceinline__ void fetch_row(const DevParams& p, const float* __restrict__ in, const D* __restrict__ cin,
                                          int row, int cl, bool has_halo, int hcol0, RowFetch<R, D>& f) {
    const size_t base = (size_t)row * p.W;
    f.t = __ldg(reinterpret_cast<const float4*>(in + base + cl));
    f.k = load_dep4<kCoherent>(cin + base + cl);
#pragma unroll
    for (int j = 0; j < R; j++) {
        f.ht[j] = 0.0f;
        f.hk[j] = 0u;
        if (has_halo) {
            // hcol0 + j lies in [-R, W + R) and W >= 8 > R: one wrap, as selects
            const int g = hcol0 + j;
            const int col = g < 0 ? g + p.W : (g >= p.W ? g - p.W : g);
            f.ht[j] = __ldg(in + base + col);
            f.hk[j] = load_dep<kCoherent>(cin + base + col);
        }
    }
}

// The fold of a cell's deposits.  From marks, which are used only when every
// deposit saturates (deposition >= 1 on t >= 0), the first deposit's
// clamp(t + dep, 0, 1) is exactly 1, so a marked cell folds to 1.0f.
template <bool kMarks>
__device__ __forceinline__ float fold_dep(float t, uint32_t k, float dep) {
    if (kMarks) return k ? 1.0f : t;
    return fold_deposits(t, k, dep);
}

template <int R, int kDecay, class D>
__device__ __forceinline__ void build_ext_row(const DevParams& p, const RowFetch<R, D>& f, bool left_edge,
                                              bool right_edge, ExtRow<R>& e) {
    constexpr bool kMarks = sizeof(D) == 1;
    float d[4] = {apply_decay_m<kDecay>(p, fold_dep<kMarks>(f.t.x, dep_at(f.k, 0), p.dep)),
                  apply_decay_m<kDecay>(p, fold_dep<kMarks>(f.t.y, dep_at(f.k, 1), p.dep)),
                  apply_decay_m<kDecay>(p, fold_dep<kMarks>(f.t.z, dep_at(f.k, 2), p.dep)),
                  apply_decay_m<kDecay>(p, fold_dep<kMarks>(f.t.w, dep_at(f.k, 3), p.dep))};
#pragma unroll
    for (int j = 0; j < 4; j++) e.v[R + j] = d[j];
#pragma unroll
    for (int j = 0; j < R; j++) {
        e.v[j] = __shfl_up_sync(0xffffffffu, d[4 - R + j], 1);
        e.v[R + 4 + j] = __shfl_down_sync(0xffffffffu, d[j], 1);
    }
#pragma unroll
    for (int j = 0; j < R; j++) {
        float h = apply_decay_m<kDecay>(p, fold_dep<kMarks>(f.ht[j], f.hk[j], p.dep));
        if (left_edge) e.v[j] = h;
        if (right_edge) e.v[R + 4 + j] = h;
    }
}

// One warp processes strip (cw, rs): columns 128*cw .. 128*cw+127, output
// rows ROWS*rs .. ROWS*rs+ROWS-1.  All 32 lanes must call it together.  With
// kUnrolled the row loop of a short strip is unrolled, so the window of 2R+1
// rows rotates by renaming registers rather than by copies (at the price of
// registers: kernels that must stay small, like the ensemble's, keep the loop).
// kDecay is the decay mode (SLIME_DECAY_*) or -1 to read it from p at run time.
// D is the deposit record's element type: uint32_t counts or uint8_t marks.
template <int R, bool kGauss, int ROWS, bool kCoherent, int kDecay, bool kUnrolled, class D>
__device__ __forceinline__ void process_strip_m(const DevParams& p, const float* __restrict__ in,
                                                const D* __restrict__ cin, float* __restrict__ out,
                                                D* __restrict__ czero, int cw, int rs) {
    const int lane = threadIdx.x & 31;
    const int W = p.W, H = p.H;
    const int y0 = rs * ROWS;
    if (y0 >= H) return; // warp-uniform
    const int c0 = cw * 128 + lane * 4;
    const bool active = c0 < W;
    const bool left_edge = lane == 0;
    const bool right_edge = active && (lane == 31 || c0 + 4 >= W);
    const int cl = active ? c0 : 0; // inactive lanes load a valid line and discard it

    constexpr int NWIN = 2 * R + 1;
    ExtRow<R> win[NWIN];
    float hwin[NWIN][4];

    // rows are fetched kRegRows ahead of their use, halo cells with them
    // (with byte marks three: since the rows are wrapped incrementally the
    // kernel issues fewer instructions, and the third row in flight measures
    // 1-2 % faster than two; with 32-bit counts, whose rows take four times
    // the registers, two)
    constexpr int NR = ROWS + 2 * R;
    const bool has_halo = active && (left_edge || right_edge);
    const int hcol0 = left_edge ? c0 - R : c0 + 4;
    constexpr int kRegRows = sizeof(D) == 1 ? 3 : 2;
    RowFetch<R, D> fq[kRegRows];
    // the input rows y0 - R .. y0 + ROWS + R - 1, wrapped: the first one
    // wrapped once, each next one by a step back to 0 after H - 1
    const auto next_row = [H](int v) { return v + 1 == H ? 0 : v + 1; };
    int fr = wrap_coord(y0 - R, H); // the next row to fetch into registers
#pragma unroll
    for (int q = 0; q < kRegRows; q++) {
        if (q < NR) fetch_row<R, kCoherent, D>(p, in, cin, fr, cl, has_halo, hcol0, fq[q]);
        fr = next_row(fr);
    }
    // rows further ahead are prefetched into L2 (kPrefetchL2 rows beyond the
    // ones held in registers) by the streaming kernel
    constexpr int kPrefetchL2 = kUnrolled ? 2 : 0;
    int pr = fr; // the next row to prefetch
#pragma unroll
    for (int q = 0; q < kPrefetchL2; q++)
        if (kRegRows + q < NR) {
            prefetch_row<D>(p, in, cin, pr, cl);
            pr = next_row(pr);
        }
    // short strips unroll completely when asked to; long ones stay rolled
    // (unrolled, their live ranges exceed the register budget and spill)
    constexpr int kUnroll = (kUnrolled && NR <= 12) ? NR : 1;
#pragma unroll kUnroll
    for (int r = 0; r < NR; r++) {
        RowFetch<R, D> cur = fq[0];
#pragma unroll
        for (int q = 0; q + 1 < kRegRows; q++) fq[q] = fq[q + 1];
        if (r + kRegRows < NR) { // row y0 - R + r + kRegRows
            fetch_row<R, kCoherent, D>(p, in, cin, fr, cl, has_halo, hcol0, fq[kRegRows - 1]);
            fr = next_row(fr);
        }
        if (kPrefetchL2 && r + kRegRows + kPrefetchL2 < NR) { // row y0 - R + r + kRegRows + kPrefetchL2
            prefetch_row<D>(p, in, cin, pr, cl);
            pr = next_row(pr);
        }
        // shift the window and add the new row
#pragma unroll
        for (int q = 0; q < NWIN - 1; q++) {
            win[q] = win[q + 1];
            if (kGauss) {
#pragma unroll
                for (int j = 0; j < 4; j++) hwin[q][j] = hwin[q + 1][j];
            }
        }
        build_ext_row<R, kDecay, D>(p, cur, left_edge && active, right_edge, win[NWIN - 1]);
        if (kGauss) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float acc = 0.0f;
#pragma unroll
                for (int q = 0; q <= 2 * R; q++) acc = slm_fma(p.w[q], win[NWIN - 1].v[j + q], acc);
                hwin[NWIN - 1][j] = acc;
            }
        }
        if (r < 2 * R) continue;
        const int y = y0 + r - 2 * R;
        if (!active || y >= H) continue;
        float o[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            float center = win[R].v[R + j];
            float blur;
            if (kGauss) {
                float acc = 0.0f;
#pragma unroll
                for (int q = 0; q <= 2 * R; q++) acc = slm_fma(p.w[q], hwin[q][j], acc);
                blur = acc;
            } else {
                float sum = 0.0f;
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                    for (int dx = 0; dx < 3; dx++) sum = slm_add(sum, win[dy].v[j + dx]);
                blur = slm_div(sum, 9.0f);
            }
            o[j] = slm_mix(center, blur, p.rate);
        }
        const size_t off = (size_t)y * W + c0;
        *reinterpret_cast<float4*>(out + off) = make_float4(o[0], o[1], o[2], o[3]);
        if (czero) zero_dep4(czero + off);
    }
}

template <int R, bool kGauss, int ROWS, bool kCoherent = false, bool kUnrolled = true, class D = uint32_t>
__device__ __forceinline__ void process_strip(const DevParams& p, const float* __restrict__ in,
                                              const D* __restrict__ cin, float* __restrict__ out,
                                              D* __restrict__ czero, int cw, int rs) {
    // the unrolled form also fixes the decay mode per instance; the rolled one
    // keeps a single copy of the loop (two would cost registers)
    if (!kUnrolled)
        process_strip_m<R, kGauss, ROWS, kCoherent, -1, false, D>(p, in, cin, out, czero, cw, rs);
    else if (p.decay_mode == SLIME_DECAY_MULTIPLY)
        process_strip_m<R, kGauss, ROWS, kCoherent, (int)SLIME_DECAY_MULTIPLY, true, D>(p, in, cin, out, czero, cw,
                                                                                     rs);
    else
        process_strip_m<R, kGauss, ROWS, kCoherent, (int)SLIME_DECAY_REF_SUBTRACT, true, D>(p, in, cin, out, czero,
                                                                                         cw, rs);
}


} // namespace slime
