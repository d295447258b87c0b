// trail.cu - fused deposit-fold + decay + diffuse.
//
// The reference runs decay_trail (compute.wgsl:148-161) and diffuse_trail
// (compute.wgsl:164-195) as two full passes over the trail, the blur in place.
// Here one kernel reads the pre-step trail and the step's deposit counts once
// (tile plus halo staged in shared memory), applies the sequential deposit
// fold and the decay while staging, blurs from shared memory, writes the new
// trail to the other buffer and zeroes the other step's count buffer.
// HBM traffic per cell: 4 B trail in + 4 B counts in + 4 B trail out +
// 4 B counts zeroed; halo re-reads hit L2.
//
// Box mode sums the nine taps in the shader's order (dy outer, dx inner,
// starting from 0.0) and divides by 9.0, so it matches the shader's arithmetic
// bit for bit; Gaussian mode is separable (horizontal then vertical, fused
// multiply-adds over taps -R..R).
#include "kernels.h"
#include "trail_stream.cuh"

namespace slime {
namespace {

constexpr int kThreads = 256;

template <int TW, int TH, int R>
__device__ __forceinline__ void stage_tile(const DevParams& p, const float* __restrict__ in,
                                           const uint32_t* __restrict__ cin, float* s, int x0, int y0) {
    constexpr int SW = TW + 2 * R, SH = TH + 2 * R;
    const int W = p.W, H = p.H;
    for (int i = threadIdx.x; i < SH * SW; i += kThreads) {
        int ly = i / SW;
        int lx = i - ly * SW;
        int gx = wrap_coord(x0 + lx - R, W);
        int gy = wrap_coord(y0 + ly - R, H);
        int gi = gy * W + gx;
        float v = fold_deposits(__ldg(in + gi), __ldg(cin + gi), p.dep);
        s[i] = apply_decay(p, v);
    }
}

template <int TW, int TH>
__global__ void __launch_bounds__(kThreads) trail_box3_kernel(const __grid_constant__ DevParams p,
                                                              const float* __restrict__ in,
                                                              const uint32_t* __restrict__ cin,
                                                              float* __restrict__ out,
                                                              uint32_t* __restrict__ czero) {
    constexpr int R = 1, SW = TW + 2 * R;
    extern __shared__ float smem[];
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    stage_tile<TW, TH, R>(p, in, cin, smem, x0, y0);
    __syncthreads();
    for (int i = threadIdx.x; i < TW * TH; i += kThreads) {
        int ly = i / TW;
        int lx = i - ly * TW;
        int gx = x0 + lx, gy = y0 + ly;
        if (gx >= p.W || gy >= p.H) continue;
        const float* c = smem + (ly + 1) * SW + (lx + 1);
        float sum = 0.0f;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++)
#pragma unroll
            for (int dx = -1; dx <= 1; dx++) sum = slm_add(sum, c[dy * SW + dx]);
        float avg = slm_div(sum, 9.0f);
        int gi = gy * p.W + gx;
        out[gi] = slm_mix(c[0], avg, p.rate);
        if (czero) czero[gi] = 0u;
    }
}

template <int TW, int TH, int R>
__global__ void __launch_bounds__(kThreads) trail_gauss_kernel(const __grid_constant__ DevParams p,
                                                               const float* __restrict__ in,
                                                               const uint32_t* __restrict__ cin,
                                                               float* __restrict__ out,
                                                               uint32_t* __restrict__ czero) {
    constexpr int SW = TW + 2 * R, SH = TH + 2 * R;
    extern __shared__ float smem[];
    float* s = smem;
    float* h = smem + SH * SW;
    const int x0 = blockIdx.x * TW, y0 = blockIdx.y * TH;
    stage_tile<TW, TH, R>(p, in, cin, s, x0, y0);
    __syncthreads();
    for (int i = threadIdx.x; i < SH * TW; i += kThreads) {
        int ly = i / TW;
        int lx = i - ly * TW;
        const float* row = s + ly * SW + lx;
        float acc = 0.0f;
#pragma unroll
        for (int t = 0; t <= 2 * R; t++) acc = slm_fma(p.w[t], row[t], acc);
        h[i] = acc;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < TW * TH; i += kThreads) {
        int ly = i / TW;
        int lx = i - ly * TW;
        int gx = x0 + lx, gy = y0 + ly;
        if (gx >= p.W || gy >= p.H) continue;
        float acc = 0.0f;
#pragma unroll
        for (int t = 0; t <= 2 * R; t++) acc = slm_fma(p.w[t], h[(ly + t) * TW + lx], acc);
        int gi = gy * p.W + gx;
        out[gi] = slm_mix(s[(ly + R) * SW + lx + R], acc, p.rate);
        if (czero) czero[gi] = 0u;
    }
}

template <int R, bool kGauss, int ROWS, class D>
__global__ void __launch_bounds__(128) trail_stream_kernel(const __grid_constant__ DevParams p,
                                                           const float* __restrict__ in, const D* __restrict__ cin,
                                                           float* __restrict__ out, D* __restrict__ czero,
                                                           int warps_x) {
    const int gw = blockIdx.x * 4 + (threadIdx.x >> 5);
    // the deposit record this reads is the agent pass's output
    pdl_wait();
    pdl_trigger();
    process_strip<R, kGauss, ROWS, false, true, D>(p, in, cin, out, czero, gw % warps_x, gw / warps_x);
}

template <int R, bool kGauss, int ROWS, class D>
cudaError_t launch_stream(const DevParams& p, const float* in, const D* cin, float* out, D* cz, cudaStream_t s,
                          const cudaAccessPolicyWindow* win, bool pdl) {
    int warps_x = (p.W + 127) / 128;
    long long warps = (long long)warps_x * ((p.H + ROWS - 1) / ROWS);
    unsigned blocks = (unsigned)((warps + 3) / 4);
    return launch_kp(trail_stream_kernel<R, kGauss, ROWS, D>, dim3(blocks), dim3(128), 0, s, win, pdl, p, in, cin,
                     out, cz, warps_x);
}

template <int ROWS, class D>
cudaError_t launch_stream_rows(const DevParams& p, const float* in, const D* cin, float* out, D* cz, cudaStream_t s,
                               const cudaAccessPolicyWindow* win, bool pdl) {
    if (p.blur_mode != SLIME_BLUR_GAUSS) return launch_stream<1, false, ROWS, D>(p, in, cin, out, cz, s, win, pdl);
    if (p.R == 1) return launch_stream<1, true, ROWS, D>(p, in, cin, out, cz, s, win, pdl);
    return launch_stream<2, true, ROWS, D>(p, in, cin, out, cz, s, win, pdl);
}

const TrailTile kTiles[] = {{32, 8}, {64, 8}, {32, 16}, {64, 16}, {128, 8}, {128, 16}, {256, 8}};
constexpr int kNumTiles = (int)(sizeof(kTiles) / sizeof(kTiles[0]));

template <int TW, int TH>
cudaError_t launch_tile(const DevParams& p, const float* in, const uint32_t* cin, float* out, uint32_t* cz,
                        cudaStream_t s, const cudaAccessPolicyWindow* win) {
    dim3 grid((p.W + TW - 1) / TW, (p.H + TH - 1) / TH);
    if (p.blur_mode == SLIME_BLUR_GAUSS && p.R > 0) {
        size_t smem;
#define SLIME_GAUSS_CASE(RR)                                                                                 \
    case RR:                                                                                                 \
        smem = sizeof(float) * ((TH + 2 * RR) * (TW + 2 * RR) + (TH + 2 * RR) * TW);                         \
        if (smem > 48 * 1024) {                                                                              \
            cudaError_t e = cudaFuncSetAttribute(trail_gauss_kernel<TW, TH, RR>,                             \
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);    \
            if (e != cudaSuccess) return e;                                                                  \
        }                                                                                                    \
        {                                                                                                    \
            cudaError_t le = launch_k(trail_gauss_kernel<TW, TH, RR>, grid, dim3(kThreads), smem, s, win, p, in,  \
                                      cin, out, cz);                                                         \
            if (le != cudaSuccess) return le;                                                                \
        }                                                                                                    \
        break;
        switch (p.R) {
            SLIME_GAUSS_CASE(1)
            SLIME_GAUSS_CASE(2)
            SLIME_GAUSS_CASE(3)
            SLIME_GAUSS_CASE(4)
            SLIME_GAUSS_CASE(5)
            SLIME_GAUSS_CASE(6)
            SLIME_GAUSS_CASE(7)
            SLIME_GAUSS_CASE(8)
        default:
            return cudaErrorInvalidValue;
        }
#undef SLIME_GAUSS_CASE
    } else if (p.blur_mode == SLIME_BLUR_GAUSS) {
        // Radius 0: the blur is the identity; weights are {1}.
        size_t smem = sizeof(float) * (TH * TW + TH * TW);
        return launch_k(trail_gauss_kernel<TW, TH, 0>, grid, dim3(kThreads), smem, s, win, p, in, cin, out, cz);
    } else {
        size_t smem = sizeof(float) * (TH + 2) * (TW + 2);
        return launch_k(trail_box3_kernel<TW, TH>, grid, dim3(kThreads), smem, s, win, p, in, cin, out, cz);
    }
    return cudaGetLastError();
}

} // namespace

// Tile table: entries 0..kNumTiles-1 are the shared-memory tiles, the next
// kNumStream entries the streaming kernel with 8, 16 and 32 rows per strip,
// the last one (kTrailTileTma) the tensor-copy tile of 128 x 32 cells.
constexpr int kNumStream = 3;
static_assert(kNumTiles + kNumStream == kTrailTileTma, "the tensor-copy tile follows the streaming ones");
int trail_tile_count() { return kNumTiles + kNumStream + 1; }
TrailTile trail_tile(int index) {
    if (index == kTrailTileTma) return TrailTile{128, 32};
    if (index >= kNumTiles && index < kNumTiles + kNumStream) return TrailTile{128, 8 << (index - kNumTiles)};
    return kTiles[(index >= 0 && index < kNumTiles) ? index : 0];
}
int trail_tile_default() { return 3; }
bool trail_tile_supported(const DevParams& p, int tile) {
    if (tile == kTrailTileTma) return trail_tma_supported(p);
    if (tile < 0 || tile >= kNumTiles + kNumStream) return false;
    if (tile < kNumTiles) return true;
    // streaming kernel: whole float4 groups per row and radius <= 2, grid
    // wider than a halo
    int R = p.blur_mode == SLIME_BLUR_GAUSS ? p.R : 1;
    return (p.W % 4) == 0 && p.W >= 8 && R >= 1 && R <= 2 && p.H >= 1;
}

bool trail_tile_streams(const DevParams& p, int tile) { return tile >= kNumTiles && trail_tile_supported(p, tile); }

cudaError_t launch_trail_marks(const DevParams& p, int tile, const float* in, const uint8_t* marks_in, float* out,
                               uint8_t* marks_zero, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl,
                               const TrailMaps* maps, int cur) {
    if (!trail_tile_streams(p, tile)) return cudaErrorInvalidValue;
    if (tile == kTrailTileTma) {
        // without tensor maps, the 8-row streaming tile (same requirements, same bits)
        if (!maps || !maps->ok) return launch_stream_rows<8>(p, in, marks_in, out, marks_zero, s, win, pdl);
        return launch_trail_tma_marks(p, *maps, cur, in, marks_in, out, marks_zero, s, win, pdl);
    }
    switch (tile) {
    case 7: return launch_stream_rows<8>(p, in, marks_in, out, marks_zero, s, win, pdl);
    case 8: return launch_stream_rows<16>(p, in, marks_in, out, marks_zero, s, win, pdl);
    default: return launch_stream_rows<32>(p, in, marks_in, out, marks_zero, s, win, pdl);
    }
}

cudaError_t launch_trail(const DevParams& p, int tile, const float* in, const uint32_t* counts_in, float* out,
                         uint32_t* counts_zero, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl,
                         const TrailMaps* maps, int cur) {
    if (!trail_tile_supported(p, tile) || (tile == kTrailTileTma && !(maps && maps->ok))) tile = trail_tile_default();
    if (tile == kTrailTileTma) return launch_trail_tma(p, *maps, cur, in, counts_in, out, counts_zero, s, win, pdl);
    switch (tile) {
    case 0: return launch_tile<32, 8>(p, in, counts_in, out, counts_zero, s, win);
    case 1: return launch_tile<64, 8>(p, in, counts_in, out, counts_zero, s, win);
    case 2: return launch_tile<32, 16>(p, in, counts_in, out, counts_zero, s, win);
    case 3: return launch_tile<64, 16>(p, in, counts_in, out, counts_zero, s, win);
    case 4: return launch_tile<128, 8>(p, in, counts_in, out, counts_zero, s, win);
    case 5: return launch_tile<128, 16>(p, in, counts_in, out, counts_zero, s, win);
    case 6: return launch_tile<256, 8>(p, in, counts_in, out, counts_zero, s, win);
    case 7: return launch_stream_rows<8>(p, in, counts_in, out, counts_zero, s, win, pdl);
    case 8: return launch_stream_rows<16>(p, in, counts_in, out, counts_zero, s, win, pdl);
    case 9: return launch_stream_rows<32>(p, in, counts_in, out, counts_zero, s, win, pdl);
    default: return cudaErrorInvalidValue;
    }
}

} // namespace slime
