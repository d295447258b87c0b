// trail_tma.cu - the fused deposit-fold + decay + diffuse pass (decay_trail,
// compute.wgsl:148-161, and diffuse_trail, compute.wgsl:164-195) with its
// input window staged by the tensor memory accelerator.
//
// A block computes an output tile of 128 columns x 32 rows.  Its input window
// (the tile plus a halo of R cells, R <= 2) arrives in shared memory as two
// 2-D tensor copies issued by one thread and completing on one mbarrier: the
// trail's box (columns x0-4 .. x0+131, so that the box starts on a 16-byte
// boundary) and the deposit record's box (counts: the same columns; byte
// marks: x0-16 .. x0+143).  The trail box is issued before the wait for the
// agent pass (which does not write this trail), the deposit box after it.
// Tiles whose window would wrap around the torus (the border tiles) load it
// with plain wrapped loads instead: a tensor copy fills outside the array
// with zeros, not with the opposite side.
//
// Then, from shared memory: the deposit fold and the decay of every window
// cell in place; each thread blurs 4 columns x 4 rows (halo columns from the
// neighbouring lanes by shuffle) and writes them with one 16-byte store per
// row, zeroing the other step's deposit record there.  Every output is the
// same sequence of operations as in the streaming kernel (trail_stream.cuh),
// so the results are bit-identical.
//
// Waits are bounded: a block whose copies do not complete within about a
// second of clock cycles records the failure in a device flag (read and
// cleared by trail_tma_take_error) and leaves its tile unwritten.
#include <cuda.h>
#include <cudaTypedefs.h>

#include "kernels.h"
#include "trail_stream.cuh"

namespace slime {
namespace {

constexpr int kTmaCols = 128;  // output columns per tile
constexpr int kTmaRows = 32;   // output rows per tile (8 warps x 4 rows)
constexpr int kTmaThreads = 256;
constexpr int kTrailBoxCols = kTmaCols + 8; // x0-4 .. x0+131
constexpr int kMarkBoxCols = kTmaCols + 32; // x0-16 .. x0+143
constexpr int kTrailLead = 4;               // window column of x0 in the trail box
constexpr int kMarkLead = 16;               // window column of x0 in the mark box

__device__ int g_tma_wait_failed;

template <class D>
struct DepBox {
    static constexpr int cols = kTrailBoxCols;
    static constexpr int lead = kTrailLead;
};
template <>
struct DepBox<uint8_t> {
    static constexpr int cols = kMarkBoxCols;
    static constexpr int lead = kMarkLead;
};

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Wait for phase 0 of the barrier; false after ~2^31 cycles (about a second).
__device__ __forceinline__ bool mbar_wait0(uint64_t* bar) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar))
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

template <int R, bool kGauss, int kDecay, class D>
__global__ void __launch_bounds__(kTmaThreads) trail_tma_kernel(const __grid_constant__ DevParams p,
                                                                const __grid_constant__ CUtensorMap map_t,
                                                                const __grid_constant__ CUtensorMap map_d,
                                                                const float* __restrict__ in,
                                                                const D* __restrict__ din, float* __restrict__ out,
                                                                D* __restrict__ dzero) {
    constexpr bool kMarks = sizeof(D) == 1;
    constexpr int WR = kTmaRows + 2 * R; // window rows
    constexpr int DC = DepBox<D>::cols, DL = DepBox<D>::lead;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    float* tw = reinterpret_cast<float*>(smem + 128);                               // WR x kTrailBoxCols
    D* dw = reinterpret_cast<D*>(smem + 128 + sizeof(float) * WR * kTrailBoxCols); // WR x DC
    const int W = p.W, H = p.H;
    const int x0 = blockIdx.x * kTmaCols, y0 = blockIdx.y * kTmaRows;
    // interior tiles: both boxes inside the array (block-uniform)
    const bool interior = x0 - DL >= 0 && x0 - DL + DC <= W && y0 - R >= 0 && y0 - R + WR <= H;
    __shared__ int ok;
    if (interior) {
        if (threadIdx.x == 0) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            const uint32_t bytes = (uint32_t)(sizeof(float) * WR * kTrailBoxCols + sizeof(D) * WR * DC);
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                         : "memory");
            // the trail this reads is not written by the agent pass
            tma_load_2d(tw, &map_t, x0 - kTrailLead, y0 - R, bar);
        }
        // the deposit record is the agent pass's output
        pdl_wait();
        if (threadIdx.x == 0) tma_load_2d(dw, &map_d, x0 - DL, y0 - R, bar);
        pdl_trigger();
        __syncthreads(); // the barrier is initialised before anyone waits on it
        const bool done = mbar_wait0(bar);
        if (threadIdx.x == 0) ok = done ? 1 : 0;
        __syncthreads();
        if (!ok) {
            if (threadIdx.x == 0) atomicExch(&g_tma_wait_failed, 1);
            return;
        }
        // fold + decay of the window's cells in place (columns x0-R .. x0+127+R)
        for (int i = threadIdx.x; i < WR * (kTmaCols + 2 * R); i += kTmaThreads) {
            const int r = i / (kTmaCols + 2 * R), c = i - r * (kTmaCols + 2 * R) - R; // c = column - x0
            float& v = tw[r * kTrailBoxCols + kTrailLead + c];
            v = apply_decay_m<kDecay>(p, fold_dep<kMarks>(v, (uint32_t)dw[r * DC + DL + c], p.dep));
        }
    } else {
        pdl_wait();
        pdl_trigger();
        // border tile: the same window from wrapped plain loads, folded and decayed
        for (int i = threadIdx.x; i < WR * (kTmaCols + 2 * R); i += kTmaThreads) {
            const int r = i / (kTmaCols + 2 * R), c = i - r * (kTmaCols + 2 * R) - R;
            const size_t gi = (size_t)wrap_coord(y0 - R + r, H) * W + wrap_coord(x0 + c, W);
            tw[r * kTrailBoxCols + kTrailLead + c] =
                apply_decay_m<kDecay>(p, fold_dep<kMarks>(__ldg(in + gi), (uint32_t)__ldg(din + gi), p.dep));
        }
    }
    __syncthreads();

    // blur: lane -> 4 columns, warp -> 4 rows
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c0 = lane * 4;
    const int ry = warp * 4; // first output row of the warp within the tile
    float e[4 + 2 * R][4 + 2 * R]; // window rows ry .. ry+3+2R, columns c0-R .. c0+3+R
#pragma unroll
    for (int r = 0; r < 4 + 2 * R; r++) {
        const float* row = tw + (ry + r) * kTrailBoxCols + kTrailLead;
        const float4 v = *reinterpret_cast<const float4*>(row + c0);
        const float d[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int j = 0; j < 4; j++) e[r][R + j] = d[j];
#pragma unroll
        for (int j = 0; j < R; j++) {
            e[r][j] = __shfl_up_sync(0xffffffffu, d[4 - R + j], 1);
            e[r][R + 4 + j] = __shfl_down_sync(0xffffffffu, d[j], 1);
        }
        if (lane == 0) {
#pragma unroll
            for (int j = 0; j < R; j++) e[r][j] = row[c0 - R + j];
        }
        if (lane == 31) {
#pragma unroll
            for (int j = 0; j < R; j++) e[r][R + 4 + j] = row[c0 + 4 + j];
        }
    }
    float h[4 + 2 * R][4]; // Gaussian: the horizontal pass of each window row
    if (kGauss) {
#pragma unroll
        for (int r = 0; r < 4 + 2 * R; r++)
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float acc = 0.0f;
#pragma unroll
                for (int q = 0; q <= 2 * R; q++) acc = slm_fma(p.w[q], e[r][j + q], acc);
                h[r][j] = acc;
            }
    }
    const int x = x0 + c0;
#pragma unroll
    for (int o = 0; o < 4; o++) {
        const int y = y0 + ry + o;
        if (y >= H || x >= W) continue;
        float res[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float center = e[o + R][R + j];
            float blur;
            if (kGauss) {
                float acc = 0.0f;
#pragma unroll
                for (int q = 0; q <= 2 * R; q++) acc = slm_fma(p.w[q], h[o + q][j], acc);
                blur = acc;
            } else {
                float sum = 0.0f;
#pragma unroll
                for (int dy = 0; dy < 3; dy++)
#pragma unroll
                    for (int dx = 0; dx < 3; dx++) sum = slm_add(sum, e[o + dy][j + dx]);
                blur = slm_div(sum, 9.0f);
            }
            res[j] = slm_mix(center, blur, p.rate);
        }
        const size_t off = (size_t)y * W + x;
        *reinterpret_cast<float4*>(out + off) = make_float4(res[0], res[1], res[2], res[3]);
        if (dzero) zero_dep4(dzero + off);
    }
}

template <int R, bool kGauss, int kDecay, class D>
cudaError_t launch_tma_k(const DevParams& p, const TrailMaps& maps, int cur, const float* in, const D* din,
                         float* out, D* dz, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl) {
    constexpr int WR = kTmaRows + 2 * R;
    const size_t smem = 128 + sizeof(float) * WR * kTrailBoxCols + sizeof(D) * WR * DepBox<D>::cols;
    // the maps' box height is the window's: 34 rows for radius 1, 36 for 2
    const CUtensorMap& mt = R == 1 ? maps.trail[cur] : maps.trail_r2[cur];
    const CUtensorMap& md = sizeof(D) == 1 ? (R == 1 ? maps.marks[cur] : maps.marks_r2[cur])
                                           : (R == 1 ? maps.counts[cur] : maps.counts_r2[cur]);
    dim3 grid((p.W + kTmaCols - 1) / kTmaCols, (p.H + kTmaRows - 1) / kTmaRows);
    return launch_kp(trail_tma_kernel<R, kGauss, kDecay, D>, grid, dim3(kTmaThreads), smem, s, win, pdl, p, mt, md,
                     in, din, out, dz);
}

template <int R, bool kGauss, class D>
cudaError_t launch_tma_d(const DevParams& p, const TrailMaps& maps, int cur, const float* in, const D* din,
                         float* out, D* dz, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl) {
    if (p.decay_mode == SLIME_DECAY_MULTIPLY)
        return launch_tma_k<R, kGauss, (int)SLIME_DECAY_MULTIPLY, D>(p, maps, cur, in, din, out, dz, s, win, pdl);
    return launch_tma_k<R, kGauss, (int)SLIME_DECAY_REF_SUBTRACT, D>(p, maps, cur, in, din, out, dz, s, win, pdl);
}

template <class D>
cudaError_t launch_tma(const DevParams& p, const TrailMaps& maps, int cur, const float* in, const D* din, float* out,
                       D* dz, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl) {
    if (!maps.ok || !trail_tma_supported(p)) return cudaErrorInvalidValue;
    if (p.blur_mode != SLIME_BLUR_GAUSS) return launch_tma_d<1, false, D>(p, maps, cur, in, din, out, dz, s, win, pdl);
    if (p.R == 1) return launch_tma_d<1, true, D>(p, maps, cur, in, din, out, dz, s, win, pdl);
    return launch_tma_d<2, true, D>(p, maps, cur, in, din, out, dz, s, win, pdl);
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &f, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (PFN_cuTensorMapEncodeTiled_v12000) nullptr;
        }
        return (PFN_cuTensorMapEncodeTiled_v12000)f;
    }();
    return fn;
}

// A W x H row-major array of `elem` bytes per cell at `base`, read in boxes of
// box_w x box_h cells (no interleave, no swizzle, zeros outside).
bool encode_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, size_t elem, uint32_t W, uint32_t H,
               uint32_t box_w, uint32_t box_h) {
    auto fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[2] = {W, H};
    const cuuint64_t strides[1] = {(cuuint64_t)W * elem};
    const cuuint32_t box[2] = {box_w, box_h};
    const cuuint32_t estr[2] = {1, 1};
    return fn(map, type, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

} // namespace

bool trail_tma_supported(const DevParams& p) {
    const int R = p.blur_mode == SLIME_BLUR_GAUSS ? p.R : 1;
    // byte-mark rows must be whole 16-byte units for a tensor map
    return p.W % 16 == 0 && p.W >= 16 && p.H >= 1 && R >= 1 && R <= 2;
}

bool make_trail_maps(TrailMaps* m, const float* const trail[2], const uint32_t* const counts[2],
                     const uint8_t* const marks[2], uint32_t W, uint32_t H) {
    m->ok = false;
    if (W % 16 != 0 || W < 16) return false;
    // one set of maps per blur radius: the box is the window, 32 rows plus a
    // halo of R on each side
    for (int i = 0; i < 2; i++) {
        if (!encode_2d(&m->trail[i], trail[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, W, H, kTrailBoxCols,
                       kTmaRows + 2) ||
            !encode_2d(&m->counts[i], counts[i], CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, W, H, kTrailBoxCols,
                       kTmaRows + 2) ||
            !encode_2d(&m->marks[i], marks[i], CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, W, H, kMarkBoxCols, kTmaRows + 2) ||
            !encode_2d(&m->trail_r2[i], trail[i], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, W, H, kTrailBoxCols,
                       kTmaRows + 4) ||
            !encode_2d(&m->counts_r2[i], counts[i], CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, W, H, kTrailBoxCols,
                       kTmaRows + 4) ||
            !encode_2d(&m->marks_r2[i], marks[i], CU_TENSOR_MAP_DATA_TYPE_UINT8, 1, W, H, kMarkBoxCols,
                       kTmaRows + 4))
            return false;
    }
    m->ok = true;
    return true;
}

cudaError_t launch_trail_tma(const DevParams& p, const TrailMaps& maps, int cur, const float* in,
                             const uint32_t* counts_in, float* out, uint32_t* counts_zero, cudaStream_t s,
                             const cudaAccessPolicyWindow* win, bool pdl) {
    return launch_tma<uint32_t>(p, maps, cur, in, counts_in, out, counts_zero, s, win, pdl);
}

cudaError_t launch_trail_tma_marks(const DevParams& p, const TrailMaps& maps, int cur, const float* in,
                                   const uint8_t* marks_in, float* out, uint8_t* marks_zero, cudaStream_t s,
                                   const cudaAccessPolicyWindow* win, bool pdl) {
    return launch_tma<uint8_t>(p, maps, cur, in, marks_in, out, marks_zero, s, win, pdl);
}

bool trail_tma_take_error() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_wait_failed, sizeof v) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (v) {
        const int zero = 0;
        cudaMemcpyToSymbol(g_tma_wait_failed, &zero, sizeof zero);
    }
    return v != 0;
}

} // namespace slime
