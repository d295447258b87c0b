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
// Blocks whose box destinations were not 128-byte aligned in the shared
// window (they took the plain-load path instead; 0 expected).
__device__ int g_tma_misaligned;

// Rounds a byte count up to a 128-byte boundary (a tensor copy's shared
// destination must be 128-byte aligned).
__host__ __device__ constexpr size_t align128(size_t b) { return (b + 127) / 128 * 128; }

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


// Parity wait on a barrier; false after ~2^31 cycles (about a second).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
    const long long t0 = clock64();
    while (true) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > (1ll << 31)) return false;
    }
}

// Shared-memory layout of a block: the mbarrier, then the trail box, then the
// deposit box, each box on a 128-byte boundary.
template <int R, class D>
struct Layout {
    static constexpr int WR = kTmaRows + 2 * R;
    static constexpr size_t trail_off = 128;
    static constexpr size_t dep_off = trail_off + align128(sizeof(float) * WR * kTrailBoxCols);
    static constexpr size_t bytes = dep_off + sizeof(D) * WR * DepBox<D>::cols;
    static constexpr uint32_t tx_bytes = (uint32_t)(sizeof(float) * WR * kTrailBoxCols + sizeof(D) * WR * DepBox<D>::cols);
};

// One block, one tile.  Every tile's window comes by the two tensor copies;
// a box that reaches outside the array is filled with zeros there, and a
// border tile then overwrites those halo cells with the opposite side's cells
// (plain loads of the wrapped rows and columns only).  One thread waits on
// the barrier; the others wait at the block barrier after it.
template <int R, bool kGauss, int kDecay, class D>
__global__ void __launch_bounds__(kTmaThreads) trail_tma_kernel(const __grid_constant__ DevParams p,
                                                                const __grid_constant__ CUtensorMap map_t,
                                                                const __grid_constant__ CUtensorMap map_d,
                                                                const float* __restrict__ in,
                                                                const D* __restrict__ din, float* __restrict__ out,
                                                                D* __restrict__ dzero) {
    constexpr bool kMarks = sizeof(D) == 1;
    typedef Layout<R, D> L;
    constexpr int WR = L::WR;
    constexpr int DC = DepBox<D>::cols, DL = DepBox<D>::lead;
    constexpr int WC = kTmaCols + 2 * R; // window columns x0-R .. x0+127+R
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem);
    float* tw = reinterpret_cast<float*>(smem + L::trail_off); // WR x kTrailBoxCols
    D* dw = reinterpret_cast<D*>(smem + L::dep_off);           // WR x DC
    __shared__ int fail;
    const int W = p.W, H = p.H;
    const int x0 = blockIdx.x * kTmaCols, y0 = blockIdx.y * kTmaRows;
    // the copies' destinations must be 128-byte aligned in the shared window:
    // checked, and a misaligned block loads its whole window by plain loads
    const bool aligned = ((smem_u32(tw) | smem_u32(dw)) & 127u) == 0u;
    const bool border = x0 - R < 0 || x0 + kTmaCols + R > W || y0 - R < 0 || y0 - R + WR > H;
    if (aligned) {
        if (threadIdx.x == 0) {
            fail = 0;
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                         "r"(L::tx_bytes)
                         : "memory");
            // the trail this reads is not written by the agent pass
            tma_load_2d(tw, &map_t, x0 - kTrailLead, y0 - R, bar);
        }
        // the deposit record is the agent pass's output
        pdl_wait();
        if (threadIdx.x == 0) {
            tma_load_2d(dw, &map_d, x0 - DL, y0 - R, bar);
            if (!mbar_wait(bar, 0)) {
                fail = 1;
                atomicExch(&g_tma_wait_failed, 1);
            }
        }
        pdl_trigger();
        __syncthreads();
        if (fail) return;
        if (border) {
            // the window's cells outside the array: the opposite side's
            for (int i = threadIdx.x; i < WR * WC; i += kTmaThreads) {
                const int r = i / WC, c = i - r * WC - R;
                const int gy = y0 - R + r, gx = x0 + c;
                if (gy >= 0 && gy < H && gx >= 0 && gx < W) continue;
                const size_t gi = (size_t)wrap_coord(gy, H) * W + wrap_coord(gx, W);
                tw[r * kTrailBoxCols + kTrailLead + c] = __ldg(in + gi);
                dw[r * DC + DL + c] = __ldg(din + gi);
            }
            __syncthreads();
        }
        // fold + decay of the window's cells in place
        for (int i = threadIdx.x; i < WR * WC; i += kTmaThreads) {
            const int r = i / WC, c = i - r * WC - R; // c = column - x0
            float& v = tw[r * kTrailBoxCols + kTrailLead + c];
            v = apply_decay_m<kDecay>(p, fold_dep<kMarks>(v, (uint32_t)dw[r * DC + DL + c], p.dep));
        }
    } else {
        if (threadIdx.x == 0) atomicAdd(&g_tma_misaligned, 1);
        pdl_wait();
        pdl_trigger();
        for (int i = threadIdx.x; i < WR * WC; i += kTmaThreads) {
            const int r = i / WC, c = i - r * WC - R;
            const size_t gi = (size_t)wrap_coord(y0 - R + r, H) * W + wrap_coord(x0 + c, W);
            tw[r * kTrailBoxCols + kTrailLead + c] =
                apply_decay_m<kDecay>(p, fold_dep<kMarks>(__ldg(in + gi), (uint32_t)__ldg(din + gi), p.dep));
        }
    }
    __syncthreads();

    // blur: lane -> 4 columns, warp -> 4 output rows, the window's rows walked
    // once with a rolling window of 2R+1 rows in registers (the horizontal
    // pass of each row for the Gaussian, the row itself for the box)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c0 = lane * 4;
    const int ry = warp * 4; // first output row of the warp within the tile
    const int x = x0 + c0;
    constexpr int NWIN = 2 * R + 1;
    float win[NWIN][4 + 2 * R]; // box: window rows, columns c0-R .. c0+3+R
    float hwin[NWIN][4];        // Gaussian: their horizontal passes
    float ctr[NWIN][4];         // the rows' own cells (the mix's centre)
#pragma unroll
    for (int r = 0; r < 4 + 2 * R; r++) {
        // shift the window
#pragma unroll
        for (int q = 0; q < NWIN - 1; q++) {
#pragma unroll
            for (int j = 0; j < 4; j++) ctr[q][j] = ctr[q + 1][j];
            if (kGauss) {
#pragma unroll
                for (int j = 0; j < 4; j++) hwin[q][j] = hwin[q + 1][j];
            } else {
#pragma unroll
                for (int j = 0; j < 4 + 2 * R; j++) win[q][j] = win[q + 1][j];
            }
        }
        const float* row = tw + (ry + r) * kTrailBoxCols + kTrailLead;
        const float4 v = *reinterpret_cast<const float4*>(row + c0);
        const float d[4] = {v.x, v.y, v.z, v.w};
        float e[4 + 2 * R];
#pragma unroll
        for (int j = 0; j < 4; j++) e[R + j] = d[j];
#pragma unroll
        for (int j = 0; j < R; j++) {
            e[j] = __shfl_up_sync(0xffffffffu, d[4 - R + j], 1);
            e[R + 4 + j] = __shfl_down_sync(0xffffffffu, d[j], 1);
        }
        if (lane == 0) {
#pragma unroll
            for (int j = 0; j < R; j++) e[j] = row[c0 - R + j];
        }
        if (lane == 31) {
#pragma unroll
            for (int j = 0; j < R; j++) e[R + 4 + j] = row[c0 + 4 + j];
        }
#pragma unroll
        for (int j = 0; j < 4; j++) ctr[NWIN - 1][j] = d[j];
        if (kGauss) {
#pragma unroll
            for (int j = 0; j < 4; j++) {
                float acc = 0.0f;
#pragma unroll
                for (int q = 0; q <= 2 * R; q++) acc = slm_fma(p.w[q], e[j + q], acc);
                hwin[NWIN - 1][j] = acc;
            }
        } else {
#pragma unroll
            for (int j = 0; j < 4 + 2 * R; j++) win[NWIN - 1][j] = e[j];
        }
        if (r < 2 * R) continue;
        const int y = y0 + ry + r - 2 * R;
        if (y >= H || x >= W) continue;
        float res[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float center = ctr[R][j];
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
                    for (int dx = 0; dx < 3; dx++) sum = slm_add(sum, win[dy][j + dx]);
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
    typedef Layout<R, D> L;
    const size_t smem = L::bytes;
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
    // byte-mark rows must be whole 16-byte units for a tensor map, and the
    // boxes (160 columns of marks, 36 rows) no larger than the array
    return p.W % 16 == 0 && p.W >= kMarkBoxCols && p.H >= kTmaRows + 4 && R >= 1 && R <= 2;
}

bool make_trail_maps(TrailMaps* m, const float* const trail[2], const uint32_t* const counts[2],
                     const uint8_t* const marks[2], uint32_t W, uint32_t H) {
    m->ok = false;
    if (W % 16 != 0 || W < (uint32_t)kMarkBoxCols || H < (uint32_t)kTmaRows + 4) return false;
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

int trail_tma_misaligned_blocks() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tma_misaligned, sizeof v) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    return v;
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
