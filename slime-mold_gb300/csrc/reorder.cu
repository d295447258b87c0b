// reorder.cu - Morton reordering of agent slots.
//
// Agents that sit in nearby cells sense and deposit into nearby trail lines;
// placing them in neighbouring slots turns the agent pass's scattered 4-byte
// gathers into a few shared lines per warp.  The order of slots does not
// change any result: sensing reads the pre-step trail, deposits are counted,
// and every slot carries its original id (which seeds the jitter hash), so the
// reorder is a pure performance transform.
//
// Counting sort on the Morton code of the agent's (cell >> cell_log2):
// key + histogram, exclusive scan, scatter to scratch, copy back.  The order
// inside one key is whatever the scatter atomics produce.  Agents whose id is
// at or above `visited` (those the reference's dispatch never updates) get
// one key past every Morton code, so they end up in the last slots and the
// updated agents fill the first ones.
#include "kernels.h"

namespace slime {
namespace {

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

__device__ __forceinline__ uint32_t spread_bits(uint32_t v) {
    v &= 0xffffu;
    v = (v | (v << 8)) & 0x00ff00ffu;
    v = (v | (v << 4)) & 0x0f0f0f0fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}

// Agents that are already nearly in order share keys with their warp
// neighbours (about 2^(2 cell_log2) per key at one agent per cell), so the
// histogram and the slot claims are aggregated per warp: the lanes holding
// one key elect a leader that adds the group's size with a single atomic.
__global__ void key_hist_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                const uint32_t* __restrict__ ids, uint64_t visited, uint32_t frozen_key, uint64_t n,
                                int W, int H, int cl, uint32_t* __restrict__ keys, uint32_t* __restrict__ hist) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int cx = min(max(slm_f2i(x[i]), 0), W - 1) >> cl;
    int cy = min(max(slm_f2i(y[i]), 0), H - 1) >> cl;
    uint32_t k = spread_bits((uint32_t)cx) | (spread_bits((uint32_t)cy) << 1);
    if (visited < n && ids[i] >= visited) k = frozen_key;
    keys[i] = k;
    const unsigned group = __match_any_sync(__activemask(), k);
    if ((int)(threadIdx.x & 31) == __ffs(group) - 1) atomicAdd(hist + k, (uint32_t)__popc(group));
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sums, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t ws = (lane < (int)(blockDim.x >> 5)) ? warp_sums[lane] : 0u;
        uint32_t wi = ws;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        warp_sums[lane] = wi - ws;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    uint32_t r = warp_sums[warp] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t* __restrict__ in, uint64_t n,
                                                                   uint32_t* __restrict__ block_sums) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++)
        if (base + j < n) s += in[base + j];
    block_exclusive_scan(s, ws, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// Single block: exclusive scan of the block sums in place.
__global__ void __launch_bounds__(kScanThreads) scan_block_sums_kernel(uint32_t* __restrict__ sums, uint32_t nb) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    uint32_t carry = 0;
    for (uint32_t base = 0; base < nb; base += kScanThreads) {
        uint32_t i = base + threadIdx.x;
        uint32_t v = i < nb ? sums[i] : 0u;
        uint32_t ex = block_exclusive_scan(v, ws, &tot);
        if (i < nb) sums[i] = carry + ex;
        carry += tot;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(uint32_t* __restrict__ data, uint64_t n,
                                                                  const uint32_t* __restrict__ block_offsets) {
    __shared__ uint32_t ws[32];
    __shared__ uint32_t tot;
    uint64_t base = (uint64_t)blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint32_t s = 0;
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        v[j] = (base + j < n) ? data[base + j] : 0u;
        s += v[j];
    }
    uint32_t ex = block_exclusive_scan(s, ws, &tot) + block_offsets[blockIdx.x];
#pragma unroll
    for (int j = 0; j < kScanItems; j++) {
        if (base + j < n) data[base + j] = ex;
        ex += v[j];
    }
}

__global__ void scatter_kernel(const float* __restrict__ x, const float* __restrict__ y,
                               const float* __restrict__ th, const float* __restrict__ v,
                               const uint32_t* __restrict__ ids, const uint32_t* __restrict__ keys, uint64_t n,
                               uint32_t* __restrict__ offsets, float* __restrict__ tx, float* __restrict__ ty,
                               float* __restrict__ tth, float* __restrict__ tv, uint32_t* __restrict__ tid) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = keys[i];
    const unsigned active = __activemask();
    const unsigned group = __match_any_sync(active, k);
    const int lane = (int)(threadIdx.x & 31);
    const int leader = __ffs(group) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(offsets + k, (uint32_t)__popc(group));
    base = __shfl_sync(active, base, leader);
    // slots of one key are claimed in lane order within the warp
    const uint32_t pos = base + (uint32_t)__popc(group & ((1u << lane) - 1u));
    tx[pos] = x[i];
    ty[pos] = y[i];
    tth[pos] = th[i];
    tv[pos] = v[i];
    tid[pos] = ids[i];
}

__global__ void iota_kernel(uint32_t* __restrict__ ids, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ids[i] = (uint32_t)i;
}

inline size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

} // namespace

cudaError_t launch_iota(uint32_t* ids, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    iota_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(ids, n);
    return cudaGetLastError();
}

cudaError_t launch_reorder(AgentsSoA& a, uint32_t W, uint32_t H, int cell_log2, ReorderScratch& scratch,
                           cudaStream_t s, uint64_t visited) {
    if (a.n == 0) return cudaSuccess;
    if (!a.ids) return cudaErrorInvalidValue; // the caller installs identity ids first
    if (cell_log2 < 0) cell_log2 = 0;
    if (cell_log2 > 15) cell_log2 = 15;
    uint32_t dx = (W + (1u << cell_log2) - 1) >> cell_log2;
    uint32_t dy = (H + (1u << cell_log2) - 1) >> cell_log2;
    uint32_t d = dx > dy ? dx : dy;
    int L = 0;
    while ((1u << L) < d) L++;
    if (L > 16) return cudaErrorInvalidValue;
    const bool partition = visited < a.n;
    if (partition && L > 15) return cudaErrorInvalidValue; // no key left past the Morton codes
    const uint32_t frozen_key = (uint32_t)(1ull << (2 * L));
    uint64_t nb = (1ull << (2 * L)) + (partition ? 1 : 0);
    uint64_t nblk = (nb + kScanTile - 1) / kScanTile;
    const uint64_t n = a.n;
    size_t need = align256(4 * n) /*keys*/ + align256(4 * nb) /*hist*/ + align256(4 * nblk) /*block sums*/ +
                  4 * align256(4 * n) /*x y th v*/ + align256(4 * n) /*ids*/;
    if (scratch.bytes < need) {
        if (scratch.buf) dev_free(scratch.buf);
        scratch.buf = nullptr;
        scratch.bytes = 0;
        cudaError_t e = dev_alloc((void**)&scratch.buf, need);
        if (e != cudaSuccess) return e;
        scratch.bytes = need;
    }
    char* p = (char*)scratch.buf;
    uint32_t* keys = (uint32_t*)p; p += align256(4 * n);
    uint32_t* hist = (uint32_t*)p; p += align256(4 * nb);
    uint32_t* bsum = (uint32_t*)p; p += align256(4 * nblk);
    float* tx = (float*)p; p += align256(4 * n);
    float* ty = (float*)p; p += align256(4 * n);
    float* tth = (float*)p; p += align256(4 * n);
    float* tv = (float*)p; p += align256(4 * n);
    uint32_t* tid = (uint32_t*)p;

    cudaError_t e = cudaMemsetAsync(hist, 0, 4 * nb, s);
    if (e != cudaSuccess) return e;
    unsigned blocks = (unsigned)((n + 255) / 256);
    key_hist_kernel<<<blocks, 256, 0, s>>>(a.x, a.y, a.ids, visited, frozen_key, n, (int)W, (int)H, cell_log2, keys,
                                          hist);
    scan_reduce_kernel<<<(unsigned)nblk, kScanThreads, 0, s>>>(hist, nb, bsum);
    scan_block_sums_kernel<<<1, kScanThreads, 0, s>>>(bsum, (uint32_t)nblk);
    scan_apply_kernel<<<(unsigned)nblk, kScanThreads, 0, s>>>(hist, nb, bsum);
    scatter_kernel<<<blocks, 256, 0, s>>>(a.x, a.y, a.th, a.v, a.ids, keys, n, hist, tx, ty, tth, tv, tid);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(a.x, tx, 4 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(a.y, ty, 4 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(a.th, tth, 4 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(a.v, tv, 4 * n, cudaMemcpyDeviceToDevice, s)) != cudaSuccess) return e;
    return cudaMemcpyAsync(a.ids, tid, 4 * n, cudaMemcpyDeviceToDevice, s);
}

} // namespace slime
