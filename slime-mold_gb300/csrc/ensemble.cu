// ensemble.cu - independent colonies of uneven sizes stepped together.
//
// All colonies' agents live in one SoA block (each colony padded to a
// multiple of 128 slots) and all trails/counts in one ping-pong pair of
// buffers.  Two engines step them (the autotuner times both):
//
// SLIME_ENSEMBLE_COOPERATIVE - one cooperative launch per step runs
//   phase 1: agent work items (256 groups of 4 or 2 agents of one colony
//            per block item),
//   a grid-wide barrier (bounded spin: gives up after about a second and
//            reports SLIME_ERR_DEVICE_TIMEOUT instead of hanging),
//   phase 2: trail strips (128 columns x ROWS rows of one colony per warp
//            item) through the same streaming code as the single-colony
//            kernel.
// SLIME_ENSEMBLE_LANES - every colony's steps are a chain of the
//   single-colony kernels (persistent agent pass, streaming trail pass, PDL
//   between them, the colony's parameters as kernel arguments) on one of up
//   to 64 capture lanes; the lanes fork from and join the ensemble's stream
//   and a chunk of steps is captured as one CUDA graph, so the chains of
//   different colonies run concurrently: small colonies fill the SMs that a
//   large colony's pass leaves idle, and the trail passes (memory-bound)
//   overlap the agent passes (issue-bound) of other colonies.
// Each colony keeps its own parameter block, so the colonies are exactly the
// runs a single Simulation would produce for them (the tests compare bit for
// bit).  The blur mode and radius must be common to all colonies (they select
// the compiled strip variant); sigma, decay, diffusion and the agent
// parameters may differ.
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "agent_step.cuh"
#include "ctx.h"
#include "kernels.h"
#include "trail_stream.cuh"

using namespace slime;

namespace {

constexpr int kEnsThreads = 256;

struct DevColony {
    DevParams p;
    uint64_t agent_off; // first slot of the colony in each SoA array
    uint64_t n;         // live agents
    uint64_t trail_off; // first cell of the colony in the trail/count buffers
    int32_t warps_x;    // 128-column strips per row band
    int32_t pad;
    cudaTextureObject_t tex[2]; // gather textures over the colony's two trails (0 = none)
};

struct GridBarrier {
    unsigned int count;
    unsigned int gen;
    int error;
    int pad;
};

struct Colony {
    uint32_t W, H;
    uint64_t n, n_pad, agent_off, trail_off;
    SlimeParams params;
    DevParams dev;
    cudaTextureObject_t tex[2] = {0, 0};
    // deposit records (as the single-colony context keeps them): whether the
    // trail is clean (finite values >= 0, or +inf) so that byte marks can
    // stand in for counts, which of the colony's two count / mark regions
    // hold deposits, and the record the captured graphs use
    bool trail_clean = true;
    bool counts_dirty[2] = {false, false};
    bool marks_dirty[2] = {false, false};
    bool marks = false;
};

// Bounded grid barrier: every block arrives once; the last one to arrive
// releases the others.  A waiter gives up after ~1 s of clock64() cycles,
// flags the error and returns false (the kernel then skips its second phase).
__device__ bool grid_barrier(GridBarrier* b, unsigned nblocks, long long limit_cycles = 2000000000ll) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        volatile unsigned int* vgen = &b->gen;
        unsigned int gen = *vgen;
        __threadfence();
        unsigned int arrived = atomicAdd(&b->count, 1u);
        if (arrived == nblocks - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            long long t0 = clock64();
            while (*vgen == gen) {
                if (clock64() - t0 > limit_cycles) {
                    atomicExch(&b->error, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Self-test of the bounded wait: one block waits at a barrier sized for two,
// so the release never comes and the wait must give up by itself.
__global__ void barrier_timeout_kernel(GridBarrier* bar, long long limit_cycles, int* reached_after) {
    bool ok = grid_barrier(bar, 2, limit_cycles);
    if (threadIdx.x == 0) *reached_after = ok ? 1 : 2;
}

// Four consecutive agents of one colony (the last group may be partial).
template <class Trail>
__device__ __forceinline__ void steps4(const DevParams& sp, float4& x, float4& y, float4& th, float4& v, const uint4& id,
                                       uint64_t base, uint64_t n, const Trail& trail, int& c0, int& c1, int& c2,
                                       int& c3) {
    if (base + 4 <= n) { // full group: no per-agent branch
        c0 = agent_step(sp, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
        c1 = agent_step(sp, x.y, y.y, th.y, v.y, (int32_t)id.y, trail);
        c2 = agent_step(sp, x.z, y.z, th.z, v.z, (int32_t)id.z, trail);
        c3 = agent_step(sp, x.w, y.w, th.w, v.w, (int32_t)id.w, trail);
    } else {
        c0 = agent_step(sp, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
        if (base + 1 < n) c1 = agent_step(sp, x.y, y.y, th.y, v.y, (int32_t)id.y, trail);
        if (base + 2 < n) c2 = agent_step(sp, x.z, y.z, th.z, v.z, (int32_t)id.z, trail);
        if (base + 3 < n) c3 = agent_step(sp, x.w, y.w, th.w, v.w, (int32_t)id.w, trail);
    }
}

// Two consecutive agents of one colony stepped as one pair (agent_step2), or
// the first alone when the second is past the colony's end.
template <class Trail>
__device__ __forceinline__ void steps2(const DevParams& sp, float2& x, float2& y, float2& th, float2& v, const uint2& id,
                                       uint64_t base, uint64_t n, const Trail& trail, int& c0, int& c1) {
    if (base + 2 <= n) {
        agent_step2(sp, x.x, y.x, th.x, v.x, (int32_t)id.x, x.y, y.y, th.y, v.y, (int32_t)id.y, trail, c0, c1);
    } else {
        c0 = agent_step(sp, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
    }
}

// One agent work item of a block: APT consecutive agents of one colony per
// thread (APT = 4: float4 accesses, each agent stepped alone; APT = 2: float2
// accesses, the two stepped as one pair).
template <int APT>
__device__ __forceinline__ void agent_item(const DevParams& sp, const DevColony& c, uint32_t g0, int parity,
                                           float* __restrict__ X, float* __restrict__ Y, float* __restrict__ TH,
                                           float* __restrict__ V, const uint32_t* __restrict__ IDS,
                                           const float* __restrict__ trail_in, uint32_t* counts_in) {
    const uint64_t g = (uint64_t)g0 + threadIdx.x; // APT-agent group within the colony
    const uint64_t base = APT * g;
    if (base >= c.n) return;
    const uint64_t slot = c.agent_off + base;
    uint32_t* counts = counts_in + c.trail_off;
    const cudaTextureObject_t tex = c.tex[parity];
    if (APT == 4) {
        float4* px = reinterpret_cast<float4*>(X + slot);
        float4* py = reinterpret_cast<float4*>(Y + slot);
        float4* pt = reinterpret_cast<float4*>(TH + slot);
        float4* pv = reinterpret_cast<float4*>(V + slot);
        float4 x = __ldcs(px), y = __ldcs(py), th = __ldcs(pt), v = __ldcs(pv);
        const uint4 id = __ldcs(reinterpret_cast<const uint4*>(IDS + slot)); // colony-local agent ids
        int c0, c1 = -1, c2 = -1, c3 = -1;
        // the colony's trail through its gather texture when it has one,
        // else through the padded buffer (block-uniform choice)
        if (tex) {
            steps4(sp, x, y, th, v, id, base, c.n, TrailTex{tex}, c0, c1, c2, c3);
        } else {
            steps4(sp, x, y, th, v, id, base, c.n, TrailPtr{trail_in + c.trail_off}, c0, c1, c2, c3);
        }
        if (c0 >= 0) atomicAdd(counts + c0, 1u);
        if (c1 >= 0) atomicAdd(counts + c1, 1u);
        if (c2 >= 0) atomicAdd(counts + c2, 1u);
        if (c3 >= 0) atomicAdd(counts + c3, 1u);
        __stcs(px, x);
        __stcs(py, y);
        __stcs(pt, th);
        __stcs(pv, v);
    } else {
        float2* px = reinterpret_cast<float2*>(X + slot);
        float2* py = reinterpret_cast<float2*>(Y + slot);
        float2* pt = reinterpret_cast<float2*>(TH + slot);
        float2* pv = reinterpret_cast<float2*>(V + slot);
        float2 x = __ldcs(px), y = __ldcs(py), th = __ldcs(pt), v = __ldcs(pv);
        const uint2 id = __ldcs(reinterpret_cast<const uint2*>(IDS + slot));
        int c0, c1 = -1;
        if (tex) {
            steps2(sp, x, y, th, v, id, base, c.n, TrailTex{tex}, c0, c1);
        } else {
            steps2(sp, x, y, th, v, id, base, c.n, TrailPtr{trail_in + c.trail_off}, c0, c1);
        }
        if (c0 >= 0) atomicAdd(counts + c0, 1u);
        if (c1 >= 0) atomicAdd(counts + c1, 1u);
        __stcs(px, x);
        __stcs(py, y);
        __stcs(pt, th);
        __stcs(pv, v);
    }
}

// Four agents per thread at four blocks per SM (a 64-register cap; a few
// bytes spilled), or two per thread stepped as one pair at three blocks per
// SM (80 registers): the autotuner times both (on 64 colonies of 256^2 to
// 2048^2, 3.54 against 3.70 ms per step; the pair loses the prefetch of the
// next group that the plain persistent kernel has).
template <int R, bool kGauss, int ROWS, int APT>
__global__ void __launch_bounds__(kEnsThreads, APT == 4 ? 4 : 3) ensemble_step_kernel(
    const DevColony* __restrict__ cols, const uint2* __restrict__ agent_items, uint32_t n_agent_items,
    const uint4* __restrict__ strip_items, uint32_t n_strip_items, float* __restrict__ X, float* __restrict__ Y,
    float* __restrict__ TH, float* __restrict__ V, const uint32_t* __restrict__ IDS, const float* __restrict__ trail_in,
    uint32_t* counts_in, float* __restrict__ trail_out, uint32_t* __restrict__ counts_zero, GridBarrier* bar,
    int parity) {
    __shared__ DevParams sp;
    // ---- phase 1: agents
    for (uint32_t item = blockIdx.x; item < n_agent_items; item += gridDim.x) {
        const uint2 it = agent_items[item];
        __syncthreads();
        {
            const uint32_t* src = reinterpret_cast<const uint32_t*>(&cols[it.x].p);
            uint32_t* dst = reinterpret_cast<uint32_t*>(&sp);
            for (int w = threadIdx.x; w < (int)(sizeof(DevParams) / 4); w += kEnsThreads) dst[w] = src[w];
        }
        __syncthreads();
        agent_item<APT>(sp, cols[it.x], it.y, parity, X, Y, TH, V, IDS, trail_in, counts_in);
    }
    // ---- grid-wide barrier: all deposits of this step are counted
    __threadfence();
    if (!grid_barrier(bar, gridDim.x)) return;
    // ---- phase 2: trail strips, one warp per item
    const uint32_t warps = gridDim.x * (kEnsThreads / 32);
    const uint32_t gw = blockIdx.x * (kEnsThreads / 32) + (threadIdx.x >> 5);
    for (uint32_t item = gw; item < n_strip_items; item += warps) {
        const uint4 it = strip_items[item];
        const DevColony& c = cols[it.x];
        process_strip<R, kGauss, ROWS, true, false>(c.p, trail_in + c.trail_off, counts_in + c.trail_off,
                                             trail_out + c.trail_off, counts_zero + c.trail_off, (int)it.y,
                                             (int)it.z);
    }
}

typedef void (*EnsKernel)(const DevColony*, const uint2*, uint32_t, const uint4*, uint32_t, float*, float*, float*,
                          float*, const uint32_t*, const float*, uint32_t*, float*, uint32_t*, GridBarrier*, int);

template <int ROWS, int APT>
EnsKernel pick_rows(int R, bool gauss) {
    if (!gauss) return ensemble_step_kernel<1, false, ROWS, APT>;
    if (R == 1) return ensemble_step_kernel<1, true, ROWS, APT>;
    return ensemble_step_kernel<2, true, ROWS, APT>;
}

template <int APT>
EnsKernel pick_apt(int rows, int R, bool gauss) {
    switch (rows) {
    case 8: return pick_rows<8, APT>(R, gauss);
    case 32: return pick_rows<32, APT>(R, gauss);
    default: return pick_rows<16, APT>(R, gauss);
    }
}

EnsKernel pick_kernel(int rows, int R, bool gauss, int apt) {
    return apt == 2 ? pick_apt<2>(rows, R, gauss) : pick_apt<4>(rows, R, gauss);
}

} // namespace

struct slime_ensemble {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<Colony> colonies;
    uint64_t total_slots = 0, total_cells = 0;
    float* agent_block = nullptr; // x | y | angle | speed, total_slots each
    uint32_t* ids = nullptr;      // slot -> colony-local agent id (identity until reordered)
    uint32_t reorder_every = 0;
    int reorder_cell_log2 = 2;
    uint64_t steps_done = 0;
    uint64_t last_reorder_step = ~0ull;
    ReorderScratch reorder;
    ReorderScratch lane_reorder[3]; // sort scratch of the lanes engine's concurrent reorders (with `reorder`)
    float* trail[2] = {nullptr, nullptr};
    uint32_t* counts[2] = {nullptr, nullptr};
    uint8_t* marks[2] = {nullptr, nullptr}; // per-cell deposit marks (lanes engine; allocated on first use)
    int cur = 0;
    DevColony* d_cols = nullptr;
    uint2* d_agent_items = nullptr;
    uint32_t n_agent_items = 0;
    uint4* d_strip_items = nullptr;
    uint32_t n_strip_items = 0;
    GridBarrier* d_bar = nullptr;
    float4* staging = nullptr;
    size_t staging_bytes = 0;
    int rows = 16;
    int apt = 4; // agents per thread of the agent phase (4 or 2)
    int R = 1;
    bool gauss = false;
    int grid = 0;
    int blocks_per_sm = 0;
    bool use_graphs = true;
    bool last_chunk_graph = false; // the last chunk of steps replayed a graph
    int engine = SLIME_ENSEMBLE_COOPERATIVE;
    int lane_agent_shape = 13; // agent-kernel shape of the lanes engine (persistent, texture gather)
    int lane_trail_tile = 8;   // trail tile of the lanes engine (streaming, 16-row strips)
    int max_lanes = 0;         // lanes of the lanes engine (0: one per colony, at most 64)
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> lane_ev;
    cudaEvent_t fork_ev = nullptr;
    std::vector<std::vector<uint32_t>> lane_cols; // colonies of each lane, in launch order
    std::map<std::pair<uint32_t, int>, cudaGraphExec_t> graphs;
    uint64_t launches = 0;
    std::string err;
};

namespace {

int ens_fail(slime_ensemble* e, int code, const char* msg) {
    e->err = msg;
    return code;
}

#define ECK(expr, what)                                                                                     \
    do {                                                                                                    \
        cudaError_t _e = (expr);                                                                            \
        if (_e != cudaSuccess) return cuda_error(e->err, _e, what);                                         \
    } while (0)

void ens_invalidate(slime_ensemble* e) {
    for (auto& kv : e->graphs) cudaGraphExecDestroy(kv.second);
    e->graphs.clear();
}

int upload_cols(slime_ensemble* e) {
    std::vector<DevColony> dc(e->colonies.size());
    for (size_t j = 0; j < e->colonies.size(); j++) {
        const Colony& c = e->colonies[j];
        memset(&dc[j], 0, sizeof(DevColony));
        dc[j].p = c.dev;
        dc[j].agent_off = c.agent_off;
        dc[j].n = c.n;
        dc[j].trail_off = c.trail_off;
        dc[j].warps_x = (int32_t)((c.W + 127) / 128);
        dc[j].tex[0] = c.tex[0];
        dc[j].tex[1] = c.tex[1];
    }
    ECK(cudaMemcpyAsync(e->d_cols, dc.data(), dc.size() * sizeof(DevColony), cudaMemcpyHostToDevice, e->stream),
        "uploading colony table");
    ECK(cudaStreamSynchronize(e->stream), "uploading colony table");
    return SLIME_OK;
}

int build_strip_items(slime_ensemble* e) {
    std::vector<uint4> items;
    for (size_t j = 0; j < e->colonies.size(); j++) {
        const Colony& c = e->colonies[j];
        uint32_t wx = (c.W + 127) / 128, strips = (c.H + e->rows - 1) / e->rows;
        for (uint32_t rs = 0; rs < strips; rs++)
            for (uint32_t cw = 0; cw < wx; cw++) items.push_back(make_uint4((uint32_t)j, cw, rs, 0));
    }
    if (e->d_strip_items) dev_free(e->d_strip_items);
    e->d_strip_items = nullptr;
    ECK(dev_alloc((void**)&e->d_strip_items, items.size() * sizeof(uint4)), "allocating strip table");
    ECK(cudaMemcpy(e->d_strip_items, items.data(), items.size() * sizeof(uint4), cudaMemcpyHostToDevice),
        "uploading strip table");
    e->n_strip_items = (uint32_t)items.size();
    return SLIME_OK;
}

// Agent work items: 256 groups of `apt` agents of one colony each.
int build_agent_items(slime_ensemble* e) {
    std::vector<uint2> ai;
    for (uint32_t j = 0; j < (uint32_t)e->colonies.size(); j++) {
        const uint64_t groups = (e->colonies[j].n + e->apt - 1) / e->apt;
        for (uint64_t g0 = 0; g0 < groups; g0 += kEnsThreads) ai.push_back(make_uint2(j, (uint32_t)g0));
    }
    if (e->d_agent_items) dev_free(e->d_agent_items);
    e->d_agent_items = nullptr;
    e->n_agent_items = 0;
    ECK(dev_alloc((void**)&e->d_agent_items, (ai.size() ? ai.size() : 1) * sizeof(uint2)), "allocating agent items");
    if (ai.size())
        ECK(cudaMemcpy(e->d_agent_items, ai.data(), ai.size() * sizeof(uint2), cudaMemcpyHostToDevice),
            "uploading agent items");
    e->n_agent_items = (uint32_t)ai.size();
    return SLIME_OK;
}

int size_grid(slime_ensemble* e) {
    EnsKernel k = pick_kernel(e->rows, e->R, e->gauss, e->apt);
    int per_sm = 0, sms = 0;
    ECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kEnsThreads, 0), "occupancy query");
    ECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device), "SM count");
    if (per_sm < 1) return ens_fail(e, SLIME_ERR_CUDA, "ensemble kernel cannot be resident");
    int want = e->blocks_per_sm > 0 ? (e->blocks_per_sm < per_sm ? e->blocks_per_sm : per_sm) : per_sm;
    e->grid = want * sms;
    return SLIME_OK;
}

cudaError_t enqueue_ens_step(slime_ensemble* e) {
    const int cur = e->cur;
    EnsKernel k = pick_kernel(e->rows, e->R, e->gauss, e->apt);
    float* X = e->agent_block;
    float* Y = X + e->total_slots;
    float* TH = Y + e->total_slots;
    float* V = TH + e->total_slots;
    const DevColony* cols = e->d_cols;
    const uint2* ai = e->d_agent_items;
    uint32_t nai = e->n_agent_items;
    const uint4* si = e->d_strip_items;
    uint32_t nsi = e->n_strip_items;
    const float* tin = e->trail[cur];
    uint32_t* cin = e->counts[cur];
    float* tout = e->trail[1 - cur];
    uint32_t* cz = e->counts[1 - cur];
    GridBarrier* bar = e->d_bar;
    const uint32_t* ids = e->ids;
    int parity = cur;
    void* args[] = {&cols, &ai, &nai, &si, &nsi, &X, &Y, &TH, &V, &ids, &tin, &cin, &tout, &cz, &bar, &parity};
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(e->grid);
    cfg.blockDim = dim3(kEnsThreads);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = e->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t err = cudaLaunchKernelExC(&cfg, (const void*)k, args);
    if (err != cudaSuccess) return err;
    e->cur = 1 - cur;
    return cudaSuccess;
}

AgentsSoA colony_soa(slime_ensemble* e, const Colony& c) {
    AgentsSoA a;
    a.x = e->agent_block + c.agent_off;
    a.y = e->agent_block + e->total_slots + c.agent_off;
    a.th = e->agent_block + 2 * e->total_slots + c.agent_off;
    a.v = e->agent_block + 3 * e->total_slots + c.agent_off;
    a.ids = e->ids + c.agent_off;
    a.n = c.n;
    a.n_pad = c.n_pad;
    return a;
}

constexpr size_t kMaxLanes = 64;

void destroy_lanes(slime_ensemble* e) {
    for (cudaStream_t s : e->lanes) cudaStreamDestroy(s);
    for (cudaEvent_t ev : e->lane_ev) cudaEventDestroy(ev);
    if (e->fork_ev) cudaEventDestroy(e->fork_ev);
    e->lanes.clear();
    e->lane_ev.clear();
    e->fork_ev = nullptr;
    e->lane_cols.clear();
}

// Lanes and their colonies: the colonies by descending work (agents plus a
// quarter of the cells), each onto the lane with the least work so far.
int ensure_lanes(slime_ensemble* e) {
    if (!e->lanes.empty()) return SLIME_OK;
    const size_t k = e->colonies.size();
    const size_t cap = e->max_lanes > 0 ? (size_t)e->max_lanes : kMaxLanes;
    const size_t nl = k < cap ? k : cap;
    cudaError_t ce = cudaEventCreateWithFlags(&e->fork_ev, cudaEventDisableTiming);
    for (size_t l = 0; l < nl && ce == cudaSuccess; l++) {
        cudaStream_t s = nullptr;
        cudaEvent_t ev = nullptr;
        if ((ce = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) break;
        e->lanes.push_back(s);
        if ((ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming)) != cudaSuccess) break;
        e->lane_ev.push_back(ev);
    }
    if (ce != cudaSuccess) { // no half-built lanes: the next step tries again
        destroy_lanes(e);
        return cuda_error(e->err, ce, "creating lanes");
    }
    std::vector<uint32_t> order(k);
    for (size_t j = 0; j < k; j++) order[j] = (uint32_t)j;
    auto work = [&](uint32_t j) {
        const Colony& c = e->colonies[j];
        return c.n + (uint64_t)c.W * c.H / 4;
    };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return work(a) > work(b); });
    e->lane_cols.assign(nl, {});
    std::vector<uint64_t> load(nl, 0);
    for (uint32_t j : order) {
        size_t best = 0;
        for (size_t l = 1; l < nl; l++)
            if (load[l] < load[best]) best = l;
        e->lane_cols[best].push_back(j);
        load[best] += work(j);
    }
    return SLIME_OK;
}


// Kernels one lanes-engine step enqueues.
uint64_t lane_kernels_per_step(const slime_ensemble* e) {
    uint64_t k = 0;
    for (const Colony& c : e->colonies) k += 1 + (uint64_t)agent_pass_kernels(c.dev, c.n, false);
    return k;
}

// m steps of every colony on the lanes (fork from the ensemble's stream,
// join back into it); flips e->cur when m is odd, as m cooperative steps do.
cudaError_t enqueue_lane_steps(slime_ensemble* e, uint32_t m) {
    cudaError_t ce = cudaEventRecord(e->fork_ev, e->stream);
    const bool tex_shape = agent_shape_uses_texture(e->lane_agent_shape);
    for (size_t l = 0; l < e->lanes.size() && ce == cudaSuccess; l++) {
        cudaStream_t s = e->lanes[l];
        if ((ce = cudaStreamWaitEvent(s, e->fork_ev, 0)) != cudaSuccess) break;
        bool after_kernel = false; // PDL only behind a kernel of this lane
        for (uint32_t j : e->lane_cols[l]) {
            const Colony& c = e->colonies[j];
            AgentsSoA a = colony_soa(e, c);
            int cur = e->cur;
            for (uint32_t i = 0; i < m && ce == cudaSuccess; i++) {
                float* tin = e->trail[cur] + c.trail_off;
                float* tout = e->trail[1 - cur] + c.trail_off;
                uint32_t* cin = e->counts[cur] + c.trail_off;
                uint8_t* min = c.marks ? e->marks[cur] + c.trail_off : nullptr;
                if (c.n) {
                    ce = launch_agents(c.dev, a, tin, cin, s, e->lane_agent_shape, nullptr, tex_shape ? c.tex[cur] : 0,
                                       min, after_kernel);
                    after_kernel = true;
                    if (ce != cudaSuccess) break;
                }
                if (c.marks)
                    ce = launch_trail_marks(c.dev, e->lane_trail_tile, tin, min, tout, e->marks[1 - cur] + c.trail_off,
                                            s, nullptr, after_kernel);
                else
                    ce = launch_trail(c.dev, e->lane_trail_tile, tin, cin, tout, e->counts[1 - cur] + c.trail_off, s,
                                      nullptr, after_kernel);
                after_kernel = true;
                cur = 1 - cur;
            }
            if (ce != cudaSuccess) break;
        }
        if (ce == cudaSuccess) ce = cudaEventRecord(e->lane_ev[l], s);
        if (ce == cudaSuccess) ce = cudaStreamWaitEvent(e->stream, e->lane_ev[l], 0);
    }
    if (ce == cudaSuccess && (m & 1)) e->cur = 1 - e->cur;
    return ce;
}

// Morton-reorder every colony's slots (results are unchanged: each slot keeps
// its colony-local id).  With the lanes engine's lanes in place the colonies'
// sorts run on four of them at once (largest first, each onto the lane with
// the fewest agents so far), each of those lanes with its own sort scratch;
// otherwise one after another on the ensemble's stream.
int reorder_all(slime_ensemble* e) {
    const size_t nr = e->lanes.size() < 4 ? e->lanes.size() : 4;
    if (e->engine == SLIME_ENSEMBLE_LANES && nr > 1) {
        ECK(cudaEventRecord(e->fork_ev, e->stream), "forking reorders");
        for (size_t l = 0; l < nr; l++) ECK(cudaStreamWaitEvent(e->lanes[l], e->fork_ev, 0), "forking reorders");
        std::vector<uint32_t> order;
        for (uint32_t j = 0; j < (uint32_t)e->colonies.size(); j++)
            if (e->colonies[j].n) order.push_back(j);
        std::stable_sort(order.begin(), order.end(),
                         [&](uint32_t a, uint32_t b) { return e->colonies[a].n > e->colonies[b].n; });
        std::vector<uint64_t> load(nr, 0);
        for (uint32_t j : order) {
            size_t l = 0;
            for (size_t k = 1; k < nr; k++)
                if (load[k] < load[l]) l = k;
            load[l] += e->colonies[j].n;
            const Colony& c = e->colonies[j];
            AgentsSoA a = colony_soa(e, c);
            ReorderScratch& scratch = l == 0 ? e->reorder : e->lane_reorder[l - 1];
            ECK(launch_reorder(a, c.W, c.H, e->reorder_cell_log2, scratch, e->lanes[l]), "reordering agents");
            e->launches += 5;
        }
        for (size_t l = 0; l < nr; l++) {
            ECK(cudaEventRecord(e->lane_ev[l], e->lanes[l]), "joining reorders");
            ECK(cudaStreamWaitEvent(e->stream, e->lane_ev[l], 0), "joining reorders");
        }
    } else {
        for (const Colony& c : e->colonies) {
            if (c.n == 0) continue;
            AgentsSoA a = colony_soa(e, c);
            ECK(launch_reorder(a, c.W, c.H, e->reorder_cell_log2, e->reorder, e->stream), "reordering agents");
            e->launches += 5;
        }
    }
    e->last_reorder_step = e->steps_done;
    return SLIME_OK;
}

int check_barrier(slime_ensemble* e) {
    GridBarrier b;
    ECK(cudaMemcpyAsync(&b, e->d_bar, sizeof b, cudaMemcpyDeviceToHost, e->stream), "reading barrier state");
    ECK(cudaStreamSynchronize(e->stream), "reading barrier state");
    if (b.error) {
        cudaMemsetAsync(e->d_bar, 0, sizeof(GridBarrier), e->stream);
        cudaStreamSynchronize(e->stream);
        return ens_fail(e, SLIME_ERR_DEVICE_TIMEOUT, "the ensemble's grid barrier timed out");
    }
    return SLIME_OK;
}

// Whether colony c records its deposits as byte marks in the next steps:
// the lanes engine on a streaming trail tile, a deposition of at least 1 on
// a clean trail that the colony's steps keep clean (every deposit then folds
// the cell to 1, so whether a cell received any carries the fold).
bool colony_marks(const slime_ensemble* e, const Colony& c) {
    return e->engine == SLIME_ENSEMBLE_LANES && c.n > 0 && c.trail_clean && c.dev.dep >= 1.0f &&
           keeps_trail_clean(c.dev) && trail_tile_streams(c.dev, e->lane_trail_tile);
}

// Before a chunk: each colony's record kind (a change drops the captured
// graphs, which hold it), and the record the chunk's first step writes
// (counts[cur] or marks[cur]) cleared where steps of the other kind or the
// other engine left deposits in it.
int prepare_ens_deposits(slime_ensemble* e) {
    bool changed = false;
    for (Colony& c : e->colonies) {
        const bool mk = colony_marks(e, c);
        changed = changed || mk != c.marks;
        c.marks = mk;
    }
    if (changed) ens_invalidate(e);
    const int cur = e->cur;
    for (Colony& c : e->colonies) {
        const size_t cells = (size_t)c.W * c.H;
        if (c.marks) {
            if (!e->marks[0]) {
                for (int i = 0; i < 2; i++) {
                    ECK(dev_alloc((void**)&e->marks[i], e->total_cells), "allocating deposit marks");
                    ECK(cudaMemsetAsync(e->marks[i], 0, e->total_cells, e->stream), "clearing deposit marks");
                }
                for (Colony& o : e->colonies) o.marks_dirty[0] = o.marks_dirty[1] = false;
            }
            if (c.marks_dirty[cur]) {
                ECK(cudaMemsetAsync(e->marks[cur] + c.trail_off, 0, cells, e->stream), "clearing deposit marks");
                c.marks_dirty[cur] = false;
            }
        } else if (c.counts_dirty[cur]) {
            ECK(cudaMemsetAsync(e->counts[cur] + c.trail_off, 0, cells * sizeof(uint32_t), e->stream),
                "clearing deposit counts");
            c.counts_dirty[cur] = false;
        }
    }
    return SLIME_OK;
}

// After m steps (e->cur already advanced): the last step's record holds its
// deposits, its trail pass cleared the other one.
void after_ens_steps(slime_ensemble* e, uint32_t m) {
    if (m == 0) return;
    for (Colony& c : e->colonies) {
        bool* dirty = c.marks ? c.marks_dirty : c.counts_dirty;
        dirty[e->cur] = false;
        dirty[1 - e->cur] = true;
        c.trail_clean = c.trail_clean && keeps_trail_clean(c.dev);
    }
}

// The graph of m steps of the current engine from the current parity,
// captured on first use; null when the capture fails (the caller then
// launches directly).
cudaGraphExec_t chunk_graph(slime_ensemble* e, uint32_t m) {
    auto key = std::make_pair(m, e->cur);
    auto it = e->graphs.find(key);
    if (it != e->graphs.end()) return it->second;
    const int saved = e->cur;
    cudaGraphExec_t exec = nullptr;
    cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
    if (e->engine == SLIME_ENSEMBLE_LANES) {
        if (ce == cudaSuccess) ce = enqueue_lane_steps(e, m);
    } else {
        for (uint32_t i = 0; i < m && ce == cudaSuccess; i++) ce = enqueue_ens_step(e);
    }
    cudaGraph_t g = nullptr;
    cudaError_t ee = cudaStreamEndCapture(e->stream, &g);
    e->cur = saved;
    if (ce == cudaSuccess && ee == cudaSuccess) ee = cudaGraphInstantiate(&exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (ce != cudaSuccess || ee != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    e->graphs[key] = exec;
    return exec;
}

constexpr uint32_t kEnsChunk = 50;

// Capture the graphs that the next n steps replay (run_ens_steps' chunks).
int prepare_ens_steps(slime_ensemble* e, uint32_t n) {
    const bool lanes = e->engine == SLIME_ENSEMBLE_LANES;
    if (!e->use_graphs && !lanes) return SLIME_OK;
    if (lanes) {
        int rc = ensure_lanes(e);
        if (rc != SLIME_OK) return rc;
    }
    // the record kinds the graphs hold (clearing a stale record early is
    // what the next step would do first)
    int rc = prepare_ens_deposits(e);
    if (rc != SLIME_OK) return rc;
    const int saved = e->cur;
    uint64_t steps = e->steps_done;
    while (n > 0) {
        uint32_t m = n < kEnsChunk ? n : kEnsChunk;
        if (e->reorder_every) {
            uint64_t to_next = e->reorder_every - steps % e->reorder_every;
            if (to_next < m) m = (uint32_t)to_next;
        }
        if (!chunk_graph(e, m)) break; // stepping will launch directly
        if (m & 1) e->cur = 1 - e->cur;
        steps += m;
        n -= m;
    }
    e->cur = saved;
    return SLIME_OK;
}

int run_ens_steps(slime_ensemble* e, uint32_t n) {
    while (n > 0) {
        uint32_t m = n < kEnsChunk ? n : kEnsChunk;
        if (e->reorder_every) {
            if (e->steps_done % e->reorder_every == 0 && e->last_reorder_step != e->steps_done) {
                int rc = reorder_all(e);
                if (rc != SLIME_OK) return rc;
            }
            uint64_t to_next = e->reorder_every - e->steps_done % e->reorder_every;
            if (to_next < m) m = (uint32_t)to_next;
        }
        const bool lanes = e->engine == SLIME_ENSEMBLE_LANES;
        if (lanes) {
            int rc = ensure_lanes(e);
            if (rc != SLIME_OK) return rc;
        }
        int rc = prepare_ens_deposits(e);
        if (rc != SLIME_OK) return rc;
        const uint64_t kernels = lanes ? m * lane_kernels_per_step(e) : m;
        cudaGraphExec_t exec = (e->use_graphs || lanes) ? chunk_graph(e, m) : nullptr;
        if (exec) {
            ECK(cudaGraphLaunch(exec, e->stream), "launching ensemble graph");
            if (m & 1) e->cur = 1 - e->cur;
            e->last_chunk_graph = true;
        } else if (lanes) { // the lane chains run directly when they cannot be captured
            ECK(enqueue_lane_steps(e, m), "launching ensemble lanes");
            e->last_chunk_graph = false;
        } else {
            // cooperative launches that cannot be captured run directly from now on
            e->use_graphs = false;
            for (uint32_t i = 0; i < m; i++) ECK(enqueue_ens_step(e), "launching ensemble step");
            e->last_chunk_graph = false;
        }
        after_ens_steps(e, m);
        e->launches += kernels;
        e->steps_done += m;
        n -= m;
    }
    return SLIME_OK;
}

int check_colony(slime_ensemble* e, uint32_t j) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    if (j >= e->colonies.size()) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "colony index out of range");
    cudaSetDevice(e->device);
    return SLIME_OK;
}

} // namespace

extern "C" {

slime_ensemble* slime_ensemble_create(uint32_t k, const uint32_t* widths, const uint32_t* heights,
                                      const uint64_t* n_agents, const SlimeParams* params, int* status) {
    int dummy;
    if (!status) status = &dummy;
    *status = SLIME_ERR_INVALID_ARGUMENT;
    if (k == 0 || !widths || !heights || !n_agents || !params) return nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        *status = SLIME_ERR_NO_DEVICE;
        return nullptr;
    }
    slime_ensemble* e = new slime_ensemble();
    cudaGetDevice(&e->device);
    uint64_t slots = 0, cells = 0;
    for (uint32_t j = 0; j < k; j++) {
        Colony c;
        c.W = widths[j];
        c.H = heights[j];
        c.n = n_agents[j];
        const char* why = nullptr;
        if (c.W < 8 || c.H < 1 || c.W % 4 != 0 || (uint64_t)c.W * c.H >= (1ull << 31) || c.n >= (1ull << 31) ||
            c.W > (1u << 24) || c.H > (1u << 24)) {
            e->err = "each colony needs width % 4 == 0, width >= 8 and width*height < 2^31";
            break;
        }
        if (!make_dev_params(params[j], c.W, c.H, &c.dev, &why)) {
            e->err = why;
            break;
        }
        if (params[j].dispatch_mode != SLIME_DISPATCH_EACH_AGENT) {
            e->err = "the reference dispatch mode is available on single-colony contexts only";
            break;
        }
        int R = params[j].blur_mode == SLIME_BLUR_GAUSS ? c.dev.R : 1;
        if (R < 1 || R > 2) {
            e->err = "ensemble blur radius must be 1 or 2";
            break;
        }
        if (j == 0) {
            e->R = R;
            e->gauss = params[j].blur_mode == SLIME_BLUR_GAUSS;
        } else if (R != e->R || e->gauss != (params[j].blur_mode == SLIME_BLUR_GAUSS)) {
            e->err = "all colonies must share blur mode and radius";
            break;
        }
        c.params = params[j];
        c.params.width = c.W;
        c.params.height = c.H;
        c.n_pad = (c.n + kAgentPad - 1) / kAgentPad * kAgentPad;
        c.agent_off = slots;
        c.trail_off = cells;
        slots += c.n_pad;
        cells += (uint64_t)c.W * c.H;
        // every colony's first cell 256-byte aligned (float4 rows, and a
        // base its gather texture accepts)
        cells = (cells + 63) & ~63ull;
        e->colonies.push_back(c);
    }
    if (e->colonies.size() != k) {
        *status = SLIME_ERR_INVALID_ARGUMENT;
        slime_ensemble_destroy(e);
        return nullptr;
    }
    e->total_slots = slots ? slots : kAgentPad;
    // every colony's sampler may read W + 1 floats past its own cell 0; the
    // last colony's are covered by this zero tail
    uint32_t maxw = 0;
    for (const Colony& c : e->colonies) maxw = c.W > maxw ? c.W : maxw;
    e->total_cells = cells + maxw + 4;
    int rc = SLIME_OK;
    cudaError_t ce = cudaSuccess;
    do {
        if ((ce = cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((ce = dev_alloc((void**)&e->agent_block, 4 * e->total_slots * sizeof(float))) != cudaSuccess) break;
        if ((ce = cudaMemset(e->agent_block, 0, 4 * e->total_slots * sizeof(float))) != cudaSuccess) break;
        if ((ce = dev_alloc((void**)&e->ids, e->total_slots * sizeof(uint32_t))) != cudaSuccess) break;
        if ((ce = cudaMemset(e->ids, 0, e->total_slots * sizeof(uint32_t))) != cudaSuccess) break;
        for (int i = 0; i < 2 && ce == cudaSuccess; i++) {
            if ((ce = dev_alloc((void**)&e->trail[i], e->total_cells * sizeof(float))) != cudaSuccess) break;
            if ((ce = dev_alloc((void**)&e->counts[i], e->total_cells * sizeof(uint32_t))) != cudaSuccess) break;
            if ((ce = cudaMemset(e->trail[i], 0, e->total_cells * sizeof(float))) != cudaSuccess) break;
            ce = cudaMemset(e->counts[i], 0, e->total_cells * sizeof(uint32_t));
        }
        if (ce != cudaSuccess) break;
        if ((ce = dev_alloc((void**)&e->d_cols, k * sizeof(DevColony))) != cudaSuccess) break;
        if ((ce = dev_alloc((void**)&e->d_bar, sizeof(GridBarrier))) != cudaSuccess) break;
        ce = cudaMemset(e->d_bar, 0, sizeof(GridBarrier));
    } while (0);
    if (ce != cudaSuccess) rc = cuda_error(e->err, ce, "creating the ensemble");
    for (uint32_t j = 0; rc == SLIME_OK && j < k; j++) {
        const Colony& c = e->colonies[j];
        cudaError_t ie = launch_iota(e->ids + c.agent_off, c.n, e->stream);
        if (ie != cudaSuccess) rc = cuda_error(e->err, ie, "initialising agent ids");
    }
    for (uint32_t j = 0; rc == SLIME_OK && j < k; j++) {
        Colony& c = e->colonies[j];
        for (int i = 0; i < 2; i++) c.tex[i] = make_trail_texture(e->trail[i] + c.trail_off, c.W, c.H);
    }
    if (rc == SLIME_OK) rc = upload_cols(e);
    if (rc == SLIME_OK) rc = build_agent_items(e);
    if (rc == SLIME_OK) rc = build_strip_items(e);
    if (rc == SLIME_OK) rc = size_grid(e);
    if (rc != SLIME_OK) {
        *status = rc;
        slime_ensemble_destroy(e);
        return nullptr;
    }
    *status = SLIME_OK;
    return e;
}

void slime_ensemble_destroy(slime_ensemble* e) {
    if (!e) return;
    cudaSetDevice(e->device);
    if (e->stream) cudaStreamSynchronize(e->stream);
    ens_invalidate(e);
    destroy_lanes(e);
    for (Colony& c : e->colonies)
        for (int i = 0; i < 2; i++)
            if (c.tex[i]) cudaDestroyTextureObject(c.tex[i]);
    void* ptrs[] = {e->agent_block, e->ids, e->trail[0], e->trail[1], e->counts[0], e->counts[1], e->marks[0],
                    e->marks[1], e->d_cols, e->d_agent_items, e->d_strip_items, e->d_bar, e->staging,
                    e->reorder.buf, e->lane_reorder[0].buf, e->lane_reorder[1].buf, e->lane_reorder[2].buf};
    for (void* p : ptrs)
        if (p) dev_free(p);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

const char* slime_ensemble_last_error(const slime_ensemble* e) { return e ? e->err.c_str() : "null ensemble"; }

int slime_ensemble_set_params(slime_ensemble* e, uint32_t j, const SlimeParams* params) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    if (!params) return SLIME_ERR_INVALID_ARGUMENT;
    Colony& c = e->colonies[j];
    DevParams d;
    const char* why = nullptr;
    if (!make_dev_params(*params, c.W, c.H, &d, &why)) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, why);
    if (params->dispatch_mode != SLIME_DISPATCH_EACH_AGENT)
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT,
                        "the reference dispatch mode is available on single-colony contexts only");
    int R = params->blur_mode == SLIME_BLUR_GAUSS ? d.R : 1;
    if (R != e->R || e->gauss != (params->blur_mode == SLIME_BLUR_GAUSS))
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "all colonies must share blur mode and radius");
    c.params = *params;
    c.params.width = c.W;
    c.params.height = c.H;
    c.dev = d;
    // the cooperative kernel reads the colony table (its graphs stay valid);
    // the lanes engine's graphs hold the parameters as kernel arguments
    if (e->engine == SLIME_ENSEMBLE_LANES) {
        cudaStreamSynchronize(e->stream);
        ens_invalidate(e);
    }
    return upload_cols(e);
}

int ensure_staging(slime_ensemble* e, size_t bytes) {
    if (e->staging_bytes >= bytes) return SLIME_OK;
    if (e->staging) dev_free(e->staging);
    e->staging = nullptr;
    e->staging_bytes = 0;
    ECK(dev_alloc((void**)&e->staging, bytes), "allocating staging");
    e->staging_bytes = bytes;
    return SLIME_OK;
}

int slime_ensemble_upload_agents(slime_ensemble* e, uint32_t j, const float* aos, uint64_t n) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    Colony& c = e->colonies[j];
    if (n != c.n || (!aos && n)) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "agent count mismatch");
    if (n == 0) return SLIME_OK;
    if ((rc = ensure_staging(e, n * sizeof(float4))) != SLIME_OK) return rc;
    ECK(cudaMemcpyAsync(e->staging, aos, n * sizeof(float4), cudaMemcpyHostToDevice, e->stream), "uploading agents");
    AgentsSoA a = colony_soa(e, c);
    ECK(launch_aos_to_soa(e->staging, a, e->stream), "converting agents");
    ECK(launch_iota(a.ids, n, e->stream), "resetting agent ids");
    ECK(cudaStreamSynchronize(e->stream), "uploading agents");
    return SLIME_OK;
}

int slime_ensemble_download_agents(slime_ensemble* e, uint32_t j, float* aos, uint64_t n) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    Colony& c = e->colonies[j];
    if (n != c.n || (!aos && n)) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "agent count mismatch");
    if (n == 0) return SLIME_OK;
    if ((rc = ensure_staging(e, n * sizeof(float4))) != SLIME_OK) return rc;
    AgentsSoA a = colony_soa(e, c);
    ECK(launch_soa_to_aos(a, e->staging, e->stream), "converting agents");
    ECK(cudaMemcpyAsync(aos, e->staging, n * sizeof(float4), cudaMemcpyDeviceToHost, e->stream), "downloading agents");
    ECK(cudaStreamSynchronize(e->stream), "downloading agents");
    return SLIME_OK;
}

int slime_ensemble_seed_agents(slime_ensemble* e, uint32_t j, uint64_t seed, float hmin, float hmax) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    if (!isfinite(hmin) || !isfinite(hmax))
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "heading bounds must be finite");
    Colony& c = e->colonies[j];
    AgentsSoA a = colony_soa(e, c);
    ECK(launch_seed_agents(a, seed, (float)c.W, (float)c.H, hmin, hmax, c.params.agent_speed_min,
                           c.params.agent_speed_max, e->stream),
        "seeding agents");
    ECK(launch_iota(a.ids, c.n, e->stream), "resetting agent ids");
    ECK(cudaStreamSynchronize(e->stream), "seeding agents");
    return SLIME_OK;
}

int slime_ensemble_set_reorder(slime_ensemble* e, uint32_t every, uint32_t cell_log2) {
    if (!e || cell_log2 > 15) return SLIME_ERR_INVALID_ARGUMENT;
    e->reorder_every = every;
    e->reorder_cell_log2 = (int)cell_log2;
    return SLIME_OK;
}

int slime_ensemble_upload_trail(slime_ensemble* e, uint32_t j, const float* trail, uint64_t n_cells) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    Colony& c = e->colonies[j];
    if (!trail || n_cells != (uint64_t)c.W * c.H) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "trail size mismatch");
    ECK(cudaMemcpyAsync(e->trail[e->cur] + c.trail_off, trail, n_cells * sizeof(float), cudaMemcpyHostToDevice,
                        e->stream), "uploading trail");
    // deposit marks need every value finite and >= 0 (or +inf): checked
    // while the copy runs
    bool clean = true;
    for (uint64_t i = 0; i < n_cells; i++) clean = clean && (trail[i] >= 0.0f);
    ECK(cudaStreamSynchronize(e->stream), "uploading trail");
    c.trail_clean = clean;
    return SLIME_OK;
}

int slime_ensemble_download_trail(slime_ensemble* e, uint32_t j, float* trail, uint64_t n_cells) {
    int rc = check_colony(e, j);
    if (rc != SLIME_OK) return rc;
    Colony& c = e->colonies[j];
    if (!trail || n_cells != (uint64_t)c.W * c.H) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "trail size mismatch");
    ECK(cudaMemcpyAsync(trail, e->trail[e->cur] + c.trail_off, n_cells * sizeof(float), cudaMemcpyDeviceToHost,
                        e->stream), "downloading trail");
    ECK(cudaStreamSynchronize(e->stream), "downloading trail");
    return SLIME_OK;
}

int slime_ensemble_prepare_steps(slime_ensemble* e, uint32_t n_steps) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return prepare_ens_steps(e, n_steps);
}

int slime_ensemble_step(slime_ensemble* e, uint32_t n_steps) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return run_ens_steps(e, n_steps);
}

int slime_ensemble_sync(slime_ensemble* e) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "synchronising");
    return check_barrier(e);
}

int slime_ensemble_get_stream(slime_ensemble* e, void** stream) {
    if (!e || !stream) return SLIME_ERR_INVALID_ARGUMENT;
    *stream = (void*)e->stream;
    return SLIME_OK;
}

int slime_ensemble_profile_reorder(slime_ensemble* e, uint32_t reps, double* ms) {
    if (!e || !ms) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    *ms = 0.0;
    if (reps == 0) return SLIME_OK;
    // the first reorder sizes the sort scratch: untimed
    int rc = reorder_all(e);
    if (rc != SLIME_OK) return rc;
    cudaEvent_t e0, e1;
    ECK(cudaEventCreate(&e0), "creating events");
    ECK(cudaEventCreate(&e1), "creating events");
    cudaError_t ce = cudaEventRecord(e0, e->stream);
    for (uint32_t r = 0; r < reps && rc == SLIME_OK && ce == cudaSuccess; r++) rc = reorder_all(e);
    if (ce == cudaSuccess) ce = cudaEventRecord(e1, e->stream);
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (ce == cudaSuccess) ce = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != SLIME_OK) return rc;
    ECK(ce, "timing reorders");
    *ms = t;
    return SLIME_OK;
}

int slime_ensemble_set_engine(slime_ensemble* e, uint32_t engine, uint32_t agent_shape, uint32_t trail_tile,
                              uint32_t lanes) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    if (lanes > kMaxLanes) return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "at most 64 lanes");
    if (engine != SLIME_ENSEMBLE_COOPERATIVE && engine != SLIME_ENSEMBLE_LANES)
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "unknown ensemble engine");
    if (agent_shape >= (uint32_t)agent_shape_count() || trail_tile >= (uint32_t)kTrailTileTma)
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "agent shape or trail tile out of range");
    for (const Colony& c : e->colonies)
        if (!trail_tile_supported(c.dev, (int)trail_tile))
            return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "trail tile not supported by every colony");
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "synchronising");
    e->engine = (int)engine;
    e->lane_agent_shape = (int)agent_shape;
    e->lane_trail_tile = (int)trail_tile;
    ens_invalidate(e);
    if (lanes != (uint32_t)e->max_lanes) {
        destroy_lanes(e);
        e->max_lanes = (int)lanes;
    }
    return SLIME_OK;
}

int slime_ensemble_set_shape(slime_ensemble* e, uint32_t strip_rows, uint32_t blocks_per_sm,
                             uint32_t agents_per_thread) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    if ((strip_rows != 8 && strip_rows != 16 && strip_rows != 32) || blocks_per_sm > 4 ||
        (agents_per_thread != 2 && agents_per_thread != 4)) {
        e->err = "ensemble shape: strip_rows must be 8, 16 or 32, blocks_per_sm at most 4, agents_per_thread 2 or 4";
        return SLIME_ERR_INVALID_ARGUMENT;
    }
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "synchronising");
    e->rows = (int)strip_rows;
    e->blocks_per_sm = (int)blocks_per_sm;
    e->apt = (int)agents_per_thread;
    ens_invalidate(e);
    int rc = build_agent_items(e);
    if (rc == SLIME_OK) rc = build_strip_items(e);
    if (rc == SLIME_OK) rc = size_grid(e);
    return rc;
}

// Time trial steps of both engines (cooperative: agents per thread, strip
// height and residency; lanes: agent shape and trail tile), keep the fastest,
// and put the state back (snapshot of agents, trails and counts).
int slime_ensemble_autotune(slime_ensemble* e, uint32_t reps) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    if (reps == 0) reps = 3;
    size_t abytes = 4 * e->total_slots * sizeof(float), tbytes = e->total_cells * sizeof(float);
    void* snap = nullptr;
    ECK(dev_alloc((void**)&snap, abytes + 2 * tbytes + 2 * tbytes), "allocating autotune snapshot");
    char* s = (char*)snap;
    cudaMemcpyAsync(s, e->agent_block, abytes, cudaMemcpyDeviceToDevice, e->stream);
    for (int i = 0; i < 2; i++) {
        cudaMemcpyAsync(s + abytes + i * tbytes, e->trail[i], tbytes, cudaMemcpyDeviceToDevice, e->stream);
        cudaMemcpyAsync(s + abytes + 2 * tbytes + i * tbytes, e->counts[i], tbytes, cudaMemcpyDeviceToDevice,
                        e->stream);
    }
    if (e->reorder_every) {
        int rrc = reorder_all(e);
        if (rrc != SLIME_OK) {
            dev_free(snap);
            return rrc;
        }
        // the snapshot must hold the reordered slots
        cudaMemcpyAsync(s, e->agent_block, abytes, cudaMemcpyDeviceToDevice, e->stream);
    }
    const uint64_t saved_steps = e->steps_done, saved_reorder = e->reorder_every;
    e->reorder_every = 0;
    const int saved_cur = e->cur;
    const bool saved_graphs = e->use_graphs;
    e->use_graphs = false;
    const std::vector<Colony> saved_cols = e->colonies; // deposit-record flags
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best_rows = e->rows, best_bps = e->blocks_per_sm, best_apt = e->apt;
    int best_engine = e->engine, best_shape = e->lane_agent_shape, best_tile = e->lane_trail_tile;
    float best = 1e30f;
    const int rows_opts[] = {8, 16, 32};
    const int bps_opts[] = {0, 2, 4};
    const int apt_opts[] = {4, 2};
    int rc = SLIME_OK;
    auto trial = [&](float* ms) -> int {
        ens_invalidate(e);
        // warm-up; the lanes engine captures its chunk graph for both
        // parities of the trail buffers here, not inside the timed steps
        run_ens_steps(e, 1);
        run_ens_steps(e, reps);
        run_ens_steps(e, reps);
        cudaEventRecord(e0, e->stream);
        run_ens_steps(e, reps);
        cudaEventRecord(e1, e->stream);
        cudaEventSynchronize(e1);
        *ms = 0;
        cudaEventElapsedTime(ms, e0, e1);
        return check_barrier(e);
    };
    // cooperative engine: agents per thread x strip rows x residency
    e->engine = SLIME_ENSEMBLE_COOPERATIVE;
    for (int ao : apt_opts) {
      e->apt = ao;
      if ((rc = build_agent_items(e)) != SLIME_OK) break;
      for (int ro : rows_opts) {
        for (int bo : bps_opts) {
            e->rows = ro;
            e->blocks_per_sm = bo;
            if ((rc = build_strip_items(e)) != SLIME_OK || (rc = size_grid(e)) != SLIME_OK) break;
            float ms = 0;
            if ((rc = trial(&ms)) != SLIME_OK) break;
            if (ms < best) {
                best = ms;
                best_engine = SLIME_ENSEMBLE_COOPERATIVE;
                best_rows = ro;
                best_bps = bo;
                best_apt = ao;
            }
        }
        if (rc != SLIME_OK) break;
      }
      if (rc != SLIME_OK) break;
    }
    // lanes engine (its chunks are always captured): agent shape x trail tile
    // (the persistent shapes; the streaming tiles)
    const int shape_opts[] = {13, 9, 15};
    const int tile_opts[] = {7, 8, 9};
    e->engine = SLIME_ENSEMBLE_LANES;
    for (int so : shape_opts) {
        if (rc != SLIME_OK || so >= agent_shape_count()) break;
        for (int to : tile_opts) {
            bool ok = true;
            for (const Colony& c : e->colonies) ok = ok && trail_tile_supported(c.dev, to);
            if (!ok) continue;
            e->lane_agent_shape = so;
            e->lane_trail_tile = to;
            float ms = 0;
            if ((rc = trial(&ms)) != SLIME_OK) break;
            if (ms < best) {
                best = ms;
                best_engine = SLIME_ENSEMBLE_LANES;
                best_shape = so;
                best_tile = to;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemcpyAsync(e->agent_block, s, abytes, cudaMemcpyDeviceToDevice, e->stream);
    for (int i = 0; i < 2; i++) {
        cudaMemcpyAsync(e->trail[i], s + abytes + i * tbytes, tbytes, cudaMemcpyDeviceToDevice, e->stream);
        cudaMemcpyAsync(e->counts[i], s + abytes + 2 * tbytes + i * tbytes, tbytes, cudaMemcpyDeviceToDevice,
                        e->stream);
    }
    // the trials' deposit marks are stale: every mark region starts clear
    for (int i = 0; i < 2; i++)
        if (e->marks[i]) cudaMemsetAsync(e->marks[i], 0, e->total_cells, e->stream);
    cudaStreamSynchronize(e->stream);
    dev_free(snap);
    for (size_t j = 0; j < e->colonies.size(); j++) {
        Colony& c = e->colonies[j];
        const Colony& o = saved_cols[j];
        c.trail_clean = o.trail_clean;
        c.counts_dirty[0] = o.counts_dirty[0];
        c.counts_dirty[1] = o.counts_dirty[1];
        c.marks_dirty[0] = c.marks_dirty[1] = false;
    }
    e->cur = saved_cur;
    e->use_graphs = saved_graphs;
    e->steps_done = saved_steps;
    e->reorder_every = saved_reorder;
    e->rows = best_rows;
    e->blocks_per_sm = best_bps;
    e->apt = best_apt;
    e->engine = best_engine;
    e->lane_agent_shape = best_shape;
    e->lane_trail_tile = best_tile;
    ens_invalidate(e);
    if (rc == SLIME_OK) rc = build_agent_items(e);
    if (rc == SLIME_OK) rc = build_strip_items(e);
    if (rc == SLIME_OK) rc = size_grid(e);
    return rc;
}

int slime_ensemble_selftest_barrier_timeout(slime_ensemble* e) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "self-test");
    int* flag = nullptr;
    ECK(dev_alloc((void**)&flag, sizeof(int)), "self-test");
    cudaMemsetAsync(flag, 0, sizeof(int), e->stream);
    // about 0.1 s at the GB300's clock
    barrier_timeout_kernel<<<1, 32, 0, e->stream>>>(e->d_bar, 200000000ll, flag);
    cudaError_t le = cudaGetLastError();
    int after = 0;
    if (le == cudaSuccess) le = cudaMemcpyAsync(&after, flag, sizeof(int), cudaMemcpyDeviceToHost, e->stream);
    if (le == cudaSuccess) le = cudaStreamSynchronize(e->stream);
    dev_free(flag);
    if (le != cudaSuccess) return cuda_error(e->err, le, "self-test");
    int rc = check_barrier(e); // reads and clears the error flag, resets the barrier
    if (after != 2 || rc != SLIME_ERR_DEVICE_TIMEOUT)
        return ens_fail(e, SLIME_ERR_STATE, "the bounded barrier did not time out as expected");
    return SLIME_ERR_DEVICE_TIMEOUT;
}

int slime_ensemble_launch_count(const slime_ensemble* e, uint64_t* out) {
    if (!e || !out) return SLIME_ERR_INVALID_ARGUMENT;
    *out = e->launches;
    return SLIME_OK;
}

int slime_ensemble_get_info(const slime_ensemble* e, SlimeEnsembleInfo* out) {
    if (!e || !out) return SLIME_ERR_INVALID_ARGUMENT;
    memset(out, 0, sizeof(*out));
    out->n_colonies = (uint32_t)e->colonies.size();
    out->graphs_in_use = e->last_chunk_graph ? 1u : 0u;
    out->steps_done = e->steps_done;
    out->kernel_launches = e->launches;
    for (const Colony& c : e->colonies) {
        out->total_agents += c.n;
        out->total_cells += (uint64_t)c.W * c.H;
    }
    out->grid_blocks = (uint32_t)e->grid;
    out->strip_rows = (uint32_t)e->rows;
    out->agents_per_thread = (uint32_t)e->apt;
    out->engine = (uint32_t)e->engine;
    out->lanes = (uint32_t)e->lanes.size();
    out->lane_agent_shape = (uint32_t)e->lane_agent_shape;
    out->lane_trail_tile = (uint32_t)e->lane_trail_tile;
    for (const Colony& c : e->colonies) out->marks_colonies += c.marks ? 1u : 0u;
    return SLIME_OK;
}

} // extern "C"
