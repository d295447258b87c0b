// ensemble.cu - independent colonies of uneven sizes in one persistent launch
// per step.
//
// All colonies' agents live in one SoA block (each colony padded to a
// multiple of 128 slots, with a slot -> colony-local id map for Morton
// reordering) and all trails/counts in one ping-pong pair of buffers.  One
// persistent launch per step (grid = resident capacity) works through a queue
// of agent items (512 agents of one colony per warp, the next pair's state
// loaded while the current pair is computed) and trail strips (128 columns x
// ROWS rows per warp, the streaming code of the single-colony kernel), the
// strips of each colony queued right after the next colony's agent items.  Warps take items with an atomic ticket; a strip of
// colony j waits until colony j's agent items are done (bounded: it gives up
// after about a second and the step reports SLIME_ERR_DEVICE_TIMEOUT).  Waits
// only target items already taken by running warps, and each colony's two
// phases run close together in time, so its counts and trail stay in L2.
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
};


struct Colony {
    uint32_t W, H;
    uint64_t n, n_pad, agent_off, trail_off;
    SlimeParams params;
    DevParams dev;
};

// Bounded wait of one thread until *ctr >= target: gives up after
// limit_cycles of clock64(), flags the error and returns false.
__device__ bool bounded_wait_geq(const unsigned int* ctr, unsigned int target, long long limit_cycles, int* error) {
    const volatile unsigned int* v = ctr;
    if (*v >= target) return true;
    long long t0 = clock64();
    while (*v < target) {
        if (clock64() - t0 > limit_cycles) {
            atomicExch(error, 1);
            return false;
        }
        __nanosleep(64);
    }
    return true;
}

// Self-test of the bounded wait: waits for a counter nothing increments.
__global__ void wait_timeout_kernel(const unsigned int* never, long long limit_cycles, int* error, int* outcome) {
    if (threadIdx.x == 0) *outcome = bounded_wait_geq(never, 1u, limit_cycles, error) ? 1 : 2;
}

// Work queue of one step, in colony order: each colony's agent items, then its
// trail strips.  A warp takes the next item with an atomic ticket; a strip of
// colony j first waits (bounded) until all of colony j's agent items are
// done, so its deposit counts are complete.  Waits only ever target items
// already taken by running warps, so no residency guarantee is needed.
enum : uint32_t { kItemAgents = 0u, kItemStrip = 1u };
constexpr int kGroupsPerLane = 8;                          // 2-agent groups per lane per agent item
constexpr uint32_t kGroupsPerItem = 32u * kGroupsPerLane;  // 512 agents per agent item

// Every colony's parameter block, passed as a kernel parameter (constant
// bank): the colony of a work item is warp-uniform, so the accesses are
// uniform constant loads.
constexpr int kMaxColonies = 128;
struct EnsParams {
    DevParams p[kMaxColonies];
};

struct FlowState {
    unsigned int ticket;
    int error;
    unsigned int pad[2];
    unsigned int done[1]; // per colony: agent items finished (sized at allocation)
};

template <int R, bool kGauss, int ROWS>
__global__ void __launch_bounds__(kEnsThreads, 4) ensemble_flow_kernel(
    const __grid_constant__ EnsParams P, const DevColony* __restrict__ cols, const uint4* __restrict__ items,
    uint32_t n_items, const uint32_t* __restrict__ agent_items_per_colony, float* __restrict__ X,
    float* __restrict__ Y, float* __restrict__ TH, float* __restrict__ V, const uint32_t* __restrict__ IDS,
    const float* __restrict__ trail_in, uint32_t* counts_in, float* __restrict__ trail_out,
    uint32_t* __restrict__ counts_zero, FlowState* st, long long wait_limit) {
    const int lane = threadIdx.x & 31;
    // the next ticket and its descriptor are fetched while the current item runs
    uint32_t t = 0;
    if (lane == 0) t = atomicAdd(&st->ticket, 1u);
    t = __shfl_sync(0xffffffffu, t, 0);
    uint4 it_next = t < n_items ? items[t] : make_uint4(0, 0, 0, 0);
    while (true) {
        if (t >= n_items) break;
        const uint4 it = it_next;
        uint32_t tn = 0;
        if (lane == 0) tn = atomicAdd(&st->ticket, 1u);
        tn = __shfl_sync(0xffffffffu, tn, 0);
        if (tn < n_items) it_next = items[tn];
        t = tn;
        const uint32_t j = it.y;
        const DevColony& c = cols[j];
        if (it.x == kItemAgents) {
            const DevParams& p = P.p[j];
            const uint64_t n = c.n;
            const float* trail = trail_in + c.trail_off;
            uint32_t* counts = counts_in + c.trail_off;
            // groups it.z + lane + 32 i, i < kGroupsPerLane, within it.w groups
            const uint32_t g_end = it.z + it.w;
            uint32_t g = it.z + lane;
            if (g < g_end) {
                uint64_t slot = c.agent_off + 2ull * g;
                float2 x = __ldcs(reinterpret_cast<const float2*>(X + slot));
                float2 y = __ldcs(reinterpret_cast<const float2*>(Y + slot));
                float2 th = __ldcs(reinterpret_cast<const float2*>(TH + slot));
                float2 v = __ldcs(reinterpret_cast<const float2*>(V + slot));
                uint2 id = __ldcs(reinterpret_cast<const uint2*>(IDS + slot));
                while (true) {
                    const uint32_t gn = g + 32u;
                    const bool more = gn < g_end;
                    const uint64_t slotn = c.agent_off + 2ull * gn;
                    float2 xn, yn, thn, vn;
                    uint2 idn;
                    if (more) {
                        xn = __ldcs(reinterpret_cast<const float2*>(X + slotn));
                        yn = __ldcs(reinterpret_cast<const float2*>(Y + slotn));
                        thn = __ldcs(reinterpret_cast<const float2*>(TH + slotn));
                        vn = __ldcs(reinterpret_cast<const float2*>(V + slotn));
                        idn = __ldcs(reinterpret_cast<const uint2*>(IDS + slotn));
                    }
                    const uint64_t local = 2ull * g;
                    int c0 = -1, c1 = -1;
                    if (local + 2 <= n) {
                        c0 = agent_step(p, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
                        c1 = agent_step(p, x.y, y.y, th.y, v.y, (int32_t)id.y, trail);
                    } else if (local < n) {
                        c0 = agent_step(p, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
                    }
                    if (c0 >= 0) atomicAdd(counts + c0, 1u);
                    if (c1 >= 0) atomicAdd(counts + c1, 1u);
                    __stcs(reinterpret_cast<float2*>(X + slot), x);
                    __stcs(reinterpret_cast<float2*>(Y + slot), y);
                    __stcs(reinterpret_cast<float2*>(TH + slot), th);
                    __stcs(reinterpret_cast<float2*>(V + slot), v);
                    if (!more) break;
                    g = gn;
                    slot = slotn;
                    x = xn;
                    y = yn;
                    th = thn;
                    v = vn;
                    id = idn;
                }
            }
            // publish: this item's deposits are counted
            __threadfence();
            __syncwarp();
            if (lane == 0) atomicAdd(&st->done[j], 1u);
        } else {
            bool ok = true;
            if (lane == 0) ok = bounded_wait_geq(&st->done[j], agent_items_per_colony[j], wait_limit, &st->error);
            ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
            __threadfence();
            if (!ok) continue; // the host reports SLIME_ERR_DEVICE_TIMEOUT
            process_strip<R, kGauss, ROWS, true>(P.p[j], trail_in + c.trail_off, counts_in + c.trail_off,
                                                 trail_out + c.trail_off, counts_zero + c.trail_off, (int)it.z,
                                                 (int)it.w);
        }
    }
}

typedef void (*EnsKernel)(const EnsParams, const DevColony*, const uint4*, uint32_t, const uint32_t*, float*, float*,
                          float*, float*, const uint32_t*, const float*, uint32_t*, float*, uint32_t*, FlowState*,
                          long long);

size_t ens_smem_bytes(size_t) { return 0; }

template <int ROWS>
EnsKernel pick_rows(int R, bool gauss) {
    if (!gauss) return ensemble_flow_kernel<1, false, ROWS>;
    if (R == 1) return ensemble_flow_kernel<1, true, ROWS>;
    return ensemble_flow_kernel<2, true, ROWS>;
}

EnsKernel pick_kernel(int rows, int R, bool gauss) {
    switch (rows) {
    case 8: return pick_rows<8>(R, gauss);
    case 32: return pick_rows<32>(R, gauss);
    default: return pick_rows<16>(R, gauss);
    }
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
    float* trail[2] = {nullptr, nullptr};
    uint32_t* counts[2] = {nullptr, nullptr};
    int cur = 0;
    DevColony* d_cols = nullptr;
    uint32_t n_cols = 0;
    EnsParams hparams; // kernel-parameter copy of every colony's DevParams
    uint4* d_items = nullptr;          // the step's work queue (agent items and strips, colony by colony)
    uint32_t n_items = 0;
    uint32_t* d_agent_items = nullptr; // per colony: number of agent items
    FlowState* d_flow = nullptr;       // ticket, error flag, per-colony done counters
    size_t flow_bytes = 0;
    float4* staging = nullptr;
    size_t staging_bytes = 0;
    int rows = 16;
    int R = 1;
    bool gauss = false;
    int grid = 0;
    int blocks_per_sm = 0;
    bool use_graphs = true;
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
    memset(&e->hparams, 0, sizeof(e->hparams));
    for (size_t j = 0; j < e->colonies.size() && j < (size_t)kMaxColonies; j++) e->hparams.p[j] = e->colonies[j].dev;
    std::vector<DevColony> dc(e->colonies.size());
    for (size_t j = 0; j < e->colonies.size(); j++) {
        const Colony& c = e->colonies[j];
        memset(&dc[j], 0, sizeof(DevColony));
        dc[j].p = c.dev;
        dc[j].agent_off = c.agent_off;
        dc[j].n = c.n;
        dc[j].trail_off = c.trail_off;
        dc[j].warps_x = (int32_t)((c.W + 127) / 128);
    }
    ECK(cudaMemcpyAsync(e->d_cols, dc.data(), dc.size() * sizeof(DevColony), cudaMemcpyHostToDevice, e->stream),
        "uploading colony table");
    ECK(cudaStreamSynchronize(e->stream), "uploading colony table");
    return SLIME_OK;
}

// Queue order: colonies from the most agents to the fewest; the strips of a
// colony follow the agent items of the next colony, so by the time a warp
// reaches them the colony's deposits are (nearly always) complete and no warp
// idles at a colony boundary.
int build_items(slime_ensemble* e) {
    const size_t k = e->colonies.size();
    std::vector<size_t> order(k);
    for (size_t j = 0; j < k; j++) order[j] = j;
    std::stable_sort(order.begin(), order.end(),
                     [&](size_t a, size_t b) { return e->colonies[a].n > e->colonies[b].n; });
    std::vector<uint4> items;
    std::vector<uint32_t> per(k, 0);
    auto push_agents = [&](size_t j) {
        const Colony& c = e->colonies[j];
        uint64_t groups = (c.n + 1) / 2;
        for (uint64_t g0 = 0; g0 < groups; g0 += kGroupsPerItem) {
            uint64_t cnt = groups - g0 < kGroupsPerItem ? groups - g0 : kGroupsPerItem;
            items.push_back(make_uint4(kItemAgents, (uint32_t)j, (uint32_t)g0, (uint32_t)cnt));
            per[j]++;
        }
    };
    auto push_strips = [&](size_t j) {
        const Colony& c = e->colonies[j];
        uint32_t wx = (c.W + 127) / 128, strips = (c.H + e->rows - 1) / e->rows;
        for (uint32_t rs = 0; rs < strips; rs++)
            for (uint32_t cw = 0; cw < wx; cw++) items.push_back(make_uint4(kItemStrip, (uint32_t)j, cw, rs));
    };
    for (size_t q = 0; q < k; q++) {
        push_agents(order[q]);
        if (q >= 1) push_strips(order[q - 1]);
    }
    if (k) push_strips(order[k - 1]);
    if (e->d_items) dev_free(e->d_items);
    e->d_items = nullptr;
    ECK(dev_alloc((void**)&e->d_items, (items.size() ? items.size() : 1) * sizeof(uint4)), "allocating work queue");
    if (!items.empty())
        ECK(cudaMemcpy(e->d_items, items.data(), items.size() * sizeof(uint4), cudaMemcpyHostToDevice),
            "uploading work queue");
    ECK(cudaMemcpy(e->d_agent_items, per.data(), per.size() * sizeof(uint32_t), cudaMemcpyHostToDevice),
        "uploading work queue");
    e->n_items = (uint32_t)items.size();
    return SLIME_OK;
}

int size_grid(slime_ensemble* e) {
    EnsKernel k = pick_kernel(e->rows, e->R, e->gauss);
    int per_sm = 0, sms = 0;
    size_t smem = ens_smem_bytes(e->n_cols);
    if (smem > 48 * 1024)
        ECK(cudaFuncSetAttribute((const void*)k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "shared memory attribute");
    ECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kEnsThreads, smem), "occupancy query");
    ECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, e->device), "SM count");
    if (per_sm < 1) return ens_fail(e, SLIME_ERR_CUDA, "ensemble kernel cannot be resident");
    int want = e->blocks_per_sm > 0 ? (e->blocks_per_sm < per_sm ? e->blocks_per_sm : per_sm) : per_sm;
    e->grid = want * sms;
    return SLIME_OK;
}

cudaError_t enqueue_ens_step(slime_ensemble* e) {
    const int cur = e->cur;
    EnsKernel k = pick_kernel(e->rows, e->R, e->gauss);
    float* X = e->agent_block;
    float* Y = X + e->total_slots;
    float* TH = Y + e->total_slots;
    float* V = TH + e->total_slots;
    // ticket, error flag and done counters start at zero every step
    cudaError_t err = cudaMemsetAsync(e->d_flow, 0, e->flow_bytes, e->stream);
    if (err != cudaSuccess) return err;
    const long long wait_limit = 2000000000ll; // ~1 s of clock64() cycles
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.gridDim = dim3(e->grid);
    cfg.blockDim = dim3(kEnsThreads);
    cfg.dynamicSmemBytes = ens_smem_bytes(e->n_cols);
    cfg.stream = e->stream;
    err = cudaLaunchKernelEx(&cfg, k, e->hparams, (const DevColony*)e->d_cols, (const uint4*)e->d_items, e->n_items,
                             (const uint32_t*)e->d_agent_items, X, Y, TH, V, (const uint32_t*)e->ids,
                             (const float*)e->trail[cur], e->counts[cur], e->trail[1 - cur], e->counts[1 - cur],
                             e->d_flow, wait_limit);
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

// Morton-reorder every colony's slots (results are unchanged: each slot keeps
// its colony-local id).
int reorder_all(slime_ensemble* e) {
    for (const Colony& c : e->colonies) {
        if (c.n == 0) continue;
        AgentsSoA a = colony_soa(e, c);
        ECK(launch_reorder(a, c.W, c.H, e->reorder_cell_log2, e->reorder, e->stream), "reordering agents");
        e->launches += 5;
    }
    e->last_reorder_step = e->steps_done;
    return SLIME_OK;
}

int check_flow(slime_ensemble* e) {
    int error = 0;
    ECK(cudaMemcpyAsync(&error, &e->d_flow->error, sizeof(int), cudaMemcpyDeviceToHost, e->stream),
        "reading the step status");
    ECK(cudaStreamSynchronize(e->stream), "reading the step status");
    if (error) {
        cudaMemsetAsync(e->d_flow, 0, e->flow_bytes, e->stream);
        cudaStreamSynchronize(e->stream);
        return ens_fail(e, SLIME_ERR_DEVICE_TIMEOUT, "a bounded device-side wait of the ensemble step timed out");
    }
    return SLIME_OK;
}

int run_ens_steps(slime_ensemble* e, uint32_t n) {
    const uint32_t chunk = 50;
    while (n > 0) {
        uint32_t m = n < chunk ? n : chunk;
        if (e->reorder_every) {
            if (e->steps_done % e->reorder_every == 0 && e->last_reorder_step != e->steps_done) {
                int rc = reorder_all(e);
                if (rc != SLIME_OK) return rc;
            }
            uint64_t to_next = e->reorder_every - e->steps_done % e->reorder_every;
            if (to_next < m) m = (uint32_t)to_next;
        }
        if (e->use_graphs) {
            auto key = std::make_pair(m, e->cur);
            auto it = e->graphs.find(key);
            cudaGraphExec_t exec = nullptr;
            if (it == e->graphs.end()) {
                const int saved = e->cur;
                cudaError_t ce = cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal);
                for (uint32_t i = 0; i < m && ce == cudaSuccess; i++) ce = enqueue_ens_step(e);
                cudaGraph_t g = nullptr;
                cudaError_t ee = cudaStreamEndCapture(e->stream, &g);
                e->cur = saved;
                if (ce == cudaSuccess && ee == cudaSuccess) ee = cudaGraphInstantiate(&exec, g, 0);
                if (g) cudaGraphDestroy(g);
                if (ce != cudaSuccess || ee != cudaSuccess) {
                    // a launch that cannot be captured runs directly
                    cudaGetLastError();
                    e->use_graphs = false;
                    continue;
                }
                e->graphs[key] = exec;
            } else {
                exec = it->second;
            }
            ECK(cudaGraphLaunch(exec, e->stream), "launching ensemble graph");
            if (m & 1) e->cur = 1 - e->cur;
        } else {
            for (uint32_t i = 0; i < m; i++) ECK(enqueue_ens_step(e), "launching ensemble step");
        }
        e->launches += m;
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
        // keep every colony's first cell 16-byte aligned
        cells = (cells + 3) & ~3ull;
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
    e->n_cols = k;
    if (k > (uint32_t)kMaxColonies) {
        e->err = "an ensemble holds at most 128 colonies";
        *status = SLIME_ERR_INVALID_ARGUMENT;
        slime_ensemble_destroy(e);
        return nullptr;
    }
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
        if ((ce = dev_alloc((void**)&e->d_agent_items, k * sizeof(uint32_t))) != cudaSuccess) break;
        e->flow_bytes = sizeof(FlowState) + k * sizeof(unsigned int);
        if ((ce = dev_alloc((void**)&e->d_flow, e->flow_bytes)) != cudaSuccess) break;
        ce = cudaMemset(e->d_flow, 0, e->flow_bytes);
    } while (0);
    if (ce != cudaSuccess) rc = cuda_error(e->err, ce, "creating the ensemble");
    for (uint32_t j = 0; rc == SLIME_OK && j < k; j++) {
        const Colony& c = e->colonies[j];
        cudaError_t ie = launch_iota(e->ids + c.agent_off, c.n, e->stream);
        if (ie != cudaSuccess) rc = cuda_error(e->err, ie, "initialising agent ids");
    }
    if (rc == SLIME_OK) rc = upload_cols(e);
    if (rc == SLIME_OK) rc = build_items(e);
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
    void* ptrs[] = {e->agent_block, e->ids, e->trail[0], e->trail[1], e->counts[0], e->counts[1], e->d_cols,
                    e->d_items, e->d_agent_items, e->d_flow, e->staging, e->reorder.buf};
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
    int R = params->blur_mode == SLIME_BLUR_GAUSS ? d.R : 1;
    if (R != e->R || e->gauss != (params->blur_mode == SLIME_BLUR_GAUSS))
        return ens_fail(e, SLIME_ERR_INVALID_ARGUMENT, "all colonies must share blur mode and radius");
    c.params = *params;
    c.params.width = c.W;
    c.params.height = c.H;
    c.dev = d;
    int urc = upload_cols(e);
    ens_invalidate(e); // the parameter blocks are baked into the captured launches
    return urc;
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
    ECK(cudaStreamSynchronize(e->stream), "uploading trail");
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

int slime_ensemble_step(slime_ensemble* e, uint32_t n_steps) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    return run_ens_steps(e, n_steps);
}

int slime_ensemble_sync(slime_ensemble* e) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "synchronising");
    return check_flow(e);
}

int slime_ensemble_get_stream(slime_ensemble* e, void** stream) {
    if (!e || !stream) return SLIME_ERR_INVALID_ARGUMENT;
    *stream = (void*)e->stream;
    return SLIME_OK;
}

// Time trial steps for every strip height and residency, keep the fastest,
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
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    int best_rows = e->rows, best_bps = e->blocks_per_sm;
    float best = 1e30f;
    const int rows_opts[] = {8, 16, 32};
    const int bps_opts[] = {0, 2, 4};
    int rc = SLIME_OK;
    for (int ro : rows_opts) {
        for (int bo : bps_opts) {
            e->rows = ro;
            e->blocks_per_sm = bo;
            if ((rc = build_items(e)) != SLIME_OK || (rc = size_grid(e)) != SLIME_OK) break;
            run_ens_steps(e, 1); // warm-up
            cudaEventRecord(e0, e->stream);
            run_ens_steps(e, reps);
            cudaEventRecord(e1, e->stream);
            cudaEventSynchronize(e1);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if ((rc = check_flow(e)) != SLIME_OK) break;
            if (ms < best) {
                best = ms;
                best_rows = ro;
                best_bps = bo;
            }
        }
        if (rc != SLIME_OK) break;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaMemcpyAsync(e->agent_block, s, abytes, cudaMemcpyDeviceToDevice, e->stream);
    for (int i = 0; i < 2; i++) {
        cudaMemcpyAsync(e->trail[i], s + abytes + i * tbytes, tbytes, cudaMemcpyDeviceToDevice, e->stream);
        cudaMemcpyAsync(e->counts[i], s + abytes + 2 * tbytes + i * tbytes, tbytes, cudaMemcpyDeviceToDevice,
                        e->stream);
    }
    cudaStreamSynchronize(e->stream);
    dev_free(snap);
    e->cur = saved_cur;
    e->use_graphs = saved_graphs;
    e->steps_done = saved_steps;
    e->reorder_every = saved_reorder;
    e->rows = best_rows;
    e->blocks_per_sm = best_bps;
    ens_invalidate(e);
    if (rc == SLIME_OK) rc = build_items(e);
    if (rc == SLIME_OK) rc = size_grid(e);
    return rc;
}

int slime_ensemble_selftest_barrier_timeout(slime_ensemble* e) {
    if (!e) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(e->device);
    ECK(cudaStreamSynchronize(e->stream), "self-test");
    int* outcome = nullptr;
    ECK(dev_alloc((void**)&outcome, sizeof(int)), "self-test");
    cudaMemsetAsync(outcome, 0, sizeof(int), e->stream);
    cudaMemsetAsync(e->d_flow, 0, e->flow_bytes, e->stream);
    // waits for pad[0], which nothing increments; about 0.1 s at the GB300's clock
    wait_timeout_kernel<<<1, 32, 0, e->stream>>>(&e->d_flow->pad[0], 200000000ll, &e->d_flow->error, outcome);
    cudaError_t le = cudaGetLastError();
    int after = 0;
    if (le == cudaSuccess) le = cudaMemcpyAsync(&after, outcome, sizeof(int), cudaMemcpyDeviceToHost, e->stream);
    if (le == cudaSuccess) le = cudaStreamSynchronize(e->stream);
    dev_free(outcome);
    if (le != cudaSuccess) return cuda_error(e->err, le, "self-test");
    int rc = check_flow(e); // reads and clears the error flag
    if (after != 2 || rc != SLIME_ERR_DEVICE_TIMEOUT)
        return ens_fail(e, SLIME_ERR_STATE, "the bounded wait did not time out as expected");
    return SLIME_ERR_DEVICE_TIMEOUT;
}

int slime_ensemble_launch_count(const slime_ensemble* e, uint64_t* out) {
    if (!e || !out) return SLIME_ERR_INVALID_ARGUMENT;
    *out = e->launches;
    return SLIME_OK;
}

} // extern "C"
