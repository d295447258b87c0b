// capi.cu - the C ABI of include/slime.h for one simulation context.
//
// Replaces the reference's PipelineManager (src/pipeline_manager.rs:19-113),
// BindGroupManager (src/bind_group_manager.rs:13-125) and the per-frame
// dispatch code (src/main.rs:1163-1235).  A context owns, on one GPU:
//   agents   SoA x/y/angle/speed (+ slot->id map once reordered)
//   trail[2] ping-pong binary32 trails (trail[cur] is the state)
//   counts[2] per-cell deposit counters: counts[cur] collects the next step's
//            deposits (kept zero between steps), counts[1-cur] holds the
//            previous step's
//   marks[2] per-cell deposit marks (bytes), the counts' stand-in for steps
//            in which every deposit saturates the fold
// and enqueues everything on its own stream.  Steps are captured in CUDA
// graphs of `graph_chunk` steps, one per starting parity, and replayed.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <stdlib.h>

#include <map>
#include <mutex>
#include <string>
#include <unordered_map>
#include <utility>
#include <vector>

#include "ctx.h"

using namespace slime;

namespace slime {

bool make_dev_params(const SlimeParams& p, uint32_t W, uint32_t H, DevParams* out, const char** why) {
    const float fs[] = {p.decay_factor, p.agent_jitter, p.agent_speed_min, p.agent_speed_max,
                        p.agent_turn_speed, p.agent_sensor_angle, p.agent_sensor_distance, p.diffusion_rate,
                        p.pheromone_deposition_amount, p.time_step};
    for (float f : fs)
        if (!isfinite(f)) {
            *why = "parameters must be finite (NaN/inf rejected)";
            return false;
        }
    if (p.width != 0 && p.width != W) {
        *why = "params.width must be 0 or the context's width";
        return false;
    }
    if (p.height != 0 && p.height != H) {
        *why = "params.height must be 0 or the context's height";
        return false;
    }
    if (p.decay_mode > SLIME_DECAY_MULTIPLY) {
        *why = "unknown decay_mode";
        return false;
    }
    if (p.blur_mode > SLIME_BLUR_GAUSS) {
        *why = "unknown blur_mode";
        return false;
    }
    if (p.dispatch_mode > SLIME_DISPATCH_REFERENCE) {
        *why = "unknown dispatch_mode";
        return false;
    }
    if (p.sensor_mode > SLIME_SENSOR_ROTATED) {
        *why = "unknown sensor_mode";
        return false;
    }
    DevParams d;
    memset(&d, 0, sizeof(d));
    d.W = (int32_t)W;
    d.H = (int32_t)H;
    d.Wf = (float)W;
    d.Hf = (float)H;
    d.Wm1f = (float)(W - 1);
    d.Hm1f = (float)(H - 1);
    d.speed_min = p.agent_speed_min;
    d.speed_max = p.agent_speed_max;
    d.turn = p.agent_turn_speed;
    d.sensor_angle = p.agent_sensor_angle;
    slm_sincos(p.agent_sensor_angle, &d.sensor_sin, &d.sensor_cos);
    d.sensor_dist = p.agent_sensor_distance;
    d.jitter = p.agent_jitter;
    d.time_step = p.time_step;
    d.dep = p.pheromone_deposition_amount;
    d.decay = p.decay_factor;
    d.decay_k = slm_mul(p.decay_factor, 0.001f);          // compute.wgsl:159
    d.rate = slm_clamp(p.diffusion_rate, 0.0f, 1.0f);     // compute.wgsl:173
    d.decay_mode = p.decay_mode;
    d.blur_mode = p.blur_mode;
    d.dispatch_mode = p.dispatch_mode;
    d.sensor_mode = p.sensor_mode;
    d.R = 1;
    if (p.blur_mode == SLIME_BLUR_GAUSS) {
        if (!isfinite(p.blur_radius) || !isfinite(p.blur_sigma)) {
            *why = "blur_radius and blur_sigma must be finite";
            return false;
        }
        d.R = slm_gauss_radius(p.blur_radius, kMaxR);
        if (slm_gauss_weights(d.R, p.blur_sigma, d.w) != 0) {
            *why = "blur_sigma must be > 0 in Gaussian mode";
            return false;
        }
        double ws = 0.0;
        for (int i = 0; i <= 2 * d.R; i++) ws += (double)d.w[i];
        d.w2sum_m1 = (float)(ws * ws - 1.0);
    }
    *out = d;
    return true;
}

namespace {
std::mutex g_alloc_mutex;
std::unordered_map<void*, size_t> g_alloc_sizes;
size_t g_alloc_live = 0;
size_t alloc_cap() {
    static size_t cap = [] {
        const char* v = getenv("SLIME_DEVICE_MEMORY_CAP");
        return (v && *v) ? (size_t)strtoull(v, nullptr, 10) : (size_t)0;
    }();
    return cap;
}
} // namespace

cudaError_t dev_alloc(void** p, size_t bytes) {
    *p = nullptr;
    std::lock_guard<std::mutex> lock(g_alloc_mutex);
    size_t cap = alloc_cap();
    if (cap && g_alloc_live + bytes > cap) return cudaErrorMemoryAllocation;
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) return e;
    g_alloc_sizes[*p] = bytes;
    g_alloc_live += bytes;
    return cudaSuccess;
}

void dev_free(void* p) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(g_alloc_mutex);
        auto it = g_alloc_sizes.find(p);
        if (it != g_alloc_sizes.end()) {
            g_alloc_live -= it->second;
            g_alloc_sizes.erase(it);
        }
    }
    cudaFree(p);
}

int set_error(std::string& err, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
}

int cuda_error(std::string& err, cudaError_t e, const char* what) {
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        return set_error(err, SLIME_ERR_OUT_OF_MEMORY, "%s: out of device memory", what);
    }
    return set_error(err, SLIME_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

} // namespace slime

#define CK(expr, what)                                                                                      \
    do {                                                                                                    \
        cudaError_t _e = (expr);                                                                            \
        if (_e != cudaSuccess) return cuda_error(ctx->err, _e, what);                                       \
    } while (0)

namespace {

void free_agents(slime_ctx* ctx) {
    if (ctx->agent_block) dev_free(ctx->agent_block);
    if (ctx->ids_storage) dev_free(ctx->ids_storage);
    ctx->agent_block = nullptr;
    ctx->ids_storage = nullptr;
    ctx->agents = AgentsSoA();
}

void free_trail(slime_ctx* ctx) {
    for (int i = 0; i < 2; i++) {
        if (ctx->trail_tex[i]) cudaDestroyTextureObject(ctx->trail_tex[i]);
        ctx->trail_tex[i] = 0;
        if (ctx->trail[i]) dev_free(ctx->trail[i]);
        if (ctx->counts[i]) dev_free(ctx->counts[i]);
        if (ctx->marks[i]) dev_free(ctx->marks[i]);
        ctx->marks[i] = nullptr;
        ctx->trail[i] = nullptr;
        ctx->counts[i] = nullptr;
    }
}

// The agent block for `n` agents replaces the context's only once it is
// allocated and cleared: on failure the context keeps its agents.  The
// caller has synchronised the stream when the old block may still be read.
int alloc_agents(slime_ctx* ctx, uint64_t n) {
    uint64_t n_pad = (n + kAgentPad - 1) / kAgentPad * kAgentPad;
    if (n_pad == 0) n_pad = kAgentPad;
    size_t bytes = 4 * n_pad * sizeof(float);
    void* block = nullptr;
    CK(dev_alloc(&block, bytes), "allocating agents");
    cudaError_t e = cudaMemsetAsync(block, 0, bytes, ctx->stream);
    if (e != cudaSuccess) {
        dev_free(block);
        return cuda_error(ctx->err, e, "clearing agents");
    }
    free_agents(ctx);
    ctx->agent_block = block;
    float* b = (float*)block;
    ctx->agents.x = b;
    ctx->agents.y = b + n_pad;
    ctx->agents.th = b + 2 * n_pad;
    ctx->agents.v = b + 3 * n_pad;
    ctx->agents.ids = nullptr;
    ctx->agents.n = n;
    ctx->agents.n_pad = n_pad;
    return SLIME_OK;
}

// Two trails with their deposit counts, marks and gather textures.
struct TrailSet {
    float* trail[2] = {nullptr, nullptr};
    uint32_t* counts[2] = {nullptr, nullptr};
    uint8_t* marks[2] = {nullptr, nullptr};
    cudaTextureObject_t tex[2] = {0, 0};

    void release() {
        for (int i = 0; i < 2; i++) {
            if (tex[i]) cudaDestroyTextureObject(tex[i]);
            dev_free(trail[i]);
            dev_free(counts[i]);
            dev_free(marks[i]);
            tex[i] = 0;
            trail[i] = nullptr;
            counts[i] = nullptr;
            marks[i] = nullptr;
        }
    }
};

cudaError_t make_trail_set(uint32_t W, uint32_t H, cudaStream_t s, TrailSet* t, const char** what) {
    const size_t cells = (size_t)W * H;
    // W + 2 zero floats past the last cell: the sampler's discarded taps
    const size_t trail_bytes = (cells + W + 2) * sizeof(float);
    const size_t mark_bytes = (cells + 15) & ~(size_t)15;
    cudaError_t e = cudaSuccess;
    for (int i = 0; i < 2 && e == cudaSuccess; i++) {
        *what = "allocating trail";
        if ((e = dev_alloc((void**)&t->trail[i], trail_bytes)) != cudaSuccess) break;
        *what = "allocating deposit counts";
        if ((e = dev_alloc((void**)&t->counts[i], cells * sizeof(uint32_t))) != cudaSuccess) break;
        *what = "allocating deposit marks";
        if ((e = dev_alloc((void**)&t->marks[i], mark_bytes)) != cudaSuccess) break;
        *what = "clearing trail";
        e = cudaMemsetAsync(t->trail[i], 0, trail_bytes, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(t->counts[i], 0, cells * sizeof(uint32_t), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(t->marks[i], 0, mark_bytes, s);
        if (e == cudaSuccess) t->tex[i] = make_trail_texture(t->trail[i], W, H);
    }
    return e;
}

// The trails for a W x H grid replace the context's only once all of them
// are allocated: on failure the context keeps its trail.  The caller has
// synchronised the stream when the old trails may still be read.
int alloc_trail(slime_ctx* ctx, uint32_t W, uint32_t H) {
    TrailSet t;
    const char* what = "allocating trail";
    cudaError_t e = make_trail_set(W, H, ctx->stream, &t, &what);
    if (e != cudaSuccess) {
        t.release();
        return cuda_error(ctx->err, e, what);
    }
    free_trail(ctx);
    for (int i = 0; i < 2; i++) {
        ctx->trail[i] = t.trail[i];
        ctx->counts[i] = t.counts[i];
        ctx->marks[i] = t.marks[i];
        ctx->trail_tex[i] = t.tex[i];
        ctx->counts_dirty[i] = false;
        ctx->marks_dirty[i] = false;
    }
    // tensor maps for the tensor-copy trail tile (none for widths it cannot take)
    make_trail_maps(&ctx->tmaps, ctx->trail, ctx->counts, ctx->marks, W, H);
    cudaGetLastError();
    ctx->cur = 0;
    ctx->last_counts_valid = false;
    ctx->trail_clean = true;
    ctx->last_marks = false;
    return SLIME_OK;
}

int ensure_staging(slime_ctx* ctx, size_t bytes) {
    if (ctx->staging_bytes >= bytes) return SLIME_OK;
    if (ctx->staging) dev_free(ctx->staging);
    ctx->staging = nullptr;
    ctx->staging_bytes = 0;
    CK(dev_alloc((void**)&ctx->staging, bytes), "allocating staging buffer");
    ctx->staging_bytes = bytes;
    return SLIME_OK;
}

// Put every agent back in id order relative to the slot->id map: after an
// upload or a seed, slot i holds agent i.
int reset_ids(slime_ctx* ctx) {
    if (ctx->agents.ids) CK(launch_iota(ctx->agents.ids, ctx->agents.n, ctx->stream), "resetting agent ids");
    ctx->reordered = false;
    return SLIME_OK;
}

int valid_size(std::string& err, uint32_t W, uint32_t H, uint64_t n) {
    if (W < 1 || H < 1) return set_error(err, SLIME_ERR_INVALID_ARGUMENT, "trail size must be at least 1x1");
    if (W > (1u << 24) || H > (1u << 24))
        return set_error(err, SLIME_ERR_INVALID_ARGUMENT, "trail sides must be <= 2^24 (exact in binary32)");
    if ((uint64_t)W * H >= (1ull << 31))
        return set_error(err, SLIME_ERR_INVALID_ARGUMENT, "width*height must be < 2^31 (the shader's i32 index)");
    if (n >= (1ull << 31))
        return set_error(err, SLIME_ERR_INVALID_ARGUMENT, "agent count must be < 2^31 (the shader's i32 index)");
    return SLIME_OK;
}

} // namespace

namespace slime {

void invalidate_graphs(slime_ctx* ctx) {
    for (auto& kv : ctx->graphs) cudaGraphExecDestroy(kv.second);
    ctx->graphs.clear();
}

// The persisting-L2 carve-out is a limit of the device's context, shared by
// every simulation on that device in the process.  Each context registers the
// carve-out it wants; the limit is the largest live request, and persisting
// lines are released once no context wants any.
std::mutex g_l2_mutex;
std::map<int, std::map<const slime_ctx*, size_t>> g_l2_grants; // device -> context -> bytes

void apply_l2_limit(int device) {
    size_t want = 0;
    for (const auto& kv : g_l2_grants[device]) want = kv.second > want ? kv.second : want;
    if (cudaDeviceSetLimit(cudaLimitPersistingL2CacheSize, want) != cudaSuccess) cudaGetLastError();
    if (want == 0 && cudaCtxResetPersistingL2Cache() != cudaSuccess) cudaGetLastError();
}

void release_l2(slime_ctx* ctx) {
    std::lock_guard<std::mutex> lock(g_l2_mutex);
    cudaSetDevice(ctx->device);
    g_l2_grants[ctx->device].erase(ctx);
    apply_l2_limit(ctx->device);
    ctx->l2_persist_bytes = 0;
}

// Size the persisting-L2 carve-out for the trail and remember the largest
// window the device accepts.  The trail persists only when all of it fits
// the device's maximum carve-out and one window: a trail larger than that
// (8192^2 binary32 is 256 MiB) would keep a random part resident at the cost
// of the L2 left to every other access, which measured slower than no
// carve-out at all.
void setup_l2(slime_ctx* ctx) {
    std::lock_guard<std::mutex> lock(g_l2_mutex);
    cudaSetDevice(ctx->device);
    auto& grants = g_l2_grants[ctx->device];
    grants.erase(ctx);
    ctx->l2_persist_bytes = 0;
    ctx->l2_max_window = 0;
    int max_persist = 0, max_window = 0;
    const size_t want = (size_t)ctx->W * ctx->H * sizeof(float);
    if (ctx->opt.l2_persist && !ctx->l2_tuned_off &&
        cudaDeviceGetAttribute(&max_persist, cudaDevAttrMaxPersistingL2CacheSize, ctx->device) == cudaSuccess &&
        cudaDeviceGetAttribute(&max_window, cudaDevAttrMaxAccessPolicyWindowSize, ctx->device) == cudaSuccess &&
        max_persist > 0 && max_window > 0 && want <= (size_t)max_persist && want <= (size_t)max_window) {
        grants[ctx] = want;
        ctx->l2_persist_bytes = want;
        ctx->l2_max_window = (size_t)max_window;
    }
    cudaGetLastError();
    apply_l2_limit(ctx->device);
}

// The access window for a launch that reads (or writes) trail buffer `t`.
bool trail_window(const slime_ctx* ctx, const float* t, cudaAccessPolicyWindow* w, unsigned pass) {
    if (!ctx->l2_persist_bytes || !(ctx->l2_window_passes & pass)) return false;
    size_t bytes = (size_t)ctx->W * ctx->H * sizeof(float);
    if (bytes > ctx->l2_max_window) bytes = ctx->l2_max_window;
    w->base_ptr = (void*)t;
    w->num_bytes = bytes;
    float ratio = (float)ctx->l2_persist_bytes / (float)bytes;
    w->hitRatio = ratio < 1.0f ? ratio : 1.0f;
    w->hitProp = cudaAccessPropertyPersisting;
    w->missProp = cudaAccessPropertyStreaming;
    return true;
}

// Whether a step keeps a clean trail clean (finite values >= 0, or +inf):
// the subtractive decay never raises a value, the multiplicative one with a
// factor in [0, 1] neither; the fold, the blur's non-negative weights and the
// clamped diffusion rate preserve it.
bool keeps_trail_clean(const DevParams& d) {
    if (d.decay_mode == SLIME_DECAY_MULTIPLY) return d.decay >= 0.0f && d.decay <= 1.0f;
    return d.decay_k >= 0.0f;
}

// Whether the next steps record deposit marks instead of counts.  With a
// deposition of at least 1 on a trail value t >= 0, the first deposit folds
// t to clamp(t + dep, 0, 1) = 1 and every further one leaves it there, so the
// fold of k deposits depends only on whether k > 0: one byte per cell carries
// it, written with plain stores instead of 32-bit atomics, and the trail pass
// reads 1 byte per cell instead of 4 and clears 1 instead of 4.  The result
// is the same, bit for bit.  The host decides, from the parameters, the tile
// (the streaming tiles read marks) and what it knows of the trail: clean
// after creation, clear and resize, checked on upload, kept by steps that
// keep it (keeps_trail_clean).
bool marks_allowed(const slime_ctx* ctx) {
    if (ctx->opt.exact_counts || ctx->agents.n == 0 || !ctx->trail_clean) return false;
    return ctx->dev.dep >= 1.0f && keeps_trail_clean(ctx->dev);
}
bool use_marks(const slime_ctx* ctx) { return marks_allowed(ctx) && trail_tile_streams(ctx->dev, ctx->tile); }

// The record the next step writes (counts[cur] or marks[cur]) must start at
// zero; a record left behind by steps of the other kind is cleared here,
// outside any captured graph.
int prepare_deposits(slime_ctx* ctx, bool marks) {
    const int cur = ctx->cur;
    const size_t cells = (size_t)ctx->W * ctx->H;
    if (marks && ctx->marks_dirty[cur]) {
        CK(cudaMemsetAsync(ctx->marks[cur], 0, cells, ctx->stream), "clearing deposit marks");
        ctx->marks_dirty[cur] = false;
    }
    if (!marks && ctx->counts_dirty[cur]) {
        CK(cudaMemsetAsync(ctx->counts[cur], 0, cells * sizeof(uint32_t), ctx->stream), "clearing deposit counts");
        ctx->counts_dirty[cur] = false;
    }
    return SLIME_OK;
}

// Bookkeeping after m steps of one kind (ctx->cur already advanced): the
// last step's record holds its deposits, the trail pass cleared the other.
void after_steps(slime_ctx* ctx, bool marks, uint32_t m) {
    if (m == 0) return;
    bool* dirty = marks ? ctx->marks_dirty : ctx->counts_dirty;
    dirty[ctx->cur] = false;
    dirty[1 - ctx->cur] = true;
    ctx->trail_clean = ctx->trail_clean && keeps_trail_clean(ctx->dev);
    ctx->last_marks = marks;
    ctx->last_counts_valid = true;
}

// The two passes of one step on the context's stream (also used under
// capture).  The agent pass keeps the trail it senses resident; the trail
// pass marks the trail it writes, which the next agent pass senses.  With
// `pdl` a pass is a programmatic dependent of the kernel just before it in
// the stream: the other pass of this context.
cudaError_t enqueue_agents_pass(slime_ctx* ctx, bool marks, bool pdl) {
    const int cur = ctx->cur;
    cudaAccessPolicyWindow wa;
    bool ha = trail_window(ctx, ctx->trail[cur], &wa, kWindowAgents);
    return launch_agents(ctx->dev, ctx->agents, ctx->trail[cur], ctx->counts[cur], ctx->stream, ctx->agent_shape,
                         ha ? &wa : nullptr, ctx->trail_tex[cur], marks ? ctx->marks[cur] : nullptr, pdl);
}

cudaError_t enqueue_trail_pass(slime_ctx* ctx, bool marks, bool pdl) {
    const int cur = ctx->cur;
    cudaAccessPolicyWindow wt;
    bool ht = trail_window(ctx, ctx->trail[1 - cur], &wt, kWindowTrail);
    if (marks)
        return launch_trail_marks(ctx->dev, ctx->tile, ctx->trail[cur], ctx->marks[cur], ctx->trail[1 - cur],
                                  ctx->marks[1 - cur], ctx->stream, ht ? &wt : nullptr, pdl, &ctx->tmaps, cur);
    return launch_trail(ctx->dev, ctx->tile, ctx->trail[cur], ctx->counts[cur], ctx->trail[1 - cur],
                        ctx->counts[1 - cur], ctx->stream, ht ? &wt : nullptr, pdl, &ctx->tmaps, cur);
}

// `chained`: the operation before this step on the stream is the previous
// step's trail pass, so the agent pass may start while it finishes; the trail
// pass always follows the agent pass's kernel when there are agents.
cudaError_t enqueue_step(slime_ctx* ctx, bool marks, bool chained) {
    const bool agents = ctx->agents.n > 0;
    cudaError_t e = enqueue_agents_pass(ctx, marks, chained && agents);
    if (e != cudaSuccess) return e;
    e = enqueue_trail_pass(ctx, marks, agents);
    if (e != cudaSuccess) return e;
    ctx->cur = 1 - ctx->cur;
    return cudaSuccess;
}

uint64_t kernels_per_step(const slime_ctx* ctx, bool marks) {
    return 1 + (uint64_t)agent_pass_kernels(ctx->dev, ctx->agents.n, marks);
}

int run_steps_direct(slime_ctx* ctx, uint32_t m, bool marks) {
    for (uint32_t i = 0; i < m; i++) {
        CK(enqueue_step(ctx, marks, i > 0), "launching a step");
        ctx->launches += kernels_per_step(ctx, marks);
        ctx->steps_done++;
    }
    ctx->last_counts_valid = true;
    return SLIME_OK;
}

// The graph of m steps from the current parity with this deposit record,
// captured on first use.
int step_graph(slime_ctx* ctx, uint32_t m, bool marks, cudaGraphExec_t* out) {
    auto key = std::make_pair(m, ctx->cur | (marks ? 2 : 0));
    auto it = ctx->graphs.find(key);
    cudaGraphExec_t exec = nullptr;
    if (it == ctx->graphs.end()) {
        const int saved = ctx->cur;
        CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal), "beginning graph capture");
        cudaError_t ce = cudaSuccess;
        for (uint32_t i = 0; i < m && ce == cudaSuccess; i++) ce = enqueue_step(ctx, marks, i > 0);
        cudaGraph_t graph = nullptr;
        cudaError_t ee = cudaStreamEndCapture(ctx->stream, &graph);
        ctx->cur = saved;
        if (ce != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            return cuda_error(ctx->err, ce, "capturing steps");
        }
        CK(ee, "ending graph capture");
        cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        CK(ie, "instantiating step graph");
        ctx->graphs[key] = exec;
    } else {
        exec = it->second;
    }
    *out = exec;
    return SLIME_OK;
}

int run_steps_graph(slime_ctx* ctx, uint32_t m, bool marks) {
    cudaGraphExec_t exec = nullptr;
    int rc = step_graph(ctx, m, marks, &exec);
    if (rc != SLIME_OK) return rc;
    CK(cudaGraphLaunch(exec, ctx->stream), "launching step graph");
    ctx->cur = (m & 1) ? 1 - ctx->cur : ctx->cur;
    ctx->launches += kernels_per_step(ctx, marks) * m;
    ctx->steps_done += m;
    ctx->last_counts_valid = true;
    return SLIME_OK;
}

int do_reorder(slime_ctx* ctx) {
    if (ctx->agents.n == 0) return SLIME_OK;
    if (!ctx->agents.ids) {
        CK(dev_alloc((void**)&ctx->ids_storage, ctx->agents.n_pad * sizeof(uint32_t)), "allocating agent ids");
        CK(cudaMemsetAsync(ctx->ids_storage, 0, ctx->agents.n_pad * sizeof(uint32_t), ctx->stream),
           "clearing agent ids");
        ctx->agents.ids = ctx->ids_storage;
        CK(launch_iota(ctx->agents.ids, ctx->agents.n, ctx->stream), "initialising agent ids");
        invalidate_graphs(ctx); // the agent kernel now reads ids
    }
    const bool partition = ctx->dev.dispatch_mode == SLIME_DISPATCH_REFERENCE;
    CK(launch_reorder(ctx->agents, ctx->W, ctx->H, (int)ctx->opt.reorder_cell_log2, ctx->reorder, ctx->stream,
                      partition ? reference_dispatch_updated(ctx->agents.n) : ~0ull),
       "reordering agents");
    ctx->launches += 5;
    ctx->reorders_done++;
    ctx->reordered = true;
    ctx->reorder_partitioned = partition;
    ctx->last_reorder_step = ctx->steps_done;
    return SLIME_OK;
}

// Whether the persisting-L2 window over the trail pays off for this context,
// and on which passes: `steps` full steps (an even number) with the window on
// both passes, on the trail pass only, on the agent pass only and without a
// carve-out, twice each in alternation, from a snapshot of the agents and the
// trail that is put back before every trial and at the end.  Without a
// snapshot buffer nothing changes.
int tune_l2_window(slime_ctx* ctx, uint32_t steps) {
    const size_t cells = (size_t)ctx->W * ctx->H;
    const size_t abytes = 4 * ctx->agents.n_pad * sizeof(float);
    const size_t tbytes = cells * sizeof(float);
    char* snap = nullptr;
    if (dev_alloc((void**)&snap, abytes + tbytes) != cudaSuccess) {
        cudaGetLastError();
        return SLIME_OK;
    }
    const int cur = ctx->cur;
    auto restore = [&]() -> cudaError_t {
        cudaError_t e = cudaMemcpyAsync(ctx->agent_block, snap, abytes, cudaMemcpyDeviceToDevice, ctx->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ctx->trail[cur], snap + abytes, tbytes, cudaMemcpyDeviceToDevice, ctx->stream);
        for (int i = 0; i < 2 && e == cudaSuccess; i++) {
            e = cudaMemsetAsync(ctx->counts[i], 0, cells * sizeof(uint32_t), ctx->stream);
            if (e == cudaSuccess) e = cudaMemsetAsync(ctx->marks[i], 0, cells, ctx->stream);
            ctx->counts_dirty[i] = ctx->marks_dirty[i] = false;
        }
        ctx->cur = cur;
        return e;
    };
    const bool marks = use_marks(ctx);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMemcpyAsync(snap, ctx->agent_block, abytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(snap + abytes, ctx->trail[cur], tbytes, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    // the window on both passes, on the trail pass only, on the agent pass
    // only, and no carve-out at all
    const unsigned passes[4] = {kWindowAgents | kWindowTrail, kWindowTrail, kWindowAgents, 0};
    float total[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    for (int round = 0; round < 2 && e == cudaSuccess; round++) {
        for (int c = 0; c < 4 && e == cudaSuccess; c++) {
            ctx->l2_tuned_off = passes[c] == 0;
            ctx->l2_window_passes = passes[c] ? passes[c] : 3;
            setup_l2(ctx);
            if (c == 0 && !ctx->l2_persist_bytes) break; // no carve-out to compare with
            e = restore();
            for (int w = 0; w < 2 && e == cudaSuccess; w++) e = enqueue_step(ctx, marks, w > 0);
            if (e == cudaSuccess) e = restore();
            if (e == cudaSuccess) e = cudaEventRecord(e0, ctx->stream);
            for (uint32_t i = 0; i < steps && e == cudaSuccess; i++) e = enqueue_step(ctx, marks, i > 0);
            if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
            if (e == cudaSuccess) e = cudaEventSynchronize(e1);
            float ms = 0.0f;
            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
            total[c] += ms;
            ctx->launches += (steps + 2) * kernels_per_step(ctx, marks);
        }
    }
    int best = 0;
    const bool measured = e == cudaSuccess && total[0] > 0.0f && total[3] > 0.0f;
    if (measured)
        for (int c = 1; c < 4; c++)
            if (total[c] > 0.0f && total[c] < total[best]) best = c;
    ctx->l2_tuned_off = passes[best] == 0;
    ctx->l2_window_passes = passes[best] ? passes[best] : 3;
    setup_l2(ctx);
    cudaError_t re = restore();
    if (re == cudaSuccess) re = cudaStreamSynchronize(ctx->stream);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    dev_free(snap);
    invalidate_graphs(ctx);
    ctx->last_counts_valid = false;
    if (e != cudaSuccess) return cuda_error(ctx->err, e, "autotuning the L2 window");
    if (re != cudaSuccess) return cuda_error(ctx->err, re, "autotuning the L2 window");
    return SLIME_OK;
}

int ensure_dispatch_order(slime_ctx* ctx) {
    if (ctx->dev.dispatch_mode != SLIME_DISPATCH_REFERENCE || !ctx->reordered || ctx->reorder_partitioned)
        return SLIME_OK;
    return do_reorder(ctx);
}

// Capture the graphs that the next n steps replay (same chunking as
// run_steps: graph_chunk steps, cut at reorder boundaries), without stepping.
int prepare_steps(slime_ctx* ctx, uint32_t n) {
    if (!ctx->opt.use_graphs || ctx->agents.n == 0) return SLIME_OK;
    const bool marks = use_marks(ctx);
    const uint32_t chunk = ctx->opt.graph_chunk ? ctx->opt.graph_chunk : 50;
    const int saved = ctx->cur;
    uint64_t steps = ctx->steps_done;
    int rc = SLIME_OK;
    while (n > 0 && rc == SLIME_OK) {
        uint32_t m = n;
        if (ctx->opt.reorder_every) {
            uint64_t to_next = ctx->opt.reorder_every - steps % ctx->opt.reorder_every;
            if (to_next < m) m = (uint32_t)to_next;
        }
        const uint32_t take = m < chunk ? m : chunk;
        cudaGraphExec_t exec = nullptr;
        rc = step_graph(ctx, take, marks, &exec);
        if (take & 1) ctx->cur = 1 - ctx->cur;
        steps += take;
        n -= take;
    }
    ctx->cur = saved;
    return rc;
}

int run_steps(slime_ctx* ctx, uint32_t n) {
    int rc;
    if ((rc = ensure_dispatch_order(ctx)) != SLIME_OK) return rc;
    while (n > 0) {
        uint32_t m = n;
        if (ctx->opt.reorder_every) {
            if (ctx->steps_done % ctx->opt.reorder_every == 0 && ctx->last_reorder_step != ctx->steps_done)
                if ((rc = do_reorder(ctx)) != SLIME_OK) return rc;
            uint64_t to_next = ctx->opt.reorder_every - ctx->steps_done % ctx->opt.reorder_every;
            if (to_next < m) m = (uint32_t)to_next;
        }
        const bool marks = use_marks(ctx);
        if ((rc = prepare_deposits(ctx, marks)) != SLIME_OK) return rc;
        if (ctx->opt.use_graphs) {
            uint32_t chunk = ctx->opt.graph_chunk ? ctx->opt.graph_chunk : 50;
            uint32_t take = m < chunk ? m : chunk;
            if ((rc = run_steps_graph(ctx, take, marks)) != SLIME_OK) return rc;
            after_steps(ctx, marks, take);
            n -= take;
        } else {
            if ((rc = run_steps_direct(ctx, m, marks)) != SLIME_OK) return rc;
            after_steps(ctx, marks, m);
            n -= m;
        }
    }
    return SLIME_OK;
}

} // namespace slime

extern "C" {

const char* slime_version(void) { return "slime-gb300 0.1 (sm_103a)"; }

const char* slime_status_string(int status) {
    switch (status) {
    case SLIME_OK: return "ok";
    case SLIME_ERR_INVALID_ARGUMENT: return "invalid argument";
    case SLIME_ERR_OUT_OF_MEMORY: return "out of device memory";
    case SLIME_ERR_CUDA: return "CUDA error";
    case SLIME_ERR_STATE: return "invalid state";
    case SLIME_ERR_DEVICE_TIMEOUT: return "device-side wait timed out";
    case SLIME_ERR_NO_DEVICE: return "no CUDA device";
    default: return "unknown status";
    }
}

slime_ctx* slime_create(uint32_t width, uint32_t height, uint64_t n_agents, int* status) {
    std::string err;
    int dummy;
    if (!status) status = &dummy;
    if ((*status = valid_size(err, width, height, n_agents)) != SLIME_OK) return nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        *status = SLIME_ERR_NO_DEVICE;
        return nullptr;
    }
    slime_ctx* ctx = new slime_ctx();
    cudaGetDevice(&ctx->device);
    ctx->W = width;
    ctx->H = height;
    ctx->opt.use_graphs = 1;
    ctx->opt.graph_chunk = 50;
    ctx->opt.reorder_every = 0;
    ctx->opt.reorder_cell_log2 = 2;
    ctx->opt.l2_persist = 1;
    ctx->opt.trail_tile = 0;
    ctx->tile = trail_tile_default();
    int rc = SLIME_OK;
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
        rc = SLIME_ERR_CUDA;
    } else if ((rc = alloc_agents(ctx, n_agents)) == SLIME_OK && (rc = alloc_trail(ctx, width, height)) == SLIME_OK) {
        SlimeSettings s;
        slime_settings_default(&s);
        slime_params_from_settings(&s, width, height, &ctx->params);
        const char* why = nullptr;
        if (!make_dev_params(ctx->params, width, height, &ctx->dev, &why)) rc = SLIME_ERR_INVALID_ARGUMENT;
        else if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) rc = SLIME_ERR_CUDA;
        else setup_l2(ctx);
    }
    if (rc != SLIME_OK) {
        slime_destroy(ctx);
        *status = rc;
        return nullptr;
    }
    *status = SLIME_OK;
    return ctx;
}

void slime_destroy(slime_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    release_l2(ctx);
    invalidate_graphs(ctx);
    free_adjoint(ctx);
    free_agents(ctx);
    free_trail(ctx);
    if (ctx->staging) dev_free(ctx->staging);
    if (ctx->reorder.buf) dev_free(ctx->reorder.buf);
    if (ctx->aux) dev_free(ctx->aux);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->display_lut) dev_free(ctx->display_lut);
    if (ctx->display_image) dev_free(ctx->display_image);
    for (int b = 0; b < 2; b++) {
        if (ctx->display_snap[b]) dev_free(ctx->display_snap[b]);
        if (ctx->snap_copied[b]) cudaEventDestroy(ctx->snap_copied[b]);
    }
    if (ctx->snap_ready) cudaEventDestroy(ctx->snap_ready);
    if (ctx->copy_done) cudaEventDestroy(ctx->copy_done);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* slime_last_error(const slime_ctx* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int slime_set_params(slime_ctx* ctx, const SlimeParams* params) {
    if (!ctx || !params) return SLIME_ERR_INVALID_ARGUMENT;
    DevParams d;
    const char* why = nullptr;
    if (!make_dev_params(*params, ctx->W, ctx->H, &d, &why))
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "%s", why);
    ctx->params = *params;
    ctx->params.width = ctx->W;
    ctx->params.height = ctx->H;
    if (memcmp(&d, &ctx->dev, sizeof d) != 0) {
        ctx->dev = d;
        invalidate_graphs(ctx); // the parameter block is baked into the captured launches
    }
    return SLIME_OK;
}

int slime_get_params(const slime_ctx* ctx, SlimeParams* out) {
    if (!ctx || !out) return SLIME_ERR_INVALID_ARGUMENT;
    *out = ctx->params;
    return SLIME_OK;
}

int slime_set_options(slime_ctx* ctx, const SlimeOptions* o) {
    if (!ctx || !o) return SLIME_ERR_INVALID_ARGUMENT;
    if (o->trail_tile > (uint32_t)trail_tile_count())
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "trail_tile out of range (0..%d)",
                         trail_tile_count());
    if (o->reorder_cell_log2 > 15)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "reorder_cell_log2 must be <= 15");
    if (o->agent_shape > (uint32_t)agent_shape_count())
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "agent_shape out of range (0..%d)",
                         agent_shape_count());
    const bool l2_changed = (o->l2_persist != 0) != (ctx->opt.l2_persist != 0);
    ctx->opt = *o;
    if (ctx->opt.graph_chunk == 0) ctx->opt.graph_chunk = 50;
    if (l2_changed) {
        ctx->l2_tuned_off = false;
        ctx->l2_window_passes = 3;
        setup_l2(ctx);
        invalidate_graphs(ctx);
    }
    int tile = o->trail_tile ? (int)o->trail_tile - 1 : (ctx->tuned_tile >= 0 ? ctx->tuned_tile : trail_tile_default());
    int shape = o->agent_shape ? (int)o->agent_shape - 1 : (ctx->tuned_shape >= 0 ? ctx->tuned_shape : 0);
    if (tile != ctx->tile || shape != ctx->agent_shape) {
        ctx->tile = tile;
        ctx->agent_shape = shape;
        invalidate_graphs(ctx);
    }
    return SLIME_OK;
}

int slime_get_options(const slime_ctx* ctx, SlimeOptions* out) {
    if (!ctx || !out) return SLIME_ERR_INVALID_ARGUMENT;
    *out = ctx->opt;
    return SLIME_OK;
}

int slime_get_info(const slime_ctx* ctx, SlimeInfo* out) {
    if (!ctx || !out) return SLIME_ERR_INVALID_ARGUMENT;
    out->width = ctx->W;
    out->height = ctx->H;
    out->n_agents = ctx->agents.n;
    out->steps_done = ctx->steps_done;
    out->kernel_launches = ctx->launches;
    out->trail_tile = (uint32_t)ctx->tile;
    out->agent_shape = (uint32_t)ctx->agent_shape;
    out->trail_texture = ctx->trail_tex[0] && ctx->trail_tex[1] ? 1u : 0u;
    out->l2_persist_bytes = ctx->l2_persist_bytes;
    out->l2_window_passes = ctx->l2_persist_bytes ? ctx->l2_window_passes : 0u;
    out->_pad = 0;
    out->reordered = ctx->reordered ? 1u : 0u;
    out->reorders_done = ctx->reorders_done;
    return SLIME_OK;
}

int slime_upload_agents(slime_ctx* ctx, const float* aos, uint64_t n) {
    if (!ctx || (!aos && n)) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (n != ctx->agents.n)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "agent count %llu != context's %llu",
                         (unsigned long long)n, (unsigned long long)ctx->agents.n);
    if (n == 0) return SLIME_OK;
    int rc;
    if ((rc = ensure_staging(ctx, n * sizeof(float4))) != SLIME_OK) return rc;
    CK(cudaMemcpyAsync(ctx->staging, aos, n * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream), "uploading agents");
    CK(launch_aos_to_soa((const float4*)ctx->staging, ctx->agents, ctx->stream), "converting agents");
    if ((rc = reset_ids(ctx)) != SLIME_OK) return rc;
    CK(cudaStreamSynchronize(ctx->stream), "uploading agents");
    return SLIME_OK;
}

int slime_download_agents(slime_ctx* ctx, float* aos, uint64_t n) {
    if (!ctx || (!aos && n)) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (n != ctx->agents.n)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "agent count %llu != context's %llu",
                         (unsigned long long)n, (unsigned long long)ctx->agents.n);
    if (n == 0) return SLIME_OK;
    int rc;
    if ((rc = ensure_staging(ctx, n * sizeof(float4))) != SLIME_OK) return rc;
    CK(launch_soa_to_aos(ctx->agents, (float4*)ctx->staging, ctx->stream), "converting agents");
    CK(cudaMemcpyAsync(aos, ctx->staging, n * sizeof(float4), cudaMemcpyDeviceToHost, ctx->stream), "downloading agents");
    CK(cudaStreamSynchronize(ctx->stream), "downloading agents");
    return SLIME_OK;
}

int slime_seed_agents(slime_ctx* ctx, uint64_t seed, float hmin, float hmax) {
    if (!ctx || !isfinite(hmin) || !isfinite(hmax)) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(launch_seed_agents(ctx->agents, seed, (float)ctx->W, (float)ctx->H, hmin, hmax, ctx->params.agent_speed_min,
                          ctx->params.agent_speed_max, ctx->stream),
       "seeding agents");
    int rc;
    if ((rc = reset_ids(ctx)) != SLIME_OK) return rc;
    CK(cudaStreamSynchronize(ctx->stream), "seeding agents");
    return SLIME_OK;
}

int slime_reassign_speeds(slime_ctx* ctx, uint64_t seed) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(launch_reassign_speeds(ctx->agents, seed, ctx->params.agent_speed_min, ctx->params.agent_speed_max, ctx->stream),
       "reassigning speeds");
    CK(cudaStreamSynchronize(ctx->stream), "reassigning speeds");
    return SLIME_OK;
}

int slime_upload_trail(slime_ctx* ctx, const float* trail, uint64_t n_cells) {
    if (!ctx || !trail) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (n_cells != (uint64_t)ctx->W * ctx->H)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "trail has %llu cells, context has %llu",
                         (unsigned long long)n_cells, (unsigned long long)ctx->W * ctx->H);
    CK(cudaMemcpyAsync(ctx->trail[ctx->cur], trail, n_cells * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
       "uploading trail");
    // deposit marks need every value finite and >= 0 (or +inf): checked
    // while the copy runs
    bool clean = true;
    for (uint64_t i = 0; i < n_cells; i++) clean = clean && (trail[i] >= 0.0f);
    CK(cudaStreamSynchronize(ctx->stream), "uploading trail");
    ctx->trail_clean = clean;
    return SLIME_OK;
}

int slime_download_trail(slime_ctx* ctx, float* trail, uint64_t n_cells) {
    if (!ctx || !trail) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (n_cells != (uint64_t)ctx->W * ctx->H)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "trail has %llu cells, context has %llu",
                         (unsigned long long)n_cells, (unsigned long long)ctx->W * ctx->H);
    CK(cudaMemcpyAsync(trail, ctx->trail[ctx->cur], n_cells * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
       "downloading trail");
    CK(cudaStreamSynchronize(ctx->stream), "downloading trail");
    return SLIME_OK;
}

int slime_clear_trail(slime_ctx* ctx) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(cudaMemsetAsync(ctx->trail[ctx->cur], 0, (size_t)ctx->W * ctx->H * sizeof(float), ctx->stream), "clearing trail");
    CK(cudaStreamSynchronize(ctx->stream), "clearing trail");
    ctx->trail_clean = true;
    return SLIME_OK;
}

int slime_resize(slime_ctx* ctx, uint32_t width, uint32_t height) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    int rc;
    if ((rc = valid_size(ctx->err, width, height, ctx->agents.n)) != SLIME_OK) return rc;
    SlimeParams np = ctx->params;
    np.width = width;
    np.height = height;
    DevParams d;
    const char* why = nullptr;
    if (!make_dev_params(np, width, height, &d, &why)) return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "%s", why);
    CK(cudaStreamSynchronize(ctx->stream), "resizing");
    // the graphs and the adjoint recording belong to the old size; the new
    // trails replace the old only once allocated, so a resize that runs out
    // of memory leaves the agents and the trail as they were
    invalidate_graphs(ctx);
    free_adjoint(ctx);
    if ((rc = alloc_trail(ctx, width, height)) != SLIME_OK) return rc;
    // src/main.rs:987-993: scale = new / old as f32 division.
    float sx = slm_div((float)width, (float)ctx->W);
    float sy = slm_div((float)height, (float)ctx->H);
    ctx->W = width;
    ctx->H = height;
    ctx->params = np;
    ctx->dev = d;
    ctx->tuned_tile = -1;
    ctx->l2_tuned_off = false;
    ctx->l2_window_passes = 3;
    setup_l2(ctx);
    CK(launch_scale_positions(ctx->agents, sx, sy, ctx->stream), "scaling agent positions");
    CK(cudaStreamSynchronize(ctx->stream), "resizing");
    return SLIME_OK;
}

int slime_set_agent_count(slime_ctx* ctx, uint64_t n, uint64_t seed) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    int rc;
    if ((rc = valid_size(ctx->err, ctx->W, ctx->H, n)) != SLIME_OK) return rc;
    CK(cudaStreamSynchronize(ctx->stream), "changing the agent count");
    // the new block replaces the agents only once allocated: out of memory,
    // the context keeps its agents
    invalidate_graphs(ctx);
    free_adjoint(ctx);
    if ((rc = alloc_agents(ctx, n)) != SLIME_OK) return rc;
    ctx->reordered = false;
    // src/main.rs:700-712 draws x, y, angle in [0, 2*pi) and speed anew.
    return slime_seed_agents(ctx, seed, 0.0f, 6.28318530718f);
}

int slime_set_steps_done(slime_ctx* ctx, uint64_t steps_done) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    ctx->steps_done = steps_done;
    // no reorder has happened at this count yet: one falls due here when
    // steps_done is a multiple of reorder_every, as in the run being resumed
    ctx->last_reorder_step = ~0ull;
    return SLIME_OK;
}

namespace {
constexpr char kStateMagic[8] = {'S', 'L', 'M', 'S', 'T', 'A', 'T', 'E'};
constexpr uint32_t kStateVersion = 1;

// The fixed-size head of a state file (little-endian on the hosts this
// library builds for: x86-64 and AArch64).
struct StateHead {
    char magic[8];
    uint32_t version, width, height, params_bytes;
    uint64_t n_agents, steps_done;
};
static_assert(sizeof(StateHead) == 40, "state file head is 40 bytes");
} // namespace

int slime_state_save(slime_ctx* ctx, const char* path) {
    if (!ctx || !path) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    const uint64_t n = ctx->agents.n;
    const size_t cells = (size_t)ctx->W * ctx->H;
    std::vector<float> agents(4 * n), trail(cells);
    int rc;
    if ((rc = slime_download_agents(ctx, agents.data(), n)) != SLIME_OK) return rc;
    if ((rc = slime_download_trail(ctx, trail.data(), cells)) != SLIME_OK) return rc;
    StateHead h;
    memcpy(h.magic, kStateMagic, 8);
    h.version = kStateVersion;
    h.width = ctx->W;
    h.height = ctx->H;
    h.params_bytes = (uint32_t)sizeof(SlimeParams);
    h.n_agents = n;
    h.steps_done = ctx->steps_done;
    FILE* f = fopen(path, "wb");
    if (!f) return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "cannot open %s for writing", path);
    bool ok = fwrite(&h, sizeof h, 1, f) == 1 && fwrite(&ctx->params, sizeof(SlimeParams), 1, f) == 1 &&
              fwrite(agents.data(), sizeof(float), agents.size(), f) == agents.size() &&
              fwrite(trail.data(), sizeof(float), trail.size(), f) == trail.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok) return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "writing %s failed", path);
    return SLIME_OK;
}

int slime_state_load(slime_ctx* ctx, const char* path) {
    if (!ctx || !path) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    FILE* f = fopen(path, "rb");
    if (!f) return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "cannot open %s", path);
    StateHead h;
    SlimeParams p;
    const size_t cells = (size_t)ctx->W * ctx->H;
    std::vector<float> agents, trail;
    const char* why = nullptr;
    if (fread(&h, sizeof h, 1, f) != 1 || memcmp(h.magic, kStateMagic, 8) != 0) why = "not a state file";
    else if (h.version != kStateVersion) why = "unknown state file version";
    else if (h.params_bytes != sizeof(SlimeParams)) why = "state file holds parameters of another layout";
    else if (h.width != ctx->W || h.height != ctx->H || h.n_agents != ctx->agents.n)
        why = "state file is of another trail size or agent count";
    else if (fread(&p, sizeof p, 1, f) != 1) why = "truncated state file";
    if (!why) {
        agents.resize(4 * h.n_agents);
        trail.resize(cells);
        if (fread(agents.data(), sizeof(float), agents.size(), f) != agents.size() ||
            fread(trail.data(), sizeof(float), trail.size(), f) != trail.size())
            why = "truncated state file";
    }
    fclose(f);
    if (why) return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "%s: %s", path, why);
    DevParams d;
    const char* bad = nullptr;
    if (!make_dev_params(p, ctx->W, ctx->H, &d, &bad))
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "%s: %s", path, bad);
    int rc;
    if ((rc = slime_set_params(ctx, &p)) != SLIME_OK) return rc;
    if ((rc = slime_upload_agents(ctx, agents.data(), h.n_agents)) != SLIME_OK) return rc;
    if ((rc = slime_upload_trail(ctx, trail.data(), cells)) != SLIME_OK) return rc;
    return slime_set_steps_done(ctx, h.steps_done);
}

int slime_prepare_steps(slime_ctx* ctx, uint32_t n_steps) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    return prepare_steps(ctx, n_steps);
}

int slime_step(slime_ctx* ctx, uint32_t n_steps) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    return run_steps(ctx, n_steps);
}

int slime_sync(slime_ctx* ctx) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream), "synchronising");
    if (ctx->tile == kTrailTileTma && trail_tma_take_error())
        return set_error(ctx->err, SLIME_ERR_DEVICE_TIMEOUT,
                         "a trail tile gave up waiting for its tensor copies; its cells were not written");
    return SLIME_OK;
}

int slime_get_stream(slime_ctx* ctx, void** stream) {
    if (!ctx || !stream) return SLIME_ERR_INVALID_ARGUMENT;
    *stream = (void*)ctx->stream;
    return SLIME_OK;
}

namespace {
// The copy stream and its events, made at the first asynchronous download.
int ensure_copy_stream(slime_ctx* ctx) {
    if (ctx->copy_stream) return SLIME_OK;
    CK(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "creating copy stream");
    CK(cudaEventCreateWithFlags(&ctx->snap_ready, cudaEventDisableTiming), "creating event");
    CK(cudaEventCreateWithFlags(&ctx->copy_done, cudaEventDisableTiming), "creating event");
    for (int b = 0; b < 2; b++)
        CK(cudaEventCreateWithFlags(&ctx->snap_copied[b], cudaEventDisableTiming), "creating event");
    return SLIME_OK;
}
} // namespace

int slime_download_trail_async(slime_ctx* ctx, float* trail, uint64_t n_cells) {
    if (!ctx || !trail) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    const size_t cells = (size_t)ctx->W * ctx->H;
    if (n_cells != cells)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "trail has %llu cells, context has %llu",
                         (unsigned long long)n_cells, (unsigned long long)cells);
    int rc = ensure_copy_stream(ctx);
    if (rc != SLIME_OK) return rc;
    if (ctx->display_cells != cells) {
        if (ctx->copy_pending) CK(cudaEventSynchronize(ctx->copy_done), "waiting for the previous copy");
        ctx->copy_pending = false;
        ctx->display_cells = 0;
        for (int b = 0; b < 2; b++) {
            if (ctx->display_snap[b]) dev_free(ctx->display_snap[b]);
            ctx->display_snap[b] = nullptr;
            ctx->snap_copy_pending[b] = false;
        }
        for (int b = 0; b < 2; b++)
            CK(dev_alloc((void**)&ctx->display_snap[b], cells * sizeof(float)), "allocating display snapshots");
        ctx->display_cells = cells;
        ctx->display_next = 0;
    }
    const int b = ctx->display_next;
    ctx->display_next = 1 - b;
    // the host copy that last read this snapshot (two calls back) must be done
    if (ctx->snap_copy_pending[b]) CK(cudaStreamWaitEvent(ctx->stream, ctx->snap_copied[b], 0), "ordering copies");
    CK(cudaMemcpyAsync(ctx->display_snap[b], ctx->trail[ctx->cur], cells * sizeof(float), cudaMemcpyDeviceToDevice,
                       ctx->stream), "snapshotting trail");
    CK(cudaEventRecord(ctx->snap_ready, ctx->stream), "recording snapshot");
    CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->snap_ready, 0), "ordering copies");
    CK(cudaMemcpyAsync(trail, ctx->display_snap[b], cells * sizeof(float), cudaMemcpyDeviceToHost, ctx->copy_stream),
       "copying trail to the host");
    CK(cudaEventRecord(ctx->snap_copied[b], ctx->copy_stream), "recording copy");
    ctx->snap_copy_pending[b] = true;
    CK(cudaEventRecord(ctx->copy_done, ctx->copy_stream), "recording copy");
    ctx->copy_pending = true;
    return SLIME_OK;
}

int slime_wait_download(slime_ctx* ctx) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->copy_pending) CK(cudaEventSynchronize(ctx->copy_done), "waiting for the trail copy");
    ctx->copy_pending = false;
    return SLIME_OK;
}

int slime_download_deposit_counts(slime_ctx* ctx, uint32_t* counts, uint64_t n_cells) {
    if (!ctx || !counts) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (n_cells != (uint64_t)ctx->W * ctx->H)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "counts have %llu cells, context has %llu",
                         (unsigned long long)n_cells, (unsigned long long)ctx->W * ctx->H);
    if (!ctx->last_counts_valid) {
        memset(counts, 0, n_cells * sizeof(uint32_t));
        return SLIME_OK;
    }
    if (ctx->last_marks)
        return set_error(ctx->err, SLIME_ERR_STATE,
                         "the last step recorded which cells received deposits, not how many (every deposit "
                         "saturated the fold); set options.exact_counts = 1 to keep counts");
    CK(cudaMemcpyAsync(counts, ctx->counts[1 - ctx->cur], n_cells * sizeof(uint32_t), cudaMemcpyDeviceToHost,
                       ctx->stream),
       "downloading deposit counts");
    CK(cudaStreamSynchronize(ctx->stream), "downloading deposit counts");
    return SLIME_OK;
}

int slime_reorder_agents(slime_ctx* ctx) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    int rc = do_reorder(ctx);
    if (rc != SLIME_OK) return rc;
    CK(cudaStreamSynchronize(ctx->stream), "reordering agents");
    return SLIME_OK;
}

int slime_profile_steps(slime_ctx* ctx, uint32_t n_steps, double* agents_ms, double* trail_ms, double* other_ms) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    cudaEvent_t ev[4];
    for (auto& e : ev) CK(cudaEventCreate(&e), "creating events");
    double ta = 0, tt = 0, to = 0;
    int rc = SLIME_OK;
    for (uint32_t i = 0; i < n_steps && rc == SLIME_OK; i++) {
        cudaEventRecord(ev[0], ctx->stream);
        rc = ensure_dispatch_order(ctx);
        if (rc == SLIME_OK && ctx->opt.reorder_every && ctx->steps_done % ctx->opt.reorder_every == 0 &&
            ctx->last_reorder_step != ctx->steps_done)
            rc = do_reorder(ctx);
        const bool marks = use_marks(ctx);
        if (rc == SLIME_OK) rc = prepare_deposits(ctx, marks);
        if (rc != SLIME_OK) break;
        cudaEventRecord(ev[1], ctx->stream);
        cudaError_t e = enqueue_agents_pass(ctx, marks, false);
        cudaEventRecord(ev[2], ctx->stream);
        if (e == cudaSuccess) e = enqueue_trail_pass(ctx, marks, false);
        cudaEventRecord(ev[3], ctx->stream);
        if (e != cudaSuccess) {
            rc = cuda_error(ctx->err, e, "profiling a step");
            break;
        }
        ctx->cur = 1 - ctx->cur;
        ctx->steps_done++;
        ctx->launches += kernels_per_step(ctx, marks);
        after_steps(ctx, marks, 1);
        if ((e = cudaEventSynchronize(ev[3])) != cudaSuccess) {
            rc = cuda_error(ctx->err, e, "profiling a step");
            break;
        }
        float a, b, c;
        cudaEventElapsedTime(&a, ev[0], ev[1]);
        cudaEventElapsedTime(&b, ev[1], ev[2]);
        cudaEventElapsedTime(&c, ev[2], ev[3]);
        to += a;
        ta += b;
        tt += c;
    }
    for (auto& e : ev) cudaEventDestroy(e);
    if (agents_ms) *agents_ms = ta;
    if (trail_ms) *trail_ms = tt;
    if (other_ms) *other_ms = to;
    return rc;
}

int slime_profile_reorder(slime_ctx* ctx, uint32_t reps, double* ms) {
    if (!ctx || !ms) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    *ms = 0.0;
    if (ctx->agents.n == 0 || reps == 0) return SLIME_OK;
    // the first reorder allocates the id map and the sort scratch: untimed
    int rc = do_reorder(ctx);
    if (rc != SLIME_OK) return rc;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "creating events");
    CK(cudaEventCreate(&e1), "creating events");
    cudaError_t e = cudaEventRecord(e0, ctx->stream);
    for (uint32_t r = 0; r < reps && rc == SLIME_OK && e == cudaSuccess; r++) rc = do_reorder(ctx);
    if (e == cudaSuccess) e = cudaEventRecord(e1, ctx->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.0f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != SLIME_OK) return rc;
    if (e != cudaSuccess) return cuda_error(ctx->err, e, "timing reorders");
    *ms = t;
    return SLIME_OK;
}

int slime_autotune(slime_ctx* ctx, uint32_t reps) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (reps == 0) reps = 5;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0), "creating events");
    CK(cudaEventCreate(&e1), "creating events");
    const int cur = ctx->cur;
    const size_t cells = (size_t)ctx->W * ctx->H;
    // 1. trail tiles.  The trial launches read trail[cur] and the (zero)
    // counts[cur] and write the other buffers, so the state is untouched; the
    // previous step's counts are overwritten with zeros.
    // Each tile runs with the deposit record the steps would use with it.
    float best = 1e30f;
    int best_tile = ctx->tile;
    const bool marks_ok = marks_allowed(ctx);
    for (int t = 0; t < trail_tile_count(); t++) {
        if (!trail_tile_supported(ctx->dev, t) || (t == kTrailTileTma && !ctx->tmaps.ok)) continue;
        const bool mk = marks_ok && trail_tile_streams(ctx->dev, t);
        auto trial = [&]() {
            return mk ? launch_trail_marks(ctx->dev, t, ctx->trail[cur], ctx->marks[cur], ctx->trail[1 - cur],
                                           ctx->marks[1 - cur], ctx->stream, nullptr, false, &ctx->tmaps, cur)
                      : launch_trail(ctx->dev, t, ctx->trail[cur], ctx->counts[cur], ctx->trail[1 - cur],
                                     ctx->counts[1 - cur], ctx->stream, nullptr, false, &ctx->tmaps, cur);
        };
        cudaError_t e = trial(); // warm-up
        if (e != cudaSuccess) continue;
        (mk ? ctx->marks_dirty : ctx->counts_dirty)[1 - cur] = false; // zeroed by the trial
        cudaEventRecord(e0, ctx->stream);
        for (uint32_t r = 0; r < reps; r++) trial();
        cudaEventRecord(e1, ctx->stream);
        CK(cudaEventSynchronize(e1), "autotuning");
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        ctx->launches += reps + 1;
        if (ms < best) {
            best = ms;
            best_tile = t;
        }
    }
    // 2. agent-kernel shapes, on a snapshot of the agents that is put back
    // afterwards (the trial passes write agents and the deposit record).
    // With reordering on, the agents are put in Morton order first, as the
    // steps will have them.  Each shape starts from the snapshot, makes one
    // untimed pass (the copy back evicts the trail from L2) and is timed over
    // `reps` passes in a row with the deposit record the steps will use;
    // twice, keeping the faster.
    if (ctx->opt.reorder_every && ctx->agents.n > 0) {
        int rrc = do_reorder(ctx);
        if (rrc != SLIME_OK) return rrc;
    }
    int best_shape = ctx->agent_shape;
    if (ctx->agents.n > 0) {
        const int tile_now = ctx->opt.trail_tile ? (int)ctx->opt.trail_tile - 1 : best_tile;
        uint8_t* mk = (marks_ok && trail_tile_streams(ctx->dev, tile_now)) ? ctx->marks[cur] : nullptr;
        const size_t abytes = 4 * ctx->agents.n_pad * sizeof(float);
        void* snap = nullptr;
        if (dev_alloc((void**)&snap, abytes) == cudaSuccess) {
            CK(cudaMemcpyAsync(snap, ctx->agent_block, abytes, cudaMemcpyDeviceToDevice, ctx->stream), "snapshot");
            float best_a = 1e30f;
            for (int round = 0; round < 2; round++)
                for (int sh = 0; sh < agent_shape_count(); sh++) {
                    // without a texture the gather shapes repeat their pointer twins
                    if (agent_shape_uses_texture(sh) && !ctx->trail_tex[cur]) continue;
                    cudaMemcpyAsync(ctx->agent_block, snap, abytes, cudaMemcpyDeviceToDevice, ctx->stream);
                    launch_agents(ctx->dev, ctx->agents, ctx->trail[cur], ctx->counts[cur], ctx->stream, sh, nullptr,
                                  ctx->trail_tex[cur], mk);
                    cudaEventRecord(e0, ctx->stream);
                    for (uint32_t r = 0; r < reps; r++)
                        launch_agents(ctx->dev, ctx->agents, ctx->trail[cur], ctx->counts[cur], ctx->stream, sh,
                                      nullptr, ctx->trail_tex[cur], mk);
                    cudaEventRecord(e1, ctx->stream);
                    CK(cudaEventSynchronize(e1), "autotuning");
                    float ms = 0;
                    cudaEventElapsedTime(&ms, e0, e1);
                    ctx->launches += (reps + 1) * (uint64_t)agent_pass_kernels(ctx->dev, ctx->agents.n, mk != nullptr);
                    if (ms < best_a) {
                        best_a = ms;
                        best_shape = sh;
                    }
                }
            CK(cudaMemcpyAsync(ctx->agent_block, snap, abytes, cudaMemcpyDeviceToDevice, ctx->stream), "restore");
            CK(cudaMemsetAsync(ctx->counts[cur], 0, cells * sizeof(uint32_t), ctx->stream), "restore");
            if (mk) CK(cudaMemsetAsync(ctx->marks[cur], 0, cells, ctx->stream), "restore");
            CK(cudaStreamSynchronize(ctx->stream), "autotuning");
            dev_free(snap);
        } else {
            cudaGetLastError();
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->last_counts_valid = false;
    ctx->tuned_tile = best_tile;
    ctx->tuned_shape = best_shape;
    int tile = ctx->opt.trail_tile ? (int)ctx->opt.trail_tile - 1 : best_tile;
    int shape = ctx->opt.agent_shape ? (int)ctx->opt.agent_shape - 1 : best_shape;
    if (tile != ctx->tile || shape != ctx->agent_shape) {
        ctx->tile = tile;
        ctx->agent_shape = shape;
        invalidate_graphs(ctx);
    }
    // 3. the persisting-L2 window, with the tile and shape just chosen
    if (ctx->opt.l2_persist && ctx->agents.n > 0) {
        ctx->l2_tuned_off = false;
        ctx->l2_window_passes = 3;
        setup_l2(ctx);
        if (ctx->l2_persist_bytes) return tune_l2_window(ctx, 2 * (reps < 5 ? 5 : reps));
    }
    return SLIME_OK;
}

int slime_colorize_async(slime_ctx* ctx, const uint8_t* lut768, uint32_t tw, uint32_t th, uint8_t* rgba_out) {
    if (!ctx || !lut768 || !rgba_out || tw == 0 || th == 0) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    int rc = ensure_copy_stream(ctx);
    if (rc != SLIME_OK) return rc;
    const size_t bytes = (size_t)tw * th * 4;
    if (ctx->display_image_bytes != bytes) {
        if (ctx->copy_pending) CK(cudaEventSynchronize(ctx->copy_done), "waiting for the previous copy");
        ctx->copy_pending = false;
        if (ctx->display_image) dev_free(ctx->display_image);
        ctx->display_image = nullptr;
        ctx->display_image_bytes = 0;
        CK(dev_alloc((void**)&ctx->display_image, bytes), "allocating display image");
        ctx->display_image_bytes = bytes;
    }
    if (!ctx->display_lut) CK(dev_alloc((void**)&ctx->display_lut, 768), "allocating display LUT");
    if (!ctx->display_lut_valid || memcmp(ctx->display_lut_host, lut768, 768) != 0) {
        // a copy from pageable memory waits for the stream: only when the LUT changes
        memcpy(ctx->display_lut_host, lut768, 768);
        CK(cudaMemcpyAsync(ctx->display_lut, ctx->display_lut_host, 768, cudaMemcpyHostToDevice, ctx->stream),
           "uploading LUT");
        CK(cudaStreamSynchronize(ctx->stream), "uploading LUT");
        ctx->display_lut_valid = true;
    }
    // the previous host copy may still read the image: finish it before overwriting
    if (ctx->copy_pending) CK(cudaStreamWaitEvent(ctx->stream, ctx->copy_done, 0), "ordering copies");
    CK(launch_colorize(ctx->trail[ctx->cur], ctx->W, ctx->H, ctx->display_lut, tw, th, ctx->display_image,
                       ctx->stream),
       "colourising");
    ctx->launches += 1;
    CK(cudaEventRecord(ctx->snap_ready, ctx->stream), "recording image");
    CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->snap_ready, 0), "ordering copies");
    CK(cudaMemcpyAsync(rgba_out, ctx->display_image, bytes, cudaMemcpyDeviceToHost, ctx->copy_stream),
       "copying the image to the host");
    CK(cudaEventRecord(ctx->copy_done, ctx->copy_stream), "recording copy");
    ctx->copy_pending = true;
    return SLIME_OK;
}

int slime_colorize(slime_ctx* ctx, const uint8_t* lut768, uint32_t tw, uint32_t th, uint8_t* rgba_out) {
    if (!ctx || !lut768 || !rgba_out || tw == 0 || th == 0) return SLIME_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    size_t need = 768 + (size_t)tw * th * 4;
    if (ctx->aux_bytes < need) {
        if (ctx->aux) dev_free(ctx->aux);
        ctx->aux = nullptr;
        ctx->aux_bytes = 0;
        CK(dev_alloc((void**)&ctx->aux, need), "allocating display buffer");
        ctx->aux_bytes = need;
    }
    uint8_t* dlut = (uint8_t*)ctx->aux;
    uint8_t* drgba = dlut + 768;
    CK(cudaMemcpyAsync(dlut, lut768, 768, cudaMemcpyHostToDevice, ctx->stream), "uploading LUT");
    CK(launch_colorize(ctx->trail[ctx->cur], ctx->W, ctx->H, dlut, tw, th, drgba, ctx->stream), "colourising");
    ctx->launches += 1;
    CK(cudaMemcpyAsync(rgba_out, drgba, (size_t)tw * th * 4, cudaMemcpyDeviceToHost, ctx->stream), "downloading image");
    CK(cudaStreamSynchronize(ctx->stream), "colourising");
    return SLIME_OK;
}

} // extern "C"
