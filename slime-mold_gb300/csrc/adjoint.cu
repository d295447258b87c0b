// adjoint.cu - checkpointed adjoint of the deposit -> decay -> diffuse chain.
//
// With the agent trajectories frozen (steering is piecewise constant in the
// trail, so its a.e. derivative is zero) the per-step deposit counts k_s are
// constants and one step is the map
//   T_{s+1} = (1 - r) u + r B(u),   u = Decay(f),   f = Fold(T_s, k_s)
// with B the toroidal blur (3x3 box or separable Gaussian; symmetric, so
// B^T = B).  Its adjoint, given g = dL/dT_{s+1}:
//   dL/dr      += sum g (B(u) - u)                       (if 0 < rate < 1)
//   g_u         = (1 - r) g + r B(g)
//   multiply:  dL/ddecay += sum g_u f,  g_f = decay g_u
//   subtract:  a = [f - decay*0.001 > 0], dL/ddecay += -0.001 sum a g_u, g_f = a g_u
//   fold:      c = [k == 0 or 0 < f < 1] (unclamped),
//              dL/ddep += sum c k g_f,  dL/dT_s = c g_f.
// The forward is recorded with a checkpoint of agents and trail every K steps;
// the backward replays each segment from its checkpoint (bit-identical to the
// recorded run), keeps T_s and k_s of the segment in HBM, and runs one fused
// stencil kernel per step backwards through it.
#include "ctx.h"

using namespace slime;

namespace slime {
namespace {

constexpr int kThreads = 256;
constexpr int kTW = 64, kTH = 16;

__device__ __forceinline__ double block_sum(double v, double* red) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; w++) t += red[w];
    __syncthreads();
    return t;
}

template <int R, bool kGauss>
__global__ void __launch_bounds__(kThreads) adjoint_kernel(const __grid_constant__ DevParams p,
                                                           const float* __restrict__ T,
                                                           const uint32_t* __restrict__ K,
                                                           const float* __restrict__ gin, float* __restrict__ gout,
                                                           double* __restrict__ acc, uint32_t rate_active) {
    constexpr int SW = kTW + 2 * R, SH = kTH + 2 * R;
    extern __shared__ float sm[];
    float* su = sm;
    float* sg = sm + SH * SW;
    float* hg = sg + SH * SW; // Gaussian only: horizontal pass of g
    __shared__ double red[kThreads / 32];
    const int W = p.W, H = p.H;
    const int x0 = blockIdx.x * kTW, y0 = blockIdx.y * kTH;
    for (int i = threadIdx.x; i < SH * SW; i += kThreads) {
        int ly = i / SW, lx = i - ly * SW;
        int gi = wrap_coord(y0 + ly - R, H) * W + wrap_coord(x0 + lx - R, W);
        su[i] = apply_decay(p, fold_deposits(__ldg(T + gi), __ldg(K + gi), p.dep));
        sg[i] = __ldg(gin + gi);
    }
    __syncthreads();
    if (kGauss) {
        for (int i = threadIdx.x; i < SH * kTW; i += kThreads) {
            int ly = i / kTW, lx = i - ly * kTW;
            float b = 0.0f;
#pragma unroll
            for (int t = 0; t <= 2 * R; t++) b = slm_fma(p.w[t], sg[ly * SW + lx + t], b);
            hg[i] = b;
        }
        __syncthreads();
    }
    float sd = 0.0f, sr = 0.0f, sp = 0.0f;
    const float r = p.rate;
    for (int i = threadIdx.x; i < kTW * kTH; i += kThreads) {
        int ly = i / kTW, lx = i - ly * kTW;
        int gx = x0 + lx, gy = y0 + ly;
        if (gx >= W || gy >= H) continue;
        int c = (ly + R) * SW + lx + R;
        float u = su[c], g = sg[c];
        // B(g) for the adjoint of the blur, and B(u) - u for the rate
        // gradient in difference form (B(u) - u is small against u, so it is
        // summed from neighbour-minus-centre differences).
        float bg, bmu;
        if (kGauss) {
            float b = 0.0f;
#pragma unroll
            for (int t = 0; t <= 2 * R; t++) b = slm_fma(p.w[t], hg[(ly + t) * kTW + lx], b);
            bg = b;
            float dsum = 0.0f;
#pragma unroll
            for (int dy = 0; dy <= 2 * R; dy++) {
                float row = 0.0f;
#pragma unroll
                for (int dx = 0; dx <= 2 * R; dx++) row += p.w[dx] * (su[(ly + dy) * SW + lx + dx] - u);
                dsum += p.w[dy] * row;
            }
            bmu = dsum + p.w2sum_m1 * u;
        } else {
            float b = 0.0f, dsum = 0.0f;
#pragma unroll
            for (int dy = -1; dy <= 1; dy++)
#pragma unroll
                for (int dx = -1; dx <= 1; dx++) {
                    b += sg[c + dy * SW + dx];
                    dsum += su[c + dy * SW + dx] - u;
                }
            bg = b * (1.0f / 9.0f);
            bmu = dsum * (1.0f / 9.0f);
        }
        if (rate_active) sr += g * bmu;
        float g_u = (1.0f - r) * g + r * bg;
        int gi = gy * W + gx;
        uint32_t k = __ldg(K + gi);
        float f = fold_deposits(__ldg(T + gi), k, p.dep);
        float g_f;
        if (p.decay_mode == SLIME_DECAY_MULTIPLY) {
            sd += g_u * f;
            g_f = p.decay * g_u;
        } else {
            bool act = slm_sub(f, p.decay_k) > 0.0f;
            sd += act ? -0.001f * g_u : 0.0f;
            g_f = act ? g_u : 0.0f;
        }
        bool unclamped = (k == 0u) || (f > 0.0f && f < 1.0f);
        if (unclamped) sp += g_f * (float)k;
        gout[gi] = unclamped ? g_f : 0.0f;
    }
    double td = block_sum((double)sd, red);
    double tr = block_sum((double)sr, red);
    double tp = block_sum((double)sp, red);
    if (threadIdx.x == 0) {
        atomicAdd(acc + 0, td);
        atomicAdd(acc + 1, tr);
        atomicAdd(acc + 2, tp);
    }
}

template <int R, bool kGauss>
cudaError_t launch_adj(const DevParams& p, const float* T, const uint32_t* K, const float* gin, float* gout,
                       double* acc, uint32_t rate_active, cudaStream_t s) {
    constexpr int SW = kTW + 2 * R, SH = kTH + 2 * R;
    size_t smem = sizeof(float) * (2 * SH * SW + (kGauss ? SH * kTW : 0));
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(adjoint_kernel<R, kGauss>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    dim3 grid((p.W + kTW - 1) / kTW, (p.H + kTH - 1) / kTH);
    adjoint_kernel<R, kGauss><<<grid, kThreads, smem, s>>>(p, T, K, gin, gout, acc, rate_active);
    return cudaGetLastError();
}

} // namespace

cudaError_t launch_adjoint_step(const DevParams& p, const float* T, const uint32_t* K, const float* gin,
                                float* gout, double* acc, uint32_t rate_active, cudaStream_t s) {
    if (p.blur_mode != SLIME_BLUR_GAUSS) return launch_adj<1, false>(p, T, K, gin, gout, acc, rate_active, s);
    switch (p.R) {
    case 0: return launch_adj<0, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 1: return launch_adj<1, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 2: return launch_adj<2, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 3: return launch_adj<3, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 4: return launch_adj<4, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 5: return launch_adj<5, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 6: return launch_adj<6, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 7: return launch_adj<7, true>(p, T, K, gin, gout, acc, rate_active, s);
    case 8: return launch_adj<8, true>(p, T, K, gin, gout, acc, rate_active, s);
    default: return cudaErrorInvalidValue;
    }
}

void free_adjoint(slime_ctx* ctx) {
    auto& a = ctx->adj;
    for (auto& kv : a.seg_graphs) cudaGraphExecDestroy(kv.second);
    a.seg_graphs.clear();
    void* ptrs[] = {a.ckpt_agents, a.ckpt_ids, a.ckpt_trail, a.seg_trail, a.seg_counts, a.g[0], a.g[1],
                    a.acc, a.agents_tmp, a.ids_tmp};
    for (void* q : ptrs)
        if (q) dev_free(q);
    a = slime_ctx::Adjoint();
}

} // namespace slime

#define CK(expr, what)                                                                                      \
    do {                                                                                                    \
        cudaError_t _e = (expr);                                                                            \
        if (_e != cudaSuccess) return cuda_error(ctx->err, _e, what);                                       \
    } while (0)

extern "C" {

int slime_forward_record(slime_ctx* ctx, uint32_t n_steps, uint32_t ckpt_every) {
    if (!ctx) return SLIME_ERR_INVALID_ARGUMENT;
    if (n_steps == 0 || ckpt_every == 0)
        return set_error(ctx->err, SLIME_ERR_INVALID_ARGUMENT, "n_steps and ckpt_every must be >= 1");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream), "forward_record");
    free_adjoint(ctx);
    int orc = ensure_dispatch_order(ctx);
    if (orc != SLIME_OK) return orc;
    auto& a = ctx->adj;
    const size_t cells = (size_t)ctx->W * ctx->H;
    const uint64_t n_pad = ctx->agents.n_pad;
    const uint32_t K = ckpt_every < n_steps ? ckpt_every : n_steps;
    a.n_steps = n_steps;
    a.ckpt_every = K;
    a.n_ckpt = (n_steps + K - 1) / K;
    a.dev = ctx->dev;
    a.tile = ctx->tile;
    a.agent_shape = ctx->agent_shape;
    a.rate_active = (ctx->params.diffusion_rate > 0.0f && ctx->params.diffusion_rate < 1.0f) ? 1u : 0u;
    a.n = ctx->agents.n;
    a.n_pad = n_pad;
    a.with_ids = ctx->agents.ids != nullptr;
    cudaError_t e;
    if ((e = dev_alloc((void**)&a.ckpt_agents, (size_t)a.n_ckpt * 4 * n_pad * sizeof(float))) != cudaSuccess ||
        (a.with_ids && (e = dev_alloc((void**)&a.ckpt_ids, (size_t)a.n_ckpt * n_pad * sizeof(uint32_t))) != cudaSuccess) ||
        (e = dev_alloc((void**)&a.ckpt_trail, (size_t)a.n_ckpt * cells * sizeof(float))) != cudaSuccess) {
        free_adjoint(ctx);
        return cuda_error(ctx->err, e, "allocating checkpoints");
    }
    for (uint32_t s = 0; s < n_steps; s++) {
        if (s % K == 0) {
            uint32_t j = s / K;
            CK(cudaMemcpyAsync(a.ckpt_agents + (size_t)j * 4 * n_pad, ctx->agent_block, 4 * n_pad * sizeof(float),
                               cudaMemcpyDeviceToDevice, ctx->stream), "checkpointing agents");
            if (a.with_ids)
                CK(cudaMemcpyAsync(a.ckpt_ids + (size_t)j * n_pad, ctx->agents.ids, n_pad * sizeof(uint32_t),
                                   cudaMemcpyDeviceToDevice, ctx->stream), "checkpointing ids");
            CK(cudaMemcpyAsync(a.ckpt_trail + (size_t)j * cells, ctx->trail[ctx->cur], cells * sizeof(float),
                               cudaMemcpyDeviceToDevice, ctx->stream), "checkpointing trail");
        }
        const bool marks = use_marks(ctx);
        int prc = prepare_deposits(ctx, marks);
        if (prc != SLIME_OK) return prc;
        CK(enqueue_step(ctx, marks, false), "recording a step");
        after_steps(ctx, marks, 1);
        ctx->launches += kernels_per_step(ctx, marks);
        ctx->steps_done++;
    }
    ctx->last_counts_valid = true;
    CK(cudaStreamSynchronize(ctx->stream), "forward_record");
    a.recorded = true;
    return SLIME_OK;
}

int slime_backward(slime_ctx* ctx, const float* dl_dtrail_final, SlimeGrads* grads, float* d_trail0) {
    if (!ctx || !dl_dtrail_final || !grads) return SLIME_ERR_INVALID_ARGUMENT;
    auto& a = ctx->adj;
    if (!a.recorded) return set_error(ctx->err, SLIME_ERR_STATE, "no recorded forward run (slime_forward_record)");
    if (a.n != ctx->agents.n || a.n_pad != ctx->agents.n_pad)
        return set_error(ctx->err, SLIME_ERR_STATE, "the agent buffer changed since the recording");
    cudaSetDevice(ctx->device);
    const size_t cells = (size_t)ctx->W * ctx->H;
    const uint32_t K = a.ckpt_every;
    cudaError_t e;
    if (!a.seg_trail) {
        // W + 2 zero floats past the last trail: the sampler's discarded taps
        if ((e = dev_alloc((void**)&a.seg_trail, ((size_t)K * cells + ctx->W + 2) * sizeof(float))) != cudaSuccess ||
            (e = cudaMemset(a.seg_trail, 0, ((size_t)K * cells + ctx->W + 2) * sizeof(float))) != cudaSuccess ||
            (e = dev_alloc((void**)&a.seg_counts, (size_t)K * cells * sizeof(uint32_t))) != cudaSuccess ||
            (e = dev_alloc((void**)&a.g[0], cells * sizeof(float))) != cudaSuccess ||
            (e = dev_alloc((void**)&a.g[1], cells * sizeof(float))) != cudaSuccess ||
            (e = dev_alloc((void**)&a.acc, 4 * sizeof(double))) != cudaSuccess ||
            (e = dev_alloc((void**)&a.agents_tmp, 4 * a.n_pad * sizeof(float))) != cudaSuccess ||
            (a.with_ids && (e = dev_alloc((void**)&a.ids_tmp, a.n_pad * sizeof(uint32_t))) != cudaSuccess))
            return cuda_error(ctx->err, e, "allocating adjoint buffers");
    }
    CK(cudaMemcpyAsync(a.g[0], dl_dtrail_final, cells * sizeof(float), cudaMemcpyHostToDevice, ctx->stream),
       "uploading dL/dT");
    CK(cudaMemsetAsync(a.acc, 0, 4 * sizeof(double), ctx->stream), "clearing gradients");
    int cg = 0;
    AgentsSoA tmp;
    tmp.x = a.agents_tmp;
    tmp.y = a.agents_tmp + a.n_pad;
    tmp.th = a.agents_tmp + 2 * a.n_pad;
    tmp.v = a.agents_tmp + 3 * a.n_pad;
    tmp.ids = a.with_ids ? a.ids_tmp : nullptr;
    tmp.n = a.n;
    tmp.n_pad = a.n_pad;
    // One segment after its restore: the replay of its m steps from the
    // checkpoint (keeping T_s and k_s), then its m backward steps, starting
    // from g[g0].  The same launches for every segment of m steps: captured
    // once per (m, g0) as a CUDA graph and replayed.
    auto enqueue_segment = [&](uint32_t m, int g0) -> cudaError_t {
        cudaError_t ce = cudaSuccess;
        for (uint32_t i = 0; i < m && ce == cudaSuccess; i++) {
            float* Ti = a.seg_trail + (size_t)i * cells;
            uint32_t* Ki = a.seg_counts + (size_t)i * cells;
            ce = launch_agents(a.dev, tmp, Ti, Ki, ctx->stream, a.agent_shape);
            if (ce == cudaSuccess && i + 1 < m) ce = launch_trail(a.dev, a.tile, Ti, Ki, Ti + cells, nullptr, ctx->stream);
        }
        int gi = g0;
        for (int64_t i = (int64_t)m - 1; i >= 0 && ce == cudaSuccess; i--) {
            ce = launch_adjoint_step(a.dev, a.seg_trail + (size_t)i * cells, a.seg_counts + (size_t)i * cells, a.g[gi],
                                     a.g[1 - gi], a.acc, a.rate_active, ctx->stream);
            gi = 1 - gi;
        }
        return ce;
    };
    auto segment_graph = [&](uint32_t m, int g0) -> cudaGraphExec_t {
        auto key = std::make_pair(m, g0);
        auto it = a.seg_graphs.find(key);
        if (it != a.seg_graphs.end()) return it->second;
        cudaGraphExec_t exec = nullptr;
        cudaError_t ce = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (ce == cudaSuccess) ce = enqueue_segment(m, g0);
        cudaGraph_t graph = nullptr;
        cudaError_t ee = cudaStreamEndCapture(ctx->stream, &graph);
        if (ce == cudaSuccess && ee == cudaSuccess) ee = cudaGraphInstantiate(&exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ce != cudaSuccess || ee != cudaSuccess) {
            cudaGetLastError();
            return nullptr; // the segment runs as direct launches
        }
        a.seg_graphs[key] = exec;
        return exec;
    };
    for (int64_t j = (int64_t)a.n_ckpt - 1; j >= 0; j--) {
        const uint32_t s0 = (uint32_t)j * K;
        const uint32_t m = (a.n_steps - s0) < K ? (a.n_steps - s0) : K;
        // Replay the segment from its checkpoint, keeping T_s and k_s.
        CK(cudaMemcpyAsync(a.agents_tmp, a.ckpt_agents + (size_t)j * 4 * a.n_pad, 4 * a.n_pad * sizeof(float),
                           cudaMemcpyDeviceToDevice, ctx->stream), "restoring agents");
        if (a.with_ids)
            CK(cudaMemcpyAsync(a.ids_tmp, a.ckpt_ids + (size_t)j * a.n_pad, a.n_pad * sizeof(uint32_t),
                               cudaMemcpyDeviceToDevice, ctx->stream), "restoring ids");
        CK(cudaMemcpyAsync(a.seg_trail, a.ckpt_trail + (size_t)j * cells, cells * sizeof(float),
                           cudaMemcpyDeviceToDevice, ctx->stream), "restoring trail");
        CK(cudaMemsetAsync(a.seg_counts, 0, (size_t)m * cells * sizeof(uint32_t), ctx->stream), "clearing counts");
        cudaGraphExec_t exec = segment_graph(m, cg);
        if (exec)
            CK(cudaGraphLaunch(exec, ctx->stream), "launching a backward segment");
        else
            CK(enqueue_segment(m, cg), "replaying a segment and its backward steps");
        ctx->launches += (uint64_t)m * agent_pass_kernels(a.dev, a.n, false) + (m - 1) + m;
        if (m & 1) cg = 1 - cg;
    }
    double acc[4];
    CK(cudaMemcpyAsync(acc, a.acc, 4 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "reading gradients");
    if (d_trail0)
        CK(cudaMemcpyAsync(d_trail0, a.g[cg], cells * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream),
           "reading dL/dT0");
    CK(cudaStreamSynchronize(ctx->stream), "backward");
    grads->d_decay_factor = acc[0];
    grads->d_diffusion_rate = acc[1];
    grads->d_deposition_amount = acc[2];
    grads->reserved = 0.0;
    return SLIME_OK;
}

} // extern "C"
