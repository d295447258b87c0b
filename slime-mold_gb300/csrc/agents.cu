// agents.cu - the agent pass (sense, turn, move, deposit) and agent-buffer
// utilities.
//
// Restates src/compute.wgsl:57-145 with the builtins of slime_math.h.  Layout
// and traffic:
//   * agent state is SoA (x[], y[], angle[], speed[], optional id[]); a thread
//     owns four consecutive slots and moves each field with one 16-byte
//     streaming load and store (__ldcs/__stcs: evict-first, so the streamed
//     32 B/agent do not push the sensed trail out of L2);
//   * the three bilinear sensor samples read the pre-step trail through the
//     read-only path (12 loads/agent, L2-resident at 4096^2);
//   * the deposit is one 32-bit atomic increment of the cell's count; the trail
//     pass folds the counts into the trail deterministically.
#include "kernels.h"

namespace slime {
namespace {

// sample_trail_map, compute.wgsl:7-29 (x1 >= W written as x0 >= W - 1).
__device__ __forceinline__ float sample_trail(const float* __restrict__ trail, int W, int H, float px, float py) {
    int x0 = slm_f2i(floorf(px));
    int y0 = slm_f2i(floorf(py));
    if (x0 < 0 || x0 >= W - 1 || y0 < 0 || y0 >= H - 1) return 0.0f;
    float dx = slm_sub(px, slm_i2f(x0));
    float dy = slm_sub(py, slm_i2f(y0));
    const float* r0 = trail + (y0 * W + x0);
    float v00 = __ldg(r0);
    float v10 = __ldg(r0 + 1);
    float v01 = __ldg(r0 + W);
    float v11 = __ldg(r0 + W + 1);
    float v0 = slm_mix(v00, v10, dx);
    float v1 = slm_mix(v01, v11, dx);
    return slm_mix(v0, v1, dy);
}

// One agent, compute.wgsl:65-144.  Returns the deposit cell or -1.
__device__ __forceinline__ int agent_step(const DevParams& p, float& x, float& y, float& angle, float& speed,
                                          int32_t index, const float* __restrict__ trail) {
    speed = slm_clamp(speed, p.speed_min, p.speed_max);

    float sl, cl, sr, cr, sc, cc;
    slm_sincos(slm_sub(angle, p.sensor_angle), &sl, &cl);
    slm_sincos(slm_add(angle, p.sensor_angle), &sr, &cr);
    slm_sincos(angle, &sc, &cc);
    float left = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cl)),
                              slm_add(y, slm_mul(p.sensor_dist, sl)));
    float right = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cr)),
                               slm_add(y, slm_mul(p.sensor_dist, sr)));
    float center = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cc)),
                                slm_add(y, slm_mul(p.sensor_dist, sc)));

    if (center > left && center > right) {
        // straight
    } else if (left > right) {
        float diff = slm_sub(slm_sub(angle, SLM_WGSL_TAU), angle);
        angle = slm_add(angle, slm_mul(slm_min(p.turn, slm_abs(diff)), slm_sign(diff)));
    } else if (right > left) {
        float diff = slm_sub(slm_add(angle, SLM_WGSL_TAU), angle);
        angle = slm_add(angle, slm_mul(slm_min(p.turn, slm_abs(diff)), slm_sign(diff)));
    }

    float rv = slm_jitter_hash(index, x, y);
    angle = slm_add(angle, slm_mul(slm_sub(slm_mul(rv, 2.0f), 1.0f), p.jitter));
    angle = slm_fmod(angle, SLM_WGSL_TWO_PI);
    if (angle < 0.0f) angle = slm_add(angle, SLM_WGSL_TWO_PI);

    float move = slm_mul(speed, p.time_step);
    float sm, cm;
    slm_sincos(angle, &sm, &cm);
    x = slm_add(x, slm_mul(move, cm));
    y = slm_add(y, slm_mul(move, sm));
    x = slm_fmod(x, p.Wf);
    if (x < 0.0f) x = slm_add(x, p.Wf);
    y = slm_fmod(y, p.Hf);
    if (y < 0.0f) y = slm_add(y, p.Hf);

    int dx = slm_f2i(x);
    int dy = slm_f2i(y);
    if (dx >= 0 && dx < p.W && dy >= 0 && dy < p.H) return dy * p.W + dx;
    return -1;
}

template <bool kIds>
__global__ void __launch_bounds__(256) agents_kernel(const __grid_constant__ DevParams p, float4* __restrict__ X,
                                                     float4* __restrict__ Y, float4* __restrict__ TH,
                                                     float4* __restrict__ V, const uint4* __restrict__ ids,
                                                     const float* __restrict__ trail, uint32_t* __restrict__ counts,
                                                     uint32_t n_groups, uint64_t n) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n_groups) return;
    float4 x = __ldcs(X + g);
    float4 y = __ldcs(Y + g);
    float4 th = __ldcs(TH + g);
    float4 v = __ldcs(V + g);
    uint4 id;
    if (kIds) {
        id = __ldcs(ids + g);
    } else {
        uint32_t b = 4u * g;
        id = make_uint4(b, b + 1, b + 2, b + 3);
    }
    uint64_t base = 4ull * g;
    int c0 = -1, c1 = -1, c2 = -1, c3 = -1;
    if (base + 0 < n) c0 = agent_step(p, x.x, y.x, th.x, v.x, (int32_t)id.x, trail);
    if (base + 1 < n) c1 = agent_step(p, x.y, y.y, th.y, v.y, (int32_t)id.y, trail);
    if (base + 2 < n) c2 = agent_step(p, x.z, y.z, th.z, v.z, (int32_t)id.z, trail);
    if (base + 3 < n) c3 = agent_step(p, x.w, y.w, th.w, v.w, (int32_t)id.w, trail);
    if (c0 >= 0) atomicAdd(counts + c0, 1u);
    if (c1 >= 0) atomicAdd(counts + c1, 1u);
    if (c2 >= 0) atomicAdd(counts + c2, 1u);
    if (c3 >= 0) atomicAdd(counts + c3, 1u);
    __stcs(X + g, x);
    __stcs(Y + g, y);
    __stcs(TH + g, th);
    __stcs(V + g, v);
}

__global__ void aos_to_soa_kernel(const float4* __restrict__ aos, float* __restrict__ x, float* __restrict__ y,
                                  float* __restrict__ th, float* __restrict__ v, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 a = aos[i];
    x[i] = a.x;
    y[i] = a.y;
    th[i] = a.z;
    v[i] = a.w;
}

__global__ void soa_to_aos_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                  const float* __restrict__ th, const float* __restrict__ v,
                                  const uint32_t* __restrict__ ids, float4* __restrict__ aos, uint64_t n) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t dst = ids ? ids[i] : i;
    aos[dst] = make_float4(x[i], y[i], th[i], v[i]);
}

// Seeded initial state (replaces src/main.rs:273-280): fields drawn with
// slm_uniform01(seed, id, field), scaled exactly as the reference scales
// rand::random::<f32>().
__global__ void seed_kernel(float* __restrict__ x, float* __restrict__ y, float* __restrict__ th,
                            float* __restrict__ v, uint64_t n, uint64_t seed, float Wf, float Hf, float hmin,
                            float hmax, float smin, float smax) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float px = slm_mul(slm_uniform01(seed, i, 0), Wf);
    float py = slm_mul(slm_uniform01(seed, i, 1), Hf);
    if (px >= Wf) px = __uint_as_float(__float_as_uint(Wf) - 1u);
    if (py >= Hf) py = __uint_as_float(__float_as_uint(Hf) - 1u);
    x[i] = px;
    y[i] = py;
    th[i] = slm_add(hmin, slm_mul(slm_uniform01(seed, i, 2), slm_sub(hmax, hmin)));
    v[i] = slm_add(smin, slm_mul(slm_uniform01(seed, i, 3), slm_sub(smax, smin)));
}

// reassign_agent_speeds (src/main.rs:101-145) on the device.
__global__ void reassign_speeds_kernel(float* __restrict__ v, const uint32_t* __restrict__ ids, uint64_t n,
                                       uint64_t seed, float smin, float smax) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint64_t id = ids ? ids[i] : i;
    v[i] = slm_add(smin, slm_mul(slm_uniform01(seed, id, 3), slm_sub(smax, smin)));
}

// Resize (src/main.rs:987-993): x *= new_w / old_w, y *= new_h / old_h.
__global__ void scale_positions_kernel(float* __restrict__ x, float* __restrict__ y, uint64_t n, float sx,
                                       float sy) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    x[i] = slm_mul(x[i], sx);
    y[i] = slm_mul(y[i], sy);
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

} // namespace

cudaError_t launch_agents(const DevParams& p, const AgentsSoA& a, const float* trail, uint32_t* counts,
                          cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    uint32_t n_groups = (uint32_t)((a.n + 3) / 4);
    unsigned blocks = blocks_for(n_groups, 256);
    if (a.ids)
        agents_kernel<true><<<blocks, 256, 0, s>>>(p, (float4*)a.x, (float4*)a.y, (float4*)a.th, (float4*)a.v,
                                                   (const uint4*)a.ids, trail, counts, n_groups, a.n);
    else
        agents_kernel<false><<<blocks, 256, 0, s>>>(p, (float4*)a.x, (float4*)a.y, (float4*)a.th, (float4*)a.v,
                                                    nullptr, trail, counts, n_groups, a.n);
    return cudaGetLastError();
}

cudaError_t launch_aos_to_soa(const float4* aos, const AgentsSoA& a, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    aos_to_soa_kernel<<<blocks_for(a.n, 256), 256, 0, s>>>(aos, a.x, a.y, a.th, a.v, a.n);
    return cudaGetLastError();
}

cudaError_t launch_soa_to_aos(const AgentsSoA& a, float4* aos, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    soa_to_aos_kernel<<<blocks_for(a.n, 256), 256, 0, s>>>(a.x, a.y, a.th, a.v, a.ids, aos, a.n);
    return cudaGetLastError();
}

cudaError_t launch_seed_agents(const AgentsSoA& a, uint64_t seed, float Wf, float Hf, float hmin, float hmax,
                               float smin, float smax, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    seed_kernel<<<blocks_for(a.n, 256), 256, 0, s>>>(a.x, a.y, a.th, a.v, a.n, seed, Wf, Hf, hmin, hmax, smin,
                                                     smax);
    return cudaGetLastError();
}

cudaError_t launch_reassign_speeds(const AgentsSoA& a, uint64_t seed, float smin, float smax, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    reassign_speeds_kernel<<<blocks_for(a.n, 256), 256, 0, s>>>(a.v, a.ids, a.n, seed, smin, smax);
    return cudaGetLastError();
}

cudaError_t launch_scale_positions(const AgentsSoA& a, float sx, float sy, cudaStream_t s) {
    if (a.n == 0) return cudaSuccess;
    scale_positions_kernel<<<blocks_for(a.n, 256), 256, 0, s>>>(a.x, a.y, a.n, sx, sy);
    return cudaGetLastError();
}

} // namespace slime
