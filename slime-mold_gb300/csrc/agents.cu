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
#include "agent_step.cuh"
#include "kernels.h"

namespace slime {
namespace {

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// Vector access to APT consecutive slots (float, float2, float4).
template <int APT>
struct Lanes;
template <>
struct Lanes<1> {
    __device__ static void load(const float* p, float* v) { v[0] = __ldcs(p); }
    __device__ static void store(float* p, const float* v) { __stcs(p, v[0]); }
    __device__ static void load_ids(const uint32_t* p, uint32_t* v) { v[0] = __ldcs(p); }
};
template <>
struct Lanes<2> {
    __device__ static void load(const float* p, float* v) {
        float2 t = __ldcs(reinterpret_cast<const float2*>(p));
        v[0] = t.x;
        v[1] = t.y;
    }
    __device__ static void store(float* p, const float* v) { __stcs(reinterpret_cast<float2*>(p), make_float2(v[0], v[1])); }
    __device__ static void load_ids(const uint32_t* p, uint32_t* v) {
        uint2 t = __ldcs(reinterpret_cast<const uint2*>(p));
        v[0] = t.x;
        v[1] = t.y;
    }
};
template <>
struct Lanes<4> {
    __device__ static void load(const float* p, float* v) {
        float4 t = __ldcs(reinterpret_cast<const float4*>(p));
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
    }
    __device__ static void store(float* p, const float* v) {
        __stcs(reinterpret_cast<float4*>(p), make_float4(v[0], v[1], v[2], v[3]));
    }
    __device__ static void load_ids(const uint32_t* p, uint32_t* v) {
        uint4 t = __ldcs(reinterpret_cast<const uint4*>(p));
        v[0] = t.x;
        v[1] = t.y;
        v[2] = t.z;
        v[3] = t.w;
    }
};

// The step's deposit at `cell`: one more on the cell's 32-bit count, or,
// when every deposit of the step saturates the fold, the cell's byte mark set
// to 1 by an atomic OR on the 32-bit word holding it (measured faster at
// 4096^2 than byte stores, which also race where agents meet).
__device__ __forceinline__ void deposit(uint32_t* __restrict__ counts, uint8_t* __restrict__ marks, int cell) {
    if (marks)
        atomicOr(reinterpret_cast<unsigned*>(marks + (cell & ~3)), 1u << (8 * (cell & 3)));
    else
        atomicAdd(counts + cell, 1u);
}

// A full group of APT agents: in pairs (agent_step2) when APT is even.
template <int APT, class Trail>
__device__ __forceinline__ void step_group(const DevParams& p, float* x, float* y, float* th, float* v,
                                           const uint32_t* id, const Trail& trail, int* cell) {
    if (APT % 2 == 0) {
#pragma unroll
        for (int j = 0; j < APT; j += 2)
            agent_step2(p, x[j], y[j], th[j], v[j], (int32_t)id[j], x[j + 1], y[j + 1], th[j + 1], v[j + 1],
                        (int32_t)id[j + 1], trail, cell[j], cell[j + 1]);
    } else {
#pragma unroll
        for (int j = 0; j < APT; j++) cell[j] = agent_step(p, x[j], y[j], th[j], v[j], (int32_t)id[j], trail);
    }
}

// The last group of a pass when fewer than APT of its agents are live, out
// of line: it runs for one thread of a launch at most, and inlined it would
// add a second copy of the agent code to the loop (instruction-cache space).
template <int APT>
struct GroupState {
    float x[APT], y[APT], th[APT], v[APT];
    uint32_t id[APT];
    int cell[APT];
};
template <int APT, class Trail>
__device__ __noinline__ GroupState<APT> step_partial_group(const DevParams& p, GroupState<APT> s, uint32_t live,
                                                           const Trail trail) {
#pragma unroll
    for (int j = 0; j < APT; j++)
        s.cell[j] = (uint32_t)j < live ? agent_step(p, s.x[j], s.y[j], s.th[j], s.v[j], (int32_t)s.id[j], trail) : -1;
    return s;
}

// A thread moves APT consecutive slots with one vector load/store per field.
// MINB > 0 asks the compiler to fit MINB blocks per SM (caps registers).
// Trail is the reader of the sensed trail (TrailPtr or TrailTex).
template <int APT, int BS, int MINB, bool kIds, class Trail>
__global__ void __launch_bounds__(BS, MINB) agents_kernel(const __grid_constant__ DevParams p, float* __restrict__ X,
                                                    float* __restrict__ Y, float* __restrict__ TH,
                                                    float* __restrict__ V, const uint32_t* __restrict__ ids,
                                                    const Trail trail, uint32_t* __restrict__ counts,
                                                    uint8_t* __restrict__ marks, uint32_t n_groups, uint64_t n) {
    const uint32_t g = blockIdx.x * BS + threadIdx.x;
    if (g >= n_groups) return;
    const uint64_t base = (uint64_t)g * APT;
    float x[APT], y[APT], th[APT], v[APT];
    uint32_t id[APT];
    Lanes<APT>::load(X + base, x);
    Lanes<APT>::load(Y + base, y);
    Lanes<APT>::load(TH + base, th);
    Lanes<APT>::load(V + base, v);
    if (kIds) {
        Lanes<APT>::load_ids(ids + base, id);
    } else {
#pragma unroll
        for (int j = 0; j < APT; j++) id[j] = (uint32_t)(base + j);
    }
    // the state is not written by the trail pass this launch may follow; the
    // trail it senses and the deposit record are
    pdl_wait();
    pdl_trigger();
    int cell[APT];
    if (base + APT <= n) {
        // full group: no per-agent branch, so the agents' work can interleave
        step_group<APT>(p, x, y, th, v, id, trail, cell);
    } else {
#pragma unroll
        for (int j = 0; j < APT; j++)
            cell[j] = (base + j < n) ? agent_step(p, x[j], y[j], th[j], v[j], (int32_t)id[j], trail) : -1;
    }
#pragma unroll
    for (int j = 0; j < APT; j++)
        if (cell[j] >= 0) deposit(counts, marks, cell[j]);
    Lanes<APT>::store(X + base, x);
    Lanes<APT>::store(Y + base, y);
    Lanes<APT>::store(TH + base, th);
    Lanes<APT>::store(V + base, v);
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

// Persistent variant: a grid sized to the resident capacity walks the groups
// with a stride, loading the next group's state while the current one is
// computed, so the stream of agent state does not wait on DRAM latency.
template <int APT, int BS, int MINB, bool kIds, class Trail>
__global__ void __launch_bounds__(BS, MINB) agents_persistent_kernel(
    const __grid_constant__ DevParams p, float* __restrict__ X, float* __restrict__ Y, float* __restrict__ TH,
    float* __restrict__ V, const uint32_t* __restrict__ ids, const Trail trail, uint32_t* __restrict__ counts,
    uint8_t* __restrict__ marks, uint32_t n_groups, uint64_t n) {
    const uint32_t stride = gridDim.x * BS;
    uint32_t g = blockIdx.x * BS + threadIdx.x;
    if (g >= n_groups) return;
    float x[APT], y[APT], th[APT], v[APT];
    uint32_t id[APT];
    uint64_t base = (uint64_t)g * APT;
    Lanes<APT>::load(X + base, x);
    Lanes<APT>::load(Y + base, y);
    Lanes<APT>::load(TH + base, th);
    Lanes<APT>::load(V + base, v);
    if (kIds) Lanes<APT>::load_ids(ids + base, id);
    // the first group's state is not written by the trail pass this launch may
    // follow; the trail it senses and the deposit record are
    pdl_wait();
    pdl_trigger();
    while (true) {
        const uint32_t gn = g + stride;
        const bool more = gn < n_groups;
        const uint64_t bn = (uint64_t)gn * APT;
        float xn[APT], yn[APT], thn[APT], vn[APT];
        uint32_t idn[APT];
        if (more) {
            Lanes<APT>::load(X + bn, xn);
            Lanes<APT>::load(Y + bn, yn);
            Lanes<APT>::load(TH + bn, thn);
            Lanes<APT>::load(V + bn, vn);
            if (kIds) Lanes<APT>::load_ids(ids + bn, idn);
        }
        if (!kIds) {
#pragma unroll
            for (int j = 0; j < APT; j++) id[j] = (uint32_t)(base + j);
        }
        int cell[APT];
        if (base + APT <= n) {
            step_group<APT>(p, x, y, th, v, id, trail, cell);
        } else {
            GroupState<APT> s;
#pragma unroll
            for (int j = 0; j < APT; j++) {
                s.x[j] = x[j];
                s.y[j] = y[j];
                s.th[j] = th[j];
                s.v[j] = v[j];
                s.id[j] = id[j];
            }
            s = step_partial_group<APT>(p, s, (uint32_t)(n - base), trail);
#pragma unroll
            for (int j = 0; j < APT; j++) {
                x[j] = s.x[j];
                y[j] = s.y[j];
                th[j] = s.th[j];
                v[j] = s.v[j];
                cell[j] = s.cell[j];
            }
        }
#pragma unroll
        for (int j = 0; j < APT; j++)
            if (cell[j] >= 0) deposit(counts, marks, cell[j]);
        Lanes<APT>::store(X + base, x);
        Lanes<APT>::store(Y + base, y);
        Lanes<APT>::store(TH + base, th);
        Lanes<APT>::store(V + base, v);
        if (!more) break;
        g = gn;
        base = bn;
#pragma unroll
        for (int j = 0; j < APT; j++) {
            x[j] = xn[j];
            y[j] = yn[j];
            th[j] = thn[j];
            v[j] = vn[j];
            if (kIds) id[j] = idn[j];
        }
    }
}

// The reference's own dispatch (SLIME_DISPATCH_REFERENCE) visits agent `id`
// slm_dispatch_visits(n, id) times (compute.wgsl:60); the agents it visits
// at all are ids 0 .. reference_dispatch_updated(n) - 1, kept in the first
// slots.  An agent visited m > 1 times moves once (each visit reads the state
// the pass found) and deposits m times: the agent kernel deposits once, this
// kernel adds the other m - 1 at the cell of the agent's new position
// (compute.wgsl:136-141), which is the cell the agent kernel used.
__global__ void extra_deposits_kernel(const float* __restrict__ X, const float* __restrict__ Y,
                                      const uint32_t* __restrict__ ids, uint64_t n_updated, int W, int H,
                                      uint32_t wy, uint32_t span, uint32_t* __restrict__ counts) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_updated) return;
    const uint32_t m = slm_dispatch_visits_in(ids ? ids[i] : (uint32_t)i, wy, span);
    if (m <= 1) return;
    const int dx = slm_f2i(X[i]);
    const int dy = slm_f2i(Y[i]);
    if ((unsigned)dx < (unsigned)W && (unsigned)dy < (unsigned)H) atomicAdd(counts + (size_t)dy * W + dx, m - 1);
}

template <int APT, int BS, int MINB, class Trail>
cudaError_t launch_agents_persistent(const DevParams& p, const AgentsSoA& a, const Trail& trail, uint32_t* counts,
                                     uint8_t* marks, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl) {
    // Resident blocks of each instantiation, found once per process (a
    // function-local static is initialised exactly once, also when contexts
    // on several threads launch at the same time).
    struct Occupancy {
        int sms = 1, per_sm[2] = {1, 1};
    };
    static const Occupancy occ = [] {
        Occupancy o;
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&o.sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o.per_sm[0],
                                                      agents_persistent_kernel<APT, BS, MINB, false, Trail>, BS, 0);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o.per_sm[1],
                                                      agents_persistent_kernel<APT, BS, MINB, true, Trail>, BS, 0);
        if (o.sms < 1) o.sms = 1;
        for (int& b : o.per_sm)
            if (b < 1) b = 1;
        return o;
    }();
    const int k = a.ids ? 1 : 0;
    uint32_t n_groups = (uint32_t)((a.n + APT - 1) / APT);
    unsigned want = (unsigned)(occ.per_sm[k] * occ.sms);
    unsigned need = blocks_for(n_groups, BS);
    dim3 grid(want < need ? want : need);
    if (a.ids)
        return launch_kp(agents_persistent_kernel<APT, BS, MINB, true, Trail>, grid, dim3(BS), 0, s, win, pdl, p, a.x, a.y,
                        a.th, a.v, (const uint32_t*)a.ids, trail, counts, marks, n_groups, a.n);
    return launch_kp(agents_persistent_kernel<APT, BS, MINB, false, Trail>, grid, dim3(BS), 0, s, win, pdl, p, a.x, a.y,
                    a.th, a.v, (const uint32_t*)nullptr, trail, counts, marks, n_groups, a.n);
}

template <int APT, int BS, int MINB, class Trail>
cudaError_t launch_agents_variant(const DevParams& p, const AgentsSoA& a, const Trail& trail, uint32_t* counts,
                                  uint8_t* marks, cudaStream_t s, const cudaAccessPolicyWindow* win, bool pdl) {
    uint32_t n_groups = (uint32_t)((a.n + APT - 1) / APT);
    dim3 grid(blocks_for(n_groups, BS));
    if (a.ids)
        return launch_kp(agents_kernel<APT, BS, MINB, true, Trail>, grid, dim3(BS), 0, s, win, pdl, p, a.x, a.y, a.th, a.v,
                        (const uint32_t*)a.ids, trail, counts, marks, n_groups, a.n);
    return launch_kp(agents_kernel<APT, BS, MINB, false, Trail>, grid, dim3(BS), 0, s, win, pdl, p, a.x, a.y, a.th, a.v,
                    (const uint32_t*)nullptr, trail, counts, marks, n_groups, a.n);
}

} // namespace

// Agent-kernel shapes: (agents per thread, threads per block, min blocks/SM).
// Entries 9..11 are the persistent, prefetching variant; 12..15 sample the
// trail through its texture (12 regular, 13-15 persistent; 15 capped at four
// blocks per SM, i.e. 64 registers) and run on the pointer path when the
// trail has no texture.
const AgentShape kAgentShapes[] = {{4, 256, 0}, {2, 256, 0}, {1, 256, 0}, {4, 128, 0}, {1, 128, 0},
                                   {2, 256, 5}, {2, 256, 6}, {4, 256, 4}, {1, 256, 8}, {2, 256, 0},
                                   {1, 256, 0}, {2, 128, 0}, {2, 256, 0}, {2, 256, 0}, {2, 128, 0},
                                   {2, 256, 4}};

int agent_shape_count() { return (int)(sizeof(kAgentShapes) / sizeof(kAgentShapes[0])); }
AgentShape agent_shape(int i) { return kAgentShapes[(i >= 0 && i < agent_shape_count()) ? i : 0]; }
bool agent_shape_uses_texture(int i) { return i >= 12 && i <= 15; }

uint64_t reference_dispatch_updated(uint64_t n) {
    if (n == 0) return 0;
    uint32_t wy = 0, span = 0;
    slm_dispatch_geometry(n, &wy, &span);
    const uint64_t reach = (uint64_t)(wy - 1) * 65535u + span; // gx + 65535 gy < reach
    return reach < n ? reach : n;
}

int agent_pass_kernels(const DevParams& p, uint64_t n, bool marks) {
    if (n == 0) return 0;
    if (p.dispatch_mode != SLIME_DISPATCH_REFERENCE || marks) return 1;
    uint32_t wy = 0, span = 0;
    slm_dispatch_geometry(n, &wy, &span);
    return wy > 1 ? 2 : 1; // some agent is visited twice only with two or more rows
}

cudaError_t launch_agents(const DevParams& p, const AgentsSoA& a, const float* trail, uint32_t* counts,
                          cudaStream_t s, int shape, const cudaAccessPolicyWindow* win, cudaTextureObject_t tex,
                          uint8_t* marks, bool pdl) {
    if (a.n == 0) return cudaSuccess;
    if (p.dispatch_mode == SLIME_DISPATCH_REFERENCE) {
        AgentsSoA updated = a;
        updated.n = reference_dispatch_updated(a.n);
        DevParams each = p;
        each.dispatch_mode = SLIME_DISPATCH_EACH_AGENT;
        cudaError_t e = launch_agents(each, updated, trail, counts, s, shape, win, tex, marks, pdl);
        if (e != cudaSuccess || agent_pass_kernels(p, a.n, marks) == 1) return e;
        uint32_t wy = 0, span = 0;
        slm_dispatch_geometry(a.n, &wy, &span);
        extra_deposits_kernel<<<blocks_for(updated.n, 256), 256, 0, s>>>(a.x, a.y, a.ids, updated.n, p.W, p.H, wy,
                                                                          span, counts);
        return cudaGetLastError();
    }
    const TrailPtr tp{trail};
    if (agent_shape_uses_texture(shape) && tex) {
        const TrailTex tt{tex};
        switch (shape) {
        case 12: return launch_agents_variant<2, 256, 0>(p, a, tt, counts, marks, s, win, pdl);
        case 13: return launch_agents_persistent<2, 256, 0>(p, a, tt, counts, marks, s, win, pdl);
        case 15: return launch_agents_persistent<2, 256, 4>(p, a, tt, counts, marks, s, win, pdl);
        default: return launch_agents_persistent<2, 128, 0>(p, a, tt, counts, marks, s, win, pdl);
        }
    }
    switch (shape) {
    case 1:
    case 12: return launch_agents_variant<2, 256, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 2: return launch_agents_variant<1, 256, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 3: return launch_agents_variant<4, 128, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 4: return launch_agents_variant<1, 128, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 5: return launch_agents_variant<2, 256, 5>(p, a, tp, counts, marks, s, win, pdl);
    case 6: return launch_agents_variant<2, 256, 6>(p, a, tp, counts, marks, s, win, pdl);
    case 7: return launch_agents_variant<4, 256, 4>(p, a, tp, counts, marks, s, win, pdl);
    case 8: return launch_agents_variant<1, 256, 8>(p, a, tp, counts, marks, s, win, pdl);
    case 9:
    case 13: return launch_agents_persistent<2, 256, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 10: return launch_agents_persistent<1, 256, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 11:
    case 14: return launch_agents_persistent<2, 128, 0>(p, a, tp, counts, marks, s, win, pdl);
    case 15: return launch_agents_persistent<2, 256, 4>(p, a, tp, counts, marks, s, win, pdl);
    default: return launch_agents_variant<4, 256, 0>(p, a, tp, counts, marks, s, win, pdl);
    }
}

// A texture over trail buffer `t` (W x H binary32, row pitch 4W bytes) for
// the gather sampler, or 0 when this device cannot describe the buffer as a
// pitch-linear texture (row pitch or base not aligned to its texture pitch
// alignment, or sides beyond its linear-texture limits).
cudaTextureObject_t make_trail_texture(const float* t, uint32_t W, uint32_t H) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    const size_t pitch = (size_t)W * sizeof(float);
    const size_t align = prop.texturePitchAlignment ? prop.texturePitchAlignment : 32;
    if (W < 2 || H < 2 || pitch % align != 0 || (uintptr_t)t % align != 0) return 0;
    if ((int64_t)W > prop.maxTexture2DLinear[0] || (int64_t)H > prop.maxTexture2DLinear[1] ||
        (int64_t)pitch > prop.maxTexture2DLinear[2])
        return 0;
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypePitch2D;
    rd.res.pitch2D.devPtr = const_cast<float*>(t);
    rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
    rd.res.pitch2D.width = W;
    rd.res.pitch2D.height = H;
    rd.res.pitch2D.pitchInBytes = pitch;
    cudaTextureDesc td = {};
    td.addressMode[0] = cudaAddressModeClamp;
    td.addressMode[1] = cudaAddressModeClamp;
    td.filterMode = cudaFilterModePoint;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t tex = 0;
    if (cudaCreateTextureObject(&tex, &rd, &td, nullptr) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return tex;
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
