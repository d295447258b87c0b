// common.cuh - device parameter block and helpers shared by the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>

#include "../../include/slime.h"
#include "../../include/slime_math.h"

namespace slime {

constexpr int kMaxR = SLIME_MAX_BLUR_RADIUS;

// Everything a step needs, derived once on the host from SlimeParams with the
// same binary32 operations the shader performs per invocation
// (compute.wgsl:159 decay_factor*0.001, :173 clamp(rate, 0, 1)).  Passed by
// value as a __grid_constant__ kernel argument, i.e. it lives in the constant
// bank like the reference's uniform buffer.
struct DevParams {
    int32_t W, H;
    float Wf, Hf;
    float Wm1f, Hm1f; // W - 1 and H - 1 (exact: sides are <= 2^24)
    float speed_min, speed_max;
    float turn;
    float sensor_angle, sensor_dist;
    float sensor_sin, sensor_cos; // slm_sincos(sensor_angle)
    float jitter;
    float time_step;
    float dep;
    float decay;    // decay_factor (multiplicative mode)
    float decay_k;  // decay_factor * 0.001 (subtractive mode)
    float rate;     // clamp(diffusion_rate, 0, 1)
    uint32_t decay_mode;
    uint32_t blur_mode;
    uint32_t dispatch_mode; // SLIME_DISPATCH_*
    uint32_t sensor_mode;   // SLIME_SENSOR_*
    int32_t R;      // Gaussian taps per side
    float w[2 * kMaxR + 1];
    float w2sum_m1; // (sum of w)^2 - 1 in binary64, rounded: B(u) - u = sum w w (u_n - u_c) + this * u_c
};

// Programmatic dependent launch: a kernel launched with `pdl` set (below)
// may start while the kernel before it in the stream finishes.  It runs what
// does not depend on that kernel, then pdl_wait() returns once that kernel has
// completed and its writes are visible (at once for a launch without such a
// predecessor).  pdl_trigger() lets the next such kernel start launching once
// every block of this grid has triggered or exited.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Launch `k` with an optional persisting-L2 access window attached to this
// launch and, with `pdl`, as a programmatic dependent of the kernel before it
// in the stream (both captured into graphs as kernel-node attributes).
template <typename... KArgs, typename... Args>
cudaError_t launch_kp(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                      const cudaAccessPolicyWindow* win, bool pdl, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    unsigned n = 0;
    if (win) {
        attr[n].id = cudaLaunchAttributeAccessPolicyWindow;
        attr[n].val.accessPolicyWindow = *win;
        n++;
    }
    if (pdl) {
        attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[n].val.programmaticStreamSerializationAllowed = 1;
        n++;
    }
    cfg.attrs = n ? attr : nullptr;
    cfg.numAttrs = n;
    return cudaLaunchKernelEx(&cfg, k, std::forward<Args>(args)...);
}
template <typename... KArgs, typename... Args>
cudaError_t launch_k(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                     const cudaAccessPolicyWindow* win, Args&&... args) {
    return launch_kp(k, grid, block, smem, s, win, false, std::forward<Args>(args)...);
}

// Device allocations of the library go through these two functions.  When
// the environment variable SLIME_DEVICE_MEMORY_CAP holds a byte count, an
// allocation that would take the library's live total above it fails with
// cudaErrorMemoryAllocation (reported as SLIME_ERR_OUT_OF_MEMORY), which lets
// the out-of-memory paths be tested without exhausting a real GPU.
cudaError_t dev_alloc(void** p, size_t bytes);
void dev_free(void* p);

// Translate SlimeParams into DevParams; returns false (with a message) on
// values the kernels cannot honour.
bool make_dev_params(const SlimeParams& p, uint32_t W, uint32_t H, DevParams* out, const char** why);

// --------------------------------------------------------------- device code
// Deposit fold: t <- clamp(t + dep, 0, 1), k times; stops once an iteration
// leaves the bits of t unchanged (every later iteration would too).  The
// first two iterations are straight-line selects (most cells receive 0, 1 or
// 2 deposits per step); only cells with k >= 3 whose value still moved after
// two iterations enter the loop.
__device__ __forceinline__ float fold_deposits(float t, uint32_t k, float dep) {
    const float t1 = slm_clamp(slm_add(t, dep), 0.0f, 1.0f);
    const float t2 = slm_clamp(slm_add(t1, dep), 0.0f, 1.0f);
    float r = k == 0 ? t : (k == 1 ? t1 : t2);
    if (k >= 3 && __float_as_uint(t2) != __float_as_uint(t1)) {
        float u = t2;
        for (uint32_t i = 2; i < k; i++) {
            float nu = slm_clamp(slm_add(u, dep), 0.0f, 1.0f);
            if (__float_as_uint(nu) == __float_as_uint(u)) break;
            u = nu;
        }
        r = u;
    }
    return r;
}

__device__ __forceinline__ float apply_decay(const DevParams& p, float v) {
    return p.decay_mode == SLIME_DECAY_MULTIPLY ? slm_mul(v, p.decay) : slm_max(slm_sub(v, p.decay_k), 0.0f);
}
// The same with the decay mode fixed at compile time (kMode: a
// SLIME_DECAY_* value, or -1 to read it from p).
template <int kMode>
__device__ __forceinline__ float apply_decay_m(const DevParams& p, float v) {
    if (kMode < 0) return apply_decay(p, v);
    return kMode == (int)SLIME_DECAY_MULTIPLY ? slm_mul(v, p.decay) : slm_max(slm_sub(v, p.decay_k), 0.0f);
}

// Wrap g into [0, n) for g in [-n*k, n*(k+1)); the loops run at most once for
// the halos the kernels use unless the grid is smaller than the blur radius.
__device__ __forceinline__ int wrap_coord(int g, int n) {
    while (g < 0) g += n;
    while (g >= n) g -= n;
    return g;
}

} // namespace slime
