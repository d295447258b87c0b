// agent_step.cuh - one agent of the shader's "main" entry point
// (src/compute.wgsl:57-145), shared by the plain and the ensemble kernels.
#pragma once

#include "common.cuh"

namespace slime {

// sample_trail_map, compute.wgsl:7-29 (x1 >= W written as x0 >= W - 1).
// The trail buffers carry W + 2 zero floats past their last cell, so the four
// taps at index 0 are always in bounds: an out-of-grid sample loads from cell
// 0 and is discarded, which keeps the sampler free of branches.
__device__ __forceinline__ float sample_trail(const float* __restrict__ trail, int W, int H, float px, float py) {
    float fx = floorf(px), fy = floorf(py);
    int x0 = slm_f2i(fx);
    int y0 = slm_f2i(fy);
    // x0 < 0 || x0 + 1 >= W  (and the same for y) as one unsigned compare each
    bool ok = (unsigned)x0 < (unsigned)(W - 1) && (unsigned)y0 < (unsigned)(H - 1);
    // in range, f32(x0) == floor(px) exactly
    float dx = slm_sub(px, fx);
    float dy = slm_sub(py, fy);
    const float* r0 = trail + (ok ? y0 * W + x0 : 0);
    float v00 = __ldg(r0);
    float v10 = __ldg(r0 + 1);
    float v01 = __ldg(r0 + W);
    float v11 = __ldg(r0 + W + 1);
    float v0 = slm_mix(v00, v10, dx);
    float v1 = slm_mix(v01, v11, dx);
    return ok ? slm_mix(v0, v1, dy) : 0.0f;
}

// One agent, compute.wgsl:65-144.  Returns the deposit cell or -1.
__device__ __forceinline__ int agent_step(const DevParams& p, float& x, float& y, float& angle, float& speed,
                                          int32_t index, const float* __restrict__ trail) {
    speed = slm_clamp(speed, p.speed_min, p.speed_max);

    float sl, cl, sr, cr, sc, cc;
    slm_sensor_dirs(angle, p.sensor_sin, p.sensor_cos, &cl, &sl, &cc, &sc, &cr, &sr);
    float left = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cl)),
                              slm_add(y, slm_mul(p.sensor_dist, sl)));
    float right = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cr)),
                               slm_add(y, slm_mul(p.sensor_dist, sr)));
    float center = sample_trail(trail, p.W, p.H, slm_add(x, slm_mul(p.sensor_dist, cc)),
                                slm_add(y, slm_mul(p.sensor_dist, sc)));

    // compute.wgsl:98-112: keep straight, or turn toward target = angle -/+ TAU
    bool turn_left = !(center > left && center > right) && (left > right);
    bool turn_right = !(center > left && center > right) && !(left > right) && (right > left);
    float target = turn_left ? slm_sub(angle, SLM_WGSL_TAU) : slm_add(angle, SLM_WGSL_TAU);
    float diff = slm_sub(target, angle);
    float turned = slm_add(angle, slm_mul(slm_min(p.turn, slm_abs(diff)), slm_sign(diff)));
    angle = (turn_left || turn_right) ? turned : angle;

    float rv = slm_jitter_hash(index, x, y);
    angle = slm_add(angle, slm_mul(slm_sub(slm_mul(rv, 2.0f), 1.0f), p.jitter));
    angle = slm_wrap(angle, SLM_WGSL_TWO_PI);

    float move = slm_mul(speed, p.time_step);
    float sm, cm;
    slm_sincos(angle, &sm, &cm);
    x = slm_add(x, slm_mul(move, cm));
    y = slm_add(y, slm_mul(move, sm));
    x = slm_wrap(x, p.Wf);
    y = slm_wrap(y, p.Hf);

    int dx = slm_f2i(x);
    int dy = slm_f2i(y);
    if ((unsigned)dx < (unsigned)p.W && (unsigned)dy < (unsigned)p.H) return dy * p.W + dx;
    return -1;
}

} // namespace slime
