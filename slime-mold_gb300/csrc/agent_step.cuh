// agent_step.cuh - one agent of the shader's "main" entry point
// (src/compute.wgsl:57-145), shared by the plain and the ensemble kernels.
#pragma once

#include "common.cuh"

namespace slime {

// Trail readers for agent_step: sample_trail_map, compute.wgsl:7-29 (x1 >= W
// written as x0 >= W - 1), on a padded global buffer or on a texture over it.
// Each sample is split in two: fetch() issues the footprint's loads and
// returns them unconsumed (a Tap), value() interpolates; operator() is both.
//
// TrailPtr: the trail buffers carry W + 2 zero floats past their last cell,
// so the four taps at index 0 are always in bounds: an out-of-grid sample
// loads from cell 0 and is discarded, which keeps the sampler free of
// branches.  In range, f32(x0) == floor(px) exactly.
//
// TrailTex: one four-texel gather returns the 2x2 footprint (raw texels, no
// filtering), so the interpolation is the shader's arithmetic on the same four
// values.  The texture is the trail buffer itself (pitch-linear binary32,
// point filtering, clamped, unnormalised coordinates); gathering at
// (x0 + 1, y0 + 1) selects texels x0..x0+1, y0..y0+1, returned as
// w = (x0, y0), z = (x0+1, y0), x = (x0, y0+1), y = (x0+1, y0+1).  An
// out-of-grid sample gathers wherever its coordinates point (the clamped
// addressing keeps every coordinate, infinite or NaN included, on the
// texture) and is discarded.  The in-grid test needs no integer x0: with
// fx = floor(px), 0 <= i32(fx) < W - 1 holds exactly when
// !(fx < 0) && !(fx >= W - 1) for every fx, NaN included (i32(NaN) = 0 is
// in the grid, and NaN fails both compares), on trails at least 2 wide and
// high, the only ones that have a texture.
struct TrailPtr {
    const float* __restrict__ t;
    struct Tap {
        float v00, v10, v01, v11, dx, dy;
        bool ok;
    };
    __device__ __forceinline__ Tap fetch(const DevParams& p, float px, float py) const {
        Tap k;
        const int W = p.W, H = p.H;
        float fx = floorf(px), fy = floorf(py);
        int x0 = slm_f2i(fx);
        int y0 = slm_f2i(fy);
        // x0 < 0 || x0 + 1 >= W  (and the same for y) as one unsigned compare each
        k.ok = (unsigned)x0 < (unsigned)(W - 1) && (unsigned)y0 < (unsigned)(H - 1);
        k.dx = slm_sub(px, fx);
        k.dy = slm_sub(py, fy);
        const float* r0 = t + (k.ok ? y0 * W + x0 : 0);
        k.v00 = __ldg(r0);
        k.v10 = __ldg(r0 + 1);
        k.v01 = __ldg(r0 + W);
        k.v11 = __ldg(r0 + W + 1);
        return k;
    }
    __device__ __forceinline__ static float value(const Tap& k) {
        float v0 = slm_mix(k.v00, k.v10, k.dx);
        float v1 = slm_mix(k.v01, k.v11, k.dx);
        return k.ok ? slm_mix(v0, v1, k.dy) : 0.0f;
    }
    __device__ __forceinline__ float operator()(const DevParams& p, float px, float py) const {
        return value(fetch(p, px, py));
    }
};
struct TrailTex {
    cudaTextureObject_t t;
    struct Tap {
        float4 g;
        float dx, dy;
        bool ok;
    };
    __device__ __forceinline__ Tap fetch(const DevParams& p, float px, float py) const {
        Tap k;
        float fx = floorf(px), fy = floorf(py);
        k.ok = !(fx < 0.0f) && !(fx >= p.Wm1f) && !(fy < 0.0f) && !(fy >= p.Hm1f);
        k.dx = slm_sub(px, fx);
        k.dy = slm_sub(py, fy);
        // in range, f32(x0 + 1) == floor(px) + 1 exactly (|x0| < 2^24); a NaN
        // position passes the test (i32(NaN) = 0) and gathers at a NaN
        // coordinate, whose texels do not matter: its weights are NaN
        k.g = tex2Dgather<float4>(t, fx + 1.0f, fy + 1.0f, 0);
        return k;
    }
    __device__ __forceinline__ static float value(const Tap& k) {
        float v0 = slm_mix(k.g.w, k.g.z, k.dx);
        float v1 = slm_mix(k.g.x, k.g.y, k.dx);
        return k.ok ? slm_mix(v0, v1, k.dy) : 0.0f;
    }
    __device__ __forceinline__ float operator()(const DevParams& p, float px, float py) const {
        return value(fetch(p, px, py));
    }
};

// The three sensor footprints of an agent (compute.wgsl:75-95), fetched.
template <class Trail>
struct Senses {
    typename Trail::Tap left, right, center;
};

// The sensor directions: by default cos/sin of angle -/+ a and of angle, as
// the shader evaluates them (compute.wgsl:75-90); with SLIME_SENSOR_ROTATED
// the centre direction rotated by -/+ a.  The mode is uniform over a launch.
template <class Trail>
__device__ __forceinline__ Senses<Trail> agent_sense(const DevParams& p, float x, float y, float angle,
                                                     const Trail& trail) {
    float sl, cl, sr, cr, sc, cc;
    if (p.sensor_mode == SLIME_SENSOR_ROTATED)
        slm_sensor_dirs(angle, p.sensor_sin, p.sensor_cos, &cl, &sl, &cc, &sc, &cr, &sr);
    else
        slm_sensor_dirs_shader(angle, p.sensor_angle, &cl, &sl, &cc, &sc, &cr, &sr);
    Senses<Trail> s;
    s.left = trail.fetch(p, slm_add(x, slm_mul(p.sensor_dist, cl)), slm_add(y, slm_mul(p.sensor_dist, sl)));
    s.right = trail.fetch(p, slm_add(x, slm_mul(p.sensor_dist, cr)), slm_add(y, slm_mul(p.sensor_dist, sr)));
    s.center = trail.fetch(p, slm_add(x, slm_mul(p.sensor_dist, cc)), slm_add(y, slm_mul(p.sensor_dist, sc)));
    return s;
}

// compute.wgsl:72 and 98-122: the speed clamp, the turn from the sensor
// samples, the jitter from the hash `rv` (slm_jitter_hash of the agent's
// index and pre-move x, y, :117) and the heading's wrap.
__device__ __forceinline__ void agent_turn(const DevParams& p, float& angle, float& speed, float rv, float left,
                                           float right, float center) {
    speed = slm_clamp(speed, p.speed_min, p.speed_max);

    // compute.wgsl:98-112: keep straight, or turn toward target = angle -/+ TAU
    bool turn_left = !(center > left && center > right) && (left > right);
    bool turn_right = !(center > left && center > right) && !(left > right) && (right > left);
    // angle - TAU or angle + TAU: the same sum with the signed constant chosen
    float target = slm_add(angle, turn_left ? -SLM_WGSL_TAU : SLM_WGSL_TAU);
    float diff = slm_sub(target, angle);
    float turned = slm_add(angle, slm_mul(slm_min(p.turn, slm_abs(diff)), slm_sign(diff)));
    angle = (turn_left || turn_right) ? turned : angle;

    // (rv * 2.0 - 1.0) as one fused multiply-add: the product is exact (a
    // power-of-two scaling), so rounding once after the sum gives the bits of
    // the shader's product-then-difference
    angle = slm_add(angle, slm_mul(slm_fma(rv, 2.0f, -1.0f), p.jitter));
    angle = slm_wrap(angle, SLM_WGSL_TWO_PI);
}

// compute.wgsl:125-141: the move along (cm, sm) = (cos, sin) of the new
// heading, the position's wrap and the deposit cell (or -1).
__device__ __forceinline__ int agent_move(const DevParams& p, float& x, float& y, float speed, float sm, float cm) {
    float move = slm_mul(speed, p.time_step);
    x = slm_add(x, slm_mul(move, cm));
    y = slm_add(y, slm_mul(move, sm));
    x = slm_wrap(x, p.Wf);
    y = slm_wrap(y, p.Hf);

    int dx = slm_f2i(x);
    int dy = slm_f2i(y);
    if ((unsigned)dx < (unsigned)p.W && (unsigned)dy < (unsigned)p.H) return dy * p.W + dx;
    return -1;
}

// The rest of the agent (compute.wgsl:72 and 98-144) once its sensor samples
// and its jitter hash are known.  Returns the deposit cell or -1.
__device__ __forceinline__ int agent_finish(const DevParams& p, float& x, float& y, float& angle, float& speed,
                                            float rv, float left, float right, float center) {
    agent_turn(p, angle, speed, rv, left, right, center);
    float sm, cm;
    slm_sincos(angle, &sm, &cm);
    return agent_move(p, x, y, speed, sm, cm);
}

// One agent, compute.wgsl:65-144.  Returns the deposit cell or -1.
template <class Trail>
__device__ __forceinline__ int agent_step(const DevParams& p, float& x, float& y, float& angle, float& speed,
                                          int32_t index, const Trail& trail) {
    const Senses<Trail> s = agent_sense(p, x, y, angle, trail);
    // the hash needs no sample: it is worked out while the footprints load
    const float rv = slm_jitter_hash(index, x, y);
    return agent_finish(p, x, y, angle, speed, rv, Trail::value(s.left), Trail::value(s.right),
                        Trail::value(s.center));
}

__device__ __forceinline__ int agent_step(const DevParams& p, float& x, float& y, float& angle, float& speed,
                                          int32_t index, const float* __restrict__ trail) {
    return agent_step(p, x, y, angle, speed, index, TrailPtr{trail});
}

// Two agents (a and b) at once: agent_step's arithmetic for each, with the
// sin/cos polynomials that the two evaluate on different arguments (centre
// directions, jitter hashes, moves) paired into packed fused multiply-adds,
// as are each agent's two side directions.  Bit for bit agent_step twice.
// The two agents' sensor directions (centre, left, right), (cos, sin) each.
struct SensorDirs2 {
    float cca, sca, ccb, scb, cla, sla, cra, sra, clb, slb, crb, srb;
};

// The sensor directions of two agents in either sensor mode, with every
// sin/cos taking its own range test: the general case, out of line.
static __device__ __noinline__ SensorDirs2 sensor_dirs2_general(const DevParams& p, float tha, float thb) {
    SensorDirs2 o;
    slm_sincos2(tha, thb, &o.sca, &o.cca, &o.scb, &o.ccb);
    if (p.sensor_mode == SLIME_SENSOR_ROTATED) {
        slm_rotate_dirs(o.cca, o.sca, p.sensor_sin, p.sensor_cos, &o.cla, &o.sla, &o.cra, &o.sra);
        slm_rotate_dirs(o.ccb, o.scb, p.sensor_sin, p.sensor_cos, &o.clb, &o.slb, &o.crb, &o.srb);
    } else {
        slm_side_dirs_shader(tha, p.sensor_angle, &o.cla, &o.sla, &o.cra, &o.sra);
        slm_side_dirs_shader(thb, p.sensor_angle, &o.clb, &o.slb, &o.crb, &o.srb);
    }
    return o;
}

template <class Trail>
__device__ __forceinline__ void agent_step2(const DevParams& p, float& xa, float& ya, float& tha, float& va,
                                            int32_t ia, float& xb, float& yb, float& thb, float& vb, int32_t ib,
                                            const Trail& trail, int& cell_a, int& cell_b) {
    float sca, cca, scb, ccb;
    float cla, sla, cra, sra, clb, slb, crb, srb;
    if (slm_abs(tha) < 4000.0f && slm_abs(thb) < 4000.0f && slm_abs(p.sensor_angle) < 64.0f) {
        // every sensor angle, angle -/+ a included, is below 4096 in magnitude
        // (all the shader produces after its first step): the packed
        // Cody-Waite forms the range tests would pick, without the tests
        slm_sincos2_cw(tha, thb, &sca, &cca, &scb, &ccb);
        if (p.sensor_mode == SLIME_SENSOR_ROTATED) {
            slm_rotate_dirs(cca, sca, p.sensor_sin, p.sensor_cos, &cla, &sla, &cra, &sra);
            slm_rotate_dirs(ccb, scb, p.sensor_sin, p.sensor_cos, &clb, &slb, &crb, &srb);
        } else {
            const float a = p.sensor_angle;
            slm_sincos2_cw(slm_sub(tha, a), slm_add(tha, a), &sla, &cla, &sra, &cra);
            slm_sincos2_cw(slm_sub(thb, a), slm_add(thb, a), &slb, &clb, &srb, &crb);
        }
    } else {
        const SensorDirs2 o = sensor_dirs2_general(p, tha, thb);
        cca = o.cca, sca = o.sca, ccb = o.ccb, scb = o.scb;
        cla = o.cla, sla = o.sla, cra = o.cra, sra = o.sra;
        clb = o.clb, slb = o.slb, crb = o.crb, srb = o.srb;
    }
    const float d = p.sensor_dist;
    const typename Trail::Tap la = trail.fetch(p, slm_add(xa, slm_mul(d, cla)), slm_add(ya, slm_mul(d, sla)));
    const typename Trail::Tap ra = trail.fetch(p, slm_add(xa, slm_mul(d, cra)), slm_add(ya, slm_mul(d, sra)));
    const typename Trail::Tap ca = trail.fetch(p, slm_add(xa, slm_mul(d, cca)), slm_add(ya, slm_mul(d, sca)));
    const typename Trail::Tap lb = trail.fetch(p, slm_add(xb, slm_mul(d, clb)), slm_add(yb, slm_mul(d, slb)));
    const typename Trail::Tap rb = trail.fetch(p, slm_add(xb, slm_mul(d, crb)), slm_add(yb, slm_mul(d, srb)));
    const typename Trail::Tap cb = trail.fetch(p, slm_add(xb, slm_mul(d, ccb)), slm_add(yb, slm_mul(d, scb)));
    // the hashes need no sample: worked out while the footprints load
    float rva, rvb;
    slm_jitter_hash2(ia, xa, ya, ib, xb, yb, &rva, &rvb);
    agent_turn(p, tha, va, rva, Trail::value(la), Trail::value(ra), Trail::value(ca));
    agent_turn(p, thb, vb, rvb, Trail::value(lb), Trail::value(rb), Trail::value(cb));
    // the new headings are wrapped into [0, 2pi] (or NaN, whose sin and cos
    // are NaN on every path), so the packed Cody-Waite form needs no range test
    float sma, cma, smb, cmb;
    slm_sincos2_cw(tha, thb, &sma, &cma, &smb, &cmb);
    cell_a = agent_move(p, xa, ya, va, sma, cma);
    cell_b = agent_move(p, xb, yb, vb, smb, cmb);
}

} // namespace slime
