// harness.cpp - C entry points around the C++ translation of the reference's
// compute shader (test infrastructure: the parity tests pin the oracle
// against it).  The translation (oracle/_ref/compute_wgsl.inc) is generated
// from the reference's src/compute.wgsl by oracle/wgsl/translate.py and
// compiled with this file by oracle/build_oracle.py into
// oracle/_ref/libwgslref.so; none of it is shipped or used by the library.
//
// The display shader (src/display.wgsl) is translated the same way into
// oracle/_ref/display_wgsl.inc.  Each entry point binds the shader's buffers
// and uniform and runs one of its entry points over the whole grid,
// invocation after invocation:
//   wref_sample   sample_trail_map at given positions;
//   wref_agents   `main` once per agent (invocation id (i, 0, 0), i.e. the
//                 intended one-invocation-per-agent mapping), sensing the
//                 trail either in place or Jacobi-style (from a snapshot);
//   wref_decay    `decay_trail` over every cell (an elementwise pass: in
//                 place is race-free);
//   wref_diffuse  `diffuse_trail` over every cell, Jacobi-style (reads from
//                 `in`, writes `out`), the race-free reading of the in-place
//                 pass;
//   wref_agents_dispatch
//                 `main` over the reference's own dispatch grid
//                 (src/main.rs:1174-1178: wx x wy workgroups of 64,
//                 invocation id (gx, gy, 0)), agents and trail both read
//                 as the pass found them, writes going to the live arrays;
//   wref_colorize display.wgsl's `main` once per pixel of a tex_width x
//                 tex_height image (the LUT as 768 u32, the reference's
//                 lut_data);
//   wref_sense    the three sensor samples `main` takes (compute.wgsl:74-95,
//                 restated here in the prelude's WGSL operations because
//                 `main` keeps them in locals), to tell a flipped turn
//                 decision from any other difference.
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../../include/slime.h"
#include "prelude.h"

namespace ref {
using namespace wgsl;
#include "../_ref/compute_wgsl.inc"
} // namespace ref

namespace ref_display {
using namespace wgsl;
#include "../_ref/display_wgsl.inc"
} // namespace ref_display

namespace {

void bind_uniform(const SlimeParams* p) {
    ref::sim_size.width = p->width;
    ref::sim_size.height = p->height;
    ref::sim_size.decay_factor = wgsl::f32(p->decay_factor);
    ref::sim_size.agent_jitter = wgsl::f32(p->agent_jitter);
    ref::sim_size.agent_speed_min = wgsl::f32(p->agent_speed_min);
    ref::sim_size.agent_speed_max = wgsl::f32(p->agent_speed_max);
    ref::sim_size.agent_turn_speed = wgsl::f32(p->agent_turn_speed);
    ref::sim_size.agent_sensor_angle = wgsl::f32(p->agent_sensor_angle);
    ref::sim_size.agent_sensor_distance = wgsl::f32(p->agent_sensor_distance);
    ref::sim_size.diffusion_rate = wgsl::f32(p->diffusion_rate);
    ref::sim_size.pheromone_deposition_amount = wgsl::f32(p->pheromone_deposition_amount);
}

void bind_trail(wgsl::f32* data, const wgsl::f32* src, uint64_t cells) {
    ref::trail_map.data = data;
    ref::trail_map.src = src;
    ref::trail_map.length = (uint32_t)cells;
}

} // namespace

extern "C" {

void wref_sample(const float* trail, uint32_t W, uint32_t H, const float* px, const float* py, uint64_t n,
                 float* out) {
    SlimeParams p;
    memset(&p, 0, sizeof p);
    p.width = W;
    p.height = H;
    bind_uniform(&p);
    std::vector<wgsl::f32> t((size_t)W * H);
    for (size_t i = 0; i < t.size(); i++) t[i] = wgsl::f32(trail[i]);
    bind_trail(t.data(), nullptr, t.size());
    for (uint64_t i = 0; i < n; i++) out[i] = ref::sample_trail_map(ref::vec2f{wgsl::f32(px[i]), wgsl::f32(py[i])}).v;
}

void wref_agents(const SlimeParams* p, float* agents, uint64_t n, float* trail, int jacobi) {
    bind_uniform(p);
    const size_t cells = (size_t)p->width * p->height;
    std::vector<wgsl::f32> t(cells), snap;
    for (size_t i = 0; i < cells; i++) t[i] = wgsl::f32(trail[i]);
    if (jacobi) snap = t;
    bind_trail(t.data(), jacobi ? snap.data() : nullptr, cells);
    std::vector<ref::vec4f> a(n);
    for (uint64_t i = 0; i < n; i++)
        a[i] = ref::vec4f{wgsl::f32(agents[4 * i]), wgsl::f32(agents[4 * i + 1]), wgsl::f32(agents[4 * i + 2]),
                          wgsl::f32(agents[4 * i + 3])};
    ref::agents.data = a.data();
    ref::agents.src = nullptr;
    ref::agents.length = (uint32_t)n;
    for (uint64_t i = 0; i < n; i++) ref::wgsl_main(ref::vec3u{(uint32_t)i, 0u, 0u});
    for (uint64_t i = 0; i < n; i++) {
        agents[4 * i] = a[i].x.v;
        agents[4 * i + 1] = a[i].y.v;
        agents[4 * i + 2] = a[i].z.v;
        agents[4 * i + 3] = a[i].w.v;
    }
    for (size_t i = 0; i < cells; i++) trail[i] = t[i].v;
}

void wref_agents_dispatch(const SlimeParams* p, float* agents, uint64_t n, float* trail) {
    bind_uniform(p);
    const size_t cells = (size_t)p->width * p->height;
    std::vector<wgsl::f32> t(cells);
    for (size_t i = 0; i < cells; i++) t[i] = wgsl::f32(trail[i]);
    const std::vector<wgsl::f32> snap = t;
    bind_trail(t.data(), snap.data(), cells);
    std::vector<ref::vec4f> a(n);
    for (uint64_t i = 0; i < n; i++)
        a[i] = ref::vec4f{wgsl::f32(agents[4 * i]), wgsl::f32(agents[4 * i + 1]), wgsl::f32(agents[4 * i + 2]),
                          wgsl::f32(agents[4 * i + 3])};
    const std::vector<ref::vec4f> a0 = a;
    ref::agents.data = a.data();
    ref::agents.src = a0.data();
    ref::agents.length = (uint32_t)n;
    /* src/main.rs:1174-1178 */
    const uint32_t workgroup_size = 64u;
    const uint32_t total = (uint32_t)((n + workgroup_size - 1) / workgroup_size);
    const uint32_t wx = total < 65535u ? total : 65535u;
    const uint32_t wy = wx ? (total + wx - 1) / wx : 0u;
    for (uint32_t gy = 0; gy < wy; gy++)
        for (uint32_t gx = 0; gx < wx * workgroup_size; gx++) ref::wgsl_main(ref::vec3u{gx, gy, 0u});
    for (uint64_t i = 0; i < n; i++) {
        agents[4 * i] = a[i].x.v;
        agents[4 * i + 1] = a[i].y.v;
        agents[4 * i + 2] = a[i].z.v;
        agents[4 * i + 3] = a[i].w.v;
    }
    for (size_t i = 0; i < cells; i++) trail[i] = t[i].v;
}

void wref_decay(const SlimeParams* p, float* trail) {
    bind_uniform(p);
    const size_t cells = (size_t)p->width * p->height;
    std::vector<wgsl::f32> t(cells);
    for (size_t i = 0; i < cells; i++) t[i] = wgsl::f32(trail[i]);
    bind_trail(t.data(), nullptr, cells);
    for (uint32_t y = 0; y < p->height; y++)
        for (uint32_t x = 0; x < p->width; x++) ref::decay_trail(ref::vec3u{x, y, 0u});
    for (size_t i = 0; i < cells; i++) trail[i] = t[i].v;
}

void wref_diffuse(const SlimeParams* p, const float* in, float* out) {
    bind_uniform(p);
    const size_t cells = (size_t)p->width * p->height;
    std::vector<wgsl::f32> src(cells), dst(cells);
    for (size_t i = 0; i < cells; i++) src[i] = wgsl::f32(in[i]);
    bind_trail(dst.data(), src.data(), cells);
    for (uint32_t y = 0; y < p->height; y++)
        for (uint32_t x = 0; x < p->width; x++) ref::diffuse_trail(ref::vec3u{x, y, 0u});
    for (size_t i = 0; i < cells; i++) out[i] = dst[i].v;
}

void wref_colorize(uint32_t W, uint32_t H, const float* trail, const uint8_t* lut768, uint32_t tw, uint32_t th,
                   uint8_t* rgba) {
    ref_display::sim_size = ref_display::SimSizeUniform{};
    ref_display::sim_size.width = W;
    ref_display::sim_size.height = H;
    const size_t cells = (size_t)W * H;
    std::vector<wgsl::f32> t(cells);
    for (size_t i = 0; i < cells; i++) t[i] = wgsl::f32(trail[i]);
    ref_display::trail_map.data = t.data();
    ref_display::trail_map.src = nullptr;
    ref_display::trail_map.length = (uint32_t)cells;
    std::vector<uint32_t> lut(lut768, lut768 + 768); /* src/main.rs:329-336: each byte as a u32 */
    ref_display::lut_data.data = lut.data();
    ref_display::lut_data.src = nullptr;
    ref_display::lut_data.length = 768;
    ref_display::display_tex.data = rgba;
    ref_display::display_tex.width = tw;
    ref_display::display_tex.height = th;
    for (uint32_t y = 0; y < th; y++)
        for (uint32_t x = 0; x < tw; x++) ref_display::wgsl_main(ref_display::vec3u{x, y, 0u});
}

void wref_sense(const SlimeParams* p, const float* agents, uint64_t n, const float* trail, float* out) {
    using wgsl::f32;
    bind_uniform(p);
    const size_t cells = (size_t)p->width * p->height;
    std::vector<f32> t(cells);
    for (size_t i = 0; i < cells; i++) t[i] = f32(trail[i]);
    bind_trail(t.data(), nullptr, cells);
    const f32 a = ref::sim_size.agent_sensor_angle, d = ref::sim_size.agent_sensor_distance;
    for (uint64_t i = 0; i < n; i++) {
        const f32 x(agents[4 * i]), y(agents[4 * i + 1]), angle(agents[4 * i + 2]);
        const f32 al = angle - a, ar = angle + a;
        out[3 * i] = ref::sample_trail_map(ref::vec2f{x + d * wgsl::cos(al), y + d * wgsl::sin(al)}).v;
        out[3 * i + 1] = ref::sample_trail_map(ref::vec2f{x + d * wgsl::cos(ar), y + d * wgsl::sin(ar)}).v;
        out[3 * i + 2] = ref::sample_trail_map(ref::vec2f{x + d * wgsl::cos(angle), y + d * wgsl::sin(angle)}).v;
    }
}

} // extern "C"
