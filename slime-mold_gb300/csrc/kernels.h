// kernels.h - launch wrappers of the CUDA kernels (host side, internal).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"

namespace slime {

// Agent state in HBM: structure of arrays, each array padded to a multiple of
// kAgentPad agents and 16-byte aligned so that one thread moves four agents
// with one float4 load/store per field.
constexpr uint64_t kAgentPad = 128;

struct AgentsSoA {
    float* x = nullptr;
    float* y = nullptr;
    float* th = nullptr;
    float* v = nullptr;
    uint32_t* ids = nullptr; // original agent id per slot; nullptr = identity order
    uint64_t n = 0;          // live agents
    uint64_t n_pad = 0;      // allocated slots
};

// ---- agents.cu
// Launch shapes of the agent kernel: agents per thread and threads per block.
struct AgentShape {
    int apt, threads, min_blocks;
};
int agent_shape_count();
AgentShape agent_shape(int index);
bool agent_shape_uses_texture(int index);
// One agent pass (compute.wgsl:57-145): reads trail, adds deposit counts.
// `tex` is a texture over `trail` (make_trail_texture) for the shapes that
// sample through it; 0 runs those shapes on the pointer path.  With `marks`
// the deposits set per-cell byte marks instead of counting (valid only when
// every deposit saturates the fold: deposition >= 1 on a trail >= 0).
// With p.dispatch_mode == SLIME_DISPATCH_REFERENCE the agents the reference's
// dispatch updates must fill the first reference_dispatch_updated(a.n)
// slots (identity ids, or a reorder given that count): the pass updates those
// and, when counting, adds the extra deposits of multiply visited agents.
// With `pdl` the launch is a programmatic dependent of the kernel before it
// in the stream, which must be the trail pass (or no kernel of this library).
cudaError_t launch_agents(const DevParams& p, const AgentsSoA& a, const float* trail, uint32_t* counts,
                          cudaStream_t s, int shape = 0, const cudaAccessPolicyWindow* win = nullptr,
                          cudaTextureObject_t tex = 0, uint8_t* marks = nullptr, bool pdl = false);
// Kernels one launch_agents call enqueues.
int agent_pass_kernels(const DevParams& p, uint64_t n, bool marks);
// How many agents (ids 0 .. this - 1) the reference's dispatch updates.
uint64_t reference_dispatch_updated(uint64_t n);
cudaTextureObject_t make_trail_texture(const float* trail, uint32_t W, uint32_t H);
// AoS staging (x, y, angle, speed per agent, id order) <-> SoA slots.
cudaError_t launch_aos_to_soa(const float4* aos, const AgentsSoA& a, cudaStream_t s);
cudaError_t launch_soa_to_aos(const AgentsSoA& a, float4* aos, cudaStream_t s);
cudaError_t launch_seed_agents(const AgentsSoA& a, uint64_t seed, float Wf, float Hf, float hmin, float hmax,
                               float smin, float smax, cudaStream_t s);
cudaError_t launch_reassign_speeds(const AgentsSoA& a, uint64_t seed, float smin, float smax, cudaStream_t s);
cudaError_t launch_scale_positions(const AgentsSoA& a, float sx, float sy, cudaStream_t s);

// ---- trail.cu
// Tile shapes of the fused deposit-fold + decay + diffuse kernel.
struct TrailTile {
    int tw, th;
};
int trail_tile_count();
TrailTile trail_tile(int index);
int trail_tile_default();
// Whether tile `index` can run this parameter set / grid (the streaming
// tiles need W % 4 == 0 and a blur radius of 1 or 2).
bool trail_tile_supported(const DevParams& p, int tile);
// Tensor maps (for the tensor-copy tile) over a context's two trails and
// their deposit records, one set per blur radius (the box is the window).
struct TrailMaps {
    CUtensorMap trail[2], counts[2], marks[2];
    CUtensorMap trail_r2[2], counts_r2[2], marks_r2[2];
    bool ok = false;
};
// The trail-table index of the tensor-copy tile.
constexpr int kTrailTileTma = 10;

// Fused trail pass: out = Diffuse(Decay(Fold(in, counts_in))); zeroes
// counts_zero (the other step's count buffer, may be null) over the same cells.
// With `pdl` a streaming tile launches as a programmatic dependent of the
// kernel before it in the stream (the agent pass); the shared-memory tiles
// always launch in order.
// The tensor-copy tile needs `maps` over the context's buffers and the index
// `cur` of the buffers `in`/`counts_in` are.
cudaError_t launch_trail(const DevParams& p, int tile, const float* in, const uint32_t* counts_in, float* out,
                         uint32_t* counts_zero, cudaStream_t s, const cudaAccessPolicyWindow* win = nullptr,
                         bool pdl = false, const TrailMaps* maps = nullptr, int cur = 0);
// Whether tile `index` is a streaming tile that runs here (the only ones that
// read deposit marks).
bool trail_tile_streams(const DevParams& p, int tile);
// The same pass folding per-cell byte marks (0/1) instead of counts; zeroes
// marks_zero.  Streaming tiles only (cudaErrorInvalidValue otherwise).
cudaError_t launch_trail_marks(const DevParams& p, int tile, const float* in, const uint8_t* marks_in, float* out,
                               uint8_t* marks_zero, cudaStream_t s, const cudaAccessPolicyWindow* win = nullptr,
                               bool pdl = false, const TrailMaps* maps = nullptr, int cur = 0);

// ---- trail_tma.cu
// The tensor-copy tile: W % 16 == 0 and a blur radius of 1 or 2.
bool trail_tma_supported(const DevParams& p);
bool make_trail_maps(TrailMaps* m, const float* const trail[2], const uint32_t* const counts[2],
                     const uint8_t* const marks[2], uint32_t W, uint32_t H);
cudaError_t launch_trail_tma(const DevParams& p, const TrailMaps& maps, int cur, const float* in,
                             const uint32_t* counts_in, float* out, uint32_t* counts_zero, cudaStream_t s,
                             const cudaAccessPolicyWindow* win, bool pdl);
cudaError_t launch_trail_tma_marks(const DevParams& p, const TrailMaps& maps, int cur, const float* in,
                                   const uint8_t* marks_in, float* out, uint8_t* marks_zero, cudaStream_t s,
                                   const cudaAccessPolicyWindow* win, bool pdl);
// Whether a tensor-copy tile gave up waiting for its copies since the last
// call (the flag is cleared).
bool trail_tma_take_error();
// Blocks that found their shared-memory boxes misaligned and used plain loads.
int trail_tma_misaligned_blocks();

// ---- adjoint.cu
// One backward step of the frozen-trajectory chain: from g_in = dL/dT_{s+1}
// and the step's input trail T_s and counts k_s, writes g_out = dL/dT_s and
// adds the step's parameter-gradient contributions to acc[0..2]
// (decay_factor, diffusion_rate, deposition), in binary64.
cudaError_t launch_adjoint_step(const DevParams& p, const float* trail_s, const uint32_t* counts_s,
                                const float* g_in, float* g_out, double* acc, uint32_t rate_active,
                                cudaStream_t s);

// ---- reorder.cu
// Morton reordering of agent slots by cell; permutes SoA in place through
// scratch buffers and keeps ids.
struct ReorderScratch {
    void* buf = nullptr;
    size_t bytes = 0;
};
cudaError_t launch_iota(uint32_t* ids, uint64_t n, cudaStream_t s);
// Morton order; agents with id >= `visited` go to the last slots.
cudaError_t launch_reorder(AgentsSoA& a, uint32_t W, uint32_t H, int cell_log2, ReorderScratch& scratch,
                           cudaStream_t s, uint64_t visited = ~0ull);

// ---- colorize.cu
cudaError_t launch_colorize(const float* trail, uint32_t W, uint32_t H, const uint8_t* lut, uint32_t tw,
                            uint32_t th, uint8_t* rgba, cudaStream_t s);

} // namespace slime
