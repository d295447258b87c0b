// ctx.h - the simulation context behind the opaque slime_ctx handle
// (internal to the library).
#pragma once

#include <map>
#include <string>
#include <utility>

#include "kernels.h"

struct slime_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t W = 0, H = 0;

    slime::AgentsSoA agents;
    void* agent_block = nullptr;     // x | y | angle | speed, n_pad floats each
    uint32_t* ids_storage = nullptr; // slot -> agent id, allocated at the first reorder
    bool reordered = false;
    // the last reorder put the agents the reference's dispatch updates first
    // (identity ids have them first too)
    bool reorder_partitioned = false;
    uint64_t last_reorder_step = ~0ull;
    uint64_t reorders_done = 0;
    slime::ReorderScratch reorder;

    float* trail[2] = {nullptr, nullptr};
    cudaTextureObject_t trail_tex[2] = {0, 0}; // gather textures over trail[] (0 = none)
    slime::TrailMaps tmaps;                    // tensor maps over trail[], counts[], marks[] (tmaps.ok)
    uint32_t* counts[2] = {nullptr, nullptr};
    int cur = 0;
    bool last_counts_valid = false;
    // Deposit marks: one byte per cell, used instead of the counts by steps
    // in which every deposit saturates the fold (see use_marks in capi.cu).
    uint8_t* marks[2] = {nullptr, nullptr};
    bool counts_dirty[2] = {false, false}; // buffer may hold non-zero entries
    bool marks_dirty[2] = {false, false};
    bool trail_clean = true; // every value of trail[cur] is finite and >= 0 (or +inf)
    bool last_marks = false; // the last step recorded marks, not counts

    SlimeParams params{};
    slime::DevParams dev{};
    SlimeOptions opt{};
    int tile = 0;
    int tuned_tile = -1;
    int agent_shape = 0; // index into the agent-kernel shape table
    int tuned_shape = -1;

    // Persisting-L2 window over the trail being sensed (0 = off).
    size_t l2_persist_bytes = 0; // carve-out granted to this context
    size_t l2_max_window = 0;    // cudaDevAttrMaxAccessPolicyWindowSize
    bool l2_tuned_off = false;   // the autotuner measured the steps faster without it
    // which passes carry the window when a carve-out is granted (bit 0 the
    // agent pass, bit 1 the trail pass; the autotuner may keep only one)
    unsigned l2_window_passes = 3;

    std::map<std::pair<uint32_t, int>, cudaGraphExec_t> graphs; // (steps, start parity) -> graph

    uint64_t steps_done = 0;
    uint64_t launches = 0;

    void* staging = nullptr; // AoS agent staging for uploads/downloads
    size_t staging_bytes = 0;
    void* aux = nullptr; // display buffer
    size_t aux_bytes = 0;
    // slime_colorize_async: the LUT on the device (uploaded when it changes)
    // and the image the copy stream reads
    uint8_t* display_lut = nullptr;
    uint8_t display_lut_host[768] = {};
    bool display_lut_valid = false;
    uint8_t* display_image = nullptr;
    size_t display_image_bytes = 0;

    // Asynchronous display feed: device snapshot + copy stream.
    cudaStream_t copy_stream = nullptr;
    // two trail snapshots used in turn, so a snapshot never waits for the
    // host copy of the one before it, only for the copy two calls back
    float* display_snap[2] = {nullptr, nullptr};
    int display_next = 0;
    cudaEvent_t snap_copied[2] = {nullptr, nullptr}; // last host copy out of display_snap[b] finished
    bool snap_copy_pending[2] = {false, false};
    size_t display_cells = 0;
    cudaEvent_t snap_ready = nullptr;  // snapshot written (main stream)
    cudaEvent_t copy_done = nullptr;   // latest host copy finished (copy stream)
    bool copy_pending = false;

    // Adjoint recording (adjoint.cu).
    struct Adjoint {
        bool recorded = false;
        uint32_t n_steps = 0, ckpt_every = 0, n_ckpt = 0;
        slime::DevParams dev{};          // parameters the recorded steps ran with
        int tile = 0;
        int agent_shape = 0;
        uint32_t rate_active = 0;         // 0 < diffusion_rate < 1
        uint64_t n = 0, n_pad = 0;
        bool with_ids = false;
        float* ckpt_agents = nullptr;     // n_ckpt * 4 * n_pad floats
        uint32_t* ckpt_ids = nullptr;     // n_ckpt * n_pad (when reordered)
        float* ckpt_trail = nullptr;      // n_ckpt * cells
        float* seg_trail = nullptr;       // ckpt_every * cells: T_s of the segment being replayed
        uint32_t* seg_counts = nullptr;   // ckpt_every * cells: k_s
        float* g[2] = {nullptr, nullptr}; // dL/dT ping-pong
        double* acc = nullptr;            // d_decay, d_rate, d_dep
        float* agents_tmp = nullptr;      // replay copy of the agents (4 * n_pad)
        uint32_t* ids_tmp = nullptr;
        // captured segments (replay and backward steps) by (steps, g buffer)
        std::map<std::pair<uint32_t, int>, cudaGraphExec_t> seg_graphs;
    } adj;

    std::string err;
};

namespace slime {

int set_error(std::string& err, int code, const char* fmt, ...);
int cuda_error(std::string& err, cudaError_t e, const char* what);
void invalidate_graphs(slime_ctx* ctx);
bool marks_allowed(const slime_ctx* ctx);
bool keeps_trail_clean(const DevParams& d);
bool use_marks(const slime_ctx* ctx);
int prepare_deposits(slime_ctx* ctx, bool marks);
cudaError_t enqueue_step(slime_ctx* ctx, bool marks, bool chained);
void after_steps(slime_ctx* ctx, bool marks, uint32_t m);
uint64_t kernels_per_step(const slime_ctx* ctx, bool marks);
// Reorder first if the reference's dispatch is on and the slots do not hold
// the agents it updates first.
int ensure_dispatch_order(slime_ctx* ctx);
int run_steps(slime_ctx* ctx, uint32_t n);
int prepare_steps(slime_ctx* ctx, uint32_t n);
void free_adjoint(slime_ctx* ctx);
void setup_l2(slime_ctx* ctx);
constexpr unsigned kWindowAgents = 1, kWindowTrail = 2;
bool trail_window(const slime_ctx* ctx, const float* t, cudaAccessPolicyWindow* w, unsigned pass);

} // namespace slime
