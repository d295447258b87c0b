/*
 * slime.h - C ABI of the GB300 Physarum core.
 *
 * The reference (Velfi/slime-mold) runs one simulation step as three wgpu
 * compute dispatches from its event loop (src/main.rs:1163-1235):
 *   "main"          agents: sense, turn, move, deposit   (src/compute.wgsl:57-145)
 *   "decay_trail"   trail decay                          (src/compute.wgsl:148-161)
 *   "diffuse_trail" 3x3 toroidal blur                    (src/compute.wgsl:164-195)
 * built by PipelineManager (src/pipeline_manager.rs:37-54) over one bind group
 * {0: agents vec4<f32>, 1: trail f32, 2: SimSizeUniform}
 * (src/bind_group_manager.rs:101-125).  This library replaces those three
 * pipelines, their bind group and the dispatch code with one context object
 * that owns the agent and trail buffers on one GPU and advances them with two
 * CUDA kernels per step (agents; fused deposit+decay+diffuse), captured in a
 * CUDA graph.
 *
 * Conventions:
 *   - every function returns an int status (SLIME_OK = 0, negative = error)
 *     unless stated; slime_last_error() gives a message for the last failure;
 *   - host pointers belong to the caller and are only read/written during the
 *     call (the call synchronises with the context's stream before returning);
 *   - agents cross the ABI as the reference's AoS layout, 4 floats per agent
 *     (x, y, angle, speed) in agent-id order (src/main.rs:263-282); trails as
 *     width*height floats, row-major (src/main.rs:285-293);
 *   - one context is used from one host thread at a time (like the winit event
 *     loop thread); distinct contexts are independent.
 *
 * Semantics where the reference has data races (documented deviations):
 *   - sensing reads the trail as it was at the start of the step (the shader
 *     reads a buffer that other invocations are depositing into);
 *   - the k deposits that land in a cell in one step are applied as the
 *     sequential fold t <- clamp(t + deposition, 0, 1), k times (the shader's
 *     non-atomic read-modify-write at compute.wgsl:140 loses updates);
 *   - decay and diffuse read one buffer and write another (the shader blurs in
 *     place);
 *   - every agent is updated exactly once per step (the shader's index
 *     gid.x + gid.y*65535 at compute.wgsl:60 leaves agents above 4,194,240
 *     frozen and updates some low indices several times).
 */
#ifndef SLIME_H
#define SLIME_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------ status codes */
#define SLIME_OK 0
#define SLIME_ERR_INVALID_ARGUMENT (-1)
#define SLIME_ERR_OUT_OF_MEMORY (-2)
#define SLIME_ERR_CUDA (-3)
#define SLIME_ERR_STATE (-4)          /* call not valid in the current state */
#define SLIME_ERR_DEVICE_TIMEOUT (-5) /* a bounded device-side wait gave up */
#define SLIME_ERR_NO_DEVICE (-6)

/* ------------------------------------------------------------ modes */
/* Trail decay (compute.wgsl:159-160 is the subtractive form). */
#define SLIME_DECAY_REF_SUBTRACT 0u /* t = max(t - decay_factor * 0.001, 0) */
#define SLIME_DECAY_MULTIPLY 1u     /* t = t * decay_factor */
/* Trail blur (compute.wgsl:175-194 is the 3x3 box). */
#define SLIME_BLUR_REF_BOX3 0u /* 3x3 toroidal box, summed in shader order, /9 */
#define SLIME_BLUR_GAUSS 1u    /* separable Gaussian, radius blur_radius, sigma blur_sigma */
#define SLIME_MAX_BLUR_RADIUS 8
/* Which agents the agent pass updates.  The reference dispatches
 * wx x wy workgroups of 64 invocations, wx = min(ceil(n / 64), 65535),
 * wy = ceil(ceil(n / 64) / wx) (src/main.rs:1174-1178), and invocation
 * (gx, gy) updates agent gx + 65535 gy (compute.wgsl:60): for n > 4,194,240
 * agents the highest ones are never updated and some are updated by several
 * invocations. */
#define SLIME_DISPATCH_EACH_AGENT 0u /* every agent once per step (the intended reading) */
#define SLIME_DISPATCH_REFERENCE 1u  /* the reference's dispatch: an agent visited by m invocations
                                        moves once (every visit reads the state the pass found)
                                        and deposits m times; m = 0 leaves it as it is */
/* How the side sensors' directions are evaluated (compute.wgsl:75-86 takes
 * cos and sin of the binary32 angles angle - sensor_angle and
 * angle + sensor_angle). */
#define SLIME_SENSOR_SHADER 0u  /* as the shader writes it: sin/cos of the rounded angle -/+ a (three
                                   sin/cos evaluations per agent; the default) */
#define SLIME_SENSOR_ROTATED 1u /* the centre direction rotated by -/+ a (one sin/cos evaluation per
                                   agent): a few ulp from the shader's directions, enough to flip the turn
                                   decision of about 5 agents in 100,000 per step at sensor angles of
                                   0.3-2.5 rad; an opt-in fast mode, not the reference's result */

/* ------------------------------------------------------------ parameters */
/* The first 14 fields are SimSizeUniform (src/main.rs:29-46) in the same
 * order and layout (56 bytes); the rest extend it with what the shader hard
 * codes.  width/height must be 0 or equal to the context's trail size. */
typedef struct SlimeParams {
    uint32_t width;
    uint32_t height;
    float decay_factor;
    float agent_jitter;
    float agent_speed_min;
    float agent_speed_max;
    float agent_turn_speed;
    float agent_sensor_angle;
    float agent_sensor_distance;
    float diffusion_rate;
    float pheromone_deposition_amount;
    float blur_radius;
    float blur_sigma;
    uint32_t _pad;
    /* extensions */
    float time_step;     /* TIME_STEP, compute.wgsl:55 (0.016) */
    uint32_t decay_mode; /* SLIME_DECAY_* */
    uint32_t blur_mode;  /* SLIME_BLUR_* */
    uint32_t dispatch_mode; /* SLIME_DISPATCH_* (0, every agent once, is the default) */
    uint32_t sensor_mode;   /* SLIME_SENSOR_* (0, the shader's evaluation, is the default) */
    uint32_t _pad2;
} SlimeParams;

/* Settings (src/settings.rs:30-47), field for field. */
typedef struct SlimeSettings {
    uint64_t agent_count;
    float agent_jitter;
    float agent_possible_starting_headings_start;
    float agent_possible_starting_headings_end;
    float agent_speed_max;
    float agent_speed_min;
    float agent_turn_speed;
    float pheromone_decay_factor;
    float pheromone_diffusion_rate;
    float pheromone_deposition_amount;
    uint32_t window_fullscreen;
    uint32_t window_height;
    uint32_t window_width;
    float agent_sensor_angle;
    float agent_sensor_distance;
    float blur_radius;
    float blur_sigma;
} SlimeSettings;

/* Engine options (no counterpart in the reference). */
typedef struct SlimeOptions {
    uint32_t use_graphs;        /* 1: capture step chunks in CUDA graphs (default 1) */
    uint32_t graph_chunk;       /* steps per captured graph (default 50) */
    uint32_t reorder_every;     /* Morton-reorder agents every k steps, 0 = never (default 0) */
    uint32_t reorder_cell_log2; /* Morton key granularity, log2 of a square of cells (default 2) */
    uint32_t l2_persist;        /* 1: persisting-L2 access window over the sensed trail (default 1) */
    uint32_t trail_tile;        /* 0: autotuned/default, otherwise 1 + an index into the tile table */
    uint32_t agent_shape;       /* 0: autotuned/default, otherwise 1 + an index into the agent-shape table */
    uint32_t exact_counts;      /* 1: always keep per-cell deposit counts (slime_download_deposit_counts); 0
                                   (default): steps in which every deposit saturates the fold (deposition >= 1
                                   on a non-negative trail) record only which cells received deposits */
} SlimeOptions;

typedef struct SlimeInfo {
    uint32_t width;
    uint32_t height;
    uint64_t n_agents;
    uint64_t steps_done;
    uint64_t kernel_launches; /* kernels enqueued by this context (graph nodes count) */
    uint32_t trail_tile;      /* tile-table index in use */
    uint32_t reordered;       /* 1 if device agent order differs from id order */
    uint32_t agent_shape;     /* agent-kernel shape index in use */
    uint32_t trail_texture;   /* 1 if the trail buffers have gather textures (texture agent shapes usable) */
    uint64_t l2_persist_bytes; /* persisting-L2 carve-out granted for the trail (0 = none) */
    uint32_t l2_window_passes; /* with a carve-out, the passes whose launches carry the window
                                  (bit 0 the agent pass, bit 1 the trail pass) */
    uint32_t _pad;
    uint64_t reorders_done; /* Morton reorders run so far (by the step schedule, slime_reorder_agents or the
                               autotuner) */
} SlimeInfo;

const char* slime_version(void);
const char* slime_status_string(int status);

/* ------------------------------------------------ settings and presets */
/* Settings::default() (src/settings.rs:49-70). */
void slime_settings_default(SlimeSettings* out);
/* The preset table of init_preset_manager() (src/presets.rs:45-155). */
int slime_preset_count(void);
/* PresetManager::get_preset_names / get_preset by position; *name is static. */
int slime_preset_get(int index, const char** name, SlimeSettings* out);
/* PresetManager::get_preset(name) (src/presets.rs:30-32). */
int slime_preset_find(const char* name, SlimeSettings* out);
/* SimSizeUniform::new(width, height, settings.pheromone_decay_factor, settings)
 * (src/main.rs:48-66) plus the reference's defaults for the extensions. */
void slime_params_from_settings(const SlimeSettings* settings, uint32_t width, uint32_t height,
                                SlimeParams* out);
/* Settings as a parameter file (the reference keeps Settings only in memory;
 * `simulation_settings.toml` is named in its .gitignore): one `key = value`
 * line per field of Settings (src/settings.rs:30-47), in the TOML subset that
 * struct maps onto: integers, floats with 9 significant digits (every
 * binary32 round-trips exactly) written with a decimal point or exponent,
 * `true` / `false`, and the heading range as
 * `agent_possible_starting_headings = { start = 0.0, end = 360.0 }`.
 * slime_settings_to_text writes the text and its NUL into buf (cap bytes) and
 * its length without the NUL into *len; SLIME_ERR_INVALID_ARGUMENT if it did
 * not fit (buf NULL and cap 0 ask for the length only). */
int slime_settings_to_text(const SlimeSettings* settings, char* buf, size_t cap, size_t* len);
/* Parse such text: start from Settings::default() and apply each line; `#`
 * starts a comment, blank lines are skipped, keys may come in any order, each
 * at most once.  An unknown or repeated key, a malformed value or an integer
 * out of its field's range returns SLIME_ERR_INVALID_ARGUMENT with the 1-based
 * line in *error_line (when not NULL); `out` is written only on success. */
int slime_settings_from_text(const char* text, SlimeSettings* out, int* error_line);
/* The same through a file. */
int slime_settings_save(const SlimeSettings* settings, const char* path);
int slime_settings_load(const char* path, SlimeSettings* out, int* error_line);

/* ------------------------------------------------ simulation context */
typedef struct slime_ctx slime_ctx;

/* Allocates agents (zeroed) and a zeroed trail on the current CUDA device and
 * installs the default settings' parameters.  Replaces buffer creation at
 * src/main.rs:263-293, PipelineManager::new and BindGroupManager::new. */
slime_ctx* slime_create(uint32_t width, uint32_t height, uint64_t n_agents, int* status);
void slime_destroy(slime_ctx* ctx);
const char* slime_last_error(const slime_ctx* ctx);

/* queue.write_buffer of the uniform (update_settings, src/main.rs:83-99). */
int slime_set_params(slime_ctx* ctx, const SlimeParams* params);
int slime_get_params(const slime_ctx* ctx, SlimeParams* out);
int slime_set_options(slime_ctx* ctx, const SlimeOptions* options);
int slime_get_options(const slime_ctx* ctx, SlimeOptions* out);
int slime_get_info(const slime_ctx* ctx, SlimeInfo* out);

/* Agent buffer writes/reads (src/main.rs:263-282 layout; readback as at
 * src/main.rs:126-131). n must equal the context's agent count. */
int slime_upload_agents(slime_ctx* ctx, const float* aos_xyzw, uint64_t n);
int slime_download_agents(slime_ctx* ctx, float* aos_xyzw, uint64_t n);
/* Seeded replacement of the unseeded host init (src/main.rs:273-280):
 * x ~ U[0,w), y ~ U[0,h), angle ~ U[heading_min, heading_max),
 * speed ~ U[speed_min, speed_max] of the current parameters. */
int slime_seed_agents(slime_ctx* ctx, uint64_t seed, float heading_min, float heading_max);
/* reassign_agent_speeds (src/main.rs:101-145), on the device, seeded. */
int slime_reassign_speeds(slime_ctx* ctx, uint64_t seed);

int slime_upload_trail(slime_ctx* ctx, const float* trail, uint64_t n_cells);
int slime_download_trail(slime_ctx* ctx, float* trail, uint64_t n_cells);
/* Trail clear on key C (src/main.rs:909-913). */
int slime_clear_trail(slime_ctx* ctx);
/* Window resize (src/main.rs:954-1015): agent x,y are scaled by new/old size,
 * the trail is reallocated zeroed.  Out of device memory it returns
 * SLIME_ERR_OUT_OF_MEMORY with the context unchanged (size, agents, trail). */
int slime_resize(slime_ctx* ctx, uint32_t width, uint32_t height);
/* Agent-count change (src/main.rs:682-791): reallocates the agent buffer and
 * seeds every agent anew (seeded; the reference uses rand::random).  Out of
 * device memory it returns SLIME_ERR_OUT_OF_MEMORY with the agents unchanged. */
int slime_set_agent_count(slime_ctx* ctx, uint64_t n_agents, uint64_t seed);

/* Checkpoint / resume (no counterpart in the reference, whose state lives
 * only in its GPU buffers).  slime_state_save writes the context's trail size,
 * agent count, step counter, parameters, agents (AoS, id order) and trail to
 * a file: the 8 bytes "SLMSTATE", then little-endian uint32 version (1),
 * width, height, sizeof(SlimeParams), uint64 agent count and step counter,
 * the SlimeParams bytes, the agents (16 bytes each) and the trail (4 bytes a
 * cell).  slime_state_load restores such a file into a context of the same
 * size and agent count (SLIME_ERR_INVALID_ARGUMENT otherwise, with the
 * context unchanged), including the step counter, so that the Morton reorder
 * schedule continues where it was; the results of the steps that follow are
 * those of the uninterrupted run, bit for bit. */
int slime_state_save(slime_ctx* ctx, const char* path);
int slime_state_load(slime_ctx* ctx, const char* path);
/* Set the step counter (SlimeInfo.steps_done), which places the Morton
 * reorders (one every options.reorder_every steps). */
int slime_set_steps_done(slime_ctx* ctx, uint64_t steps_done);

/* Advance n_steps steps: the agent dispatch, the decay dispatch and the
 * diffuse dispatch of src/main.rs:1163-1235, n_steps times.  Asynchronous with
 * respect to the host; use slime_sync or any download to wait. */
int slime_step(slime_ctx* ctx, uint32_t n_steps);
/* Capture now the CUDA graphs that the next n_steps steps will replay (the
 * same chunks slime_step cuts), without stepping: the first slime_step over
 * them then only replays.  Graphs stay valid until a parameter, option or
 * buffer change (or the first reorder, which adds the id buffer) drops them. */
int slime_prepare_steps(slime_ctx* ctx, uint32_t n_steps);
int slime_sync(slime_ctx* ctx);
/* The cudaStream_t the context enqueues on. */
int slime_get_stream(slime_ctx* ctx, void** stream);
/* Display feed without stalling the step loop: snapshot the current trail on
 * the device (two snapshot buffers used in turn, so a snapshot waits only for
 * the copy two calls back) and copy it to `trail` (width*height floats) on a
 * separate copy stream, so the copy overlaps the steps enqueued after it.
 * Returns at once;
 * `trail` is complete after slime_wait_download (or the next
 * slime_download_trail_async, which first waits for the previous copy).  With
 * page-locked `trail` the copy is asynchronous; with pageable memory the CUDA
 * runtime performs it synchronously. */
int slime_download_trail_async(slime_ctx* ctx, float* trail, uint64_t n_cells);
int slime_wait_download(slime_ctx* ctx);
/* Deposit counts of the most recent step (cells receiving k agents hold k). */
int slime_download_deposit_counts(slime_ctx* ctx, uint32_t* counts, uint64_t n_cells);
/* Reorder agents in Morton order of their cell now (results are unchanged:
 * every agent keeps its id, which seeds its jitter hash). */
int slime_reorder_agents(slime_ctx* ctx);

/* Run n_steps steps without graphs, timing each kernel with CUDA events on
 * the context's stream; totals in milliseconds (NULL outputs are skipped). */
int slime_profile_steps(slime_ctx* ctx, uint32_t n_steps, double* agents_ms, double* trail_ms,
                        double* other_ms);
/* Run `reps` Morton reorders back to back on the context's stream, timed with
 * CUDA events; total milliseconds in *ms.  The agents' results do not change
 * (every agent keeps its id). */
int slime_profile_reorder(slime_ctx* ctx, uint32_t reps, double* ms);
/* Pick the fastest trail tile and agent-kernel shape for this context by
 * timing each candidate in the deposit mode the steps will use, then (with
 * l2_persist on) whether and on which passes the persisting-L2 window pays
 * off, by timing full steps (agents and trail are restored afterwards; the
 * previous step's deposit counts are cleared).  SlimeInfo reports the
 * choices. */
int slime_autotune(slime_ctx* ctx, uint32_t reps);

/* ------------------------------------------------ adjoint (frozen trajectories) */
/* Gradients of a scalar trail loss L(T_final) with respect to the trail-chain
 * parameters, holding the recorded agent trajectories (hence the per-step
 * deposit counts) fixed. */
typedef struct SlimeGrads {
    double d_decay_factor;
    double d_diffusion_rate;
    double d_deposition_amount;
    double reserved;
} SlimeGrads;

/* Run n_steps forward steps from the current state, keeping a checkpoint of
 * agents and trail every ckpt_every steps in device memory. */
int slime_forward_record(slime_ctx* ctx, uint32_t n_steps, uint32_t ckpt_every);
/* Back-propagate dL/dT_final (host, width*height floats) through the recorded
 * steps, recomputing each checkpoint segment; writes the parameter gradients
 * and, if d_trail0 is not NULL, dL/dT_0 (host, width*height floats). */
int slime_backward(slime_ctx* ctx, const float* dl_dtrail_final, SlimeGrads* grads, float* d_trail0);

/* ------------------------------------------------ batched ensemble */
/* Independent colonies of uneven sizes advanced together by one of two
 * engines (SLIME_ENSEMBLE_LANES / SLIME_ENSEMBLE_COOPERATIVE below): every
 * colony's result is the one a single context would produce for it. */
typedef struct slime_ensemble slime_ensemble;

slime_ensemble* slime_ensemble_create(uint32_t n_colonies, const uint32_t* widths,
                                      const uint32_t* heights, const uint64_t* n_agents,
                                      const SlimeParams* params, int* status);
void slime_ensemble_destroy(slime_ensemble* ens);
const char* slime_ensemble_last_error(const slime_ensemble* ens);
int slime_ensemble_set_params(slime_ensemble* ens, uint32_t colony, const SlimeParams* params);
int slime_ensemble_upload_agents(slime_ensemble* ens, uint32_t colony, const float* aos_xyzw, uint64_t n);
int slime_ensemble_download_agents(slime_ensemble* ens, uint32_t colony, float* aos_xyzw, uint64_t n);
int slime_ensemble_seed_agents(slime_ensemble* ens, uint32_t colony, uint64_t seed, float heading_min,
                               float heading_max);
int slime_ensemble_upload_trail(slime_ensemble* ens, uint32_t colony, const float* trail, uint64_t n_cells);
int slime_ensemble_download_trail(slime_ensemble* ens, uint32_t colony, float* trail, uint64_t n_cells);
/* Milliseconds that `reps` back-to-back Morton reorders of every colony take
 * on the device (after one untimed reorder); results do not change. */
int slime_ensemble_profile_reorder(slime_ensemble* ens, uint32_t reps, double* ms);
/* Morton-reorder every colony's agents every `every` steps (0 = never);
 * results do not change, only the memory order of the agents. */
int slime_ensemble_set_reorder(slime_ensemble* ens, uint32_t every, uint32_t cell_log2);
int slime_ensemble_step(slime_ensemble* ens, uint32_t n_steps);
/* As slime_prepare_steps: capture the graphs of the next n_steps steps now. */
int slime_ensemble_prepare_steps(slime_ensemble* ens, uint32_t n_steps);
int slime_ensemble_sync(slime_ensemble* ens);
int slime_ensemble_get_stream(slime_ensemble* ens, void** stream);
int slime_ensemble_autotune(slime_ensemble* ens, uint32_t reps);
/* Engines of slime_ensemble_step (slime_ensemble_autotune times both):
 * COOPERATIVE - one cooperative persistent launch per step (all colonies'
 *   agents, a bounded grid barrier, all colonies' trail strips);
 * LANES - each colony's steps as a chain of the single-colony kernels on one
 *   of up to 64 lanes forked from the ensemble's stream, one CUDA graph per
 *   chunk of steps, so that the colonies' chains run concurrently. */
#define SLIME_ENSEMBLE_COOPERATIVE 0u
#define SLIME_ENSEMBLE_LANES 1u
/* Choose the engine by hand; for LANES also the agent-kernel shape and trail
 * tile (indices of the single-colony tables; the tensor-copy tile is not
 * available here) and the number of lanes (1..64; 0 = one per colony up to
 * 64), over which the colonies are spread largest first onto the least
 * loaded lane.  Results do not change. */
int slime_ensemble_set_engine(slime_ensemble* ens, uint32_t engine, uint32_t lane_agent_shape,
                              uint32_t lane_trail_tile, uint32_t lanes);
/* Choose the cooperative step's launch shape by hand (what slime_ensemble_autotune picks
 * by timing): trail rows per strip item (8, 16 or 32), resident blocks per SM
 * (0 = as many as fit, else 1..4) and agents per thread of the agent phase
 * (4: each stepped alone; 2: stepped as one pair).  Results do not change. */
int slime_ensemble_set_shape(slime_ensemble* ens, uint32_t strip_rows, uint32_t blocks_per_sm,
                             uint32_t agents_per_thread);
/* Total kernels enqueued so far. */
int slime_ensemble_launch_count(const slime_ensemble* ens, uint64_t* out);
typedef struct SlimeEnsembleInfo {
    uint32_t n_colonies;
    uint32_t graphs_in_use; /* 1: the last step chunk was replayed from a captured CUDA graph; 0: the
                               steps ran as direct cooperative launches (no step yet, or the capture
                               was refused, after which the ensemble keeps launching directly) */
    uint64_t steps_done;
    uint64_t kernel_launches;
    uint64_t total_agents;
    uint64_t total_cells;
    uint32_t grid_blocks;   /* blocks of the persistent launch (a multiple of the SM count) */
    uint32_t strip_rows;    /* trail rows per strip work item (autotuned) */
    uint32_t agents_per_thread; /* cooperative engine: agents a thread steps per agent work item, 4
                                   (each alone) or 2 (as one pair); autotuned */
    uint32_t engine;            /* SLIME_ENSEMBLE_COOPERATIVE or SLIME_ENSEMBLE_LANES */
    uint32_t lanes;             /* capture lanes of the lanes engine (0 until it first steps) */
    uint32_t lane_agent_shape;  /* lanes engine: agent-kernel shape (slime_set_agent_shape's table) */
    uint32_t lane_trail_tile;   /* lanes engine: trail tile (slime_set_trail_tile's table) */
    uint32_t marks_colonies;    /* colonies whose last steps recorded deposits as byte marks (lanes
                                   engine, deposition >= 1 on a clean trail) instead of counts */
} SlimeEnsembleInfo;
int slime_ensemble_get_info(const slime_ensemble* ens, SlimeEnsembleInfo* out);
/* Failure-detection self-test: runs one block at the ensemble's grid barrier
 * sized for two, so the release never comes; the bounded wait gives up after
 * ~0.1 s.  Returns SLIME_ERR_DEVICE_TIMEOUT when the timeout was detected and
 * cleared (the ensemble stays usable), another code otherwise. */
int slime_ensemble_selftest_barrier_timeout(slime_ensemble* ens);

/* ------------------------------------------------ step without allocation */
/* No counterpart in the reference.  One step (agents, then deposit fold +
 * decay + diffuse) over caller-owned device buffers, for callers that may not
 * allocate device memory while they run (an engine that owns all device
 * memory in a pre-reserved arena, a frame loop that cannot afford the device
 * synchronisation a cudaMalloc may cause).  It calls no cudaMalloc/cudaFree:
 * the deposit counts live in a fixed array inside the library, sized for
 * trails of at most 1,048,576 cells (4 MiB, held on every GPU that loads the
 * library until the process exits); larger trails, width or height < 2 and
 * d_trail_in == d_trail_out return SLIME_ERR_INVALID_ARGUMENT.  d_x, d_y,
 * d_angle, d_speed: n_agents floats each (agent i has id i), updated in place;
 * d_trail_in / d_trail_out: width*height floats.  Work is enqueued on
 * `stream` (a cudaStream_t, NULL = legacy default stream) and not waited for.
 * Every call looks up the array's device address on the current device (a
 * lookup that allocates nothing, so a device reset cannot leave a stale
 * address behind); the first call on a device also loads the library's
 * device code there, so make it before any stream capture.  All calls share
 * the array and clear it at their start, so calls that overlap on the GPU
 * race. */
int slime_step_noalloc(const SlimeParams* params, uint32_t width, uint32_t height, uint64_t n_agents, float* d_x,
                       float* d_y, float* d_angle, float* d_speed, const float* d_trail_in, float* d_trail_out,
                       void* stream);
/* The same step with the deposit counts in the caller's device memory:
 * d_counts holds width*height uint32 words (cleared by the call).  No limit
 * on the trail size beyond width*height < 2^31, and calls with separate count
 * arrays may overlap on the GPU. */
int slime_step_noalloc_scratch(const SlimeParams* params, uint32_t width, uint32_t height, uint64_t n_agents,
                               float* d_x, float* d_y, float* d_angle, float* d_speed, const float* d_trail_in,
                               float* d_trail_out, uint32_t* d_counts, void* stream);

/* ------------------------------------------------ display feed */
/* Headless equivalent of src/display.wgsl:44-86: colourise the current trail
 * through a 256-entry LUT (768 bytes: R[256] G[256] B[256], the .lut format)
 * into an RGBA8 image of tex_width x tex_height with the same aspect fit. */
int slime_colorize(slime_ctx* ctx, const uint8_t* lut768, uint32_t tex_width, uint32_t tex_height,
                   uint8_t* rgba_out);
/* The same without stalling the step loop (the per-frame display of
 * src/main.rs:1199-1212 fed to a host presenter): colourise the current trail
 * on the context's stream and copy the image to `rgba_out` on the copy stream
 * slime_download_trail_async uses, overlapping the steps enqueued after it.
 * Returns at once; `rgba_out` is complete after slime_wait_download (or the
 * next asynchronous download).  The LUT is uploaded only when its bytes
 * change.  With page-locked `rgba_out` the copy is asynchronous. */
int slime_colorize_async(slime_ctx* ctx, const uint8_t* lut768, uint32_t tex_width, uint32_t tex_height,
                         uint8_t* rgba_out);

#ifdef __cplusplus
}
#endif

#endif /* SLIME_H */
