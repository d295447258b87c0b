//! Rust binding of `libslime_gb300`, the GB300 CUDA core that replaces the
//! reference's three wgpu compute passes.
//!
//! Velfi/slime-mold advances its simulation with the `compute`, `decay` and
//! `diffuse` pipelines built by `PipelineManager` (src/pipeline_manager.rs:37-54)
//! over the bind group of `BindGroupManager` (src/bind_group_manager.rs:101-125),
//! dispatched from the event loop (src/main.rs:1163-1235).  A [`Simulation`]
//! owns the agents and the trail on one GPU and advances them with
//! [`Simulation::step`]; [`Simulation::backward`] is the hand-written adjoint of
//! the deposit -> decay -> diffuse chain (the role an `autograd.Function` plays
//! in PyTorch); [`Ensemble`] steps many independent colonies in one launch per
//! step.
//!
//! The `ffi` module declares every entry point of `include/slime.h` one to one;
//! the safe wrappers check each status and turn it into [`SlimeError`].
//! `SlimeParams` begins with the reference's `SimSizeUniform`
//! (src/main.rs:29-46), field for field, so the struct the reference already
//! fills converts with [`SlimeParams::from_sim_size_bytes`].
#![allow(non_camel_case_types)]

use std::ffi::{CStr, CString, c_char, c_int, c_void};
use std::marker::PhantomData;
use std::path::Path;

pub mod ffi {
    //! `include/slime.h`, declaration for declaration.
    use std::ffi::{c_char, c_int, c_void};

    pub const SLIME_OK: c_int = 0;
    pub const SLIME_ERR_INVALID_ARGUMENT: c_int = -1;
    pub const SLIME_ERR_OUT_OF_MEMORY: c_int = -2;
    pub const SLIME_ERR_CUDA: c_int = -3;
    pub const SLIME_ERR_STATE: c_int = -4;
    pub const SLIME_ERR_DEVICE_TIMEOUT: c_int = -5;
    pub const SLIME_ERR_NO_DEVICE: c_int = -6;

    pub const SLIME_DECAY_REF_SUBTRACT: u32 = 0;
    pub const SLIME_DECAY_MULTIPLY: u32 = 1;
    pub const SLIME_BLUR_REF_BOX3: u32 = 0;
    pub const SLIME_BLUR_GAUSS: u32 = 1;
    pub const SLIME_MAX_BLUR_RADIUS: u32 = 8;
    pub const SLIME_DISPATCH_EACH_AGENT: u32 = 0;
    pub const SLIME_DISPATCH_REFERENCE: u32 = 1;
    pub const SLIME_SENSOR_SHADER: u32 = 0;
    pub const SLIME_SENSOR_ROTATED: u32 = 1;
    pub const SLIME_ENSEMBLE_COOPERATIVE: u32 = 0;
    pub const SLIME_ENSEMBLE_LANES: u32 = 1;

    /// `SimSizeUniform` (src/main.rs:29-46) in its first 14 fields, then the
    /// constants the shader hard-codes and the engine's modes.
    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq, bytemuck::Pod, bytemuck::Zeroable)]
    pub struct SlimeParams {
        pub width: u32,
        pub height: u32,
        pub decay_factor: f32,
        pub agent_jitter: f32,
        pub agent_speed_min: f32,
        pub agent_speed_max: f32,
        pub agent_turn_speed: f32,
        pub agent_sensor_angle: f32,
        pub agent_sensor_distance: f32,
        pub diffusion_rate: f32,
        pub pheromone_deposition_amount: f32,
        pub blur_radius: f32,
        pub blur_sigma: f32,
        pub _pad: u32,
        pub time_step: f32,
        pub decay_mode: u32,
        pub blur_mode: u32,
        pub dispatch_mode: u32,
        pub sensor_mode: u32,
        pub _pad2: u32,
    }

    /// `Settings` (src/settings.rs:30-47), field for field (the heading range
    /// as its two ends, the fullscreen flag as 0 or 1).
    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq)]
    pub struct SlimeSettings {
        pub agent_count: u64,
        pub agent_jitter: f32,
        pub agent_possible_starting_headings_start: f32,
        pub agent_possible_starting_headings_end: f32,
        pub agent_speed_max: f32,
        pub agent_speed_min: f32,
        pub agent_turn_speed: f32,
        pub pheromone_decay_factor: f32,
        pub pheromone_diffusion_rate: f32,
        pub pheromone_deposition_amount: f32,
        pub window_fullscreen: u32,
        pub window_height: u32,
        pub window_width: u32,
        pub agent_sensor_angle: f32,
        pub agent_sensor_distance: f32,
        pub blur_radius: f32,
        pub blur_sigma: f32,
    }

    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq)]
    pub struct SlimeOptions {
        pub use_graphs: u32,
        pub graph_chunk: u32,
        pub reorder_every: u32,
        pub reorder_cell_log2: u32,
        pub l2_persist: u32,
        pub trail_tile: u32,
        pub agent_shape: u32,
        pub exact_counts: u32,
    }

    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq)]
    pub struct SlimeInfo {
        pub width: u32,
        pub height: u32,
        pub n_agents: u64,
        pub steps_done: u64,
        pub kernel_launches: u64,
        pub trail_tile: u32,
        pub reordered: u32,
        pub agent_shape: u32,
        pub trail_texture: u32,
        pub l2_persist_bytes: u64,
        pub l2_window_passes: u32,
        pub _pad: u32,
        pub reorders_done: u64,
    }

    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq)]
    pub struct SlimeGrads {
        pub d_decay_factor: f64,
        pub d_diffusion_rate: f64,
        pub d_deposition_amount: f64,
        pub reserved: f64,
    }

    #[repr(C)]
    #[derive(Copy, Clone, Debug, Default, PartialEq)]
    pub struct SlimeEnsembleInfo {
        pub n_colonies: u32,
        pub graphs_in_use: u32,
        pub steps_done: u64,
        pub kernel_launches: u64,
        pub total_agents: u64,
        pub total_cells: u64,
        pub grid_blocks: u32,
        pub strip_rows: u32,
        pub agents_per_thread: u32,
        pub engine: u32,
        pub lanes: u32,
        pub lane_agent_shape: u32,
        pub lane_trail_tile: u32,
        pub marks_colonies: u32,
    }

    #[repr(C)]
    pub struct slime_ctx {
        _opaque: [u8; 0],
    }

    #[repr(C)]
    pub struct slime_ensemble {
        _opaque: [u8; 0],
    }

    #[link(name = "slime_gb300")]
    unsafe extern "C" {
        pub fn slime_version() -> *const c_char;
        pub fn slime_status_string(status: c_int) -> *const c_char;

        pub fn slime_settings_default(out: *mut SlimeSettings);
        pub fn slime_preset_count() -> c_int;
        pub fn slime_preset_get(index: c_int, name: *mut *const c_char, out: *mut SlimeSettings) -> c_int;
        pub fn slime_preset_find(name: *const c_char, out: *mut SlimeSettings) -> c_int;
        pub fn slime_params_from_settings(settings: *const SlimeSettings, width: u32, height: u32, out: *mut SlimeParams);
        pub fn slime_settings_to_text(settings: *const SlimeSettings, buf: *mut c_char, cap: usize, len: *mut usize) -> c_int;
        pub fn slime_settings_from_text(text: *const c_char, out: *mut SlimeSettings, error_line: *mut c_int) -> c_int;
        pub fn slime_settings_save(settings: *const SlimeSettings, path: *const c_char) -> c_int;
        pub fn slime_settings_load(path: *const c_char, out: *mut SlimeSettings, error_line: *mut c_int) -> c_int;

        pub fn slime_create(width: u32, height: u32, n_agents: u64, status: *mut c_int) -> *mut slime_ctx;
        pub fn slime_destroy(ctx: *mut slime_ctx);
        pub fn slime_last_error(ctx: *const slime_ctx) -> *const c_char;
        pub fn slime_set_params(ctx: *mut slime_ctx, params: *const SlimeParams) -> c_int;
        pub fn slime_get_params(ctx: *const slime_ctx, out: *mut SlimeParams) -> c_int;
        pub fn slime_set_options(ctx: *mut slime_ctx, options: *const SlimeOptions) -> c_int;
        pub fn slime_get_options(ctx: *const slime_ctx, out: *mut SlimeOptions) -> c_int;
        pub fn slime_get_info(ctx: *const slime_ctx, out: *mut SlimeInfo) -> c_int;
        pub fn slime_upload_agents(ctx: *mut slime_ctx, aos_xyzw: *const f32, n: u64) -> c_int;
        pub fn slime_download_agents(ctx: *mut slime_ctx, aos_xyzw: *mut f32, n: u64) -> c_int;
        pub fn slime_seed_agents(ctx: *mut slime_ctx, seed: u64, heading_min: f32, heading_max: f32) -> c_int;
        pub fn slime_reassign_speeds(ctx: *mut slime_ctx, seed: u64) -> c_int;
        pub fn slime_upload_trail(ctx: *mut slime_ctx, trail: *const f32, n_cells: u64) -> c_int;
        pub fn slime_download_trail(ctx: *mut slime_ctx, trail: *mut f32, n_cells: u64) -> c_int;
        pub fn slime_clear_trail(ctx: *mut slime_ctx) -> c_int;
        pub fn slime_resize(ctx: *mut slime_ctx, width: u32, height: u32) -> c_int;
        pub fn slime_set_agent_count(ctx: *mut slime_ctx, n_agents: u64, seed: u64) -> c_int;
        pub fn slime_state_save(ctx: *mut slime_ctx, path: *const c_char) -> c_int;
        pub fn slime_state_load(ctx: *mut slime_ctx, path: *const c_char) -> c_int;
        pub fn slime_set_steps_done(ctx: *mut slime_ctx, steps_done: u64) -> c_int;
        pub fn slime_step(ctx: *mut slime_ctx, n_steps: u32) -> c_int;
        pub fn slime_prepare_steps(ctx: *mut slime_ctx, n_steps: u32) -> c_int;
        pub fn slime_sync(ctx: *mut slime_ctx) -> c_int;
        pub fn slime_get_stream(ctx: *mut slime_ctx, stream: *mut *mut c_void) -> c_int;
        pub fn slime_download_trail_async(ctx: *mut slime_ctx, trail: *mut f32, n_cells: u64) -> c_int;
        pub fn slime_wait_download(ctx: *mut slime_ctx) -> c_int;
        pub fn slime_download_deposit_counts(ctx: *mut slime_ctx, counts: *mut u32, n_cells: u64) -> c_int;
        pub fn slime_reorder_agents(ctx: *mut slime_ctx) -> c_int;
        pub fn slime_profile_steps(ctx: *mut slime_ctx, n_steps: u32, agents_ms: *mut f64, trail_ms: *mut f64,
                                   other_ms: *mut f64) -> c_int;
        pub fn slime_profile_reorder(ctx: *mut slime_ctx, reps: u32, ms: *mut f64) -> c_int;
        pub fn slime_autotune(ctx: *mut slime_ctx, reps: u32) -> c_int;
        pub fn slime_forward_record(ctx: *mut slime_ctx, n_steps: u32, ckpt_every: u32) -> c_int;
        pub fn slime_backward(ctx: *mut slime_ctx, dl_dtrail_final: *const f32, grads: *mut SlimeGrads,
                              d_trail0: *mut f32) -> c_int;

        pub fn slime_ensemble_create(n_colonies: u32, widths: *const u32, heights: *const u32, n_agents: *const u64,
                                     params: *const SlimeParams, status: *mut c_int) -> *mut slime_ensemble;
        pub fn slime_ensemble_destroy(ens: *mut slime_ensemble);
        pub fn slime_ensemble_last_error(ens: *const slime_ensemble) -> *const c_char;
        pub fn slime_ensemble_set_params(ens: *mut slime_ensemble, colony: u32, params: *const SlimeParams) -> c_int;
        pub fn slime_ensemble_upload_agents(ens: *mut slime_ensemble, colony: u32, aos_xyzw: *const f32, n: u64) -> c_int;
        pub fn slime_ensemble_download_agents(ens: *mut slime_ensemble, colony: u32, aos_xyzw: *mut f32, n: u64) -> c_int;
        pub fn slime_ensemble_seed_agents(ens: *mut slime_ensemble, colony: u32, seed: u64, heading_min: f32,
                                          heading_max: f32) -> c_int;
        pub fn slime_ensemble_upload_trail(ens: *mut slime_ensemble, colony: u32, trail: *const f32, n_cells: u64) -> c_int;
        pub fn slime_ensemble_download_trail(ens: *mut slime_ensemble, colony: u32, trail: *mut f32, n_cells: u64) -> c_int;
        pub fn slime_ensemble_set_reorder(ens: *mut slime_ensemble, every: u32, cell_log2: u32) -> c_int;
        pub fn slime_ensemble_step(ens: *mut slime_ensemble, n_steps: u32) -> c_int;
        pub fn slime_ensemble_prepare_steps(ens: *mut slime_ensemble, n_steps: u32) -> c_int;
        pub fn slime_ensemble_profile_reorder(ens: *mut slime_ensemble, reps: u32, ms: *mut f64) -> c_int;
        pub fn slime_ensemble_sync(ens: *mut slime_ensemble) -> c_int;
        pub fn slime_ensemble_get_stream(ens: *mut slime_ensemble, stream: *mut *mut c_void) -> c_int;
        pub fn slime_ensemble_autotune(ens: *mut slime_ensemble, reps: u32) -> c_int;
        pub fn slime_ensemble_set_engine(
            ens: *mut slime_ensemble,
            engine: u32,
            lane_agent_shape: u32,
            lane_trail_tile: u32,
            lanes: u32,
        ) -> c_int;
        pub fn slime_ensemble_set_shape(
            ens: *mut slime_ensemble,
            strip_rows: u32,
            blocks_per_sm: u32,
            agents_per_thread: u32,
        ) -> c_int;
        pub fn slime_ensemble_launch_count(ens: *const slime_ensemble, out: *mut u64) -> c_int;
        pub fn slime_ensemble_get_info(ens: *const slime_ensemble, out: *mut SlimeEnsembleInfo) -> c_int;
        pub fn slime_ensemble_selftest_barrier_timeout(ens: *mut slime_ensemble) -> c_int;

        pub fn slime_step_noalloc(params: *const SlimeParams, width: u32, height: u32, n_agents: u64, d_x: *mut f32,
                                  d_y: *mut f32, d_angle: *mut f32, d_speed: *mut f32, d_trail_in: *const f32,
                                  d_trail_out: *mut f32, stream: *mut c_void) -> c_int;
        pub fn slime_step_noalloc_scratch(params: *const SlimeParams, width: u32, height: u32, n_agents: u64,
                                          d_x: *mut f32, d_y: *mut f32, d_angle: *mut f32, d_speed: *mut f32,
                                          d_trail_in: *const f32, d_trail_out: *mut f32, d_counts: *mut u32,
                                          stream: *mut c_void) -> c_int;

        pub fn slime_colorize(ctx: *mut slime_ctx, lut768: *const u8, tex_width: u32, tex_height: u32,
                              rgba_out: *mut u8) -> c_int;
        pub fn slime_colorize_async(ctx: *mut slime_ctx, lut768: *const u8, tex_width: u32, tex_height: u32,
                                    rgba_out: *mut u8) -> c_int;
    }
}

pub use ffi::{SlimeEnsembleInfo, SlimeGrads, SlimeInfo, SlimeOptions, SlimeParams, SlimeSettings};

/// A failed call: the library's status code and its message.
#[derive(Debug, Clone, PartialEq)]
pub struct SlimeError {
    pub status: i32,
    pub message: String,
}

impl std::fmt::Display for SlimeError {
    fn fmt(&self, f: &mut std::fmt::Formatter<'_>) -> std::fmt::Result {
        write!(f, "slime_gb300 error {}: {}", self.status, self.message)
    }
}

impl std::error::Error for SlimeError {}

pub type Result<T> = std::result::Result<T, SlimeError>;

fn status_text(status: c_int) -> String {
    // SAFETY: slime_status_string returns a static NUL-terminated string.
    unsafe { CStr::from_ptr(ffi::slime_status_string(status)) }.to_string_lossy().into_owned()
}

fn invalid(message: &str) -> SlimeError {
    SlimeError { status: ffi::SLIME_ERR_INVALID_ARGUMENT, message: message.to_owned() }
}

fn c_path(path: &Path) -> Result<CString> {
    CString::new(path.to_string_lossy().as_bytes()).map_err(|_| invalid("path contains a NUL byte"))
}

fn len_u64(len: usize) -> u64 {
    len as u64
}

/// The library's version string.
pub fn version() -> String {
    // SAFETY: a static NUL-terminated string.
    unsafe { CStr::from_ptr(ffi::slime_version()) }.to_string_lossy().into_owned()
}

impl SlimeParams {
    /// The parameters from the reference's `SimSizeUniform` bytes
    /// (src/main.rs:29-46, 56 bytes as `bytemuck::bytes_of` gives them), with
    /// the shader's time step, its subtractive decay and box blur, its agent
    /// indexing and its sensor evaluation.
    pub fn from_sim_size_bytes(uniform: &[u8]) -> Result<Self> {
        if uniform.len() != 56 {
            return Err(invalid("SimSizeUniform is 56 bytes"));
        }
        let mut p = SlimeParams::default();
        bytemuck::bytes_of_mut(&mut p)[..56].copy_from_slice(uniform);
        p.time_step = 0.016;
        p.decay_mode = ffi::SLIME_DECAY_REF_SUBTRACT;
        p.blur_mode = ffi::SLIME_BLUR_REF_BOX3;
        p.dispatch_mode = ffi::SLIME_DISPATCH_EACH_AGENT;
        p.sensor_mode = ffi::SLIME_SENSOR_SHADER;
        Ok(p)
    }

    /// `SimSizeUniform::new(width, height, settings.pheromone_decay_factor,
    /// settings)` (src/main.rs:48-66) plus the reference's extensions.
    pub fn from_settings(settings: &SlimeSettings, width: u32, height: u32) -> Self {
        let mut p = SlimeParams::default();
        // SAFETY: both pointers are valid for the call.
        unsafe { ffi::slime_params_from_settings(settings, width, height, &mut p) };
        p
    }
}

impl SlimeSettings {
    /// `Settings::default()` (src/settings.rs:49-70).
    pub fn reference_default() -> Self {
        let mut s = SlimeSettings::default();
        // SAFETY: `s` is valid for writes.
        unsafe { ffi::slime_settings_default(&mut s) };
        s
    }

    /// The preset table of `init_preset_manager()` (src/presets.rs:45-155):
    /// (name, settings) in the reference's order.
    pub fn presets() -> Vec<(String, SlimeSettings)> {
        // SAFETY: plain query.
        let n = unsafe { ffi::slime_preset_count() };
        let mut out = Vec::with_capacity(n.max(0) as usize);
        for i in 0..n {
            let mut name: *const c_char = std::ptr::null();
            let mut s = SlimeSettings::default();
            // SAFETY: valid out-pointers; the name is static.
            if unsafe { ffi::slime_preset_get(i, &mut name, &mut s) } == ffi::SLIME_OK && !name.is_null() {
                out.push((unsafe { CStr::from_ptr(name) }.to_string_lossy().into_owned(), s));
            }
        }
        out
    }

    /// `PresetManager::get_preset(name)` (src/presets.rs:30-32).
    pub fn preset(name: &str) -> Option<SlimeSettings> {
        let c = CString::new(name).ok()?;
        let mut s = SlimeSettings::default();
        // SAFETY: valid pointers for the call.
        (unsafe { ffi::slime_preset_find(c.as_ptr(), &mut s) } == ffi::SLIME_OK).then_some(s)
    }

    /// The settings as parameter-file text (TOML, one line per field).
    pub fn to_text(&self) -> String {
        let mut len = 0usize;
        // SAFETY: a NULL buffer with capacity 0 asks for the length.
        unsafe { ffi::slime_settings_to_text(self, std::ptr::null_mut(), 0, &mut len) };
        let mut buf = vec![0u8; len + 1];
        // SAFETY: `buf` holds len + 1 bytes.
        let rc = unsafe { ffi::slime_settings_to_text(self, buf.as_mut_ptr() as *mut c_char, buf.len(), &mut len) };
        assert_eq!(rc, ffi::SLIME_OK, "slime_settings_to_text");
        buf.truncate(len);
        String::from_utf8(buf).expect("the settings text is ASCII")
    }

    /// Settings from parameter-file text; the error names the bad line.
    pub fn from_text(text: &str) -> Result<Self> {
        let c = CString::new(text).map_err(|_| invalid("settings text contains a NUL byte"))?;
        let mut s = SlimeSettings::default();
        let mut line: c_int = 0;
        // SAFETY: valid pointers for the call.
        let rc = unsafe { ffi::slime_settings_from_text(c.as_ptr(), &mut s, &mut line) };
        if rc != ffi::SLIME_OK {
            return Err(SlimeError { status: rc, message: format!("settings text: bad line {line}") });
        }
        Ok(s)
    }

    pub fn save(&self, path: &Path) -> Result<()> {
        let c = c_path(path)?;
        // SAFETY: valid pointers for the call.
        let rc = unsafe { ffi::slime_settings_save(self, c.as_ptr()) };
        if rc != ffi::SLIME_OK {
            return Err(SlimeError { status: rc, message: format!("cannot write {}", path.display()) });
        }
        Ok(())
    }

    pub fn load(path: &Path) -> Result<Self> {
        let c = c_path(path)?;
        let mut s = SlimeSettings::default();
        let mut line: c_int = 0;
        // SAFETY: valid pointers for the call.
        let rc = unsafe { ffi::slime_settings_load(c.as_ptr(), &mut s, &mut line) };
        if rc != ffi::SLIME_OK {
            return Err(SlimeError { status: rc, message: format!("{}: cannot read settings (line {line})", path.display()) });
        }
        Ok(s)
    }
}

/// Per-kernel times of [`Simulation::profile_steps`], in milliseconds.
#[derive(Copy, Clone, Debug, Default, PartialEq)]
pub struct StepProfile {
    pub agents_ms: f64,
    pub trail_ms: f64,
    pub other_ms: f64,
}

/// One colony on one GPU: the agent buffer, the trail and the step.
pub struct Simulation {
    ctx: *mut ffi::slime_ctx,
    width: u32,
    height: u32,
    n_agents: u64,
}

// A context may move between threads; it is used from one thread at a time.
unsafe impl Send for Simulation {}

impl Simulation {
    /// Allocates agents (zeroed) and a zeroed trail on the current CUDA
    /// device with the default settings' parameters (src/main.rs:263-293).
    pub fn new(width: u32, height: u32, n_agents: u64) -> Result<Self> {
        let mut status: c_int = 0;
        // SAFETY: `status` is valid for writes.
        let ctx = unsafe { ffi::slime_create(width, height, n_agents, &mut status) };
        if ctx.is_null() {
            return Err(SlimeError { status, message: format!("slime_create: {}", status_text(status)) });
        }
        Ok(Self { ctx, width, height, n_agents })
    }

    pub fn with_params(width: u32, height: u32, n_agents: u64, params: &SlimeParams) -> Result<Self> {
        let mut sim = Self::new(width, height, n_agents)?;
        sim.set_params(params)?;
        Ok(sim)
    }

    pub fn width(&self) -> u32 {
        self.width
    }
    pub fn height(&self) -> u32 {
        self.height
    }
    pub fn n_agents(&self) -> u64 {
        self.n_agents
    }
    fn cells(&self) -> usize {
        self.width as usize * self.height as usize
    }

    fn check(&self, rc: c_int) -> Result<()> {
        if rc == ffi::SLIME_OK {
            return Ok(());
        }
        // SAFETY: the context is alive; the message is NUL-terminated.
        let message = unsafe { CStr::from_ptr(ffi::slime_last_error(self.ctx)) }.to_string_lossy().into_owned();
        Err(SlimeError { status: rc, message })
    }

    fn check_len(&self, got: usize, want: usize, what: &str) -> Result<()> {
        if got != want {
            return Err(invalid(&format!("{what}: {got} elements, expected {want}")));
        }
        Ok(())
    }

    /// `queue.write_buffer` of the uniform (update_settings, src/main.rs:83-99).
    pub fn set_params(&mut self, params: &SlimeParams) -> Result<()> {
        self.check(unsafe { ffi::slime_set_params(self.ctx, params) })
    }
    pub fn params(&self) -> Result<SlimeParams> {
        let mut p = SlimeParams::default();
        self.check(unsafe { ffi::slime_get_params(self.ctx, &mut p) })?;
        Ok(p)
    }
    pub fn set_options(&mut self, options: &SlimeOptions) -> Result<()> {
        self.check(unsafe { ffi::slime_set_options(self.ctx, options) })
    }
    pub fn options(&self) -> Result<SlimeOptions> {
        let mut o = SlimeOptions::default();
        self.check(unsafe { ffi::slime_get_options(self.ctx, &mut o) })?;
        Ok(o)
    }
    pub fn info(&self) -> Result<SlimeInfo> {
        let mut i = SlimeInfo::default();
        self.check(unsafe { ffi::slime_get_info(self.ctx, &mut i) })?;
        Ok(i)
    }

    /// Agents as the reference lays them out: x, y, angle, speed per agent
    /// (src/main.rs:263-282), `4 * n_agents` floats in id order.
    pub fn upload_agents(&mut self, aos_xyzw: &[f32]) -> Result<()> {
        self.check_len(aos_xyzw.len(), 4 * self.n_agents as usize, "upload_agents")?;
        self.check(unsafe { ffi::slime_upload_agents(self.ctx, aos_xyzw.as_ptr(), self.n_agents) })
    }
    pub fn download_agents(&mut self, aos_xyzw: &mut [f32]) -> Result<()> {
        self.check_len(aos_xyzw.len(), 4 * self.n_agents as usize, "download_agents")?;
        self.check(unsafe { ffi::slime_download_agents(self.ctx, aos_xyzw.as_mut_ptr(), self.n_agents) })
    }
    /// Seeded stand-in for the reference's unseeded init (src/main.rs:273-280).
    pub fn seed_agents(&mut self, seed: u64, heading_min: f32, heading_max: f32) -> Result<()> {
        self.check(unsafe { ffi::slime_seed_agents(self.ctx, seed, heading_min, heading_max) })
    }
    /// `reassign_agent_speeds` (src/main.rs:101-145), on the device.
    pub fn reassign_speeds(&mut self, seed: u64) -> Result<()> {
        self.check(unsafe { ffi::slime_reassign_speeds(self.ctx, seed) })
    }
    pub fn upload_trail(&mut self, trail: &[f32]) -> Result<()> {
        self.check_len(trail.len(), self.cells(), "upload_trail")?;
        self.check(unsafe { ffi::slime_upload_trail(self.ctx, trail.as_ptr(), len_u64(trail.len())) })
    }
    /// The display pass's input (src/main.rs:1201-1217), width * height floats.
    pub fn download_trail(&mut self, trail: &mut [f32]) -> Result<()> {
        self.check_len(trail.len(), self.cells(), "download_trail")?;
        self.check(unsafe { ffi::slime_download_trail(self.ctx, trail.as_mut_ptr(), len_u64(trail.len())) })
    }
    /// Key C (src/main.rs:909-913).
    pub fn clear_trail(&mut self) -> Result<()> {
        self.check(unsafe { ffi::slime_clear_trail(self.ctx) })
    }
    /// Window resize (src/main.rs:954-1015).  Out of device memory the library
    /// keeps the old size, agents and trail, so the wrapper's size changes only
    /// on success.
    pub fn resize(&mut self, width: u32, height: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_resize(self.ctx, width, height) })?;
        self.width = width;
        self.height = height;
        Ok(())
    }
    /// Agent-count change (src/main.rs:682-791), reseeded.
    pub fn set_agent_count(&mut self, n_agents: u64, seed: u64) -> Result<()> {
        self.check(unsafe { ffi::slime_set_agent_count(self.ctx, n_agents, seed) })?;
        self.n_agents = n_agents;
        Ok(())
    }

    /// The agent, decay and diffuse dispatches of src/main.rs:1163-1235,
    /// `n_steps` times (asynchronous; [`Simulation::sync`] or any download waits).
    pub fn step(&mut self, n_steps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_step(self.ctx, n_steps) })
    }
    /// Capture the CUDA graphs the next `n_steps` steps replay, without stepping.
    pub fn prepare_steps(&mut self, n_steps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_prepare_steps(self.ctx, n_steps) })
    }
    pub fn sync(&mut self) -> Result<()> {
        self.check(unsafe { ffi::slime_sync(self.ctx) })
    }
    /// The `cudaStream_t` the context enqueues on.
    pub fn stream(&mut self) -> Result<*mut c_void> {
        let mut s: *mut c_void = std::ptr::null_mut();
        self.check(unsafe { ffi::slime_get_stream(self.ctx, &mut s) })?;
        Ok(s)
    }

    /// Start copying the current trail into `trail` without stalling the
    /// steps; the borrow lasts until [`TrailCopy::wait`] (or the guard's drop)
    /// has waited for the copy.
    pub fn download_trail_async<'a>(&'a mut self, trail: &'a mut [f32]) -> Result<TrailCopy<'a>> {
        self.check_len(trail.len(), self.cells(), "download_trail_async")?;
        self.check(unsafe { ffi::slime_download_trail_async(self.ctx, trail.as_mut_ptr(), len_u64(trail.len())) })?;
        Ok(TrailCopy { sim: self, _buf: PhantomData })
    }

    /// The headless display pass (display.wgsl:44-86): the trail through a
    /// 768-byte LUT into `tex_width * tex_height * 4` RGBA bytes.
    pub fn colorize(&mut self, lut768: &[u8], tex_width: u32, tex_height: u32, rgba: &mut [u8]) -> Result<()> {
        self.check_len(lut768.len(), 768, "colorize LUT")?;
        self.check_len(rgba.len(), tex_width as usize * tex_height as usize * 4, "colorize image")?;
        self.check(unsafe { ffi::slime_colorize(self.ctx, lut768.as_ptr(), tex_width, tex_height, rgba.as_mut_ptr()) })
    }
    /// The same overlapped with the steps; complete after [`TrailCopy::wait`].
    pub fn colorize_async<'a>(&'a mut self, lut768: &[u8], tex_width: u32, tex_height: u32,
                              rgba: &'a mut [u8]) -> Result<TrailCopy<'a>> {
        self.check_len(lut768.len(), 768, "colorize LUT")?;
        self.check_len(rgba.len(), tex_width as usize * tex_height as usize * 4, "colorize image")?;
        self.check(unsafe {
            ffi::slime_colorize_async(self.ctx, lut768.as_ptr(), tex_width, tex_height, rgba.as_mut_ptr())
        })?;
        Ok(TrailCopy { sim: self, _buf: PhantomData })
    }

    /// Deposit counts of the most recent step (needs `exact_counts` when every
    /// deposit saturates the fold).
    pub fn download_deposit_counts(&mut self, counts: &mut [u32]) -> Result<()> {
        self.check_len(counts.len(), self.cells(), "download_deposit_counts")?;
        self.check(unsafe { ffi::slime_download_deposit_counts(self.ctx, counts.as_mut_ptr(), len_u64(counts.len())) })
    }
    pub fn reorder_agents(&mut self) -> Result<()> {
        self.check(unsafe { ffi::slime_reorder_agents(self.ctx) })
    }
    pub fn autotune(&mut self, reps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_autotune(self.ctx, reps) })
    }
    pub fn profile_steps(&mut self, n_steps: u32) -> Result<StepProfile> {
        let mut p = StepProfile::default();
        self.check(unsafe {
            ffi::slime_profile_steps(self.ctx, n_steps, &mut p.agents_ms, &mut p.trail_ms, &mut p.other_ms)
        })?;
        Ok(p)
    }
    pub fn profile_reorder(&mut self, reps: u32) -> Result<f64> {
        let mut ms = 0.0f64;
        self.check(unsafe { ffi::slime_profile_reorder(self.ctx, reps, &mut ms) })?;
        Ok(ms)
    }

    /// Checkpoint to a file (size, agent count, step counter, parameters,
    /// agents, trail).
    pub fn save_state(&mut self, path: &Path) -> Result<()> {
        let c = c_path(path)?;
        self.check(unsafe { ffi::slime_state_save(self.ctx, c.as_ptr()) })
    }
    /// Resume from a checkpoint of the same size and agent count.
    pub fn load_state(&mut self, path: &Path) -> Result<()> {
        let c = c_path(path)?;
        self.check(unsafe { ffi::slime_state_load(self.ctx, c.as_ptr()) })
    }
    pub fn set_steps_done(&mut self, steps_done: u64) -> Result<()> {
        self.check(unsafe { ffi::slime_set_steps_done(self.ctx, steps_done) })
    }

    /// Run `n_steps` steps from the current state keeping a checkpoint every
    /// `ckpt_every` steps, for [`Simulation::backward`].
    pub fn forward_record(&mut self, n_steps: u32, ckpt_every: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_forward_record(self.ctx, n_steps, ckpt_every) })
    }

    /// The `autograd.Function` role: the gradients of a scalar trail loss with
    /// respect to decay, diffusion rate and deposition amount, holding the
    /// recorded agent trajectories fixed, from `dl_dtrail_final` = dL/dT_final;
    /// with `d_trail0` also dL/dT_0.
    pub fn backward(&mut self, dl_dtrail_final: &[f32], d_trail0: Option<&mut [f32]>) -> Result<SlimeGrads> {
        self.check_len(dl_dtrail_final.len(), self.cells(), "backward dL/dT")?;
        let d0 = match d_trail0 {
            Some(buf) => {
                self.check_len(buf.len(), self.cells(), "backward dL/dT0")?;
                buf.as_mut_ptr()
            }
            None => std::ptr::null_mut(),
        };
        let mut g = SlimeGrads::default();
        self.check(unsafe { ffi::slime_backward(self.ctx, dl_dtrail_final.as_ptr(), &mut g, d0) })?;
        Ok(g)
    }
}

impl Drop for Simulation {
    fn drop(&mut self) {
        // SAFETY: the context came from slime_create and is destroyed once;
        // slime_destroy waits for the copies in flight.
        unsafe { ffi::slime_destroy(self.ctx) }
    }
}

/// An asynchronous copy into a host buffer that stays borrowed until the copy
/// has been waited for.
pub struct TrailCopy<'a> {
    sim: &'a mut Simulation,
    _buf: PhantomData<&'a mut [u8]>,
}

impl TrailCopy<'_> {
    pub fn wait(self) -> Result<()> {
        let rc = unsafe { ffi::slime_wait_download(self.sim.ctx) };
        let r = self.sim.check(rc);
        std::mem::forget(self);
        r
    }
}

impl Drop for TrailCopy<'_> {
    fn drop(&mut self) {
        // SAFETY: waiting makes the buffer's borrow end after the copy.
        unsafe { ffi::slime_wait_download(self.sim.ctx) };
    }
}

/// Independent colonies of uneven sizes advanced in one launch per step.
pub struct Ensemble {
    ens: *mut ffi::slime_ensemble,
    sizes: Vec<(u32, u32, u64)>,
}

unsafe impl Send for Ensemble {}

impl Ensemble {
    /// One colony per entry of `colonies`: (width, height, agents, parameters).
    pub fn new(colonies: &[(u32, u32, u64, SlimeParams)]) -> Result<Self> {
        let w: Vec<u32> = colonies.iter().map(|c| c.0).collect();
        let h: Vec<u32> = colonies.iter().map(|c| c.1).collect();
        let n: Vec<u64> = colonies.iter().map(|c| c.2).collect();
        let p: Vec<SlimeParams> = colonies.iter().map(|c| c.3).collect();
        let mut status: c_int = 0;
        // SAFETY: the four arrays hold colonies.len() entries each.
        let ens = unsafe {
            ffi::slime_ensemble_create(colonies.len() as u32, w.as_ptr(), h.as_ptr(), n.as_ptr(), p.as_ptr(),
                                       &mut status)
        };
        if ens.is_null() {
            return Err(SlimeError { status, message: format!("slime_ensemble_create: {}", status_text(status)) });
        }
        Ok(Self { ens, sizes: colonies.iter().map(|c| (c.0, c.1, c.2)).collect() })
    }

    fn check(&self, rc: c_int) -> Result<()> {
        if rc == ffi::SLIME_OK {
            return Ok(());
        }
        let message = unsafe { CStr::from_ptr(ffi::slime_ensemble_last_error(self.ens)) }.to_string_lossy().into_owned();
        Err(SlimeError { status: rc, message })
    }

    fn colony(&self, j: u32) -> Result<(u32, u32, u64)> {
        self.sizes.get(j as usize).copied().ok_or_else(|| invalid("colony index out of range"))
    }

    pub fn set_params(&mut self, colony: u32, params: &SlimeParams) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_set_params(self.ens, colony, params) })
    }
    pub fn upload_agents(&mut self, colony: u32, aos_xyzw: &[f32]) -> Result<()> {
        let (_, _, n) = self.colony(colony)?;
        if aos_xyzw.len() != 4 * n as usize {
            return Err(invalid("upload_agents: 4 floats per agent"));
        }
        self.check(unsafe { ffi::slime_ensemble_upload_agents(self.ens, colony, aos_xyzw.as_ptr(), n) })
    }
    pub fn download_agents(&mut self, colony: u32, aos_xyzw: &mut [f32]) -> Result<()> {
        let (_, _, n) = self.colony(colony)?;
        if aos_xyzw.len() != 4 * n as usize {
            return Err(invalid("download_agents: 4 floats per agent"));
        }
        self.check(unsafe { ffi::slime_ensemble_download_agents(self.ens, colony, aos_xyzw.as_mut_ptr(), n) })
    }
    pub fn seed_agents(&mut self, colony: u32, seed: u64, heading_min: f32, heading_max: f32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_seed_agents(self.ens, colony, seed, heading_min, heading_max) })
    }
    pub fn upload_trail(&mut self, colony: u32, trail: &[f32]) -> Result<()> {
        let (w, h, _) = self.colony(colony)?;
        if trail.len() != w as usize * h as usize {
            return Err(invalid("upload_trail: width * height floats"));
        }
        self.check(unsafe { ffi::slime_ensemble_upload_trail(self.ens, colony, trail.as_ptr(), len_u64(trail.len())) })
    }
    pub fn download_trail(&mut self, colony: u32, trail: &mut [f32]) -> Result<()> {
        let (w, h, _) = self.colony(colony)?;
        if trail.len() != w as usize * h as usize {
            return Err(invalid("download_trail: width * height floats"));
        }
        self.check(unsafe {
            ffi::slime_ensemble_download_trail(self.ens, colony, trail.as_mut_ptr(), len_u64(trail.len()))
        })
    }
    pub fn set_reorder(&mut self, every: u32, cell_log2: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_set_reorder(self.ens, every, cell_log2) })
    }
    pub fn step(&mut self, n_steps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_step(self.ens, n_steps) })
    }
    pub fn prepare_steps(&mut self, n_steps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_prepare_steps(self.ens, n_steps) })
    }
    /// Milliseconds that `reps` back-to-back reorders of every colony take.
    pub fn profile_reorder(&mut self, reps: u32) -> Result<f64> {
        let mut ms = 0.0f64;
        self.check(unsafe { ffi::slime_ensemble_profile_reorder(self.ens, reps, &mut ms) })?;
        Ok(ms)
    }
    pub fn sync(&mut self) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_sync(self.ens) })
    }
    pub fn stream(&mut self) -> Result<*mut c_void> {
        let mut s: *mut c_void = std::ptr::null_mut();
        self.check(unsafe { ffi::slime_ensemble_get_stream(self.ens, &mut s) })?;
        Ok(s)
    }
    pub fn autotune(&mut self, reps: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_autotune(self.ens, reps) })
    }
    /// Engine by hand (`SLIME_ENSEMBLE_COOPERATIVE` / `SLIME_ENSEMBLE_LANES`),
    /// with the lanes engine's agent shape, trail tile and lane count (0: one
    /// per colony, at most 64).
    pub fn set_engine(&mut self, engine: u32, lane_agent_shape: u32, lane_trail_tile: u32, lanes: u32) -> Result<()> {
        self.check(unsafe {
            ffi::slime_ensemble_set_engine(self.ens, engine, lane_agent_shape, lane_trail_tile, lanes)
        })
    }
    /// Cooperative launch shape by hand: strip rows (8, 16, 32), blocks per SM (0 = all
    /// that fit), agents per thread (4 or 2).
    pub fn set_shape(&mut self, strip_rows: u32, blocks_per_sm: u32, agents_per_thread: u32) -> Result<()> {
        self.check(unsafe { ffi::slime_ensemble_set_shape(self.ens, strip_rows, blocks_per_sm, agents_per_thread) })
    }
    pub fn launch_count(&self) -> Result<u64> {
        let mut v = 0u64;
        self.check(unsafe { ffi::slime_ensemble_launch_count(self.ens, &mut v) })?;
        Ok(v)
    }
    pub fn info(&self) -> Result<SlimeEnsembleInfo> {
        let mut i = SlimeEnsembleInfo::default();
        self.check(unsafe { ffi::slime_ensemble_get_info(self.ens, &mut i) })?;
        Ok(i)
    }
    /// The failure-detection self-test of the bounded grid barrier: `Ok(true)`
    /// when the wait ran out, was reported and cleared.
    pub fn selftest_barrier_timeout(&mut self) -> Result<bool> {
        let rc = unsafe { ffi::slime_ensemble_selftest_barrier_timeout(self.ens) };
        if rc == ffi::SLIME_ERR_DEVICE_TIMEOUT {
            return Ok(true);
        }
        self.check(rc).map(|_| false)
    }
}

impl Drop for Ensemble {
    fn drop(&mut self) {
        // SAFETY: created by slime_ensemble_create, destroyed once.
        unsafe { ffi::slime_ensemble_destroy(self.ens) }
    }
}

/// One step over device buffers the caller owns, allocating nothing
/// (`slime_step_noalloc`); the trail is limited to 1,048,576 cells and calls
/// must not overlap on the GPU.
///
/// # Safety
/// Every pointer is a device address valid for the sizes given
/// (`n_agents` floats for each agent array, `width * height` floats for each
/// trail, the two trails distinct), and `stream` is a `cudaStream_t` or null.
pub unsafe fn step_noalloc(params: &SlimeParams, width: u32, height: u32, n_agents: u64, d_x: *mut f32,
                           d_y: *mut f32, d_angle: *mut f32, d_speed: *mut f32, d_trail_in: *const f32,
                           d_trail_out: *mut f32, stream: *mut c_void) -> Result<()> {
    // SAFETY: the caller's contract above.
    let rc = unsafe {
        ffi::slime_step_noalloc(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in, d_trail_out,
                                stream)
    };
    if rc != ffi::SLIME_OK {
        return Err(SlimeError { status: rc, message: status_text(rc) });
    }
    Ok(())
}

/// The same with the deposit counts in `d_counts` (`width * height` words of
/// the caller's device memory): any trail size.
///
/// # Safety
/// As [`step_noalloc`], and `d_counts` is valid for `width * height` words.
pub unsafe fn step_noalloc_scratch(params: &SlimeParams, width: u32, height: u32, n_agents: u64, d_x: *mut f32,
                                   d_y: *mut f32, d_angle: *mut f32, d_speed: *mut f32, d_trail_in: *const f32,
                                   d_trail_out: *mut f32, d_counts: *mut u32, stream: *mut c_void) -> Result<()> {
    // SAFETY: the caller's contract above.
    let rc = unsafe {
        ffi::slime_step_noalloc_scratch(params, width, height, n_agents, d_x, d_y, d_angle, d_speed, d_trail_in,
                                        d_trail_out, d_counts, stream)
    };
    if rc != ffi::SLIME_OK {
        return Err(SlimeError { status: rc, message: status_text(rc) });
    }
    Ok(())
}

#[cfg(test)]
mod tests {
    use super::*;

    #[test]
    fn layouts_match_the_header() {
        assert_eq!(std::mem::size_of::<SlimeParams>(), 80);
        assert_eq!(std::mem::size_of::<SlimeSettings>(), 72);
        assert_eq!(std::mem::size_of::<SlimeOptions>(), 32);
        assert_eq!(std::mem::size_of::<SlimeInfo>(), 72);
        assert_eq!(std::mem::size_of::<SlimeGrads>(), 32);
        assert_eq!(std::mem::size_of::<SlimeEnsembleInfo>(), 72);
    }

    #[test]
    fn settings_round_trip_without_a_device() {
        for (name, s) in SlimeSettings::presets() {
            assert_eq!(SlimeSettings::from_text(&s.to_text()).unwrap(), s, "{name}");
        }
        assert!(SlimeSettings::from_text("no_such_key = 1\n").is_err());
    }
}
