"""Python host API of the GB300 Physarum core (ctypes over libslime_gb300.so).

Mirrors the reference's parameter surface -- Settings (src/settings.rs:30-47),
the presets (src/presets.rs:45-155), SimSizeUniform::new (src/main.rs:48-66) --
and replaces its wgpu compute passes (src/compute.wgsl "main", "decay_trail",
"diffuse_trail", dispatched from src/main.rs:1163-1235) with a Simulation
object whose step() runs the CUDA kernels.  Every call goes through the C ABI
of include/slime.h; there is no CPU fallback.
"""
import ctypes as C

import numpy as np

from . import _abi
from ._abi import (BLUR_GAUSS, BLUR_REF_BOX3, DECAY_MULTIPLY, DECAY_REF_SUBTRACT, DISPATCH_EACH_AGENT,
                   DISPATCH_REFERENCE, ENSEMBLE_COOPERATIVE, ENSEMBLE_LANES, MAX_BLUR_RADIUS, SENSOR_ROTATED, SENSOR_SHADER, SlimeEnsembleInfo,
                   SlimeGrads, SlimeInfo, SlimeOptions, SlimeParams, SlimeSettings)

__all__ = [
    "SlimeError", "Settings", "default_settings", "preset_names", "preset", "params_from_settings",
    "settings_to_text", "settings_from_text", "save_settings", "load_settings", "SlimeEnsembleInfo",
    "Simulation", "Ensemble", "SlimeParams", "SlimeOptions", "SlimeGrads", "lib",
    "DECAY_REF_SUBTRACT", "DECAY_MULTIPLY", "BLUR_REF_BOX3", "BLUR_GAUSS", "MAX_BLUR_RADIUS",
    "DISPATCH_EACH_AGENT", "DISPATCH_REFERENCE", "SENSOR_SHADER", "SENSOR_ROTATED",
    "ENSEMBLE_COOPERATIVE", "ENSEMBLE_LANES",
]

Settings = SlimeSettings


class SlimeError(RuntimeError):
    def __init__(self, status, message):
        super().__init__(f"[{status}] {message}")
        self.status = status


def lib():
    return _abi.load()


def _f32p(a):
    return a.ctypes.data_as(_abi.F32P)


def _host_out(out, dtype, size, what):
    """`out` as a destination the library may fill with `size` elements of
    `dtype`: the C functions write exactly that many, so anything smaller,
    strided or of another type is refused before the call."""
    if not isinstance(out, np.ndarray) or out.dtype != dtype or not out.flags.c_contiguous \
            or not out.flags.writeable or out.size != size:
        raise ValueError(f"{what}: expected a writeable C-contiguous {np.dtype(dtype).name} array of "
                         f"{size} elements")
    return out


def default_settings():
    """Settings::default() (src/settings.rs:49-70)."""
    s = SlimeSettings()
    lib().slime_settings_default(C.byref(s))
    return s


def preset_names():
    """PresetManager::get_preset_names() of init_preset_manager()."""
    L = lib()
    out = []
    for i in range(L.slime_preset_count()):
        name = C.c_char_p()
        L.slime_preset_get(i, C.byref(name), None)
        out.append(name.value.decode())
    return out


def preset(name):
    """PresetManager::get_preset(name).settings, or KeyError."""
    s = SlimeSettings()
    if lib().slime_preset_find(name.encode(), C.byref(s)) != 0:
        raise KeyError(name)
    return s


def params_from_settings(settings, width, height, **overrides):
    """SimSizeUniform::new(width, height, decay, settings) plus the
    extensions (time_step=0.016, reference decay and blur modes)."""
    p = SlimeParams()
    lib().slime_params_from_settings(C.byref(settings), width, height, C.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def settings_to_text(settings):
    """The settings as parameter-file text (slime_settings_to_text)."""
    L = lib()
    n = C.c_size_t()
    L.slime_settings_to_text(C.byref(settings), None, 0, C.byref(n))
    buf = C.create_string_buffer(n.value + 1)
    if L.slime_settings_to_text(C.byref(settings), buf, n.value + 1, C.byref(n)) != 0:
        raise SlimeError(_abi.SLIME_ERR_INVALID_ARGUMENT, "settings_to_text failed")
    return buf.value.decode()


def settings_from_text(text):
    """Settings parsed from parameter-file text; ValueError names the bad line."""
    s, line = SlimeSettings(), C.c_int()
    if lib().slime_settings_from_text(text.encode(), C.byref(s), C.byref(line)) != 0:
        raise ValueError(f"settings text: bad line {line.value}")
    return s


def save_settings(settings, path):
    if lib().slime_settings_save(C.byref(settings), str(path).encode()) != 0:
        raise OSError(f"cannot write settings to {path}")


def load_settings(path):
    s, line = SlimeSettings(), C.c_int()
    if lib().slime_settings_load(str(path).encode(), C.byref(s), C.byref(line)) != 0:
        raise ValueError(f"{path}: cannot read settings" + (f" (bad line {line.value})" if line.value else ""))
    return s


class Simulation:
    """One colony on one GPU: the agent buffer, the trail and the step."""

    def __init__(self, width, height, n_agents, params=None):
        self._inflight = {}  # host buffers the asynchronous copies still fill
        self._L = lib()
        st = C.c_int(0)
        self._h = self._L.slime_create(width, height, n_agents, C.byref(st))
        if not self._h:
            raise SlimeError(st.value, f"slime_create({width}, {height}, {n_agents}) failed: "
                             + self._L.slime_status_string(st.value).decode())
        self.width, self.height, self.n_agents = width, height, n_agents
        if params is not None:
            self.set_params(params)

    # -- lifecycle
    def close(self):
        if getattr(self, "_h", None):
            self._L.slime_destroy(self._h)  # waits for the copies in flight
            self._h = None
        self._inflight = {}

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc, what):
        if rc != 0:
            msg = self._L.slime_last_error(self._h)
            raise SlimeError(rc, f"{what}: {msg.decode() if msg else ''}")

    @property
    def handle(self):
        return self._h

    # -- parameters and options
    def set_params(self, params):
        self._check(self._L.slime_set_params(self._h, C.byref(params)), "set_params")

    def params(self):
        p = SlimeParams()
        self._check(self._L.slime_get_params(self._h, C.byref(p)), "get_params")
        return p

    def options(self):
        o = SlimeOptions()
        self._check(self._L.slime_get_options(self._h, C.byref(o)), "get_options")
        return o

    def set_options(self, **kw):
        o = self.options()
        for k, v in kw.items():
            setattr(o, k, v)
        self._check(self._L.slime_set_options(self._h, C.byref(o)), "set_options")

    def info(self):
        i = SlimeInfo()
        self._check(self._L.slime_get_info(self._h, C.byref(i)), "get_info")
        return i

    # -- state
    def upload_agents(self, aos):
        a = np.ascontiguousarray(aos, dtype=np.float32).reshape(-1, 4)
        self._check(self._L.slime_upload_agents(self._h, _f32p(a), a.shape[0]), "upload_agents")

    def download_agents(self, out=None):
        a = _host_out(out, np.float32, 4 * self.n_agents, "download_agents") if out is not None \
            else np.empty((self.n_agents, 4), np.float32)
        self._check(self._L.slime_download_agents(self._h, _f32p(a), self.n_agents), "download_agents")
        return a

    def seed_agents(self, seed, heading_min=0.0, heading_max=6.28318530718):
        self._check(self._L.slime_seed_agents(self._h, seed, heading_min, heading_max), "seed_agents")

    def reassign_speeds(self, seed):
        self._check(self._L.slime_reassign_speeds(self._h, seed), "reassign_speeds")

    def upload_trail(self, trail):
        t = np.ascontiguousarray(trail, dtype=np.float32).reshape(-1)
        self._check(self._L.slime_upload_trail(self._h, _f32p(t), t.size), "upload_trail")

    def download_trail(self, out=None):
        t = _host_out(out, np.float32, self.width * self.height, "download_trail") if out is not None \
            else np.empty((self.height, self.width), np.float32)
        self._check(self._L.slime_download_trail(self._h, _f32p(t), self.width * self.height), "download_trail")
        return t

    def download_trail_async(self, out):
        """Start copying the current trail into `out` (a C-contiguous float32
        array, ideally page-locked); complete after wait_download(), until
        which this object keeps a reference to `out`."""
        _host_out(out, np.float32, self.width * self.height, "download_trail_async")
        self._check(self._L.slime_download_trail_async(self._h, _f32p(out), out.size), "download_trail_async")
        self._inflight[id(out)] = out

    def wait_download(self):
        self._check(self._L.slime_wait_download(self._h), "wait_download")
        self._inflight = {}

    def download_deposit_counts(self):
        c = np.empty((self.height, self.width), np.uint32)
        self._check(self._L.slime_download_deposit_counts(self._h, c.ctypes.data_as(_abi.U32P), c.size),
                    "download_deposit_counts")
        return c

    def clear_trail(self):
        self._check(self._L.slime_clear_trail(self._h), "clear_trail")

    def resize(self, width, height):
        self._check(self._L.slime_resize(self._h, width, height), "resize")
        self.width, self.height = width, height

    def set_agent_count(self, n, seed=0):
        self._check(self._L.slime_set_agent_count(self._h, n, seed), "set_agent_count")
        self.n_agents = n

    # -- stepping
    def step(self, n_steps=1):
        self._check(self._L.slime_step(self._h, n_steps), "step")

    def prepare_steps(self, n_steps):
        """Capture the CUDA graphs the next n_steps steps replay, without
        stepping (slime_prepare_steps)."""
        self._check(self._L.slime_prepare_steps(self._h, n_steps), "prepare_steps")

    def sync(self):
        self._check(self._L.slime_sync(self._h), "sync")

    def stream_ptr(self):
        s = C.c_void_p()
        self._check(self._L.slime_get_stream(self._h, C.byref(s)), "get_stream")
        return s.value or 0

    def reorder_agents(self):
        self._check(self._L.slime_reorder_agents(self._h), "reorder_agents")

    def profile_steps(self, n_steps):
        a, t, o = C.c_double(), C.c_double(), C.c_double()
        self._check(self._L.slime_profile_steps(self._h, n_steps, C.byref(a), C.byref(t), C.byref(o)),
                    "profile_steps")
        return a.value, t.value, o.value

    def profile_reorder(self, reps=5):
        """Milliseconds that `reps` back-to-back Morton reorders take on the device."""
        ms = C.c_double()
        self._check(self._L.slime_profile_reorder(self._h, reps, C.byref(ms)), "profile_reorder")
        return ms.value

    def autotune(self, reps=5):
        self._check(self._L.slime_autotune(self._h, reps), "autotune")

    # -- checkpoint / resume
    def save_state(self, path):
        """Write trail size, agent count, step counter, parameters, agents
        (id order, AoS) and trail to a state file (slime_state_save)."""
        self._check(self._L.slime_state_save(self._h, str(path).encode()), "save_state")

    def restore_state(self, path):
        """Load a state file of this simulation's size and agent count into
        it, step counter included (slime_state_load)."""
        self._check(self._L.slime_state_load(self._h, str(path).encode()), "load_state")

    @classmethod
    def load_state(cls, path):
        """A new Simulation holding the state saved by save_state."""
        import struct
        with open(path, "rb") as f:
            head = f.read(40)
        if len(head) != 40 or head[:8] != b"SLMSTATE":
            raise ValueError(f"{path}: not a state file")
        _, W, H, _ = struct.unpack_from("<4I", head, 8)
        n, _ = struct.unpack_from("<2Q", head, 24)
        sim = cls(W, H, n)
        sim.restore_state(path)
        return sim

    def set_steps_done(self, steps):
        self._check(self._L.slime_set_steps_done(self._h, steps), "set_steps_done")

    # -- adjoint
    def forward_record(self, n_steps, ckpt_every=50):
        self._check(self._L.slime_forward_record(self._h, n_steps, ckpt_every), "forward_record")

    def backward(self, dl_dtrail_final, want_trail_grad=True):
        g = np.ascontiguousarray(dl_dtrail_final, dtype=np.float32).reshape(-1)
        if g.size != self.width * self.height:
            raise ValueError(f"backward: dL/dT has {g.size} cells, the trail {self.width * self.height}")
        out = SlimeGrads()
        d0 = np.empty((self.height, self.width), np.float32) if want_trail_grad else None
        self._check(self._L.slime_backward(self._h, _f32p(g), C.byref(out),
                                           _f32p(d0) if d0 is not None else None), "backward")
        return out, d0

    # -- display feed
    def colorize(self, lut768, tex_width, tex_height):
        lut = np.ascontiguousarray(lut768, dtype=np.uint8).reshape(-1)
        if lut.size != 768:
            raise ValueError("a LUT has 768 bytes (R[256] G[256] B[256])")
        img = np.empty((tex_height, tex_width, 4), np.uint8)
        self._check(self._L.slime_colorize(self._h, lut.ctypes.data_as(_abi.U8P), tex_width, tex_height,
                                           img.ctypes.data_as(_abi.U8P)), "colorize")
        return img

    def colorize_async(self, lut768, out):
        """Start colourising the current trail into `out` (a C-contiguous
        (height, width, 4) uint8 image, ideally page-locked); complete after
        wait_download()."""
        lut = np.ascontiguousarray(lut768, dtype=np.uint8).reshape(-1)
        if lut.size != 768:
            raise ValueError("a LUT has 768 bytes (R[256] G[256] B[256])")
        if not isinstance(out, np.ndarray) or out.ndim != 3 or out.shape[2] != 4:
            raise ValueError("colorize_async: expected a (height, width, 4) uint8 image")
        _host_out(out, np.uint8, out.size, "colorize_async")
        self._check(self._L.slime_colorize_async(self._h, lut.ctypes.data_as(_abi.U8P), out.shape[1], out.shape[0],
                                                 out.ctypes.data_as(_abi.U8P)), "colorize_async")
        self._inflight[id(out)] = out


class Ensemble:
    """Independent colonies of uneven sizes advanced together."""

    def __init__(self, widths, heights, n_agents, params):
        self._L = lib()
        k = len(widths)
        if not (len(heights) == k and len(n_agents) == k and len(params) == k):
            raise ValueError("widths, heights, n_agents and params need one entry per colony")
        W = (C.c_uint32 * k)(*widths)
        H = (C.c_uint32 * k)(*heights)
        N = (C.c_uint64 * k)(*n_agents)
        P = (SlimeParams * k)(*params)
        st = C.c_int(0)
        self._h = self._L.slime_ensemble_create(k, W, H, N, P, C.byref(st))
        if not self._h:
            raise SlimeError(st.value, "slime_ensemble_create failed: "
                             + self._L.slime_status_string(st.value).decode())
        self.widths, self.heights, self.n_agents = list(widths), list(heights), list(n_agents)

    def close(self):
        if getattr(self, "_h", None):
            self._L.slime_ensemble_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != 0:
            msg = self._L.slime_ensemble_last_error(self._h)
            raise SlimeError(rc, f"{what}: {msg.decode() if msg else ''}")

    def set_params(self, colony, params):
        self._check(self._L.slime_ensemble_set_params(self._h, colony, C.byref(params)), "set_params")

    def upload_agents(self, colony, aos):
        a = np.ascontiguousarray(aos, dtype=np.float32).reshape(-1, 4)
        self._check(self._L.slime_ensemble_upload_agents(self._h, colony, _f32p(a), a.shape[0]), "upload_agents")

    def download_agents(self, colony):
        a = np.empty((self.n_agents[colony], 4), np.float32)
        self._check(self._L.slime_ensemble_download_agents(self._h, colony, _f32p(a), a.shape[0]),
                    "download_agents")
        return a

    def seed_agents(self, colony, seed, heading_min=0.0, heading_max=6.28318530718):
        self._check(self._L.slime_ensemble_seed_agents(self._h, colony, seed, heading_min, heading_max),
                    "seed_agents")

    def upload_trail(self, colony, trail):
        t = np.ascontiguousarray(trail, dtype=np.float32).reshape(-1)
        self._check(self._L.slime_ensemble_upload_trail(self._h, colony, _f32p(t), t.size), "upload_trail")

    def download_trail(self, colony):
        t = np.empty((self.heights[colony], self.widths[colony]), np.float32)
        self._check(self._L.slime_ensemble_download_trail(self._h, colony, _f32p(t), t.size), "download_trail")
        return t

    def set_reorder(self, every, cell_log2=2):
        self._check(self._L.slime_ensemble_set_reorder(self._h, every, cell_log2), "set_reorder")

    def step(self, n_steps=1):
        self._check(self._L.slime_ensemble_step(self._h, n_steps), "step")

    def prepare_steps(self, n_steps):
        """Capture the graphs of the next n_steps steps now (slime_ensemble_prepare_steps)."""
        self._check(self._L.slime_ensemble_prepare_steps(self._h, n_steps), "prepare_steps")

    def profile_reorder(self, reps=3):
        """Milliseconds that `reps` back-to-back reorders of every colony take."""
        ms = C.c_double()
        self._check(self._L.slime_ensemble_profile_reorder(self._h, reps, C.byref(ms)), "profile_reorder")
        return ms.value

    def sync(self):
        self._check(self._L.slime_ensemble_sync(self._h), "sync")

    def stream_ptr(self):
        s = C.c_void_p()
        self._check(self._L.slime_ensemble_get_stream(self._h, C.byref(s)), "get_stream")
        return s.value or 0

    def autotune(self, reps=5):
        self._check(self._L.slime_ensemble_autotune(self._h, reps), "autotune")

    def set_engine(self, engine, lane_agent_shape=13, lane_trail_tile=8, lanes=0):
        """Pick the stepping engine by hand (slime_ensemble_set_engine):
        ENSEMBLE_COOPERATIVE or ENSEMBLE_LANES with its agent shape, trail
        tile and number of lanes (0: one per colony, at most 64)."""
        self._check(self._L.slime_ensemble_set_engine(self._h, engine, lane_agent_shape, lane_trail_tile, lanes),
                    "set_engine")

    def set_shape(self, strip_rows=16, blocks_per_sm=0, agents_per_thread=4):
        """Pick the cooperative step's launch shape by hand (slime_ensemble_set_shape)."""
        self._check(self._L.slime_ensemble_set_shape(self._h, strip_rows, blocks_per_sm, agents_per_thread),
                    "set_shape")

    def selftest_barrier_timeout(self):
        """Make the grid barrier's bounded wait run out; returns the status
        (SLIME_ERR_DEVICE_TIMEOUT = -5 when detected and cleared)."""
        return self._L.slime_ensemble_selftest_barrier_timeout(self._h)

    def launch_count(self):
        v = C.c_uint64()
        self._check(self._L.slime_ensemble_launch_count(self._h, C.byref(v)), "launch_count")
        return v.value

    def info(self):
        i = SlimeEnsembleInfo()
        self._check(self._L.slime_ensemble_get_info(self._h, C.byref(i)), "get_info")
        return i
