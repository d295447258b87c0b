"""ctypes declarations of include/slime.h.

The structures mirror the C layouts field for field; SlimeParams' first 14
fields are the reference's SimSizeUniform (src/main.rs:29-46).
"""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(_HERE), "lib", "libslime_gb300.so")

SLIME_OK = 0
SLIME_ERR_INVALID_ARGUMENT = -1
SLIME_ERR_OUT_OF_MEMORY = -2
SLIME_ERR_CUDA = -3
SLIME_ERR_STATE = -4
SLIME_ERR_DEVICE_TIMEOUT = -5
SLIME_ERR_NO_DEVICE = -6

DECAY_REF_SUBTRACT = 0
DECAY_MULTIPLY = 1
BLUR_REF_BOX3 = 0
BLUR_GAUSS = 1
MAX_BLUR_RADIUS = 8
DISPATCH_EACH_AGENT = 0
DISPATCH_REFERENCE = 1
SENSOR_SHADER = 0
SENSOR_ROTATED = 1
ENSEMBLE_COOPERATIVE = 0
ENSEMBLE_LANES = 1


class SlimeParams(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("decay_factor", C.c_float),
        ("agent_jitter", C.c_float),
        ("agent_speed_min", C.c_float),
        ("agent_speed_max", C.c_float),
        ("agent_turn_speed", C.c_float),
        ("agent_sensor_angle", C.c_float),
        ("agent_sensor_distance", C.c_float),
        ("diffusion_rate", C.c_float),
        ("pheromone_deposition_amount", C.c_float),
        ("blur_radius", C.c_float),
        ("blur_sigma", C.c_float),
        ("_pad", C.c_uint32),
        ("time_step", C.c_float),
        ("decay_mode", C.c_uint32),
        ("blur_mode", C.c_uint32),
        ("dispatch_mode", C.c_uint32),
        ("sensor_mode", C.c_uint32),
        ("_pad2", C.c_uint32),
    ]

    def copy(self):
        p = SlimeParams()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(SlimeParams))
        return p

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SlimeSettings(C.Structure):
    _fields_ = [
        ("agent_count", C.c_uint64),
        ("agent_jitter", C.c_float),
        ("agent_possible_starting_headings_start", C.c_float),
        ("agent_possible_starting_headings_end", C.c_float),
        ("agent_speed_max", C.c_float),
        ("agent_speed_min", C.c_float),
        ("agent_turn_speed", C.c_float),
        ("pheromone_decay_factor", C.c_float),
        ("pheromone_diffusion_rate", C.c_float),
        ("pheromone_deposition_amount", C.c_float),
        ("window_fullscreen", C.c_uint32),
        ("window_height", C.c_uint32),
        ("window_width", C.c_uint32),
        ("agent_sensor_angle", C.c_float),
        ("agent_sensor_distance", C.c_float),
        ("blur_radius", C.c_float),
        ("blur_sigma", C.c_float),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SlimeOptions(C.Structure):
    _fields_ = [
        ("use_graphs", C.c_uint32),
        ("graph_chunk", C.c_uint32),
        ("reorder_every", C.c_uint32),
        ("reorder_cell_log2", C.c_uint32),
        ("l2_persist", C.c_uint32),
        ("trail_tile", C.c_uint32),
        ("agent_shape", C.c_uint32),
        ("exact_counts", C.c_uint32),
    ]


class SlimeInfo(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("n_agents", C.c_uint64),
        ("steps_done", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("trail_tile", C.c_uint32),
        ("reordered", C.c_uint32),
        ("agent_shape", C.c_uint32),
        ("trail_texture", C.c_uint32),
        ("l2_persist_bytes", C.c_uint64),
        ("l2_window_passes", C.c_uint32),
        ("_pad", C.c_uint32),
        ("reorders_done", C.c_uint64),
    ]


class SlimeEnsembleInfo(C.Structure):
    _fields_ = [
        ("n_colonies", C.c_uint32),
        ("graphs_in_use", C.c_uint32),
        ("steps_done", C.c_uint64),
        ("kernel_launches", C.c_uint64),
        ("total_agents", C.c_uint64),
        ("total_cells", C.c_uint64),
        ("grid_blocks", C.c_uint32),
        ("strip_rows", C.c_uint32),
        ("agents_per_thread", C.c_uint32),
        ("engine", C.c_uint32),
        ("lanes", C.c_uint32),
        ("lane_agent_shape", C.c_uint32),
        ("lane_trail_tile", C.c_uint32),
        ("marks_colonies", C.c_uint32),
    ]


class SlimeGrads(C.Structure):
    _fields_ = [
        ("d_decay_factor", C.c_double),
        ("d_diffusion_rate", C.c_double),
        ("d_deposition_amount", C.c_double),
        ("reserved", C.c_double),
    ]


P = C.c_void_p
F32P = C.POINTER(C.c_float)
U32P = C.POINTER(C.c_uint32)
U8P = C.POINTER(C.c_uint8)

# name -> (restype, argtypes), one entry per declaration in include/slime.h
SIGNATURES = {
    "slime_version": (C.c_char_p, []),
    "slime_status_string": (C.c_char_p, [C.c_int]),
    "slime_settings_default": (None, [C.POINTER(SlimeSettings)]),
    "slime_preset_count": (C.c_int, []),
    "slime_preset_get": (C.c_int, [C.c_int, C.POINTER(C.c_char_p), C.POINTER(SlimeSettings)]),
    "slime_preset_find": (C.c_int, [C.c_char_p, C.POINTER(SlimeSettings)]),
    "slime_params_from_settings": (None, [C.POINTER(SlimeSettings), C.c_uint32, C.c_uint32, C.POINTER(SlimeParams)]),
    "slime_settings_to_text": (C.c_int, [C.POINTER(SlimeSettings), C.c_char_p, C.c_size_t, C.POINTER(C.c_size_t)]),
    "slime_settings_from_text": (C.c_int, [C.c_char_p, C.POINTER(SlimeSettings), C.POINTER(C.c_int)]),
    "slime_settings_save": (C.c_int, [C.POINTER(SlimeSettings), C.c_char_p]),
    "slime_settings_load": (C.c_int, [C.c_char_p, C.POINTER(SlimeSettings), C.POINTER(C.c_int)]),
    "slime_create": (P, [C.c_uint32, C.c_uint32, C.c_uint64, C.POINTER(C.c_int)]),
    "slime_destroy": (None, [P]),
    "slime_last_error": (C.c_char_p, [P]),
    "slime_set_params": (C.c_int, [P, C.POINTER(SlimeParams)]),
    "slime_get_params": (C.c_int, [P, C.POINTER(SlimeParams)]),
    "slime_set_options": (C.c_int, [P, C.POINTER(SlimeOptions)]),
    "slime_get_options": (C.c_int, [P, C.POINTER(SlimeOptions)]),
    "slime_get_info": (C.c_int, [P, C.POINTER(SlimeInfo)]),
    "slime_upload_agents": (C.c_int, [P, F32P, C.c_uint64]),
    "slime_download_agents": (C.c_int, [P, F32P, C.c_uint64]),
    "slime_seed_agents": (C.c_int, [P, C.c_uint64, C.c_float, C.c_float]),
    "slime_reassign_speeds": (C.c_int, [P, C.c_uint64]),
    "slime_upload_trail": (C.c_int, [P, F32P, C.c_uint64]),
    "slime_download_trail": (C.c_int, [P, F32P, C.c_uint64]),
    "slime_clear_trail": (C.c_int, [P]),
    "slime_resize": (C.c_int, [P, C.c_uint32, C.c_uint32]),
    "slime_set_agent_count": (C.c_int, [P, C.c_uint64, C.c_uint64]),
    "slime_state_save": (C.c_int, [P, C.c_char_p]),
    "slime_state_load": (C.c_int, [P, C.c_char_p]),
    "slime_set_steps_done": (C.c_int, [P, C.c_uint64]),
    "slime_step": (C.c_int, [P, C.c_uint32]),
    "slime_prepare_steps": (C.c_int, [P, C.c_uint32]),
    "slime_sync": (C.c_int, [P]),
    "slime_get_stream": (C.c_int, [P, C.POINTER(C.c_void_p)]),
    "slime_download_deposit_counts": (C.c_int, [P, U32P, C.c_uint64]),
    "slime_download_trail_async": (C.c_int, [P, F32P, C.c_uint64]),
    "slime_wait_download": (C.c_int, [P]),
    "slime_reorder_agents": (C.c_int, [P]),
    "slime_profile_steps": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]),
    "slime_profile_reorder": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_double)]),
    "slime_autotune": (C.c_int, [P, C.c_uint32]),
    "slime_forward_record": (C.c_int, [P, C.c_uint32, C.c_uint32]),
    "slime_backward": (C.c_int, [P, F32P, C.POINTER(SlimeGrads), F32P]),
    "slime_ensemble_create": (P, [C.c_uint32, U32P, U32P, C.POINTER(C.c_uint64), C.POINTER(SlimeParams),
                                  C.POINTER(C.c_int)]),
    "slime_ensemble_destroy": (None, [P]),
    "slime_ensemble_last_error": (C.c_char_p, [P]),
    "slime_ensemble_set_params": (C.c_int, [P, C.c_uint32, C.POINTER(SlimeParams)]),
    "slime_ensemble_upload_agents": (C.c_int, [P, C.c_uint32, F32P, C.c_uint64]),
    "slime_ensemble_download_agents": (C.c_int, [P, C.c_uint32, F32P, C.c_uint64]),
    "slime_ensemble_seed_agents": (C.c_int, [P, C.c_uint32, C.c_uint64, C.c_float, C.c_float]),
    "slime_ensemble_upload_trail": (C.c_int, [P, C.c_uint32, F32P, C.c_uint64]),
    "slime_ensemble_download_trail": (C.c_int, [P, C.c_uint32, F32P, C.c_uint64]),
    "slime_ensemble_set_reorder": (C.c_int, [P, C.c_uint32, C.c_uint32]),
    "slime_ensemble_step": (C.c_int, [P, C.c_uint32]),
    "slime_ensemble_prepare_steps": (C.c_int, [P, C.c_uint32]),
    "slime_ensemble_profile_reorder": (C.c_int, [P, C.c_uint32, C.POINTER(C.c_double)]),
    "slime_ensemble_sync": (C.c_int, [P]),
    "slime_ensemble_get_stream": (C.c_int, [P, C.POINTER(C.c_void_p)]),
    "slime_ensemble_autotune": (C.c_int, [P, C.c_uint32]),
    "slime_ensemble_set_shape": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32]),
    "slime_ensemble_set_engine": (C.c_int, [P, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32]),
    "slime_ensemble_launch_count": (C.c_int, [P, C.POINTER(C.c_uint64)]),
    "slime_ensemble_get_info": (C.c_int, [P, C.POINTER(SlimeEnsembleInfo)]),
    "slime_ensemble_selftest_barrier_timeout": (C.c_int, [P]),
    "slime_colorize": (C.c_int, [P, U8P, C.c_uint32, C.c_uint32, U8P]),
    "slime_colorize_async": (C.c_int, [P, U8P, C.c_uint32, C.c_uint32, U8P]),
    "slime_step_noalloc": (C.c_int, [C.POINTER(SlimeParams), C.c_uint32, C.c_uint32, C.c_uint64, P, P, P, P, P, P,
                                     P]),
    "slime_step_noalloc_scratch": (C.c_int, [C.POINTER(SlimeParams), C.c_uint32, C.c_uint32, C.c_uint64, P, P, P,
                                             P, P, P, P, P]),
}

_lib = None


def load(path=None):
    """Load the CUDA library (raises if it has not been built: there is no
    CPU fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: build it with `python slime-mold_gb300/build.py` "
                           "(the simulation has no CPU fallback)")
    lib = C.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
