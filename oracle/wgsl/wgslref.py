"""ctypes binding of the translated reference shader (oracle/_ref/libwgslref.so).

TEST INFRASTRUCTURE: used by tests/test_reference_pin.py and
tests/golden/make_reference_golden.py to pin the oracle against the
reference's own src/compute.wgsl (translated by translate.py, run by
harness.cpp).  Available only where the reference's source tree is present;
`available()` says whether it is.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
import build_oracle  # noqa: E402

_lib = None


def _params_type():
    sys.path.insert(0, os.path.join(HERE, "..", "..", "slime-mold_gb300"))
    from slime_gb300._abi import SlimeParams
    return SlimeParams


def available():
    return os.path.exists(build_oracle.REF_WGSL)


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build_reference()
        if path is None:
            raise FileNotFoundError(f"the reference shader {build_oracle.REF_WGSL} is not present")
        L = C.CDLL(path)
        f32 = C.POINTER(C.c_float)
        SP = C.POINTER(_params_type())
        L.wref_sample.argtypes = [f32, C.c_uint32, C.c_uint32, f32, f32, C.c_uint64, f32]
        L.wref_agents.argtypes = [SP, f32, C.c_uint64, f32, C.c_int]
        L.wref_decay.argtypes = [SP, f32]
        L.wref_diffuse.argtypes = [SP, f32, f32]
        L.wref_sense.argtypes = [SP, f32, C.c_uint64, f32, f32]
        L.wref_agents_dispatch.argtypes = [SP, f32, C.c_uint64, f32]
        u8 = C.POINTER(C.c_uint8)
        L.wref_colorize.argtypes = [C.c_uint32, C.c_uint32, f32, u8, C.c_uint32, C.c_uint32, u8]
        L.wref_colorize.restype = None
        for f in (L.wref_sample, L.wref_agents, L.wref_decay, L.wref_diffuse, L.wref_sense, L.wref_agents_dispatch):
            f.restype = None
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def sample(trail, px, py):
    """sample_trail_map at positions (px, py)."""
    t = np.ascontiguousarray(trail, np.float32)
    H, W = t.shape
    x = np.ascontiguousarray(px, np.float32)
    y = np.ascontiguousarray(py, np.float32)
    out = np.empty(x.size, np.float32)
    lib().wref_sample(_p(t), W, H, _p(x), _p(y), x.size, _p(out))
    return out


def agents_pass(params, agents, trail):
    """`main` once per agent, sensing the trail as the pass found it; each
    deposit writes clamp(that value + dep, 0, 1) into the returned trail."""
    a = np.ascontiguousarray(agents, np.float32).copy()
    t = np.ascontiguousarray(trail, np.float32).copy()
    lib().wref_agents(C.byref(params), _p(a), a.shape[0], _p(t), 1)
    return a, t


def agents_pass_dispatch(params, agents, trail):
    """`main` over the reference's own dispatch grid (wx x wy workgroups of
    64, src/main.rs:1174-1178), agents and trail read as the pass found them;
    a deposit writes clamp(that value + dep, 0, 1)."""
    a = np.ascontiguousarray(agents, np.float32).copy()
    t = np.ascontiguousarray(trail, np.float32).copy()
    lib().wref_agents_dispatch(C.byref(params), _p(a), a.shape[0], _p(t))
    return a, t


def decay(params, trail):
    t = np.ascontiguousarray(trail, np.float32).copy()
    lib().wref_decay(C.byref(params), _p(t))
    return t


def diffuse(params, trail):
    t = np.ascontiguousarray(trail, np.float32)
    out = np.empty_like(t)
    lib().wref_diffuse(C.byref(params), _p(t), _p(out))
    return out


def sense(params, agents, trail):
    """The (left, right, centre) sensor samples `main` takes."""
    a = np.ascontiguousarray(agents, np.float32)
    t = np.ascontiguousarray(trail, np.float32)
    out = np.empty((a.shape[0], 3), np.float32)
    lib().wref_sense(C.byref(params), _p(a), a.shape[0], _p(t), _p(out))
    return out


def colorize(trail, lut768, tex_width, tex_height):
    """display.wgsl's `main` over a tex_width x tex_height RGBA8 image."""
    t = np.ascontiguousarray(trail, np.float32)
    H, W = t.shape
    lut = np.ascontiguousarray(lut768, np.uint8).reshape(-1)
    assert lut.size == 768
    out = np.zeros((tex_height, tex_width, 4), np.uint8)
    u8 = C.POINTER(C.c_uint8)
    lib().wref_colorize(W, H, _p(t), lut.ctypes.data_as(u8), tex_width, tex_height, out.ctypes.data_as(u8))
    return out


def frame(params, agents, trail):
    """The reference's frame (src/main.rs:1163-1235): the agent pass, then
    decay_trail, then diffuse_trail (read from the decayed trail)."""
    a, t = agents_pass(params, agents, trail)
    return a, diffuse(params, decay(params, t))
