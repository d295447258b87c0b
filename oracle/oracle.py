"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the checker or the timed CPU baseline.
Pinned against a mechanical C++ translation of the reference's own shader
(oracle/wgsl/, tests/test_reference_pin.py; see slime_oracle.cpp).
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_lib = None


def _params_type():
    sys.path.insert(0, os.path.join(HERE, "..", "slime-mold_gb300"))
    from slime_gb300._abi import SlimeParams
    return SlimeParams


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        SP = C.POINTER(_params_type())
        f32, f64, u32 = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        L.oracle_agents_pass.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_uint64, f32, u32, f32, u32, C.c_int]
        L.oracle_agents_pass.restype = None
        L.oracle_trail_pass.argtypes = [SP, C.c_uint32, C.c_uint32, f32, u32, f32, C.c_int]
        L.oracle_trail_pass.restype = None
        L.oracle_trail_pass_f64.argtypes = [SP, C.c_uint32, C.c_uint32, f64, u32, f64, C.c_int]
        L.oracle_trail_pass_f64.restype = None
        L.oracle_run.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_uint64, f32, f32, C.c_uint32, u32, C.c_int]
        L.oracle_run.restype = None
        L.oracle_chain_loss_f64.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double, f64,
                                            u32, C.c_uint32, f64, f64, C.c_int]
        L.oracle_chain_loss_f64.restype = C.c_double
        L.oracle_chain_adjoint_f64.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                               f64, u32, C.c_uint32, f64, f64, f64, f64, C.c_int]
        L.oracle_chain_adjoint_f64.restype = C.c_double
        L.oracle_chain_adjoint_f64_along.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_double, C.c_double, C.c_double,
                                                     f32, u32, C.c_uint32, f64, f64, f64, C.c_int]
        L.oracle_chain_adjoint_f64_along.restype = C.c_double
        L.oracle_colorize.argtypes = [C.c_uint32, C.c_uint32, f32, C.POINTER(C.c_uint8), C.c_uint32, C.c_uint32,
                                      C.POINTER(C.c_uint8)]
        L.oracle_colorize.restype = None
        L.oracle_num_threads.restype = C.c_int
        L.oracle_sincos.argtypes = [f32, C.c_uint64, f32, f32]
        L.oracle_ph_window_mismatches.argtypes = [C.c_uint32, C.c_uint32]
        L.oracle_sample.argtypes = [f32, C.c_uint32, C.c_uint32, f32, f32, C.c_uint64, f32]
        L.oracle_sample.restype = None
        L.oracle_sense.argtypes = [SP, C.c_uint32, C.c_uint32, C.c_uint64, f32, f32, f32]
        L.oracle_sense.restype = None
        L.oracle_dispatch_visits.argtypes = [C.c_uint64, C.POINTER(C.c_uint64), C.c_uint64, u32]
        L.oracle_dispatch_visits.restype = None
        L.oracle_ph_window_mismatches.restype = C.c_uint64
        L.oracle_ph_finish_mismatches.argtypes = [C.c_uint32, C.c_uint32]
        L.oracle_ph_finish_mismatches.restype = C.c_uint64
        L.oracle_jitter_hash.argtypes = [C.POINTER(C.c_int32), f32, f32, C.c_uint64, f32]
        L.oracle_uniform01.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, f32]
        L.oracle_gauss_weights.argtypes = [C.c_float, C.c_float, f32]
        L.oracle_gauss_weights.restype = C.c_int
        _lib = L
    return _lib


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


def agents_pass(params, W, H, agents, trail, ids=None, counts=None, threads=0):
    """One agent pass; updates `agents` (n,4 float32) in place and returns the
    deposit counts (H, W uint32)."""
    assert agents.dtype == np.float32 and agents.flags.c_contiguous
    tr = np.ascontiguousarray(trail, np.float32).reshape(-1)
    cnt = counts if counts is not None else np.zeros(W * H, np.uint32)
    idp = _p(np.ascontiguousarray(ids, np.uint32), C.c_uint32) if ids is not None else None
    lib().oracle_agents_pass(C.byref(params), W, H, agents.shape[0], _p(agents, C.c_float), idp,
                             _p(tr, C.c_float), _p(cnt, C.c_uint32), threads)
    return cnt.reshape(H, W)


def trail_pass(params, W, H, trail, counts, threads=0):
    tr = np.ascontiguousarray(trail, np.float32).reshape(-1)
    cn = np.ascontiguousarray(counts, np.uint32).reshape(-1)
    out = np.empty(W * H, np.float32)
    lib().oracle_trail_pass(C.byref(params), W, H, _p(tr, C.c_float), _p(cn, C.c_uint32), _p(out, C.c_float),
                            threads)
    return out.reshape(H, W)


def trail_pass_f64(params, W, H, trail, counts, threads=0):
    tr = np.ascontiguousarray(trail, np.float64).reshape(-1)
    cn = np.ascontiguousarray(counts, np.uint32).reshape(-1)
    out = np.empty(W * H, np.float64)
    lib().oracle_trail_pass_f64(C.byref(params), W, H, _p(tr, C.c_double), _p(cn, C.c_uint32),
                                _p(out, C.c_double), threads)
    return out.reshape(H, W)


def run(params, W, H, agents, trail, steps, record_counts=False, threads=0):
    """`steps` full steps in place; returns per-step counts if asked."""
    assert agents.dtype == np.float32 and agents.flags.c_contiguous
    assert trail.dtype == np.float32 and trail.flags.c_contiguous
    counts = np.zeros((steps, H, W), np.uint32) if record_counts else None
    lib().oracle_run(C.byref(params), W, H, agents.shape[0], _p(agents, C.c_float), _p(trail, C.c_float), steps,
                     _p(counts, C.c_uint32) if counts is not None else None, threads)
    return counts


def chain_loss_f64(params, W, H, decay, rate, dep, trail0, counts, target, threads=0):
    t0 = np.ascontiguousarray(trail0, np.float64).reshape(-1)
    cn = np.ascontiguousarray(counts, np.uint32)
    tg = np.ascontiguousarray(target, np.float64).reshape(-1)
    fin = np.empty(W * H, np.float64)
    loss = lib().oracle_chain_loss_f64(C.byref(params), W, H, decay, rate, dep, _p(t0, C.c_double),
                                       _p(cn, C.c_uint32), cn.shape[0], _p(tg, C.c_double), _p(fin, C.c_double),
                                       threads)
    return loss, fin.reshape(H, W)


def chain_adjoint_f64(params, W, H, decay, rate, dep, trail0, counts, target=None, g_final=None, threads=0):
    t0 = np.ascontiguousarray(trail0, np.float64).reshape(-1)
    cn = np.ascontiguousarray(counts, np.uint32)
    tg = np.ascontiguousarray(target, np.float64).reshape(-1) if target is not None else None
    gf = np.ascontiguousarray(g_final, np.float64).reshape(-1) if g_final is not None else None
    d0 = np.empty(W * H, np.float64)
    grads = np.zeros(3, np.float64)
    loss = lib().oracle_chain_adjoint_f64(C.byref(params), W, H, decay, rate, dep, _p(t0, C.c_double),
                                          _p(cn, C.c_uint32), cn.shape[0],
                                          _p(tg, C.c_double) if tg is not None else None,
                                          _p(gf, C.c_double) if gf is not None else None,
                                          _p(d0, C.c_double), _p(grads, C.c_double), threads)
    return loss, grads, d0.reshape(H, W)


def chain_adjoint_f64_along(params, W, H, decay, rate, dep, trails, counts, g_final, threads=0):
    """The binary64 adjoint along given trails T_0..T_steps (steps + 1 grids,
    binary32), e.g. those of the binary32 forward a GPU backward differentiates."""
    tr = np.ascontiguousarray(trails, np.float32)
    cn = np.ascontiguousarray(counts, np.uint32)
    assert tr.shape[0] == cn.shape[0] + 1
    gf = np.ascontiguousarray(g_final, np.float64).reshape(-1)
    d0 = np.empty(W * H, np.float64)
    grads = np.zeros(3, np.float64)
    lib().oracle_chain_adjoint_f64_along(C.byref(params), W, H, decay, rate, dep, _p(tr, C.c_float),
                                         _p(cn, C.c_uint32), cn.shape[0], _p(gf, C.c_double), _p(d0, C.c_double),
                                         _p(grads, C.c_double), threads)
    return grads, d0.reshape(H, W)


def colorize(W, H, trail, lut768, tw, th):
    tr = np.ascontiguousarray(trail, np.float32).reshape(-1)
    lut = np.ascontiguousarray(lut768, np.uint8).reshape(-1)
    out = np.empty((th, tw, 4), np.uint8)
    lib().oracle_colorize(W, H, _p(tr, C.c_float), _p(lut, C.c_uint8), tw, th, _p(out, C.c_uint8))
    return out


def sample(trail, px, py):
    """sample_trail_map (compute.wgsl:7-29) at positions (px, py)."""
    t = np.ascontiguousarray(trail, np.float32)
    H, W = t.shape
    x = np.ascontiguousarray(px, np.float32)
    y = np.ascontiguousarray(py, np.float32)
    out = np.empty(x.size, np.float32)
    lib().oracle_sample(_p(t, C.c_float), W, H, _p(x, C.c_float), _p(y, C.c_float), x.size, _p(out, C.c_float))
    return out


def sense(params, W, H, agents, trail):
    """The (left, right, centre) sensor samples of each agent (compute.wgsl:74-95)."""
    a = np.ascontiguousarray(agents, np.float32)
    t = np.ascontiguousarray(trail, np.float32).reshape(-1)
    out = np.empty((a.shape[0], 3), np.float32)
    lib().oracle_sense(C.byref(params), W, H, a.shape[0], _p(a, C.c_float), _p(t, C.c_float), _p(out, C.c_float))
    return out


def dispatch_visits(n, index):
    """How many invocations of the reference's agent dispatch update each of
    `index` among n agents (slm_dispatch_visits)."""
    idx = np.ascontiguousarray(index, np.uint64).reshape(-1)
    out = np.empty(idx.size, np.uint32)
    lib().oracle_dispatch_visits(n, _p(idx, C.c_uint64), idx.size, _p(out, C.c_uint32))
    return out


def ph_window_mismatches(e_lo=139, e_hi=170):
    """Inputs with biased exponent e_lo..e_hi on which the fixed-window and the
    table-driven Payne-Hanek reductions disagree (0 expected)."""
    return int(lib().oracle_ph_window_mismatches(e_lo, e_hi))


def ph_finish_mismatches(e_lo=139, e_hi=254):
    """Inputs with biased exponent e_lo..e_hi on which the 32-bit-word
    Payne-Hanek tail and its 64-bit statement disagree (0 expected)."""
    return int(lib().oracle_ph_finish_mismatches(e_lo, e_hi))


def sincos(x):
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().oracle_sincos(_p(x, C.c_float), x.size, _p(s, C.c_float), _p(c, C.c_float))
    return s, c


def jitter_hash(index, x, y):
    i = np.ascontiguousarray(index, np.int32).reshape(-1)
    x = np.ascontiguousarray(x, np.float32).reshape(-1)
    y = np.ascontiguousarray(y, np.float32).reshape(-1)
    out = np.empty(i.size, np.float32)
    lib().oracle_jitter_hash(_p(i, C.c_int32), _p(x, C.c_float), _p(y, C.c_float), i.size, _p(out, C.c_float))
    return out


def uniform01(seed, n, field):
    out = np.empty(n, np.float32)
    lib().oracle_uniform01(seed, n, field, _p(out, C.c_float))
    return out


def gauss_weights(radius, sigma):
    w = np.zeros(2 * 8 + 1, np.float32)
    R = lib().oracle_gauss_weights(radius, sigma, _p(w, C.c_float))
    return None if R < 0 else w[: 2 * R + 1]


def num_threads():
    return lib().oracle_num_threads()
