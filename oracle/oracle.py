"""ctypes loader for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It wraps oracle/_build/libtmoracle.so (built by `make -C oracle`)
and, where present, the reference harness libraries in oracle/_ref/.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libtmoracle.so")

REM_EULER_EXACT, REM_RK4 = 0, 1
SAMPLER_EXACT, SAMPLER_REF_GAUSS100, SAMPLER_OFF = 0, 1, 2


class DPParams(C.Structure):
    _fields_ = [("a_start", C.c_double), ("a_step", C.c_double), ("b", C.c_double), ("c", C.c_double),
                ("D", C.c_double), ("sigma", C.c_double), ("dt", C.c_double), ("dx", C.c_double),
                ("clamp_lo", C.c_double), ("clamp_eps", C.c_double),
                ("remainder", C.c_int), ("sampler", C.c_int)]


class RKParams(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("R", "alpha", "k2", "W0", "gmax", "k1", "c", "d", "rW",
                                          "DP", "DW", "DO", "sigma", "dt", "dx", "clamp_lo", "clamp_eps")] + \
               [("sampler", C.c_int)]


class DornicConsts(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("beta", "lambda_", "expbdt", "pm", "inv_lambda", "mean_a1", "mean_a2")]


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        u32p = C.POINTER(C.c_uint32)
        dp = C.POINTER(C.c_double)
        fp = C.POINTER(C.c_float)
        i64p = C.POINTER(C.c_int64)
        L.tmo_philox4x32_10.argtypes = [u32p, u32p, u32p]
        for nm, t in (("f64", C.c_double), ("f32", C.c_float)):
            for fn in ("log", "exp", "log1p", "negexpm1", "inv_sqrt"):
                f = getattr(L, f"tmo_{fn}_{nm}")
                f.argtypes = [t]
                f.restype = t
            ptr = dp if nm == "f64" else fp
            for fn in ("poisson", "gamma"):
                getattr(L, f"tmo_sample_{fn}_{nm}").argtypes = [t, C.c_uint64, C.c_int64, C.c_int, C.c_int64, ptr, u32p]
            getattr(L, f"tmo_sample_normal_{nm}").argtypes = [C.c_uint64, C.c_int64, C.c_int64, ptr]
            getattr(L, f"tmo_sample_dornic_{nm}").argtypes = [t, t, t, C.c_uint64, C.c_int64, C.c_int, C.c_int64, ptr, u32p]
            getattr(L, f"tmo_dp_step_{nm}").argtypes = [C.POINTER(DPParams), C.c_int, C.c_uint64, C.c_int64, ptr, ptr, u32p]
            getattr(L, f"tmo_dp_step_sb_{nm}").argtypes = [C.POINTER(DPParams), C.c_int, C.c_uint64, C.c_int64, ptr, ptr,
                                                           u32p, ptr]
            getattr(L, f"tmo_rk_step_{nm}").argtypes = [C.POINTER(RKParams), C.c_int, C.c_uint64, C.c_int64, ptr, ptr, u32p]
            getattr(L, f"tmo_rk_det_step_{nm}").argtypes = [C.POINTER(RKParams), C.c_int, ptr, ptr]
            getattr(L, f"tmo_dp_det_step_{nm}").argtypes = [C.c_double] * 6 + [C.c_int, C.c_int, C.c_int, ptr, ptr]
            getattr(L, f"tmo_dp_remainder_{nm}").argtypes = [C.POINTER(DPParams), C.c_int64, ptr, ptr]
            getattr(L, f"tmo_rk_remainder_{nm}").argtypes = [C.POINTER(RKParams), C.c_int, ptr, ptr]
            getattr(L, f"tmo_observe_{nm}").argtypes = [ptr, C.c_int64, dp, dp]
            getattr(L, f"tmo_dp_run_{nm}").argtypes = [C.POINTER(DPParams), C.c_int, C.c_uint64, ptr, C.c_int64, i64p,
                                                       C.c_int, dp, dp, ptr, u32p]
            getattr(L, f"tmo_rk_run_{nm}").argtypes = [C.POINTER(RKParams), C.c_int, C.c_uint64, ptr, C.c_int64, i64p,
                                                       C.c_int, dp, dp, ptr, u32p]
        L.tmo_fke_advdiff_f64.argtypes = [C.c_int, dp, dp, dp, dp, C.c_double, C.c_double, dp, C.c_int, dp, C.c_int,
                                          dp]
        L.tmo_set_sampler_cap.argtypes = [C.c_int]
        L.tmo_dornic_consts_compute.argtypes = [C.c_double] * 5 + [C.POINTER(DornicConsts)]
        L.tmo_dp_batch_run_f32.argtypes = [C.POINTER(DPParams), C.POINTER(C.c_int), C.POINTER(C.c_uint64),
                                           C.POINTER(fp), C.c_int, C.c_int64, C.c_int]
        L.tmo_dp_batch_run_f64.argtypes = [C.POINTER(DPParams), C.POINTER(C.c_int), C.POINTER(C.c_uint64),
                                           C.POINTER(dp), C.c_int, C.c_int64, C.c_int]
        _lib = L
    return _lib


def _ptr(a):
    if a.dtype == np.float64:
        return a.ctypes.data_as(C.POINTER(C.c_double))
    if a.dtype == np.float32:
        return a.ctypes.data_as(C.POINTER(C.c_float))
    if a.dtype == np.int64:
        return a.ctypes.data_as(C.POINTER(C.c_int64))
    if a.dtype == np.uint32:
        return a.ctypes.data_as(C.POINTER(C.c_uint32))
    raise TypeError(a.dtype)


def _sfx(dtype):
    return "f64" if np.dtype(dtype) == np.float64 else "f32"


def set_sampler_cap(cap=64):
    """Attempts of every rejection loop (64 by default; 1 matches TM_PROBE_SAMPLER_CAP1)."""
    lib().tmo_set_sampler_cap(int(cap))


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32).copy()
    k = np.asarray(key, dtype=np.uint32).copy()
    o = np.zeros(4, np.uint32)
    lib().tmo_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


def scalar_fn(name, x, dtype=np.float64):
    return getattr(lib(), f"tmo_{name}_{_sfx(dtype)}")(x)


def sample(kind, n, seed=0, step=0, sampler=SAMPLER_EXACT, dtype=np.float64, **kw):
    out = np.zeros(n, dtype)
    st = np.zeros(1, np.uint32)
    L = lib()
    s = _sfx(dtype)
    if kind == "poisson":
        getattr(L, f"tmo_sample_poisson_{s}")(kw["m"], seed, step, sampler, n, _ptr(out), _ptr(st))
    elif kind == "gamma":
        getattr(L, f"tmo_sample_gamma_{s}")(kw["k"], seed, step, sampler, n, _ptr(out), _ptr(st))
    elif kind == "normal":
        getattr(L, f"tmo_sample_normal_{s}")(seed, step, n, _ptr(out))
    elif kind == "dornic":
        getattr(L, f"tmo_sample_dornic_{s}")(kw["m"], kw["mu1"], kw["inv_lambda"], seed, step, sampler, n,
                                             _ptr(out), _ptr(st))
    else:
        raise ValueError(kind)
    return out, int(st[0])


def dornic_consts(lin, D, sigma, dt, dx):
    o = DornicConsts()
    lib().tmo_dornic_consts_compute(lin, D, sigma, dt, dx, C.byref(o))
    return {n: getattr(o, n) for n, _ in DornicConsts._fields_}


def dp_params(a=0.72, a_end=None, n_steps=1, b=2.0, c=0.0, D=1.0, sigma=1.0, dt=0.1, dx=1.0,
              clamp_lo=0.0, clamp_eps=0.0, remainder=REM_EULER_EXACT, sampler=SAMPLER_EXACT):
    a_step = 0.0 if a_end is None else (a_end - a) / float(n_steps)
    return DPParams(a, a_step, b, c, D, sigma, dt, dx, clamp_lo, clamp_eps, remainder, sampler)


def rk_params(R=0.9, alpha=0.2, k2=5.0, W0=0.2, gmax=0.05, k1=5.0, c=10.0, d=0.25, rW=0.2,
              DP=0.1, DW=0.1, DO=100.0, sigma=0.5, dt=1e-3, dx=1.0, clamp_lo=0.0, clamp_eps=1e-10,
              sampler=SAMPLER_REF_GAUSS100):
    return RKParams(R, alpha, k2, W0, gmax, k1, c, d, rW, DP, DW, DO, sigma, dt, dx, clamp_lo, clamp_eps, sampler)


def dp_step(p, rho, seed, step):
    rho = np.ascontiguousarray(rho)
    L = rho.shape[0]
    out = np.empty_like(rho)
    st = np.zeros(1, np.uint32)
    getattr(lib(), f"tmo_dp_step_{_sfx(rho.dtype)}")(C.byref(p), L, seed, step, _ptr(rho), _ptr(out), _ptr(st))
    return out, int(st[0])


def dp_step_sb(p, rho, seed, step, site_b):
    rho = np.ascontiguousarray(rho)
    sb = np.ascontiguousarray(site_b, dtype=rho.dtype)
    out = np.empty_like(rho)
    st = np.zeros(1, np.uint32)
    getattr(lib(), f"tmo_dp_step_sb_{_sfx(rho.dtype)}")(C.byref(p), rho.shape[0], seed, step, _ptr(rho), _ptr(out),
                                                          _ptr(st), _ptr(sb))
    return out, int(st[0])


def rk_step(p, fields, seed, step):
    fields = np.ascontiguousarray(fields)
    L = fields.shape[1]
    out = np.empty_like(fields)
    st = np.zeros(1, np.uint32)
    getattr(lib(), f"tmo_rk_step_{_sfx(fields.dtype)}")(C.byref(p), L, seed, step, _ptr(fields), _ptr(out), _ptr(st))
    return out, int(st[0])


def rk_det_step(p, fields):
    fields = np.ascontiguousarray(fields)
    out = np.empty_like(fields)
    getattr(lib(), f"tmo_rk_det_step_{_sfx(fields.dtype)}")(C.byref(p), fields.shape[1], _ptr(fields), _ptr(out))
    return out


def dp_remainder(p, rho):
    rho = np.ascontiguousarray(rho)
    out = np.empty_like(rho)
    getattr(lib(), f"tmo_dp_remainder_{_sfx(rho.dtype)}")(C.byref(p), rho.size, _ptr(rho), _ptr(out))
    return out


def rk_remainder(p, fields):
    fields = np.ascontiguousarray(fields)
    out = np.empty_like(fields)
    getattr(lib(), f"tmo_rk_remainder_{_sfx(fields.dtype)}")(C.byref(p), fields.shape[1], _ptr(fields), _ptr(out))
    return out


def dp_det_step(rho, a, b, c, D, dt, dx, stencil=5, integrator=1):
    rho = np.ascontiguousarray(rho)
    out = np.empty_like(rho)
    rc = getattr(lib(), f"tmo_dp_det_step_{_sfx(rho.dtype)}")(a, b, c, D, dt, dx, stencil, integrator,
                                                                rho.shape[0], _ptr(rho), _ptr(out))
    assert rc == 0
    return out


def dp_run(p, rho0, seed, n_steps, meas_steps):
    rho0 = np.ascontiguousarray(rho0)
    ms = np.ascontiguousarray(meas_steps, dtype=np.int64)
    mean = np.zeros(len(ms)); act = np.zeros(len(ms))
    fin = np.empty_like(rho0)
    st = np.zeros(1, np.uint32)
    getattr(lib(), f"tmo_dp_run_{_sfx(rho0.dtype)}")(C.byref(p), rho0.shape[0], seed, _ptr(rho0), n_steps, _ptr(ms),
                                                       len(ms), _ptr(mean), _ptr(act), _ptr(fin), _ptr(st))
    return mean, act, fin, int(st[0])


def rk_run(p, f0, seed, n_steps, meas_steps):
    f0 = np.ascontiguousarray(f0)
    ms = np.ascontiguousarray(meas_steps, dtype=np.int64)
    mean = np.zeros((len(ms), 3)); act = np.zeros(len(ms))
    fin = np.empty_like(f0)
    st = np.zeros(1, np.uint32)
    getattr(lib(), f"tmo_rk_run_{_sfx(f0.dtype)}")(C.byref(p), f0.shape[1], seed, _ptr(f0), n_steps, _ptr(ms), len(ms),
                                                     _ptr(mean), _ptr(act), _ptr(fin), _ptr(st))
    return mean, act, fin, int(st[0])


def dp_batch_run(params, Ls, seeds, fields, n_steps, n_threads=0):
    """Run independent DP instances on host threads (FP32 or FP64 by the fields'
    dtype, all alike); fields are updated in place."""
    n = len(Ls)
    P = (DPParams * n)(*params)
    Larr = (C.c_int * n)(*Ls)
    S = (C.c_uint64 * n)(*seeds)
    f64 = fields[0].dtype == np.float64
    ptrs = (C.POINTER(C.c_double if f64 else C.c_float) * n)(*[_ptr(f) for f in fields])
    fn = lib().tmo_dp_batch_run_f64 if f64 else lib().tmo_dp_batch_run_f32
    rc = fn(P, Larr, S, ptrs, n, n_steps, n_threads)
    assert rc == 0


def dp_batch_run_f32(params, Ls, seeds, fields, n_steps, n_threads=0):
    """Run independent FP32 DP instances on host threads; fields are updated in place."""
    dp_batch_run(params, Ls, seeds, fields, n_steps, n_threads)


_scatter = None


def fke_scatter_lib():
    """libtmo_fke_scatter.so: the reference's GPU scatter (updateMovement) restated,
    for same-box comparisons with the library's gather (tmo_fke_scatter_f64)."""
    global _scatter
    if _scatter is None:
        path = os.path.join(HERE, "_build", "libtmo_fke_scatter.so")
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.tmo_fke_scatter_f64.argtypes = [vp, vp, vp, vp, C.c_int, C.c_double, C.c_double, vp, C.c_int, vp, C.c_int,
                                          vp, vp]
        L.tmo_fke_scatter_f64.restype = C.c_int
        _scatter = L
    return _scatter


def fke_advdiff(rho, gamma, vx, vy, pref, gD, gV, eps=1e-10):
    L = int(round(np.sqrt(rho.size)))
    a = [np.ascontiguousarray(x, np.float64).ravel() for x in (rho, gamma, vx, vy)]
    gD = np.ascontiguousarray(gD, np.float64)
    gV = np.ascontiguousarray(gV, np.float64)
    out = np.zeros(L * L)
    lib().tmo_fke_advdiff_f64(L, _ptr(a[0]), _ptr(a[1]), _ptr(a[2]), _ptr(a[3]), pref, eps, _ptr(gD), len(gD) - 1,
                              _ptr(gV), len(gV) - 1, _ptr(out))
    return out
