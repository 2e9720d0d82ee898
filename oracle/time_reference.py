"""Time the reference's own DP integrator against the CPU restatement on one core
and on all cores (TEST INFRASTRUCTURE ONLY; needs `make -C oracle ref ref-perf`, so
the reference checkout).  Workload: L = 256, a = 0.53, b = 2, D = 1, sigma = 1,
dt = 0.1, 50 steps from rho0 = 1 + U(-0.01, 0.01); one replicate per core, and on
all cores one value of a per thread (the reference's parallel model) against the
port's OpenMP over instances.

    python oracle/time_reference.py      # median of five interleaved runs per leg
"""
import ctypes as C
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# run as a script, the oracle directory itself is first on the path: put the repository first
sys.path[:] = [os.path.dirname(HERE)] + [q for q in sys.path if os.path.abspath(q or ".") != HERE]

from oracle import oracle as o  # noqa: E402

L, STEPS, A = 256, 50, 0.53


def reference_rate(libname):
    dp = C.POINTER(C.c_double)
    lib = C.CDLL(os.path.join(HERE, "_ref", libname))
    lib.ref_percolation_dornic.argtypes = [dp, C.c_int, dp] + [C.c_double] * 7 + [C.c_int, C.c_int, dp, C.c_int]
    rho0 = 1 + np.random.default_rng(0).uniform(-0.01, 0.01, L * L)
    tm = np.array([2.0, 3.0, 5.0])
    rows = np.zeros((1000, 8))
    t0 = time.perf_counter()
    lib.ref_percolation_dornic(tm.ctypes.data_as(dp), len(tm), rho0.ctypes.data_as(dp), 5.0, A, 2.0, 1.0, 1.0, 0.1,
                               1.0, 1, L, rows.ctypes.data_as(dp), 1000)
    return L * L * STEPS / (time.perf_counter() - t0)


def reference_rate_all(libname, threads):
    dp = C.POINTER(C.c_double)
    lib = C.CDLL(os.path.join(HERE, "_ref", libname))
    lib.ref_percolation_dornic_par.restype = C.c_double
    lib.ref_percolation_dornic_par.argtypes = [dp, C.c_int, dp, C.c_double, dp, C.c_int] + [C.c_double] * 5 + \
        [C.c_int, C.c_int]
    rho0 = 1 + np.random.default_rng(0).uniform(-0.01, 0.01, L * L)
    tm = np.array([2.0, 3.0, 5.0])
    avs = np.linspace(A - 0.01, A + 0.01, threads)
    sec = lib.ref_percolation_dornic_par(tm.ctypes.data_as(dp), len(tm), rho0.ctypes.data_as(dp), 5.0,
                                         avs.ctypes.data_as(dp), threads, 2.0, 1.0, 1.0, 0.1, 1.0, L, threads)
    return threads * L * L * STEPS / sec


def port_rate_all(threads):
    rho = (1 + np.random.default_rng(0).uniform(-0.01, 0.01, (L, L))).astype(np.float32)
    avs = np.linspace(A - 0.01, A + 0.01, threads)
    fields = [rho.copy() for _ in range(threads)]
    t0 = time.perf_counter()
    o.dp_batch_run([o.dp_params(a=float(a)) for a in avs], [L] * threads, list(range(threads)), fields, STEPS,
                   threads)
    return threads * L * L * STEPS / (time.perf_counter() - t0)


def port_rate(fp32):
    rho = 1 + np.random.default_rng(0).uniform(-0.01, 0.01, (L, L))
    t0 = time.perf_counter()
    if fp32:
        o.dp_batch_run_f32([o.dp_params(a=A)], [L], [1], [rho.astype(np.float32)], STEPS, 1)
    else:
        o.dp_run(o.dp_params(a=A), rho, 1, STEPS, [STEPS])
    return L * L * STEPS / (time.perf_counter() - t0)


def main(reps=5):
    o.build()
    legs = {}
    for name in ("libref_dp_o3.so", "libref_dp.so"):
        if os.path.exists(os.path.join(HERE, "_ref", name)):
            legs["reference " + name] = lambda n=name: reference_rate(n)
    legs["oracle FP64"] = lambda: port_rate(False)
    legs["oracle FP32 batch, 1 thread"] = lambda: port_rate(True)
    n = os.cpu_count() or 1
    for name in ("libref_dp_o3.so", "libref_dp.so"):
        if os.path.exists(os.path.join(HERE, "_ref", name)):
            legs[f"reference {name}, {n} threads (total)"] = lambda nm=name: reference_rate_all(nm, n)
    legs[f"oracle FP32 batch, {n} threads (total)"] = lambda: port_rate_all(n)
    rates = {k: [] for k in legs}
    for _ in range(reps):              # interleaved, so drifts of a shared machine hit every leg alike
        for k, f in legs.items():
            rates[k].append(f())
    for k, v in rates.items():
        print(f"{k:48s} median {np.median(v):.3g} site-updates/s  (runs: {', '.join('%.3g' % x for x in v)})")


if __name__ == "__main__":
    main()
