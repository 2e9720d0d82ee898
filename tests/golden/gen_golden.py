"""Generate the golden fixtures in this folder from the reference's own code.

Needs the reference checkout and its harness libraries, built by
`make -C oracle ref REF_ROOT=<reference checkout>` (__graft_entry__.build()
runs it where the checkout exists).  The fixtures are committed; tests only
read them.

    python tests/golden/gen_golden.py

Fixtures
--------
ref_pins.npz       deterministic outputs of the reference's stage functions
                   (noise-off Rietkerk RK4, stochastic-remainder RK4s, the
                   4th-order noise-off DP RK4, logarithm10_time_bins).
ref_csv.npz        files written by the reference's own save_frame / save_prelimframe
                   (multiSPDP.cpp:1493-1643), byte for byte.
ref_fke.npz        the consumer species' FKE advection-diffusion (advdiff_FKE_MultiSp,
                   rietkerk_bjork_FKE.cpp:3614-3695) with its stencils.
ref_dp_ensemble.npz  per-replicate trajectories of percolationDornic_2D
                   (stochasticSPDP.cpp:940), one replicate per call.  The
                   reference seeds std::mt19937_64 from std::random_device, so
                   these draws are not reproducible; they are a fixed sample of
                   the reference's ensemble, compared statistically.
ref_spectrum.npz   radially averaged power spectra computed by the reference's own
                   gen_FFT_PowerSpectra (glow_up.py:632-847, run through
                   glow_up_harness.py) on frame files written by the reference's
                   save_frame; each case keeps the field as the estimator read it
                   (save_frame prints 6 significant digits), k and the power
                   (NaN where the reference leaves a bin empty).
ref_lnspace.npz    the reference's lnspace<int> (stochasticSPDP.cpp:281-301), which picks
                   the lattice sides of the stationary finite-size sweep.
ref_libstdcxx.npz  draws of the libstdc++ poisson_distribution / gamma_distribution
                   the reference's Dornic step constructs (stochasticSPDP.cpp:1055-1059),
                   from a seeded std::mt19937_64, alone and composed as the step's whole
                   draw Gamma(mu1 + Poisson(m)).

    python tests/golden/gen_golden.py --spectrum   # only ref_spectrum.npz (needs TM_REF_ROOT)
    python tests/golden/gen_golden.py --lnspace    # only ref_lnspace.npz
    python tests/golden/gen_golden.py --fke        # only ref_fke.npz
    python tests/golden/gen_golden.py --libstdcxx  # only ref_libstdcxx.npz
    python tests/golden/gen_golden.py --rk-ensemble  # only ref_rk_ensemble.npz

ref_rk_ensemble.npz  replicates of the reference's stochastic Rietkerk step (P-Dornic loop
                   with libstdc++ draws from one seeded std::mt19937_64 per replicate, the
                   reference's compiled RK4_Integrate_Stochastic_1Sp, the clamp) on one
                   16^2 start: per replicate the final mean P, W, O, the occupied P sites
                   and P at two sites, compared statistically with the GPU's ensemble.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(REPO, "oracle", "_ref")
dp = C.POINTER(C.c_double)


def _p(a):
    return a.ctypes.data_as(dp)


def load(names=("dp", "rietkerk", "multisp")):
    # the FKE harness is a -DSPB=2 build of the same sources as the -DSPB=1 one:
    # their header-defined globals clash, so it is loaded in its own process
    libs = {}
    for nm in names:
        path = os.path.join(REF, f"libref_{nm}.so")
        if not os.path.exists(path):
            sys.exit(f"missing {path}: run `make -C oracle ref` first")
        libs[nm] = C.CDLL(path)
    if "fke" in libs:
        ip = C.POINTER(C.c_int)
        libs["fke"].ref_fke_advdiff.argtypes = [dp, dp, dp, dp, C.c_int] + [C.c_double] * 5 + \
            [dp, dp, ip, dp, ip, dp, C.c_int]
        return libs
    d = libs["dp"]
    d.ref_percolation_dornic.argtypes = [dp, C.c_int, dp] + [C.c_double] * 7 + [C.c_int, C.c_int, dp, C.c_int]
    d.ref_perc_nodiff.argtypes = [dp, C.c_int, dp] + [C.c_double] * 6 + [C.c_int, dp, C.c_int]
    d.ref_rk4_first_order.argtypes = [dp, C.c_int] + [C.c_double] * 7
    d.ref_logarithm10_time_bins.argtypes = [C.c_double, C.c_double, dp, C.c_int]
    d.ref_libstdcxx_draws.argtypes = [C.c_int, C.c_double, C.c_ulonglong, C.c_int, dp]
    d.ref_libstdcxx_dornic.argtypes = [C.c_double, C.c_double, C.c_ulonglong, C.c_int, dp]
    if "rietkerk" not in libs:
        return libs
    r = libs["rietkerk"]
    r.ref_rk_det_steps.argtypes = [dp, C.c_int, C.c_int] + [C.c_double] * 14
    r.ref_rk_stoch_remainder.argtypes = [dp, C.c_int] + [C.c_double] * 12
    r.ref_rk_stoch_steps.argtypes = [dp, C.c_int, C.c_int, C.c_ulonglong] + [C.c_double] * 16
    libs["multisp"].ref_ms_rk4_remainder.argtypes = [dp, C.c_int, C.c_double, C.c_double, C.c_double]
    cs = C.c_char_p
    libs["multisp"].ref_save_frame.argtypes = [dp, C.c_int, cs, cs, C.c_double, C.c_int, cs]
    libs["multisp"].ref_save_prelim.argtypes = [dp, C.c_int, C.c_int, cs, cs, C.c_double, C.c_int, cs]
    return libs


# Rietkerk parameters of the 256^2 three-field workload (alpha, k2, W0, gmax, k1, c, d, rW, DP, DW, DO, sigma)
RK = dict(alpha=0.2, k2=5.0, W0=0.2, gmax=0.05, k1=5.0, c=10.0, d=0.25, rW=0.2, DP=0.1, DW=0.1, DO=100.0)


def pins(libs, rng):
    out = {}
    # 1) noise-off Rietkerk RK4 (f_2D + RK4_Integrate), L=12, 60 steps of dt=1e-3, and a
    #    larger dt for a stiffer comparison
    for tag, L, n, dt, R in (("rkdet_a", 12, 60, 1e-3, 0.9), ("rkdet_b", 9, 25, 2e-3, 1.2)):
        f0 = np.concatenate([rng.uniform(0, 1, L * L), 0.5 + rng.uniform(-0.1, 0.1, L * L),
                             1.0 + rng.uniform(-0.1, 0.1, L * L)]).astype(np.float64)
        f = f0.copy()
        libs["rietkerk"].ref_rk_det_steps(_p(f), L, n, R, RK["c"], RK["gmax"], RK["alpha"], RK["d"], RK["rW"],
                                          RK["W0"], RK["DP"], RK["DW"], RK["DO"], RK["k1"], RK["k2"], dt, 1.0)
        out[f"{tag}_in"] = f0.reshape(3, L, L)
        out[f"{tag}_out"] = f.reshape(3, L, L)
        out[f"{tag}_meta"] = np.array([L, n, dt, R])
    # 2) stochastic-remainder RK4 of the Rietkerk step (f_2Dor)
    L = 10
    f0 = np.concatenate([rng.uniform(0, 3, L * L), rng.uniform(0.1, 2, L * L), rng.uniform(0.1, 2, L * L)])
    f = f0.copy()
    libs["rietkerk"].ref_rk_stoch_remainder(_p(f), L, 0.9, RK["c"], RK["gmax"], RK["alpha"], RK["rW"], RK["W0"],
                                            RK["DW"], RK["DO"], RK["k1"], RK["k2"], 1e-3, 1.0)
    out["rkrem_in"] = f0.reshape(3, L, L)
    out["rkrem_out"] = f.reshape(3, L, L)
    # 3) MultiSp DP remainder RK4 (f_DP_Dor_1Sp: -b rho^2), b=2, dt=0.1
    x0 = rng.uniform(0, 3, 100)
    x = x0.copy()
    libs["multisp"].ref_ms_rk4_remainder(_p(x), 10, 2.0, 0.1, 1.0)
    out["msrem_in"], out["msrem_out"] = x0, x
    # 4) first-order DP remainder RK4 (-b rho^2 - c rho^3), b=-2, c=1 (the first-order model)
    x0 = rng.uniform(0, 3, 100)
    x = x0.copy()
    libs["dp"].ref_rk4_first_order(_p(x), 10, -0.7, -2.0, 1.0, 1.0, 0.0, 0.1, 1.0)
    out["forem_in"], out["forem_out"] = x0, x
    # 5) noise-off DP with the 4th-order Laplacian (percNoDiff_2D), L=8, frames after 1, 5, 10 steps
    L = 8
    r0 = 0.5 + rng.uniform(-0.2, 0.2, L * L)
    ts = np.array([0.1, 0.5, 1.0])
    frames = np.zeros((3, L * L))
    nf = libs["dp"].ref_perc_nodiff(_p(ts), 3, _p(r0), 1.0, 0.8, 2.0, 1.0, 0.1, 1.0, L, _p(frames), 3)
    assert nf == 3, nf
    out["nodiff_in"], out["nodiff_out"] = r0.reshape(L, L), frames.reshape(3, L, L)
    out["nodiff_meta"] = np.array([L, 0.8, 2.0, 1.0, 0.1, 1.0])  # L a b D dt dx
    # 6) measurement-time grid
    cases = [(1e4, 0.1), (1e5, 0.1), (1000.0, 0.01), (100.0, 1.0), (50.0, 0.1), (2.0, 0.1)]
    for k, (tmax, dt) in enumerate(cases):
        buf = np.zeros(2000)
        n = libs["dp"].ref_logarithm10_time_bins(tmax, dt, _p(buf), 2000)
        out[f"tbins_{k}"] = buf[:n].copy()
        out[f"tbins_{k}_meta"] = np.array([tmax, dt])
    return out


def ensemble(libs, rng, L, a, tm, n_rep, b=2.0, D=1.0, sigma=1.0, dt=0.1, dx=1.0):
    tm = np.asarray(tm, np.float64)
    rho0 = (1.0 + rng.uniform(-0.01, 0.01, L * L)).astype(np.float64)
    rows = np.zeros((1000, 8))
    means, act = [], []
    for _ in range(n_rep):
        n = libs["dp"].ref_percolation_dornic(_p(tm), len(tm), _p(rho0), tm[-1], a, b, D, sigma, dt, dx, 1, L,
                                              _p(rows), 1000)
        means.append(rows[:n, 3].copy())
        act.append(rows[:n, 6].copy())
    return dict(t=rows[:n, 2].copy(), mean=np.array(means), active=np.array(act), rho0=rho0.reshape(L, L),
                meta=np.array([L, a, b, D, sigma, dt, dx]))


def csv_writers(libs, rng):
    """Files written by the reference's save_frame / save_prelimframe, including the
    collision-safe renumbering when a file of the same name exists."""
    import tempfile
    out = {}
    with tempfile.TemporaryDirectory() as d:
        g = 6
        rho = np.concatenate([rng.uniform(0, 2, g * g - 4), [0.0, 1e-30, 123456.789, 0.1]])
        pat = "/FRAME_T_G_6_a_0.72_R_"
        hdr = "a_c,  x,  P(x; t) \n"
        for _ in range(3):  # R_0, then renumbered R_1, R_2
            libs["multisp"].ref_save_frame(_p(rho), g, d.encode(), pat.encode(), 0.72, 0, hdr.encode())
        for k in range(3):
            out[f"frame_R_{k}"] = np.frombuffer(open(f"{d}{pat}{k}.csv", "rb").read(), np.uint8)
        out["frame_in"] = rho
        rows = np.stack([np.arange(7) * 0.5, rng.uniform(0, 1, 7), rng.uniform(0, 0.01, 7),
                         rng.integers(0, 5, 7).astype(float), rng.integers(0, 36, 7).astype(float)], axis=1)
        rows[3, 1] = 1.0 / 3.0
        ppat = "/PRELIM_AGG_T_G_6_a_0.72_R_"
        phdr = " a , r, L, t , <<P(x; t)>_x>_r, Var[<P(x; t)>_x]_r, # Surviving Runs P(x; t), # Active Sites P(x; t), \n"
        libs["multisp"].ref_save_prelim(_p(np.ascontiguousarray(rows)), 7, g, d.encode(), ppat.encode(), 0.72, 4,
                                        phdr.encode())
        out["prelim_R_4"] = np.frombuffer(open(f"{d}{ppat}4.csv", "rb").read(), np.uint8)
        out["prelim_in"] = rows
    return out


def fke(libs, rng):
    """advdiff_FKE_MultiSp (rietkerk_bjork_FKE.cpp:3614-3695) on the grazer field,
    with the parameters and stencils set_global_FKE_params / precompute_gaussian
    give; L = 9 makes the stencils wrap the lattice more than once."""
    out = {}
    for tag, L, Dg, vg, sg, dta, vmax in (("a", 24, 1.0, 1.0, 1.5, 1.0, 3.0), ("b", 9, 1.0, 2.0, 2.0, 1.0, 2.0)):
        rho = rng.uniform(0, 2, L * L)
        rho[rng.random(L * L) < 0.2] = 0.0
        rho[3] = 1e-12                       # below the reference's epsilon: not moved
        gam = rng.uniform(0, 1, L * L)
        vx = rng.uniform(-vmax, vmax, L * L)
        vy = rng.uniform(-vmax, vmax, L * L)
        o = np.zeros(L * L)
        gD = np.zeros(64); gV = np.zeros(64)
        RD = C.c_int(); RV = C.c_int(); pref = C.c_double()
        rc = libs["fke"].ref_fke_advdiff(_p(rho), _p(gam), _p(vx), _p(vy), L, Dg, vg, sg, dta, 1.0, _p(o), _p(gD),
                                         C.byref(RD), _p(gV), C.byref(RV), C.byref(pref), 64)
        assert rc == 0, rc
        out.update({f"fke_{tag}_rho": rho, f"fke_{tag}_gamma": gam, f"fke_{tag}_vx": vx, f"fke_{tag}_vy": vy,
                    f"fke_{tag}_out": o, f"fke_{tag}_gD": gD[:RD.value + 1].copy(),
                    f"fke_{tag}_gV": gV[:RV.value + 1].copy(), f"fke_{tag}_meta": np.array([L, pref.value])})
    return out


LNSPACE_CASES = ((32, 1024, 6), (40, 400, 10), (31, 257, 7), (64, 64, 1), (50, 200, 4), (33, 1000, 25))


def lnspace_cases():
    lib = C.CDLL(os.path.join(REF, "libref_lnspace.so"))
    lib.ref_lnspace.argtypes = [C.c_int, C.c_int, C.c_int, dp, C.c_int]
    out = {}
    for k, (a, b, n) in enumerate(LNSPACE_CASES):
        buf = np.zeros(64)
        m = lib.ref_lnspace(a, b, n, _p(buf), 64)
        out[f"lnspace_{k}"] = buf[:m].copy()
    out["cases"] = np.array(LNSPACE_CASES)
    return out


def spectrum_frames(rng):
    """Fields of the power-spectrum fixture: stripes, an odd side, spots with an
    empty region, an all-zero lattice (no power: every bin empty) and a
    three-cosine pattern."""
    out = {}
    L = 32
    y, x = np.mgrid[0:L, 0:L]
    out["stripes32"] = 1.0 + 0.5 * np.sin(2 * np.pi * x / 8.0) + 0.05 * rng.random((L, L))
    out["random33"] = rng.uniform(0, 2, (33, 33))
    L = 48
    y, x = np.mgrid[0:L, 0:L]
    f = (1.0 + np.cos(2 * np.pi * x / 12.0)) * (1.0 + np.cos(2 * np.pi * y / 6.0)) + 0.1 * rng.random((L, L))
    f[:10, :14] = 0.0
    out["spots48"] = f
    out["zeros20"] = np.zeros((20, 20))
    L = 64
    y, x = np.mgrid[0:L, 0:L]
    q = 2 * np.pi / 16.0
    f = sum(np.cos(q * (np.cos(th) * x + np.sin(th) * y)) for th in (0.0, 2 * np.pi / 3, 4 * np.pi / 3))
    out["hex64"] = np.maximum(f, 0.0) + 0.02 * rng.random((L, L))
    return out


def spectrum(libs, rng):
    """gen_FFT_PowerSpectra of the reference on frames written by the reference's
    save_frame (one field per file, header of the reference's DP frames)."""
    import shutil
    import tempfile
    sys.path.insert(0, HERE)
    import glow_up_harness as gh
    ref_root = os.environ.get("TM_REF_ROOT")
    if not ref_root:
        sys.exit("set TM_REF_ROOT to the reference checkout")
    out = {}
    d = tempfile.mkdtemp()
    home = tempfile.mkdtemp()
    try:
        gu = gh.load_glow_up(ref_root, home)
        for name, f in spectrum_frames(rng).items():
            L = f.shape[0]
            sub = os.path.join(d, name)
            os.makedirs(sub)
            pat = "/FRAME_T_100_a_0.9_R_"
            libs["multisp"].ref_save_frame(_p(np.ascontiguousarray(f.ravel())), L, sub.encode(), pat.encode(), 0.9, 0,
                                           "a_c,  x,  P(x; t) \n".encode())
            path = f"{sub}{pat}0.csv"
            read = gh.read_csv(path)
            k, p = gh.spectrum_of_frame(gu, path)
            out[f"{name}_field"] = read[read.columns[2]].values.reshape(L, L)
            out[f"{name}_k"], out[f"{name}_power"] = k, p
        out["names"] = np.array(list(spectrum_frames(np.random.default_rng(0)).keys()))
    finally:
        shutil.rmtree(d)
        shutil.rmtree(home)
    return out


# means and shapes of the sampler-level comparison with libstdc++
LIBSTDCXX_POISSON = (0.3, 3.0, 17.0, 50.0, 250.0)
LIBSTDCXX_GAMMA = (0.4, 1.7, 8.0, 60.0)
# (m, mu1) of the whole-draw comparison, from the dilute to the dense regime
LIBSTDCXX_DORNIC = ((16.7, 6.0), (4.0, 1.5), (3.9, 1.5), (8.0, 1.4), (8.0, 2.0), (50.0, 12.0), (2.0, 0.8),
                    (120.0, 40.0))
LIBSTDCXX_N = 6000


def libstdcxx(libs):
    """Draws of the libstdc++ Poisson and Gamma distributions the reference's Dornic step
    constructs per site (stochasticSPDP.cpp:1055-1059), for a sampler-level comparison."""
    out = {}
    for kind, params in ((0, LIBSTDCXX_POISSON), (1, LIBSTDCXX_GAMMA)):
        for k, v in enumerate(params):
            x = np.zeros(LIBSTDCXX_N)
            libs["dp"].ref_libstdcxx_draws(kind, v, 1000 + 17 * k + kind, LIBSTDCXX_N, _p(x))
            out[f"{'poisson' if kind == 0 else 'gamma'}_{k}"] = x.astype(np.float32)
    for k, (m, mu1) in enumerate(LIBSTDCXX_DORNIC):
        x = np.zeros(LIBSTDCXX_N)
        libs["dp"].ref_libstdcxx_dornic(m, mu1, 5000 + 31 * k, LIBSTDCXX_N, _p(x))
        out[f"dornic_{k}"] = x.astype(np.float32)
    out["poisson_params"] = np.array(LIBSTDCXX_POISSON)
    out["gamma_params"] = np.array(LIBSTDCXX_GAMMA)
    out["dornic_params"] = np.array(LIBSTDCXX_DORNIC)
    return out


# the Rietkerk ensemble case: 16^2, R = 1.0, sigma = 0.5, dt = 1e-3, 500 steps, 400 replicates;
# P ~ U(0,1) with a bare 4 x 4 patch (its edge sites draw with Poisson mean 0) and a 4 x 4 patch
# at P = 2e-3 (Poisson means near 16: the exact Poisson and Gamma branches)
RK_ENS = dict(L=16, R=1.0, sigma=0.5, dt=1e-3, steps=500, n_rep=400, seed0=1000, eps=1e-10,
              site_a=(10, 10), site_b=(5, 12))


def rk_ensemble_start(rng):
    L = RK_ENS["L"]
    P = rng.uniform(0, 1, (L, L))
    P[0:4, 0:4] = 0.0
    P[8:12, 8:12] = 2e-3
    return np.stack([P, np.full((L, L), 0.5), np.ones((L, L))])


def rk_ensemble(libs):
    e = RK_ENS
    L = e["L"]
    f0 = rk_ensemble_start(np.random.default_rng(77))
    rows = []
    for j in range(e["n_rep"]):
        f = np.ascontiguousarray(f0.reshape(-1).copy())
        libs["rietkerk"].ref_rk_stoch_steps(_p(f), L, e["steps"], e["seed0"] + j, e["R"], RK["c"], RK["gmax"],
                                            RK["alpha"], RK["d"], RK["rW"], RK["W0"], RK["DP"], RK["DW"], RK["DO"],
                                            RK["k1"], RK["k2"], e["sigma"], e["dt"], 1.0, e["eps"])
        g = f.reshape(3, L, L)
        rows.append([g[0].mean(), g[1].mean(), g[2].mean(), float((g[0] > 0).sum()), g[0][e["site_a"]],
                     g[0][e["site_b"]]])
    np.savez_compressed(os.path.join(HERE, "ref_rk_ensemble.npz"), start=f0, rows=np.array(rows),
                        columns=np.array(["mean_P", "mean_W", "mean_O", "occupied_P", "P_site_a", "P_site_b"]),
                        meta=np.array([L, e["R"], e["sigma"], e["dt"], e["steps"], e["n_rep"], e["seed0"], e["eps"]]))


def main():
    if "--rk-ensemble" in sys.argv:
        rk_ensemble(load(("dp", "rietkerk", "multisp")))
        return
    if "--libstdcxx" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "ref_libstdcxx.npz"), **libstdcxx(load(("dp",))))
        return
    if "--lnspace" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "ref_lnspace.npz"), **lnspace_cases())
        return
    if "--spectrum" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "ref_spectrum.npz"),
                            **spectrum(load(("dp", "rietkerk", "multisp")), np.random.default_rng(5)))
        return
    if "--fke" in sys.argv:
        np.savez_compressed(os.path.join(HERE, "ref_fke.npz"), **fke(load(("fke",)), np.random.default_rng(11)))
        return
    import subprocess
    subprocess.run([sys.executable, os.path.abspath(__file__), "--fke"], check=True)
    subprocess.run([sys.executable, os.path.abspath(__file__), "--spectrum"], check=True)
    subprocess.run([sys.executable, os.path.abspath(__file__), "--lnspace"], check=True)
    subprocess.run([sys.executable, os.path.abspath(__file__), "--rk-ensemble"], check=True)
    libs = load()
    rng = np.random.default_rng(20261203)
    np.savez_compressed(os.path.join(HERE, "ref_pins.npz"), **pins(libs, rng))
    np.savez_compressed(os.path.join(HERE, "ref_csv.npz"), **csv_writers(libs, np.random.default_rng(7)))
    ens = {}
    tm = [1.5, 2.0, 3.0, 5.0, 8.0, 10.0, 20.0, 50.0]
    for tag, L, a, n in (("crit", 8, 0.72, 1500), ("active", 8, 2.0, 800), ("site", 1, 0.72, 3000)):
        e = ensemble(libs, rng, L, a, tm, n)
        for k, v in e.items():
            ens[f"{tag}_{k}"] = v
    np.savez_compressed(os.path.join(HERE, "ref_dp_ensemble.npz"), **ens)
    np.savez_compressed(os.path.join(HERE, "ref_libstdcxx.npz"), **libstdcxx(libs))
    print("wrote", os.listdir(HERE))


if __name__ == "__main__":
    main()
