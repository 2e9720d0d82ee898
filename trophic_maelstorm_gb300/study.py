"""Precision studies: the same runs with FP32 and with FP64 state.

Rietkerk three-field model (default): same initial condition and Philox
streams, compared through the mean plant density and the pattern wavelength
(peak of the radially averaged power spectrum of P, glow_up.py:752-827
semantics).

    python -m trophic_maelstorm_gb300.study --L 4096 --steps 20000 [--every 2000]

DP model near its critical point (--dp): ensembles with the same seeds in both
precisions, compared per observable (ensemble mean density, survival fraction,
distribution of the spatial mean over replicates) against their standard
errors.  Trajectories separate once a rounding difference changes one Poisson
draw, so the comparison is statistical.

    python -m trophic_maelstorm_gb300.study --dp --L 256 --reps 64 --t-max 1000

Rietkerk rainfall sweep in both precisions (--rietkerk-sweep): 8 values of R in
[0.6, 1.2] x 16 replicates at 256^2 (rietkerk_DorFPE_2D_MultiSp's workload,
rietkerk_bjork_FKE.cpp:3697-4664), same initial frames and Philox keys in FP32
and FP64, compared per R and time through the replicate means of P, W, O, the
active-P fraction and survival, each difference in combined standard errors.

    python -m trophic_maelstorm_gb300.study --rietkerk-sweep --L 256 --reps 16 --steps 100000

Pattern scan (--pattern-scan) and a patterned case in both precisions
(--pattern): the rainfall where P forms a pattern (spectrum peak at k well below
L/2), and the FP32-vs-FP64 difference of its wavelength there.

The whole finite-size sweep, timed (--sweep-run): 2560 instances (L in
{64..1024} x 16 a x 32 replicates) from the fully active start with 60
log-spaced measurements.

Each prints one JSON object.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api, _lib as T


def rietkerk_precision_study(L=4096, steps=20000, every=2000, R=0.9, sigma=0.5, dt=1e-3, seed=2024, device=0,
                             precisions=("f32", "f64")):
    ctx = api.Context(device)
    rng = np.random.default_rng(seed)
    f0 = np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.full((L, L), 1.0)])
    checkpoints = list(range(0, steps + 1, every))
    if checkpoints[-1] != steps:
        checkpoints.append(steps)
    out = {"L": L, "steps": steps, "R": R, "sigma": sigma, "dt": dt, "checkpoints": checkpoints}
    for prec in precisions:
        P = T.TM_FP32 if prec == "f32" else T.TM_FP64
        b = api.Batch(ctx, api.rietkerk_model(sigma=sigma, dt=dt), api.instances([L], [seed], R), P)
        b.upload([f0.astype(np.float32 if prec == "f32" else np.float64)])
        t0 = time.perf_counter()
        obs, st = b.advance(steps, checkpoints)
        el = time.perf_counter() - t0
        kv, pw = b.power_spectrum(0, 0)
        out[prec] = {"means_PWO": obs[:, 0, :3].tolist(), "active_P": obs[:, 0, 3].tolist(),
                     "ms_per_step": 1e3 * el / steps, "status": int(st[0]),
                     "wavelength": api.pattern_wavelength(L, kv, pw),
                     "spectrum_peak_k": float(kv[int(np.argmax(pw))])}
        b.close()
    if "f32" in out and "f64" in out:
        m32 = np.array(out["f32"]["means_PWO"])
        m64 = np.array(out["f64"]["means_PWO"])
        out["rel_diff_means_PWO"] = (np.abs(m32 - m64) / np.maximum(np.abs(m64), 1e-300)).tolist()
        out["wavelength_diff"] = out["f32"]["wavelength"] - out["f64"]["wavelength"]
    ctx.close()
    return out


def dp_precision_study(L=256, n_rep=64, a=0.53, t_max=1000.0, seed=4242, device=0):
    """FP32 against FP64 state for the DP model at a (default: the measured a_c):
    per measurement time the ensemble mean density and survival fraction in both
    precisions, their difference in units of the combined standard error, and the
    two-sample KS p-value of the replicate spatial means."""
    from scipy import stats
    from . import surrogate as sg
    ctx = api.Context(device)
    res = {"L": L, "replicates": n_rep, "a": a, "t_max": t_max}
    per = {}
    for prec, P in (("f32", T.TM_FP32), ("f64", T.TM_FP64)):
        inst = api.instances([L] * n_rep, [seed + j for j in range(n_rep)], a)
        steps = sg.measurement_steps(t_max, 0.1, 30)
        b = api.Batch(ctx, api.dp_model(), inst, P)
        rng = np.random.default_rng(seed)
        b.upload([(1.0 + rng.uniform(-0.01, 0.01, (L, L))) for _ in range(n_rep)])
        t0 = time.perf_counter()
        obs, st = b.advance(int(steps[-1]), steps)
        per[prec] = {"mean": obs[:, :, 0].T, "alive": obs[:, :, 1].T > 0,
                     "seconds": time.perf_counter() - t0, "status": int(np.bitwise_or.reduce(st))}
        b.close()
    m32, m64 = per["f32"]["mean"], per["f64"]["mean"]
    s32, s64 = per["f32"]["alive"].mean(0), per["f64"]["alive"].mean(0)
    se = np.sqrt(m32.var(0) / n_rep + m64.var(0) / n_rep)
    z = np.where(se > 0, (m32.mean(0) - m64.mean(0)) / np.where(se > 0, se, 1), 0.0)
    ses = np.sqrt(s32 * (1 - s32) / n_rep + s64 * (1 - s64) / n_rep)
    zs = np.where(ses > 0, (s32 - s64) / np.where(ses > 0, ses, 1), 0.0)
    ks = [float(stats.ks_2samp(m32[:, j], m64[:, j]).pvalue) if m32[:, j].std() > 0 and m64[:, j].std() > 0
          else 1.0 for j in range(m32.shape[1])]
    res.update({"t": (steps * 0.1).tolist(), "rho_f32": m32.mean(0).tolist(), "rho_f64": m64.mean(0).tolist(),
                "rel_diff_rho": (np.abs(m32.mean(0) - m64.mean(0)) / np.maximum(m64.mean(0), 1e-300)).tolist(),
                "z_rho": z.tolist(), "surv_f32": s32.tolist(), "surv_f64": s64.tolist(), "z_surv": zs.tolist(),
                "ks_p": ks, "max_abs_z_rho": float(np.abs(z).max()), "max_abs_z_surv": float(np.abs(zs).max()),
                "min_ks_p": float(min(ks)), "seconds_f32": per["f32"]["seconds"],
                "seconds_f64": per["f64"]["seconds"], "status": [per["f32"]["status"], per["f64"]["status"]]})
    ctx.close()
    return res


def rietkerk_fixed_point(R, alpha=0.2, k2=5.0, W0=0.2, gmax=0.05, k1=5.0, c=10.0, d=0.25, rW=0.2):
    """Homogeneous vegetated fixed point of the Rietkerk right-hand side (rietkerk_bjork_FKE.cpp:
    1760-1785): W* = d k1 / (c gmax - d), P* from dW = 0 with infiltration = R, O* from
    dO = 0.  P* > 0 needs R > rW W* (the mean-field threshold)."""
    Ws = d * k1 / (c * gmax - d)
    Ps = (R - rW * Ws) * (Ws + k1) / (gmax * Ws)
    Os = R * (Ps + k2) / (alpha * (Ps + k2 * W0))
    return Ps, Ws, Os


def _rk_initial(L, reps, seed):
    """P ~ U(0, 1), W = 0.5, O = 1 per replicate (the Rietkerk sweep's start)."""
    rng = np.random.default_rng(seed)
    return [np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.full((L, L), 1.0)]) for _ in range(reps)]


def _rk_vegetated(L, reps, seed, R, amp=0.1):
    """The vegetated fixed point with P perturbed by U(-amp, amp) relative, per replicate."""
    rng = np.random.default_rng(seed)
    Ps, Ws, Os = rietkerk_fixed_point(R)
    return [np.stack([Ps * (1.0 + rng.uniform(-amp, amp, (L, L))), np.full((L, L), Ws), np.full((L, L), Os)])
            for _ in range(reps)]


def _log_steps(steps, n):
    s = np.unique(np.round(np.geomspace(1, steps, n)).astype(np.int64))
    return np.concatenate([[0], s[s < steps], [steps]]).astype(np.int64)


def rietkerk_sweep_precision_study(L=256, Rs=None, reps=16, steps=100000, n_meas=30, seed=7, sigma=0.5, dt=1e-3,
                                   device=0):
    """FP32 against FP64 state over a rainfall sweep of the Rietkerk model.  Both
    precisions start from the same frames with the same Philox keys.  Per R and
    measurement: replicate means of <P>, <W>, <O> and of the active-P fraction,
    the surviving fraction (replicates with an active P site), the FP32 - FP64
    differences in units of their combined standard error, the relative
    differences, and the two-sample KS p-value of the replicate <P>.  At the end:
    the spectrum-peak wavelength of P per replicate in both precisions."""
    from scipy import stats
    Rs = list(api.linspace(0.6, 1.2, 8)) if Rs is None else list(Rs)
    ctx = api.Context(device)
    meas = _log_steps(steps, n_meas)
    init = _rk_initial(L, reps, seed)
    Ls, keys, av, fields = [], [], [], []
    for i, R in enumerate(Rs):
        for j in range(reps):
            Ls.append(L); keys.append(seed * 1000 + 97 * i + j); av.append(R); fields.append(init[j])
    inst = api.instances(Ls, keys, av)
    res = {"L": L, "R": Rs, "replicates": reps, "steps": steps, "dt": dt, "sigma": sigma,
           "t": (meas * dt).tolist(), "init": "P ~ U(0,1), W = 0.5, O = 1; replicate j starts from frame j at every R"}
    per = {}
    for prec, P in (("f32", T.TM_FP32), ("f64", T.TM_FP64)):
        dtype = np.float32 if prec == "f32" else np.float64
        b = api.Batch(ctx, api.rietkerk_model(sigma=sigma, dt=dt), inst, P)
        b.upload([f.astype(dtype) for f in fields])
        t0 = time.perf_counter()
        obs, st = b.advance(steps, meas)
        sec = time.perf_counter() - t0
        wl = []
        for k in range(len(Ls)):
            kv, pw = b.power_spectrum(k, 0)
            wl.append(api.pattern_wavelength(L, kv, pw) if np.any(pw > 0) else float("nan"))
        b.close()
        # obs: [meas, inst, (P, W, O, active P)] -> [R, rep, meas, 4]
        per[prec] = {"obs": obs.transpose(1, 0, 2).reshape(len(Rs), reps, len(meas), 4), "seconds": sec,
                     "status": int(np.bitwise_or.reduce(st)), "wavelength": np.array(wl).reshape(len(Rs), reps)}
    o32, o64 = per["f32"]["obs"], per["f64"]["obs"]
    n = float(L * L)

    def zstat(a, b):
        se = np.sqrt(a.var(1, ddof=1) / reps + b.var(1, ddof=1) / reps)
        d = a.mean(1) - b.mean(1)
        return np.where(se > 0, d / np.where(se > 0, se, 1), np.where(d == 0, 0.0, np.inf)), d, se

    # per observable: the FP32 - FP64 difference d, its combined standard error se
    # and z = d / se; rel_diff = |d| / |FP64|.  Where the replicates agree closely
    # (W and O once P has died out) se -> 0 and d is the rounding difference itself,
    # so "excess" = |d| - 5 se - 1e-5 |FP64| measures what neither explains.
    table = {}
    for f, name in ((0, "P"), (1, "W"), (2, "O")):
        z, d, se = zstat(o32[..., f], o64[..., f])
        m64 = o64[..., f].mean(1)
        table[name] = {"f32": o32[..., f].mean(1).tolist(), "f64": m64.tolist(), "z": z.tolist(),
                       "se": se.tolist(), "rel_diff": (np.abs(d) / np.maximum(np.abs(m64), 1e-300)).tolist(),
                       "max_abs_z": float(np.abs(z).max()),
                       "max_excess": float((np.abs(d) - 5 * se - 1e-5 * np.abs(m64)).max())}
    a32, a64 = o32[..., 3] / n, o64[..., 3] / n
    z, d, se = zstat(a32, a64)
    table["active_P_fraction"] = {"f32": a32.mean(1).tolist(), "f64": a64.mean(1).tolist(), "z": z.tolist(),
                                  "se": se.tolist(), "max_abs_z": float(np.abs(z).max()),
                                  "max_excess": float((np.abs(d) - 5 * se - 1e-5 * a64.mean(1)).max())}
    s32, s64 = (o32[..., 3] > 0).mean(1), (o64[..., 3] > 0).mean(1)
    ses = np.sqrt(s32 * (1 - s32) / reps + s64 * (1 - s64) / reps)
    zs = np.where(ses > 0, (s32 - s64) / np.where(ses > 0, ses, 1), np.where(s32 == s64, 0.0, np.inf))
    table["survival"] = {"f32": s32.tolist(), "f64": s64.tolist(), "z": zs.tolist(),
                         "max_abs_z": float(np.abs(zs).max()),
                         "max_excess": float((np.abs(s32 - s64) - 5 * ses).max())}
    ks = np.ones((len(Rs), len(meas)))
    for i in range(len(Rs)):
        for j in range(len(meas)):
            x, y = o32[i, :, j, 0], o64[i, :, j, 0]
            if x.std() > 0 and y.std() > 0:
                ks[i, j] = stats.ks_2samp(x, y).pvalue
    table["ks_p_P"] = ks.tolist()
    res.update({"observables": table, "min_ks_p_P": float(ks.min()),
                "wavelength_f32": per["f32"]["wavelength"].tolist(),
                "wavelength_f64": per["f64"]["wavelength"].tolist(),
                "seconds_f32": per["f32"]["seconds"], "seconds_f64": per["f64"]["seconds"],
                "ms_per_step_f32": 1e3 * per["f32"]["seconds"] / steps,
                "ms_per_step_f64": 1e3 * per["f64"]["seconds"] / steps,
                "status": [per["f32"]["status"], per["f64"]["status"]]})
    ctx.close()
    return res


def _peak(L, kv, pw):
    """Spectrum peak: wavelength L/k and its prominence (peak power over the median
    of the non-empty bins)."""
    if not np.any(pw > 0):
        return float("nan"), 0.0
    j = int(np.argmax(pw))
    med = float(np.median(pw[pw > 0]))
    return float(L / kv[j]), float(pw[j] / med) if med > 0 else float("inf")


def rietkerk_pattern_scan(L=128, Rs=(1.02, 1.05, 1.1, 1.15, 1.2, 1.3, 1.4, 1.6), reps=2, steps=200000, n_meas=8,
                          seed=3, sigma=0.5, dt=1e-3, device=0, precision="f32", init="vegetated"):
    """Where does P form a pattern?  Per R: mean P and the spectrum peak of P
    (wavelength, prominence) per replicate at log-spaced times.  init "vegetated"
    starts at the homogeneous fixed point (P perturbed 10 %), "sweep" at the
    rainfall sweep's P ~ U(0, 1), W = 0.5, O = 1."""
    ctx = api.Context(device)
    P = T.TM_FP32 if precision == "f32" else T.TM_FP64
    Ls, keys, av, fields = [], [], [], []
    for i, R in enumerate(Rs):
        fr = _rk_vegetated(L, reps, seed + i, R) if init == "vegetated" else _rk_initial(L, reps, seed)
        for j in range(reps):
            Ls.append(L); keys.append(seed * 1000 + 97 * i + j); av.append(R); fields.append(fr[j])
    b = api.Batch(ctx, api.rietkerk_model(sigma=sigma, dt=dt), api.instances(Ls, keys, av), P)
    b.upload([f.astype(np.float32 if precision == "f32" else np.float64) for f in fields])
    checkpoints = _log_steps(steps, n_meas)[1:]
    out = {"L": L, "R": list(Rs), "replicates": reps, "init": init, "t": (checkpoints * dt).tolist(), "rows": []}
    t0 = time.perf_counter()
    for c in checkpoints:
        obs, _ = b.advance(int(c) - b.step, [int(c)])
        for k in range(len(Ls)):
            kv, pw = b.power_spectrum(k, 0)
            wl, prom = _peak(L, kv, pw)
            out["rows"].append({"t": float(c * dt), "R": av[k], "rep": k % reps, "mean_P": float(obs[0, k, 0]),
                                "wavelength": wl, "prominence": prom})
    out["seconds"] = time.perf_counter() - t0
    b.close()
    ctx.close()
    return out


def rietkerk_pattern_precision(L=256, R=1.2, reps=4, steps=500000, n_meas=12, seed=5, sigma=0.5, dt=1e-3, device=0):
    """A patterned case in both precisions (same frames and keys, started at the
    perturbed vegetated fixed point): spectrum-peak wavelength and prominence of P
    over time, mean P, and the whole final spectra."""
    ctx = api.Context(device)
    init = _rk_vegetated(L, reps, seed, R)
    inst = api.instances([L] * reps, [seed * 1000 + j for j in range(reps)], R)
    checkpoints = _log_steps(steps, n_meas)[1:]
    out = {"L": L, "R": R, "replicates": reps, "steps": steps, "sigma": sigma, "dt": dt,
           "t": (checkpoints * dt).tolist()}
    for prec, P in (("f32", T.TM_FP32), ("f64", T.TM_FP64)):
        b = api.Batch(ctx, api.rietkerk_model(sigma=sigma, dt=dt), inst, P)
        b.upload([f.astype(np.float32 if prec == "f32" else np.float64) for f in init])
        t0 = time.perf_counter()
        rows = []
        for c in checkpoints:
            obs, st = b.advance(int(c) - b.step, [int(c)])
            r = {"t": float(c * dt), "mean_P": obs[0, :, 0].tolist(), "wavelength": [], "prominence": []}
            for k in range(reps):
                kv, pw = b.power_spectrum(k, 0)
                wl, prom = _peak(L, kv, pw)
                r["wavelength"].append(wl)
                r["prominence"].append(prom)
            rows.append(r)
        spectra = [b.power_spectrum(k, 0)[1].tolist() for k in range(reps)]
        out[prec] = {"rows": rows, "seconds": time.perf_counter() - t0, "status": int(np.bitwise_or.reduce(st)),
                     "final_spectra": spectra, "k": b.power_spectrum(0, 0)[0].tolist()}
        b.close()
    w32 = np.array(out["f32"]["rows"][-1]["wavelength"])
    w64 = np.array(out["f64"]["rows"][-1]["wavelength"])
    out["final_wavelength_f32"] = w32.tolist()
    out["final_wavelength_f64"] = w64.tolist()
    out["final_wavelength_mean_diff"] = float(w32.mean() - w64.mean())
    out["final_wavelength_rel_diff"] = float(abs(w32.mean() - w64.mean()) / w64.mean())
    s32 = np.array(out["f32"]["final_spectra"]).mean(0)
    s64 = np.array(out["f64"]["final_spectra"]).mean(0)
    out["mean_spectrum_rel_l2_diff"] = float(np.linalg.norm(s32 - s64) / np.linalg.norm(s64))
    ctx.close()
    return out


def sweep_workload(Ls=(64, 128, 256, 512, 1024), reps=32, n_a=16, a_center=0.530, span=0.02):
    """The ragged finite-size sweep: every L x n_a values of a log-spaced within
    +-span of a_center x reps replicates, in (L, a, replicate) order, replicate k
    of the list keyed 1_000_003 k + 17.  Returns (Ls, keys, a values)."""
    avs = list(np.geomspace(a_center * (1 - span), a_center * (1 + span), n_a))
    Ls_, keys, av = [], [], []
    k = 0
    for L in Ls:
        for a in avs:
            for _ in range(reps):
                Ls_.append(int(L)); keys.append(1_000_003 * k + 17); av.append(float(a)); k += 1
    return Ls_, keys, av


def sweep_full_run(steps=10000, n_meas=60, device=0, dt=0.1):
    """The whole sweep (2560 instances, FP32 state) run from the fully active start
    rho0 = 1 + U(-0.01, 0.01) for `steps` steps with n_meas log-spaced measurements
    of every instance, as one device-resident batch.  Reports the wall time, the
    site-updates it advanced (extinct instances count as advanced) and, per L, the
    mean density and the surviving fraction over its replicates and a-values."""
    from . import surrogate as sg
    ctx = api.Context(device)
    Ls, keys, av = sweep_workload()
    inst = api.instances(Ls, keys, av)
    b = api.Batch(ctx, api.dp_model(dt=dt), inst, T.TM_FP32)
    rng = np.random.default_rng(0)
    b.upload([(1.0 + rng.uniform(-0.01, 0.01, (L, L))).astype(np.float32) for L in Ls])
    meas = sg.measurement_steps(steps * dt, dt, n_meas)
    meas = meas[meas <= steps]
    t0 = time.perf_counter()
    obs, st = b.advance(int(steps), meas)
    sec = time.perf_counter() - t0
    b.close()
    ctx.close()
    sites = float(sum(L * L for L in Ls))
    Ls_arr = np.array(Ls)
    per_L = {}
    for L in sorted(set(Ls)):
        sel = Ls_arr == L
        per_L[str(L)] = {"rho": obs[:, sel, 0].mean(1).tolist(), "surviving": (obs[:, sel, 1] > 0).mean(1).tolist()}
    return {"instances": len(Ls), "sites_per_step": sites, "steps": int(steps), "t_max": steps * dt,
            "measurements": len(meas), "t": (meas * dt).tolist(), "seconds": sec,
            "site_updates": sites * steps, "site_updates_per_s": sites * steps / sec,
            "status_or": int(np.bitwise_or.reduce(st)), "per_L": per_L}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--every", type=int, default=2000)
    ap.add_argument("--R", type=float, default=0.9)
    ap.add_argument("--precisions", default="f32,f64")
    ap.add_argument("--dp", action="store_true", help="DP ensembles near a_c instead of the Rietkerk run")
    ap.add_argument("--reps", type=int, default=64)
    ap.add_argument("--t-max", type=float, default=1000.0)
    ap.add_argument("--a", type=float, default=0.53)
    ap.add_argument("--rietkerk-sweep", action="store_true", help="FP32 vs FP64 over 8 R in [0.6, 1.2]")
    ap.add_argument("--pattern-scan", action="store_true", help="where P forms a pattern (FP32)")
    ap.add_argument("--pattern", action="store_true", help="a patterned case in both precisions")
    ap.add_argument("--sweep-run", action="store_true", help="the whole 2560-instance sweep, timed")
    a = ap.parse_args()
    if a.rietkerk_sweep:
        print(json.dumps(rietkerk_sweep_precision_study(a.L if a.L != 4096 else 256, None, a.reps if a.reps != 64
                                                        else 16, a.steps if a.steps != 20000 else 100000)))
        return
    if a.pattern_scan:
        print(json.dumps(rietkerk_pattern_scan(a.L if a.L != 4096 else 128, steps=a.steps if a.steps != 20000
                                               else 200000)))
        return
    if a.pattern:
        print(json.dumps(rietkerk_pattern_precision(a.L if a.L != 4096 else 256, a.R if a.R != 0.9 else 1.2,
                                                    reps=a.reps if a.reps != 64 else 4,
                                                    steps=a.steps if a.steps != 20000 else 500000)))
        return
    if a.sweep_run:
        print(json.dumps(sweep_full_run(a.steps if a.steps != 20000 else 10000)))
        return
    if a.dp:
        print(json.dumps(dp_precision_study(a.L if a.L != 4096 else 256, a.reps, a.a, a.t_max)))
        return
    print(json.dumps(rietkerk_precision_study(a.L, a.steps, a.every, a.R, precisions=tuple(a.precisions.split(",")))))


if __name__ == "__main__":
    main()
