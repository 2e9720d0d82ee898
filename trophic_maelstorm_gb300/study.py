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
    a = ap.parse_args()
    if a.dp:
        print(json.dumps(dp_precision_study(a.L if a.L != 4096 else 256, a.reps, a.a, a.t_max)))
        return
    print(json.dumps(rietkerk_precision_study(a.L, a.steps, a.every, a.R, precisions=tuple(a.precisions.split(",")))))


if __name__ == "__main__":
    main()
