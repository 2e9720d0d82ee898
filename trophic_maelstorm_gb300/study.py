"""Precision study of the Rietkerk three-field model: the same run in FP32 and
FP64 state (same initial condition, same Philox streams), compared through
the mean plant density and the pattern wavelength (peak of the radially
averaged power spectrum of P, glow_up.py:752-827 semantics).

    python -m trophic_maelstorm_gb300.study --L 4096 --steps 20000 [--every 2000]

Prints one JSON object: per checkpoint the spatial means of P, W, O in both
precisions and their relative differences, the final wavelengths, and the step
times.
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=4096)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--every", type=int, default=2000)
    ap.add_argument("--R", type=float, default=0.9)
    ap.add_argument("--precisions", default="f32,f64")
    a = ap.parse_args()
    print(json.dumps(rietkerk_precision_study(a.L, a.steps, a.every, a.R, precisions=tuple(a.precisions.split(",")))))


if __name__ == "__main__":
    main()
