"""Time the library's FKE gather beside the reference's GPU scatter design on the
same GB300 (TEST INFRASTRUCTURE ONLY).

The reference moves its consumer species with updateMovement
(simulations/Rietkerk_FPE/kernel_advdiff_FKE2D.cu:92-180): one thread per source,
FP64 atomicAdd into the output.  oracle/fke_scatter_ref.cu restates it; this
script times it and the library's two entry points (tm_fke_advdiff_device, which
allocates its scratch and synchronises, and tm_fke_advdiff_device_ws on a reused
workspace) with CUDA events on one stream, on the same L x L FP64 inputs, and
prints one JSON object with the times and the largest relative difference.

    python oracle/time_fke_scatter.py [--L 1024] [--reps 20]
"""
import argparse
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[:] = [os.path.dirname(HERE)] + [q for q in sys.path if os.path.abspath(q or ".") != HERE]

from oracle import oracle as o  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=1024)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--v", type=float, default=1.0)
    a = ap.parse_args()
    import torch
    import trophic_maelstorm_gb300 as tmg
    from trophic_maelstorm_gb300 import _lib as T
    L = a.L
    rng = np.random.default_rng(3)
    rho = rng.uniform(0, 3, (L, L))
    rho[rng.random((L, L)) < 0.3] = 0.0
    gam = rng.uniform(0, 1, (L, L))
    vx = rng.uniform(-a.v, a.v, (L, L))
    vy = rng.uniform(-a.v, a.v, (L, L))
    p = tmg.fke_parameters(1.0, a.v, 1.0, 1.2)
    dev = torch.device("cuda", 0)
    ts = [torch.as_tensor(x, dtype=torch.float64, device=dev) for x in (rho, gam, vx, vy)]
    gD = torch.as_tensor(p.gD, dtype=torch.float64, device=dev)
    gV = torch.as_tensor(p.gV, dtype=torch.float64, device=dev)
    lib = o.fke_scatter_lib()
    stream = torch.cuda.current_stream(dev)
    out_ref = torch.empty_like(ts[0])

    def scatter():
        rc = lib.tmo_fke_scatter_f64(*(t.data_ptr() for t in ts), L, p.pref, 1e-10, gD.data_ptr(), len(p.gD) - 1,
                                     gV.data_ptr(), len(p.gV) - 1, out_ref.data_ptr(), stream.cuda_stream)
        assert rc == 0

    ws = tmg.api.fke_workspace(L, T.TM_FP64)

    def gather_ws():
        return tmg.fke_advdiff(*ts, p, workspace=ws)

    def gather_alloc():
        return tmg.fke_advdiff(*ts, p)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(a.reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / a.reps

    t_ref = timed(scatter)
    t_ws = timed(gather_ws)
    t_alloc = timed(gather_alloc)
    got = gather_ws().cpu().numpy()
    got_alloc = gather_alloc().cpu().numpy()
    scatter()
    torch.cuda.synchronize()
    want = out_ref.cpu().numpy()
    rel = float(np.max(np.abs(got - want)) / np.max(np.abs(want)))
    print(json.dumps({"L": L, "RD": int(len(p.gD) - 1), "RV": int(len(p.gV) - 1), "reps": a.reps,
                      "reference_scatter_ms": t_ref, "gather_workspace_ms": t_ws, "gather_allocating_ms": t_alloc,
                      "speedup_vs_reference_scatter": t_ref / t_ws, "max_rel_diff_vs_scatter": rel,
                      "ws_equals_allocating": bool(np.array_equal(got, got_alloc)),
                      "note": "CUDA events on one stream; the scatter's time includes zeroing its output, "
                              "which its atomics need"}))


if __name__ == "__main__":
    main()
