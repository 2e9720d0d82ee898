"""Sweep surrogate: a small network trained on the integrator's own runs that
proposes where to look for the critical point of the DP Langevin model.

The reference locates a_c by uniform sweeps of the control parameter
(critical_exp_delta, simulations/Percolation_FD/stochasticSPDP.cpp:1309-1422),
one full simulation per grid value.  Here:

* `generate_runs` runs ensembles of the batched integrator (one ragged batch for
  all (a, L) points) and records the ensemble mean density rho(t) and the
  survival fraction at logarithmic times;
* `MLP` is the 3-128-128-128-2 GELU network of include/tm.h (tm_mlp_*): BF16
  weights, FP32 accumulation, forward and backward on the tensor cores,
  full-batch Adam;
* `Surrogate` fits it to (a, log L, log t) -> (log10 rho, survival) and gives
  the local decay exponent delta_eff(a) = -d log rho / d log t over a late window;
* `locate_critical_point` is the search the surrogate guides: it proposes the
  bracket [a_hat - h, a_hat + h] around the root of delta_eff(a) = delta_DP and
  verifies both ends by full simulations, moving the bracket until the
  simulations confirm it; `uniform_sweep` is the method without it.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _lib as T
from . import api

H = 128
NPARAMS = T.TM_MLP_NPARAMS
DELTA_DP_2D = 0.4505          # survival/decay exponent of 2-D directed percolation (literature value)


def init_params(seed=0):
    """Uniform fan-in initialisation: weights U(-l, l) with l = sqrt(6 / fan_in) / 2,
    biases 0, in the tm_mlp parameter layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for shape, is_w in (((H, 3), True), ((H,), False), ((H, H), True), ((H,), False), ((H, H), True),
                        ((H,), False), ((2, H), True), ((2,), False)):
        if is_w:
            lim = math.sqrt(6.0 / shape[1]) / 2
            parts.append(rng.uniform(-lim, lim, shape).ravel())
        else:
            parts.append(np.zeros(shape))
    p = np.concatenate(parts).astype(np.float32)
    assert p.size == NPARAMS
    return p


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


class MLP:
    """tm_mlp_*: the network's parameters, Adam state and training set in HBM."""

    def __init__(self, ctx: api.Context, params=None, seed=0):
        self.ctx = ctx
        p = np.ascontiguousarray(init_params(seed) if params is None else params, np.float32)
        if p.size != NPARAMS:
            raise T.TMError(T.TM_ERR_INVALID, "MLP: parameter vector size")
        self._h = C.c_void_p()
        T.check(T.lib().tm_mlp_create(ctx.handle, _fp(p), C.byref(self._h)), "tm_mlp_create")
        self.n = 0

    def set_params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        T.check(T.lib().tm_mlp_set_params(self._h, _fp(p)), "tm_mlp_set_params")

    def get_params(self):
        p = np.empty(NPARAMS, np.float32)
        T.check(T.lib().tm_mlp_get_params(self._h, _fp(p)), "tm_mlp_get_params")
        return p

    def set_data(self, x, t, w=None):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 2)
        w = np.ones_like(t) if w is None else np.ascontiguousarray(w, np.float32).reshape(-1, 2)
        if not (len(x) == len(t) == len(w)):
            raise T.TMError(T.TM_ERR_INVALID, "MLP.set_data: x, t, w lengths")
        T.check(T.lib().tm_mlp_set_data(self._h, _fp(x), _fp(t), _fp(w), len(x)), "tm_mlp_set_data")
        self.n = len(x)

    def loss_grad(self, inv_norm=None):
        inv = 1.0 / self.n if inv_norm is None else inv_norm
        loss = C.c_double()
        g = np.empty(NPARAMS, np.float32)
        T.check(T.lib().tm_mlp_loss_grad(self._h, inv, C.byref(loss), _fp(g)), "tm_mlp_loss_grad")
        return loss.value, g

    def train(self, steps, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, inv_norm=None):
        inv = 1.0 / self.n if inv_norm is None else inv_norm
        hist = np.empty(max(steps, 1), np.float64)
        T.check(T.lib().tm_mlp_train(self._h, steps, lr, beta1, beta2, eps, inv,
                                     hist.ctypes.data_as(C.POINTER(C.c_double))), "tm_mlp_train")
        return hist[:steps]

    def predict(self, x):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, 3)
        y = np.empty((len(x), 2), np.float32)
        T.check(T.lib().tm_mlp_predict(self._h, _fp(x), len(x), _fp(y)), "tm_mlp_predict")
        return y

    def close(self):
        if self._h:
            T.lib().tm_mlp_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


# ------------------------------------------------------------------ full simulations
def measurement_steps(t_max, dt, n_meas=60, t_min=1.0):
    """Step indices of n_meas log-spaced times in [t_min, t_max] (duplicates removed)."""
    s = np.unique(np.rint(np.logspace(np.log10(t_min), np.log10(t_max), n_meas) / dt).astype(np.int64))
    return s[s > 0]


@dataclass
class Ensembles:
    a: np.ndarray            # control value of each point
    L: np.ndarray            # lattice side of each point
    t: np.ndarray            # measurement times
    rho: np.ndarray          # [point, time] replicate mean of the spatial mean density (extinct runs count 0)
    surv: np.ndarray         # [point, time] fraction of replicates with an active site
    n_rep: int
    site_updates: float      # lattice sites x steps advanced (live and extinct)
    seconds: float           # wall time of the batched run

    @property
    def runs(self):
        return len(self.a) * self.n_rep


def run_ensembles(ctx, a_values, Ls, n_rep, t_max, *, dt=0.1, b=2.0, D=1.0, sigma=1.0, seed=0, n_meas=60,
                  precision=T.TM_FP32, point_seeds=None):
    """Full simulations: n_rep replicates of the DP Langevin model (the config of
    percolationDornic_2D with FP32 state) for every (a, L) point, all in one ragged
    batch, from rho0 = 1 + U(-0.01, 0.01).  Replicate j of point i has the key
    k = seed + i * n_rep + j, or point_seeds[i] + j when given; k seeds both its
    Philox stream and its initial field, so a run does not depend on the rest of
    the batch."""
    import time
    import torch
    a_values = np.asarray(a_values, np.float64)
    Ls = np.broadcast_to(np.asarray(Ls, np.int64), a_values.shape)
    npt = len(a_values)
    if point_seeds is None:
        keys = [seed + i for i in range(npt * n_rep)]
    else:
        keys = [int(point_seeds[i]) + j for i in range(npt) for j in range(n_rep)]
    inst = api.instances([int(L) for L in Ls for _ in range(n_rep)], keys, np.repeat(a_values, n_rep))
    steps = measurement_steps(t_max, dt, n_meas)
    model = api.dp_model(b=b, D=D, sigma=sigma, dt=dt)
    batch = api.Batch(ctx, model, inst, precision)
    total, off, _ = api.layout(inst, 1)
    dtype = torch.float32 if precision == T.TM_FP32 else torch.float64
    dev = torch.device("cuda", ctx.device)
    g = torch.Generator(device=dev)
    buf = torch.zeros(total, dtype=dtype, device=dev)
    for k in range(len(inst)):
        n = inst[k].L * inst[k].L
        g.manual_seed(keys[k] & 0x7FFFFFFFFFFFFFFF)
        buf[int(off[k]):int(off[k]) + n].uniform_(0.99, 1.01, generator=g)
    torch.cuda.synchronize(dev)
    batch.upload_device(buf.data_ptr())
    ctx.sync()                                   # the copy reads buf on the library's stream
    del buf
    t0 = time.perf_counter()
    obs, _ = batch.advance(int(steps[-1]), steps)
    sec = time.perf_counter() - t0
    batch.close()
    mean = obs[:, :, 0].reshape(len(steps), npt, n_rep)
    act = obs[:, :, 1].reshape(len(steps), npt, n_rep)
    sites = float(sum(int(L) * int(L) for L in Ls)) * n_rep * float(steps[-1])
    return Ensembles(a_values, np.asarray(Ls), steps * dt, mean.mean(axis=2).T.copy(),
                     (act > 0).mean(axis=2).T.copy(), n_rep, sites, sec)


def delta_eff(rho_t1, rho_t2, t1, t2):
    """Local decay exponent -d ln rho / d ln t between two times."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return -(np.log(rho_t2) - np.log(rho_t1)) / (math.log(t2) - math.log(t1))


# ------------------------------------------------------------------ the surrogate
A_CENTER, A_SCALE = 0.53, 0.03        # feature scaling of a (the measured a_c of b=2, D=1, sigma=1, dt=0.1)
WINDOW = (0.50, 0.56)                 # search window: a_c +- 0.03


def features(a, L, t):
    a, L, t = np.broadcast_arrays(np.asarray(a, np.float64), np.asarray(L, np.float64), np.asarray(t, np.float64))
    return np.stack([(a - A_CENTER) / A_SCALE, (np.log2(L) - 8.0) / 2.0, (np.log10(t) - 1.5) / 1.5],
                    -1).astype(np.float32)


class Surrogate:
    """(a, log L, log t) -> (log10 of the ensemble mean density, survival fraction),
    fitted on Ensembles by the tensor-core MLP."""

    def __init__(self, ctx, seed=0):
        self.mlp = MLP(ctx, seed=seed)
        self.loss = None

    def fit(self, ens: Ensembles, schedule=((2500, 3e-3), (2500, 1e-3), (2000, 3e-4)), rho_floor=1e-6):
        npt, nt = ens.rho.shape
        a = np.repeat(ens.a, nt)
        L = np.repeat(ens.L, nt)
        t = np.tile(ens.t, npt)
        rho = ens.rho.reshape(-1)
        ok = rho > rho_floor
        y = np.stack([np.where(ok, np.log10(np.maximum(rho, rho_floor)), 0.0), ens.surv.reshape(-1)], 1)
        w = np.stack([ok.astype(np.float64), np.ones(len(rho))], 1)
        self.mlp.set_data(features(a, L, t), y, w)
        hist = [self.mlp.train(n, lr=lr) for n, lr in schedule]
        self.loss = np.concatenate(hist)
        return self.loss

    def predict(self, a, L, t):
        y = self.mlp.predict(features(a, L, t).reshape(-1, 3))
        return 10.0 ** y[:, 0].astype(np.float64), y[:, 1].astype(np.float64)

    def delta_eff(self, a, L, t1, t2):
        a = np.asarray(a, np.float64)
        r1, _ = self.predict(a, L, t1)
        r2, _ = self.predict(a, L, t2)
        return delta_eff(r1, r2, t1, t2)

    def propose(self, L, t1, t2, lo=WINDOW[0], hi=WINDOW[1], n=1201):
        """Root of delta_eff(a) = delta_DP on a fine grid (first crossing from the
        absorbing side); the grid point nearest to it when there is none."""
        a = np.linspace(lo, hi, n)
        d = self.delta_eff(a, L, t1, t2) - DELTA_DP_2D
        idx = np.nonzero((d[:-1] > 0) & (d[1:] <= 0))[0]
        if len(idx) == 0:
            return float(a[int(np.argmin(np.abs(d)))])
        k = int(idx[0])
        return float(a[k] + (a[k + 1] - a[k]) * d[k] / (d[k] - d[k + 1]))

    def close(self):
        self.mlp.close()


class Judge:
    """Full simulations that decide on which side of the transition a value of a
    lies: delta_eff of n_rep replicates at lattice side L between t1 and t_max,
    against delta_DP.  Results are cached per a; `runs` counts the simulations.

    Common random numbers: replicate j has the same key (initial field and
    Philox stream) at every a, so two values of a differ by the control
    parameter only, not by independent sampling noise.  delta_eff(a) is then a
    smooth function of a for a given judge, and every search that asks the
    same judge (or one with the same seed) sees the same crossing."""

    def __init__(self, ctx, L, n_rep, t_max, t1, seed=7):
        self.ctx, self.L, self.n_rep, self.t_max, self.t1, self.seed = ctx, L, n_rep, t_max, t1, seed
        self.cache = {}
        self.runs = 0
        self.seconds = 0.0

    def _seed(self, a):
        return self.seed

    def delta(self, a_values):
        a_values = [round(float(a), 9) for a in a_values]
        todo = [a for a in dict.fromkeys(a_values) if a not in self.cache]
        if todo:            # one batch; replicate j has the same key at every value
            e = run_ensembles(self.ctx, todo, self.L, self.n_rep, self.t_max,
                              point_seeds=[self._seed(a) for a in todo])
            i1 = int(np.argmin(np.abs(e.t - self.t1)))
            d = delta_eff(e.rho[:, i1], e.rho[:, -1], e.t[i1], e.t[-1])
            for a, v in zip(todo, d):
                self.cache[a] = float(v)
            self.runs += self.n_rep * len(todo)
            self.seconds += e.seconds
        return np.array([self.cache[a] for a in a_values])


def uniform_sweep(judge: Judge, lo=WINDOW[0], hi=WINDOW[1], h=1e-3):
    """The method without the surrogate: full simulations on the grid lo, lo + 2h, ...,
    hi; a_c is bracketed by the first grid interval where delta_eff crosses delta_DP."""
    grid = lo + 2 * h * np.arange(int(round((hi - lo) / (2 * h))) + 1)
    d = judge.delta(grid)
    idx = np.nonzero((d[:-1] > DELTA_DP_2D) & (d[1:] <= DELTA_DP_2D))[0]
    if len(idx) == 0:
        return None, judge.runs
    k = int(idx[0])
    return (float(grid[k]), float(grid[k + 1])), judge.runs


def guided_search(judge: Judge, a_hat, h=1e-3, lo=WINDOW[0], hi=WINDOW[1], max_moves=40):
    """The surrogate's bracket [a_hat - h, a_hat + h], verified by full simulations at
    both ends and moved by 2h toward the transition until the simulations confirm a
    crossing of delta_DP inside it (the fallback when the surrogate is off)."""
    a_lo, a_hi = a_hat - h, a_hat + h
    for _ in range(max_moves):
        d_lo, d_hi = judge.delta([a_lo, a_hi])
        if d_lo > DELTA_DP_2D >= d_hi:
            return (float(a_lo), float(a_hi)), judge.runs
        if d_hi > DELTA_DP_2D:                   # both ends on the absorbing side
            a_lo, a_hi = a_hi, a_hi + 2 * h
        elif d_lo <= DELTA_DP_2D:                # both ends on the active side
            a_lo, a_hi = a_lo - 2 * h, a_lo
        else:                                    # ends inverted by noise: widen
            a_lo, a_hi = a_lo - h, a_hi + h
        if a_lo < lo - 2 * h or a_hi > hi + 2 * h:
            break
    return None, judge.runs


def training_corpus(ctx, Ls=(64, 128, 256, 512, 1024), n_a=40, n_rep=15, t_max=1000.0, lo=WINDOW[0],
                    hi=WINDOW[1], seed=0):
    """n_a values of a drawn uniformly from [lo, hi] for every L, n_rep replicates each:
    len(Ls) * n_a * n_rep full runs in one ragged batch."""
    rng = np.random.default_rng(seed)
    a = np.concatenate([rng.uniform(lo, hi, n_a) for _ in Ls])
    L = np.repeat(np.asarray(Ls), n_a)
    return run_ensembles(ctx, a, L, n_rep, t_max, seed=10_000_000 + seed)


def critical_point_study(ctx, Ls=(64, 128, 256, 512, 1024), n_a=40, n_rep=15, judge_L=512, judge_rep=8,
                         t_max=1000.0, t1=100.0, seed=0):
    """Train the surrogate on a corpus of full runs, then locate a_c at judge_L to
    +-1e-3 twice -- guided by the surrogate and by the uniform sweep -- and count
    the full simulations each needed."""
    import time
    t0 = time.perf_counter()
    corpus = training_corpus(ctx, Ls, n_a, n_rep, t_max, seed=seed)
    t_corpus = time.perf_counter() - t0
    sur = Surrogate(ctx, seed=seed)
    t0 = time.perf_counter()
    loss = sur.fit(corpus)
    t_fit = time.perf_counter() - t0
    a_hat = sur.propose(judge_L, t1, t_max)
    jg = Judge(ctx, judge_L, judge_rep, t_max, t1)
    g_bracket, g_runs = guided_search(jg, a_hat)
    ju = Judge(ctx, judge_L, judge_rep, t_max, t1)
    u_bracket, u_runs = uniform_sweep(ju)
    grid = np.array(sorted(ju.cache))
    res = {
        "window": list(WINDOW), "judge": {"L": judge_L, "replicates": judge_rep, "t1": t1, "t_max": t_max,
                                          "delta_DP": DELTA_DP_2D},
        "corpus": {"Ls": list(Ls), "a_per_L": n_a, "replicates": n_rep, "runs": corpus.runs,
                   "site_updates": corpus.site_updates, "seconds": t_corpus},
        "fit": {"samples": int(corpus.rho.size), "adam_steps": int(len(loss)), "loss_first": float(loss[0]),
                "loss_last": float(loss[-1]), "seconds": t_fit},
        "surrogate_a_hat": a_hat,
        "guided": {"bracket": g_bracket, "runs": g_runs, "seconds": jg.seconds,
                   "points": {str(k): v for k, v in sorted(jg.cache.items())}},
        "uniform": {"bracket": u_bracket, "runs": u_runs, "seconds": ju.seconds,
                    "points": {str(k): v for k, v in sorted(ju.cache.items())}},
        "surrogate_delta_on_grid": {str(round(float(a), 9)): float(d) for a, d in
                                    zip(grid, sur.delta_eff(grid, judge_L, t1, t_max))},
        "runs_ratio_uniform_over_guided": (u_runs / g_runs) if g_runs else None,
    }
    sur.close()
    return res


NU_PERP_DP_2D = 0.733            # correlation-length exponent of 2-D directed percolation (literature value)


def critical_point_vs_L(ctx, judge_Ls=(256, 512, 1024), Ls=(64, 128, 256, 512, 1024), n_a=40, n_rep=15,
                        judge_rep=8, t_max=1000.0, t1=100.0, seed=0):
    """One corpus and one fitted surrogate, then the guided and the uniform search
    judged at every side in judge_Ls, and a finite-size extrapolation of the
    bracket centres: a_c(L) = a_c(inf) + c L^(-1/nu_perp), fitted by least squares
    (nu_perp of 2-D DP).  The judge's window (t1, t_max) is the same at every L,
    so a_c(L) is the pseudo-critical point of that window."""
    import time
    t0 = time.perf_counter()
    corpus = training_corpus(ctx, Ls, n_a, n_rep, t_max, seed=seed)
    t_corpus = time.perf_counter() - t0
    sur = Surrogate(ctx, seed=seed)
    loss = sur.fit(corpus)
    per_L = {}
    for L in judge_Ls:
        a_hat = sur.propose(L, t1, t_max)
        jg = Judge(ctx, L, judge_rep, t_max, t1)
        g_bracket, g_runs = guided_search(jg, a_hat)
        ju = Judge(ctx, L, judge_rep, t_max, t1)
        u_bracket, u_runs = uniform_sweep(ju)
        per_L[int(L)] = {"a_hat": a_hat, "guided": {"bracket": g_bracket, "runs": g_runs, "seconds": jg.seconds},
                         "uniform": {"bracket": u_bracket, "runs": u_runs, "seconds": ju.seconds,
                                     "points": {str(k): v for k, v in sorted(ju.cache.items())}}}
    sur.close()
    fit = {}
    for which in ("guided", "uniform"):
        pts = [(L, 0.5 * sum(r[which]["bracket"])) for L, r in per_L.items() if r[which]["bracket"]]
        if len(pts) >= 2:
            x = np.array([L ** (-1.0 / NU_PERP_DP_2D) for L, _ in pts])
            y = np.array([a for _, a in pts])
            A = np.stack([np.ones_like(x), x], 1)
            coef, *_ = np.linalg.lstsq(A, y, rcond=None)
            fit[which] = {"a_c_inf": float(coef[0]), "c": float(coef[1]), "centres": {str(L): a for L, a in pts}}
    return {"judge": {"replicates": judge_rep, "t1": t1, "t_max": t_max, "delta_DP": DELTA_DP_2D},
            "corpus": {"Ls": list(Ls), "a_per_L": n_a, "replicates": n_rep, "runs": corpus.runs,
                       "site_updates": corpus.site_updates, "seconds": t_corpus},
            "fit_loss_last": float(loss[-1]), "per_L": per_L, "extrapolation": fit,
            "nu_perp": NU_PERP_DP_2D}


def main():
    import argparse
    import json
    ap = argparse.ArgumentParser(description="surrogate-guided vs uniform search for the DP critical point")
    ap.add_argument("--Ls", default="64,128,256,512,1024")
    ap.add_argument("--n-a", type=int, default=40)
    ap.add_argument("--n-rep", type=int, default=15)
    ap.add_argument("--judge-L", type=int, default=512)
    ap.add_argument("--judge-rep", type=int, default=8)
    ap.add_argument("--t-max", type=float, default=1000.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--judge-Ls", default="", help="comma list: judge at every side and extrapolate a_c(L)")
    a = ap.parse_args()
    ctx = api.Context(0)
    if a.judge_Ls:
        res = critical_point_vs_L(ctx, tuple(int(x) for x in a.judge_Ls.split(",")),
                                  tuple(int(x) for x in a.Ls.split(",")), a.n_a, a.n_rep, a.judge_rep, a.t_max,
                                  a.t_max / 10, a.seed)
        print(json.dumps(res))
        return
    res = critical_point_study(ctx, tuple(int(x) for x in a.Ls.split(",")), a.n_a, a.n_rep, a.judge_L,
                               a.judge_rep, a.t_max, a.t_max / 10, a.seed)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
