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
