"""CPU restatement of the surrogate network's arithmetic (TEST INFRASTRUCTURE ONLY).

Only tests/ import this module: it is the checker for the BF16 forward,
backward and Adam kernels of trophic_maelstorm_gb300/csrc/tm_mlp.cu, never
a path the library takes.  The reference has no learned part; this network is
defined here, so the restatement below is its specification.

Network (input features f = (a, log L, log t) after the caller's affine
normalisation; outputs y = (log mean rho, survival fraction) in the caller's
scaling):

    z1 = W1 f + b1            W1: 128 x 3     (FP32 arithmetic, BF16 weights)
    h1 = bf16(gelu(z1))
    a2 = h1 W2^T + b2         W2: 128 x 128   (BF16 x BF16, FP32 accumulation)
    h2 = bf16(gelu(a2))
    a3 = h2 W3^T + b3         W3: 128 x 128
    h3 = gelu(a3)             (FP32)
    y  = W4 h3 + b4           W4: 2 x 128

gelu is the tanh form 0.5 x (1 + tanh(sqrt(2/pi)(x + 0.044715 x^3)))
(Hendrycks & Gimpel 2016).  Every weight matrix is used as its BF16 rounding
(round to nearest even) of the FP32 master copy; biases stay FP32.

Loss: sum over samples of w0 (y0 - t0)^2 + w1 (y1 - t1)^2, times inv_norm.
Backward (the kernel's rounding points):

    dy   = 2 w (y - t) inv_norm
    dz3  = bf16(dy W4 * gelu'(a3))      the MMA operand of both GEMMs below
    dz2  = bf16((dz3 W3) * gelu'(a2))
    dz1  = (dz2 W2) * gelu'(z1)         (FP32)
    gW4 = dy^T h3, gW3 = dz3^T h2, gW2 = dz2^T h1, gW1 = dz1^T f, gb = column sums

Adam (Kingma & Ba 2015) on the FP32 masters with host-computed bias
corrections c1 = 1/(1 - beta1^t), c2 = 1/(1 - beta2^t):

    m = beta1 m + (1 - beta1) g;  v = beta2 v + (1 - beta2) g g
    p = p - lr (m c1) / (sqrt(v c2) + eps)

Parameter vector layout (FP32, NPARAMS values): W1 | b1 | W2 | b2 | W3 | b3 | W4 | b4,
matrices row-major [out][in].
"""
from __future__ import annotations

import numpy as np

H = 128
N_IN = 3
N_OUT = 2
SEGMENTS = (("W1", (H, N_IN)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
            ("W4", (N_OUT, H)), ("b4", (N_OUT,)))
OFFSETS = {}
_o = 0
for _n, _s in SEGMENTS:
    OFFSETS[_n] = (_o, _s)
    _o += int(np.prod(_s))
NPARAMS = _o

F32 = np.float32
GELU_C = F32(0.7978845608028654)   # sqrt(2/pi)
GELU_K = F32(0.044715)


def unpack(p):
    p = np.asarray(p, F32)
    return {n: p[o:o + int(np.prod(s))].reshape(s) for n, (o, s) in OFFSETS.items()}


def pack(d):
    out = np.zeros(NPARAMS, F32)
    for n, (o, s) in OFFSETS.items():
        out[o:o + int(np.prod(s))] = np.asarray(d[n], F32).reshape(-1)
    return out


def bf16(x):
    """Round FP32 values to the nearest BF16 (ties to even), returned as FP32."""
    x = np.ascontiguousarray(x, F32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(F32)
    return np.where(np.isnan(x), x, out).astype(F32)


def gelu(a):
    a = a.astype(F32)
    th = np.tanh(GELU_C * (a + GELU_K * (a * a * a))).astype(F32)
    return (F32(0.5) * a * (F32(1) + th)).astype(F32)


def gelu_grad(a):
    a = a.astype(F32)
    th = np.tanh(GELU_C * (a + GELU_K * (a * a * a))).astype(F32)
    return (F32(0.5) * (F32(1) + th) +
            F32(0.5) * a * (F32(1) - th * th) * GELU_C * (F32(1) + F32(3) * GELU_K * (a * a))).astype(F32)


def _mm(a, b):
    """FP32-accumulated product of FP32 operands (the order of the sums is free)."""
    return (a.astype(np.float64) @ b.astype(np.float64)).astype(F32)


def forward(params, f, rounding=True):
    q = unpack(params)
    r = bf16 if rounding else (lambda x: np.asarray(x, F32))
    W1, W2, W3, W4 = (r(q[n]) for n in ("W1", "W2", "W3", "W4"))
    f = np.asarray(f, F32)
    z1 = ((W1[:, 0][None] * f[:, 0:1] + W1[:, 1][None] * f[:, 1:2]) + W1[:, 2][None] * f[:, 2:3]) + q["b1"][None]
    z1 = z1.astype(F32)
    h1 = r(gelu(z1))
    a2 = (_mm(h1, W2.T) + q["b2"][None]).astype(F32)
    h2 = r(gelu(a2))
    a3 = (_mm(h2, W3.T) + q["b3"][None]).astype(F32)
    h3 = gelu(a3)
    y = (_mm(h3, W4.T) + q["b4"][None]).astype(F32)
    return y, dict(f=f, z1=z1, h1=h1, a2=a2, h2=h2, a3=a3, h3=h3, W1=W1, W2=W2, W3=W3, W4=W4)


def loss_and_grad(params, f, t, w, inv_norm, rounding=True):
    """Loss (float64 sum of the FP32 per-sample terms) and the FP32 gradient vector."""
    r = bf16 if rounding else (lambda x: np.asarray(x, F32))
    y, c = forward(params, f, rounding)
    t = np.asarray(t, F32)
    w = np.asarray(w, F32)
    e = (y - t).astype(F32)
    per = (w[:, 0] * e[:, 0] * e[:, 0] + w[:, 1] * e[:, 1] * e[:, 1]).astype(F32)
    loss = float(per.astype(np.float64).sum()) * float(inv_norm)
    dy = ((F32(2) * w) * e * F32(inv_norm)).astype(F32)
    g = {"W4": _mm(dy.T, c["h3"]), "b4": dy.astype(np.float64).sum(0).astype(F32)}
    dz3 = r((_mm(dy, c["W4"]) * gelu_grad(c["a3"])).astype(F32))
    g["W3"] = _mm(dz3.T, c["h2"])
    g["b3"] = dz3.astype(np.float64).sum(0).astype(F32)
    dz2 = r((_mm(dz3, c["W3"]) * gelu_grad(c["a2"])).astype(F32))
    g["W2"] = _mm(dz2.T, c["h1"])
    g["b2"] = dz2.astype(np.float64).sum(0).astype(F32)
    dz1 = (_mm(dz2, c["W2"]) * gelu_grad(c["z1"])).astype(F32)
    g["W1"] = _mm(dz1.T, c["f"])
    g["b1"] = dz1.astype(np.float64).sum(0).astype(F32)
    return loss, pack(g)


def adam_step(p, m, v, g, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in the kernel's FP32 operation order; returns new (p, m, v)."""
    p, m, v, g = (np.asarray(x, F32).copy() for x in (p, m, v, g))
    b1, b2 = F32(beta1), F32(beta2)
    c1 = F32(1.0 / (1.0 - float(b1) ** step))      # host double arithmetic on the FP32 betas
    c2 = F32(1.0 / (1.0 - float(b2) ** step))
    m = (b1 * m + (F32(1) - b1) * g).astype(F32)
    v = (b2 * v + (F32(1) - b2) * (g * g)).astype(F32)
    p = (p - F32(lr) * (m * c1) / (np.sqrt((v * c2).astype(F32)) + F32(eps))).astype(F32)
    return p, m, v

