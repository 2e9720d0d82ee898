"""Failure detection, in forms that fault no GPU.

The reference checks every new state for NaN/Inf and negative densities, logs
them and exits (multiSPDP.cpp:2949-2955, 3186-3195, 3237-3255;
rietkerk_bjork_FKE.cpp:4352-4370).  The library reports the same conditions as
per-instance TM_STATUS_* bits and bounded device waits as TM_ERR_TIMEOUT.
These tests make each condition happen on purpose:

  * NaN, +Inf and negative values planted in an initial frame on the host;
  * a negative density produced by a step (a negative loss coefficient b) and
    an explicitly unstable Rietkerk step (dt far above the diffusion bound);
  * the samplers' rejection loops capped at one attempt (TM_PROBE_SAMPLER_CAP1);
  * a tile-copy wait and a tensor-core commit wait that run out with nothing in
    flight (TM_PROBE_TILE_WAIT, TM_PROBE_MLP_WAIT), after which the same
    context must still compute correct results.

The oracle sees the same inputs and must report the same bits; where its
arithmetic is the kernels' (everything but the +Inf draws), fields agree bit
for bit, NaNs included.
"""
import numpy as np
import pytest

NAN, NEG, CAP, WAIT = 0x1, 0x2, 0x4, 0x8


def _planted(L, dtype, kind, seed=0):
    rng = np.random.default_rng(seed)
    f = (1.0 + rng.uniform(-0.01, 0.01, (L, L))).astype(dtype)
    if kind == "nan":
        f[L // 3, L // 2] = np.nan
    elif kind == "inf":
        f[L // 2, 1] = np.inf
    elif kind == "neg":
        f[2, L - 3] = -0.25
    return f


# --------------------------------------------------------------- oracle (CPU)
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_oracle_reports_planted_values(oracle, dtype):
    p = oracle.dp_params(a=0.72)
    for kind, bit in (("clean", 0), ("nan", NAN), ("inf", NAN), ("neg", NEG)):
        _, _, _, st = oracle.dp_run(p, _planted(16, dtype, kind), 3, 0, [0])
        assert st == bit, kind
    rk = oracle.rk_params()
    f = np.stack([_planted(16, dtype, "clean"), np.full((16, 16), 0.5, dtype), np.ones((16, 16), dtype)])
    f[2, 3, 4] = -1.0
    _, _, _, st = oracle.rk_run(rk, f, 1, 0, [0])
    assert st == NEG


def test_oracle_sampler_cap_one_attempt(oracle):
    # dense sites (Poisson mean ~ 85: the rejection sampler) with one attempt per loop
    rho = np.full((32, 32), 5.0)
    p = oracle.dp_params(a=0.72)
    try:
        oracle.set_sampler_cap(1)
        _, st1 = oracle.dp_step(p, rho, 3, 0)
    finally:
        oracle.set_sampler_cap(64)
    _, st64 = oracle.dp_step(p, rho, 3, 0)
    assert st1 & CAP and not st64 & CAP


# ------------------------------------------------------------------ GPU
@pytest.fixture(scope="module")
def tmg():
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as m
    return m


@pytest.fixture(scope="module")
def ctx(tmg):
    c = tmg.Context(0)
    yield c
    c.set_test_probe(0)


def _oracle_dp(oracle, model, a):
    return oracle.DPParams(a, 0.0, model.b, model.c, model.D, model.sigma, model.dt, model.dx, model.clamp_lo,
                           model.clamp_eps, model.remainder, model.sampler)


def _oracle_rk(oracle, m, R):
    return oracle.RKParams(R, m.alpha, m.k2, m.W0, m.gmax, m.k1, m.c, m.d, m.rW, m.DP, m.DW, m.DO, m.sigma, m.dt,
                           m.dx, m.clamp_lo, m.clamp_eps, m.sampler)


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_planted_values_in_initial_frame_set_status(tmg, oracle, ctx, prec):
    precision = tmg.TM_FP64 if prec == "f64" else tmg.TM_FP32
    dtype = np.float64 if prec == "f64" else np.float32
    kinds = ["clean", "nan", "inf", "neg"]
    Ls = [24, 40, 33, 64]
    seeds = [5, 6, 7, 8]
    init = [_planted(L, dtype, kd, k) for k, (L, kd) in enumerate(zip(Ls, kinds))]
    model = tmg.dp_model()
    b = tmg.Batch(ctx, model, tmg.instances(Ls, seeds, 0.72), precision)
    b.upload(init)
    _, st0 = b.advance(0)
    assert list(st0) == [0, NAN, NAN, NEG]
    _, st = b.advance(2)
    fin = b.download()
    for k, kd in enumerate(kinds):
        _, _, ofin, ost = oracle.dp_run(_oracle_dp(oracle, model, 0.72), init[k], seeds[k], 2, [])
        assert st[k] & st0[k] == st0[k]
        if kd != "inf":   # +Inf enters the samplers' special cases, where only the status is specified
            assert st[k] == ost, kd
            assert np.array_equal(fin[k], ofin, equal_nan=True), kd
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_negative_density_from_a_step_sets_status(tmg, oracle, ctx, prec):
    # b < 0 makes the Euler-exact remainder rho/(1 + b rho dt) change sign
    precision = tmg.TM_FP64 if prec == "f64" else tmg.TM_FP32
    dtype = np.float64 if prec == "f64" else np.float32
    model = tmg.dp_model(b=-20.0)
    Ls, seeds = [32, 48], [1, 2]
    init = [_planted(L, dtype, "clean", k) for k, L in enumerate(Ls)]
    b = tmg.Batch(ctx, model, tmg.instances(Ls, seeds, 0.72), precision)
    b.upload(init)
    _, st = b.advance(3)
    fin = b.download()
    for k in range(len(Ls)):
        _, _, ofin, ost = oracle.dp_run(_oracle_dp(oracle, model, 0.72), init[k], seeds[k], 3, [])
        assert st[k] & NEG
        assert st[k] == ost
        assert np.array_equal(fin[k], ofin, equal_nan=True)
    b.close()


@pytest.mark.gpu
def test_unstable_rietkerk_step_sets_status(tmg, oracle, ctx):
    # dt = 0.05 puts D_O dt / dx^2 = 5 far above the explicit stability bound: the
    # O field oscillates, goes negative, and overflows to Inf/NaN
    m = tmg.rietkerk_model(dt=0.05, deterministic=1)
    L = 32
    rng = np.random.default_rng(3)
    f0 = np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), 1.0 + rng.uniform(-0.1, 0.1, (L, L))])
    b = tmg.Batch(ctx, m, tmg.instances([L], [4], 0.9), tmg.TM_FP64)
    b.upload([f0])
    _, st2 = b.advance(2)
    _, st = b.advance(60)
    fin = b.download()[0]
    assert st2[0] & NEG
    assert st[0] & NAN
    want = f0.copy()
    for _ in range(62):
        want = oracle.rk_det_step(_oracle_rk(oracle, m, 0.9), want)
    assert np.array_equal(fin, want, equal_nan=True)
    b.close()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["f64", "f32"])
def test_sampler_cap_probe(tmg, oracle, ctx, prec):
    precision = tmg.TM_FP64 if prec == "f64" else tmg.TM_FP32
    dtype = np.float64 if prec == "f64" else np.float32
    model = tmg.dp_model()
    Ls, seeds = [32, 64], [3, 9]
    init = [np.full((L, L), 5.0, dtype) for L in Ls]   # Poisson means ~ 85: the rejection sampler
    ctx.set_test_probe(tmg._lib.TM_PROBE_SAMPLER_CAP1)
    try:
        b = tmg.Batch(ctx, model, tmg.instances(Ls, seeds, 0.72), precision)
    finally:
        ctx.set_test_probe(0)
    b.upload(init)
    _, st = b.advance(2)
    fin = b.download()
    b.close()
    try:
        oracle.set_sampler_cap(1)
        for k in range(len(Ls)):
            _, _, ofin, ost = oracle.dp_run(_oracle_dp(oracle, model, 0.72), init[k], seeds[k], 2, [])
            assert st[k] & CAP
            assert st[k] == ost
            assert np.array_equal(fin[k], ofin)
    finally:
        oracle.set_sampler_cap(64)
    # the probe applied only to that batch
    b2 = tmg.Batch(ctx, model, tmg.instances(Ls, seeds, 0.72), precision)
    b2.upload(init)
    _, st2 = b2.advance(2)
    assert not (st2 & CAP).any()
    b2.close()


@pytest.mark.gpu
@pytest.mark.parametrize("det", [0, 1])
def test_tile_wait_runs_out_and_context_stays_usable(tmg, oracle, ctx, det):
    m = tmg.rietkerk_model(deterministic=det)
    Ls, seeds = [128, 96], [2, 3]
    rng = np.random.default_rng(1)
    f0 = [np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.ones((L, L))]).astype(np.float32)
          for L in Ls]
    ctx.set_test_probe(tmg._lib.TM_PROBE_TILE_WAIT)
    try:
        b = tmg.Batch(ctx, m, tmg.instances(Ls, seeds, 0.9), tmg.TM_FP32)
    finally:
        ctx.set_test_probe(0)
    b.upload(f0)
    with pytest.raises(tmg.TMError) as ei:
        b.advance(1)
    assert ei.value.code == tmg._lib.TM_ERR_TIMEOUT
    st = np.zeros(len(Ls), np.uint32)
    import ctypes as C
    rc = tmg._lib.lib().tm_batch_advance(b.handle, 0, None, 0, None, st.ctypes.data_as(C.POINTER(C.c_uint32)))
    assert rc == tmg._lib.TM_ERR_TIMEOUT and (st & WAIT).all()
    b.close()
    # the same context computes correctly afterwards
    b2 = tmg.Batch(ctx, m, tmg.instances(Ls, seeds, 0.9), tmg.TM_FP32)
    b2.upload(f0)
    _, st2 = b2.advance(2)
    fin = b2.download()
    b2.close()
    assert not st2.any()
    for k in range(len(Ls)):
        if det:
            want = f0[k]
            for _ in range(2):
                want = oracle.rk_det_step(_oracle_rk(oracle, m, 0.9), want)
        else:
            _, _, want, _ = oracle.rk_run(_oracle_rk(oracle, m, 0.9), f0[k], seeds[k], 2, [])
        assert np.array_equal(fin[k], want)


@pytest.mark.gpu
def test_mlp_wait_runs_out_and_parameters_stay(tmg, ctx):
    from oracle import surrogate_oracle as so
    from trophic_maelstorm_gb300 import surrogate as sg
    rng = np.random.default_rng(0)
    x = rng.normal(size=(300, 3)).astype(np.float32)
    t = np.stack([np.sin(x[:, 0]), np.cos(x[:, 1])], 1).astype(np.float32)
    p = sg.init_params(2)
    net = sg.MLP(ctx, p)
    net.set_data(x, t)
    ctx.set_test_probe(tmg._lib.TM_PROBE_MLP_WAIT)
    try:
        with pytest.raises(tmg.TMError) as e1:
            net.predict(x)
        assert e1.value.code == tmg._lib.TM_ERR_TIMEOUT
        with pytest.raises(tmg.TMError) as e2:
            net.train(2, lr=1e-2)
        assert e2.value.code == tmg._lib.TM_ERR_TIMEOUT
    finally:
        ctx.set_test_probe(0)
    assert np.array_equal(net.get_params(), p)
    y = net.predict(x)
    want, _ = so.forward(p, x)
    assert np.linalg.norm(y - want) <= 2e-3 * np.linalg.norm(want)
    net.train(1, lr=1e-3)
    assert not np.array_equal(net.get_params(), p)
    net.close()
