"""GPU kernels (through the C ABI) against the CPU oracle.

The kernels and the oracle implement one operation-by-operation specification
of the Dornic step (same Philox stream, same own log/exp, same evaluation
order), so fields must agree bit for bit in FP64 and in FP32; spatial means are
FP64 sums in a different order and must agree to 1e-12 relative; active-site
counts exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MEAN_RTOL = 1e-12


@pytest.fixture(scope="module")
def tmg():
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as m
    return m


@pytest.fixture(scope="module")
def ctx(tmg):
    return tmg.Context(0)


def _init_fields(Ls, seed, zeros=True):
    rng = np.random.default_rng(seed)
    out = []
    for L in Ls:
        f = 1.0 + rng.uniform(-0.01, 0.01, (L, L))
        if zeros and L >= 4:
            f[: L // 2, : L // 3] = 0.0      # an absorbing patch
            f[L - 1, L - 1] = 1e-30          # a nearly empty site
        out.append(f)
    return out


def _oracle_dp_params(oracle, model, a, a_step):
    return oracle.DPParams(a, a_step, model.b, model.c, model.D, model.sigma, model.dt, model.dx, model.clamp_lo,
                           model.clamp_eps, model.remainder, model.sampler)


def _compare_dp(tmg, oracle, ctx, model, Ls, a, a_step, n_steps, meas, precision, seed0=11, init_seed=0,
                zeros=True):
    dtype = np.float64 if precision == tmg.TM_FP64 else np.float32
    seeds = [seed0 + 7 * k for k in range(len(Ls))]
    inst = tmg.instances(Ls, seeds, a, a_step)
    init = [f.astype(dtype) for f in _init_fields(Ls, init_seed, zeros)]
    b = tmg.Batch(ctx, model, inst, precision)
    b.upload(init)
    obs, st = b.advance(n_steps, meas)
    fin = b.download()
    aa = np.broadcast_to(np.asarray(a, float), (len(Ls),))
    asx = np.broadcast_to(np.asarray(a_step, float), (len(Ls),))
    for k, L in enumerate(Ls):
        p = _oracle_dp_params(oracle, model, aa[k], asx[k])
        m, act, ofin, ost = oracle.dp_run(p, init[k], seeds[k], n_steps, meas)
        assert np.array_equal(fin[k], ofin), (k, L, np.max(np.abs(fin[k] - ofin)))
        np.testing.assert_allclose(obs[:, k, 0], m, rtol=MEAN_RTOL, atol=0)
        assert np.array_equal(obs[:, k, 1], act), (k, L)
        assert st[k] == ost, (k, st[k], ost)
    b.close()
    return obs, st, fin


LS = [1, 3, 8, 33, 64, 100]


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("sampler", [0, 1, 2], ids=["exact", "gauss100", "off"])
@pytest.mark.parametrize("remainder", [0, 1], ids=["euler", "rk4"])
def test_dp_step_matches_oracle(tmg, oracle, ctx, precision, sampler, remainder):
    model = tmg.dp_model(b=2.0, D=1.0, sigma=1.0, dt=0.1, remainder=remainder, sampler=sampler)
    _compare_dp(tmg, oracle, ctx, model, LS, 0.72, 0.0, 6, [0, 1, 3, 6], precision)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_dp_graph_chunks_and_ramp(tmg, oracle, ctx, precision):
    # 100 steps: graph replays of 32 steps between measurements, direct steps around them;
    # a ramped 0.72 -> 0.70 as in the 128^2 workload
    model = tmg.dp_model()
    n = 100
    _compare_dp(tmg, oracle, ctx, model, [16, 40, 128], 0.72, (0.70 - 0.72) / n, n, [0, 5, 37, 38, 100],
                precision)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_dp_multisp_clamp_and_first_order(tmg, oracle, ctx, precision):
    # multiSPDP semantics: RK4 remainder, Gaussian above 100, clamp [-1e-80, 1e-12) -> 0
    m1 = tmg.dp_model(b=2.0, remainder=1, sampler=1, clamp_lo=-1e-80, clamp_eps=1e-12)
    _compare_dp(tmg, oracle, ctx, m1, [8, 50], 0.72, 0.0, 20, [0, 10, 20], precision)
    # first-order model: a < 0, b < 0, cubic c > 0 (stochasticSPDP.cpp:1766-1805)
    m2 = tmg.dp_model(b=-2.0, c=1.0, remainder=1)
    _compare_dp(tmg, oracle, ctx, m2, [8, 50], -0.7, 0.0, 20, [0, 10, 20], precision)


def test_dp_extinction(tmg, oracle, ctx):
    model = tmg.dp_model(b=2.0)
    Ls = [8, 12]
    inst = tmg.instances(Ls, [1, 2], -5.0)  # strongly absorbing
    init = [np.zeros((8, 8)), np.zeros((12, 12))]
    init[0][3, 3] = 1e-3
    init[1][5, 5] = 1.0
    b = tmg.Batch(ctx, model, inst, tmg.TM_FP64)
    b.upload(init)
    meas = [0, 1, 2, 5, 10, 40, 60]
    obs, st = b.advance(60, meas)
    fin = b.download()
    for k in range(2):
        p = oracle.DPParams(-5.0, 0.0, 2.0, 0.0, 1.0, 1.0, 0.1, 1.0, 0.0, 0.0, 0, 0)
        m, act, ofin, _ = oracle.dp_run(p, init[k], k + 1, 60, meas)
        np.testing.assert_allclose(obs[:, k, 0], m, rtol=MEAN_RTOL, atol=0)
        assert np.array_equal(obs[:, k, 1], act)
        assert np.array_equal(fin[k], ofin)
    assert obs[-1, :, 1].sum() == 0  # both extinct by t = 6
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_launch_shape_and_path_invariance(tmg, ctx, precision):
    """Rows per task, CTAs per SM and graph vs direct launches change nothing."""
    model = tmg.dp_model()
    Ls = [64, 128, 96]
    inst = tmg.instances(Ls, [5, 6, 7], 0.72)
    dtype = np.float64 if precision == 0 else np.float32
    init = [f.astype(dtype) for f in _init_fields(Ls, 3)]
    res = []
    for rows, ctas, chunks in ((8, 4, [70]), (4, 2, [70]), (16, 8, [70]), (16, 1, [1] * 70), (1, 4, [70]),
                               (2, 3, [70])):
        b = tmg.Batch(ctx, model, inst, precision)
        b.set_launch(rows, ctas)
        b.upload(init)
        for c in chunks:
            b.advance(c)
        res.append(b.download_packed())
        b.close()
    for r in res[1:]:
        assert np.array_equal(r, res[0])


def test_upload_paths_agree(tmg, ctx):
    """Uploads from pageable memory (copy engines), from page-locked memory (copy kernel)
    and from page-locked memory 4 bytes off a 16-byte boundary (copy engines) leave the
    same state, and the check of the uploaded state runs on each."""
    torch = pytest.importorskip("torch")
    Ls = [64, 33, 100]
    inst = tmg.instances(Ls, [1, 2, 3], 0.72)
    b = tmg.Batch(ctx, tmg.dp_model(), inst, tmg.TM_FP32)
    init = tmg.pack([f.astype(np.float32) for f in _init_fields(Ls, 4)], inst, 1, np.float32)
    b.upload(init)
    assert np.array_equal(b.download_packed(), init)
    pinned = torch.empty(init.size + 1, dtype=torch.float32, pin_memory=True)
    pn = pinned.numpy()
    pn[:init.size] = init
    b.upload(pn[:init.size])
    assert np.array_equal(b.download_packed(), init)
    pn[1:] = init
    b.upload(pn[1:])
    assert np.array_equal(b.download_packed(), init)
    _, off, _ = tmg.layout(inst, 1)
    pn[:init.size] = init
    pn[off[1] + 5] = -1.0
    b.upload(pn[:init.size])
    _, st = b.advance(0, [])
    assert st.tolist() == [0, tmg.TM_STATUS_NEGATIVE, 0]
    b.close()


def test_small_batch_gets_short_tasks(tmg, ctx):
    """A batch with too few 8-row tasks to fill the GPU starts with fewer rows per task
    (one 128^2 lattice: 64 tasks of 8 rows); a large batch keeps 8."""
    small = tmg.Batch(ctx, tmg.dp_model(), tmg.instances([128], [1], 0.72), 0)
    assert small.get_launch()[0] < 8
    small.close()
    big = tmg.Batch(ctx, tmg.dp_model(), tmg.instances([1024] * 4, [1, 2, 3, 4], 0.72), 1)
    assert big.get_launch()[0] == 8
    big.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("sampler", [1, 0], ids=["gauss100", "exact"])
def test_rietkerk_matches_oracle(tmg, oracle, ctx, precision, sampler):
    model = tmg.rietkerk_model(sampler=sampler)
    Ls = [5, 16, 37]
    R = [0.6, 0.9, 1.2]
    dtype = np.float64 if precision == 0 else np.float32
    rng = np.random.default_rng(1)
    init = [np.stack([rng.uniform(0, 1, (L, L)), np.full((L, L), 0.5), np.full((L, L), 1.0)]).astype(dtype)
            for L in Ls]
    inst = tmg.instances(Ls, [3, 4, 5], R)
    b = tmg.Batch(ctx, model, inst, precision)
    b.upload(init)
    meas = [0, 7, 15]
    obs, st = b.advance(15, meas)
    fin = b.download()
    for k, L in enumerate(Ls):
        p = oracle.rk_params(R=R[k], sampler=sampler)
        m, act, ofin, ost = oracle.rk_run(p, init[k], [3, 4, 5][k], 15, meas)
        assert np.array_equal(fin[k], ofin), (k, np.max(np.abs(fin[k] - ofin)))
        np.testing.assert_allclose(obs[:, k, :3], m, rtol=MEAN_RTOL, atol=0)
        assert np.array_equal(obs[:, k, 3], act)
        assert st[k] == ost
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_rietkerk_ensemble_matches_reference(tmg, ctx, golden, precision):
    """The GPU's stochastic Rietkerk step against replicates of the reference's step (its
    P-Dornic loop with libstdc++ draws, its compiled remainder RK4, the clamp): 400
    replicates of 500 steps, one batch; final mean P, W, O, occupied sites, two sites."""
    from conftest import rk_ensemble_rows, assert_same_ensemble
    g = golden["rk_ens"]
    L, R, sigma, dt, steps, n_rep, _, eps = g["meta"]
    L, steps, n_rep = int(L), int(steps), int(n_rep)
    dtype = np.float64 if precision == 0 else np.float32
    model = tmg.rietkerk_model(sigma=sigma, dt=dt, clamp_eps=eps)
    inst = tmg.instances([L] * n_rep, list(range(n_rep)), R)
    b = tmg.Batch(ctx, model, inst, precision)
    b.upload([g["start"].astype(dtype)] * n_rep)
    _, st = b.advance(steps, [steps])
    assert not st.any()
    fins = b.download()
    b.close()
    assert_same_ensemble(rk_ensemble_rows(fins), g["rows"], g["columns"])


def test_rietkerk_noise_off_matches_reference(tmg, ctx, golden):
    """Noise-off Rietkerk RK4 (f_2D / RK4_Integrate) on the GPU against the reference's
    own output, to 1e-10 relative (the noise-off parity bar)."""
    g = golden["pins"]
    for tag in ("rkdet_a", "rkdet_b"):
        L, n, dt, R = g[f"{tag}_meta"]
        L, n = int(L), int(n)
        model = tmg.rietkerk_model(dt=dt, deterministic=1)
        b = tmg.Batch(ctx, model, tmg.instances([L], [0], R), tmg.TM_FP64)
        b.upload([g[f"{tag}_in"]])
        b.advance(n)
        out = b.download()[0]
        np.testing.assert_allclose(out, g[f"{tag}_out"], rtol=1e-10, atol=0)
        b.close()


@pytest.mark.parametrize("stencil", [5, 9])
@pytest.mark.parametrize("integrator", [0, 1])
def test_dp_noise_off_lattice_matches_oracle(tmg, oracle, ctx, stencil, integrator):
    model = tmg.dp_model(b=2.0, c=0.5, D=1.0, dt=0.05, deterministic=1, stencil=stencil, integrator=integrator)
    Ls = [7, 32]
    init = _init_fields(Ls, 4, zeros=False)
    b = tmg.Batch(ctx, model, tmg.instances(Ls, [0, 0], 0.8), tmg.TM_FP64)
    b.upload(init)
    b.advance(12)
    fin = b.download()
    for k in range(2):
        r = init[k]
        for _ in range(12):
            r = oracle.dp_det_step(r, 0.8, 2.0, 0.5, 1.0, 0.05, 1.0, stencil=stencil, integrator=integrator)
        assert np.array_equal(fin[k], r)
    b.close()


def test_dp_noise_off_4th_order_matches_reference(tmg, ctx, golden):
    g = golden["pins"]
    L, a, b_, D, dt, dx = g["nodiff_meta"]
    model = tmg.dp_model(b=b_, D=D, dt=dt, dx=dx, deterministic=1, stencil=9, integrator=1)
    b = tmg.Batch(ctx, model, tmg.instances([int(L)], [0], a), tmg.TM_FP64)
    b.upload([g["nodiff_in"]])
    frames = []
    for _ in range(10):
        b.advance(1)
        frames.append(b.download()[0])
    got = np.array([frames[0], frames[4], frames[9]])
    np.testing.assert_allclose(got, g["nodiff_out"], rtol=1e-10, atol=0)
    b.close()


def test_full_size_step_matches_oracle(tmg, oracle, ctx):
    """Two steps of a 1024^2 FP32 lattice, bit for bit."""
    model = tmg.dp_model()
    L = 1024
    rng = np.random.default_rng(2)
    init = (1.0 + rng.uniform(-0.01, 0.01, (L, L))).astype(np.float32)
    b = tmg.Batch(ctx, model, tmg.instances([L], [99], 0.72), tmg.TM_FP32)
    b.upload([init])
    obs, st = b.advance(2, [0, 2])
    fin = b.download()[0]
    p = oracle.dp_params(a=0.72)
    m, act, ofin, ost = oracle.dp_run(p, init, 99, 2, [0, 2])
    assert np.array_equal(fin, ofin)
    np.testing.assert_allclose(obs[:, 0, 0], m, rtol=MEAN_RTOL)
    assert np.array_equal(obs[:, 0, 1], act)
    b.close()


def test_one_shot_call_equals_batch(tmg, ctx):
    model = tmg.dp_model()
    Ls = [24, 64]
    inst = tmg.instances(Ls, [3, 4], 0.72)
    init = tmg.pack(_init_fields(Ls, 9), inst, 1, np.float32)
    obs1, st1, fin1 = tmg.run_dp(ctx, model, inst, init, 40, [0, 20, 40], tmg.TM_FP32)
    b = tmg.Batch(ctx, model, inst, tmg.TM_FP32)
    b.upload(init)
    obs2, st2 = b.advance(40, [0, 20, 40])
    assert np.array_equal(obs1, obs2) and np.array_equal(fin1, b.download_packed())
    b.close()


def test_reproducible_per_seed(tmg, ctx):
    model = tmg.dp_model()
    inst = tmg.instances([256, 512], [1, 2], 0.72)
    init = tmg.pack(_init_fields([256, 512], 1), inst, 1, np.float32)
    outs = []
    for _ in range(2):
        obs, st, fin = tmg.run_dp(ctx, model, inst, init, 50, [50], tmg.TM_FP32)
        outs.append((obs, fin))
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    inst2 = tmg.instances([256, 512], [3, 2], 0.72)
    obs, st, fin = tmg.run_dp(ctx, model, inst2, init, 50, [50], tmg.TM_FP32)
    assert not np.array_equal(fin[:256 * 256], outs[0][1][:256 * 256])
    assert np.array_equal(fin[256 * 256:], outs[0][1][256 * 256:])


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("tag,n_rep", [("crit", 1500), ("active", 400), ("site", 3000)])
def test_gpu_ensemble_matches_reference(tmg, ctx, golden, tag, n_rep, precision):
    """percolation_dornic_2d on the GPU (every replicate in one batch) against the
    reference's ensembles at L = 8 near the absorbing transition, L = 8 active and a single
    site: rho(t) and survival within 3.5 combined standard errors, and the distribution of
    rho(t) over replicates by two-sample KS, p > 0.01 / n_t at every time."""
    from scipy import stats
    ens = golden["ens"]
    L, a, b, D, sig, dt, dx = ens[f"{tag}_meta"]
    t = ens[f"{tag}_t"]
    steps = np.rint(t / dt).astype(np.int64)
    dtype = np.float64 if precision == 0 else np.float32
    inst = tmg.instances([int(L)] * n_rep, range(5000, 5000 + n_rep), a)
    model = tmg.dp_model(b=b, D=D, sigma=sig, dt=dt, dx=dx)
    init = tmg.pack([ens[f"{tag}_rho0"]] * n_rep, inst, 1, dtype)
    obs, st, _ = tmg.run_dp(ctx, model, inst, init, int(steps[-1]), steps, precision)
    assert not st.any()
    M, A = obs[:, :, 0].T, obs[:, :, 1].T
    R, RA = ens[f"{tag}_mean"], ens[f"{tag}_active"]
    n_t = len(t)
    for j in range(1, n_t):
        se = np.sqrt(M[:, j].var() / len(M) + R[:, j].var() / len(R))
        if se > 0:
            assert abs(M[:, j].mean() - R[:, j].mean()) < 3.5 * se, (tag, j)
        ps, pr = (A[:, j] > 0).mean(), (RA[:, j] > 0).mean()
        se_s = np.sqrt(ps * (1 - ps) / len(A) + pr * (1 - pr) / len(RA))
        if se_s > 0:
            assert abs(ps - pr) < 3.5 * se_s, (tag, j)
        if M[:, j].std() > 0 and R[:, j].std() > 0:
            assert stats.ks_2samp(M[:, j], R[:, j]).pvalue > 0.01 / n_t, (tag, j)


def test_reference_rows_shape(tmg, ctx):
    rows, st = tmg.percolation_dornic_2d([1.5, 2.0, 5.0], np.ones(64), 5.0, 0.72, 2.0, 1.0, 1.0, 0.1, 1.0, 8, 8,
                                         seed=3, ctx=ctx)
    assert rows.shape == (11 + 3, 8)
    assert np.allclose(rows[:, 0], 0.72) and np.allclose(rows[:, 1], 8)
    assert rows[0, 3] == pytest.approx(1.0) and rows[0, 5] == 8


def test_fp32_state_is_statistically_equivalent_to_fp64(tmg, ctx):
    """FP32 field state against FP64 near the critical point (same seeds): the
    ensemble mean density and survival agree within 3.5 combined standard errors and
    the replicate spatial means pass KS at p > 0.01 / n_t at every time."""
    from trophic_maelstorm_gb300 import study
    r = study.dp_precision_study(L=64, n_rep=96, a=0.53, t_max=100.0, seed=11)
    n_t = len(r["t"])
    assert r["status"] == [0, 0]
    assert r["max_abs_z_rho"] < 3.5 and r["max_abs_z_surv"] < 3.5
    assert r["min_ks_p"] > 0.01 / n_t


def test_sweep_rows_do_not_depend_on_the_split(tmg, ctx):
    """The sharded sweep's blocks (what each rank of critical_exp_delta(distributed=True)
    runs) reproduce the single-batch rows bit for bit: keys depend on the value, not the rank."""
    from trophic_maelstorm_gb300 import api
    args = (np.ones(16 * 16), 10.0, 2.0, 1.0, 1.0, 0.1, 1.0, 3, 16, 7, tmg.TM_FP32)
    avals = api.linspace(0.5, 0.6, 5)
    full = api._sweep_block(ctx, list(range(5)), avals, *args)
    parts = {}
    for rank in range(3):
        parts.update(api._sweep_block(ctx, api.shard_indices(5, rank, 3), avals, *args))
    for ia in range(5):
        assert np.array_equal(full[ia][0], parts[ia][0]) and np.array_equal(full[ia][1], parts[ia][1])


def test_full_sweep_batch_matches_oracle_on_sampled_instances(tmg, oracle, ctx):
    """The bench's whole workload -- L in {64..1024} x 32 replicates x 16 a (2560 instances,
    715,128,832 sites, FP32) -- advanced two steps in one batch: sampled instances of every L
    equal the oracle bit for bit, and every instance keeps a finite, non-negative state."""
    torch = pytest.importorskip("torch")
    LS, REPS, NA = (64, 128, 256, 512, 1024), 32, 16
    avals = np.geomspace(0.53 * 0.98, 0.53 * 1.02, NA)
    Ls, seeds, av = [], [], []
    for L in LS:
        for a in avals:
            for r in range(REPS):
                Ls.append(L); seeds.append(1_000_003 * len(Ls) + 17); av.append(float(a))
    inst = tmg.instances(Ls, seeds, av)
    b = tmg.Batch(ctx, tmg.dp_model(), inst, tmg.TM_FP32)
    total, off, _ = tmg.layout(inst, 1)
    buf = torch.zeros(total, dtype=torch.float32, device="cuda")
    for k, L in enumerate(Ls):
        buf[int(off[k]):int(off[k]) + L * L] = 1.0
    rng = np.random.default_rng(123)
    picks = [k for i, L in enumerate(LS) for k in (i * NA * REPS + int(rng.integers(NA * REPS)),)]
    picks.append(len(Ls) - 1)
    init = {}
    for k in picks:
        L = Ls[k]
        init[k] = (1.0 + rng.uniform(-0.01, 0.01, (L, L))).astype(np.float32)
        buf[int(off[k]):int(off[k]) + L * L] = torch.from_numpy(init[k].reshape(-1)).cuda()
    torch.cuda.synchronize()
    b.upload_device(buf.data_ptr())
    ctx.sync()
    del buf
    obs, st = b.advance(2, [2])
    assert int(np.bitwise_or.reduce(st)) == 0
    m = obs[0, :, 0]
    assert np.all(np.isfinite(m)) and np.all(m > 0)
    for k in picks:
        p = oracle.dp_params(a=av[k])
        _, _, want, _ = oracle.dp_run(p, init[k], seeds[k], 2, [2])
        assert np.array_equal(b.snapshot(k), want), (k, Ls[k])
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("R", [4, 8, 16])
def test_large_absorbing_regions_match_oracle(tmg, oracle, ctx, precision, R):
    """Lattices that are mostly absorbing (L = 20 < 32, ragged L = 70 and 128, one small
    occupied patch, subcritical a so the empty area grows), 80 steps for every task height:
    the fields equal the oracle bit for bit, also after an upload in the middle and across
    graph chunks."""
    dtype = np.float64 if precision == 0 else np.float32
    Ls = [20, 70, 128]
    rng = np.random.default_rng(R)
    init = []
    for L in Ls:
        f = np.zeros((L, L))
        f[L // 3: L // 3 + max(2, L // 6), L // 4: L // 4 + max(2, L // 5)] = rng.uniform(0.5, 1.5)
        init.append(f.astype(dtype))
    seeds = [31, 32, 33]
    inst = tmg.instances(Ls, seeds, 0.35)
    b = tmg.Batch(ctx, tmg.dp_model(), inst, precision)
    b.set_launch(R, 2)
    b.upload(init)
    b.advance(45)
    mid = b.download()
    b.upload(mid, step=45)
    b.advance(35)
    fin = b.download()
    for k, L in enumerate(Ls):
        p = oracle.dp_params(a=0.35)
        _, _, want, _ = oracle.dp_run(p, init[k], seeds[k], 80, [80])
        assert np.array_equal(fin[k], want), L
        assert np.count_nonzero(want) < 0.5 * L * L      # the skipped region exists
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_rietkerk_bulk_copied_tiles_match_oracle(tmg, oracle, ctx, precision):
    """Lattices where the RK4 tiles take the bulk-copy path (L % 4 == 0, tiles not wrapping
    in x: L = 200 and 256) beside ones that take per-thread loads (L = 130, L = 132): fields
    equal the oracle bit for bit."""
    model = tmg.rietkerk_model()
    Ls = [200, 256, 130, 132]
    R = [0.7, 0.9, 1.1, 1.0]
    dtype = np.float64 if precision == 0 else np.float32
    rng = np.random.default_rng(8)
    init = [np.stack([rng.uniform(0, 1, (L, L)), 0.5 + rng.uniform(-0.1, 0.1, (L, L)),
                      1.0 + rng.uniform(-0.1, 0.1, (L, L))]).astype(dtype) for L in Ls]
    seeds = [41, 42, 43, 44]
    inst = tmg.instances(Ls, seeds, R)
    b = tmg.Batch(ctx, model, inst, precision)
    b.upload(init)
    b.advance(6)
    fin = b.download()
    for k, L in enumerate(Ls):
        p = oracle.rk_params(R=R[k])
        _, _, want, _ = oracle.rk_run(p, init[k], seeds[k], 6, [6])
        assert np.array_equal(fin[k], want), L
    b.close()
