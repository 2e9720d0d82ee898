"""GPU tests of the rows next to the step: pattern wavelength (power spectrum),
checkpoint/resume, the command-line sweep driver and its CSV outputs."""
import os
import subprocess

import numpy as np
import pytest
from spectrum_restatement import spectrum_numpy

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tmg():
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as m
    return m


@pytest.fixture(scope="module")
def ctx(tmg):
    return tmg.Context(0)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("case", ["stripes32", "random33", "spots48", "zeros20", "hex64"])
def test_power_spectrum_matches_reference_estimator(tmg, ctx, precision, case):
    """Against the reference's own gen_FFT_PowerSpectra (glow_up.py:632-847), run on
    frames written by its save_frame (tests/golden/ref_spectrum.npz).  Empty bins:
    NaN there, 0 here.  FP64 state: 1e-9 of the largest power; FP32 state rounds the
    field once (2^-24 relative), so 2e-6."""
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_spectrum.npz"))
    f, rk, rp = g[f"{case}_field"], g[f"{case}_k"], g[f"{case}_power"]
    L = f.shape[0]
    dtype = np.float64 if precision == 0 else np.float32
    b = tmg.Batch(ctx, tmg.dp_model(), tmg.instances([L], [0], 0.72), precision)
    b.upload([f.astype(dtype)])
    kv, pw = b.power_spectrum(0)
    b.close()
    np.testing.assert_allclose(kv, rk, rtol=0, atol=1e-12)
    want = np.nan_to_num(rp, nan=0.0)
    tol = 1e-9 if precision == 0 else 2e-6
    np.testing.assert_allclose(pw, want, rtol=tol, atol=tol * max(1.0, want.max()))
    if np.isfinite(rp).any():
        assert tmg.pattern_wavelength(L, kv, pw) == pytest.approx(L / rk[np.nanargmax(rp)])


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("L", [16, 33, 128])
def test_power_spectrum_matches_reference_semantics(tmg, ctx, precision, L):
    rng = np.random.default_rng(L)
    y, x = np.mgrid[0:L, 0:L]
    lam = L / 4.0
    f = 1.0 + 0.5 * np.sin(2 * np.pi * x / lam) + 0.05 * rng.random((L, L))  # stripes, |k| = L/lam
    f = np.stack([f, rng.random((L, L)), np.zeros((L, L))])
    dtype = np.float64 if precision == 0 else np.float32
    b = tmg.Batch(ctx, tmg.rietkerk_model(), tmg.instances([L], [0], 0.9), precision)
    b.upload([f.astype(dtype)])
    for field in range(3):
        kv, pw = b.power_spectrum(0, field)
        rk, rp = spectrum_numpy(f[field].astype(dtype))
        np.testing.assert_allclose(kv, rk, rtol=0, atol=1e-12)
        np.testing.assert_allclose(pw, rp, rtol=1e-9, atol=1e-9 * max(1.0, rp.max()))
    kv, pw = b.power_spectrum(0, 0)
    if L % 4 == 0:
        assert tmg.pattern_wavelength(L, kv, pw) == pytest.approx(lam)
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_checkpoint_resume_is_bit_exact(tmg, ctx, tmp_path, precision):
    from trophic_maelstorm_gb300 import io
    dtype = np.float64 if precision == 0 else np.float32
    Ls = [32, 64]
    inst = tmg.instances(Ls, [11, 12], 0.72)
    rng = np.random.default_rng(0)
    init = [(1 + rng.uniform(-0.01, 0.01, (L, L))).astype(dtype) for L in Ls]
    full = tmg.Batch(ctx, tmg.dp_model(), inst, precision)
    full.upload(init)
    full.advance(80)
    ref = full.download_packed()
    half = tmg.Batch(ctx, tmg.dp_model(), inst, precision)
    half.upload(init)
    half.advance(45)
    path = str(tmp_path / "ck.npz")
    io.save_checkpoint(half, path)
    half.close()
    again = tmg.Batch(ctx, tmg.dp_model(), inst, precision)
    assert io.load_checkpoint(again, path) == 45
    again.advance(35)
    assert np.array_equal(again.download_packed(), ref)
    full.close()
    again.close()


def test_sweep_driver_matches_python_api(tmg, ctx, tmp_path):
    exe = os.path.join(REPO, "trophic_maelstorm_gb300", "lib", "tm_sweep")
    out = str(tmp_path / "sweep")
    r = subprocess.run([exe, "0.1", "5", "16", "6", "0.7", "0.8", "2", "0", "T", "--seed", "100", "--out", out],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    stats = [f for f in os.listdir(out) if f.startswith("T_P_c_Delta")]
    assert len(stats) == 1
    with open(os.path.join(out, stats[0])) as fh:
        head = fh.readline()
        got = np.loadtxt(fh, delimiter=",", ndmin=2)
    assert head.startswith(" a , L, t")
    # the same sweep through the Python API: 2 a-values x 6 replicates, seeds 100 + index
    t_meas = tmg.logarithm10_time_bins(5.0, 0.1)
    rows = []
    for ia, a in enumerate([0.7, 0.8]):
        rr, _ = tmg.percolation_dornic_2d(t_meas, np.ones(256), 5.0, a, 2.0, 1.0, 1.0, 0.1, 1.0, 6, 16,
                                          seed=100 + ia * 6, ctx=ctx)
        rows.append(rr)
    want = np.concatenate(rows)
    assert got.shape == want.shape
    np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-12)   # 6 printed digits
    assert len(os.listdir(os.path.join(out, "TimeSeries"))) == 2
    frames = sorted(f for f in os.listdir(out) if f.startswith("FRAME_"))
    assert len(frames) == 2
    from trophic_maelstorm_gb300 import io
    fr = io.read_frame(os.path.join(out, frames[0]), 16)
    assert fr.shape == (16, 16) and np.all(fr >= 0)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("remainder", [0, 1], ids=["euler", "rk4"])
def test_site_coefficient_field_matches_oracle(tmg, oracle, ctx, precision, remainder):
    """Per-site loss coefficient b_v (the Fortran RFT mound field) against the oracle, bit for bit."""
    dtype = np.float64 if precision == 0 else np.float32
    Ls = [24, 40]
    rng = np.random.default_rng(5)
    init = [(1 + rng.uniform(-0.01, 0.01, (L, L))).astype(dtype) for L in Ls]
    bv = []
    for L in Ls:
        y, x = np.mgrid[0:L, 0:L]
        mound = ((x - L / 2) ** 2 + (y - L / 3) ** 2) < (L / 5) ** 2
        bv.append(np.where(mound, 0.5, 2.0).astype(dtype))
    model = tmg.dp_model(b=2.0, c=0.3, remainder=remainder)
    inst = tmg.instances(Ls, [1, 2], 0.72)
    b = tmg.Batch(ctx, model, inst, precision)
    b.set_site_coeff(bv)
    b.upload(init)
    b.advance(12)
    fin = b.download()
    for k, L in enumerate(Ls):
        p = oracle.DPParams(0.72, 0.0, 2.0, 0.3, 1.0, 1.0, 0.1, 1.0, 0.0, 0.0, remainder, 0)
        r = init[k]
        for s in range(12):
            r, _ = oracle.dp_step_sb(p, r, [1, 2][k], s, bv[k])
        assert np.array_equal(fin[k], r)
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_box_means(tmg, ctx, precision):
    dtype = np.float64 if precision == 0 else np.float32
    L = 64
    rng = np.random.default_rng(1)
    f = rng.random((3, L, L)).astype(dtype)
    b = tmg.Batch(ctx, tmg.rietkerk_model(), tmg.instances([L], [0], 0.9), precision)
    b.upload([f])
    for field in range(3):
        for box in (1, 4, 16, 64):
            got = b.box_means(0, box, field)
            want = f[field].astype(np.float64).reshape(L // box, box, L // box, box).mean(axis=(1, 3))
            np.testing.assert_allclose(got, want, rtol=1e-12)
    b.close()


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
@pytest.mark.parametrize("tag,D,v,sigma", [("a", 1.0, 1.0, 1.5), ("b", 1.0, 2.0, 2.0)])
def test_fke_advdiff_matches_reference_fixture(tmg, oracle, precision, tag, D, v, sigma):
    """Consumer movement (advdiff_FKE_MultiSp) on the reference's own fixture, L = 24
    and L = 9 (stencils wrapping the lattice): the gather sums in another order than
    the reference's scatter, so FP64 agrees to rounding, FP32 to single precision."""
    pytest.importorskip("torch")
    g = np.load(os.path.join(REPO, "tests", "golden", "ref_fke.npz"))
    L = int(g[f"fke_{tag}_meta"][0])
    fields = [g[f"fke_{tag}_{k}"].reshape(L, L) for k in ("rho", "gamma", "vx", "vy")]
    p = tmg.fke_parameters(D, v, 1.0, sigma)
    dtype = np.float64 if precision == 0 else np.float32
    got = tmg.fke_advdiff(*[f.astype(dtype) for f in fields], p, precision=precision)
    want = g[f"fke_{tag}_out"].reshape(L, L)
    if precision == 0:
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-15)
    else:
        np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-6 * want.max())


@pytest.mark.parametrize("L,v", [(7, 3.0), (64, 1.0), (200, 4.0)])
def test_fke_advdiff_matches_oracle(tmg, oracle, L, v):
    """FP64 gather against the oracle's scatter on larger lattices: windowed gather
    (L = 64, 200) and the whole-lattice case (L = 7); extinct sites and a site
    just below eps included."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(L)
    rho = rng.uniform(0, 3, (L, L))
    rho[rng.random((L, L)) < 0.3] = 0.0
    rho[0, 1] = 5e-11
    gam = rng.uniform(0, 1, (L, L))
    vx = rng.uniform(-v, v, (L, L))
    vy = rng.uniform(-v, v, (L, L))
    p = tmg.fke_parameters(1.0, v, 1.0, 1.2)
    got = tmg.fke_advdiff(rho, gam, vx, vy, p)
    want = oracle.fke_advdiff(rho, gam, vx, vy, p.pref, p.gD, p.gV).reshape(L, L)
    np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-14)
    assert got.sum() == pytest.approx(rho[rho >= 1e-10].sum(), rel=1e-12)


@pytest.mark.parametrize("L", [9, 64, 256])
def test_fke_workspace_entry_point_matches_and_reference_scatter_agrees(tmg, oracle, L):
    """tm_fke_advdiff_device_ws on a reused workspace equals the allocating entry point
    bit for bit (two calls in a row), and both agree with a restatement of the
    reference's GPU scatter (updateMovement, FP64 atomics) to rounding."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(L + 1)
    rho = rng.uniform(0, 3, (L, L))
    rho[rng.random((L, L)) < 0.3] = 0.0
    gam = rng.uniform(0, 1, (L, L))
    vx = rng.uniform(-2.0, 2.0, (L, L))
    vy = rng.uniform(-2.0, 2.0, (L, L))
    p = tmg.fke_parameters(1.0, 2.0, 1.0, 1.2)
    dev = torch.device("cuda", 0)
    ts = [torch.as_tensor(x, dtype=torch.float64, device=dev) for x in (rho, gam, vx, vy)]
    ws = tmg.api.fke_workspace(L)
    a1 = tmg.fke_advdiff(*ts, p, workspace=ws).cpu().numpy()
    a2 = tmg.fke_advdiff(*ts, p, workspace=ws).cpu().numpy()
    ref = tmg.fke_advdiff(rho, gam, vx, vy, p)
    assert np.array_equal(a1, ref) and np.array_equal(a2, ref)
    lib = oracle.fke_scatter_lib()
    gD = torch.as_tensor(p.gD, dtype=torch.float64, device=dev)
    gV = torch.as_tensor(p.gV, dtype=torch.float64, device=dev)
    out = torch.empty_like(ts[0])
    s = torch.cuda.current_stream(dev)
    assert lib.tmo_fke_scatter_f64(*(t.data_ptr() for t in ts), L, p.pref, 1e-10, gD.data_ptr(), len(p.gD) - 1,
                                   gV.data_ptr(), len(p.gV) - 1, out.data_ptr(), s.cuda_stream) == 0
    np.testing.assert_allclose(ref, out.cpu().numpy(), rtol=1e-12, atol=1e-14)
    # the workspace entry point rejects a short or misaligned workspace
    from trophic_maelstorm_gb300 import _lib as T
    import ctypes as C
    args = [t.data_ptr() for t in ts] + [T.TM_FP64, L, p.pref, 1e-10, np.ascontiguousarray(p.gD).ctypes.data_as(
        C.POINTER(C.c_double)), len(p.gD) - 1, np.ascontiguousarray(p.gV).ctypes.data_as(C.POINTER(C.c_double)),
        len(p.gV) - 1, out.data_ptr()]
    need = T.lib().tm_fke_workspace_bytes(T.TM_FP64, L)
    base = (ws.data_ptr() + 255) // 256 * 256
    assert T.lib().tm_fke_advdiff_device_ws(*args, base, need - 1, s.cuda_stream) == T.TM_ERR_INVALID
    assert T.lib().tm_fke_advdiff_device_ws(*args, base + 8, need, s.cuda_stream) == T.TM_ERR_INVALID


@pytest.mark.parametrize("model,nf", [("multisp", 1), ("rietkerk", 3)])
def test_sweep_driver_other_models(tmg, tmp_path, model, nf):
    """tm_sweep with the MultiSp DP and the Rietkerk models: the sweep table, one
    prelim file per control value and a final frame of the model's fields."""
    from trophic_maelstorm_gb300 import io
    exe = os.path.join(REPO, "trophic_maelstorm_gb300", "lib", "tm_sweep")
    out = str(tmp_path / model)
    dt, tmax = ("0.1", "3") if model == "multisp" else ("0.002", "1.2")
    a1, a2 = ("0.7", "0.8") if model == "multisp" else ("0.9", "1.1")
    r = subprocess.run([exe, dt, tmax, "24", "3", a1, a2, "2", "0", "M", "--model", model, "--precision", "fp32",
                        "--seed", "5", "--out", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    stats = [f for f in os.listdir(out) if f.startswith("M_P_c_Delta")]
    assert len(stats) == 1
    with open(os.path.join(out, stats[0])) as fh:
        fh.readline()
        got = np.loadtxt(fh, delimiter=",", ndmin=2)
    assert got.shape[0] > 0 and np.all(np.isfinite(got))
    assert set(np.round(got[:, 0], 6)) == {float(a1), float(a2)}
    assert len(os.listdir(os.path.join(out, "TimeSeries"))) == 2
    frames = sorted(f for f in os.listdir(out) if f.startswith("FRAME_"))
    assert len(frames) == 2
    fr = io.read_frame(os.path.join(out, frames[0]), 24, nf)
    assert np.all(np.isfinite(fr)) and np.all(fr >= 0)
