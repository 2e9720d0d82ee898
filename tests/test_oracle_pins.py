"""The oracle against the reference's own code (golden fixtures made by
tests/golden/gen_golden.py from the compiled reference sources)."""
import os

import numpy as np
import pytest
from scipy import stats


def test_philox_known_answers(oracle):
    # Random123 known-answer vectors for Philox4x32-10
    assert [hex(v) for v in oracle.philox([0, 0, 0, 0], [0, 0])] == \
        ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(v) for v in oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == \
        ["0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(v) for v in oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                                          [0xA4093822, 0x299F31D0])] == \
        ["0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


@pytest.mark.parametrize("tag", ["rkdet_a", "rkdet_b"])
def test_rietkerk_noise_off_rk4_matches_reference(oracle, golden, tag):
    g = golden["pins"]
    L, n, dt, R = g[f"{tag}_meta"]
    p = oracle.rk_params(R=R, dt=dt)
    f = g[f"{tag}_in"].copy()
    for _ in range(int(n)):
        f = oracle.rk_det_step(p, f)
    ref = g[f"{tag}_out"]
    np.testing.assert_allclose(f, ref, rtol=1e-10, atol=0)
    assert np.array_equal(f, ref)  # same operation order: identical bits


def test_rietkerk_stochastic_remainder_matches_reference(oracle, golden):
    g = golden["pins"]
    f = oracle.rk_remainder(oracle.rk_params(R=0.9, dt=1e-3), g["rkrem_in"])
    np.testing.assert_allclose(f, g["rkrem_out"], rtol=1e-10, atol=0)
    assert np.array_equal(f, g["rkrem_out"])


def test_multisp_rk4_remainder_matches_reference(oracle, golden):
    g = golden["pins"]
    x = oracle.dp_remainder(oracle.dp_params(b=2.0, dt=0.1, remainder=oracle.REM_RK4), g["msrem_in"])
    assert np.array_equal(x, g["msrem_out"])


def test_first_order_rk4_remainder_matches_reference(oracle, golden):
    g = golden["pins"]
    x = oracle.dp_remainder(oracle.dp_params(b=-2.0, c=1.0, dt=0.1, remainder=oracle.REM_RK4), g["forem_in"])
    assert np.array_equal(x, g["forem_out"])


def test_dp_noise_off_4th_order_matches_reference(oracle, golden):
    g = golden["pins"]
    L, a, b, D, dt, dx = g["nodiff_meta"]
    r = g["nodiff_in"].copy()
    frames = []
    for _ in range(10):
        r = oracle.dp_det_step(r, a, b, 0.0, D, dt, dx, stencil=9, integrator=1)
        frames.append(r)
    got = np.array([frames[0], frames[4], frames[9]])
    np.testing.assert_allclose(got, g["nodiff_out"], rtol=1e-10, atol=0)


def _oracle_ensemble(oracle, ens, tag, n_rep, seed0=1000):
    L, a, b, D, sig, dt, dx = ens[f"{tag}_meta"]
    steps = np.rint(ens[f"{tag}_t"] / dt).astype(np.int64)
    p = oracle.dp_params(a=a, b=b, D=D, sigma=sig, dt=dt, dx=dx)
    M, A = [], []
    for k in range(n_rep):
        m, act, _, st = oracle.dp_run(p, ens[f"{tag}_rho0"], seed0 + k, int(steps[-1]), steps)
        assert st == 0
        M.append(m); A.append(act)
    return np.array(M), np.array(A)


@pytest.mark.parametrize("tag,n_rep", [("crit", 1500), ("active", 400), ("site", 3000)])
def test_dp_ensemble_matches_reference(oracle, golden, tag, n_rep):
    """rho(t), survival and the distribution of rho(t) over replicates agree with the
    reference's percolationDornic_2D ensemble: means within 3 combined standard errors,
    two-sample KS p > 0.01 at every time (Bonferroni over the time points)."""
    ens = golden["ens"]
    M, A = _oracle_ensemble(oracle, ens, tag, n_rep)
    R, RA = ens[f"{tag}_mean"], ens[f"{tag}_active"]
    n_t = R.shape[1]
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


# (tag, D, v, sigma, dt_adv) of the two cases in ref_fke.npz: L = 24, and L = 9
# where the stencils wrap the lattice more than once
FKE_CASES = [("a", 1.0, 1.0, 1.5, 1.0), ("b", 1.0, 2.0, 2.0, 1.0)]


@pytest.mark.parametrize("tag,D,v,sigma,dt_adv", FKE_CASES, ids=[c[0] for c in FKE_CASES])
def test_fke_parameters_match_reference(golden, tag, D, v, sigma, dt_adv):
    """fke_parameters restates set_global_FKE_params / precompute_gaussian: same
    prefactor and stencils, bit for bit."""
    from trophic_maelstorm_gb300 import api
    g = golden["fke"]
    p = api.fke_parameters(D, v, dt_adv, sigma)
    assert p.pref == g[f"fke_{tag}_meta"][1]
    assert np.array_equal(p.gD, g[f"fke_{tag}_gD"]) and np.array_equal(p.gV, g[f"fke_{tag}_gV"])


@pytest.mark.parametrize("tag", ["a", "b"])
def test_fke_advdiff_matches_reference(oracle, golden, tag):
    """The oracle's scatter (advdiff_FKE_MultiSp order) equals the reference bit for bit."""
    g = golden["fke"]
    L = int(g[f"fke_{tag}_meta"][0])
    sh = (L, L)
    out = oracle.fke_advdiff(g[f"fke_{tag}_rho"].reshape(sh), g[f"fke_{tag}_gamma"].reshape(sh),
                             g[f"fke_{tag}_vx"].reshape(sh), g[f"fke_{tag}_vy"].reshape(sh),
                             float(g[f"fke_{tag}_meta"][1]), g[f"fke_{tag}_gD"], g[f"fke_{tag}_gV"])
    assert np.array_equal(out.reshape(-1), g[f"fke_{tag}_out"])
    # mass is conserved up to the sites below eps, which the reference drops
    rho = g[f"fke_{tag}_rho"]
    assert out.sum() == pytest.approx(rho[rho >= 1e-10].sum(), rel=1e-12)


def test_spectrum_restatement_matches_reference_estimator():
    """The numpy restatement the GPU spectrum tests also use equals the reference's
    gen_FFT_PowerSpectra output (empty bins: NaN there, 0 here)."""
    from spectrum_restatement import spectrum_numpy
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_spectrum.npz"))
    for case in g["names"]:
        k, p = spectrum_numpy(g[f"{case}_field"])
        np.testing.assert_array_equal(k, g[f"{case}_k"])
        want = np.nan_to_num(g[f"{case}_power"], nan=0.0)
        np.testing.assert_allclose(p, want, rtol=1e-12, atol=1e-12 * max(1.0, want.max()))


@pytest.mark.parametrize("dtype", [np.float64, np.float32], ids=["fp64", "fp32"])
def test_rietkerk_ensemble_matches_reference(oracle, golden, dtype):
    """The oracle's stochastic Rietkerk step (Philox, own samplers), FP64 and FP32 state,
    against replicates of the reference's step (its P-Dornic loop with libstdc++ draws, its
    compiled remainder RK4, the clamp): 400 replicates of 500 steps on a 16^2 start with bare
    and nearly bare patches; final mean P, W, O, occupied sites and two single-site values."""
    from conftest import rk_ensemble_rows, assert_same_ensemble
    g = golden["rk_ens"]
    L, R, sigma, dt, steps, n_rep, _, eps = g["meta"]
    steps, n_rep = int(steps), int(n_rep)
    p = oracle.rk_params(R=R, sigma=sigma, dt=dt, clamp_eps=eps)
    start = g["start"].astype(dtype)
    fins = [oracle.rk_run(p, start, j, steps, [steps])[2] for j in range(n_rep)]
    assert_same_ensemble(rk_ensemble_rows(fins), g["rows"], g["columns"])
