"""The oracle's samplers against scipy's distributions and the published
properties of the Dornic transition kernel."""
import numpy as np
import pytest
from scipy import stats


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m", [1e-3, 0.5, 3.7, 9.99, 10.0, 17.0, 250.0, 1e4])
def test_poisson_chi2(oracle, dtype, m):
    N = 100000
    x, st = oracle.sample("poisson", N, seed=7, m=m, dtype=dtype)
    assert st == 0
    sd = np.sqrt(m)
    lo, hi = max(0, int(m - 6 * sd)), int(m + 6 * sd) + 2
    edges = np.unique(np.linspace(lo, hi, min(40, hi - lo + 1)).astype(int))
    obs, _ = np.histogram(x, bins=np.concatenate([[-np.inf], edges, [np.inf]]))
    cdf = np.concatenate([[0.0], stats.poisson.cdf(edges - 1, m), [1.0]])
    exp = np.diff(cdf) * N
    keep = exp > 10
    chi = ((obs[keep] - exp[keep]) ** 2 / exp[keep]).sum()
    dof = max(1, keep.sum() - 1)
    assert stats.chi2.sf(chi, dof) > 1e-3
    assert abs(x.mean() - m) < 5 * sd / np.sqrt(N)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("k", [0.3, 1.0, 2.5, 25.0, 99.0, 400.0])
def test_gamma_ks(oracle, dtype, k):
    x, st = oracle.sample("gamma", 50000, seed=3, k=k, dtype=dtype)
    assert st == 0
    assert stats.kstest(x.astype(np.float64), stats.gamma(k).cdf).pvalue > 1e-3


def test_gamma_tiny_shape_mean(oracle):
    x, _ = oracle.sample("gamma", 200000, seed=5, k=1e-3)
    assert abs(x.mean() - 1e-3) < 5 * np.sqrt(1e-3 / 200000)


def test_normal_ks(oracle):
    for dt in (np.float64, np.float32):
        x, _ = oracle.sample("normal", 50000, seed=9, dtype=dt)
        assert stats.kstest(x.astype(np.float64), "norm").pvalue > 1e-3


def test_gauss100_switches(oracle):
    # above 100 the REF_GAUSS100 sampler is N(m, m) truncated to an integer (multiSPDP.cpp:2922-2927)
    x, _ = oracle.sample("poisson", 50000, seed=1, m=400.0, sampler=oracle.SAMPLER_REF_GAUSS100)
    z = (x - 400.0) / 20.0
    assert stats.kstest(z + 0.5 / 20.0, "norm").pvalue > 1e-4 or abs(z.mean()) < 0.05
    g, _ = oracle.sample("gamma", 50000, seed=2, k=250.0, sampler=oracle.SAMPLER_REF_GAUSS100)
    assert stats.kstest((g - 250.0) / np.sqrt(250.0), "norm").pvalue > 1e-3


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_dornic_kernel_moments(oracle, dtype):
    """E[rho*] = e^{beta dt} rho + alpha (e^{beta dt}-1)/beta: the noise-off limit of the Dornic kernel."""
    c = oracle.dornic_consts(0.72, 1.0, 1.0, 0.1, 1.0)
    rho, alpha = 0.8, 2.4
    m = c["pm"] * rho
    mu1 = alpha * 2.0
    x, st = oracle.sample("dornic", 200000, seed=4, m=m, mu1=mu1, inv_lambda=c["inv_lambda"], dtype=dtype)
    assert st == 0
    mean = c["mean_a1"] * rho + c["mean_a2"] * alpha
    # Var[rho*] = (mu1 + 2 m)/lambda^2 for Gamma(mu1 + Poisson(m))/lambda
    var = (mu1 + 2 * m) * c["inv_lambda"] ** 2
    assert abs(x.mean() - mean) < 5 * np.sqrt(var / len(x))
    assert abs(x.var() / var - 1) < 0.02


def test_determinism_and_precision_consistency(oracle):
    rng = np.random.default_rng(0)
    rho = (1 + rng.uniform(-0.01, 0.01, (16, 16)))
    p = oracle.dp_params()
    a1, _ = oracle.dp_step(p, rho, 5, 3)
    a2, _ = oracle.dp_step(p, rho, 5, 3)
    assert np.array_equal(a1, a2)
    b1, _ = oracle.dp_step(p, rho, 6, 3)
    assert not np.array_equal(a1, b1)
    # noise-off: the step is the conditional mean followed by the exact -b rho^2 flow
    po = oracle.dp_params(sampler=oracle.SAMPLER_OFF)
    m64, _ = oracle.dp_step(po, rho, 0, 0)
    m32, _ = oracle.dp_step(po, rho.astype(np.float32), 0, 0)
    np.testing.assert_allclose(m32, m64, rtol=1e-6)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("m,mu1", [(16.7, 6.0), (3.0, 0.9), (0.2, 0.55), (50.0, 1.2), (7.0, 0.3), (0.05, 0.1),
                                   (250.0, 30.0), (30.0, 100.0)])
def test_dornic_draw_law(oracle, dtype, m, mu1):
    """The whole Dornic draw against its exact law: for X = Gamma(mu1 + Poisson(m)), 2X is
    noncentral chi-square with 2 mu1 degrees of freedom and noncentrality 2m (KS p > 1e-3),
    over the inversion (m < 32) and PTRS (m >= 32) ranges and shapes below and above 1."""
    x, st = oracle.sample("dornic", 60000, seed=17, m=m, mu1=mu1, inv_lambda=1.0, dtype=dtype)
    assert st == 0
    assert stats.kstest(2.0 * x.astype(np.float64), stats.ncx2(2 * mu1, 2 * m).cdf).pvalue > 1e-3


def _libstdcxx():
    import os
    return np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_libstdcxx.npz"))


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_poisson_matches_libstdcxx(oracle, dtype):
    """The oracle's Poisson draws against the libstdc++ poisson_distribution the reference
    constructs per site: chi-square homogeneity of the binned counts, p > 1e-3, at every mean."""
    z = _libstdcxx()
    for k, m in enumerate(z["poisson_params"]):
        ref = z[f"poisson_{k}"].astype(np.int64)
        x, st = oracle.sample("poisson", len(ref), seed=31 + k, m=float(m), dtype=dtype)
        assert st == 0
        x = x.astype(np.int64)
        lo, hi = np.percentile(np.concatenate([ref, x]), [0.5, 99.5]).astype(int)
        edges = np.unique(np.linspace(lo, hi + 1, min(30, hi - lo + 2)).astype(int))
        a = np.histogram(np.clip(x, lo, hi), edges)[0]
        b = np.histogram(np.clip(ref, lo, hi), edges)[0]
        keep = (a + b) > 0
        assert stats.chi2_contingency(np.stack([a[keep], b[keep]]))[1] > 1e-3, m


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_gamma_matches_libstdcxx(oracle, dtype):
    """The oracle's Gamma draws against the libstdc++ gamma_distribution: two-sample KS, p > 1e-3."""
    z = _libstdcxx()
    for k, shape in enumerate(z["gamma_params"]):
        ref = z[f"gamma_{k}"].astype(np.float64)
        x, st = oracle.sample("gamma", len(ref), seed=57 + k, k=float(shape), dtype=dtype)
        assert st == 0
        assert stats.ks_2samp(x.astype(np.float64), ref).pvalue > 1e-3, shape


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_dornic_draw_matches_libstdcxx(oracle, dtype):
    """The oracle's whole Dornic draw against the reference's own: a libstdc++ Poisson count,
    then a libstdc++ Gamma of shape mu1 + count (stochasticSPDP.cpp:1053-1059).  Two-sample KS,
    p > 1e-3, from the dilute to the dense regime and across the inversion/PTRS switch."""
    z = _libstdcxx()
    for k, (m, mu1) in enumerate(z["dornic_params"]):
        ref = z[f"dornic_{k}"].astype(np.float64)
        x, st = oracle.sample("dornic", len(ref), seed=71 + k, m=float(m), mu1=float(mu1), inv_lambda=1.0,
                              dtype=dtype)
        assert st == 0
        assert stats.ks_2samp(x.astype(np.float64), ref).pvalue > 1e-3, (m, mu1)


def _rsqrt_correct(x, r):
    """r is the correctly rounded 1/sqrt(x): the interval of reals that round to r
    contains 1/sqrt(x), i.e. lo^2 x <= 1 <= hi^2 x for its end points (exact)."""
    from fractions import Fraction
    import math
    m, e = math.frexp(r)                       # r = m 2^e, m in [0.5, 1)
    up = Fraction(2) ** (e - 24)               # ulp of r
    down = up / 2 if m == 0.5 else up          # ulp below a power of two
    fx, fr = Fraction(x), Fraction(r)
    lo, hi = fr - down / 2, fr + up / 2
    return lo * lo * fx <= 1 <= hi * hi * fx


def test_inv_sqrt_f32_is_correctly_rounded(oracle):
    """The Marsaglia-Tsang constant c = 1/sqrt(9d) in FP32 is the correctly rounded
    1/sqrt, as __frsqrt_rn gives it in the kernels: the oracle rounds the double
    quotient once.  An exhaustive exact check over [1, 4) (every normal float, by
    scaling by 4) found no misrounding; this rechecks the inputs closest to a
    rounding midpoint and 20000 random normal floats."""
    hard = [float.fromhex(h) for h in ("0x1.7431c6p+1", "0x1.a4411ep+0", "0x1.fffffcp+1", "0x1.fbc3c2p+1",
                                       "0x1.745472p+0", "0x1.13e07p+1", "0x1.14b90cp+0", "0x1.85da2cp+1",
                                       "0x1.da646p+0", "0x1.b5d284p+0", "0x1.3ba2d4p+1", "0x1.fb7758p+1")]
    rng = np.random.default_rng(5)
    bits = rng.integers(0x00800000, 0x7f800000, 20000, dtype=np.uint32)
    xs = [float(v) for v in bits.view(np.float32)] + [float(np.float32(h)) for h in hard]
    bad = [x for x in xs if not _rsqrt_correct(x, float(oracle.scalar_fn("inv_sqrt", x, np.float32)))]
    assert not bad, bad[:5]
    # the two-rounding form 1.0f / sqrtf(x) differs on most of the hard inputs
    two = [float(np.float32(1.0) / np.sqrt(np.float32(h))) for h in hard]
    assert sum(not _rsqrt_correct(float(np.float32(h)), t) for h, t in zip(hard, two)) >= 1
