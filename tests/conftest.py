import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libtm.so")


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as o
    o.build()
    return o


def rk_ensemble_rows(fin_fields):
    """Per-replicate rows of the Rietkerk ensemble fixture (ref_rk_ensemble.npz): final
    mean P, W, O, occupied P sites, P at sites (10, 10) and (5, 12)."""
    import numpy as np
    return np.array([[f[0].mean(), f[1].mean(), f[2].mean(), float((f[0] > 0).sum()), f[0][10, 10], f[0][5, 12]]
                     for f in fin_fields], dtype=np.float64)


def assert_same_ensemble(rows, ref, columns, max_z=3.0, min_p=0.01):
    """Column by column: means within max_z combined standard errors, two-sample KS p above min_p."""
    import numpy as np
    from scipy import stats
    for c, name in enumerate(columns):
        a, b = rows[:, c], ref[:, c]
        se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
        if se > 0:
            assert abs(a.mean() - b.mean()) <= max_z * se, (str(name), a.mean(), b.mean(), se)
        else:
            assert a.mean() == b.mean(), str(name)
        assert stats.ks_2samp(a, b).pvalue > min_p, (str(name), stats.ks_2samp(a, b).pvalue)


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    d = os.path.join(REPO, "tests", "golden")
    return {"pins": np.load(os.path.join(d, "ref_pins.npz")), "ens": np.load(os.path.join(d, "ref_dp_ensemble.npz")),
            "fke": np.load(os.path.join(d, "ref_fke.npz")), "rk_ens": np.load(os.path.join(d, "ref_rk_ensemble.npz"))}
