"""FP32 field state against FP64 for the Rietkerk model, per observable.

Both precisions start from the same frames with the same Philox keys; their
trajectories separate once a rounding difference changes one draw, so P and
the active/surviving fractions are compared statistically (combined standard
errors); where the replicates agree closely (W and O once P has died out) the
difference is the rounding error itself, so every observable is held to 5
standard errors plus 1e-5 relative.  The full studies are
`python -m trophic_maelstorm_gb300.study --rietkerk-sweep` and `--pattern`;
these are small cases of each.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def study():
    from trophic_maelstorm_gb300 import build
    build.build()
    from trophic_maelstorm_gb300 import study as s
    return s


def test_rietkerk_sweep_fp32_is_statistically_equivalent_to_fp64(study):
    r = study.rietkerk_sweep_precision_study(L=32, Rs=[0.7, 1.1], reps=16, steps=4000, n_meas=12, seed=3)
    obs = r["observables"]
    assert r["status"] == [0, 0]
    # every difference within 5 combined standard errors plus 1e-5 relative (rounding)
    for name in ("P", "W", "O", "active_P_fraction", "survival"):
        assert obs[name]["max_excess"] <= 0.0, name
    assert r["min_ks_p_P"] > 1e-3 / (2 * len(r["t"]))


def test_patterned_rietkerk_wavelength_fp32_matches_fp64(study):
    """A case that forms a pattern (vegetated start at R = 1.2): both precisions show
    a clear spectrum peak of P at the same wavelength within one k-bin."""
    r = study.rietkerk_pattern_precision(L=128, R=1.2, reps=2, steps=300000, n_meas=4, seed=5)
    assert r["f32"]["status"] == 0 and r["f64"]["status"] == 0
    for prec in ("f32", "f64"):
        assert min(r[prec]["rows"][-1]["prominence"]) > 20.0
    k32 = 128.0 / np.array(r["final_wavelength_f32"])
    k64 = 128.0 / np.array(r["final_wavelength_f64"])
    assert abs(k32.mean() - k64.mean()) <= 0.5 + 1e-9
