"""Output formats against the files the reference's own writers produce
(tests/golden/ref_csv.npz, made by tests/golden/gen_golden.py)."""
import os

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def csvg():
    return np.load(os.path.join(REPO, "tests", "golden", "ref_csv.npz"))


def test_frame_bytes_and_renumbering_match_reference(tmp_path, csvg):
    from trophic_maelstorm_gb300 import io
    d = str(tmp_path)
    rho = csvg["frame_in"].reshape(6, 6)
    pat = "/FRAME_T_G_6_a_0.72_R_"
    paths = [io.save_frame(rho, d, pat, 0.72, 0) for _ in range(3)]
    assert [os.path.basename(p) for p in paths] == [f"FRAME_T_G_6_a_0.72_R_{k}.csv" for k in range(3)]
    for k in range(3):
        assert open(paths[k], "rb").read() == bytes(csvg[f"frame_R_{k}"])


def test_prelim_bytes_match_reference(tmp_path, csvg):
    from trophic_maelstorm_gb300 import io
    p = io.save_prelimframe(csvg["prelim_in"], str(tmp_path), "/PRELIM_AGG_T_G_6_a_0.72_R_", 0.72, 4, 6)
    assert open(p, "rb").read() == bytes(csvg["prelim_R_4"])


def test_frame_round_trip(tmp_path):
    from trophic_maelstorm_gb300 import io
    rng = np.random.default_rng(0)
    f = rng.uniform(0, 2, (3, 5, 5))
    p = io.save_frame(f, str(tmp_path), "/F_R_", 0.9, 1)
    back = io.read_frame(p, 5)
    np.testing.assert_allclose(back, f, rtol=5e-6)   # 6 significant digits
    assert back.shape == (3, 5, 5)


def test_fmt_matches_cxx_defaults():
    from trophic_maelstorm_gb300.io import fmt
    assert [fmt(v) for v in (0.0, 1.0, 0.1, 1e-30, 123456.789, 1234567.0, 2.5e-5, 5)] == \
        ["0", "1", "0.1", "1e-30", "123457", "1.23457e+06", "2.5e-05", "5"]
