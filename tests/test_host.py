"""Host-side logic and the C ABI surface (no GPU needed)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def tmlib():
    from trophic_maelstorm_gb300 import build, _lib
    build.build()
    return _lib


def test_library_exports_every_declared_symbol(tmlib):
    hdr = open(os.path.join(REPO, "include", "tm.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    declared = set(re.findall(r"\b(tm_[a-z0-9_]+)\s*\(", hdr))
    assert declared, "no declarations parsed"
    lib = C.CDLL(tmlib.LIB_PATH)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert not missing, missing
    assert declared == set(tmlib.EXPORTS)
    assert tmlib.lib().tm_abi_version() == 1
    assert tmlib.lib().tm_error_string(-1) == b"invalid argument"


def test_layout_is_aligned_and_packs_round_trip(tmlib):
    import trophic_maelstorm_gb300 as tmg
    inst = tmg.instances([1, 3, 33, 64, 100], range(5), 0.7)
    for nf in (1, 3):
        total, off, fs = tmg.layout(inst, nf)
        assert all(o % 32 == 0 for o in off) and all(f % 32 == 0 for f in fs)
        assert total == off[-1] + nf * fs[-1]
        rng = np.random.default_rng(nf)
        fields = [rng.random((nf, i.L, i.L)) if nf > 1 else rng.random((i.L, i.L)) for i in inst]
        back = tmg.unpack(tmg.pack(fields, inst, nf, np.float64), inst, nf)
        for a, b in zip(fields, back):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("k", range(6))
def test_time_bins_match_reference(golden, k):
    import trophic_maelstorm_gb300 as tmg
    g = golden["pins"]
    tmax, dt = g[f"tbins_{k}_meta"]
    assert np.array_equal(np.array(tmg.logarithm10_time_bins(tmax, dt)), g[f"tbins_{k}"])


def test_reference_step_grid():
    import trophic_maelstorm_gb300 as tmg
    steps, times, n_early = tmg.reference_step_grid([1.5, 2.0, 10.0], 0.1)
    assert n_early == 11 and steps[:11] == list(range(11)) and steps[11:] == [15, 20, 100]


def test_replicate_rows_statistics():
    import trophic_maelstorm_gb300 as tmg
    mean = np.array([[1.0, 0.5, 0.2], [1.0, 0.7, 0.0], [1.0, 0.3, 0.4]])
    act = np.array([[4, 2, 1], [4, 3, 0], [4, 1, 2]], float)
    rows = tmg.replicate_rows(0.7, 2, [0.0, 0.1, 2.0], 2, mean, act)
    assert rows.shape == (3, 8)
    assert rows[2, 5] == 2 and rows[2, 3] == pytest.approx(0.3) and rows[2, 4] == pytest.approx(0.02)
    assert rows[1, 4] == pytest.approx(np.var([0.5, 0.7, 0.3], ddof=1))
    assert rows[0, 7] == 3 and rows[2, 7] == 2


def test_invalid_arguments_are_rejected_without_gpu(tmlib):
    """Every entry point answers a NULL handle, a NULL buffer or an impossible size with
    TM_ERR_INVALID before it touches the device (the reference exits instead)."""
    L = tmlib.lib()
    bad = tmlib.TM_ERR_INVALID
    assert L.tm_create(None, 0) == bad
    assert L.tm_destroy(None) == bad
    assert L.tm_batch_step(None) == bad
    calls = {
        "tm_batch_create_dp": (None, None, None, 0, 1, None),
        "tm_batch_create_rietkerk": (None, None, None, 0, 1, None),
        "tm_batch_destroy": (None,),
        "tm_batch_total_elems": (None,),
        "tm_batch_instance_offset": (None, 0),
        "tm_batch_field_stride": (None, 0),
        "tm_batch_upload": (None, None, 0),
        "tm_batch_download": (None, None),
        "tm_batch_upload_device": (None, None, 0),
        "tm_batch_download_device": (None, None),
        "tm_batch_snapshot": (None, 0, None),
        "tm_batch_advance": (None, 1, None, 0, None, None),
        "tm_batch_enqueue_steps": (None, 1),
        "tm_batch_set_launch": (None, 8, 4),
        "tm_batch_get_launch": (None, None, None),
        "tm_batch_autotune": (None, 2),
        "tm_batch_set_site_coeff": (None, None),
        "tm_batch_box_means": (None, 0, 0, 4, None),
        "tm_batch_power_spectrum": (None, 0, 0, 0.5, None, None, 0, None),
        "tm_run_dp": (None, None, None, 1, 1, None, 1, None, 0, None, None, None),
        "tm_run_rietkerk": (None, None, None, 1, 1, None, 1, None, 0, None, None, None),
        "tm_observe_noalloc": (None, 1, None, None, 1, None, None),
        "tm_power_spectrum_device": (None, 1, 0, 0.5, None, None, None, 10, None),
        "tm_fke_advdiff_device": (None, None, None, None, 1, 0, 1.0, 1e-10, None, 1, None, 1, None, None),
        "tm_mlp_create": (None, None, None),
        "tm_mlp_destroy": (None,),
        "tm_mlp_set_params": (None, None),
        "tm_mlp_get_params": (None, None),
        "tm_mlp_set_data": (None, None, None, None, 0),
        "tm_mlp_loss_grad": (None, 1.0, None, None),
        "tm_mlp_train": (None, 1, 1e-3, 0.9, 0.999, 1e-8, 1.0, None),
        "tm_mlp_predict": (None, None, 0, None),
        "tm_set_test_probe": (None, 0),
        "tm_batch_set_spreading": (None, 1, -1, -1),
        "tm_fke_advdiff_device_ws": (None, None, None, None, 1, 0, 1.0, 1e-10, None, 1, None, 1, None, None, 0,
                                     None),
    }
    for name, args in calls.items():
        assert getattr(L, name)(*args) == bad, name
    # workspace sizing needs no device: 0 for an impossible request, else the five L^2 arrays,
    # the two wrapped stencils and the counter, each on a 256-byte boundary
    assert L.tm_fke_workspace_bytes(7, 64) == 0 and L.tm_fke_workspace_bytes(tmlib.TM_FP64, 0) == 0
    a256 = lambda v: (v + 255) // 256 * 256
    for prec, es in ((tmlib.TM_FP64, 8), (tmlib.TM_FP32, 4)):
        for n in (1, 33, 1024):
            o = 0
            for size in (n * n * es, n * n * es, n * n * es, n * n * 4, n * n * 4, n * es, n * es):
                o = a256(o + size)
            assert L.tm_fke_workspace_bytes(prec, n) == o + 256


def test_lnspace_matches_reference():
    """api.lnspace equals the reference's lnspace<int> (the stationary finite-size
    sweep's lattice sides) double for double."""
    import os
    from trophic_maelstorm_gb300 import api
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_lnspace.npz"))
    for k, (a, b, n) in enumerate(g["cases"]):
        want = g[f"lnspace_{k}"]
        got = np.array(api.lnspace(int(a), int(b), int(n)))
        assert np.array_equal(got, want), (a, b, n)
        assert [int(x) for x in got] == [int(x) for x in want]


def test_stationary_windows_follow_reference():
    from trophic_maelstorm_gb300 import api
    assert api.stationary_window(31) == (300.0, 900.0) and api.stationary_window(50) == (300.0, 900.0)
    assert api.stationary_window(51) == (1000.0, 2500.0) and api.stationary_window(100) == (1000.0, 2500.0)
    assert api.stationary_window(101) == (1250.0, 8000.0) and api.stationary_window(150) == (1250.0, 8000.0)
    assert api.stationary_window(151) == (1400.0, 10000.0) and api.stationary_window(200) == (1400.0, 10000.0)
    assert api.stationary_window(201) == (2000.0, 15000.0)
    with pytest.raises(ValueError):
        api.stationary_window(30)


def test_spreading_rows_average_over_running_replicates():
    from trophic_maelstorm_gb300 import api
    n = np.array([[1, 4, 0], [1, 2, 6]], float)       # replicate 0 stops after t1
    sq = np.array([[0, 8, 0], [0, 2, 30]], float)
    rows = api.spreading_rows(3, 0.7, [0.0, 0.1, 0.2], n, sq)
    assert rows[0].tolist() == [3.0, 0.7, 0.0, 1.0, 0.0, 2.0]
    assert rows[1].tolist() == [3.0, 0.7, 0.1, 3.0, 1.5, 2.0]
    assert rows[2].tolist() == [3.0, 0.7, 0.2, 6.0, 5.0, 1.0]
