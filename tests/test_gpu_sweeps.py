"""The reference's sweep interfaces beyond the a-sweep, on the GPU:
finite-size collapse and stationary sweeps (stochasticSPDP.cpp:1424-1670) as
ragged batches, and spreading runs from a single seed (critical_exp_theta_delta,
spreading_exp_Dornic_2D, :1145-1298, 1673-1764) checked against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def tmg():
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as m
    return m


@pytest.fixture(scope="module")
def ctx(tmg):
    return tmg.Context(0)


def _oracle_spreading(oracle, L, seed, a, n_steps, dtype):
    """Per step s: stop if a border site is occupied, else record (occupied sites,
    summed squared distance from (L/2, L/2)) and stop if none is occupied; then step."""
    p = oracle.dp_params(a=a)
    rho = np.zeros((L, L), dtype)
    h = int(L / 2.0)
    rho[h, h] = 1.0
    yy, xx = np.mgrid[0:L, 0:L]
    d2 = (yy - h) ** 2 + (xx - h) ** 2
    N = np.zeros(n_steps + 1)
    S = np.zeros(n_steps + 1)
    for s in range(n_steps + 1):
        occ = rho > 0
        if occ[0].any() or occ[-1].any() or occ[:, 0].any() or occ[:, -1].any():
            break
        if not occ.any():
            break
        N[s], S[s] = occ.sum(), d2[occ].sum()
        if s < n_steps:
            rho, _ = oracle.dp_step(p, rho, seed, s)
    return N, S


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_spreading_measurements_and_border_stop_match_oracle(tmg, oracle, ctx, precision):
    dtype = np.float64 if precision == 0 else np.float32
    L, n_steps, a = 15, 120, 0.9
    seeds = [3, 4, 5, 6, 7, 8]
    b = tmg.Batch(ctx, tmg.dp_model(), tmg.instances([L] * len(seeds), seeds, a), precision)
    b.set_spreading(True)
    assert b.obs_width == 3
    seed_frame = tmg.api.init_solitarytear(L).reshape(L, L).astype(dtype)
    b.upload([seed_frame] * len(seeds))
    obs, _ = b.advance(n_steps, list(range(n_steps + 1)))
    b.close()
    stopped = 0
    for k, sd in enumerate(seeds):
        N, S = _oracle_spreading(oracle, L, sd, a, n_steps, dtype)
        assert np.array_equal(obs[:, k, 1], N), k
        assert np.array_equal(obs[:, k, 2], S), k
        stopped += int(N[-1] == 0 and N[0] == 1)
    assert stopped > 0   # some replicate reached the edge or died within the run


def test_theta_delta_rows(tmg, ctx):
    rows, st = tmg.critical_exp_theta_delta(None, 2, 20.0, 0.9, 2.0, 1.0, 1.0, 0.1, 1.0, 3, 41, seed=5,
                                            precision=tmg.TM_FP32, ctx=ctx)
    assert not st.any()
    n_t = len(rows) // 2
    assert rows[0].tolist() == [0.0, 0.9, 0.0, 1.0, 0.0, 3.0]
    assert rows[n_t][0] == 1.0
    assert np.all(rows[:, 5] <= 3) and np.all(np.diff(rows[:n_t, 5]) <= 0)


def test_fss_collapse_rows_equal_single_size_runs(tmg, ctx):
    """The ragged collapse sweep equals per-side percolation_dornic_2d runs with the
    same keys (side i, replicate j: seed + i r + j), row for row."""
    r, seed = 3, 40
    rows, st = tmg.critical_exp_finite_scaling_collapse(3, 16, 40, 20.0, 0.53, 2.0, 1.0, 1.0, 0.1, 1.0, r,
                                                        seed=seed, precision=tmg.TM_FP32, ctx=ctx)
    assert not st.any()
    sides = [int(g) for g in tmg.linspace(16, 40, 3)]
    assert sorted(set(rows[:, 1].astype(int))) == sides
    t_meas = tmg.logarithm10_time_bins(20.0, 0.1)
    for i, g in enumerate(sides):
        want, _ = tmg.percolation_dornic_2d(t_meas, np.ones(g * g), 20.0, 0.53, 2.0, 1.0, 1.0, 0.1, 1.0, r, g,
                                            seed=seed + i * r, precision=tmg.TM_FP32, ctx=ctx)
        assert np.array_equal(rows[rows[:, 1] == g], want)


def test_fss_stationary_windows(tmg, ctx):
    """Sides from the reference's lnspace, cast to int as it does (lnspace(40, 60, 2)
    starts at 39.999..., so side 39), each measured on its window."""
    rows, st = tmg.critical_exp_finite_scaling_stationary(2, 40, 60, 0.0, 0.0, 0.53, 2.0, 1.0, 1.0, 0.1, 1.0, 2,
                                                          precision=tmg.TM_FP32, ctx=ctx)
    assert not st.any()
    sides = [int(g) for g in tmg.api.lnspace(40, 60, 2)]
    assert sides == [39, 60] and sorted(set(rows[:, 1].astype(int))) == sides
    for g, (t0, t1) in zip(sides, ((300.0, 900.0), (1000.0, 2500.0))):
        ts = rows[rows[:, 1] == g][:, 2]
        late = ts[ts > 1.0]
        assert np.allclose(late, tmg.linspace(t0, t1, 30), rtol=0, atol=1e-9)
