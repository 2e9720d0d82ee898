"""Host logic of the critical-point searches (no GPU): a judge whose delta_eff is a
known decreasing function of a stands in for the full simulations."""
import numpy as np
import pytest


class FakeJudge:
    def __init__(self, a_c, slope=30.0, noise=None):
        self.a_c, self.slope, self.noise = a_c, slope, noise or {}
        self.runs, self.n_rep, self.cache = 0, 8, {}

    def delta(self, a_values):
        from trophic_maelstorm_gb300.surrogate import DELTA_DP_2D
        out = []
        for a in a_values:
            a = round(float(a), 9)
            if a not in self.cache:
                self.cache[a] = DELTA_DP_2D + self.slope * (self.a_c - a) + self.noise.get(a, 0.0)
                self.runs += self.n_rep
            out.append(self.cache[a])
        return np.array(out)


@pytest.mark.parametrize("a_c", [0.5011, 0.5305, 0.5318, 0.5589])
def test_uniform_sweep_brackets_the_crossing(a_c):
    from trophic_maelstorm_gb300 import surrogate as sg
    j = FakeJudge(a_c)
    br, runs = sg.uniform_sweep(j)
    assert br[0] <= a_c < br[1] and br[1] - br[0] == pytest.approx(2e-3)
    assert runs == 31 * 8


@pytest.mark.parametrize("a_hat", [0.5305, 0.524, 0.545, 0.5012])
def test_guided_search_moves_to_the_crossing(a_hat):
    from trophic_maelstorm_gb300 import surrogate as sg
    a_c = 0.5305
    j = FakeJudge(a_c)
    br, runs = sg.guided_search(j, a_hat)
    assert br[0] < a_c <= br[1] and br[1] - br[0] == pytest.approx(2e-3)
    moves = int(np.ceil(max(abs(a_hat - a_c) - 1e-3, 0) / 2e-3))
    assert runs == 8 * (2 + moves)     # each move reuses one end


def test_guided_search_gives_up_outside_the_window():
    from trophic_maelstorm_gb300 import surrogate as sg
    br, runs = sg.guided_search(FakeJudge(0.70), 0.53)
    assert br is None and runs > 0
    br, _ = sg.uniform_sweep(FakeJudge(0.70))
    assert br is None


def test_features_scale_the_window_to_unit_range():
    from trophic_maelstorm_gb300 import surrogate as sg
    f = sg.features([0.50, 0.56], [64, 1024], [1.0, 1000.0])
    np.testing.assert_allclose(f, [[-1, -1, -1], [1, 1, 1]], atol=1e-6)


def test_judge_uses_common_random_numbers(monkeypatch):
    """Every value of a is judged with the same replicate keys (initial fields and Philox
    streams), so two judges with the same seed see the same delta_eff(a) and the
    values differ by the control parameter only; cached values are not re-run."""
    from trophic_maelstorm_gb300 import surrogate as sg
    calls = []

    def fake_run(ctx, a_values, L, n_rep, t_max, point_seeds=None, **kw):
        calls.append((list(a_values), list(point_seeds)))
        t = np.array([1.0, 100.0, 1000.0])
        rho = np.array([[1.0, 0.1, 0.1 * 10 ** (-(0.45 + (0.53 - a)))] for a in a_values])
        return sg.Ensembles(np.asarray(a_values), np.full(len(a_values), L), t, rho, np.ones_like(rho), n_rep,
                            0.0, 0.0)

    monkeypatch.setattr(sg, "run_ensembles", fake_run)
    j = sg.Judge(None, 64, 4, 1000.0, 100.0, seed=7)
    d1 = j.delta([0.52, 0.54])
    d2 = j.delta([0.54, 0.53])
    assert len(calls) == 2 and calls[1][0] == [0.53]            # 0.54 came from the cache
    assert all(s == 7 for _, seeds in calls for s in seeds)      # one key set for every a
    assert d1[1] == d2[0] and j.runs == 3 * 4
    assert d1[0] > d2[1] > d1[1]                                 # decreasing in a
