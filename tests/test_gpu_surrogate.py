"""The surrogate network's tensor-core kernels (tm_mlp_*) against the oracle's
restatement of the same arithmetic (oracle/surrogate_oracle.py).

Tolerances: the GPU sums the 128-term products in another order than the
oracle, and tanhf may differ from numpy's tanh in the last place, so a BF16
rounding of an activation can land on the other side in rare elements.  Outputs
and gradients are compared by relative Frobenius error (2e-3) per parameter
block; the Adam update itself, given the GPU's own gradient, is bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    from trophic_maelstorm_gb300 import build
    build.build()
    import trophic_maelstorm_gb300 as tmg
    from trophic_maelstorm_gb300 import surrogate as sg
    from oracle import surrogate_oracle as so
    return tmg, sg, so, tmg.Context(0)


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, 3)).astype(np.float32)
    t = np.stack([np.sin(x[:, 0]) + 0.5 * x[:, 1], np.tanh(x[:, 2] - x[:, 0])], 1).astype(np.float32)
    w = rng.uniform(0.2, 1.0, (n, 2)).astype(np.float32)
    return x, t, w


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


@pytest.mark.parametrize("n", [1, 128, 1000])
def test_forward_matches_oracle(env, n):
    tmg, sg, so, ctx = env
    p = sg.init_params(3)
    p[so.OFFSETS["b1"][0]:so.OFFSETS["b1"][0] + 128] = np.linspace(-0.2, 0.2, 128)
    x, _, _ = _data(n, n)
    m = sg.MLP(ctx, p)
    y = m.predict(x)
    want, _ = so.forward(p, x)
    assert _rel(y, want) < 2e-3
    np.testing.assert_allclose(y, want, rtol=0, atol=2e-2 * max(1.0, np.abs(want).max()))
    m.close()


@pytest.mark.parametrize("n", [128, 777, 4096])
def test_gradient_matches_oracle(env, n):
    tmg, sg, so, ctx = env
    p = sg.init_params(5)
    x, t, w = _data(n, 7 + n)
    m = sg.MLP(ctx, p)
    m.set_data(x, t, w)
    loss, g = m.loss_grad(1.0 / n)
    wl, wg = so.loss_and_grad(p, x, t, w, 1.0 / n)
    assert loss == pytest.approx(wl, rel=2e-3)
    for name, (o, s) in so.OFFSETS.items():
        k = int(np.prod(s))
        assert _rel(g[o:o + k], wg[o:o + k]) < 2e-3, name
    m.close()


def test_adam_step_is_bit_exact_given_the_gradient(env):
    tmg, sg, so, ctx = env
    p = sg.init_params(11)
    x, t, w = _data(500, 1)
    m = sg.MLP(ctx, p)
    m.set_data(x, t, w)
    _, g = m.loss_grad(1.0 / 500)
    m.train(1, lr=3e-3, inv_norm=1.0 / 500)
    got = m.get_params()
    want, _, _ = so.adam_step(p, np.zeros_like(p), np.zeros_like(p), g, 1, 3e-3)
    assert np.array_equal(got, want)
    m.close()


def test_training_is_reproducible_and_reduces_the_loss(env):
    tmg, sg, so, ctx = env
    x, t, w = _data(3000, 2)
    runs = []
    for _ in range(2):
        m = sg.MLP(ctx, sg.init_params(1))
        m.set_data(x, t, w)
        hist = m.train(300, lr=2e-3)
        runs.append((hist, m.get_params()))
        m.close()
    assert np.array_equal(runs[0][1], runs[1][1])
    assert np.array_equal(runs[0][0], runs[1][0])
    hist = runs[0][0]
    assert hist[-1] < 0.1 * hist[0]


def test_guided_search_needs_fewer_full_runs(env):
    """What the network gains: on a small judge (L = 128, 16 replicates, t <= 300)
    the surrogate-guided bracket agrees with the uniform sweep's and needs at
    least 4x fewer full simulations."""
    tmg, sg, so, ctx = env
    res = sg.critical_point_study(ctx, Ls=(64, 128), n_a=24, n_rep=8, judge_L=128, judge_rep=16, t_max=300.0,
                                  t1=30.0, seed=3)
    gb, ub = res["guided"]["bracket"], res["uniform"]["bracket"]
    assert gb is not None and ub is not None
    assert abs(sum(gb) / 2 - sum(ub) / 2) <= 4e-3
    assert res["guided"]["runs"] * 4 <= res["uniform"]["runs"]
    assert res["fit"]["loss_last"] < 0.05 * res["fit"]["loss_first"]
