"""Host side of the surrogate, without a GPU: the CPU FP64 reference network
against central differences, its BF16 rounding against torch's, the feature
transform and the (state, dt) sampler."""
import numpy as np
import pytest

from oracle import mlp_ref

torch = pytest.importorskip("torch")


def raw(n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(300, 3800, n), 10 ** rng.uniform(4.7, 7, n), rng.uniform(0, .05, n),
                     rng.uniform(0, .05, n), rng.uniform(.85, .95, n), rng.uniform(0, .02, n),
                     10 ** rng.uniform(-9, -5, n)], 1)


MEAN = np.array([0.6, 6.0, -1.8, -1.8, -0.05, -2.3, -7.0])
STD = np.array([0.5, 0.7, 0.5, 0.5, 0.02, 0.8, 1.2])


def test_reference_gradient_matches_central_differences():
    from rocketcombustor_gb300 import surrogate
    p = surrogate.init_params(1).astype(np.float64)
    x = raw(64, 0)
    t = np.random.default_rng(1).normal(size=(64, 4))
    _, g, _ = mlp_ref.loss_and_grad(p, x, t, MEAN, STD, bf=False)
    rng = np.random.default_rng(2)
    for k in rng.choice(p.size, 25, replace=False):
        h = 1e-6 * max(1.0, abs(p[k]))
        pp = p.copy(); pp[k] += h
        lp, _, _ = mlp_ref.loss_and_grad(pp, x, t, MEAN, STD, bf=False)
        pp[k] -= 2 * h
        lm, _, _ = mlp_ref.loss_and_grad(pp, x, t, MEAN, STD, bf=False)
        fd = (lp - lm) / (2 * h)
        assert abs(g[k] - fd) <= 1e-6 * max(abs(fd), 1e-3), (k, g[k], fd)


def test_bf16_rounding_matches_torch():
    a = np.random.default_rng(3).normal(size=4096).astype(np.float32) * 10 ** np.random.default_rng(4).uniform(-5, 5, 4096)
    ref = torch.tensor(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(mlp_ref.bf16(a), ref)


def test_features_and_sampler():
    from rocketcombustor_gb300 import surrogate
    x = torch.tensor(raw(100, 5))
    f = surrogate.features(x).numpy()
    np.testing.assert_allclose(f[:, 0], 1000.0 / x[:, 0].numpy())
    np.testing.assert_allclose(f[:, 6], np.log10(x[:, 6].numpy()))
    np.testing.assert_allclose(mlp_ref.features(x.numpy(), np.zeros(7), np.ones(7)), f, rtol=1e-12)
    pool = torch.tensor(np.stack([np.full(50, 1e6), np.zeros(50), np.zeros(50), np.full(50, 2000.0),
                                  np.full(50, 0.03), np.full(50, 0.01), np.full(50, 0.9)]))
    P, dt = surrogate.sample_states(pool, 10000, seed=1)
    T, p = P[3].numpy(), P[0].numpy()
    assert T.min() >= surrogate.T_RANGE[0] and T.max() <= surrogate.T_RANGE[1]
    assert p.min() >= surrogate.P_RANGE[0] and p.max() <= surrogate.P_RANGE[1]
    assert dt.min() >= surrogate.DT_RANGE[0] and dt.max() <= surrogate.DT_RANGE[1]
    assert 0.4 < (T == 2000.0).mean() < 0.6  # half kept, half redrawn
