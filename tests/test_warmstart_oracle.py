"""The FP64 gradient oracle of the warm-start network against finite differences."""
import numpy as np

from oracle import warmstart_oracle as WO


def test_oracle_gradient_matches_finite_differences():
    n = sum(co * ci * 5 + co for ci, co, d, a in WO.LAYERS)
    assert n == 43073  # 5 -> 64 -> 64 -> 64 -> 1, kernel 5, with biases
    r = np.random.default_rng(0)
    p = r.normal(0, 0.1, n)
    f = r.uniform(-1, 1, (2, 5, 256))
    t = r.normal(0, 1, (2, 256))
    _, g = WO.loss_grad(p, f, t)
    for i in [0, 7, 1279, 1300, 20000, 41000, n - 2, n - 1]:
        e = np.zeros(n)
        e[i] = 1e-6
        fd = (WO.loss_grad(p + e, f, t)[0] - WO.loss_grad(p - e, f, t)[0]) / 2e-6
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), i


def test_features_layout():
    x = np.linspace(0.0, 4.0, 33)
    f0 = (1 - np.exp(-(x / 0.25) ** 2)) * (1 - np.exp(-((4 - x) / 0.25) ** 2))
    feat, tgt = WO.features(x, f0, 2048, np.sin(x))
    assert feat.shape == (5, 256) and tgt.shape == (256,)
    assert feat[0, 0] == -1 and feat[0, -1] == 1
    assert np.allclose(feat[1], -0.5) and np.allclose(feat[2], (11 - 10.5) / 1.5)
