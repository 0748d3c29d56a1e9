"""The FP64 network oracle's gradient against central finite differences."""
import numpy as np

from oracle import nn_oracle as NN


def _problem(shape=(9, 9, 9), seed=0):
    rng = np.random.default_rng(seed)
    N = int(np.prod(shape))
    r = rng.standard_normal(3 * N)
    t = rng.standard_normal(3 * N)
    feat = np.zeros(2 * N)
    feat[:N] = rng.standard_normal(N) * 0.3
    feat[N:N + 81] = 1.0  # first z-layer masked
    p = rng.standard_normal(NN.num_params()) * 0.05
    return p, r, t, feat, shape


def test_gradient_matches_finite_differences():
    p, r, t, feat, shape = _problem()
    loss, g, _, _ = NN.loss_and_grad(p, r, t, feat, shape)
    assert np.isfinite(loss) and g.shape == p.shape
    rng = np.random.default_rng(3)
    idx = rng.choice(p.size, 12, replace=False)
    eps = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (NN.loss_and_grad(pp, r, t, feat, shape)[0] - NN.loss_and_grad(pm, r, t, feat, shape)[0]) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_parameter_count():
    assert 250_000 < NN.num_params() < 320_000
