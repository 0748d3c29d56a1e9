"""Host-side pieces of the learned preconditioner's data pipeline
(serac_gb300/learned.py): the Gaussian random field behind the lognormal
material fields and the per-node network features."""
import numpy as np

from serac_gb300.learned import gaussian_random_field, node_features


def test_random_field_statistics():
    """Unit variance, zero mean, reproducible by seed, and correlation
    exp(-r^2 / (2 ell^2)) along a grid axis (averaged over seeds)."""
    n, ell = 48, 0.1
    g = gaussian_random_field(n, ell, 3)
    assert g.shape == (n, n, n)
    assert abs(g.mean()) < 1e-12 and abs(g.std() - 1.0) < 1e-12
    assert np.array_equal(g, gaussian_random_field(n, ell, 3))
    lags = np.arange(8)
    acc = np.zeros(lags.size)
    seeds = range(6)
    for seed in seeds:
        f = gaussian_random_field(n, ell, seed)
        for i, lag in enumerate(lags):
            acc[i] += np.mean(f[:, :, :n - lag] * f[:, :, lag:])
    emp = acc / len(seeds)
    model = np.exp(-0.5 * (lags / n) ** 2 / ell ** 2)
    assert np.abs(emp - model).max() < 0.06
    assert np.abs(emp - np.exp(-2.0 * (lags / n) ** 2 / ell ** 2)).max() > 0.1  # not a length of ell / 2


def test_node_features():
    """Per-node mean of the incident elements' values and the constraint
    channel (1 clamped, 0.25 partially constrained)."""
    n, order = 3, 2
    f = np.arange(n ** 3, dtype=np.float64)
    N1 = order * n + 1
    feat = node_features(n, order, f, clamped_nodes=[0], partial_nodes=[5])
    assert feat.dtype == np.float32 and feat.shape == (2 * N1 ** 3,)
    assert feat[0] == f[0]  # box corner: one element
    assert np.isclose(feat[1], f[0])  # mid-edge node of element 0 only
    # the vertex node (2, 2, 2) is shared by the 8 elements with ex, ey, ez in {0, 1}
    node = 2 + N1 * (2 + N1 * 2)
    shared = [ex + n * (ey + n * ez) for ez in (0, 1) for ey in (0, 1) for ex in (0, 1)]
    assert np.isclose(feat[node], f[shared].mean())
    assert feat[N1 ** 3 + 0] == 1.0 and feat[N1 ** 3 + 5] == 0.25
