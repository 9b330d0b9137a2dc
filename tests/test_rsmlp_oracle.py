"""CPU checks of the neighbour-radius predictor's test infrastructure and
host logic: the FP64 oracle's gradient against central finite differences
(so the GPU gradient check below rests on a verified oracle), the training
label against a brute-force count under the kernel's membership test, and
the feature matrix."""
import numpy as np
import pytest

from oracle import mlp_oracle


def _params(rng):
    P = mlp_oracle.H * mlp_oracle.I + mlp_oracle.H + mlp_oracle.H * mlp_oracle.H + \
        mlp_oracle.H + mlp_oracle.H + 1
    return rng.normal(0.0, 0.3, P)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    w = _params(rng)
    X = rng.normal(size=(40, 8))
    T = rng.normal(size=40)
    W = rng.random(40)
    g, loss = mlp_oracle.gradient(w, w, X, T, W)
    assert g.shape == w.shape and loss > 0
    idx = np.concatenate([rng.choice(512, 12, replace=False),             # W1
                          512 + rng.choice(64, 4, replace=False),         # b1
                          576 + rng.choice(4096, 16, replace=False),      # W2
                          4672 + rng.choice(64, 4, replace=False),        # b2
                          4736 + rng.choice(64, 6, replace=False),        # W3
                          [4800]])                                        # b3
    h = 1e-6
    for p in idx:
        wp, wm = w.copy(), w.copy()
        wp[p] += h
        wm[p] -= h
        fd = (mlp_oracle.gradient(wp, wp, X, T, W)[1] - mlp_oracle.gradient(wm, wm, X, T, W)[1]) / (2 * h)
        assert abs(fd - g[p]) <= 1e-7 + 1e-6 * abs(g[p]), p


def test_label_radius_gives_exact_membership():
    pytest.importorskip("scipy")
    from nbody6ppgpu_gb300.rsharness import label_log_radius
    rng = np.random.default_rng(2)
    n = 3000
    x = rng.normal(size=(n, 3))
    v = 0.5 * rng.normal(size=(n, 3))
    dtr = rng.choice([0.01, 0.05, 0.2], size=n)
    idx = rng.choice(n, 150, replace=False)
    ks = rng.integers(1, 90, size=150)
    L = label_log_radius(x, v, dtr, idx, ks)
    for q, i in enumerate(idx):
        dx = x - x[i]
        dp = dx + dtr[i] * (v - v[i])
        key = np.minimum(np.einsum("ij,ij->i", dx, dx), np.einsum("ij,ij->i", dp, dp))
        assert int((key < np.exp(2 * L[q])).sum()) - 1 == ks[q]


def test_features_shape_and_values():
    from nbody6ppgpu_gb300.rsmlp import NF, features
    rng = np.random.default_rng(0)
    n = 7
    x = rng.normal(size=(n, 3))
    F = features(x, rng.normal(size=(n, 3)), np.full(n, 2.0), np.full(n, 0.1),
                 np.array([0, 1, 5, 50, 100, 120, 3]), rng.normal(size=(n, 3)),
                 rng.normal(size=(n, 3)), np.full(n, 0.01), 100)
    assert F.shape == (n, NF) and np.all(np.isfinite(F))
    assert F[:, 0] == pytest.approx(np.log(np.linalg.norm(x, axis=1) + 1e-6))
    assert F[4, 2] == pytest.approx(1.0)
    assert F[:, 6] == pytest.approx(np.log(2.0))
