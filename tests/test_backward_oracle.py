"""The FP64 backward oracle (oracle/backward.py) on the CPU: its scores
restate the reference's forward chain (against the C oracle's LOF), and its
autograd gradient agrees with central finite differences."""

from __future__ import annotations

import numpy as np
import pytest

import oracle
from oracle import backward as ob
from culof_gb300 import synthetic

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("normalize", [False, True])
def test_oracle_scores_match_forward(normalize):
    X = synthetic.clusters_with_outliers(600, 6, seed=41)
    X[:, 2] *= 30.0
    k = 12
    Xc, _, _ = oracle.center(X, normalize)
    idx, _, _ = oracle.knn(Xc, k)
    s = ob.lof_fixed(torch.tensor(X.astype(np.float64)), idx, normalize).numpy()
    ref = oracle.lof(X, k, normalize).astype(np.float64)
    assert np.max(np.abs(s - ref) / ref) < 2e-5


@pytest.mark.parametrize("normalize", [False, True])
def test_oracle_gradient_matches_finite_differences(normalize):
    rng = np.random.default_rng(42)
    X = synthetic.clusters_with_outliers(400, 5, seed=43)
    k = 10
    Xc, _, _ = oracle.center(X, normalize)
    idx, _, _ = oracle.knn(Xc, k)
    w = rng.standard_normal(len(X))
    g, _ = ob.grad_fixed(X, idx, w, normalize)
    for _ in range(3):
        v = np.zeros_like(X, dtype=np.float64)
        pts = rng.choice(len(X), 64, replace=False)
        v[pts] = rng.standard_normal((64, X.shape[1]))
        fd = ob.fd_directional(X, idx, w, v, 1e-6, normalize)
        an = float((g * v).sum())
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(an)), (fd, an)
