"""Seeded synthetic inputs for the benchmark workloads and tests.

No public dataset is involved: the reference benchmarks on generated clusters
(benchmarks/benchmark.py:58-66) and these generators play the same role with
the shapes and distributions of the engine's target workloads.
"""

from __future__ import annotations

import numpy as np


def clusters_with_outliers(
    n: int,
    d: int = 8,
    seed: int = 0,
    n_clusters: int = 5,
    centre_box: float = 10.0,
    sigma=(0.5, 2.0),
    outlier_frac: float = 0.01,
    outlier_box: float = 15.0,
) -> np.ndarray:
    """Equal-weight isotropic Gaussian clusters plus uniform outliers, float32.

    Defaults are the plain exact-LOF workload: 5 clusters with centres
    uniform in [-10, 10]^d and sigma uniform in [0.5, 2]; 1% of the rows are
    uniform in [-15, 15]^d, placed at random row positions.
    """
    rng = np.random.default_rng(seed)
    n_out = int(round(n * outlier_frac))
    centres = rng.uniform(-centre_box, centre_box, size=(n_clusters, d))
    sig = rng.uniform(sigma[0], sigma[1], size=n_clusters)
    lab = rng.integers(0, n_clusters, size=n - n_out)
    inl = centres[lab] + sig[lab, None] * rng.standard_normal((n - n_out, d))
    out = rng.uniform(-outlier_box, outlier_box, size=(n_out, d))
    perm = rng.permutation(n)
    X = np.empty((n, d), np.float32)
    X[perm[:n_out]] = out
    X[perm[n_out:]] = inl
    return X


def factor_model(
    n: int, d: int = 128, seed: int = 0, rank: int = 16, noise: float = 0.1, shift: float = 5.0,
    noisy_frac: float = 0.005, noisy_box: float = 3.0,
) -> np.ndarray:
    """Rank-16 Gaussian factor model plus noise, shifted by a constant mean.

    Factors N(0, 1), loadings N(0, 1/rank), noise N(0, noise^2), every feature
    shifted by ``shift`` (this stresses the |a|^2 + |b|^2 - 2 a.b cancellation
    of Gram-based distances); ``noisy_frac`` of the rows get uniform noise in
    [-noisy_box, noisy_box]^d added.
    """
    rng = np.random.default_rng(seed)
    F = rng.standard_normal((n, rank))
    L = rng.standard_normal((rank, d)) / np.sqrt(rank)
    X = F @ L + noise * rng.standard_normal((n, d)) + shift
    m = int(round(n * noisy_frac))
    rows = rng.choice(n, size=m, replace=False)
    X[rows] += rng.uniform(-noisy_box, noisy_box, size=(m, d))
    return X.astype(np.float32)


def gradient_mixture(n: int = 50_000, d: int = 32, seed: int = 0) -> np.ndarray:
    """8-cluster mixture (centres U[-8,8]^d, sigma U[0.5,1.5]) + 1% U[-12,12]^d."""
    return clusters_with_outliers(
        n, d, seed, n_clusters=8, centre_box=8.0, sigma=(0.5, 1.5), outlier_frac=0.01, outlier_box=12.0
    )


def batched_problems(count: int = 2048, d: int = 16, seed: int = 0, n_range=(128, 16384), k_range=(10, 40)):
    """Many independent problems: n_i log-uniform, k_i uniform, 3 clusters + 2% outliers."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_range[0]), np.log(n_range[1]), size=count)).astype(np.int64)
    ks = rng.integers(k_range[0], k_range[1] + 1, size=count)
    seeds = rng.integers(0, 2**31 - 1, size=count)
    probs = []
    for n_i, s_i in zip(ns, seeds):
        probs.append(
            clusters_with_outliers(
                int(n_i), d, int(s_i), n_clusters=3, centre_box=6.0, sigma=(1.0, 1.0), outlier_frac=0.02,
                outlier_box=10.0,
            )
        )
    return probs, [int(k) for k in ks]


def reference_test_data(n: int, d: int, seed: int, n_outliers: int = 0) -> np.ndarray:
    """Standard normal rows with the first ``n_outliers`` uniform in [-15, 15]^d.

    The same distribution as the reference test suite's fixture generator
    (tests/python/conftest.py:19-30), so parity cases read like its tests.
    """
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)).astype(np.float32)
    if n_outliers:
        X[:n_outliers] = rng.uniform(-15, 15, size=(n_outliers, d)).astype(np.float32)
    return X
