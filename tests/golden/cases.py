"""The golden cases' inputs, regenerated from seeds (numpy only).

Shared by make_golden.py (which adds scikit-learn outputs) and the tests
(which check a SHA-256 of every regenerated input against the fixture).
"""

from __future__ import annotations

import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))

from culof_gb300 import synthetic  # noqa: E402


def case_inputs():
    """(name, X, k, normalize, sklearn_input) for every golden case."""
    out = []
    # Value parity over (n, d, k), mirroring test_parity.py:20-34.
    for n, d, k in [(500, 2, 20), (2000, 2, 20), (2000, 8, 20), (3000, 16, 10), (1500, 64, 35),
                    (1000, 3, 1), (1000, 3, 100)]:
        X = synthetic.reference_test_data(n, d, seed=n + d + k, n_outliers=max(1, n // 100))
        out.append((f"values_n{n}_d{d}_k{k}", X, k, False, X))
    # Large k (test_parity.py:37-41).
    for k in (33, 64, 128, 256):
        X = synthetic.reference_test_data(1000, 4, seed=k)
        out.append((f"largek_k{k}", X, k, False, X))
    # Extreme k incl. n-1 (test_culof.cu:125-132, same shape, different generator).
    X = synthetic.reference_test_data(128, 2, seed=7, n_outliers=4)
    for k in (1, 2, 127):
        out.append((f"extremek_k{k}", X, k, False, X))
    # Drop-in labels (test_parity.py:44-54).
    X = synthetic.reference_test_data(3000, 6, seed=7, n_outliers=30)
    out.append(("dropin_n3000_d6", X, 20, False, X))
    # Heavy duplicates (test_regressions.py:58-67).
    rng = np.random.default_rng(4)
    X = np.repeat(rng.standard_normal((50, 2)).astype(np.float32), 20, axis=0)
    X[:5] += 5.0
    out.append(("duplicates", X, 20, False, X))
    # normalize=True against scikit-learn on the z-scored array (test_regressions.py:70-78).
    rng = np.random.default_rng(5)
    X = (rng.standard_normal((2000, 4)) * [1.0, 50.0, 0.1, 5.0]).astype(np.float32)
    X[:20] += 8.0
    Z = ((X - X.mean(0)) / X.std(0)).astype(np.float32)
    out.append(("normalize", X, 20, True, Z))
    # Far from the origin (test_regressions.py:90-104).
    rng = np.random.default_rng(7)
    X = rng.standard_normal((1500, 3)).astype(np.float32)
    X[:15] = rng.uniform(-15, 15, size=(15, 3)).astype(np.float32)
    X = (X + 5000.0).astype(np.float32)
    out.append(("shifted5000", X, 20, False, X))
    # The plain exact-LOF workload at n=20,000 (d=8, k=20, contamination 0.01).
    X = synthetic.clusters_with_outliers(20_000, 8, seed=20_000)
    out.append(("clusters_n20000_d8_k20", X, 20, False, X))
    # The reference's near-tie template input (test_parity.py:70-100).
    X = synthetic.reference_test_data(20_000, 8, seed=99, n_outliers=200)
    out.append(("neartie_n20000_d8_k20", X, 20, False, X))
    return out
