"""Pin the CPU oracle against the reference's own oracles (no GPU needed).

* scikit-learn LocalOutlierFactor outputs (the reference's test oracle,
  tests/python/conftest.py:10-12; its CPU comparison path) in
  tests/golden/sklearn_cases.npz, with the reference's tolerances
  (test_parity.py:17 REL_TOL 2e-4; near-tie template :70-100);
* the reference's Python layer (offset_ via np.percentile, predict labels,
  validation messages) in tests/golden/reference_python_layer.npz;
* a dense FP64 restatement of the reference's cpu_lof (test_culof.cu:39-80);
* numpy itself for the percentile arithmetic.
"""

from __future__ import annotations

import hashlib

import numpy as np
import pytest
from conftest import fp64_lof, golden_case_arrays, max_rel_err, rel_err

import oracle

REL_TOL = 2e-4  # test_parity.py:17

CASES = golden_case_arrays()
SMALL = [name for name, (X, k, _) in CASES.items() if X.shape[0] <= 3000]


def test_golden_inputs_regenerate_exactly(sk_golden):
    for name, (X, _, _) in CASES.items():
        assert hashlib.sha256(np.ascontiguousarray(X).tobytes()).hexdigest() == sk_golden.meta[name]["sha256"], name


@pytest.mark.parametrize("name", SMALL)
def test_oracle_matches_sklearn(name, sk_golden):
    X, k, normalize = CASES[name]
    got = oracle.lof(X, k, normalize)
    want = sk_golden[f"{name}/scores"]
    if name == "duplicates":
        # test_regressions.py:58-67: heavy ties, absolute 1e-2
        assert np.max(np.abs(got - want)) < 1e-2
        assert len(np.unique(got)) > 1
        return
    rel = rel_err(got, want)
    if rel.max() >= REL_TOL:
        # Only float32 near-ties of the k-th / (k+1)-th neighbour may disagree.
        bad = np.flatnonzero(rel >= REL_TOL)
        dk, dk1 = sk_golden[f"{name}/dist_k"], sk_golden[f"{name}/dist_k1"]
        gap = (dk1 - dk) / np.maximum(dk, 1e-12)
        assert gap[bad].max() < 1e-3, f"{name}: disagreement away from a near-tie"
        assert len(bad) < max(2, X.shape[0] // 100)


@pytest.mark.parametrize("name", ["clusters_n20000_d8_k20", "neartie_n20000_d8_k20"])
def test_oracle_near_tie_template(name, sk_golden):
    """test_parity.py:70-100, with the tighter medians this engine targets."""
    X, k, _ = CASES[name]
    got = oracle.lof(X, k)
    want = sk_golden[f"{name}/scores"]
    rel = rel_err(got, want)
    assert np.median(rel) < 1e-6
    assert np.percentile(rel, 99) < 1e-5
    bad = np.flatnonzero(rel > 1e-4)
    assert len(bad) < X.shape[0] // 100
    gap = (sk_golden[f"{name}/dist_k1"] - sk_golden[f"{name}/dist_k"]) / np.maximum(sk_golden[f"{name}/dist_k"], 1e-12)
    if len(bad):
        assert gap[bad].max() < 1e-3
    top = X.shape[0] // 100
    assert set(np.argsort(-got)[:top]) == set(np.argsort(-want)[:top])
    # flagged set at contamination 0.01 equals scikit-learn's
    labels, _, _ = oracle.fit_predict(X, k, 0.01)
    want_out = np.unpackbits(sk_golden[f"{name}/outlier_bits"])[: X.shape[0]].astype(bool)
    assert np.array_equal(labels == -1, want_out)


@pytest.mark.parametrize("n,d,k,seed", [(400, 3, 20, 11), (512, 32, 15, 3), (128, 2, 127, 7), (600, 4, 257, 5)])
def test_oracle_matches_fp64_restatement(n, d, k, seed):
    """test_culof.cu:102-132 shapes against the FP64 dense LOF (rel < 1e-4)."""
    rng = np.random.default_rng(seed)
    X = rng.standard_normal((n, d)).astype(np.float32)
    X[: max(1, n // 50)] = rng.uniform(-12, 12, (max(1, n // 50), d)).astype(np.float32)
    Xc, _, _ = oracle.center(X)
    assert max_rel_err(oracle.lof(X, k), fp64_lof(Xc, k)) < 1e-4


def test_centring_matches_fp64():
    rng = np.random.default_rng(0)
    X = (rng.standard_normal((1000, 5)) * 3 + 7).astype(np.float32)
    Xc, mean, inv = oracle.center(X)
    np.testing.assert_allclose(mean, X.astype(np.float64).mean(0), rtol=1e-13)
    assert np.all(inv == 1.0)
    np.testing.assert_array_equal(Xc, (X.astype(np.float64) - mean).astype(np.float32))
    Z, mean, inv = oracle.center(X, normalize=True)
    np.testing.assert_allclose(inv, 1.0 / X.astype(np.float64).std(0), rtol=1e-12)
    X[:, 2] = 4.0  # zero variance keeps scale 1 (preprocess.cu:62-65)
    Z, _, inv = oracle.center(X, normalize=True)
    assert inv[2] == 1.0 and np.all(Z[:, 2] == 0.0)


def test_distance_is_direct_difference_fma_order():
    rng = np.random.default_rng(1)
    a, b = rng.standard_normal(7).astype(np.float32), rng.standard_normal(7).astype(np.float32)
    s = np.float32(0.0)
    for f in range(7):
        t = np.float32(a[f] - b[f])
        s = np.float32(np.float64(t) * np.float64(t) + np.float64(s))  # fma: exact product, one rounding
    assert oracle.dist2(a, b) == s
    assert oracle.dist2(a, b) == oracle.dist2(b, a)


def test_knn_tie_rule_and_slot_order():
    """Equal distances break by ascending index; slots list keys below the
    k-th by index, then the ties (knn.cu:190-224)."""
    X = np.array([[0.0], [1.0], [-1.0], [2.0], [-2.0], [1.0], [3.0]], np.float32)
    idx, d2, kd = oracle.knn(X, 3)
    # point 0: d2 = 1 for 1, 2, 5 (tie at the 3rd): all three selected; sorted by index
    assert kd[0] == 1.0
    assert list(idx[:, 0]) == [1, 2, 5]
    # point 1: dist to 5 is 0, then 0 and 3 at 1: k=3 -> {5} below, ties {0, 3}
    assert list(idx[:, 1]) == [5, 0, 3] and kd[1] == 1.0


@pytest.mark.parametrize("name", ["values_n2000_d8_k20", "largek_k64"])
def test_oracle_knn_matches_bruteforce_sort(name):
    X, k, _ = CASES[name]
    Xc, _, _ = oracle.center(X)
    idx, d2, kd = oracle.knn(Xc, k)
    n = X.shape[0]
    for i in range(0, n, 97):
        D = np.array([oracle.dist2(Xc[i], Xc[j]) if j != i else np.inf for j in range(n)], np.float32)
        order = np.lexsort((np.arange(n), D))[:k]
        assert set(order) == set(idx[:, i])
        assert kd[i] == D[order[-1]]


def test_percentile_offset_matches_numpy():
    rng = np.random.default_rng(2)
    for n in (2, 3, 10, 1000, 20_001):
        nof = -(1.0 + np.abs(rng.standard_normal(n))).astype(np.float32)
        nof[rng.choice(n, size=n // 4, replace=False)] = nof[0]
        for c in (0.001, 0.01, 0.0123, 0.05, 0.1, 0.25, 0.3333, 0.5, 1e-6):
            assert oracle.percentile_offset(nof, c) == float(np.percentile(nof, 100.0 * c)), (n, c)


def test_offset_and_labels_match_reference_python_layer(ref_layer_golden):
    for case in ref_layer_golden.meta["cases"]:
        scores = ref_layer_golden[f"{case['scores']}/scores"]
        nof = -scores
        c = case["contamination"]
        off = -1.5 if c == "auto" else oracle.percentile_offset(nof, c)
        assert off == case["offset"], case
        want = np.unpackbits(ref_layer_golden[f"{case['key']}/outlier_bits"])[: case["n"]].astype(bool)
        assert np.array_equal(oracle.labels(nof, off) == -1, want), case


def test_ref_select_tile_restatement():
    """Injected distances through the Gram contract: norms 0 and tile = -d2/2
    give raw = d2 exactly (power-of-two scaling)."""
    rng = np.random.default_rng(3)
    n, rows, k = 300, 40, 17
    D = np.abs(rng.standard_normal((rows, n))).astype(np.float32)
    D[:, ::7] = D[:, 3:4]  # many exact ties
    tile = (-D / 2).astype(np.float32)
    idx, d2, kd = oracle.ref_select_tile(tile, np.zeros(n, np.float32), row_offset=100, k=k)
    for r in range(rows):
        i = 100 + r
        key = D[r].copy()
        key[i] = np.inf
        order = np.lexsort((np.arange(n), key))[:k]
        assert kd[i] == key[order[-1]]
        kth = kd[i]
        lt = sorted(j for j in order if key[j] < kth)
        eq = sorted(j for j in order if key[j] == kth)
        assert list(idx[:, i]) == lt + eq
        np.testing.assert_array_equal(d2[:, i], key[lt + eq])
