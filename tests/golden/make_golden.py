"""Generate the golden fixtures in this directory (run in a container that has
scikit-learn and the reference source tree; the committed .npz files are what
the tests read, so neither is needed at test time).

Two kinds of golden data:

1. ``sklearn_cases.npz``: scikit-learn ``LocalOutlierFactor`` outputs (float64)
   on seeded inputs. scikit-learn is the reference's own test oracle
   (tests/python/conftest.py:10-12, test_parity.py) and its CPU comparison path
   (benchmarks/benchmark.py:91-94). Inputs are regenerated from their seeds at
   test time; a SHA-256 of each input array is stored to catch generator drift.
   For the near-tie analysis the k-th and (k+1)-th neighbour distances
   (NearestNeighbors, stored as float32) are kept too (test_parity.py:70-100).
   Labels are stored as packed bits (1 = outlier) at contamination 0.01.

2. ``reference_python_layer.npz``: the reference's own Python layer
   (src/culof/__init__.py) imported with a stub native module that returns given
   scores, so ``LOF.fit``'s offset_ (np.percentile) and ``predict`` labels are the
   reference's exact outputs for those scores, plus the messages of the
   ValueErrors its validation raises.

3. ``fullsize_clusters_n200000.npz``: scikit-learn's flagged set (packed
   outlier bits at contamination 0.01), offset_ and the float32 scores of the
   plain exact-LOF workload at full size (n = 200,000, d = 8, k = 20; the
   seeded 5-cluster + 1% outlier generator, seed 1), which the GPU test of that
   workload compares against (the reference's near-tie template,
   test_parity.py:70-100, and its benchmark's agreement gate,
   benchmarks/benchmark.py:102-116).

Usage:  python tests/golden/make_golden.py --reference REF_ROOT [--only sklearn|layer|fullsize]
(REF_ROOT is the reference's source tree, also taken from $CULOF_REFERENCE;
only the ``layer`` fixtures read it.)
"""

from __future__ import annotations

import hashlib
import importlib.util
import json
import os
import sys
import types

import numpy as np
from sklearn.neighbors import LocalOutlierFactor, NearestNeighbors

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import case_inputs  # noqa: E402  (tests/golden/cases.py)


def sha(X: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(X).tobytes()).hexdigest()


def make_sklearn_cases(path: str) -> None:
    arrays = {}
    meta = {}
    for name, X, k, normalize, Xs in case_inputs():
        lof = LocalOutlierFactor(n_neighbors=k, contamination=0.01).fit(Xs)
        arrays[f"{name}/scores"] = -lof.negative_outlier_factor_.astype(np.float64)
        arrays[f"{name}/outlier_bits"] = np.packbits(lof.fit_predict(Xs) == -1)
        kk = min(k + 2, X.shape[0])
        dist, _ = NearestNeighbors(n_neighbors=kk).fit(Xs).kneighbors(Xs)
        # column 0 is the point itself; the k-th neighbour is column k. float32
        # is ample for the near-tie gap (a relative threshold of 1e-3).
        arrays[f"{name}/dist_k"] = dist[:, k].astype(np.float32)
        if k + 1 < kk:
            arrays[f"{name}/dist_k1"] = dist[:, k + 1].astype(np.float32)
        meta[name] = {"n": int(X.shape[0]), "d": int(X.shape[1]), "k": int(k), "normalize": bool(normalize),
                      "sha256": sha(X), "offset_c001": float(lof.offset_)}
    arrays["meta_json"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrays)


def import_reference_python_layer(ref_root: str, fake_scores):
    """Import the reference's src/culof package with a stub native module."""
    pkg_dir = os.path.join(ref_root, "src", "culof")
    fake = types.ModuleType("culof_refpkg._culof")
    fake.cuda_available = lambda: True
    fake.device_info = lambda: "stub"
    fake.lof = lambda arr, k, normalize: fake_scores(arr, k, normalize)
    sys.modules["culof_refpkg._culof"] = fake
    spec = importlib.util.spec_from_file_location(
        "culof_refpkg", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir]
    )
    mod = importlib.util.module_from_spec(spec)
    sys.modules["culof_refpkg"] = mod
    spec.loader.exec_module(mod)
    return mod


def make_reference_layer(path: str, ref_root: str) -> None:
    rng = np.random.default_rng(1234)
    current = {}
    ref = import_reference_python_layer(ref_root, lambda arr, k, normalize: current["scores"])
    arrays = {}
    cases = []
    # Score vectors with many shapes: continuous, heavy ties, tiny n.
    for ci, n in enumerate([2, 3, 7, 100, 1001, 4096, 20_000]):
        s = (1.0 + np.abs(rng.standard_normal(n)) * rng.uniform(0.01, 3.0)).astype(np.float32)
        if ci % 2 == 0 and n > 10:
            s[rng.choice(n, size=n // 3, replace=False)] = s[0]  # ties at one value
        arrays[f"s{ci}/scores"] = s
        for c in ["auto", 0.001, 0.01, 0.0123, 0.05, 0.1, 0.25, 0.3333, 0.5]:
            current["scores"] = s
            X = np.zeros((n, 1), np.float32)
            m = ref.LOF(n_neighbors=1, contamination=c).fit(X)
            key = f"c{len(cases)}"
            arrays[f"{key}/outlier_bits"] = np.packbits(m.predict() == -1)
            cases.append({"key": key, "scores": f"s{ci}", "n": n, "contamination": c,
                          "offset": float(m.offset_)})
    # Validation messages (__init__.py:37-80, 159-171).
    errors = {}
    for label, fn in [
        ("k0", lambda: ref.LOF(n_neighbors=0)),
        ("contam_bad", lambda: ref.LOF(contamination=0.9)),
        ("k_too_big", lambda: ref.LOF(n_neighbors=100).fit(np.zeros((100, 2), np.float32))),
        ("not_2d", lambda: ref.lof(np.zeros(10, np.float32), 3)),
        ("nan", lambda: ref.lof(np.array([[0.0, np.nan], [1.0, 1.0], [2.0, 2.0]], np.float32), 1)),
        ("overflow", lambda: ref.lof((np.ones((64, 4)) * 1e20).astype(np.float32), 5)),
        ("no_features", lambda: ref.lof(np.zeros((5, 0), np.float32), 1)),
        ("unfitted", lambda: ref.LOF().predict()),
    ]:
        try:
            fn()
            errors[label] = None
        except Exception as e:  # noqa: BLE001
            errors[label] = [type(e).__name__, str(e)]
    meta = {"cases": cases, "errors": errors, "repr": repr(ref.LOF(n_neighbors=7)),
            "version": ref.__version__, "all": list(ref.__all__)}
    arrays["meta_json"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8)
    np.savez_compressed(path, **arrays)


FULLSIZE = {"n": 200_000, "d": 8, "k": 20, "contamination": 0.01, "seed": 1}


def make_fullsize(path: str) -> None:
    from culof_gb300 import synthetic

    f = FULLSIZE
    X = synthetic.clusters_with_outliers(f["n"], f["d"], seed=f["seed"])
    lof = LocalOutlierFactor(n_neighbors=f["k"], contamination=f["contamination"], n_jobs=-1)
    labels = lof.fit_predict(X.astype(np.float64))
    meta = dict(f, sha256=sha(X), offset=float(lof.offset_), n_outliers=int(np.sum(labels == -1)))
    np.savez_compressed(
        path,
        outlier_bits=np.packbits(labels == -1),
        scores=(-lof.negative_outlier_factor_).astype(np.float32),
        meta_json=np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8),
    )


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("CULOF_REFERENCE"),
                    help="the reference's source tree (needed for the 'layer' fixtures)")
    ap.add_argument("--only", choices=["sklearn", "layer", "fullsize"])
    a = ap.parse_args()
    if a.only in (None, "sklearn"):
        make_sklearn_cases(os.path.join(HERE, "sklearn_cases.npz"))
    if a.only in (None, "layer"):
        if not a.reference:
            ap.error("--reference (or $CULOF_REFERENCE) is required for the reference-layer fixtures")
        make_reference_layer(os.path.join(HERE, "reference_python_layer.npz"), a.reference)
    if a.only in (None, "fullsize"):
        make_fullsize(os.path.join(HERE, "fullsize_clusters_n200000.npz"))
    print("wrote", sorted(os.listdir(HERE)))
