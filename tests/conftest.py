"""Shared fixtures: builds, markers, golden data and helpers."""

from __future__ import annotations

import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")
    # Build the CUDA library and the CPU oracle once per session (the builder
    # is loaded by path: importing the package needs the library it builds).
    import __graft_entry__

    __graft_entry__._load_builder().build()
    import oracle

    oracle.build()


def has_gpu() -> bool:
    import culof_gb300

    return culof_gb300.cuda_available()


@pytest.fixture(scope="session")
def gpu_available() -> bool:
    return has_gpu()


@pytest.fixture(autouse=True)
def _skip_gpu_without_device(request):
    if request.node.get_closest_marker("gpu") and not has_gpu():
        pytest.skip("no CUDA device")


def max_rel_err(got, want) -> float:
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return float(np.max(np.abs(got - want) / np.maximum(np.abs(want), 1e-9)))


def rel_err(got, want) -> np.ndarray:
    got = np.asarray(got, np.float64)
    want = np.asarray(want, np.float64)
    return np.abs(got - want) / np.maximum(np.abs(want), 1e-9)


class Golden:
    """Lazy access to the committed .npz fixtures."""

    def __init__(self, name: str):
        self.z = np.load(os.path.join(GOLDEN, name))
        self.meta = json.loads(bytes(self.z["meta_json"]).decode())

    def __getitem__(self, key):
        return self.z[key]


@pytest.fixture(scope="session")
def sk_golden() -> Golden:
    return Golden("sklearn_cases.npz")


@pytest.fixture(scope="session")
def ref_layer_golden() -> Golden:
    return Golden("reference_python_layer.npz")


def golden_case_arrays():
    """{name: (X, k, normalize)} regenerated from the golden cases' seeds."""
    if GOLDEN not in sys.path:
        sys.path.insert(0, GOLDEN)
    from cases import case_inputs

    return {name: (X, k, normalize) for name, X, k, normalize, _ in case_inputs()}


def fp64_lof(X: np.ndarray, k: int) -> np.ndarray:
    """Dense FP64 LOF, straight from Breunig et al. (the reference's cpu_lof,
    tests/cpp/test_culof.cu:39-80): ties in distance broken by index."""
    X = np.asarray(X, np.float64)
    n = X.shape[0]
    D = np.sqrt(((X[:, None, :] - X[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(D, np.inf)
    order = np.lexsort((np.broadcast_to(np.arange(n), (n, n)), D), axis=1)[:, :k]
    nbr = order
    kdist = D[np.arange(n), nbr[:, -1]]
    reach = np.maximum(kdist[nbr], D[np.arange(n)[:, None], nbr])
    lrd = 1.0 / (reach.mean(1) + 1e-10)
    return (lrd[nbr] / lrd[:, None]).mean(1)
