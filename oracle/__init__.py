"""CPU oracle for exact LOF: TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg (and its ``--impl reference`` arm) may import this package, and only as
the checker or the timed CPU baseline. The product package ``culof_gb300``
never imports it.

``build()`` compiles ``lof_oracle.c`` with gcc into ``oracle/_build/``;
the functions below are thin ctypes wrappers with numpy in and out.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "liblof_oracle.so")
_SRC = os.path.join(_HERE, "lof_oracle.c")
_HDR = os.path.join(_HERE, "lof_oracle.h")

# -ffp-contract=off: every float operation rounds exactly as written in the C
# source (no silent FMA contraction); no -ffast-math and no -march=native, so
# the x86 build here and the aarch64 build on the GPU host give equal bits.
CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread", "-std=c11"]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle library if it is missing or older than its sources."""
    os.makedirs(_BUILD, exist_ok=True)
    stale = (
        force
        or not os.path.exists(_LIB_PATH)
        or os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(_SRC), os.path.getmtime(_HDR))
    )
    if stale:
        tmp = _LIB_PATH + f".tmp{os.getpid()}"
        subprocess.run(["gcc", *CFLAGS, "-o", tmp, _SRC, "-lm"], check=True)
        os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def _load():
    global _lib
    with _lock:
        if _lib is None:
            build()
            lib = ctypes.CDLL(_LIB_PATH)
            P = ctypes.c_void_p
            i64, i32, dbl = ctypes.c_int64, ctypes.c_int, ctypes.c_double
            lib.oracle_center.argtypes = [P, i64, i32, i32, P, P, P]
            lib.oracle_norms.argtypes = [P, i64, i32, P]
            lib.oracle_dist2.argtypes = [P, P, i32]
            lib.oracle_dist2.restype = ctypes.c_float
            lib.oracle_knn_rows.argtypes = [P, i64, i32, i32, i64, i64, P, P, P, i32]
            lib.oracle_lrd.argtypes = [P, P, P, i64, i32, P]
            lib.oracle_score.argtypes = [P, P, i64, i32, P]
            lib.oracle_lof.argtypes = [P, i64, i32, i32, i32, P, i32]
            lib.oracle_lof.restype = i32
            lib.oracle_percentile_offset.argtypes = [P, i64, dbl]
            lib.oracle_percentile_offset.restype = dbl
            lib.oracle_labels.argtypes = [P, i64, dbl, P]
            lib.oracle_ref_select_tile.argtypes = [P, P, i32, i64, i64, i32, P, P, P]
            lib.oracle_knn_list.argtypes = [P, i64, i32, i32, P, i64, P, P, P, i32]
            lib.oracle_knn_f64.argtypes = [P, i64, i32, i32, i32, P, i64, P, P, i32]
            lib.oracle_lof_f64.argtypes = [P, i64, i32, i32, i32, P, i32]
            lib.oracle_lof_f64.restype = i32
            _lib = lib
    return _lib


def _ptr(a: np.ndarray) -> int:
    """Address of a's data. The caller must hold a reference to `a` until the
    C call returns (never pass a temporary conversion)."""
    return a.ctypes.data


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def center(X, normalize: bool = False):
    """Centred (optionally z-scored) float32 copy plus the FP64 means and 1/std."""
    X = _f32(X)
    n, d = X.shape
    out = np.empty_like(X)
    mean = np.empty(d, np.float64)
    inv = np.empty(d, np.float64)
    _load().oracle_center(_ptr(X), n, d, int(normalize), _ptr(out), _ptr(mean), _ptr(inv))
    return out, mean, inv


def norms(Xc) -> np.ndarray:
    Xc = _f32(Xc)
    n, d = Xc.shape
    out = np.empty(n, np.float32)
    _load().oracle_norms(_ptr(Xc), n, d, _ptr(out))
    return out


def dist2(a, b) -> float:
    a, b = _f32(a), _f32(b)
    return float(_load().oracle_dist2(_ptr(a), _ptr(b), a.shape[0]))


def knn(Xc, k: int, rows=None, nthreads: int = 0):
    """Exact k-NN of ``rows`` (a (begin, end) pair, default all) over all of Xc.

    Returns (nbr_idx int32 (k, n), nbr_d2 float32 (k, n), kdist2 float32 (n,)),
    in the reference's transposed layout; only the columns of the requested
    rows are written (the rest are -1 / NaN).
    """
    Xc = _f32(Xc)
    n, d = Xc.shape
    b, e = (0, n) if rows is None else rows
    idx = np.full((k, n), -1, np.int32)
    d2 = np.full((k, n), np.nan, np.float32)
    kd = np.full(n, np.nan, np.float32)
    _load().oracle_knn_rows(_ptr(Xc), n, d, k, b, e, _ptr(idx), _ptr(d2), _ptr(kd), nthreads)
    return idx, d2, kd


def lrd(nbr_idx, nbr_d2, kdist2) -> np.ndarray:
    idx = np.ascontiguousarray(nbr_idx, np.int32)
    d2, kd = _f32(nbr_d2), _f32(kdist2)
    k, n = idx.shape
    out = np.empty(n, np.float32)
    _load().oracle_lrd(_ptr(idx), _ptr(d2), _ptr(kd), n, k, _ptr(out))
    return out


def score(nbr_idx, lrd_) -> np.ndarray:
    idx = np.ascontiguousarray(nbr_idx, np.int32)
    lr = _f32(lrd_)
    k, n = idx.shape
    out = np.empty(n, np.float32)
    _load().oracle_score(_ptr(idx), _ptr(lr), n, k, _ptr(out))
    return out


def lof(X, k: int = 20, normalize: bool = False, nthreads: int = 0) -> np.ndarray:
    """Whole pipeline: positive LOF scores (float32)."""
    X = _f32(X)
    n, d = X.shape
    out = np.empty(n, np.float32)
    rc = _load().oracle_lof(_ptr(X), n, d, k, int(normalize), _ptr(out), nthreads)
    if rc != 0:
        raise ValueError("oracle_lof: invalid arguments")
    return out


def percentile_offset(nof, contamination: float) -> float:
    nof = _f32(nof)
    return float(_load().oracle_percentile_offset(_ptr(nof), nof.shape[0], float(contamination)))


def labels(nof, offset: float) -> np.ndarray:
    nof = _f32(nof)
    out = np.empty(nof.shape[0], np.int64)
    _load().oracle_labels(_ptr(nof), nof.shape[0], float(offset), _ptr(out))
    return out


def fit_predict(X, k: int = 20, contamination="auto", normalize: bool = False, nthreads: int = 0):
    """(labels, negative_outlier_factor_, offset_) as the reference's LOF.fit_predict."""
    scores = lof(X, k, normalize, nthreads)
    nof = -scores
    off = -1.5 if contamination == "auto" else percentile_offset(nof, float(contamination))
    return labels(nof, off), nof, off


def ref_select_tile(tile, norms_, row_offset: int, k: int):
    """The reference's Gram-tile select restated (knn.cu:119-232)."""
    tile = _f32(tile)
    rows, n = tile.shape
    idx = np.full((k, n), -1, np.int32)
    d2 = np.full((k, n), np.nan, np.float32)
    kd = np.full(n, np.nan, np.float32)
    nrm = _f32(norms_)
    _load().oracle_ref_select_tile(_ptr(tile), _ptr(nrm), rows, row_offset, n, k, _ptr(idx), _ptr(d2), _ptr(kd))
    return idx, d2, kd


def knn_list(Xc, k: int, rows, nthreads: int = 0):
    """Exact k-NN (the same select as ``knn``) of the listed rows over all of
    Xc: (nbr_idx int32 (k, m), nbr_d2 float32 (k, m), kdist2 float32 (m,)),
    column r for row ``rows[r]``."""
    Xc = _f32(Xc)
    n, d = Xc.shape
    rows = np.ascontiguousarray(rows, np.int64)
    m = rows.shape[0]
    idx = np.empty((k, m), np.int32)
    d2 = np.empty((k, m), np.float32)
    kd = np.empty(m, np.float32)
    _load().oracle_knn_list(_ptr(Xc), n, d, k, _ptr(rows), m, _ptr(idx), _ptr(d2), _ptr(kd), nthreads)
    return idx, d2, kd


def knn_f64(X, kk: int, normalize: bool = False, rows=None, nthreads: int = 0):
    """FP64 brute-force neighbours of the listed rows (default all): the kk
    nearest by (Euclidean distance, index), as (idx int64 (m, kk), dist
    float64 (m, kk)), ascending. Centres (and z-scores) in double first."""
    X = _f32(X)
    n, d = X.shape
    lst = None if rows is None else np.ascontiguousarray(rows, np.int64)
    m = n if lst is None else lst.shape[0]
    idx = np.empty((m, kk), np.int64)
    dist = np.empty((m, kk), np.float64)
    _load().oracle_knn_f64(_ptr(X), n, d, int(normalize), kk, None if lst is None else _ptr(lst), m,
                           _ptr(idx), _ptr(dist), nthreads)
    return idx, dist


def lof_f64(X, k: int = 20, normalize: bool = False, nthreads: int = 0) -> np.ndarray:
    """FP64 brute-force LOF scores from the definitions (the yardstick of the
    float32 engine's error; not bit-exact with it)."""
    X = _f32(X)
    n, d = X.shape
    out = np.empty(n, np.float64)
    if _load().oracle_lof_f64(_ptr(X), n, d, k, int(normalize), _ptr(out), nthreads) != 0:
        raise ValueError("oracle_lof_f64: invalid arguments")
    return out


def fp64_error(scores, X, k: int, normalize: bool = False) -> dict:
    """Median, p99 and max relative error of float32 LOF scores against the
    FP64 brute force of the same points."""
    ref = lof_f64(X, k, normalize)
    rel = np.abs(np.asarray(scores, np.float64) - ref) / np.maximum(np.abs(ref), 1e-300)
    return {"median": float(np.median(rel)), "p99": float(np.quantile(rel, 0.99)), "max": float(rel.max())}
