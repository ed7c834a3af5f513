"""Binding to libculof_gb300.so over its C ABI (include/culof_c.h).

Mirrors the reference's pybind11 module ``_culof`` (src/cuda/binding.cpp:25-56):
``lof(points, k, normalize)`` coerces to C-contiguous float32 (binding.cpp:23),
rejects non-2-D input with ValueError (:27-30), releases the GIL while the
GPU works (ctypes foreign calls do), and returns a fresh float32 array
(:40-42); ``cuda_available()``, ``device_info()`` and the ``CudaError``
RuntimeError subclass (:55). Invalid arguments raise ValueError, as pybind11
translates the reference's std::invalid_argument.

There is no CPU fallback: if the library is missing, importing this module
fails with the build instruction.
"""

from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libculof_gb300.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_NO_DEVICE = 3
ERR_INTERNAL = 4
ERR_KERNEL = 5

PATH_AUTO, PATH_FAST, PATH_GENERAL, PATH_TENSOR = 0, 1, 2, 3


class CudaError(RuntimeError):
    """Any CUDA failure (the reference's culof::CudaError)."""


if not os.path.exists(LIB_PATH):
    raise ImportError(
        f"{LIB_PATH} is missing: build the CUDA library first "
        "(python -c 'import culof_gb300._build as b; b.build()')"
    )

_lib = ctypes.CDLL(LIB_PATH)

_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_I = ctypes.c_int
_D = ctypes.c_double
_SZ = ctypes.c_size_t

_SIGS = {
    "culof_version": ([], ctypes.c_char_p),
    "culof_last_error": ([], ctypes.c_char_p),
    "culof_cuda_available": ([], _I),
    "culof_device_info": ([ctypes.c_char_p, _SZ], _I),
    "culof_context_create": ([ctypes.POINTER(_P)], _I),
    "culof_context_destroy": ([_P], None),
    "culof_context_set_stream": ([_P, _P], _I),
    "culof_context_synchronize": ([_P], _I),
    "culof_context_set_path": ([_P, _I], _I),
    "culof_context_last_path": ([_P], _I),
    "culof_context_set_timing": ([_P, _I], _I),
    "culof_context_stage_times": ([_P, _P, _I], _I),
    "culof_kernel_launch_count": ([], ctypes.c_ulonglong),
    "culof_probe_fp32_tflops": ([_I, ctypes.POINTER(_D)], _I),
    "culof_lof": ([_P, _I64, _I, _I, _I, _P], _I),
    "culof_context_lof": ([_P, _P, _I64, _I, _I, _I, _P], _I),
    "culof_fit_predict": ([_P, _I64, _I, _I, _I, _D, _P, _P, _P], _I),
    "culof_context_fit_predict": ([_P, _P, _I64, _I, _I, _I, _D, _P, _P, _P], _I),
    "culof_context_lof_device": ([_P, _P, _I64, _I, _I, _I, _P], _I),
    "culof_context_fit_predict_device": ([_P, _P, _I64, _I, _I, _I, _D, _P, _P, _P], _I),
    "culof_choose_tile_rows": ([_I64, _SZ], _I),
    "culof_select_knn_tile": ([_P, _P, _P, _I, _I64, _I64, _I, _P, _P, _P], _I),
    "culof_context_knn_device": ([_P, _P, _I64, _I, _I, _I, _P, _P, _P], _I),
    "culof_compute_lrd": ([_P, _P, _P, _P, _I64, _I, _P], _I),
    "culof_context_lof_backward_device": ([_P, _P, _I64, _I, _I, _I, _P, _P, _P, _P], _I),
    "culof_context_lof_batched_device": ([_P, _I, _P, _P, _P, _I, _I, _P], _I),
    "culof_context_set_graphs": ([_P, _I], _I),
    "culof_context_batched_tuning": ([_P, _P, ctypes.POINTER(_I), ctypes.POINTER(_I)], _I),
    "culof_lof_batched": ([_I, _P, _P, _P, _I, _I, _P], _I),
    "culof_context_lof_batched": ([_P, _I, _P, _P, _P, _I, _I, _P], _I),
    "culof_context_pair_stats": ([_P, ctypes.POINTER(_D), ctypes.POINTER(_D)], _I),
    "culof_context_probe_bounded_wait": ([_P, ctypes.c_longlong], _I),
    "culof_compute_scores": ([_P, _P, _P, _I64, _I, _P], _I),
    "culof_context_knn_shard_device": ([_P, _P, _I64, _I, _I, _I, _I, _I, _P, _P, _P, _P, ctypes.POINTER(_I64)], _I),
    "culof_compute_lrd_rows": ([_P, _P, _P, _P, _I64, _I, _P, _I64, _P], _I),
    "culof_compute_scores_rows": ([_P, _P, _P, _I64, _I, _P, _I64, _P], _I),
    "culof_context_contamination_offset_device": ([_P, _P, _I64, _D, _P], _I),
    "culof_contamination_offset_noalloc": ([_P, _P, _I64, _D, _P], _I),
    "culof_context_bf16_gram": ([_P, _P, _I64, _P, _I64, _I, _P], _I),
}
for _name, (_args, _res) in _SIGS.items():
    _fn = getattr(_lib, _name)
    _fn.argtypes = _args
    _fn.restype = _res

EXPORTED = tuple(_SIGS)


def _check(rc: int) -> None:
    if rc == OK:
        return
    msg = _lib.culof_last_error().decode(errors="replace")
    if rc == ERR_INVALID_ARGUMENT:
        raise ValueError(msg)
    raise CudaError(msg or f"culof error status {rc}")


def _as_points(points) -> np.ndarray:
    arr = np.ascontiguousarray(points, dtype=np.float32)
    if arr.ndim != 2:
        raise ValueError("expected a 2-D array of shape (n_samples, n_features)")
    return arr


def version() -> str:
    return _lib.culof_version().decode()


def cuda_available() -> bool:
    return bool(_lib.culof_cuda_available())


def device_info() -> str:
    buf = ctypes.create_string_buffer(512)
    if _lib.culof_device_info(buf, 512) != OK:
        return "unknown device"
    return buf.value.decode(errors="replace")


def lof(points, k: int, normalize: bool) -> np.ndarray:
    """Raw LOF scores (positive) for a (n_samples, n_features) array."""
    arr = _as_points(points)
    out = np.empty(arr.shape[0], np.float32)
    _check(_lib.culof_lof(arr.ctypes.data, arr.shape[0], arr.shape[1], int(k), int(bool(normalize)), out.ctypes.data))
    return out


def fit_predict(points, k: int, normalize: bool, contamination):
    """(negative_outlier_factor_, labels, offset_) computed on the GPU."""
    arr = _as_points(points)
    n = arr.shape[0]
    nof = np.empty(n, np.float32)
    labels = np.empty(n, np.int64)
    off = ctypes.c_double(0.0)
    c = -1.0 if contamination == "auto" else float(contamination)
    _check(
        _lib.culof_fit_predict(
            arr.ctypes.data, n, arr.shape[1], int(k), int(bool(normalize)), c, nof.ctypes.data,
            labels.ctypes.data, ctypes.addressof(off),
        )
    )
    return nof, labels, off.value


def lof_batched(problems, ks, normalize: bool) -> list:
    """Raw LOF scores of many independent problems (each (n_i, d) float32,
    one k per problem) in one GPU call; a list of float32 arrays."""
    arrs = [_as_points(p) for p in problems]
    if not arrs:
        return []
    d = arrs[0].shape[1]
    if any(a.shape[1] != d for a in arrs):
        raise ValueError("every problem must have the same number of features")
    kk = np.ascontiguousarray(ks, dtype=np.int32)
    if kk.shape != (len(arrs),):
        raise ValueError("one k per problem")
    off = np.zeros(len(arrs) + 1, np.int64)
    off[1:] = np.cumsum([a.shape[0] for a in arrs])
    X = np.ascontiguousarray(np.concatenate(arrs), dtype=np.float32)
    out = np.empty(X.shape[0], np.float32)
    _check(_lib.culof_lof_batched(len(arrs), off.ctypes.data, kk.ctypes.data, X.ctypes.data, d,
                                  int(bool(normalize)), out.ctypes.data))
    return [out[off[i]:off[i + 1]].copy() for i in range(len(arrs))]


def contamination_offset_noalloc(stream: int, nof: int, n_points: int, contamination, offset: int) -> None:
    """offset_ of a device nof array into a device double, allocating nothing
    (culof_contamination_offset_noalloc: for callers that cannot allocate
    device memory while they run; n_points <= 2^31 - 1; concurrent calls race)."""
    c = -1.0 if contamination == "auto" else float(contamination)
    _check(_lib.culof_contamination_offset_noalloc(stream, nof, int(n_points), c, offset))


def kernel_launch_count() -> int:
    """Kernels this library has launched in this process."""
    return int(_lib.culof_kernel_launch_count())


def probe_fp32_tflops(packed: bool = True) -> float:
    """Measured FP32 FMA throughput of the current device (TFLOP/s)."""
    v = _D(0.0)
    _check(_lib.culof_probe_fp32_tflops(int(bool(packed)), ctypes.byref(v)))
    return v.value


def choose_tile_rows(n_points: int, budget_bytes: int) -> int:
    return int(_lib.culof_choose_tile_rows(int(n_points), int(budget_bytes)))


def select_knn_tile(stream: int, tile: int, norms: int, rows: int, row_offset: int, n_points: int, k: int,
                    nbr_idx: int, nbr_d2: int, kdist2: int) -> None:
    """The reference's select_knn tile contract on device pointers (ints)."""
    _check(_lib.culof_select_knn_tile(stream, tile, norms, rows, row_offset, n_points, k, nbr_idx, nbr_d2, kdist2))


def compute_lrd(stream: int, nbr_idx: int, nbr_d2: int, kdist2: int, n_points: int, k: int, lrd: int) -> None:
    _check(_lib.culof_compute_lrd(stream, nbr_idx, nbr_d2, kdist2, n_points, k, lrd))


def compute_lrd_rows(stream: int, nbr_idx: int, nbr_d2: int, kdist2: int, n_points: int, k: int, rows: int,
                     num_rows: int, lrd: int) -> None:
    _check(_lib.culof_compute_lrd_rows(stream, nbr_idx, nbr_d2, kdist2, n_points, k, rows, num_rows, lrd))


def compute_scores_rows(stream: int, nbr_idx: int, lrd: int, n_points: int, k: int, rows: int, num_rows: int,
                        scores: int) -> None:
    _check(_lib.culof_compute_scores_rows(stream, nbr_idx, lrd, n_points, k, rows, num_rows, scores))


def compute_scores(stream: int, nbr_idx: int, lrd: int, n_points: int, k: int, scores: int) -> None:
    _check(_lib.culof_compute_scores(stream, nbr_idx, lrd, n_points, k, scores))


class Context:
    """A culof_context: own stream and grow-only device workspaces.

    Device-pointer methods take integers (e.g. ``tensor.data_ptr()``) and
    queue work on the context stream without synchronising.
    """

    def __init__(self) -> None:
        h = _P()
        _check(_lib.culof_context_create(ctypes.byref(h)))
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.culof_context_destroy(self._h)
            self._h = None

    def __del__(self) -> None:  # pragma: no cover - interpreter teardown
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self) -> "Context":
        return self

    def __exit__(self, *exc) -> None:
        self.close()

    def set_stream(self, stream: int) -> None:
        _check(_lib.culof_context_set_stream(self._h, stream))

    def synchronize(self) -> None:
        _check(_lib.culof_context_synchronize(self._h))

    def set_path(self, path: int) -> None:
        _check(_lib.culof_context_set_path(self._h, int(path)))

    def last_path(self) -> int:
        return int(_lib.culof_context_last_path(self._h))

    STAGES = ("prep", "order", "seed", "sweep", "merge", "lrd_score", "offset_labels")

    def set_timing(self, on: bool) -> None:
        _check(_lib.culof_context_set_timing(self._h, int(bool(on))))

    def stage_times(self) -> dict:
        """Milliseconds per stage of the last call (CUDA events; synchronises)."""
        buf = (ctypes.c_float * len(self.STAGES))()
        _check(_lib.culof_context_stage_times(self._h, buf, len(self.STAGES)))
        return {name: float(v) for name, v in zip(self.STAGES, buf) if v >= 0}

    @property
    def handle(self) -> int:
        return self._h.value

    def lof(self, points, k: int, normalize: bool = False) -> np.ndarray:
        arr = _as_points(points)
        out = np.empty(arr.shape[0], np.float32)
        _check(_lib.culof_context_lof(self._h, arr.ctypes.data, arr.shape[0], arr.shape[1], int(k),
                                      int(bool(normalize)), out.ctypes.data))
        return out

    def fit_predict(self, points, k: int, normalize: bool = False, contamination="auto"):
        arr = _as_points(points)
        n = arr.shape[0]
        nof = np.empty(n, np.float32)
        labels = np.empty(n, np.int64)
        off = ctypes.c_double(0.0)
        c = -1.0 if contamination == "auto" else float(contamination)
        _check(_lib.culof_context_fit_predict(self._h, arr.ctypes.data, n, arr.shape[1], int(k),
                                              int(bool(normalize)), c, nof.ctypes.data, labels.ctypes.data,
                                              ctypes.addressof(off)))
        return nof, labels, off.value

    def fit_predict_host_ptr(self, points: int, n: int, d: int, k: int, normalize: bool, contamination,
                             nof: int, labels: int, offset: int) -> None:
        """Host-pointer fit_predict on raw addresses (e.g. pinned buffers)."""
        c = -1.0 if contamination == "auto" else float(contamination)
        _check(_lib.culof_context_fit_predict(self._h, points, n, d, int(k), int(bool(normalize)), c, nof,
                                              labels, offset))

    def lof_device(self, points: int, n: int, d: int, k: int, normalize: bool, scores: int) -> None:
        _check(_lib.culof_context_lof_device(self._h, points, n, d, int(k), int(bool(normalize)), scores))

    def fit_predict_device(self, points: int, n: int, d: int, k: int, normalize: bool, contamination,
                           nof: int, labels: int, offset: int) -> None:
        c = -1.0 if contamination == "auto" else float(contamination)
        _check(_lib.culof_context_fit_predict_device(self._h, points, n, d, int(k), int(bool(normalize)), c, nof,
                                                     labels, offset))

    def knn_device(self, points: int, n: int, d: int, k: int, normalize: bool, nbr_idx: int, nbr_d2: int,
                   kdist2: int) -> None:
        _check(_lib.culof_context_knn_device(self._h, points, n, d, int(k), int(bool(normalize)), nbr_idx, nbr_d2,
                                             kdist2))

    def knn_shard_device(self, points: int, n: int, d: int, k: int, normalize: bool, shard: int, num_shards: int,
                         nbr_idx: int, nbr_d2: int, kdist2: int, rows: int) -> int:
        """One shard of a row-sharded k-NN; returns the number of rows it wrote."""
        m = ctypes.c_int64(0)
        _check(_lib.culof_context_knn_shard_device(self._h, points, n, d, int(k), int(bool(normalize)), int(shard),
                                                   int(num_shards), nbr_idx, nbr_d2, kdist2, rows,
                                                   ctypes.byref(m)))
        return int(m.value)

    def lof_batched_device(self, offsets, ks, points: int, d: int, normalize: bool, scores: int) -> None:
        """LOF scores of many problems in one call (device points/scores,
        host offsets[num + 1] and ks[num]); graph-replayed when repeated."""
        off = np.ascontiguousarray(offsets, dtype=np.int64)
        kk = np.ascontiguousarray(ks, dtype=np.int32)
        if off.ndim != 1 or kk.ndim != 1 or off.shape[0] != kk.shape[0] + 1:
            raise ValueError("offsets must have one more entry than ks")
        _check(_lib.culof_context_lof_batched_device(self._h, int(kk.shape[0]), off.ctypes.data, kk.ctypes.data,
                                                     points, int(d), int(bool(normalize)), scores))

    def pair_stats(self):
        """(evaluated pairs, unpruned pairs) of the last small-d FP32 sweep."""
        ev, tot = _D(0.0), _D(0.0)
        _check(_lib.culof_context_pair_stats(self._h, ctypes.byref(ev), ctypes.byref(tot)))
        return ev.value, tot.value

    def probe_bounded_wait(self, spin_limit: int = 1 << 14) -> None:
        """Run a bounded wait that never completes; raises CudaError (the
        failure path of every kernel wait), the context stays usable."""
        _check(_lib.culof_context_probe_bounded_wait(self._h, int(spin_limit)))

    def batched_tuning(self) -> dict:
        """The batched autotuner's variant times (ms) and choice for the current layout."""
        ms = np.zeros(4, np.float32)
        per, pairs = ctypes.c_int(0), ctypes.c_int(0)
        _check(_lib.culof_context_batched_tuning(self._h, ms.ctypes.data, ctypes.byref(per), ctypes.byref(pairs)))
        times = {f"{c}cta_{p}pair": float(ms[2 * (c - 1) + (p - 1)]) for c in (1, 2) for p in (1, 2)
                 if ms[2 * (c - 1) + (p - 1)] >= 0}
        return {"ms": times, "ctas_per_sm": per.value, "pairs_per_lane": pairs.value}

    def set_graphs(self, on: bool) -> None:
        _check(_lib.culof_context_set_graphs(self._h, int(bool(on))))

    def lof_backward_device(self, points: int, n: int, d: int, k: int, normalize: bool, nbr_idx: int,
                            grad_scores: int, grad_points: int, scores_out: int = 0) -> None:
        """FP64 gradient of sum_i g_i score_i w.r.t. the points, neighbour sets fixed (device pointers)."""
        _check(_lib.culof_context_lof_backward_device(self._h, points, n, d, int(k), int(bool(normalize)), nbr_idx,
                                                      grad_scores, grad_points, scores_out or None))

    def bf16_gram(self, A: int, rows_a: int, B: int, rows_b: int, K: int, G: int) -> None:
        """G = A B^T on the tensor cores (bf16 in, f32 out; device pointers)."""
        _check(_lib.culof_context_bf16_gram(self._h, A, rows_a, B, rows_b, K, G))

    def offset_device(self, nof: int, n: int, contamination, offset: int) -> None:
        c = -1.0 if contamination == "auto" else float(contamination)
        _check(_lib.culof_context_contamination_offset_device(self._h, nof, n, c, offset))
