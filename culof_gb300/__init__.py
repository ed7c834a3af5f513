"""culof_gb300: exact Local Outlier Factor on NVIDIA GB300 (sm_103a).

The Python surface mirrors the reference cuLOF 0.2.0 package
(src/culof/__init__.py:1-227) name for name, so ``import culof_gb300 as culof``
is a drop-in for the fit_predict path:

    >>> from culof_gb300 import LOF
    >>> labels = LOF(n_neighbors=20, contamination=0.01).fit_predict(X)   # -1 outlier, 1 inlier

    >>> from culof_gb300 import lof
    >>> scores = lof(X, k=20)                         # ~1.0 normal, higher = more anomalous

Every numeric stage runs in hand-written CUDA kernels behind the C ABI of
libculof_gb300.so (include/culof_c.h); there is no CPU fallback.
"""

from __future__ import annotations

import math
from typing import TYPE_CHECKING

import numpy as np

from . import _culof
from ._version import __version__

if TYPE_CHECKING:  # pragma: no cover
    from numpy.typing import ArrayLike, NDArray

__all__ = ["LOF", "__version__", "cuda_available", "device_info", "lof"]

cuda_available = _culof.cuda_available
device_info = _culof.device_info
CudaError = _culof.CudaError


def _validate(X: ArrayLike, k: int) -> NDArray[np.float32]:
    """Input checks of the reference's _validate (__init__.py:37-55), same messages."""
    arr = np.ascontiguousarray(X, dtype=np.float32)
    if arr.ndim != 2:
        raise ValueError(f"expected a 2-D array of shape (n_samples, n_features), got shape {arr.shape}")
    n_samples, n_features = arr.shape
    if n_features < 1:
        raise ValueError("need at least one feature")
    if k < 1:
        raise ValueError(f"n_neighbors must be >= 1, got {k}")
    if k >= n_samples:
        raise ValueError(f"n_neighbors={k} requires at least {k + 1} samples, got {n_samples}")
    if not np.isfinite(arr).all():
        raise ValueError("input contains NaN or infinity")
    _check_representable(arr, n_features)
    return arr


def _check_representable(arr: NDArray[np.float32], n_features: int) -> None:
    """Reject input whose squared distances would overflow float32 (__init__.py:58-80).

    Centring bounds each coordinate by twice the input maximum, so a squared
    distance is at most ``n_features * (4 * max|x|)**2``; past FLT_MAX every
    selection key would tie at infinity and every score would be NaN. The
    bound is evaluated in logs so the check itself cannot overflow.
    """
    if arr.size == 0:
        return
    max_abs = float(np.max(np.abs(arr)))
    if max_abs == 0.0:
        return
    log_bound = math.log(n_features) + 2.0 * math.log(4.0 * max_abs)
    if log_bound > math.log(float(np.finfo(np.float32).max)):
        raise ValueError(
            f"input magnitude {max_abs:.3g} overflows float32 when squared "
            f"({n_features} features): distances would saturate to infinity and "
            f"every score would be NaN. Rescale the data, or pass normalize=True "
            f"to z-score each feature first."
        )


def _check_finite_scores(scores: np.ndarray) -> None:
    """Backstop (__init__.py:105-112): non-finite scores must raise, not be returned."""
    if not np.isfinite(scores).all():
        raise ValueError(
            "LOF produced non-finite scores; this indicates float32 overflow or "
            "underflow in the distance computation. Rescale the data, or pass "
            "normalize=True."
        )


def lof(X: ArrayLike, k: int = 20, normalize: bool = False) -> NDArray[np.float32]:
    """Local Outlier Factor of every row of ``X`` (__init__.py:83-113).

    Parameters
    ----------
    X : array-like of shape (n_samples, n_features)
        Converted to C-contiguous float32 if it is not already.
    k : int, default=20
        Neighbours per point, excluding the point itself; ``1 <= k <= n_samples - 1``.
    normalize : bool, default=False
        Z-score each feature before computing distances.

    Returns
    -------
    ndarray of shape (n_samples,)
        Around 1.0 for a point as densely surrounded as its neighbours, larger
        for one in a comparatively sparse region.
    """
    scores = _culof.lof(_validate(X, k), k, normalize)
    _check_finite_scores(scores)
    return scores


def lof_batched(problems, k=20, normalize: bool = False) -> list:
    """LOF of many independent problems in one GPU call (an extension: the
    reference computes one problem per call).

    Parameters
    ----------
    problems : sequence of array-likes, each of shape (n_i, n_features)
        The same number of features in every problem.
    k : int or sequence of int, default=20
        Neighbours per point, one value for all problems or one per problem;
        each ``1 <= k_i <= n_i - 1`` and ``k_i <= 48``.
    normalize : bool, default=False
        Z-score each feature of each problem before computing distances.

    Returns
    -------
    list of ndarray
        Each problem's scores, bit-identical to ``lof(problem, k_i)``.
    """
    arrs = list(problems)
    ks = [int(k)] * len(arrs) if np.ndim(k) == 0 else [int(v) for v in k]
    if len(ks) != len(arrs):
        raise ValueError("k must be one value or one value per problem")
    checked = [_validate(X, ki) for X, ki in zip(arrs, ks)]
    out = _culof.lof_batched(checked, ks, normalize)
    for scores in out:
        _check_finite_scores(scores)
    return out


class LOF:
    """Unsupervised outlier detection with Local Outlier Factor, on the GPU.

    The transductive ``fit_predict`` workflow of
    :class:`sklearn.neighbors.LocalOutlierFactor` with the same sign
    conventions, as the reference's ``culof.LOF`` (__init__.py:116-227).
    ``offset_`` for a numeric contamination is computed on the GPU and equals
    ``np.percentile(negative_outlier_factor_, 100 * contamination)``.

    Parameters
    ----------
    n_neighbors : int, default=20
    contamination : {'auto'} or float in (0, 0.5], default='auto'
    normalize : bool, default=False

    Attributes
    ----------
    negative_outlier_factor_ : ndarray of shape (n_samples,)
    offset_ : float
    n_neighbors_ : int
    """

    def __init__(self, n_neighbors: int = 20, contamination: str | float = "auto", normalize: bool = False) -> None:
        if n_neighbors < 1:
            raise ValueError(f"n_neighbors must be >= 1, got {n_neighbors}")
        if contamination != "auto" and not 0.0 < float(contamination) <= 0.5:
            raise ValueError(f"contamination must be 'auto' or in (0, 0.5], got {contamination!r}")
        self.n_neighbors = n_neighbors
        self.contamination = contamination
        self.normalize = normalize

    def fit(self, X: ArrayLike, y: object = None) -> LOF:
        """Compute the LOF of every sample in ``X``. Returns ``self``."""
        del y
        arr = _validate(X, self.n_neighbors)
        c = "auto" if self.contamination == "auto" else float(self.contamination)
        nof, labels, offset = _culof.fit_predict(arr, self.n_neighbors, self.normalize, c)
        _check_finite_scores(nof)
        self.n_neighbors_ = self.n_neighbors
        self.negative_outlier_factor_ = nof
        self.offset_ = -1.5 if self.contamination == "auto" else float(offset)
        self._labels = labels
        return self

    def fit_predict(self, X: ArrayLike, y: object = None) -> NDArray[np.intp]:
        """Fit and return a label per sample: ``-1`` for outliers, ``1`` for inliers."""
        del y
        return self.fit(X).predict()

    def score_samples(self) -> NDArray[np.float32]:
        """Opposite of the LOF for the fitted data; takes no X (__init__.py:193-206)."""
        return self._check_fitted()

    def predict(self) -> NDArray[np.intp]:
        """Label the fitted samples ``-1`` (outlier) or ``1`` (inlier)."""
        return np.where(self.score_samples() < self._check_offset(), -1, 1)

    def _check_fitted(self) -> NDArray[np.float32]:
        if not hasattr(self, "negative_outlier_factor_"):
            raise ValueError("this LOF instance is not fitted yet - call fit() or fit_predict() first")
        return self.negative_outlier_factor_

    def _check_offset(self) -> float:
        self._check_fitted()
        return self.offset_

    def __repr__(self) -> str:
        return (
            f"LOF(n_neighbors={self.n_neighbors}, "
            f"contamination={self.contamination!r}, normalize={self.normalize})"
        )
