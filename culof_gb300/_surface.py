"""The Python surface of the engine (``LOF`` and ``lof``), written once and
bound to a native binding by the two packages that expose it:
``culof_gb300`` (the ctypes binding ``culof_gb300._culof``) and ``culof``
(the compiled binding ``culof._culof``, the reference's import name).

A binding provides ``lof(points, k, normalize)``,
``fit_predict(points, k, normalize, contamination)``, ``cuda_available()``,
``device_info()`` and ``CudaError``. Names, messages and sign conventions
follow the reference's package (src/culof/__init__.py:31-227).
"""

from __future__ import annotations

import math
from typing import TYPE_CHECKING

import numpy as np

if TYPE_CHECKING:  # pragma: no cover
    from numpy.typing import ArrayLike, NDArray

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


def lof_with(native, X: ArrayLike, k: int = 20, normalize: bool = False) -> NDArray[np.float32]:
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
    scores = native.lof(_validate(X, k), k, normalize)
    _check_finite_scores(scores)
    return scores


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

    _native = None  # the binding; set by the package that exposes the class

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
        nof, labels, offset = self._native.fit_predict(arr, self.n_neighbors, self.normalize, c)
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
