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

from typing import TYPE_CHECKING

import numpy as np

from . import _culof, _surface
from ._surface import _check_finite_scores, _check_representable, _validate  # noqa: F401
from ._version import __version__

if TYPE_CHECKING:  # pragma: no cover
    from numpy.typing import ArrayLike, NDArray

__all__ = ["LOF", "__version__", "cuda_available", "device_info", "lof"]

cuda_available = _culof.cuda_available
device_info = _culof.device_info
CudaError = _culof.CudaError


def lof(X: ArrayLike, k: int = 20, normalize: bool = False) -> NDArray[np.float32]:
    return _surface.lof_with(_culof, X, k, normalize)


lof.__doc__ = _surface.lof_with.__doc__


class LOF(_surface.LOF):
    __doc__ = _surface.LOF.__doc__
    _native = _culof


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
