"""culof: the reference's import name for this engine.

``import culof`` gives the same public surface as the reference cuLOF 0.2.0
package (src/culof/__init__.py:31: ``LOF``, ``lof``, ``cuda_available``,
``device_info``, ``__version__``), bound to the compiled binding
``culof._culof`` (the counterpart of the reference's pybind11 module,
src/cuda/binding.cpp:25-56), so code written against the reference runs
unchanged:

    >>> from culof import LOF
    >>> labels = LOF(n_neighbors=20, contamination=0.01).fit_predict(X)

The engine's extensions (batched problems, device-pointer contexts, the
differentiable scores) live in the ``culof_gb300`` package.
"""

from __future__ import annotations

from typing import TYPE_CHECKING

from culof_gb300 import _surface
from culof_gb300._version import __version__

from . import _culof

if TYPE_CHECKING:  # pragma: no cover
    import numpy as np
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
