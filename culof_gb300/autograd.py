"""Differentiable LOF scores for PyTorch.

``lof_scores(X, k, normalize)`` returns the positive LOF scores of the
points X (a CUDA float32 tensor, n x d) exactly as ``lof`` computes them
(exact k-NN on the GPU, the reference's lrd and score), and is differentiable
with respect to X: the backward holds the neighbour sets fixed and runs the
sparse FP64 kernel of the C ABI (culof_context_lof_backward_device), which
gathers over each point's k neighbours and, through a transposed neighbour
list, over the points that name it as a neighbour. The reference has no
backward; the gradient is checked against an FP64 autograd restatement and
finite differences.
"""

from __future__ import annotations

import threading

import torch

from . import _culof

_contexts: dict[int, _culof.Context] = {}
_lock = threading.Lock()


def _context(device: torch.device) -> _culof.Context:
    idx = device.index if device.index is not None else torch.cuda.current_device()
    with _lock:
        c = _contexts.get(idx)
        if c is None:
            with torch.cuda.device(idx):
                c = _culof.Context()
            _contexts[idx] = c
        return c


class LOFScores(torch.autograd.Function):
    """scores = LOF(X); dL/dX by the sparse backward with fixed neighbours."""

    @staticmethod
    def forward(ctx, X: torch.Tensor, k: int, normalize: bool):
        if not X.is_cuda or X.dtype != torch.float32 or X.dim() != 2:
            raise ValueError("lof_scores expects a 2-D float32 CUDA tensor")
        X = X.contiguous()
        n, d = X.shape
        c = _context(X.device)
        stream = torch.cuda.current_stream(X.device).cuda_stream
        c.set_stream(stream)
        idx = torch.empty((k, n), dtype=torch.int32, device=X.device)
        d2 = torch.empty((k, n), dtype=torch.float32, device=X.device)
        kd = torch.empty(n, dtype=torch.float32, device=X.device)
        c.knn_device(X.data_ptr(), n, d, k, normalize, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
        lrd = torch.empty(n, dtype=torch.float32, device=X.device)
        scores = torch.empty(n, dtype=torch.float32, device=X.device)
        _culof.compute_lrd(stream, idx.data_ptr(), d2.data_ptr(), kd.data_ptr(), n, k, lrd.data_ptr())
        _culof.compute_scores(stream, idx.data_ptr(), lrd.data_ptr(), n, k, scores.data_ptr())
        ctx.save_for_backward(X, idx)
        ctx.k, ctx.normalize = k, bool(normalize)
        return scores

    @staticmethod
    def backward(ctx, grad_scores: torch.Tensor):
        X, idx = ctx.saved_tensors
        n, d = X.shape
        c = _context(X.device)
        c.set_stream(torch.cuda.current_stream(X.device).cuda_stream)
        g = grad_scores.detach().to(torch.float64).contiguous()
        gx = torch.empty((n, d), dtype=torch.float64, device=X.device)
        c.lof_backward_device(X.data_ptr(), n, d, ctx.k, ctx.normalize, idx.data_ptr(), g.data_ptr(), gx.data_ptr())
        return gx.to(X.dtype), None, None


def lof_scores(X: torch.Tensor, k: int = 20, normalize: bool = False) -> torch.Tensor:
    """Positive LOF scores of X (CUDA float32, n x d), differentiable in X."""
    if not 1 <= int(k) < X.shape[0]:
        raise ValueError(f"k must satisfy 1 <= k <= n_points - 1 (got k={k}, n_points={X.shape[0]})")
    return LOFScores.apply(X, int(k), bool(normalize))
