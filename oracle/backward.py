"""FP64 oracle of the sparse LOF backward: TEST INFRASTRUCTURE ONLY.

The reference computes LOF scores but no gradient, so the backward's parity
is pinned here by two independent checks instead of the reference:
  * ``lof_fixed(X, nbr, normalize)``: the LOF scores as a differentiable
    PyTorch FP64 function of the points with the neighbour sets held fixed
    (the forward chain of lof.cu:32-62 of the reference, restated), whose
    autograd gradient the GPU backward must match;
  * central finite differences of the same function, which pin the oracle
    itself.
Conventions shared with the GPU backward: slot k-1 of each point's neighbour
list designates its k-th neighbour; max(kd2_j, d2_ij) passes the gradient to
d2_ij only when d2_ij > kd2_j; a zero reach distance has zero gradient;
normalising divides by the population std, features with std <= 1e-12 keep
scale 1 (the forward centring's rule).
"""

from __future__ import annotations

import numpy as np


def lof_fixed(X, nbr, normalize: bool = False):
    """LOF scores (torch FP64) of points X (n x d torch FP64) with fixed
    neighbour slots nbr (k x n integer array or tensor)."""
    import torch

    n, d = X.shape
    nbr = torch.as_tensor(np.asarray(nbr), dtype=torch.int64, device=X.device) if not torch.is_tensor(nbr) \
        else nbr.to(device=X.device, dtype=torch.int64)
    k = nbr.shape[0]
    mean = X.mean(0)
    Xc = X - mean
    if normalize:
        var = (Xc * Xc).mean(0)
        scaled = torch.sqrt(var.detach()) > 1e-12
        # sqrt only of scaled features' variances (its derivative at 0 is infinite)
        sd = torch.sqrt(torch.where(scaled, var, torch.ones_like(var)))
        Xc = torch.where(scaled, Xc / sd, Xc)
    diff = Xc.unsqueeze(0) - Xc[nbr]                      # k x n x d
    d2 = (diff * diff).sum(-1)                             # k x n
    kd2 = d2[k - 1]                                        # n
    kdj = kd2[nbr]                                         # k x n
    m = torch.where(d2 > kdj, d2, kdj)
    reach = torch.where(m > 0, torch.sqrt(torch.clamp(m, min=1e-300)), torch.zeros_like(m))
    lrd = 1.0 / (reach.sum(0) / k + 1e-10)
    S = lrd[nbr].sum(0)
    return S / (k * lrd)


def grad_fixed(X, nbr, w, normalize: bool = False):
    """Autograd gradient of sum_i w_i score_i (numpy FP64 in and out)."""
    import torch

    Xt = torch.tensor(np.asarray(X, np.float64), requires_grad=True)
    s = lof_fixed(Xt, nbr, normalize)
    (s * torch.as_tensor(np.asarray(w, np.float64))).sum().backward()
    return Xt.grad.numpy(), s.detach().numpy()


def fd_directional(X, nbr, w, v, h: float = 1e-6, normalize: bool = False) -> float:
    """Central difference of sum_i w_i score_i along direction v (FP64)."""
    import torch

    X64 = np.asarray(X, np.float64)
    wt = torch.as_tensor(np.asarray(w, np.float64))

    def L(Y):
        return float((lof_fixed(torch.as_tensor(Y), nbr, normalize) * wt).sum())

    return (L(X64 + h * v) - L(X64 - h * v)) / (2 * h)
