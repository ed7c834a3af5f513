"""GPU sparse LOF backward (culof_context_lof_backward_device and the
torch.autograd wrapper) against the FP64 autograd oracle with the same fixed
neighbour sets. The reference has no backward; its forward chain is what the
oracle restates (oracle/backward.py)."""

from __future__ import annotations

import numpy as np
import pytest

from oracle import backward as ob
from culof_gb300 import _culof, synthetic

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _gpu_grad(ctx, X, k, normalize, w):
    n, d = X.shape
    dx = torch.from_numpy(np.ascontiguousarray(X, np.float32)).cuda()
    idx = torch.empty((k, n), dtype=torch.int32, device="cuda")
    d2 = torch.empty((k, n), dtype=torch.float32, device="cuda")
    kd = torch.empty(n, dtype=torch.float32, device="cuda")
    ctx.knn_device(dx.data_ptr(), n, d, k, normalize, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
    g = torch.from_numpy(np.asarray(w, np.float64)).cuda()
    gx = torch.full((n, d), float("nan"), dtype=torch.float64, device="cuda")
    sc = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    ctx.lof_backward_device(dx.data_ptr(), n, d, k, normalize, idx.data_ptr(), g.data_ptr(), gx.data_ptr(),
                            sc.data_ptr())
    ctx.synchronize()
    return idx.cpu().numpy(), gx.cpu().numpy(), sc.cpu().numpy()


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


CASES = [
    ("d8_k20", lambda: synthetic.clusters_with_outliers(3000, 8, seed=51), 20, False),
    ("d8_k20_norm", lambda: synthetic.clusters_with_outliers(3000, 8, seed=52) * np.array(
        [1, 50, 1, 1, 0.01, 1, 1, 3], np.float32), 20, True),
    ("d32_k20", lambda: synthetic.clusters_with_outliers(2500, 32, seed=53), 20, False),
    ("d3_k1", lambda: synthetic.clusters_with_outliers(800, 3, seed=54), 1, False),
    ("constant_feature_norm", lambda: np.hstack([synthetic.clusters_with_outliers(1200, 4, seed=55),
                                                 np.full((1200, 1), 7.0, np.float32)]), 15, True),
    ("dups", lambda: np.repeat(np.random.default_rng(56).standard_normal((100, 4)).astype(np.float32), 8,
                               axis=0), 10, False),
    ("d128_k50", lambda: synthetic.factor_model(3000, 128, seed=57), 50, False),
    # more features than one block of the column reduction (128)
    ("d200_k10_norm", lambda: synthetic.reference_test_data(1500, 200, seed=61, n_outliers=15), 10, True),
]


@pytest.mark.parametrize("name,make,k,normalize", CASES, ids=[c[0] for c in CASES])
def test_backward_matches_fp64_autograd(name, make, k, normalize):
    X = make()
    w = np.random.default_rng(7).standard_normal(len(X))
    with _culof.Context() as ctx:
        idx, gx, sc = _gpu_grad(ctx, X, k, normalize, w)
    g_ref, s_ref = ob.grad_fixed(X, idx, w, normalize)
    assert np.isfinite(gx).all()
    assert _rel(sc, s_ref) < 1e-12
    assert _rel(gx, g_ref) < 1e-10


def test_backward_is_deterministic():
    X = synthetic.clusters_with_outliers(20000, 16, seed=58)
    w = np.random.default_rng(8).standard_normal(len(X))
    with _culof.Context() as ctx:
        a = _gpu_grad(ctx, X, 20, False, w)[1]
        b = _gpu_grad(ctx, X, 20, False, w)[1]
    np.testing.assert_array_equal(a.view(np.uint64), b.view(np.uint64))


def test_autograd_function_end_to_end():
    from culof_gb300.autograd import lof_scores

    X = synthetic.clusters_with_outliers(4000, 32, seed=59)
    w = np.random.default_rng(9).standard_normal(len(X))
    Xt = torch.from_numpy(X).cuda().requires_grad_(True)
    s = lof_scores(Xt, 20)
    (s.double() * torch.from_numpy(w).cuda()).sum().backward()
    torch.cuda.synchronize()
    with _culof.Context() as ctx:
        np.testing.assert_array_equal(s.detach().cpu().numpy(), ctx.lof(X, 20))
        idx = _gpu_grad(ctx, X, 20, False, w)[0]
    g_ref, _ = ob.grad_fixed(X, idx, w, False)
    got = Xt.grad.cpu().numpy().astype(np.float64)
    # float32 result of an FP64 gradient
    assert _rel(got, g_ref) < 1e-6


def test_backward_mixture_n50000_d32():
    # the gradient workload (8-cluster mixture, n = 50,000, d = 32, k = 20):
    # the sparse backward against FP64 autograd evaluated by torch on the GPU
    # with the same neighbour slots
    X = synthetic.gradient_mixture(50000, 32, seed=60)
    w = np.random.default_rng(10).standard_normal(len(X))
    with _culof.Context() as ctx:
        idx, gx, _ = _gpu_grad(ctx, X, 20, False, w)
    Xt = torch.from_numpy(X.astype(np.float64)).cuda().requires_grad_(True)
    s = ob.lof_fixed(Xt, torch.from_numpy(idx.astype(np.int64)).cuda(), False)
    (s * torch.from_numpy(w).cuda()).sum().backward()
    assert _rel(gx, Xt.grad.cpu().numpy()) < 1e-10
