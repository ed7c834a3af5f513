"""The tensor-core path.

* the building block (tcgen05.mma with TMEM accumulators): a bf16 Gram tile
  against exact products summed in FP64, within the FP32-accumulation bound
  of K terms;
* the f16-filtered k-NN sweep: bit-exact against the oracle on scale,
  tie and duplicate edge cases, and identical to the FP32 sweep at sizes
  the oracle is too slow for (both paths are exact, so any filter that
  dropped a true neighbour would show as a difference).
"""

from __future__ import annotations

import numpy as np
import pytest

from culof_gb300 import _culof, synthetic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rows_a,rows_b", [(128, 128), (256, 384)])
def test_bf16_gram_tile(rows_a, rows_b):
    import torch

    K = 128
    g = torch.Generator().manual_seed(rows_a + rows_b)
    A = (torch.randn(rows_a, K, generator=g) * 3).to(torch.bfloat16)
    B = (torch.randn(rows_b, K, generator=g) * 3).to(torch.bfloat16)
    dA, dB = A.cuda(), B.cuda()
    dG = torch.full((rows_a, rows_b), float("nan"), dtype=torch.float32, device="cuda")
    with _culof.Context() as ctx:
        ctx.set_stream(0)
        ctx.bf16_gram(dA.data_ptr(), rows_a, dB.data_ptr(), rows_b, K, dG.data_ptr())
        ctx.synchronize()
    got = dG.cpu().numpy().astype(np.float64)
    a = A.float().numpy().astype(np.float64)
    b = B.float().numpy().astype(np.float64)
    want = a @ b.T
    bound = K * 2.0**-23 * (np.abs(a) @ np.abs(b).T) + 1e-30
    assert np.isfinite(got).all()
    assert np.all(np.abs(got - want) <= bound), float(np.max(np.abs(got - want) / bound))


# ---- the tensor-core k-NN path (f16 filter + exact FP32 rescoring) ---------

def _knn(ctx, X, k, path):
    import torch

    n, d = X.shape
    dx = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    idx = torch.full((k, n), -1, dtype=torch.int32, device="cuda")
    d2 = torch.full((k, n), float("nan"), dtype=torch.float32, device="cuda")
    kd = torch.full((n,), float("nan"), dtype=torch.float32, device="cuda")
    ctx.set_path(path)
    ctx.knn_device(dx.data_ptr(), n, d, k, False, idx.data_ptr(), d2.data_ptr(), kd.data_ptr())
    ctx.synchronize()
    assert ctx.last_path() == path
    return idx.cpu().numpy(), d2.cpu().numpy(), kd.cpu().numpy()


def _assert_same(a, b):
    np.testing.assert_array_equal(a[2].view(np.uint32), b[2].view(np.uint32))
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1].view(np.uint32), b[1].view(np.uint32))


def _oracle_knn(X, k):
    import oracle

    Xc, _, _ = oracle.center(X)
    return oracle.knn(Xc, k)


TENSOR_CASES = [
    # the f16 scale: tiny and huge coordinates (2^S within range), one far
    # outlier that sets the scale while the bulk sits near the f16 subnormals
    ("tiny", lambda: (synthetic.clusters_with_outliers(2000, 24, seed=31) * 1e-12).astype(np.float32), 20),
    ("huge", lambda: (synthetic.clusters_with_outliers(2000, 24, seed=32) * 1e15).astype(np.float32), 20),
    ("outlier_scale", lambda: np.vstack([synthetic.clusters_with_outliers(2500, 40, seed=33) * 1e-3,
                                         np.full((1, 40), 5e3, np.float32)]).astype(np.float32), 15),
    # coordinates too small for any f16 scale: the filter is disabled and every pair is rescored
    ("filter_off", lambda: (synthetic.clusters_with_outliers(1500, 16, seed=34) * 1e-24).astype(np.float32), 10),
    # integer grid: many exact distance ties across tiles
    ("grid_ties", lambda: np.random.default_rng(35).integers(-2, 3, (3000, 12)).astype(np.float32), 30),
    ("dups_d32", lambda: np.repeat(np.random.default_rng(36).standard_normal((60, 32)).astype(np.float32), 40,
                                   axis=0)[np.random.default_rng(37).permutation(2400)], 45),
    ("d65_k64", lambda: synthetic.reference_test_data(2000, 65, seed=38, n_outliers=20), 64),
    ("factor_d128_k50_n9000", lambda: synthetic.factor_model(9000, 128, seed=39), 50),
]


@pytest.mark.parametrize("name,make,k", TENSOR_CASES, ids=[c[0] for c in TENSOR_CASES])
def test_tensor_knn_bit_exact_vs_oracle(name, make, k):
    X = make()
    with _culof.Context() as ctx:
        got = _knn(ctx, X, k, _culof.PATH_TENSOR)
    _assert_same(got, _oracle_knn(X, k))


@pytest.mark.parametrize("n,d,k", [(60000, 64, 20), (40000, 128, 50), (30000, 17, 33)])
def test_tensor_equals_fp32_sweep_at_scale(n, d, k):
    # two exact paths with different filters must select identical neighbours
    X = synthetic.factor_model(n, d, seed=n + d)
    with _culof.Context() as ctx:
        t = _knn(ctx, X, k, _culof.PATH_TENSOR)
        f = _knn(ctx, X, k, _culof.PATH_FAST)
    _assert_same(t, f)
