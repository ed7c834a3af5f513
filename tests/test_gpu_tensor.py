"""The tensor-core building block (tcgen05.mma with TMEM accumulators): a bf16
Gram tile against exact products summed in FP64, within the FP32-accumulation
bound of K terms."""

from __future__ import annotations

import numpy as np
import pytest

from culof_gb300 import _culof

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
