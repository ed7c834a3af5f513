"""The allocation-free offset entry point, culof_contamination_offset_noalloc.

It serves callers that cannot allocate device memory while they run (for
example an operator inside a framework that owns all device memory through its
own pool): they pass device buffers for the input and the output, and the
select's scratch is a fixed array inside the library. This file is collected
last so that a run stopping at the first failure has run every other test.
Each check calls the new entry point twice in a row on different inputs, so a
second call that saw the first call's leftovers in the shared array would fail.
"""

from __future__ import annotations

import numpy as np
import pytest

from culof_gb300 import _culof, synthetic

pytestmark = pytest.mark.gpu


def _offsets(nof_np: np.ndarray, contamination):
    import torch

    n = nof_np.shape[0]
    nof = torch.from_numpy(np.ascontiguousarray(nof_np, np.float32)).cuda()
    existing = torch.zeros(1, dtype=torch.float64, device="cuda")
    with _culof.Context() as ctx:
        ctx.offset_device(nof.data_ptr(), n, contamination, existing.data_ptr())
        ctx.synchronize()
    noalloc = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    _culof.contamination_offset_noalloc(0, nof.data_ptr(), n, contamination, noalloc.data_ptr())
    torch.cuda.synchronize()
    return float(existing.item()), float(noalloc.item())


def test_noalloc_offset_equals_existing_entry_point_on_two_calls_in_a_row(ref_layer_golden):
    cases = [c for c in ref_layer_golden.meta["cases"] if c["n"] >= 1000 and c["contamination"] in (0.01, 0.25)]
    assert len(cases) >= 2
    for case in cases[:4]:
        nof = -ref_layer_golden[f"{case['scores']}/scores"]
        want, got = _offsets(nof, case["contamination"])
        # offsets are compared exactly throughout the tests (they equal np.percentile)
        assert got == want == case["offset"], case


def test_noalloc_offset_on_engine_scores():
    X = synthetic.clusters_with_outliers(20_000, 8, seed=41)
    with _culof.Context() as ctx:
        nof, _, off = ctx.fit_predict(X, 20, False, 0.01)
    for c in (0.01, 0.1):
        want, got = _offsets(nof, c)
        assert got == want
        assert got == float(np.percentile(nof, 100.0 * c))
    assert _offsets(nof, 0.01)[1] == off
    assert _offsets(nof, "auto") == (-1.5, -1.5)


def test_noalloc_rejects_sizes_beyond_its_maximum():
    import torch

    buf = torch.zeros(4, dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError, match="at most 2147483647"):
        _culof.contamination_offset_noalloc(0, buf.data_ptr(), 2**31, 0.01, buf.data_ptr())
    with pytest.raises(ValueError, match="contamination"):
        _culof.contamination_offset_noalloc(0, buf.data_ptr(), 4, 0.9, buf.data_ptr())
