"""The Python surface on the GPU: the reference's test_api.py and
test_regressions.py contracts, run against culof_gb300."""

from __future__ import annotations

import numpy as np
import pytest

import culof_gb300
import oracle
from culof_gb300 import LOF, lof, synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture
def data() -> np.ndarray:
    """1,000 points in 3-D with 25 planted outliers in the first rows (conftest.py:33-36)."""
    return synthetic.reference_test_data(1000, 3, seed=42, n_outliers=25)


def test_device_is_reported():
    assert culof_gb300.cuda_available()
    info = culof_gb300.device_info()
    assert "sm_" in info and "SMs" in info and "MiB" in info


def test_scores_separate_outliers(data):
    scores = lof(data, 20)
    assert scores.shape == (len(data),)
    assert scores.dtype == np.float32
    assert scores[:25].min() > np.median(scores[25:]) * 2


def test_fit_predict_returns_labels(data):
    labels = LOF(n_neighbors=20, contamination=0.025).fit_predict(data)
    assert set(np.unique(labels)) <= {-1, 1}
    assert abs((labels == -1).sum() - 25) <= 3


def test_negative_outlier_factor_is_negated(data):
    model = LOF(n_neighbors=20).fit(data)
    np.testing.assert_array_equal(-model.negative_outlier_factor_, lof(data, 20))


def test_score_samples_without_argument_uses_fit(data):
    model = LOF(n_neighbors=20).fit(data)
    np.testing.assert_array_equal(model.score_samples(), model.negative_outlier_factor_)


def test_predict_flags_lowest_scores_and_matches_gpu_labels(data):
    model = LOF(n_neighbors=20, contamination=0.05).fit(data)
    flagged = model.predict() == -1
    assert (model.negative_outlier_factor_[flagged] < model.offset_).all()
    np.testing.assert_array_equal(model.predict(), model._labels)
    assert model.offset_ == float(np.percentile(model.negative_outlier_factor_, 5.0))


def test_auto_offset(data):
    assert LOF().fit(data).offset_ == -1.5


@pytest.mark.parametrize("bad", [100, 500])
def test_rejects_n_neighbors_above_sample_count(bad):
    X = synthetic.reference_test_data(100, 2, seed=1)
    with pytest.raises(ValueError, match="requires at least"):
        LOF(n_neighbors=bad).fit(X)


def test_accepts_lists():
    X = [[0.0, 0.0], [0.1, 0.1], [0.2, 0.0], [5.0, 5.0], [0.05, 0.2]]
    assert lof(X, 2).shape == (5,)


def test_output_is_not_a_constant():
    rng = np.random.default_rng(0)
    X = rng.standard_normal((500, 2)).astype(np.float32)
    X[:5] += 8.0
    scores = lof(X, 20)
    assert scores.strides == (scores.itemsize,)
    assert scores.std() > 0.0
    assert len(np.unique(scores)) > 400


def test_non_contiguous_and_fortran_input():
    rng = np.random.default_rng(1)
    base = rng.standard_normal((2000, 3)).astype(np.float32)
    base[:20] += 8.0
    view = base[::2]
    assert not view.flags["C_CONTIGUOUS"]
    np.testing.assert_array_equal(lof(view, 20), lof(np.ascontiguousarray(view), 20))
    X = np.asfortranarray(rng.standard_normal((800, 4)).astype(np.float32))
    np.testing.assert_array_equal(lof(X, 20), lof(np.ascontiguousarray(X), 20))


def test_float64_input_is_converted():
    rng = np.random.default_rng(3)
    X64 = rng.standard_normal((600, 3))
    np.testing.assert_array_equal(lof(X64, 15), lof(X64.astype(np.float32), 15))


def test_far_from_origin_is_numerically_stable():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((1500, 3)).astype(np.float32)
    X[:15] = rng.uniform(-15, 15, size=(15, 3)).astype(np.float32)
    shifted = (X + 5000.0).astype(np.float32)
    np.testing.assert_array_equal(lof(shifted, 20), oracle.lof(shifted, 20))


def test_overflow_guard_leaves_ordinary_data_alone():
    rng = np.random.default_rng(0)
    for scale in (1e-6, 1.0, 1e3, 1e9):
        X = (rng.standard_normal((64, 4)) * scale).astype(np.float32)
        assert np.isfinite(lof(X, 5)).all(), scale


def test_float32_overflow_raises_instead_of_returning_nan():
    rng = np.random.default_rng(0)
    X = (rng.standard_normal((64, 4)) * 1e20).astype(np.float32)
    with pytest.raises(ValueError, match="overflow"):
        lof(X, 5)


def test_rejects_non_finite_input():
    X = np.ones((100, 2), dtype=np.float32)
    X[3, 1] = np.nan
    with pytest.raises(ValueError, match="NaN or infinity"):
        lof(X, 10)


def test_expired_bounded_wait_reports_an_error_and_the_context_stays_usable():
    # every wait in the kernels is bounded: when one runs out the kernel sets
    # a status word and returns, and the call fails instead of hanging
    from culof_gb300 import _culof

    X = synthetic.clusters_with_outliers(2000, 8, seed=40)
    with _culof.Context() as ctx:
        with pytest.raises(_culof.CudaError, match="bounded wait"):
            ctx.probe_bounded_wait(1 << 12)
        got = ctx.lof(X, 20)
        with pytest.raises(ValueError):
            ctx.probe_bounded_wait(0)
    np.testing.assert_array_equal(got.view(np.uint32), oracle.lof(X, 20).view(np.uint32))
