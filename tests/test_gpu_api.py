"""The Python surface on the GPU: the reference's test_api.py and
test_regressions.py contracts, run against both import names: culof_gb300
(ctypes binding) and culof (the compiled binding culof._culof, the
reference's package name)."""

from __future__ import annotations

import numpy as np
import pytest

import importlib

import oracle
from culof_gb300 import synthetic

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["culof_gb300", "culof"])
def api(request):
    return importlib.import_module(request.param)


@pytest.fixture
def data() -> np.ndarray:
    """1,000 points in 3-D with 25 planted outliers in the first rows (conftest.py:33-36)."""
    return synthetic.reference_test_data(1000, 3, seed=42, n_outliers=25)


def test_device_is_reported(api):
    assert api.cuda_available()
    info = api.device_info()
    assert "sm_" in info and "SMs" in info and "MiB" in info


def test_scores_separate_outliers(api, data):
    scores = api.lof(data, 20)
    assert scores.shape == (len(data),)
    assert scores.dtype == np.float32
    assert scores[:25].min() > np.median(scores[25:]) * 2


def test_fit_predict_returns_labels(api, data):
    labels = api.LOF(n_neighbors=20, contamination=0.025).fit_predict(data)
    assert set(np.unique(labels)) <= {-1, 1}
    assert abs((labels == -1).sum() - 25) <= 3


def test_negative_outlier_factor_is_negated(api, data):
    model = api.LOF(n_neighbors=20).fit(data)
    np.testing.assert_array_equal(-model.negative_outlier_factor_, api.lof(data, 20))


def test_score_samples_without_argument_uses_fit(api, data):
    model = api.LOF(n_neighbors=20).fit(data)
    np.testing.assert_array_equal(model.score_samples(), model.negative_outlier_factor_)


def test_predict_flags_lowest_scores_and_matches_gpu_labels(api, data):
    model = api.LOF(n_neighbors=20, contamination=0.05).fit(data)
    flagged = model.predict() == -1
    assert (model.negative_outlier_factor_[flagged] < model.offset_).all()
    np.testing.assert_array_equal(model.predict(), model._labels)
    assert model.offset_ == float(np.percentile(model.negative_outlier_factor_, 5.0))


def test_auto_offset(api, data):
    assert api.LOF().fit(data).offset_ == -1.5


@pytest.mark.parametrize("bad", [100, 500])
def test_rejects_n_neighbors_above_sample_count(api, bad):
    X = synthetic.reference_test_data(100, 2, seed=1)
    with pytest.raises(ValueError, match="requires at least"):
        api.LOF(n_neighbors=bad).fit(X)


def test_accepts_lists(api):
    X = [[0.0, 0.0], [0.1, 0.1], [0.2, 0.0], [5.0, 5.0], [0.05, 0.2]]
    assert api.lof(X, 2).shape == (5,)


def test_output_is_not_a_constant(api):
    rng = np.random.default_rng(0)
    X = rng.standard_normal((500, 2)).astype(np.float32)
    X[:5] += 8.0
    scores = api.lof(X, 20)
    assert scores.strides == (scores.itemsize,)
    assert scores.std() > 0.0
    assert len(np.unique(scores)) > 400


def test_non_contiguous_and_fortran_input(api):
    rng = np.random.default_rng(1)
    base = rng.standard_normal((2000, 3)).astype(np.float32)
    base[:20] += 8.0
    view = base[::2]
    assert not view.flags["C_CONTIGUOUS"]
    np.testing.assert_array_equal(api.lof(view, 20), api.lof(np.ascontiguousarray(view), 20))
    X = np.asfortranarray(rng.standard_normal((800, 4)).astype(np.float32))
    np.testing.assert_array_equal(api.lof(X, 20), api.lof(np.ascontiguousarray(X), 20))


def test_float64_input_is_converted(api):
    rng = np.random.default_rng(3)
    X64 = rng.standard_normal((600, 3))
    np.testing.assert_array_equal(api.lof(X64, 15), api.lof(X64.astype(np.float32), 15))


def test_far_from_origin_is_numerically_stable(api):
    rng = np.random.default_rng(7)
    X = rng.standard_normal((1500, 3)).astype(np.float32)
    X[:15] = rng.uniform(-15, 15, size=(15, 3)).astype(np.float32)
    shifted = (X + 5000.0).astype(np.float32)
    np.testing.assert_array_equal(api.lof(shifted, 20), oracle.lof(shifted, 20))


def test_overflow_guard_leaves_ordinary_data_alone(api):
    rng = np.random.default_rng(0)
    for scale in (1e-6, 1.0, 1e3, 1e9):
        X = (rng.standard_normal((64, 4)) * scale).astype(np.float32)
        assert np.isfinite(api.lof(X, 5)).all(), scale


def test_float32_overflow_raises_instead_of_returning_nan(api):
    rng = np.random.default_rng(0)
    X = (rng.standard_normal((64, 4)) * 1e20).astype(np.float32)
    with pytest.raises(ValueError, match="overflow"):
        api.lof(X, 5)


def test_rejects_non_finite_input(api):
    X = np.ones((100, 2), dtype=np.float32)
    X[3, 1] = np.nan
    with pytest.raises(ValueError, match="NaN or infinity"):
        api.lof(X, 10)


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


def test_reference_import_name_is_a_drop_in():
    # code written against the reference runs unchanged: `from culof import LOF`
    # through the compiled binding, bit for bit with the oracle
    import sysconfig

    import culof
    from culof import LOF

    assert culof._culof.__file__.endswith(sysconfig.get_config_var("EXT_SUFFIX"))
    X = synthetic.clusters_with_outliers(20_000, 8, seed=1)
    model = LOF(20, 0.01)
    labels = model.fit_predict(X)
    o_labels, o_nof, o_off = oracle.fit_predict(X, 20, 0.01)
    np.testing.assert_array_equal(labels, o_labels)
    np.testing.assert_array_equal(model.negative_outlier_factor_.view(np.uint32), o_nof.view(np.uint32))
    assert model.offset_ == o_off
    scores = culof._culof.lof(X, 20, False)
    assert scores.dtype == np.float32 and scores.strides == (4,)
    np.testing.assert_array_equal(scores, -o_nof)
    nof, lab, off = culof._culof.fit_predict(X[::2], 20, False, 0.05)
    o_lab2, o_nof2, o_off2 = oracle.fit_predict(np.ascontiguousarray(X[::2]), 20, 0.05)
    np.testing.assert_array_equal(nof, o_nof2)
    np.testing.assert_array_equal(lab, o_lab2)
    assert off == o_off2
