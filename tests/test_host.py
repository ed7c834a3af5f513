"""Host-side logic and the C-ABI boundary, no GPU needed.

Mirrors the reference's CPU-checkable contract: argument validation and its
messages (src/culof/__init__.py:37-80, 159-171; pipeline.cu:133-141),
choose_tile_rows (test_culof.cu:207-212), repr/version/__all__ (test_api.py,
test_regressions.py), and that the library loads and exports every entry
point include/*.h declares.
"""

from __future__ import annotations

import os
import re
import subprocess

import numpy as np
import pytest
from conftest import ROOT

import culof_gb300
from culof_gb300 import LOF, _culof, lof


def declared_c_symbols() -> list[str]:
    text = open(os.path.join(ROOT, "include", "culof_c.h")).read()
    return re.findall(r"CULOF_API\s+[\w\s\*]*?\b(culof_\w+)\s*\(", text)


def test_library_exports_every_declared_c_symbol():
    names = declared_c_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(_culof._lib, name), name
    assert set(names) == set(_culof.EXPORTED)


def test_library_exports_cxx_api():
    out = subprocess.run(["nm", "-D", "-C", "--defined-only", _culof.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        pytest.skip("nm unavailable")
    for sig in ("culof::lof(float const*, int, int, int, bool)", "culof::cuda_available()", "culof::device_info"):
        assert sig in out.stdout, sig


def test_choose_tile_rows_respects_budget():
    # test_culof.cu:207-212: 1000 points is 4000 bytes per row
    assert _culof.choose_tile_rows(1000, 40000) == 10
    assert _culof.choose_tile_rows(1000, 0) == 1
    assert _culof.choose_tile_rows(1000, 1 << 40) == 1000


@pytest.mark.parametrize("pkg", ["culof_gb300", "culof"])
def test_version_and_surface(pkg, ref_layer_golden):
    import importlib

    mod = importlib.import_module(pkg)
    meta = ref_layer_golden.meta
    assert mod.__version__ == meta["version"] == _culof.version()
    assert sorted(mod.__all__) == sorted(meta["all"])
    assert repr(mod.LOF(n_neighbors=7)) == meta["repr"]
    for name in mod.__all__:
        assert hasattr(mod, name), name


def test_compiled_binding_module():
    # culof._culof: the compiled counterpart of the reference's pybind11
    # module (binding.cpp:47-56), over the C ABI
    import sysconfig

    import culof
    from culof import _culof as native

    assert native.__file__.endswith(sysconfig.get_config_var("EXT_SUFFIX"))
    for name in ("lof", "fit_predict", "cuda_available", "device_info", "CudaError"):
        assert hasattr(native, name), name
    assert issubclass(native.CudaError, RuntimeError) and culof.CudaError is native.CudaError
    assert isinstance(native.cuda_available(), bool)
    with pytest.raises(ValueError, match="2-D array"):
        native.lof(np.zeros(10, np.float32), 3, False)
    with pytest.raises(ValueError, match="2-D array"):
        native.lof(np.zeros((2, 3, 4), np.float32), 3, False)
    with pytest.raises(ValueError, match="contamination"):
        native.fit_predict(np.zeros((10, 2), np.float32), 3, False, -0.5)
    with pytest.raises(TypeError):
        native.lof(np.zeros((10, 2), np.float32), "three", False)


@pytest.mark.parametrize(
    "label,call",
    [
        ("k0", lambda m: m.LOF(n_neighbors=0)),
        ("contam_bad", lambda m: m.LOF(contamination=0.9)),
        ("k_too_big", lambda m: m.LOF(n_neighbors=100).fit(np.zeros((100, 2), np.float32))),
        ("not_2d", lambda m: m.lof(np.zeros(10, np.float32), 3)),
        ("nan", lambda m: m.lof(np.array([[0.0, np.nan], [1.0, 1.0], [2.0, 2.0]], np.float32), 1)),
        ("overflow", lambda m: m.lof((np.ones((64, 4)) * 1e20).astype(np.float32), 5)),
        ("no_features", lambda m: m.lof(np.zeros((5, 0), np.float32), 1)),
        ("unfitted", lambda m: m.LOF().predict()),
    ],
)
@pytest.mark.parametrize("pkg", ["culof_gb300", "culof"])
def test_validation_messages_match_reference(pkg, label, call, ref_layer_golden):
    import importlib

    kind, msg = ref_layer_golden.meta["errors"][label]
    with pytest.raises(ValueError) as ei:
        call(importlib.import_module(pkg))
    assert type(ei.value).__name__ == kind
    assert str(ei.value) == msg


@pytest.mark.parametrize("bad", [0.0, 0.9, 1.0, -0.1])
def test_rejects_bad_contamination(bad):
    with pytest.raises(ValueError, match="contamination"):
        LOF(contamination=bad)


def test_predict_and_score_samples_take_no_x():
    m = LOF()
    with pytest.raises(TypeError):
        m.predict(np.zeros((3, 2)))
    with pytest.raises(TypeError):
        m.score_samples(np.zeros((3, 2)))


def test_c_abi_argument_errors_before_device_check():
    """Invalid arguments are reported as ValueError (std::invalid_argument in
    the reference, checked before cuda_available, pipeline.cu:133-142)."""
    X = np.zeros((50, 2), np.float32)
    with pytest.raises(ValueError, match="k must satisfy"):
        _culof.lof(X, 50, False)
    with pytest.raises(ValueError, match="k must satisfy"):
        _culof.lof(X, 0, False)
    with pytest.raises(ValueError, match="n_points must be >= 2"):
        _culof.lof(X[:1], 1, False)
    with pytest.raises(ValueError, match="2-D"):
        _culof.lof(X.ravel(), 1, False)


def test_no_device_raises_cuda_error(gpu_available):
    if gpu_available:
        pytest.skip("a device is present")
    assert culof_gb300.cuda_available() is False
    assert culof_gb300.device_info() == "no CUDA device"
    with pytest.raises(culof_gb300.CudaError, match="no CUDA device available"):
        _culof.lof(np.random.default_rng(0).standard_normal((50, 2)).astype(np.float32), 5, False)
    assert issubclass(culof_gb300.CudaError, RuntimeError)
    with pytest.raises(culof_gb300.CudaError):
        _culof.Context()


CXX_CALLER = r"""
#include <culof.h>
#include <cstdio>
#include <stdexcept>
#include <vector>
int main() {
    std::vector<float> x(200 * 4);
    for (size_t i = 0; i < x.size(); ++i) x[i] = static_cast<float>((i * 37) % 101) * 0.01f;
    try {
        culof::lof(nullptr, 200, 4, 20);
    } catch (const std::invalid_argument& e) {
        std::printf("invalid_argument: %s\n", e.what());
    }
    try {
        std::printf("scores: %zu\n", culof::lof(x.data(), 200, 4, 20).size());
    } catch (const culof::CudaError& e) {
        std::printf("CudaError: %s\n", e.what());
    }
    return 0;
}
"""


def test_cxx_caller_relinks_unchanged(tmp_path, gpu_available):
    # a program written against the reference's culof.h builds and links
    # against this library, with the reference's exceptions and messages
    src = tmp_path / "app.cpp"
    src.write_text(CXX_CALLER)
    exe = tmp_path / "app"
    libdir = os.path.dirname(_culof.LIB_PATH)
    try:
        build = subprocess.run(["g++", str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir, "-lculof_gb300",
                                f"-Wl,-rpath,{libdir}", "-o", str(exe)], capture_output=True, text=True)
    except FileNotFoundError:
        pytest.skip("g++ unavailable")
    assert build.returncode == 0, build.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120).stdout
    assert "invalid_argument: points must not be null" in out
    assert ("scores: 200" if gpu_available else "CudaError: no CUDA device available") in out
