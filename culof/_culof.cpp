// culof._culof: the compiled Python binding of the exact-LOF engine, written
// against the CPython C API over the library's C ABI (include/culof_c.h).
//
// It is the counterpart of the reference's pybind11 module _culof
// (src/cuda/binding.cpp:25-56), with the same functions and behaviour:
//   lof(points, k, normalize) -> float32 array of n positive LOF scores.
//       `points` is coerced to a C-contiguous float32 array whatever the
//       caller passes (numpy.ascontiguousarray with dtype float32: a strided
//       view such as X[::2] is materialised, never read through its
//       strides); a result that is not 2-D raises ValueError; the GIL is
//       released while the GPU works; the result is a fresh array.
//   cuda_available() -> bool, device_info() -> str.
//   CudaError, a RuntimeError subclass, for CUDA failures.
// Invalid arguments raise ValueError (the reference's std::invalid_argument).
// One extension beyond the reference: fit_predict(points, k, normalize,
// contamination) -> (negative_outlier_factor_, labels, offset_), which
// computes offset_ (np.percentile of the scores) on the GPU.
//
// numpy is used through its Python API only (no numpy headers), so the
// module builds against any numpy the interpreter has.
#define PY_SSIZE_T_CLEAN
#include <Python.h>

#include <stdint.h>
#include <string.h>

#include "culof_c.h"

namespace {

PyObject* g_numpy = nullptr;
PyObject* g_float32 = nullptr;
PyObject* g_int64 = nullptr;
PyObject* g_cuda_error = nullptr;

// Raises the Python exception of a failed C ABI call; returns nullptr.
PyObject* raise_status(int rc) {
    const char* msg = culof_last_error();
    if (rc == CULOF_ERR_INVALID_ARGUMENT) {
        PyErr_SetString(PyExc_ValueError, msg && *msg ? msg : "invalid argument");
    } else {
        PyErr_Format(g_cuda_error, "%s", msg && *msg ? msg : "CUDA error");
    }
    return nullptr;
}

// numpy.<fn>(arg, dtype=<dtype>)
PyObject* numpy_call(const char* fn, PyObject* arg, PyObject* dtype) {
    PyObject* f = PyObject_GetAttrString(g_numpy, fn);
    if (!f) return nullptr;
    PyObject* args = PyTuple_Pack(1, arg);
    PyObject* kw = Py_BuildValue("{s:O}", "dtype", dtype);
    PyObject* out = (args && kw) ? PyObject_Call(f, args, kw) : nullptr;
    Py_XDECREF(kw);
    Py_XDECREF(args);
    Py_DECREF(f);
    return out;
}

// A C-contiguous float32 view of `points` (n x d). On success the caller owns
// `arr` and must release `view`.
bool as_points(PyObject* points, PyObject** arr, Py_buffer* view) {
    *arr = numpy_call("ascontiguousarray", points, g_float32);
    if (!*arr) return false;
    if (PyObject_GetBuffer(*arr, view, PyBUF_C_CONTIGUOUS | PyBUF_FORMAT) != 0) {
        Py_CLEAR(*arr);
        return false;
    }
    if (view->ndim != 2) {
        PyBuffer_Release(view);
        Py_CLEAR(*arr);
        PyErr_SetString(PyExc_ValueError, "expected a 2-D array of shape (n_samples, n_features)");
        return false;
    }
    return true;
}

// A fresh 1-D numpy array of n elements and a writable view of it.
PyObject* new_vector(Py_ssize_t n, PyObject* dtype, Py_buffer* view) {
    PyObject* size = PyLong_FromSsize_t(n);
    if (!size) return nullptr;
    PyObject* out = numpy_call("empty", size, dtype);
    Py_DECREF(size);
    if (!out) return nullptr;
    if (PyObject_GetBuffer(out, view, PyBUF_C_CONTIGUOUS | PyBUF_WRITABLE) != 0) {
        Py_DECREF(out);
        return nullptr;
    }
    return out;
}

PyObject* py_lof(PyObject*, PyObject* args, PyObject* kwargs) {
    static const char* names[] = {"points", "k", "normalize", nullptr};
    PyObject* points = nullptr;
    int k = 0, normalize = 0;
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "Oip", const_cast<char**>(names), &points, &k, &normalize))
        return nullptr;
    PyObject* arr = nullptr;
    Py_buffer in;
    if (!as_points(points, &arr, &in)) return nullptr;
    const int64_t n = in.shape[0];
    const int d = static_cast<int>(in.shape[1]);
    Py_buffer ov;
    PyObject* out = new_vector(static_cast<Py_ssize_t>(n), g_float32, &ov);
    if (!out) {
        PyBuffer_Release(&in);
        Py_DECREF(arr);
        return nullptr;
    }
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = culof_lof(static_cast<const float*>(in.buf), n, d, k, normalize, static_cast<float*>(ov.buf));
    Py_END_ALLOW_THREADS
    PyBuffer_Release(&ov);
    PyBuffer_Release(&in);
    Py_DECREF(arr);
    if (rc != CULOF_OK) {
        Py_DECREF(out);
        return raise_status(rc);
    }
    return out;
}

PyObject* py_fit_predict(PyObject*, PyObject* args, PyObject* kwargs) {
    static const char* names[] = {"points", "k", "normalize", "contamination", nullptr};
    PyObject* points = nullptr;
    PyObject* contam = nullptr;
    int k = 0, normalize = 0;
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "OipO", const_cast<char**>(names), &points, &k, &normalize,
                                     &contam))
        return nullptr;
    double c = -1.0;  // 'auto' (offset_ = -1.5)
    if (!(PyUnicode_Check(contam) && PyUnicode_CompareWithASCIIString(contam, "auto") == 0)) {
        c = PyFloat_AsDouble(contam);
        if (c == -1.0 && PyErr_Occurred()) return nullptr;
        if (!(c > 0.0)) {
            PyErr_Format(PyExc_ValueError, "contamination must be 'auto' or in (0, 0.5], got %R", contam);
            return nullptr;
        }
    }
    PyObject* arr = nullptr;
    Py_buffer in;
    if (!as_points(points, &arr, &in)) return nullptr;
    const int64_t n = in.shape[0];
    const int d = static_cast<int>(in.shape[1]);
    Py_buffer nv, lv;
    PyObject* nof = new_vector(static_cast<Py_ssize_t>(n), g_float32, &nv);
    PyObject* labels = nof ? new_vector(static_cast<Py_ssize_t>(n), g_int64, &lv) : nullptr;
    if (!labels) {
        if (nof) {
            PyBuffer_Release(&nv);
            Py_DECREF(nof);
        }
        PyBuffer_Release(&in);
        Py_DECREF(arr);
        return nullptr;
    }
    double offset = 0.0;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = culof_fit_predict(static_cast<const float*>(in.buf), n, d, k, normalize, c, static_cast<float*>(nv.buf),
                           static_cast<int64_t*>(lv.buf), &offset);
    Py_END_ALLOW_THREADS
    PyBuffer_Release(&lv);
    PyBuffer_Release(&nv);
    PyBuffer_Release(&in);
    Py_DECREF(arr);
    if (rc != CULOF_OK) {
        Py_DECREF(nof);
        Py_DECREF(labels);
        return raise_status(rc);
    }
    return Py_BuildValue("(NNd)", nof, labels, offset);
}

PyObject* py_cuda_available(PyObject*, PyObject*) { return PyBool_FromLong(culof_cuda_available()); }

PyObject* py_device_info(PyObject*, PyObject*) {
    char buf[512];
    const int rc = culof_device_info(buf, sizeof buf);
    if (rc != CULOF_OK) return raise_status(rc);
    return PyUnicode_DecodeUTF8(buf, static_cast<Py_ssize_t>(strlen(buf)), "replace");
}

PyMethodDef methods[] = {
    {"lof", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(py_lof)), METH_VARARGS | METH_KEYWORDS,
     "lof(points, k, normalize) -> float32 array: raw LOF scores for a (n_samples, n_features) array."},
    {"fit_predict", reinterpret_cast<PyCFunction>(reinterpret_cast<void (*)(void)>(py_fit_predict)),
     METH_VARARGS | METH_KEYWORDS,
     "fit_predict(points, k, normalize, contamination) -> (negative_outlier_factor_, labels, offset_)."},
    {"cuda_available", py_cuda_available, METH_NOARGS, "True if a CUDA device is usable."},
    {"device_info", py_device_info, METH_NOARGS, "'<name> (sm_XY, <SMs> SMs, <MiB> MiB)'."},
    {nullptr, nullptr, 0, nullptr},
};

PyModuleDef module = {PyModuleDef_HEAD_INIT, "_culof", "Exact LOF engine for GB300 (compiled binding).", -1,
                      methods};

}  // namespace

PyMODINIT_FUNC PyInit__culof(void) {
    PyObject* m = PyModule_Create(&module);
    if (!m) return nullptr;
    g_numpy = PyImport_ImportModule("numpy");
    if (!g_numpy) goto fail;
    g_float32 = PyObject_GetAttrString(g_numpy, "float32");
    g_int64 = PyObject_GetAttrString(g_numpy, "int64");
    if (!g_float32 || !g_int64) goto fail;
    g_cuda_error = PyErr_NewExceptionWithDoc("_culof.CudaError", "A CUDA failure inside the engine.",
                                             PyExc_RuntimeError, nullptr);
    if (!g_cuda_error) goto fail;
    Py_INCREF(g_cuda_error);
    if (PyModule_AddObject(m, "CudaError", g_cuda_error) != 0) {
        Py_DECREF(g_cuda_error);
        goto fail;
    }
    return m;
fail:
    Py_DECREF(m);
    return nullptr;
}
