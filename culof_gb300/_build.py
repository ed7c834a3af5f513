"""Build libculof_gb300.so in-tree with nvcc for sm_103a (no cmake), and the
compiled Python binding ``culof._culof`` over its C ABI with g++.

Translation units compile in parallel into ``culof_gb300/_build/`` and link
into ``culof_gb300/libculof_gb300.so``; ``culof/_culof.cpp`` compiles into
``culof/_culof<EXT_SUFFIX>``, which finds the library through its run path.
A stamp of the sources and flags avoids rebuilding up-to-date files.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libculof_gb300.so")
PYEXT_SRC = os.path.join(ROOT, "culof", "_culof.cpp")
PYEXT = os.path.join(ROOT, "culof", "_culof" + (sysconfig.get_config_var("EXT_SUFFIX") or ".so"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC,-O2,-fvisibility=hidden",
    "-Xptxas",
    "-warn-spills",
    *ARCH,
]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest() -> str:
    h = hashlib.sha256()
    files = sorted(
        [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
        + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
        + [PYEXT_SRC]
    )
    for p in files:
        with open(p, "rb") as fh:
            h.update(p.encode())
            h.update(fh.read())
    h.update(" ".join(NVCC_FLAGS).encode())
    h.update(nvcc().encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every .cu in csrc/ for sm_103a and link the shared library."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    dig = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(PYEXT) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == dig:
                return LIB

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [nvcc(), *NVCC_FLAGS, "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")
        if verbose and (res.stdout or res.stderr):
            print(res.stdout, res.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    build_pyext()
    with open(stamp, "w") as fh:
        fh.write(dig)
    return LIB


def build_pyext() -> str:
    """culof/_culof.cpp -> culof/_culof<EXT_SUFFIX>, linked to the library
    beside culof_gb300/ through a relative run path."""
    tmp = PYEXT + f".tmp{os.getpid()}"
    cmd = [
        os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
        "-I", sysconfig.get_paths()["include"], "-I", INCLUDE, PYEXT_SRC, "-o", tmp,
        "-L", HERE, "-lculof_gb300", "-Wl,-rpath,$ORIGIN/../culof_gb300",
    ]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"building the Python binding failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, PYEXT)
    return PYEXT


if __name__ == "__main__":
    print(build(force=True, verbose=True))
