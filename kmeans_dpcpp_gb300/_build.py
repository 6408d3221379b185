"""In-tree build of the engine's native parts.

* ``libkmeans_gb300.so``: CUDA kernels + C++ host driver + the C ABI declared in
  ``include/kmeans_gb300.h``, compiled by nvcc for sm_103a only.
* ``_kmeans_dpcpp*.so``: the pybind11 module that mirrors the reference's
  ``python_api/_kmeans_lloyd.cpp`` surface on top of the C ABI (g++, pybind11
  headers shipped with PyTorch, no CUDA code).

Translation units are compiled in parallel and only when their inputs changed.
"""
from __future__ import annotations

import concurrent.futures as _cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys
import sysconfig

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
CSRC = os.path.join(PKG_DIR, "csrc")
INCLUDE = os.path.join(REPO_DIR, "include")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_NAME = "libkmeans_gb300.so"
LIB_PATH = os.path.join(PKG_DIR, LIB_NAME)

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = GENCODE + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-O3", "-I" + INCLUDE,
]

CU_SOURCES = [
    "kernels_util.cu",
    "kernels_lloyd.cu",
    "kernels_reloc.cu",
    "kernels_mixed.cu",
    "driver.cu",
    "capi.cu",
    "noalloc.cu",
    "batch_kernels.cu",
    "serve.cu",
    "init.cu",
]
HEADERS = ["km_common.cuh", "km_kernels.cuh", "km_fit.cuh", "km_mixed.cuh", "km_batch.cuh"]


def _digest(paths, extra=""):
    h = hashlib.sha256((platform.machine() + extra).encode())
    for p in paths:
        if os.path.exists(p):
            with open(p, "rb") as f:
                h.update(f.read())
    return h.hexdigest()[:16]


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _hdrs():
    return [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "kmeans_gb300.h")]


def _compile_cu(src):
    os.makedirs(BUILD_DIR, exist_ok=True)
    path = os.path.join(CSRC, src)
    tag = _digest([path] + _hdrs(), " ".join(NVCC_FLAGS))
    obj = os.path.join(BUILD_DIR, src.replace(".cu", f".{tag}.o"))
    if not os.path.exists(obj):
        _run([NVCC] + NVCC_FLAGS + ["-c", path, "-o", obj + ".tmp"])
        os.replace(obj + ".tmp", obj)
    return obj


def build_library(verbose=False):
    """Compile the CUDA sources and link libkmeans_gb300.so (sm_103a)."""
    srcs = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with _cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile_cu, srcs))
    tag = _digest(objs)
    stamp = os.path.join(BUILD_DIR, "lib.stamp")
    if os.path.exists(LIB_PATH) and os.path.exists(stamp) and open(stamp).read() == tag:
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    _run([NVCC] + GENCODE + ["-shared", "-o", tmp] + objs + ["-cudart", "static"])
    os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(tag)
    if verbose:
        print("built", LIB_PATH)
    return LIB_PATH


def _pybind_include():
    import torch  # pybind11 headers ship with PyTorch

    inc = os.path.join(os.path.dirname(torch.__file__), "include")
    if not os.path.exists(os.path.join(inc, "pybind11", "pybind11.h")):
        raise RuntimeError("pybind11 headers not found under " + inc)
    return inc


def pymod_path():
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    return os.path.join(PKG_DIR, "_kmeans_dpcpp" + suffix)


def build_pymodule(verbose=False):
    """Build the pybind11 module _kmeans_dpcpp against libkmeans_gb300.so."""
    src = os.path.join(CSRC, "py_kmeans_dpcpp.cpp")
    out = pymod_path()
    cxx = os.environ.get("CXX", "g++")
    flags = ["-O2", "-std=c++17", "-shared", "-fPIC", "-fvisibility=hidden",
             "-I" + sysconfig.get_paths()["include"], "-I" + _pybind_include(), "-I" + INCLUDE]
    tag = _digest([src, os.path.join(INCLUDE, "kmeans_gb300.h"), LIB_PATH], " ".join(flags))
    stamp = os.path.join(BUILD_DIR, "pymod.stamp")
    if os.path.exists(out) and os.path.exists(stamp) and open(stamp).read() == tag:
        return out
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = out + ".tmp"
    _run([cxx] + flags + [src, "-o", tmp, "-L" + PKG_DIR, "-lkmeans_gb300",
                          "-Wl,-rpath,$ORIGIN"])
    os.replace(tmp, out)
    with open(stamp, "w") as f:
        f.write(tag)
    if verbose:
        print("built", out)
    return out


def build_all(verbose=False):
    build_library(verbose)
    build_pymodule(verbose)


def clean():
    shutil.rmtree(BUILD_DIR, ignore_errors=True)
    for p in (LIB_PATH, pymod_path()):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
