"""ctypes binding of the C ABI in ``include/kmeans_gb300.h``.

The prototypes are read from the header itself, so every declared entry point
gets ``argtypes``/``restype`` without a hand-maintained list.  This is the
binding a Python caller (or a test) uses to reach the engine below the
pybind11 surface; pointers are passed as integers (``tensor.data_ptr()``).
"""
from __future__ import annotations

import ctypes
import os
import re

_PKG = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(_PKG), "include", "kmeans_gb300.h")
LIB_PATH = os.path.join(_PKG, "libkmeans_gb300.so")

KMC_OK = 0

_CTYPES = {
    "int": ctypes.c_int,
    "int64_t": ctypes.c_int64,
    "int32_t": ctypes.c_int32,
    "uint64_t": ctypes.c_uint64,
    "double": ctypes.c_double,
    "float": ctypes.c_float,
    "void": None,
}

PRINT_FN = ctypes.CFUNCTYPE(None, ctypes.c_char_p, ctypes.c_void_p)


class ServeRequest(ctypes.Structure):
    """kmc_serve_request_t"""
    _fields_ = [("arrival_s", ctypes.c_double), ("kind", ctypes.c_int32),
                ("n_features", ctypes.c_int32), ("n_samples", ctypes.c_int64),
                ("n_clusters", ctypes.c_int64), ("n_centers", ctypes.c_int64),
                ("seed", ctypes.c_uint64), ("tol", ctypes.c_double), ("max_iter", ctypes.c_int64),
                ("model", ctypes.c_int64), ("std_lo", ctypes.c_float), ("std_hi", ctypes.c_float)]


class ServeResult(ctypes.Structure):
    """kmc_serve_result_t"""
    _fields_ = [("admit_s", ctypes.c_double), ("finish_s", ctypes.c_double),
                ("n_iter", ctypes.c_int64), ("inertia", ctypes.c_double),
                ("status", ctypes.c_int32), ("pad", ctypes.c_int32)]


def _strip_comments(text: str) -> str:
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    return re.sub(r"//[^\n]*", " ", text)


def parse_header(path: str = HEADER):
    """Return {name: (restype_str, [param_type_str, ...])} for every kmc_* prototype."""
    text = _strip_comments(open(path).read())
    protos = {}
    for m in re.finditer(r"([A-Za-z_][\w \*]*?)\b(kmc_\w+)\s*\(([^;{]*?)\)\s*;", text):
        ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
        if ret.startswith("typedef"):
            continue
        ptypes = []
        if params and params != "void":
            for p in params.split(","):
                p = " ".join(p.split())
                # drop the parameter name
                pm = re.match(r"(.*?)([A-Za-z_]\w*)$", p)
                t = pm.group(1).strip() if pm else p
                ptypes.append(t)
        protos[name] = (ret, ptypes)
    return protos


def _ctype(t: str):
    t = t.replace("const ", "").strip()
    if t.endswith("*") or t in ("kmc_stream_t", "kmc_event_t", "kmc_fit_t", "kmc_batch_t",
                                "kmc_server_t"):
        if t == "char *" or t == "char*":
            return ctypes.c_char_p
        return ctypes.c_void_p
    if t == "kmc_print_fn":
        return PRINT_FN
    return _CTYPES[t]


_lib = None


def lib():
    """Load libkmeans_gb300.so and attach prototypes from the header."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise OSError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
    L = ctypes.CDLL(LIB_PATH)
    for name, (ret, ptypes) in parse_header().items():
        fn = getattr(L, name)
        fn.argtypes = [_ctype(t) for t in ptypes]
        fn.restype = ctypes.c_char_p if "char" in ret else _ctype(ret)
    _lib = L
    return L


def check(rc: int):
    if rc != KMC_OK:
        raise RuntimeError(f"kmc error {rc}: {lib().kmc_last_error().decode()}")
