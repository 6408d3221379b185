"""numpy front-end of the CPU oracle (oracle/kmref.cpp).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product package.  Arrays follow the
reference layouts: X_t (d, n), centroids (d, k); labels are int64 here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_DIR, "libkmref.so")

_c_i64 = ctypes.c_int64
_c_dbl = ctypes.c_double
_p = ctypes.c_void_p


def build():
    """Build libkmref.so with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", _DIR, "libkmref.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        for suf, ct in (("f32", ctypes.c_float), ("f64", ctypes.c_double)):
            getattr(L, f"kmref_half_norm_{suf}").argtypes = [_p, _p, _c_i64, _c_i64]
            getattr(L, f"kmref_broadcast_divide_{suf}").argtypes = [_p, _p, _c_i64, _c_i64]
            f = getattr(L, f"kmref_threshold_{suf}")
            f.argtypes = [_p, _c_i64, _c_i64]
            f.restype = ct
            getattr(L, f"kmref_shifts_{suf}").argtypes = [_p, _p, _p, _c_i64, _c_i64]
            getattr(L, f"kmref_distances_{suf}").argtypes = [_p, _p, _p, _c_i64, _c_i64, _c_i64]
            f = getattr(L, f"kmref_sum_{suf}")
            f.argtypes = [_p, _c_i64]
            f.restype = _c_dbl
            getattr(L, f"kmref_reduce_centroids_{suf}").argtypes = [_p] * 6 + [_c_i64] * 3
            getattr(L, f"kmref_select_{suf}").argtypes = [_c_i64, _p, ct, _p, _p, _p, _c_i64]
            getattr(L, f"kmref_relocate_{suf}").argtypes = [_c_i64] + [_p] * 8 + [_c_i64] * 3
            getattr(L, f"kmref_assignment_{suf}").argtypes = [_p] * 4 + [_c_i64] * 3
            getattr(L, f"kmref_inertia_{suf}").argtypes = [_p] * 5 + [_c_i64] * 3
            getattr(L, f"kmref_fused_step_{suf}").argtypes = [_p] * 7 + [_c_i64] * 3
            f = getattr(L, f"kmref_iteration_{suf}")
            f.argtypes = [_p] * 5 + [_c_i64] * 3 + [_p]
            f.restype = _c_dbl
            f = getattr(L, f"kmref_driver_{suf}")
            f.argtypes = [_p] * 5 + [_c_i64] * 3 + [_c_dbl, _c_i64, _p, _p]
            f.restype = _c_i64
        for suf in ("f32", "f64"):
            getattr(L, f"kmref_kmeanspp_{suf}").argtypes = [_p, _p, _c_i64, _c_i64, _c_i64,
                                                             ctypes.c_uint64, _p, _p]
        L.kmref_num_threads.restype = ctypes.c_int
        L.kmref_set_num_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _suf(dtype):
    dt = np.dtype(dtype)
    if dt == np.float32:
        return "f32"
    if dt == np.float64:
        return "f64"
    raise ValueError(f"unsupported dtype {dt}")


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _c(a, dtype=None):
    return np.ascontiguousarray(a if dtype is None else np.asarray(a, dtype=dtype))


def num_threads():
    return lib().kmref_num_threads()


def set_num_threads(t):
    lib().kmref_set_num_threads(int(t))


def half_l2_norm_squared(C):
    C = _c(C)
    d, k = C.shape
    out = np.empty(k, C.dtype)
    getattr(lib(), f"kmref_half_norm_{_suf(C.dtype)}")(_ptr(C), _ptr(out), d, k)
    return out


def broadcast_divide(X, y):
    X = _c(X).copy()
    y = _c(y, X.dtype)
    getattr(lib(), f"kmref_broadcast_divide_{_suf(X.dtype)}")(_ptr(X), _ptr(y), X.shape[0], X.shape[1])
    return X


def compute_threshold(data, topk):
    data = _c(data)
    return getattr(lib(), f"kmref_threshold_{_suf(data.dtype)}")(_ptr(data), data.shape[0], int(topk))


def centroid_shifts(a, b):
    a, b = _c(a), _c(b)
    out = np.empty(a.shape[1], a.dtype)
    getattr(lib(), f"kmref_shifts_{_suf(a.dtype)}")(_ptr(a), _ptr(b), _ptr(out), a.shape[0], a.shape[1])
    return out


def distances(X_t, C):
    X_t, C = _c(X_t), _c(C)
    d, n = X_t.shape
    k = C.shape[1]
    out = np.empty((k, n), X_t.dtype)
    getattr(lib(), f"kmref_distances_{_suf(X_t.dtype)}")(_ptr(X_t), _ptr(C), _ptr(out), n, d, k)
    return out


def sum_ld(x):
    x = _c(x)
    return getattr(lib(), f"kmref_sum_{_suf(x.dtype)}")(_ptr(x), x.shape[0])


def reduce_centroids(sizes_cp, cent_cp, n_empty_init=0, list_fill=None):
    sizes_cp, cent_cp = _c(sizes_cp), _c(cent_cp)
    P, d, k = cent_cp.shape
    osz = np.empty(k, sizes_cp.dtype)
    oc = np.empty((d, k), sizes_cp.dtype)
    lst = np.full(k, -1 if list_fill is None else list_fill, np.int64)
    ne = np.array([n_empty_init], np.int64)
    getattr(lib(), f"kmref_reduce_centroids_{_suf(sizes_cp.dtype)}")(
        _ptr(sizes_cp), _ptr(cent_cp), _ptr(osz), _ptr(oc), _ptr(lst), _ptr(ne), P, d, k)
    return osz, oc, lst, int(ne[0])


def select_samples_far_from_centroid(n_selected, dist, thr, fill=0, n_gt=0, n_eq=1):
    dist = _c(dist)
    n = dist.shape[0]
    sel = np.full(n, fill, np.int64)
    ng = np.array([n_gt], np.int64)
    nq = np.array([n_eq], np.int64)
    getattr(lib(), f"kmref_select_{_suf(dist.dtype)}")(int(n_selected), _ptr(dist), thr, _ptr(sel),
                                                       _ptr(ng), _ptr(nq), n)
    return sel, int(ng[0]), int(nq[0])


def relocate_empty_clusters(n_empty, X_t, w, labels, empty_list, sq_dist, C, sizes, inertia):
    X_t, w = _c(X_t), _c(w)
    lab, lst = _c(labels, np.int64), _c(empty_list, np.int64)
    sq = _c(sq_dist)
    C, sizes, inertia = _c(C).copy(), _c(sizes).copy(), _c(inertia).copy()
    d, n = X_t.shape
    k = C.shape[1]
    getattr(lib(), f"kmref_relocate_{_suf(X_t.dtype)}")(
        int(n_empty), _ptr(X_t), _ptr(w), _ptr(lab), _ptr(lst), _ptr(sq), _ptr(C), _ptr(sizes),
        _ptr(inertia), n, d, k)
    return C, sizes, inertia


def assignment(X_t, C, hn=None):
    X_t, C = _c(X_t), _c(C)
    if hn is None:
        hn = half_l2_norm_squared(C)
    hn = _c(hn)
    d, n = X_t.shape
    k = C.shape[1]
    lab = np.empty(n, np.int64)
    getattr(lib(), f"kmref_assignment_{_suf(X_t.dtype)}")(_ptr(X_t), _ptr(C), _ptr(hn), _ptr(lab), n, d, k)
    return lab


def compute_inertia(X_t, w, C, labels):
    X_t, C = _c(X_t), _c(C)
    w = None if w is None else _c(w)
    lab = _c(labels, np.int64)
    d, n = X_t.shape
    out = np.empty(n, X_t.dtype)
    getattr(lib(), f"kmref_inertia_{_suf(X_t.dtype)}")(_ptr(X_t), _ptr(w), _ptr(C), _ptr(lab), _ptr(out),
                                                       n, d, C.shape[1])
    return out


def fused_lloyd_single_step(X_t, w, C, hn=None):
    X_t, w, C = _c(X_t), _c(w), _c(C)
    if hn is None:
        hn = half_l2_norm_squared(C)
    hn = _c(hn)
    d, n = X_t.shape
    k = C.shape[1]
    lab = np.empty(n, np.int64)
    sums = np.empty((d, k), X_t.dtype)
    sizes = np.empty(k, X_t.dtype)
    getattr(lib(), f"kmref_fused_step_{_suf(X_t.dtype)}")(_ptr(X_t), _ptr(w), _ptr(C), _ptr(hn), _ptr(lab),
                                                          _ptr(sums), _ptr(sizes), n, d, k)
    return lab, sums, sizes


def lloyd_iteration(X_t, w, C):
    """One pass of the driver's loop body from centroids C (d, k).

    Returns (labels against C, next centroids (d, k), shift total, relocated)."""
    X_t, w, C = _c(X_t), _c(w), _c(C)
    d, n = X_t.shape
    k = C.shape[1]
    lab = np.empty(n, np.int64)
    nxt = np.empty_like(C)
    rel = np.zeros(1, np.int64)
    sh = getattr(lib(), f"kmref_iteration_{_suf(X_t.dtype)}")(
        _ptr(X_t), _ptr(w), _ptr(C), _ptr(lab), _ptr(nxt), n, d, k, _ptr(rel))
    return lab, nxt, float(sh), bool(rel[0])


def kmeans_lloyd_driver(X_t, w, init_C, tol, max_iter):
    """Returns (n_iter, labels, centroids (d, k), inertia (float64), relocations)."""
    X_t, w = _c(X_t), _c(w)
    C = _c(init_C).copy()
    d, n = X_t.shape
    k = C.shape[1]
    lab = np.empty(n, np.int64)
    res = np.empty_like(C)
    inr = np.zeros(1, np.float64)
    rel = np.zeros(1, np.int64)
    it = getattr(lib(), f"kmref_driver_{_suf(X_t.dtype)}")(
        _ptr(X_t), _ptr(w), _ptr(C), _ptr(lab), _ptr(res), n, d, k, float(tol), int(max_iter),
        _ptr(inr), _ptr(rel))
    return int(it), lab, res, float(inr[0]), int(rel[0])


def kmeans_plusplus(X_t, k, seed, w=None):
    """k-means++ rows and centroids (d, k), the engine's seeding restated."""
    X_t = _c(X_t)
    w = None if w is None else _c(w, X_t.dtype)
    d, n = X_t.shape
    C = np.empty((d, k), X_t.dtype)
    rows = np.empty(k, np.int32)
    getattr(lib(), f"kmref_kmeanspp_{_suf(X_t.dtype)}")(_ptr(X_t), _ptr(w), n, d, k, seed, _ptr(C), _ptr(rows))
    return rows, C
