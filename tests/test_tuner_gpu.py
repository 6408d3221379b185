"""The single-fit tile autotuner.

Every centroid-tile width of the plain kernels computes each (sample,
centroid) score with the same arithmetic, so fits forced to each width give
the same labels, iteration counts and centroids (float64 sums may differ in
the last bit when the tile width changes the launch shape).  The autotuner's
choice is cached per (d, power-of-two bucket of k, dtype): asking again (for
any k of the bucket) gives the same variant without another measurement, and
the choice is written to the tile cache file.
"""
import ctypes
import os

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


def _fit(L, capi, X, C0, variant, tol=0.0, max_iter=20):
    import torch

    d, n = X.shape
    k = C0.shape[1]
    Xg = torch.from_numpy(X).cuda()
    w = torch.ones(n, dtype=Xg.dtype, device="cuda")
    cur = torch.from_numpy(C0.copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    create = L.kmc_fit_create_f64_i32 if X.dtype == np.float64 else L.kmc_fit_create_f32_i32
    fit = ctypes.c_void_p()
    capi.check(create(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(), res.data_ptr(),
                      n, d, k, tol, max_iter, 0, torch.cuda.current_stream().cuda_stream,
                      ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_set_tile_variant(fit, variant))
        capi.check(L.kmc_fit_run(fit))
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    return it.value, lab.cpu().numpy(), res.cpu().numpy(), inr.value


@pytest.mark.parametrize("n,d,k", [(50_000, 14, 16), (40_000, 14, 127), (20_000, 33, 300),
                                   (9_000, 5, 3)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_tile_variants_give_the_same_fit(oracle, n, d, k, dt):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.0, n + k, dtype=dt)
    C0 = bench.random_row_init(X, k, n + k)
    runs = [_fit(L, capi, X, C0, v) for v in (0, 1, 2)]
    it0, lab0, C0r, inr0 = runs[0]
    for it, lab, C, inr in runs[1:]:
        assert it == it0
        np.testing.assert_array_equal(lab, lab0)
        if dt == np.float32:
            np.testing.assert_array_equal(C, C0r)
        else:
            np.testing.assert_allclose(C, C0r, rtol=1e-12, atol=1e-12 * np.abs(C0r).max())
        assert inr == pytest.approx(inr0, rel=1e-12)
    np.testing.assert_array_equal(lab0, oracle.assignment(X, C0r))
    with pytest.raises(RuntimeError, match="kmc error 1"):
        _fit(L, capi, X, C0, 3)


def test_tuner_choice_is_cached(tmp_path):
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    cache = tmp_path / "tiles.txt"
    old = os.environ.get("KMC_TILE_CACHE")
    os.environ["KMC_TILE_CACHE"] = str(cache)
    try:
        s = torch.cuda.current_stream().cuda_stream
        v1, v2, v3 = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        capi.check(L.kmc_fit_tile_variant(23, 77, 4, s, ctypes.byref(v1)))
        capi.check(L.kmc_fit_tile_variant(23, 100, 4, s, ctypes.byref(v2)))   # same bucket (128)
        capi.check(L.kmc_fit_tile_variant(23, 77, 8, s, ctypes.byref(v3)))     # float64: own key
        assert v1.value in (0, 1, 2) and v2.value == v1.value and v3.value in (0, 1)
        lines = cache.read_text().split("\n")
        assert lines.count(f"23 128 fit-f32 {v1.value}") == 1
        assert lines.count(f"23 128 fit-f64 {v3.value}") == 1
        assert L.kmc_fit_tile_variant(23, 77, 2, s, ctypes.byref(v1)) == 1
    finally:
        if old is None:
            del os.environ["KMC_TILE_CACHE"]
        else:
            os.environ["KMC_TILE_CACHE"] = old


# ---------------------------------------------------------------------------
# Mixed forms: the kernel variant (ring depth, and up to 32 features the
# fixed-point cluster sums with 4 or 2 columns per update thread or float
# reductions) is chosen by the same autotuner.  Every variant must give a fit
# whose final labels are the exact float32 labels of its centroids and whose
# centroids follow the oracle; the fixed-point variants (integer sums) give
# bit-identical centroids.
MIXED_FP16 = 2


def _mixed_fit(L, capi, X, C0, max_iter):
    import torch

    d, n = X.shape
    k = C0.shape[1]
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    w = torch.ones(n, dtype=torch.float32, device="cuda")
    cur = torch.from_numpy(C0.copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    fit = ctypes.c_void_p()
    rc = L.kmc_fit_create_f32_i32(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                  res.data_ptr(), n, d, k, 0.0, max_iter, MIXED_FP16,
                                  torch.cuda.current_stream().cuda_stream, ctypes.byref(fit))
    if rc != 0:
        return rc, None
    try:
        v = ctypes.c_int()
        capi.check(L.kmc_fit_mixed_variant(fit, ctypes.byref(v)))
        capi.check(L.kmc_fit_run(fit))
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    return 0, (v.value, it.value, lab.cpu().numpy(), res.cpu().numpy())


@pytest.mark.parametrize("n,d,k", [(60_000, 16, 40), (50_000, 32, 100), (40_000, 64, 200)])
def test_mixed_variants_give_the_same_fit(oracle, n, d, k):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.0, n + d)
    C0 = np.ascontiguousarray(bench.random_row_init(X, k, n + d))
    iters = 2
    _, _, C_o, _, _ = oracle.kmeans_lloyd_driver(X, np.ones(n, np.float32), C0, 0.0, iters)
    runs = {}
    try:
        for code in [10 * s + f for s in (4, 3, 2) for f in (4, 2, 0)]:
            capi.check(L.kmc_debug_force_mixed_variant(code))
            rc, out = _mixed_fit(L, capi, X, C0, iters)
            if rc == 1:  # this variant does not fit the shape
                continue
            capi.check(rc)
            runs[code] = out
    finally:
        capi.check(L.kmc_debug_force_mixed_variant(-1))
    assert len(runs) >= 2 if d <= 32 else len(runs) >= 1
    fixed = []
    for code, (v, it, lab, C) in runs.items():
        assert v == code and it == iters
        np.testing.assert_array_equal(lab, oracle.assignment(X, C))
        np.testing.assert_allclose(C, C_o, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
        if code % 10:
            fixed.append(C)
    for C in fixed[1:]:
        np.testing.assert_array_equal(C, fixed[0])
    if d <= 32:
        assert fixed, "no fixed-point variant fits"


def test_mixed_tuner_choice_is_cached(tmp_path):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    cache = tmp_path / "tiles.txt"
    old = os.environ.get("KMC_TILE_CACHE")
    os.environ["KMC_TILE_CACHE"] = str(cache)
    try:
        # a shape no other test uses, so the choice is not already in memory
        X, _, _ = bench.make_blobs(30_000, 19, 16, (-10, 10), 1.0, 5)
        out = []
        for k in (37, 50):  # the same bucket (64)
            C0 = np.ascontiguousarray(bench.random_row_init(X, k, 5))
            rc, res = _mixed_fit(L, capi, X, C0, 1)
            capi.check(rc)
            out.append(res[0])
        assert out[0] == out[1] and out[0] // 10 in (2, 3, 4) and out[0] % 10 in (0, 2, 4)
        assert cache.read_text().split("\n").count(f"19 64 mixed-fp16 {out[0]}") == 1
    finally:
        if old is None:
            del os.environ["KMC_TILE_CACHE"]
        else:
            os.environ["KMC_TILE_CACHE"] = old
