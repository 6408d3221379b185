"""Row-major input (kmc_fit_create_rowmajor_*) against the feature-major sessions.

The mixed forms read a row-major X directly in their one-time operand
conversion and every later kernel (assignment, recheck, sums, inertia,
relocation) reads the row-major fp32 copy, so a fit from X (n, d) must give
what the same fit from X_t (d, n) gives.  The plain form makes one
feature-major copy and then runs the identical path.  Relocation is exercised
by a far-away initial centroid that empties its cluster in the first
iteration.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

FORMS = {"plain": 0, "bf16": 1, "fp16": 2}
SUF = {np.float32: "f32_i32", np.float64: "f64_i32"}


def _fit(X_t, C0, form, max_iter, rowmajor, dtype):
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    d, n = X_t.shape
    k = C0.shape[1]
    Xsrc = np.ascontiguousarray(X_t.T if rowmajor else X_t, dtype=dtype)
    Xg = torch.from_numpy(Xsrc).cuda()
    w = torch.ones(n, dtype=Xg.dtype, device="cuda")
    cur = torch.from_numpy(np.ascontiguousarray(C0, dtype=dtype).copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    name = ("kmc_fit_create_rowmajor_" if rowmajor else "kmc_fit_create_") + SUF[dtype]
    capi.check(getattr(L, name)(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                res.data_ptr(), n, d, k, 0.0, max_iter, FORMS[form],
                                stream.cuda_stream, ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_run(fit))
        it, inertia = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inertia)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    return it.value, lab.cpu().numpy(), res.cpu().numpy(), inertia.value


# (n, d, centres, k, form, dtype, iterations): d <= 32 keeps float64 sums in the
# mixed form (bit-stable trajectories); beyond that one iteration is compared
# (float32 reductions arrive in any order).
CASES = [(30_000, 14, 40, 64, "plain", np.float32, 5),
         (20_000, 20, 40, 64, "plain", np.float64, 5),
         (40_000, 24, 60, 100, "fp16", np.float32, 5),
         (40_000, 64, 150, 300, "fp16", np.float32, 1),
         (30_000, 100, 100, 200, "bf16", np.float32, 1),
         (8_193, 7, 10, 16, "bf16", np.float32, 4)]


@pytest.mark.parametrize("n,d,centres,k,form,dtype,iters", CASES)
def test_rowmajor_fit_equals_feature_major_fit(oracle, n, d, centres, k, form, dtype, iters):
    X_t, _, _ = bench.make_blobs(n, d, centres, (-5, 5), 1.0, seed=n + d, dtype=dtype)
    C0 = bench.random_row_init(X_t, k, seed=d, far_first=True)   # empties a cluster
    it_f, lab_f, C_f, inr_f = _fit(X_t, C0, form, iters, False, dtype)
    it_r, lab_r, C_r, inr_r = _fit(X_t, C0, form, iters, True, dtype)
    assert it_r == it_f == iters
    np.testing.assert_array_equal(lab_r, lab_f)
    if form == "plain" or d <= 32:
        # float64 sums in arrival order: the two runs agree to the last bit
        # of the rounded result, give or take one unit
        rt = 1e-13 if dtype == np.float64 else 2.5e-7
        np.testing.assert_allclose(C_r, C_f, rtol=rt, atol=rt * np.abs(C_f).max())
        assert inr_r == pytest.approx(inr_f, rel=1e-12 if dtype == np.float64 else 1e-6)
    else:
        np.testing.assert_allclose(C_r, C_f, rtol=1e-5, atol=1e-5 * np.abs(C_f).max())
        assert inr_r == pytest.approx(inr_f, rel=1e-5)
    # the final labels are the exact assignment against the final centroids
    np.testing.assert_array_equal(lab_r, oracle.assignment(X_t, C_r.astype(X_t.dtype)))
