"""Parity at the full sizes the measurements are quoted on.

* 10M x 64 float32, k = 1024 (1024 blobs in [-5, 5]^64, per-blob sigma in
  [0.5, 2], seed 2; random-row init), mixed fp16 and bf16 forms.  The session
  is stepped one Lloyd iteration at a time.  After each step, the labels must
  equal the oracle's exactly for all 10M samples, against that step's input
  centroids (samples the tensor-core margin does not certify are re-evaluated
  in exact float32).  The step's new centroids must be within 1e-5 relative of
  the oracle's pass from the same input centroids: float32 cluster sums arrive
  in any order, as the reference's atomics do.  After the final pass, labels
  equal the oracle's assignment, and the inertia is within 1e-5 of the
  oracle's long-double sum.
* 5M x 14, k = 127 (127 blobs, sigma 1.5, seed 1; centroid 0 = 1e3 * ones, so
  the first iteration relocates), tol = 0, max_iter = 100, float32 and
  float64, plain form, against the oracle's whole driver run.  The iteration
  count must be equal, labels identical except where the oracle's two best
  centroids are within 1e-5 relative, and centroids and inertia within 1e-5
  (float32) / 1e-12 (float64).

The oracle runs on all host cores: about 4 s per 10M x 64 x 1024 pass.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

FORMS = {"fp16": 2, "bf16": 1}
RTOL = {np.float32: 1e-5, np.float64: 1e-12}


@pytest.fixture(scope="module")
def c3_data():
    X, C0 = bench.workload_data("c3")
    return X, C0


@pytest.mark.parametrize("form", ["fp16", "bf16"])
def test_c3_mixed_steps_equal_oracle(oracle, c3_data, form):
    import torch

    from kmeans_dpcpp_gb300 import capi

    X, C0 = c3_data
    d, n = X.shape
    k = C0.shape[1]
    L = capi.lib()
    w_h = np.ones(n, np.float32)
    Xg = torch.from_numpy(X).cuda()
    w = torch.ones(n, dtype=torch.float32, device="cuda")
    cur = torch.from_numpy(C0.copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    steps = 3
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, 0.0, steps, FORMS[form],
                                        stream.cuda_stream, ctypes.byref(fit)))
    try:
        C_prev = C0.copy()
        relocated = 0
        for step in range(steps):
            capi.check(L.kmc_fit_step(fit, 1))
            torch.cuda.synchronize()
            lab_g = lab.cpu().numpy()
            C_g = cur.cpu().numpy()
            lab_o, C_o, _, rel = oracle.lloyd_iteration(X, w_h, C_prev)
            relocated += rel
            bad = np.flatnonzero(lab_g != lab_o)
            assert bad.size == 0, f"step {step}: {bad.size} labels differ, first {bad[:8]}"
            scale = np.abs(C_o).max()
            np.testing.assert_allclose(C_g, C_o, rtol=1e-5, atol=1e-5 * scale,
                                       err_msg=f"centroids after step {step}")
            C_prev = C_g
        it, done, sh = ctypes.c_int64(), ctypes.c_int(), ctypes.c_double()
        capi.check(L.kmc_fit_status(fit, ctypes.byref(it), ctypes.byref(done), ctypes.byref(sh)))
        assert it.value == steps
        n_it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(n_it), ctypes.byref(inr)))
        err, total = ctypes.c_int(), ctypes.c_int64()
        capi.check(L.kmc_fit_rechecked(fit, None, ctypes.byref(total), ctypes.byref(err)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    assert err.value == 0
    C_fin = res.cpu().numpy()
    np.testing.assert_array_equal(C_fin, C_prev)
    lab_fin = oracle.assignment(X, C_fin)
    np.testing.assert_array_equal(lab.cpu().numpy(), lab_fin)
    inr_o = oracle.sum_ld(oracle.compute_inertia(X, w_h, C_fin, lab_fin))
    assert inr.value == pytest.approx(inr_o, rel=1e-5)
    # rechecks are a small share of the (steps + final pass) * n evaluations
    assert 0 < total.value < 0.2 * (steps + 1) * n


def _near_tie(X, C, i, rel=1e-5):
    """True when sample i's two nearest centroids are within `rel` of each other (float64)."""
    x = X[:, i].astype(np.float64)
    d2 = ((C.astype(np.float64) - x[:, None]) ** 2).sum(axis=0)
    a, b = np.sort(d2)[:2]
    return (b - a) <= rel * max(b, 1e-300)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_c2_whole_trajectory_equals_oracle(kdp, oracle, dt):
    import torch

    n, d, k = 5_000_000, 14, 127
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.5, 1, dtype=dt)
    C0 = bench.random_row_init(X, k, 1, far_first=True)
    it_o, lab_o, C_o, inr_o, rel_o = oracle.kmeans_lloyd_driver(X, np.ones(n, dt), C0, 0.0, 100)
    assert rel_o >= 1

    Xg = torch.from_numpy(X).cuda()
    w = torch.ones(n, dtype=Xg.dtype, device="cuda")
    init = torch.from_numpy(C0.copy()).cuda()
    res_c = torch.empty_like(init)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    it_g, inertia = kdp.kmeans_lloyd_driver(Xg, w, init, lab, res_c, 0.0, False, 100, 8, 128, 0.7, None)
    lab_g, C_g = lab.cpu().numpy(), res_c.cpu().numpy()

    assert it_g == it_o
    bad = np.flatnonzero(lab_g != lab_o)
    assert bad.size <= 16, f"{bad.size} labels differ"
    for i in bad:
        assert _near_tie(X, C_o, i), f"sample {i} differs without a near-tie"
    np.testing.assert_allclose(C_g, C_o, rtol=RTOL[dt], atol=RTOL[dt] * np.abs(C_o).max())
    assert float(inertia[0]) == pytest.approx(inr_o, rel=RTOL[dt])


# The c2 configuration in the mixed form (d = 14: the tensor-core assignment
# with the fixed-point integer cluster sums): the whole 100-iteration
# trajectory equals the oracle's as in the plain form.
@pytest.mark.parametrize("form", ["mixed-fp16", "mixed-bf16"])
def test_c2_mixed_whole_trajectory_equals_oracle(kdp, oracle, form):
    import torch

    n, d, k = 5_000_000, 14, 127
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.5, 1)
    C0 = bench.random_row_init(X, k, 1, far_first=True)
    it_o, lab_o, C_o, inr_o, rel_o = oracle.kmeans_lloyd_driver(X, np.ones(n, np.float32), C0, 0.0, 100)
    assert rel_o >= 1

    Xg = torch.from_numpy(X).cuda()
    w = torch.ones(n, dtype=Xg.dtype, device="cuda")
    init = torch.from_numpy(C0.copy()).cuda()
    res_c = torch.empty_like(init)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    it_g, inertia = kdp.kmeans_lloyd_driver(Xg, w, init, lab, res_c, 0.0, False, 100, 8, 128, 0.7, None,
                                            form=form)
    lab_g, C_g = lab.cpu().numpy(), res_c.cpu().numpy()

    assert it_g == it_o
    bad = np.flatnonzero(lab_g != lab_o)
    assert bad.size <= 16, f"{bad.size} labels differ"
    for i in bad:
        assert _near_tie(X, C_o, i), f"sample {i} differs without a near-tie"
    np.testing.assert_allclose(C_g, C_o, rtol=RTOL[np.float32], atol=RTOL[np.float32] * np.abs(C_o).max())
    assert float(inertia[0]) == pytest.approx(inr_o, rel=RTOL[np.float32])
