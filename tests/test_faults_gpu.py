"""Failure paths: a device-side wait that runs out, and allocations that fail.

Nothing here faults or hangs the GPU.  The timeout test arms a one-shot wait
on a barrier that no role of the tensor-core kernel completes, with a limit of
about a millisecond; the kernel must then wind down by itself (waiting for the
copies and tensor-core operations it already issued), stop the loop and report
KMC_ERR_DEVICE_TIMEOUT, and a fit started afterwards in the same process must
give the oracle's labels.  The allocation test makes the n-th scratch
allocation fail on the host, for every n a fit creation makes, and checks the
error code and that no scratch memory stays in use.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

KMC_ERR_OUT_OF_MEMORY = 3
KMC_ERR_DEVICE_TIMEOUT = 5
FORMS = {"plain": 0, "bf16": 1, "fp16": 2}


def _session(L, capi, X, C0, form, max_iter=5):
    import torch

    d, n = X.shape
    k = C0.shape[1]
    t = dict(X=torch.from_numpy(np.ascontiguousarray(X)).cuda(),
             w=torch.ones(n, dtype=torch.float32, device="cuda"),
             C=torch.from_numpy(np.ascontiguousarray(C0).copy()).cuda(),
             lab=torch.full((n,), -1, dtype=torch.int32, device="cuda"))
    t["res"] = torch.empty_like(t["C"])
    fit = ctypes.c_void_p()
    rc = L.kmc_fit_create_f32_i32(t["X"].data_ptr(), t["w"].data_ptr(), t["C"].data_ptr(),
                                  t["lab"].data_ptr(), t["res"].data_ptr(), n, d, k, 0.0, max_iter,
                                  FORMS[form], torch.cuda.current_stream().cuda_stream,
                                  ctypes.byref(fit))
    return rc, fit, t


def _data(n=256, d=64, k=256, seed=3):
    X, _, _ = bench.make_blobs(n, d, 16, (-5, 5), 1.0, seed=seed)
    C0 = np.random.default_rng(seed).uniform(-5, 5, (d, k)).astype(np.float32)
    return X, C0


@pytest.mark.parametrize("form", ["fp16", "bf16"])
@pytest.mark.parametrize("where", ["step", "final"])
def test_device_wait_timeout_is_reported_and_the_context_stays_usable(oracle, form, where):
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, C0 = _data()
    rc, fit, t = _session(L, capi, X, C0, form)
    capi.check(rc)
    try:
        # about a millisecond at the GB300's clock
        capi.check(L.kmc_fit_set_wait_limit(fit, 2_000_000, 1))
        if where == "step":
            capi.check(L.kmc_fit_step(fit, 1))
            it, done, sh = ctypes.c_int64(), ctypes.c_int(), ctypes.c_double()
            rc = L.kmc_fit_status(fit, ctypes.byref(it), ctypes.byref(done), ctypes.byref(sh))
        else:
            it, inr = ctypes.c_int64(), ctypes.c_double()
            rc = L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr))
        assert rc == KMC_ERR_DEVICE_TIMEOUT, (rc, L.kmc_last_error().decode())
        assert "device-side wait" in L.kmc_last_error().decode()
        err = ctypes.c_int()
        capi.check(L.kmc_fit_rechecked(fit, None, None, ctypes.byref(err)))
        assert err.value == 1
        # the loop was stopped: later steps are no-ops and keep reporting the error
        capi.check(L.kmc_fit_step(fit, 2))
        assert L.kmc_fit_run(fit) == KMC_ERR_DEVICE_TIMEOUT
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    torch.cuda.synchronize()  # no CUDA error is pending in the context

    # a fresh session in the same process gives the exact labels
    rc, fit, t = _session(L, capi, X, C0, form, max_iter=0)
    capi.check(rc)
    try:
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
        err = ctypes.c_int()
        capi.check(L.kmc_fit_rechecked(fit, None, None, ctypes.byref(err)))
        assert err.value == 0
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    np.testing.assert_array_equal(t["lab"].cpu().numpy(), oracle.assignment(X, C0))


def test_default_wait_limit_restored(oracle):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, C0 = _data(n=1000, seed=4)
    rc, fit, t = _session(L, capi, X, C0, "fp16", max_iter=0)
    capi.check(rc)
    try:
        capi.check(L.kmc_fit_set_wait_limit(fit, 2_000_000, 0))
        capi.check(L.kmc_fit_set_wait_limit(fit, 0, 0))   # back to the default
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    np.testing.assert_array_equal(t["lab"].cpu().numpy(), oracle.assignment(X, C0))


def _in_use(L):
    import torch

    torch.cuda.synchronize()
    v = ctypes.c_int64()
    L.kmc_scratch_bytes_in_use(ctypes.byref(v))
    return v.value


@pytest.mark.parametrize("form", ["plain", "fp16"])
def test_every_failed_allocation_of_a_fit_is_reported_without_leaks(oracle, form):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, C0 = _data(n=3000, d=20, k=40, seed=6)
    base = _in_use(L)
    failures = 0
    try:
        for after in range(64):
            capi.check(L.kmc_debug_fail_allocation(after))
            rc, fit, t = _session(L, capi, X, C0, form, max_iter=3)
            if rc == 0:
                break
            assert rc == KMC_ERR_OUT_OF_MEMORY, (rc, L.kmc_last_error().decode())
            assert "injected" in L.kmc_last_error().decode()
            assert _in_use(L) == base
            failures += 1
        else:
            pytest.fail("fit creation never succeeded")
    finally:
        capi.check(L.kmc_debug_fail_allocation(-1))
    assert failures >= 1
    try:
        capi.check(L.kmc_fit_run(fit))
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    assert _in_use(L) == base
    n_it, lab, C, _, _ = oracle.kmeans_lloyd_driver(X, np.ones(X.shape[1], np.float32), C0, 0.0, 3)
    assert it.value == n_it
    np.testing.assert_array_equal(t["lab"].cpu().numpy(), lab)


def test_driver_surface_raises_on_allocation_failure(kdp):
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, C0 = _data(n=2000, d=8, k=10, seed=7)
    Xg = torch.from_numpy(X).cuda()
    w = torch.ones(X.shape[1], dtype=torch.float32, device="cuda")
    lab = torch.empty(X.shape[1], dtype=torch.int32, device="cuda")
    capi.check(L.kmc_debug_fail_allocation(0))
    try:
        with pytest.raises((RuntimeError, MemoryError)):
            kdp.kmeans_lloyd_driver(Xg, w, torch.from_numpy(C0.copy()).cuda(), lab,
                                    torch.empty_like(torch.from_numpy(C0)).cuda(), 0.0, False, 5, 8,
                                    128, 0.7, None)
    finally:
        capi.check(L.kmc_debug_fail_allocation(-1))
    n_iter, _ = kdp.kmeans_lloyd_driver(Xg, w, torch.from_numpy(C0.copy()).cuda(), lab,
                                        torch.empty_like(torch.from_numpy(C0)).cuda(), 0.0, False, 5,
                                        8, 128, 0.7, None)
    assert n_iter == 5
