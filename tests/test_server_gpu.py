"""The request server (kmc_server_*) on caller buffers.

A mix of fits, predictions and transforms of different sizes is submitted at
once and served together; every result must equal the same request served
alone (bit-equal in the plain form; in the mixed form labels equal the exact
float32 labels and centroids agree within 1e-5), and the plain fits equal the
oracle's driver.  Also: cancellation (pending and running), predictions of a
cancelled model, requests that can never fit the budget, invalid calls.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

FORMS = {"plain": 0, "fp16": 2}
REQ_DONE, REQ_FAILED, REQ_CANCELLED = 2, 3, 4
ERR_INVALID, ERR_OOM, ERR_CANCELLED = 1, 3, 6

# (n, d, k, seed, tol, max_iter)
FITS = [(30_000, 16, 20, 1, 1e-4, 50), (50_000, 8, 5, 2, 0.0, 30), (20_000, 64, 100, 3, 0.0, 8),
        (4_000, 3, 7, 4, 1e-6, 100), (60_000, 32, 256, 5, 0.0, 6), (9_000, 100, 40, 6, 0.0, 5)]


class Req:
    """Device buffers of one request (kept alive until the test ends)."""

    def __init__(self, kind, X, C0=None, model=None, tol=0.0, max_iter=0):
        import torch

        self.kind, self.tol, self.max_iter, self.model = kind, tol, max_iter, model
        self.Xh = X
        self.X = torch.from_numpy(X).cuda()
        d, n = X.shape
        self.n, self.d = n, d
        if kind == 0:
            self.C0h = C0
            self.k = C0.shape[1]
            self.w = torch.ones(n, dtype=torch.float32, device="cuda")
            self.C0 = torch.from_numpy(C0.copy()).cuda()
            self.Cout = torch.full_like(self.C0, np.nan)
        else:
            self.k = model.k
        self.labels = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        self.dist = torch.full((self.k, n), np.nan, dtype=torch.float32, device="cuda") \
            if kind == 2 else None
        self.ticket = None

    def submit(self, L, srv):
        t = ctypes.c_int64()
        if self.kind == 0:
            rc = L.kmc_server_submit_fit_f32(srv, self.X.data_ptr(), self.w.data_ptr(),
                                             self.C0.data_ptr(), self.labels.data_ptr(),
                                             self.Cout.data_ptr(), self.n, self.d, self.k,
                                             self.tol, self.max_iter, ctypes.byref(t))
        elif self.kind == 1:
            rc = L.kmc_server_submit_predict_f32(srv, self.X.data_ptr(), self.model.ticket,
                                                 self.labels.data_ptr(), self.n, ctypes.byref(t))
        else:
            rc = L.kmc_server_submit_transform_f32(srv, self.X.data_ptr(), self.model.ticket,
                                                   self.dist.data_ptr(), self.n, ctypes.byref(t))
        self.ticket = t.value
        return rc

    def result(self):
        out = {"labels": self.labels.cpu().numpy()}
        if self.kind == 0:
            out["C"] = self.Cout.cpu().numpy()
        if self.kind == 2:
            out["dist"] = self.dist.cpu().numpy()
        return out


def _open(L, capi, form, budget=100 * 2 ** 30, max_active=4):
    import torch

    srv = ctypes.c_void_p()
    capi.check(L.kmc_server_open(FORMS[form], budget, max_active,
                                 torch.cuda.current_stream().cuda_stream, ctypes.byref(srv)))
    return srv


def _wait(L, capi, srv, r):
    st, it, inr = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double()
    capi.check(L.kmc_server_wait(srv, r.ticket, ctypes.byref(st), ctypes.byref(it), ctypes.byref(inr)))
    return st.value, it.value, inr.value


def _near_tie(X, C, i, rel=1e-5):
    """Sample i's two nearest centroids are within `rel` of each other (float64)."""
    d2 = ((C.astype(np.float64) - X[:, i].astype(np.float64)[:, None]) ** 2).sum(axis=0)
    a, b = np.sort(d2)[:2]
    return (b - a) <= rel * max(b, 1e-300)


def _requests():
    reqs = []
    for (n, d, k, seed, tol, mi) in FITS:
        X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.0, seed)
        fit = Req(0, X, C0=bench.random_row_init(X, k, seed), tol=tol, max_iter=mi)
        reqs.append(fit)
        Xp, _, _ = bench.make_blobs(n // 3 + 17, d, k, (-10, 10), 1.0, seed + 100)
        reqs.append(Req(1, Xp, model=fit))
        if seed % 2 == 0:
            reqs.append(Req(2, Xp[:, :999].copy(), model=fit))
    return reqs


@pytest.mark.parametrize("form", ["plain", "fp16"])
def test_served_together_equals_served_alone(oracle, form):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    reqs = _requests()
    srv = _open(L, capi, form)
    try:
        for r in reqs:
            capi.check(r.submit(L, srv))
        mixed = []
        for r in reqs:
            st, it, inr = _wait(L, capi, srv, r)
            assert st == 0, (st, L.kmc_last_error().decode())
            mixed.append((it, inr, r.result()))
        pend, run, used = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        capi.check(L.kmc_server_stats(srv, ctypes.byref(pend), ctypes.byref(run), ctypes.byref(used)))
        assert (pend.value, run.value, used.value) == (0, 0, 0)
    finally:
        capi.check(L.kmc_server_close(srv))

    for i, r in enumerate(reqs):
        if r.kind != 0:
            continue
        # the fit alone, then its predictions and transforms alone
        alone_srv = _open(L, capi, form, max_active=1)
        try:
            group = [r] + [q for q in reqs if q.kind != 0 and q.model is r]
            saved = {}
            for q in group:
                capi.check(q.submit(L, alone_srv))
                saved[id(q)] = _wait(L, capi, alone_srv, q) + (q.result(),)
        finally:
            capi.check(L.kmc_server_close(alone_srv))
        C_alone = saved[id(r)][3]["C"]
        for q in group:
            it_m, inr_m, res_m = mixed[reqs.index(q)]
            it_a, inr_a, res_a = saved[id(q)][1], saved[id(q)][2], saved[id(q)][3]
            # plain fits, and mixed fits up to 32 features (float64 sums), give
            # the same bits alone and in the mix; mixed fits beyond 32 features
            # sum in float32 in arrival order
            exact = form == "plain" or q.d <= 32
            if exact:
                assert it_m == it_a, (q.kind, q.n, q.d)
                assert inr_m == inr_a or (form != "plain" and inr_m == pytest.approx(inr_a, rel=1e-12))
                for key in res_m:
                    np.testing.assert_array_equal(res_m[key], res_a[key])
            else:
                assert it_m == it_a
                bad = np.flatnonzero(res_m["labels"] != res_a["labels"])
                assert bad.size <= max(3, q.n // 1000)
                for i in bad:
                    assert _near_tie(q.Xh, C_alone, i)
                if "C" in res_m:
                    np.testing.assert_allclose(res_m["C"], res_a["C"], rtol=1e-5,
                                               atol=1e-5 * np.abs(res_a["C"]).max())
                if "dist" in res_m:
                    np.testing.assert_allclose(res_m["dist"], res_a["dist"], rtol=1e-5, atol=1e-4)
                assert inr_m == pytest.approx(inr_a, rel=1e-5)

    # every fit's labels are the exact assignment against its centroids, and
    # the plain fits follow the oracle's driver
    for i, r in enumerate(reqs):
        it, inr, res = mixed[i]
        if r.kind == 0:
            np.testing.assert_array_equal(res["labels"], oracle.assignment(r.Xh, res["C"]))
            if form == "plain":
                it_o, lab_o, C_o, inr_o, _ = oracle.kmeans_lloyd_driver(
                    r.Xh, np.ones(r.n, np.float32), r.C0h, r.tol, r.max_iter)
                assert it == it_o
                np.testing.assert_array_equal(res["labels"], lab_o)
                np.testing.assert_allclose(res["C"], C_o, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
        elif r.kind == 1:
            C = mixed[reqs.index(r.model)][2]["C"]
            np.testing.assert_array_equal(res["labels"], oracle.assignment(r.Xh, C))
        else:
            C = mixed[reqs.index(r.model)][2]["C"]
            np.testing.assert_array_equal(res["dist"], oracle.distances(r.Xh, C))


@pytest.mark.parametrize("form", ["plain", "fp16"])
def test_cancel_pending_and_running(form):
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    # uniform samples and tol = 0: the fit runs for many iterations
    X = np.random.default_rng(9).uniform(-1, 1, (16, 200_000)).astype(np.float32)
    long_fit = Req(0, X, C0=bench.random_row_init(X, 50, 9), max_iter=100_000)
    pred = Req(1, X[:, :5000].copy(), model=long_fit)
    other = Req(0, X[:, :20000].copy(), C0=bench.random_row_init(X[:, :20000], 10, 3), max_iter=10)
    queued = Req(0, X[:, :20000].copy(), C0=bench.random_row_init(X[:, :20000], 10, 4), max_iter=10)
    srv = _open(L, capi, form, max_active=2)
    try:
        for r in (long_fit, pred, other, queued):
            capi.check(r.submit(L, srv))
        st = ctypes.c_int()
        for _ in range(3):
            capi.check(L.kmc_server_poll(srv, long_fit.ticket, ctypes.byref(st), None, None, None))
        assert st.value == 1                       # running
        capi.check(L.kmc_server_cancel(srv, queued.ticket))   # still pending (2 running)
        capi.check(L.kmc_server_cancel(srv, long_fit.ticket))
        assert _wait(L, capi, srv, long_fit)[0] == ERR_CANCELLED
        assert _wait(L, capi, srv, pred)[0] == ERR_INVALID
        assert _wait(L, capi, srv, queued)[0] == ERR_CANCELLED
        s_other, it_other, _ = _wait(L, capi, srv, other)
        assert s_other == 0 and it_other == 10
        capi.check(L.kmc_server_poll(srv, long_fit.ticket, ctypes.byref(st), None, None, None))
        assert st.value == REQ_CANCELLED
        capi.check(L.kmc_server_cancel(srv, other.ticket))      # finished: no effect
        capi.check(L.kmc_server_poll(srv, other.ticket, ctypes.byref(st), None, None, None))
        assert st.value == REQ_DONE
    finally:
        capi.check(L.kmc_server_close(srv))


def test_budget_and_invalid_calls():
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, _, _ = bench.make_blobs(100_000, 16, 8, (-10, 10), 1.0, 11)
    big = Req(0, X, C0=bench.random_row_init(X, 8, 11), max_iter=5)
    srv = _open(L, capi, "plain", budget=1 << 20)            # 1 MiB: can never fit
    try:
        capi.check(big.submit(L, srv))
        assert _wait(L, capi, srv, big)[0] == ERR_OOM
        t = ctypes.c_int64()
        assert L.kmc_server_submit_predict_f32(srv, big.X.data_ptr(), 12345, big.labels.data_ptr(),
                                               10, ctypes.byref(t)) == ERR_INVALID
        assert L.kmc_server_wait(srv, 999, None, None, None) == ERR_INVALID
        assert L.kmc_server_release(srv, big.ticket) == 0
        assert L.kmc_server_poll(srv, big.ticket, None, None, None, None) == ERR_INVALID
        assert L.kmc_server_submit_fit_f32(srv, big.X.data_ptr(), big.w.data_ptr(), big.C0.data_ptr(),
                                           big.labels.data_ptr(), big.Cout.data_ptr(), 5, 16, 8,
                                           0.0, 5, ctypes.byref(t)) == ERR_INVALID   # k > n
    finally:
        capi.check(L.kmc_server_close(srv))
    bad = ctypes.c_void_p()
    assert L.kmc_server_open(7, 1 << 30, 4, None, ctypes.byref(bad)) == ERR_INVALID


def test_many_concurrent_mixed_sessions_all_finish_and_match_single_fits():
    """Dozens of tensor-core sessions of small, uneven fits run at once (their
    kernels on several streams).  Every fit must finish without a device-side
    wait running out, and up to 32 features (integer cluster sums, the same bits
    in any order) give bit-identical labels and centroids to the same fit run
    alone."""
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    rng = np.random.default_rng(21)
    reqs = []
    for i in range(48):
        n = int(np.exp(rng.uniform(np.log(2_000), np.log(200_000))))
        d = int(rng.choice([8, 16, 32, 64]))
        k = int(min(np.exp(rng.uniform(np.log(4), np.log(160))), n))
        X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.0, 100 + i)
        C0 = np.ascontiguousarray(bench.random_row_init(X, k, 100 + i))
        reqs.append(Req(0, np.ascontiguousarray(X), C0, tol=0.0, max_iter=15))
    srv = _open(L, capi, "fp16", max_active=len(reqs))
    try:
        for r in reqs:
            capi.check(r.submit(L, srv))
        for r in reqs:
            st, it, _ = _wait(L, capi, srv, r)
            assert st == 0, (st, r.n, r.d, r.k, L.kmc_last_error().decode())
    finally:
        capi.check(L.kmc_server_close(srv))
    stream = torch.cuda.current_stream()
    for r in reqs:
        if r.d > 32:
            continue
        C = torch.from_numpy(r.C0h.copy()).cuda()
        res = torch.empty_like(C)
        lab = torch.empty(r.n, dtype=torch.int32, device="cuda")
        fit = ctypes.c_void_p()
        capi.check(L.kmc_fit_create_f32_i32(r.X.data_ptr(), r.w.data_ptr(), C.data_ptr(), lab.data_ptr(),
                                            res.data_ptr(), r.n, r.d, r.k, 0.0, 15, FORMS["fp16"],
                                            stream.cuda_stream, ctypes.byref(fit)))
        try:
            capi.check(L.kmc_fit_run(fit))
            it, inr = ctypes.c_int64(), ctypes.c_double()
            capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
        finally:
            capi.check(L.kmc_fit_destroy(fit))
        out = r.result()
        # integer (fixed-point) cluster sums: the same bits in any order
        np.testing.assert_array_equal(out["labels"], lab.cpu().numpy())
        np.testing.assert_array_equal(out["C"], res.cpu().numpy())
