"""Batched fits and the serving loop against single fits and the oracle.

A batched fit follows kmeans_lloyd_driver's semantics with the plain form's
arithmetic, so its labels equal a single plain fit's; centroids and inertia
agree up to the order of float64 additions (1e-6 relative here).  A request
served in a mix of others gives the same result as served alone.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


def _lib():
    from kmeans_dpcpp_gb300 import capi

    return capi, capi.lib()


def _single_fit(X, C0, tol, max_iter):
    import torch

    capi, L = _lib()
    d, n = X.shape
    k = C0.shape[1]
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    w = torch.ones(n, dtype=torch.float32, device="cuda")
    cur = torch.from_numpy(np.ascontiguousarray(C0).copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, tol, max_iter, 0, stream.cuda_stream,
                                        ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_run(fit))
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    return it.value, lab.cpu().numpy(), res.cpu().numpy(), inr.value


class Batch:
    def __init__(self, cap=64):
        import torch

        self.capi, self.L = _lib()
        self.stream = torch.cuda.current_stream()
        self.h = ctypes.c_void_p()
        self.capi.check(self.L.kmc_batch_create(cap, self.stream.cuda_stream, ctypes.byref(self.h)))
        self.keep = {}

    def add_fit(self, X, C0, tol, max_iter):
        import torch

        d, n = X.shape
        k = C0.shape[1]
        Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        w = torch.ones(n, dtype=torch.float32, device="cuda")
        C = torch.from_numpy(np.ascontiguousarray(C0).copy()).cuda()
        lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        inst = ctypes.c_int64()
        self.capi.check(self.L.kmc_batch_add_fit_f32(self.h, Xg.data_ptr(), w.data_ptr(), C.data_ptr(),
                                                     lab.data_ptr(), n, d, k, tol, max_iter,
                                                     ctypes.byref(inst)))
        self.keep[inst.value] = (Xg, w, C, lab)
        return inst.value

    def add_predict(self, X, C):
        import torch

        d, n = X.shape
        k = C.shape[1]
        Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
        Cg = torch.from_numpy(np.ascontiguousarray(C)).cuda()
        lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        inst = ctypes.c_int64()
        self.capi.check(self.L.kmc_batch_add_predict_f32(self.h, Xg.data_ptr(), Cg.data_ptr(),
                                                         lab.data_ptr(), n, d, k, ctypes.byref(inst)))
        self.keep[inst.value] = (Xg, None, Cg, lab)
        return inst.value

    def run(self):
        self.capi.check(self.L.kmc_batch_run(self.h))
        self.stream.synchronize()

    def result(self, inst):
        fin, it, inr = ctypes.c_int(), ctypes.c_int64(), ctypes.c_double()
        self.capi.check(self.L.kmc_batch_result(self.h, inst, ctypes.byref(fin), ctypes.byref(it),
                                                ctypes.byref(inr)))
        _, _, C, lab = self.keep[inst]
        return bool(fin.value), it.value, lab.cpu().numpy(), C.cpu().numpy(), inr.value

    def stats(self):
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self.capi.check(self.L.kmc_batch_stats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def close(self):
        self.capi.check(self.L.kmc_batch_destroy(self.h))


# (n, d, centers, k, seed, tol, max_iter, far_first)
CASES = [(3000, 3, 8, 8, 11, 0.0, 12, False), (20000, 14, 16, 16, 0, 1e-4, 100, False),
         (6000, 14, 40, 40, 1, 0.0, 10, True), (12345, 33, 60, 100, 3, 0.0, 6, False),
         (4096, 64, 200, 300, 4, 0.0, 4, False), (700, 130, 5, 9, 5, 0.0, 8, False),
         (50000, 8, 4, 4, 6, 1e-3, 50, False)]


def _case_data(case):
    n, d, centers, k, seed, tol, max_iter, far = case
    X, _, _ = bench.make_blobs(n, d, centers, (-10, 10), 1.0, seed)
    C0 = bench.random_row_init(X, k, seed, far_first=far)
    return X, C0, tol, max_iter


def test_batched_fits_equal_single_plain_fits():
    data = [_case_data(c) for c in CASES]
    b = Batch()
    try:
        ids = [b.add_fit(X, C0, tol, mi) for X, C0, tol, mi in data]
        b.run()
        steps, builds, relocs = b.stats()
        assert relocs >= 1          # the far-first case empties a cluster
        assert builds >= 2          # the graph is rebuilt as fits finish
        for inst, (X, C0, tol, mi) in zip(ids, data):
            fin, it, lab, C, inr = b.result(inst)
            it_s, lab_s, C_s, inr_s = _single_fit(X, C0, tol, mi)
            assert fin and it == it_s
            np.testing.assert_array_equal(lab, lab_s)
            np.testing.assert_allclose(C, C_s, rtol=1e-6, atol=1e-6 * np.abs(C_s).max())
            assert inr == pytest.approx(inr_s, rel=1e-6)
    finally:
        b.close()


def test_batched_fit_tracks_oracle(oracle):
    X, C0, tol, mi = _case_data(CASES[1])
    it_o, lab_o, C_o, inr_o, _ = oracle.kmeans_lloyd_driver(X, np.ones(X.shape[1], np.float32), C0, tol, mi)
    b = Batch()
    try:
        inst = b.add_fit(X, C0, tol, mi)
        b.run()
        fin, it, lab, C, inr = b.result(inst)
    finally:
        b.close()
    assert fin and it == it_o
    np.testing.assert_array_equal(lab, lab_o)
    np.testing.assert_allclose(C, C_o, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
    assert inr == pytest.approx(inr_o, rel=1e-5)


def test_batched_predictions_equal_oracle_assignment(oracle):
    rng = np.random.default_rng(9)
    b = Batch()
    try:
        cases = []
        for n, d, k in [(1000, 5, 7), (33333, 64, 513), (257, 129, 33)]:
            X = rng.standard_normal((d, n)).astype(np.float32)
            C = rng.standard_normal((d, k)).astype(np.float32)
            cases.append((b.add_predict(X, C), X, C))
        b.run()
        for inst, X, C in cases:
            fin, it, lab, _, _ = b.result(inst)
            assert fin and it == 0
            np.testing.assert_array_equal(lab, oracle.assignment(X, C))
    finally:
        b.close()


def test_result_is_the_same_alone_and_in_the_mix():
    X, C0, tol, mi = _case_data(CASES[3])
    alone = Batch()
    try:
        a = alone.add_fit(X, C0, tol, mi)
        alone.run()
        r_alone = alone.result(a)
    finally:
        alone.close()
    mix = Batch()
    try:
        others = [_case_data(c) for c in CASES[:3]]
        for Xo, Co, to, mo in others[:2]:
            mix.add_fit(Xo, Co, to, mo)
        m = mix.add_fit(X, C0, tol, mi)
        mix.add_fit(*others[2])
        mix.run()
        r_mix = mix.result(m)
    finally:
        mix.close()
    assert r_alone[1] == r_mix[1]
    np.testing.assert_array_equal(r_alone[2], r_mix[2])
    np.testing.assert_allclose(r_alone[3], r_mix[3], rtol=1e-6, atol=1e-6 * np.abs(r_alone[3]).max())
    assert r_alone[4] == pytest.approx(r_mix[4], rel=1e-9)


def test_tile_autotuner_is_cached():
    import torch

    capi, L = _lib()
    v1, v2 = ctypes.c_int(), ctypes.c_int()
    s = torch.cuda.current_stream().cuda_stream
    capi.check(L.kmc_tile_variant(24, 40, s, ctypes.byref(v1)))
    capi.check(L.kmc_tile_variant(24, 37, s, ctypes.byref(v2)))   # same power-of-two bucket
    assert v1.value in (0, 1, 2) and v2.value == v1.value


def _requests(spec):
    """spec: list of (arrival, kind, n, d, k, seed, tol, max_iter, model)."""
    from kmeans_dpcpp_gb300 import capi

    arr = (capi.ServeRequest * len(spec))()
    for r, (t, kind, n, d, k, seed, tol, mi, model) in enumerate(spec):
        arr[r] = capi.ServeRequest(t, kind, d, n, k, max(2, k // 2) if kind == 0 else 2, seed, tol, mi,
                                   model, 0.5, 1.5)
    return arr


def _serve(spec, form, budget=150 * 2 ** 30, max_active=64):
    import torch

    capi, L = _lib()
    reqs = _requests(spec)
    res = (capi.ServeResult * len(spec))()
    mk = ctypes.c_double()
    capi.check(L.kmc_serve_run(reqs, len(spec), form, budget, max_active,
                               torch.cuda.current_stream().cuda_stream, res, ctypes.byref(mk)))
    return list(res), mk.value


SPEC = [(0.000, 0, 20000, 16, 24, 1, 1e-4, 300, -1),
        (0.005, 0, 5000, 32, 100, 2, 1e-4, 300, -1),
        (0.010, 0, 80000, 64, 300, 3, 0.0, 60, -1),
        (0.012, 1, 3000, 16, 24, 4, 0.0, 0, 0),
        (0.020, 0, 12000, 16, 8, 5, 1e-4, 300, -1),
        (0.030, 1, 9000, 64, 300, 6, 0.0, 0, 2),
        (0.031, 0, 40000, 32, 700, 7, 1e-4, 40, -1)]


@pytest.mark.parametrize("form", [0, 2])
def test_serving_loop_matches_requests_served_alone(form):
    mixed, _ = _serve(SPEC, form)
    for r, out in enumerate(mixed):
        assert out.status == 0, r
        assert out.admit_s >= SPEC[r][0] - 1e-6 and out.finish_s >= out.admit_s
        if SPEC[r][1] == 0:
            assert out.n_iter >= 1
    # every fit alone (a fresh replay with only that request) gives the same
    # fit: float64-order differences for the plain engine; the tensor-core
    # sessions reduce d > 32 sums in float32 arrival order
    rel = 1e-6 if form == 0 else 1e-5
    for r, s in enumerate(SPEC):
        if s[1] != 0:
            continue
        alone, _ = _serve([(0.0,) + s[1:]], form)
        assert alone[0].n_iter == mixed[r].n_iter
        assert alone[0].inertia == pytest.approx(mixed[r].inertia, rel=rel)


def _served_fit_direct(spec_row, form):
    """The fit a request describes, run as a direct fit session on the same
    device-generated blobs and seeded initial rows the serving loop uses."""
    import torch

    capi, L = _lib()
    _, kind, n, d, k, seed, tol, mi, _ = spec_row
    req = _requests([spec_row])[0]
    s = torch.cuda.current_stream()
    X = torch.empty((d, n), dtype=torch.float32, device="cuda")
    capi.check(L.kmc_generate_blobs_f32(X.data_ptr(), n, d, req.n_centers, -10.0, 10.0, req.std_lo,
                                        req.std_hi, seed, s.cuda_stream))
    rows = (ctypes.c_int32 * k)()
    capi.check(L.kmc_seeded_rows(n, k, seed ^ 0x9999, rows))
    cur = X[:, torch.tensor(list(rows), dtype=torch.int64, device="cuda")].contiguous()
    res = torch.empty_like(cur)
    w = torch.ones(n, dtype=torch.float32, device="cuda")
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(X.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, tol, mi, form, s.cuda_stream,
                                        ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_run(fit))
        it, inr = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    return it.value, inr.value


def test_mixed_serving_equals_direct_fit_sessions():
    """The tensor-core serving sessions (one captured iteration replayed per visit, results
    read back without host waits) give the fits a direct session gives; up to 32
    features their sums are float64, so iteration counts match exactly."""
    mixed, _ = _serve(SPEC, 2)
    for r, row in enumerate(SPEC):
        if row[1] != 0 or row[3] > 32:
            continue
        it, inr = _served_fit_direct(row, 2)
        assert mixed[r].status == 0
        assert mixed[r].n_iter == it, r
        assert mixed[r].inertia == pytest.approx(inr, rel=1e-6), r


def test_serving_admission_respects_the_memory_budget():
    from kmeans_dpcpp_gb300 import capi

    _, L = _lib()
    spec = [(0.0, 0, 30000, 16, 16, 10 + r, 1e-4, 300, -1) for r in range(4)]
    need = ctypes.c_int64()
    capi.check(L.kmc_serve_bytes_needed(0, 30000, 16, 16, 0, ctypes.byref(need)))
    res, _ = _serve(spec, 0, budget=int(need.value * 1.5))   # room for one at a time
    order = sorted(range(4), key=lambda r: res[r].admit_s)
    for a, b in zip(order, order[1:]):
        assert res[b].admit_s >= res[a].finish_s - 1e-6
    assert all(r.status == 0 for r in res)


def _distances_single(X, C):
    import torch

    capi, L = _lib()
    d, n = X.shape
    k = C.shape[1]
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    Cg = torch.from_numpy(np.ascontiguousarray(C)).cuda()
    out = torch.empty((k, n), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    capi.check(L.kmc_compute_centroid_to_sample_distances_f32(Xg.data_ptr(), Cg.data_ptr(),
                                                              out.data_ptr(), n, d, k, 256, 128,
                                                              s.cuda_stream))
    s.synchronize()
    return out.cpu().numpy()


def test_batched_transforms_equal_single_distance_calls(oracle):
    """Transform instances run through the persistent tiles beside fits and
    predictions; their distances are bit-equal to the single-call kernel's
    and match the oracle's."""
    import torch

    rng = np.random.default_rng(21)
    b = Batch()
    try:
        outs = []
        fitX, fitC, tol, mi = _case_data(CASES[0])
        b.add_fit(fitX, fitC, tol, mi)
        for n, d, k in [(1000, 5, 7), (20001, 64, 300), (257, 129, 33), (4096, 16, 1024)]:
            X = rng.standard_normal((d, n)).astype(np.float32)
            C = rng.standard_normal((d, k)).astype(np.float32)
            Xg = torch.from_numpy(X).cuda()
            Cg = torch.from_numpy(C).cuda()
            D = torch.full((k, n), -1.0, dtype=torch.float32, device="cuda")
            inst = ctypes.c_int64()
            b.capi.check(b.L.kmc_batch_add_transform_f32(b.h, Xg.data_ptr(), Cg.data_ptr(),
                                                         D.data_ptr(), n, d, k, ctypes.byref(inst)))
            b.keep[inst.value] = (Xg, None, Cg, D)
            outs.append((inst.value, X, C, D))
            if n == 257:
                b.add_predict(X, C)
        b.run()
        for inst, X, C, D in outs:
            fin, it, _, _, _ = b.result(inst)
            assert fin and it == 0
            got = D.cpu().numpy()
            np.testing.assert_array_equal(got, _distances_single(X, C))
            np.testing.assert_array_equal(got, oracle.distances(X, C))
    finally:
        b.close()


@pytest.mark.parametrize("form", [0, 2])
def test_serving_transforms_match_transforms_served_alone(form):
    """Transform requests (kind 2) in a mix of fits and predictions give the
    float64 total of their distance matrix that the same request gives when
    served right after its model alone."""
    spec = SPEC + [(0.032, 2, 7000, 16, 24, 8, 0.0, 0, 0),
                   (0.033, 2, 3000, 64, 300, 9, 0.0, 0, 2),
                   (0.034, 1, 2000, 16, 8, 10, 0.0, 0, 4)]
    mixed, _ = _serve(spec, form)
    assert all(o.status == 0 for o in mixed)
    for r, s in enumerate(spec):
        if s[1] != 2:
            continue
        assert mixed[r].n_iter == 0 and mixed[r].inertia > 0
        fit = (0.0,) + spec[s[8]][1:]
        alone, _ = _serve([fit, (0.0,) + s[1:8] + (0,)], form)
        assert alone[1].status == 0
        assert alone[1].inertia == pytest.approx(mixed[r].inertia, rel=1e-5)


def test_serving_sizes_transform_requests():
    from kmeans_dpcpp_gb300 import capi

    _, L = _lib()
    a, b = ctypes.c_int64(), ctypes.c_int64()
    capi.check(L.kmc_serve_bytes_needed(1, 100000, 32, 256, 0, ctypes.byref(a)))
    capi.check(L.kmc_serve_bytes_needed(2, 100000, 32, 256, 0, ctypes.byref(b)))
    assert b.value >= a.value + 4 * 100000 * 256
