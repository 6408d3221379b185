"""Initialisation, row-major input and the KMeans estimator (GPU).

k-means++ seeding on the device is deterministic for a seed and selects
exactly the rows of the oracle's sequential restatement; the estimator's fit
equals the oracle driver run from the same initial centroids with tol scaled
by the mean per-feature variance.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu


def _lib():
    from kmeans_dpcpp_gb300 import capi

    return capi, capi.lib()


def _dev(a):
    import torch

    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _stream():
    import torch

    return torch.cuda.current_stream().cuda_stream


@pytest.mark.parametrize("n,d", [(1, 1), (33, 7), (1000, 64), (4097, 129), (70000, 3)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_transpose_matches_numpy(n, d, dt):
    capi, L = _lib()
    X = np.random.default_rng(n + d).standard_normal((n, d)).astype(dt)
    Xg = _dev(X)
    out = _dev(np.zeros((d, n), dt))
    suf = "f32" if dt == np.float32 else "f64"
    capi.check(getattr(L, f"kmc_transpose_{suf}")(Xg.data_ptr(), out.data_ptr(), n, d, _stream()))
    np.testing.assert_array_equal(out.cpu().numpy(), X.T)


def test_gather_rows_and_rejects_out_of_range():
    capi, L = _lib()
    Xt = np.random.default_rng(1).standard_normal((5, 100)).astype(np.float32)
    rows = np.array([3, 99, 0, 42], np.int32)
    Xg, rg = _dev(Xt), _dev(rows)   # device arrays must outlive the calls
    C = _dev(np.zeros((5, 4), np.float32))
    capi.check(L.kmc_gather_rows_f32(Xg.data_ptr(), 100, 5, rg.data_ptr(), 4, C.data_ptr(), _stream()))
    np.testing.assert_array_equal(C.cpu().numpy(), Xt[:, rows])
    bad = _dev(np.array([3, 100], np.int32))
    assert L.kmc_gather_rows_f32(Xg.data_ptr(), 100, 5, bad.data_ptr(), 2, C.data_ptr(), _stream()) == 1


@pytest.mark.parametrize("n,d,k,seed,weighted", [(5000, 14, 16, 7, False), (20000, 64, 100, 8, True),
                                                 (9000, 3, 300, 9, False), (4096 * 3 + 5, 8, 40, 10, True)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_kmeans_plusplus_selects_the_oracles_rows(oracle, n, d, k, seed, weighted, dt):
    capi, L = _lib()
    X, _, _ = bench.make_blobs(n, d, max(2, k // 2), (-10, 10), 1.0, seed)
    X = X.astype(dt)
    w = np.random.default_rng(seed).uniform(0.5, 2.0, n).astype(dt) if weighted else None
    rows_o, C_o = oracle.kmeans_plusplus(X, k, seed, w)
    suf = "f32" if dt == np.float32 else "f64"
    Xg = _dev(X)
    wg = _dev(w) if weighted else None
    C = _dev(np.zeros((d, k), dt))
    rows = _dev(np.zeros(k, np.int32))
    capi.check(getattr(L, f"kmc_kmeans_plusplus_{suf}")(Xg.data_ptr(), wg.data_ptr() if weighted else None,
                                                        n, d, k, seed, C.data_ptr(), rows.data_ptr(), _stream()))
    np.testing.assert_array_equal(rows.cpu().numpy(), rows_o)
    np.testing.assert_array_equal(C.cpu().numpy(), C_o)
    assert len(set(rows_o.tolist())) == k


def test_mean_feature_variance():
    capi, L = _lib()
    Xt = np.random.default_rng(3).normal(2.0, 3.0, (6, 50001)).astype(np.float32)
    out = ctypes.c_double()
    Xg = _dev(Xt)
    capi.check(L.kmc_mean_feature_variance_f32(Xg.data_ptr(), 50001, 6, ctypes.byref(out), _stream()))
    assert out.value == pytest.approx(float(np.mean(np.var(Xt.astype(np.float64), axis=1))), rel=1e-10)


@pytest.mark.parametrize("tol,max_iter", [(1e-4, 100), (0.0, 7)])
def test_estimator_fit_equals_oracle_driver(oracle, tol, max_iter):
    from kmeans_dpcpp_gb300 import KMeans

    X_t, _, _ = bench.make_blobs(30000, 10, 12, (-10, 10), 1.0, 21)
    C0 = bench.random_row_init(X_t, 12, 21)
    X = np.ascontiguousarray(X_t.T)
    km = KMeans(12, init=C0.T.copy(), tol=tol, max_iter=max_iter).fit(X)
    tol_abs = np.mean(np.var(X_t.astype(np.float64), axis=1)) * tol
    it_o, lab_o, C_o, inr_o, _ = oracle.kmeans_lloyd_driver(X_t, np.ones(30000, np.float32), C0, tol_abs,
                                                            max_iter)
    assert km.n_iter_ == it_o
    np.testing.assert_array_equal(km.labels_, lab_o)
    np.testing.assert_allclose(km.cluster_centers_, C_o.T, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
    assert km.inertia_ == pytest.approx(inr_o, rel=1e-5)
    np.testing.assert_array_equal(km.predict(X), oracle.assignment(X_t, km.cluster_centers_.T.copy()))
    dist = km.transform(X[:500])
    ref = np.sqrt(np.maximum(0.0, ((X[:500, None, :].astype(np.float64)
                                    - km.cluster_centers_[None].astype(np.float64)) ** 2).sum(-1)))
    np.testing.assert_allclose(dist, ref, rtol=1e-4, atol=1e-4)
    assert km.score(X) == pytest.approx(-km.inertia_, rel=1e-5)


def test_estimator_kmeans_plusplus_is_deterministic_and_n_init_keeps_the_best():
    from kmeans_dpcpp_gb300 import KMeans

    X_t, _, _ = bench.make_blobs(20000, 8, 20, (-10, 10), 1.0, 5)
    X = np.ascontiguousarray(X_t.T)
    a = KMeans(20, random_state=3, max_iter=50).fit(X)
    b = KMeans(20, random_state=3, max_iter=50).fit(X)
    np.testing.assert_array_equal(a.labels_, b.labels_)
    assert a.inertia_ == b.inertia_
    best = KMeans(20, random_state=3, n_init=4, max_iter=50).fit(X)
    assert best.inertia_ <= a.inertia_ * (1 + 1e-12)
    r = KMeans(20, init="random", random_state=1, max_iter=50).fit(X)
    assert r.cluster_centers_.shape == (20, 8) and r.n_iter_ >= 1


def test_estimator_mixed_form_and_float64():
    from kmeans_dpcpp_gb300 import KMeans

    X_t, _, _ = bench.make_blobs(40000, 32, 50, (-5, 5), 1.0, 6)
    X = np.ascontiguousarray(X_t.T)
    C0 = np.ascontiguousarray(X[:50])
    plain = KMeans(50, init=C0, tol=0.0, max_iter=5).fit(X)
    mixed = KMeans(50, init=C0, tol=0.0, max_iter=5, form="mixed-fp16").fit(X)
    assert mixed.n_iter_ == plain.n_iter_ == 5
    assert mixed.inertia_ == pytest.approx(plain.inertia_, rel=1e-5)
    f64 = KMeans(50, init=C0.astype(np.float64), tol=0.0, max_iter=5).fit(X.astype(np.float64))
    assert f64.cluster_centers_.dtype == np.float64
    assert f64.inertia_ == pytest.approx(plain.inertia_, rel=1e-4)
