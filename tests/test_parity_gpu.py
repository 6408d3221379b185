"""GB300 kernels vs the CPU oracle (oracle/kmref.cpp) on seeded inputs.

The plain FP32/FP64 path performs the reference's arithmetic in the same order
(sequential fused multiply-adds over features, strict-< argmin), so labels,
distances, inertia and thresholds must be bit-identical; centroid sums are
accumulated in float64 on both sides and rounded once, so driver trajectories
match too (tolerances below are the bars the comparisons must meet).
"""
import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

RTOL_C = {np.float32: 1e-5, np.float64: 1e-12}


def T(a, dtype=None):
    import torch

    # np.array(copy=True, order="C") keeps 0-d arrays 0-d
    a = np.array(a, dtype=dtype, copy=True, order="C")
    return torch.from_numpy(a).cuda()


def H(t):
    return t.cpu().numpy()


SHAPES = [(1, 3, 1), (7, 1, 2), (129, 17, 31), (1000, 3, 8), (4099, 14, 16), (5000, 64, 129),
          (20000, 14, 127), (3000, 70, 300), (2048, 64, 1024), (777, 2, 5)]


@pytest.mark.parametrize("n,d,k", SHAPES)
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_assignment_bit_exact(kdp, oracle, n, d, k, dt):
    import torch

    rng = np.random.default_rng(n * 31 + d * 7 + k)
    X = rng.standard_normal((d, n)).astype(dt)
    C = rng.standard_normal((d, k)).astype(dt)
    hn = oracle.half_l2_norm_squared(C)
    Xg, Cg = T(X), T(C)
    hg = torch.empty(k, dtype=Xg.dtype, device="cuda")
    kdp.half_l2_norm_squared(Cg, hg, 256, None)[0].wait()
    np.testing.assert_array_equal(H(hg), hn)
    lab = torch.empty(n, dtype=torch.int64, device="cuda")
    kdp.assignment(Xg, Cg, hg, lab, 8, 256, None)[0].wait()
    np.testing.assert_array_equal(H(lab), oracle.assignment(X, C, hn))


def test_assignment_ties_pick_lowest_index(kdp, oracle):
    import torch

    # duplicated centroids: every sample ties between j and j + 4
    rng = np.random.default_rng(3)
    C = rng.standard_normal((5, 4)).astype(np.float32)
    C = np.ascontiguousarray(np.concatenate([C, C], axis=1))
    X = rng.standard_normal((5, 3001)).astype(np.float32)
    hg = torch.empty(8, dtype=torch.float32, device="cuda")
    Cg = T(C)
    kdp.half_l2_norm_squared(Cg, hg, 32, None)[0].wait()
    lab = torch.empty(3001, dtype=torch.int32, device="cuda")
    kdp.assignment(T(X), Cg, hg, lab, 8, 256, None)[0].wait()
    got = H(lab)
    assert got.max() < 4
    np.testing.assert_array_equal(got, oracle.assignment(X, C))


@pytest.mark.parametrize("n,d,k", [(1000, 3, 8), (50000, 14, 16), (20000, 64, 1024), (333, 5, 7)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("weights", ["ones", "random"])
def test_fused_step_parity(kdp, oracle, n, d, k, dt, weights):
    import torch

    rng = np.random.default_rng(n + d + k)
    X = rng.standard_normal((d, n)).astype(dt)
    C = rng.standard_normal((d, k)).astype(dt)
    w = np.ones(n, dt) if weights == "ones" else rng.uniform(0.5, 2.0, n).astype(dt)
    hn = oracle.half_l2_norm_squared(C)
    lab_o, sums_o, sizes_o = oracle.fused_lloyd_single_step(X, w, C, hn)
    P = 3
    lab = torch.empty(n, dtype=torch.int32, device="cuda")
    cc = torch.zeros((P, d, k), dtype=T(X).dtype, device="cuda")
    szc = torch.zeros((P, k), dtype=cc.dtype, device="cuda")
    kdp.fused_lloyd_single_step(T(X), T(w), T(C), T(hn), lab, cc, szc, 8, 256, None)[0].wait()
    np.testing.assert_array_equal(H(lab), lab_o)
    # dataT atomics in arbitrary order: bound the error by the absolute mass
    absmass = np.zeros((d, k))
    np.add.at(absmass.T, lab_o, np.abs(X.T * w[:, None]).astype(np.float64))
    eps = np.finfo(dt).eps
    got_sums = H(cc).astype(np.float64).sum(axis=0)
    assert np.all(np.abs(got_sums - sums_o) <= 4 * n * eps * absmass + 1e-30)
    got_sizes = H(szc).astype(np.float64).sum(axis=0)
    np.testing.assert_allclose(got_sizes, sizes_o, rtol=4 * n * eps)


@pytest.mark.parametrize("n,d,k", [(10, 3, 4), (1000, 14, 16), (4097, 33, 70)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_distances_and_inertia_bit_exact(kdp, oracle, n, d, k, dt):
    import torch

    rng = np.random.default_rng(11 + n)
    X = rng.standard_normal((d, n)).astype(dt)
    C = rng.standard_normal((d, k)).astype(dt)
    dm = torch.empty((k, n), dtype=T(X).dtype, device="cuda")
    kdp.compute_centroid_to_sample_distances(T(X), T(C), dm, 256, 8, None)[0].wait()
    np.testing.assert_array_equal(H(dm), oracle.distances(X, C))
    lab = rng.integers(0, k, n)
    w = rng.uniform(0.5, 2, n).astype(dt)
    out = torch.empty(n, dtype=dm.dtype, device="cuda")
    kdp.compute_inertia(T(X), T(w), T(C), T(lab, np.int64), out, 256, None)[0].wait()
    np.testing.assert_array_equal(H(out), oracle.compute_inertia(X, w, C, lab))
    s = kdp.reduce_vector_blocking(out, None)
    assert s == pytest.approx(oracle.sum_ld(H(out)), rel=np.finfo(dt).eps * 4)


@pytest.mark.parametrize("dt", [np.float32, np.float64])
@pytest.mark.parametrize("topk", [1, 2, 3, 17, 1000, 4096, 4097, 100000])
@pytest.mark.parametrize("ties", [False, True])
def test_threshold_and_select_parity(kdp, oracle, dt, topk, ties):
    import torch

    rng = np.random.default_rng(topk * 3 + ties)
    x = rng.standard_gamma(4, size=100003).astype(dt)
    if ties:
        x = np.round(x, 1).astype(dt)          # many equal values
        x[[5, 77, 9000]] = x.max()              # tie at the top
    thr_o = oracle.compute_threshold(x, topk)
    xg = T(x)
    thr = torch.empty((), dtype=xg.dtype, device="cuda")
    kdp.compute_threshold(xg, topk, thr, None)[0].wait()
    assert H(thr).item() == float(thr_o)
    sel = T(np.full(x.size, -5), np.int64)
    ngt, neq = T(np.zeros(()), np.int64), T(np.ones(()), np.int64)
    kdp.select_samples_far_from_centroid(topk, xg, thr, sel, ngt, neq, 256, None)[0].wait()
    sel_o, ng_o, nq_o = oracle.select_samples_far_from_centroid(topk, x, thr_o, fill=-5)
    assert (H(ngt).item(), H(neq).item()) == (ng_o, nq_o)
    np.testing.assert_array_equal(H(sel), sel_o)


def test_select_many_samples_is_fast_and_exact(kdp, oracle):
    """300,000 selections out of 2M samples: the strictly-greater samples are ranked by a
    merge sort (O(m log^2 m)), not by counting all pairs (~10^11 compares here)."""
    import time

    import torch

    rng = np.random.default_rng(12)
    x = np.round(rng.standard_gamma(4, size=2_000_000), 2).astype(np.float32)
    topk = 300_000
    thr_o = oracle.compute_threshold(x, topk)
    xg, thr = T(x), T(np.array(thr_o, np.float32))
    sel = T(np.full(x.size, -5), np.int32)
    ngt, neq = T(np.zeros(()), np.int32), T(np.ones(()), np.int32)
    kdp.select_samples_far_from_centroid(topk, xg, thr, sel, ngt, neq, 256, None)[0].wait()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(3):
        sel.fill_(-5)
        ngt.fill_(0)
        neq.fill_(1)
        kdp.select_samples_far_from_centroid(topk, xg, thr, sel, ngt, neq, 256, None)[0].wait()
    torch.cuda.synchronize()
    per_call = (time.perf_counter() - t0) / 3
    sel_o, ng_o, nq_o = oracle.select_samples_far_from_centroid(topk, x, thr_o, fill=-5)
    assert (H(ngt).item(), H(neq).item()) == (ng_o, nq_o)
    assert ng_o > 4096                           # the merge-sort path ran
    np.testing.assert_array_equal(H(sel), sel_o)
    assert per_call < 0.25, per_call


@pytest.mark.parametrize("n_empty", [1, 2, 3, 5])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_relocate_parity(kdp, oracle, n_empty, dt):
    rng = np.random.default_rng(n_empty)
    n, d, k = 5000, 6, 12
    X = rng.standard_normal((d, n)).astype(dt)
    w = rng.uniform(0.5, 2, n).astype(dt)
    lab = rng.integers(0, k - n_empty, n)
    C = rng.standard_normal((d, k)).astype(dt)
    sq = oracle.compute_inertia(X, None, C, lab)
    sq[[10, 20, 30]] = sq.max()               # ties at the top
    sums = np.zeros((d, k), dt)
    sizes = np.zeros(k, dt)
    np.add.at(sums.T, lab, (X.T * w[:, None]).astype(dt))
    np.add.at(sizes, lab, w)
    empty = np.full(k, -1)
    empty[:n_empty] = np.arange(k - n_empty, k)
    C_o, sz_o, inr_o = oracle.relocate_empty_clusters(n_empty, X, w, lab, empty, sq, sums, sizes, sq)
    Cg, szg, inrg = T(sums), T(sizes), T(sq)
    kdp.relocate_empty_clusters(n_empty, T(X), T(w), T(lab, np.int32), T(empty, np.int32), T(sq),
                                Cg, szg, inrg, 256, None)[0].wait()
    np.testing.assert_array_equal(H(Cg), C_o)
    np.testing.assert_array_equal(H(szg), sz_o)
    np.testing.assert_array_equal(H(inrg), inr_o)


def _run_driver(kdp, X, C0, tol, max_iter, it=np.int32):
    import torch

    d, n = X.shape
    k = C0.shape[1]
    Xg = T(X)
    init = T(C0)
    res_c = torch.empty_like(init)
    lab = torch.empty(n, dtype=torch.int32 if it == np.int32 else torch.int64, device="cuda")
    w = torch.ones(n, dtype=Xg.dtype, device="cuda")
    n_iter, inertia = kdp.kmeans_lloyd_driver(Xg, w, init, lab, res_c, tol, False, max_iter, 8, 128,
                                              0.7, None)
    return n_iter, H(lab), H(res_c), float(inertia[0])


DRIVER_CASES = {
    # name: (n, d, centers, k, box, std, seed, tol, max_iter, far_first)
    "c1_50k_d14_k16": (50_000, 14, 16, 16, (-10, 10), 1.0, 0, 1e-4, 100, False),
    "c2_small_forced_empty": (200_000, 14, 127, 127, (-10, 10), 1.5, 1, 0.0, 12, True),
    "d64_k256": (60_000, 64, 256, 256, (-5, 5), 1.0, 2, 0.0, 6, False),
    "more_clusters_than_blobs": (30_000, 5, 4, 40, (-10, 10), 1.0, 3, 1e-6, 30, False),
    # zero tolerance, converging long before max_iter: the stop needs a centroid
    # shift of exactly zero once the labels settle
    "converges_tol0": (300_000, 3, 6, 6, (-10, 10), 0.7, 5, 0.0, 200, False),
}


@pytest.mark.parametrize("case", sorted(DRIVER_CASES))
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_driver_parity(kdp, oracle, case, dt):
    n, d, centers, k, box, std, seed, tol, max_iter, far = DRIVER_CASES[case]
    X, _, _ = bench.make_blobs(n, d, centers, box, std, seed, dtype=dt)
    C0 = bench.random_row_init(X, k, seed, far_first=far)
    it_o, lab_o, C_o, inr_o, rel_o = oracle.kmeans_lloyd_driver(X, np.ones(n, dt), C0, tol, max_iter)
    it_g, lab_g, C_g, inr_g = _run_driver(kdp, X, C0, tol, max_iter)
    assert it_g == it_o
    np.testing.assert_array_equal(lab_g, lab_o)
    np.testing.assert_allclose(C_g, C_o, rtol=RTOL_C[dt], atol=RTOL_C[dt] * np.abs(C_o).max())
    assert inr_g == pytest.approx(inr_o, rel=RTOL_C[dt])
    if far:
        assert rel_o >= 1  # the forced empty cluster was relocated


def test_driver_full_size_float64_fixed_point(kdp, oracle):
    """5M x 14, k = 127 in float64 (the at-scale workload, centroid 0 forced empty), tol = 0,
    max_iter = 100: two runs give the same iteration count and the same bits; labels are the
    exact argmin against the returned centroids (20k subset); the inertia equals the float64
    sum of per-sample inertia; and if the fit stopped early, one more iteration from its
    centroids leaves them unchanged (an exactly zero shift, the reference's stop)."""
    n, d, k = 5_000_000, 14, 127
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.5, 1, dtype=np.float64)
    C0 = bench.random_row_init(X, k, 1, far_first=True)
    it, lab, C, inr = _run_driver(kdp, X, C0, 0.0, 100)
    it2, lab2, C2, inr2 = _run_driver(kdp, X, C0, 0.0, 100)
    assert it == it2 and inr == inr2
    np.testing.assert_array_equal(lab, lab2)
    np.testing.assert_array_equal(C, C2)
    sub = np.random.default_rng(0).choice(n, 20_000, replace=False)
    np.testing.assert_array_equal(lab[sub], oracle.assignment(np.ascontiguousarray(X[:, sub]), C))
    assert np.bincount(lab, minlength=k).sum() == n
    per = oracle.compute_inertia(X, np.ones(n), C, lab)
    assert inr == pytest.approx(oracle.sum_ld(per), rel=1e-12)
    if it < 100:
        it3, _, C3, _ = _run_driver(kdp, X, C, 0.0, 1)
        assert it3 == 1
        np.testing.assert_array_equal(C3, C)


def test_driver_float64_reproducible(kdp):
    """float64 fits sum each CTA's samples in a fixed order: two runs of the same fit give
    the same bits, and a zero tolerance stops once the labels settle."""
    X, _, _ = bench.make_blobs(400_000, 5, 20, (-10, 10), 1.0, 11, dtype=np.float64)
    C0 = bench.random_row_init(X, 20, 11)
    r1 = _run_driver(kdp, X, C0, 0.0, 300)
    r2 = _run_driver(kdp, X, C0, 0.0, 300)
    assert r1[0] == r2[0] < 300
    np.testing.assert_array_equal(r1[1], r2[1])
    np.testing.assert_array_equal(r1[2], r2[2])
    assert r1[3] == r2[3]


@pytest.mark.parametrize("n,d,k", [(5, 3, 8), (1, 2, 3), (40, 1, 1), (3, 4, 3)])
def test_driver_edge_cases(kdp, oracle, n, d, k):
    rng = np.random.default_rng(n * 10 + k)
    X = rng.standard_normal((d, n)).astype(np.float64)
    C0 = rng.standard_normal((d, k)).astype(np.float64)
    it_o, lab_o, C_o, inr_o, _ = oracle.kmeans_lloyd_driver(X, np.ones(n), C0, 0.0, 5)
    it_g, lab_g, C_g, inr_g = _run_driver(kdp, X, C0, 0.0, 5, it=np.int64)
    assert it_g == it_o
    np.testing.assert_array_equal(lab_g, lab_o)
    # clusters emptied by relocation divide a cancelled sum by zero: NaN or an
    # inf whose sign depends on summation order -- only finite entries compare
    np.testing.assert_array_equal(np.isfinite(C_g), np.isfinite(C_o))
    ok = np.isfinite(C_o)
    np.testing.assert_allclose(C_g[ok], C_o[ok], rtol=1e-12)


def test_driver_zero_iterations_copies_init(kdp):
    X = np.random.default_rng(0).standard_normal((3, 100)).astype(np.float32)
    C0 = np.ascontiguousarray(X[:, :4])
    it, lab, C, inr = _run_driver(kdp, X, C0, 0.0, 0)
    assert it == 0
    np.testing.assert_array_equal(C, C0)


def test_driver_verbose_prints(kdp, capsys):
    X, _, _ = bench.make_blobs(2000, 3, 4, (-5, 5), 0.5, 9)
    C0 = bench.random_row_init(X, 4, 9)
    import torch

    Xg, init = T(X), T(C0)
    res_c = torch.empty_like(init)
    lab = torch.empty(2000, dtype=torch.int32, device="cuda")
    w = torch.ones(2000, dtype=torch.float32, device="cuda")
    n_iter, _ = kdp.kmeans_lloyd_driver(Xg, w, init, lab, res_c, 0.0, True, 3, 8, 128, 0.7, None)
    out = capsys.readouterr().out
    lines = [ln for ln in out.splitlines() if ln.startswith("Iteration: ")]
    assert len(lines) == n_iter == 3
    assert lines[0].startswith("Iteration: 0 Inertia: ")


def test_driver_full_size_properties(kdp, oracle):
    """5M x 14, k = 127 (the at-scale float32 workload, 10 iterations): labels are the exact
    argmin against the returned centroids (checked by the oracle on a 20k subset), cluster
    masses add up, and the returned inertia equals the float64 sum of per-sample inertia."""
    import torch

    n, d, k = 5_000_000, 14, 127
    X, _, _ = bench.make_blobs(n, d, k, (-10, 10), 1.5, 1)
    C0 = bench.random_row_init(X, k, 1, far_first=True)
    it, lab, C, inr = _run_driver(kdp, X, C0, 0.0, 10)
    assert it == 10
    sub = np.random.default_rng(0).choice(n, 20_000, replace=False)
    np.testing.assert_array_equal(lab[sub], oracle.assignment(np.ascontiguousarray(X[:, sub]), C))
    assert np.bincount(lab, minlength=k).sum() == n
    per = oracle.compute_inertia(X, np.ones(n, np.float32), C, lab)
    assert inr == pytest.approx(oracle.sum_ld(per), rel=1e-6)
    del torch
