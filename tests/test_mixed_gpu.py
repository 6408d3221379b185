"""Mixed tensor-core forms (fp16 / bf16 operands, fp32 accumulation) vs the oracle.

Labels from one mixed assignment pass must equal the exact reference labels
for every sample: samples whose tensor-core margin does not certify them are
re-evaluated in exact float32.  Full fits are compared with tolerances: labels
identical except for samples whose top-two relative gap is below 1e-5,
centroids and inertia within 1e-5 relative.
"""
import ctypes

import numpy as np
import pytest

import bench

pytestmark = pytest.mark.gpu

FORMS = {"fp16": 2, "bf16": 1}


def _fit_labels(X, C0, form, max_iter=0, tol=0.0):
    import torch

    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    d, n = X.shape
    k = C0.shape[1]
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    w = torch.ones(n, dtype=torch.float32, device="cuda")
    cur = torch.from_numpy(np.ascontiguousarray(C0).copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), w.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, tol, max_iter, form,
                                        stream.cuda_stream, ctypes.byref(fit)))
    try:
        capi.check(L.kmc_fit_run(fit))
        it, inertia = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inertia)))
        last, total, err = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        capi.check(L.kmc_fit_rechecked(fit, ctypes.byref(last), ctypes.byref(total), ctypes.byref(err)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    assert err.value == 0, "tensor-core kernel reported a device-side timeout"
    return it.value, lab.cpu().numpy(), res.cpu().numpy(), inertia.value, last.value, total.value


SHAPES = [(300, 64, 256), (1000, 3, 8), (5000, 14, 127), (20000, 64, 1024), (7777, 100, 300),
          (4096, 33, 511), (129, 128, 512), (20000, 16, 1024), (3001, 65, 257),
          # several column passes (k beyond one launch) and 3-4 feature blocks
          (20000, 64, 2048), (5000, 64, 1025), (3000, 100, 513), (4000, 200, 300), (3000, 129, 64),
          (2000, 256, 100), (6000, 20, 3000), (2500, 180, 700)]


@pytest.mark.parametrize("n,d,k", SHAPES)
@pytest.mark.parametrize("form", sorted(FORMS))
def test_mixed_assignment_equals_reference_labels(oracle, n, d, k, form):
    X, _, _ = bench.make_blobs(n, d, max(1, k // 2), (-5, 5), 1.0, seed=n + d + k)
    if k <= n:
        C0 = bench.random_row_init(X, k, seed=k)
    else:
        C0 = np.random.default_rng(k).uniform(-5, 5, (d, k)).astype(np.float32)
    _, lab, _, _, last, _ = _fit_labels(X, C0, FORMS[form])
    np.testing.assert_array_equal(lab, oracle.assignment(X, C0))
    assert 0 <= last <= n


@pytest.mark.parametrize("d,k", [(257, 64), (300, 8)])
def test_mixed_rejects_more_than_256_features(d, k):
    X = np.zeros((d, 256), np.float32)
    C = np.zeros((d, k), np.float32)
    with pytest.raises(RuntimeError, match="kmc error 4"):
        _fit_labels(X, C, FORMS["fp16"])


@pytest.mark.parametrize("form", sorted(FORMS))
def test_mixed_assignment_ties_and_duplicates(oracle, form):
    rng = np.random.default_rng(5)
    C = rng.standard_normal((64, 128)).astype(np.float32)
    C = np.ascontiguousarray(np.concatenate([C, C], axis=1))   # exact duplicates: all ties
    X = rng.standard_normal((64, 3000)).astype(np.float32)
    _, lab, _, _, last, _ = _fit_labels(X, C, FORMS[form])
    np.testing.assert_array_equal(lab, oracle.assignment(X, C))
    assert last == 3000          # every sample ties between j and j + 128
    assert lab.max() < 128


def _near_tie_mask(X, C, rel=1e-5):
    """Samples whose two smallest distances differ by less than rel (relative)."""
    d2 = np.maximum(0.0, (X.astype(np.float64) ** 2).sum(0)[:, None]
                    - 2 * X.T.astype(np.float64) @ C.astype(np.float64)
                    + (C.astype(np.float64) ** 2).sum(0)[None, :])
    part = np.partition(d2, 1, axis=1)[:, :2]
    return (part[:, 1] - part[:, 0]) <= rel * np.maximum(part[:, 1], 1e-30)


# Up to 32 features the cluster sums are reduced in float64, so whole
# trajectories follow the oracle's (iteration count included).
# The forced-empty case relocates a cluster in its first iteration: the samples moved
# are chosen by the squared distances the assignment pass writes.
@pytest.mark.parametrize("case", [("c1_50k_d14_k16", 50_000, 14, 16, 16, (-10, 10), 1.0, 0, 1e-4, 100),
                                  ("d32_k200", 40_000, 32, 100, 200, (-5, 5), 1.0, 3, 0.0, 10),
                                  ("d16_k1500_passes", 60_000, 16, 700, 1500, (-10, 10), 1.0, 5, 0.0,
                                   6),
                                  ("d14_k127_forced_empty", 100_000, 14, 127, 127, (-10, 10), 1.5, 1,
                                   0.0, 8, True)])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_mixed_driver_tracks_oracle(oracle, case, form):
    name, n, d, centers, k, box, std, seed, tol, max_iter = case[:10]
    far = len(case) > 10 and case[10]
    X, _, _ = bench.make_blobs(n, d, centers, box, std, seed)
    C0 = bench.random_row_init(X, k, seed, far_first=far)
    it_o, lab_o, C_o, inr_o, rel_o = oracle.kmeans_lloyd_driver(X, np.ones(n, np.float32), C0, tol,
                                                                max_iter)
    if far:
        assert rel_o >= 1
    it_g, lab_g, C_g, inr_g, _, total = _fit_labels(X, C0, FORMS[form], max_iter=max_iter, tol=tol)
    assert it_g == it_o
    diff = lab_g != lab_o
    assert not np.any(diff & ~_near_tie_mask(X, C_o)), int(diff.sum())
    np.testing.assert_allclose(C_g, C_o, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
    assert inr_g == pytest.approx(inr_o, rel=1e-5)


# Beyond 32 features the sums are float32 reductions in arrival order (as the
# reference's atomics are), so trajectories are compared one iteration at a
# time: labels exact against the oracle at that iteration's centroids, the
# update within float32 accumulation tolerance, and the final pass exact.
@pytest.mark.parametrize("case", [("d64_k256", 60_000, 64, 256, 256, (-5, 5), 1.0, 2, 6),
                                  ("d64_k1024_sigma", 100_000, 64, 1024, 1024, (-5, 5), (0.5, 2.0), 2, 4),
                                  ("d100_k300", 30_000, 100, 150, 300, (-5, 5), 1.0, 4, 3),
                                  ("d64_k256_forced_empty", 60_000, 64, 256, 256, (-5, 5), 1.0, 6, 3,
                                   True),
                                  ("d64_k2048_passes", 60_000, 64, 1500, 2048, (-5, 5), 1.0, 7, 3),
                                  ("d200_k600_passes_forced_empty", 20_000, 200, 300, 600, (-5, 5),
                                   1.0, 8, 3, True)])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_mixed_iterations_match_oracle_step_by_step(oracle, case, form):
    import torch

    from kmeans_dpcpp_gb300 import capi

    name, n, d, centers, k, box, std, seed, iters = case[:9]
    far = len(case) > 9 and case[9]
    X, _, _ = bench.make_blobs(n, d, centers, box, std, seed)
    C0 = bench.random_row_init(X, k, seed, far_first=far)
    relocated = 0
    w = np.ones(n, np.float32)
    L = capi.lib()
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    wg = torch.from_numpy(w).cuda()
    cur = torch.from_numpy(np.ascontiguousarray(C0).copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), wg.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, 0.0, iters, FORMS[form],
                                        stream.cuda_stream, ctypes.byref(fit)))
    try:
        for _ in range(iters):
            C_before = cur.cpu().numpy().copy()
            capi.check(L.kmc_fit_step(fit, 1))
            stream.synchronize()
            np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assignment(X, C_before))
            _, _, C_o, _, rel = oracle.kmeans_lloyd_driver(X, w, C_before, 0.0, 1)
            relocated += rel
            C_after = cur.cpu().numpy()
            np.testing.assert_allclose(C_after, C_o, rtol=1e-5, atol=1e-5 * np.abs(C_o).max())
        it, inertia = ctypes.c_int64(), ctypes.c_double()
        capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inertia)))
        last, total, err = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int()
        capi.check(L.kmc_fit_rechecked(fit, ctypes.byref(last), ctypes.byref(total), ctypes.byref(err)))
    finally:
        capi.check(L.kmc_fit_destroy(fit))
    assert err.value == 0 and it.value == iters
    if far:
        assert relocated >= 1
    C_final = res.cpu().numpy()
    lab_final = lab.cpu().numpy()
    np.testing.assert_array_equal(lab_final, oracle.assignment(X, C_final))
    inr_o = float(np.sum(oracle.compute_inertia(X, w, C_final, lab_final).astype(np.float64)))
    assert inertia.value == pytest.approx(inr_o, rel=1e-6)


# Up to 32 features the tensor-core kernel adds the cluster sums as integers
# (fixed point, scaled by the data's bounds); values below that scale's
# resolution (a feature a trillion times smaller than the rest, weights of
# 1e-30) take a float64 side path.  Every centroid coordinate must still follow
# the oracle on its own scale.
@pytest.mark.parametrize("d,k", [(8, 8), (20, 40), (32, 64)])
@pytest.mark.parametrize("form", sorted(FORMS))
def test_mixed_fixed_point_sums_with_tiny_values_and_weights(oracle, d, k, form):
    import torch

    from kmeans_dpcpp_gb300 import capi

    n, iters = 30_000, 3
    X, _, _ = bench.make_blobs(n, d, k, (-5, 5), 1.0, 11)
    X = np.ascontiguousarray(X)
    X[0] *= np.float32(1e-12)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.5, 2.0, n).astype(np.float32)
    w[rng.choice(n, 300, replace=False)] = np.float32(1e-30)
    w[rng.choice(n, 300, replace=False)] = 0.0
    C0 = np.ascontiguousarray(bench.random_row_init(X, k, 11))
    L = capi.lib()
    Xg = torch.from_numpy(X).cuda()
    wg = torch.from_numpy(w).cuda()
    cur = torch.from_numpy(C0.copy()).cuda()
    res = torch.empty_like(cur)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    fit = ctypes.c_void_p()
    capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), wg.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                        res.data_ptr(), n, d, k, 0.0, iters, FORMS[form],
                                        stream.cuda_stream, ctypes.byref(fit)))
    try:
        for _ in range(iters):
            C_before = cur.cpu().numpy().copy()
            capi.check(L.kmc_fit_step(fit, 1))
            stream.synchronize()
            np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assignment(X, C_before))
            _, _, C_o, _, _ = oracle.kmeans_lloyd_driver(X, w, C_before, 0.0, 1)
            C_after = cur.cpu().numpy()
            for f in range(d):
                scale = float(np.abs(C_o[f]).max())
                np.testing.assert_allclose(C_after[f], C_o[f], rtol=1e-6, atol=1e-6 * scale,
                                           err_msg=f"feature {f}")
    finally:
        capi.check(L.kmc_fit_destroy(fit))


# Up to 32 features the cluster sums are integer totals, added in any order to
# the same bits: two runs of a fit give bit-identical centroids and labels
# (k = 1500 takes two column passes, whose combine adds the integer totals).
@pytest.mark.parametrize("d,k", [(8, 30), (32, 64), (16, 1500)])
def test_mixed_fixed_point_fits_are_bit_reproducible(d, k):
    import torch

    from kmeans_dpcpp_gb300 import capi

    n = 400_000
    X, _, _ = bench.make_blobs(n, d, k, (-5, 5), 1.0, 17)
    C0 = np.ascontiguousarray(bench.random_row_init(X, k, 17))
    rng = np.random.default_rng(17)
    w = rng.uniform(0.25, 4.0, n).astype(np.float32)
    L = capi.lib()
    Xg = torch.from_numpy(np.ascontiguousarray(X)).cuda()
    wg = torch.from_numpy(w).cuda()
    stream = torch.cuda.current_stream()
    outs = []
    for _ in range(2):
        cur = torch.from_numpy(C0.copy()).cuda()
        res = torch.empty_like(cur)
        lab = torch.empty(n, dtype=torch.int32, device="cuda")
        fit = ctypes.c_void_p()
        capi.check(L.kmc_fit_create_f32_i32(Xg.data_ptr(), wg.data_ptr(), cur.data_ptr(), lab.data_ptr(),
                                            res.data_ptr(), n, d, k, 0.0, 12, FORMS["fp16"],
                                            stream.cuda_stream, ctypes.byref(fit)))
        try:
            capi.check(L.kmc_fit_run(fit))
            it, inr = ctypes.c_int64(), ctypes.c_double()
            capi.check(L.kmc_fit_finalize(fit, ctypes.byref(it), ctypes.byref(inr)))
        finally:
            capi.check(L.kmc_fit_destroy(fit))
        outs.append((it.value, res.cpu().numpy(), lab.cpu().numpy()))
    assert outs[0][0] == outs[1][0]
    np.testing.assert_array_equal(outs[0][1], outs[1][1])
    np.testing.assert_array_equal(outs[0][2], outs[1][2])


def test_fit_after_trimming_the_memory_pool_gives_the_same_labels(oracle):
    """Scratch comes from a pool that keeps freed memory mapped; trimming it
    between fits hands the memory back and the next fit allocates afresh."""
    from kmeans_dpcpp_gb300 import capi

    L = capi.lib()
    X, _, _ = bench.make_blobs(20000, 64, 300, (-5, 5), 1.0, seed=11)
    C0 = bench.random_row_init(X, 300, seed=11)
    first = _fit_labels(X, C0, FORMS["fp16"])[1]
    assert L.kmc_trim_cached_memory() == 0
    second = _fit_labels(X, C0, FORMS["fp16"])[1]
    np.testing.assert_array_equal(first, second)
    np.testing.assert_array_equal(first, oracle.assignment(X, C0))
