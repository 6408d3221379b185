"""Generate tests/golden/known_answers.npz from the reference's known-answer tests.

Every case below restates one test of the reference's tests/test_kernels.py
(file:line cited per case): the same shapes, distributions and expected
answers.  The reference draws most inputs from the unseeded global numpy
generator; here each case has a fixed seed so the fixture is reproducible, and
the inputs are stored so that tests do not depend on the numpy version's
random streams.  The driver case reproduces the reference's own seeded input
(default_rng(12345)) exactly.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "known_answers.npz")

CORNERS = np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [-1, 1, 1],
                    [1, -1, -1], [-1, 1, -1], [-1, -1, 1], [-1, -1, -1]])


def main():
    g = {}
    for dt in (np.float32, np.float64):
        s = "f32" if dt == np.float32 else "f64"

        # test_broadcast_divide_fp32/fp64, tests/test_kernels.py:14-43
        g[f"broadcast_divide_{s}/X"] = np.full((16, 5), 27.0, dtype=dt)
        g[f"broadcast_divide_{s}/y"] = np.array([1, 3, 9, 3, 1], dtype=dt)
        g[f"broadcast_divide_{s}/expected"] = np.full((16, 5), np.array([27, 9, 3, 9, 27], dtype=dt))

        # test_half_l2_norm_squared_fp32/fp64, tests/test_kernels.py:46-83
        X = np.empty((3, 6), dtype=dt)
        X[:, :4] = 2.0
        X[:, 4:] = 1.0
        g[f"half_l2_norm_{s}/X"] = X
        g[f"half_l2_norm_{s}/expected"] = np.array([6., 6., 6., 6., 1.5, 1.5], dtype=dt)

        # test_reduce_centroids_data_fp32/fp64, tests/test_kernels.py:86-174
        rng = np.random.default_rng(101)
        szc = np.array([[2, 1, 3, 1], [1, 2, 3, 1], [0, 1, 0, 1]], dtype=dt)
        cc = rng.standard_normal((3, 2, 4)).astype(dt)
        g[f"reduce_centroids_{s}/sizes_cp"] = szc
        g[f"reduce_centroids_{s}/cent_cp"] = cc
        g[f"reduce_centroids_{s}/expected_sums"] = cc.sum(axis=0)
        g[f"reduce_centroids_{s}/expected_sizes"] = szc.sum(axis=0)
        g[f"reduce_centroids_{s}/expected_n_empty"] = np.array(0)
        g[f"reduce_centroids_{s}/expected_list"] = np.full(4, 10, dtype=np.int32)

        # test_reduce_centroids_data_empty_fp32/fp64, tests/test_kernels.py:177-262
        rng = np.random.default_rng(102)
        szc = np.array([[2, 1, 3, 0], [1, 2, 3, 0], [1, 1, 0, 0]], dtype=dt)
        cc = rng.standard_normal((3, 2, 4)).astype(dt)
        np.put(cc, np.arange(3, 12, step=4, dtype=np.int32), np.zeros(3, dtype=dt))
        g[f"reduce_centroids_empty_{s}/sizes_cp"] = szc
        g[f"reduce_centroids_empty_{s}/cent_cp"] = cc
        g[f"reduce_centroids_empty_{s}/expected_sums"] = cc.sum(axis=0)
        g[f"reduce_centroids_empty_{s}/expected_sizes"] = szc.sum(axis=0)
        g[f"reduce_centroids_empty_{s}/expected_n_empty"] = np.array(1)
        g[f"reduce_centroids_empty_{s}/expected_list"] = np.array([3, 10, 10, 10], dtype=np.int32)

        # test_compute_threshold_1/2, tests/test_kernels.py:265-326
        rng = np.random.default_rng(103)
        n = 255 * 23
        x = rng.standard_normal(n).astype(dt)
        g[f"threshold_{s}/data"] = x
        g[f"threshold_{s}/expected_top1"] = np.array(x.max(), dtype=dt)
        g[f"threshold_{s}/expected_top2"] = np.array(np.partition(x, kth=n - 2)[n - 2], dtype=dt)

        # test_select_samples_far_from_centroid_kernel, tests/test_kernels.py:329-400
        rng = np.random.default_rng(104)
        g[f"select_{s}/distance"] = rng.standard_gamma(4, size=10 ** 5).astype(dt)
        g[f"select_{s}/n_empty"] = np.array(3)

        # test_relocate_empty_clusters, tests/test_kernels.py:403-516
        Xr = np.array([[+1, +1, +1], [+1, +1, -1], [+1, -1, +1], [-1, +1, +1],
                       [-1, -1, +1], [-1, +1, -1], [+1, -1, -1], [-1, -1, -1]], dtype=dt)
        Cr = np.array([[0.11, -0.1, 0.09], [5, 5, 5]], dtype=dt)
        sq = np.min(np.square(Xr[:, np.newaxis, :] - Cr[np.newaxis, :, :]).sum(axis=-1), axis=-1)
        exp_inr = np.copy(sq)
        exp_inr[5] = 0
        g[f"relocate_{s}/X_t"] = np.ascontiguousarray(Xr.T)
        g[f"relocate_{s}/C_t"] = np.ascontiguousarray(Cr.T)
        g[f"relocate_{s}/sq_dist"] = sq.astype(dt)
        g[f"relocate_{s}/empty_list"] = np.array([1, 0], dtype=np.int32)
        g[f"relocate_{s}/sizes"] = np.array([8, 0], dtype=dt)
        g[f"relocate_{s}/labels"] = np.zeros(8, dtype=np.int32)
        g[f"relocate_{s}/expected_C_t"] = np.array(
            [[0.11 + 1, -1], [-0.1 - 1, 1], [0.09 + 1, -1]], dtype=dt)
        g[f"relocate_{s}/expected_sizes"] = np.array([7, 1], dtype=dt)
        g[f"relocate_{s}/expected_inertia"] = exp_inr.astype(dt)

        # test_centroid_shifts, tests/test_kernels.py:519-558
        g[f"shifts_{s}/C1_t"] = np.array([[1, -5], [2, -4], [3, -3], [4, -2], [5, -1]], dtype=dt)
        g[f"shifts_{s}/C2_t"] = np.array([[2, -4], [3, -3], [4, -2], [5, -1], [6, 1]], dtype=dt)
        g[f"shifts_{s}/expected"] = np.array([5, 8], dtype=dt)

        # test_compute_centroid_to_sample_distances, tests/test_kernels.py:561-642
        rng = np.random.default_rng(105)
        ps = CORNERS.astype(dt)
        Xd = np.concatenate([rng.normal(0, 0.1, size=(8, 3)).astype(dt) + p for p in ps], axis=0)
        Xd_t = np.ascontiguousarray(Xd.T)
        Cd_t = np.ascontiguousarray(ps.T)
        g[f"distances_{s}/X_t"] = Xd_t
        g[f"distances_{s}/C_t"] = Cd_t
        g[f"distances_{s}/expected"] = np.sqrt(
            np.sum(np.square(Xd_t[:, np.newaxis, :] - Cd_t[:, :, np.newaxis]), axis=0))

        # test_assignment_fp32 (cloud 1734) / _fp64 (cloud 32), tests/test_kernels.py:645-777
        rng = np.random.default_rng(106)
        cloud = 1734 if dt == np.float32 else 32
        Xa = np.concatenate([rng.normal(0, 0.1, size=(cloud, 3)).astype(dt) + p for p in ps], axis=0)
        g[f"assignment_{s}/X_t"] = np.ascontiguousarray(Xa.T)
        g[f"assignment_{s}/C_t"] = np.ascontiguousarray(ps.T)
        g[f"assignment_{s}/expected"] = np.repeat(np.arange(8, dtype=np.int32), cloud)

        # test_compute_inertia, tests/test_kernels.py:780-871
        rng = np.random.default_rng(107)
        Xi = np.concatenate([rng.normal(0, 0.1, size=(32, 3)).astype(dt) + p for p in ps], axis=0)
        Xi_t = np.ascontiguousarray(Xi.T)
        Ci_t = np.ascontiguousarray(ps.T)
        ids = np.repeat(np.arange(8, dtype=np.int32), 32)
        g[f"inertia_{s}/X_t"] = Xi_t
        g[f"inertia_{s}/C_t"] = Ci_t
        g[f"inertia_{s}/labels"] = ids
        g[f"inertia_{s}/expected"] = np.sum(
            np.square(Xi_t - np.take_along_axis(Ci_t, ids[np.newaxis, :], axis=1)), axis=0)

        # test_reduce_vector_blocking, tests/test_kernels.py:874-893
        g[f"reduce_vector_{s}/data"] = np.arange(100, dtype=dt)
        g[f"reduce_vector_{s}/expected"] = np.array(50 * 99, dtype=dt)

        # test_lloyd_single_step, tests/test_kernels.py:896-1027
        rng = np.random.default_rng(108)
        Xf = np.concatenate([rng.normal(0, 0.1, size=(16, 3)).astype(dt) + p for p in ps], axis=0)
        Xf_t = np.ascontiguousarray(Xf.T)
        Cf_t = np.ascontiguousarray(ps.T)
        g[f"fused_step_{s}/X_t"] = Xf_t
        g[f"fused_step_{s}/C_t"] = Cf_t
        g[f"fused_step_{s}/half_norm"] = (np.sum(np.square(Cf_t), axis=0) / 2).astype(dt)
        g[f"fused_step_{s}/n_copies"] = np.array(4)
        g[f"fused_step_{s}/expected_labels"] = np.repeat(np.arange(8, dtype=np.int32), 16)
        g[f"fused_step_{s}/expected_sizes"] = np.full(8, 16, dtype=dt)
        g[f"fused_step_{s}/expected_sums"] = np.reshape(Xf_t, (3, 8, 16)).sum(axis=-1)

        # test_kmeans_lloyd_driver, tests/test_kernels.py:1030-1147 (the
        # reference's own seed: default_rng(12345))
        rs = np.random.default_rng(seed=12345)
        Xk = np.concatenate([rs.normal(0, 0.1, size=(32, 3)).astype(dt) + p for p in ps], axis=0)
        g[f"driver_{s}/X_t"] = np.ascontiguousarray(Xk.T)
        g[f"driver_{s}/init_C_t"] = np.ascontiguousarray(ps.T)
        g[f"driver_{s}/tol"] = np.array(1e-6)
        g[f"driver_{s}/max_iter"] = np.array(255)
        g[f"driver_{s}/expected_labels"] = np.repeat(np.arange(8, dtype=np.int32), 32)
        g[f"driver_{s}/expected_n_iters"] = np.array(2)

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes,", len(g), "arrays")


if __name__ == "__main__":
    main()
