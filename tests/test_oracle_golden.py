"""Pins the CPU oracle to the reference's known answers (tests/test_kernels.py).

Each test restates one reference test against oracle/kmref.cpp, with the
reference test's own tolerance (np.finfo(dtype).resolution unless noted).
"""
import numpy as np
import pytest

DTYPES = [("f32", np.float32), ("f64", np.float64)]


def res(dt):
    return np.finfo(dt).resolution


@pytest.mark.parametrize("s,dt", DTYPES)
def test_broadcast_divide(golden, oracle, s, dt):
    out = oracle.broadcast_divide(golden[f"broadcast_divide_{s}/X"], golden[f"broadcast_divide_{s}/y"])
    np.testing.assert_allclose(out, golden[f"broadcast_divide_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_half_l2_norm_squared(golden, oracle, s, dt):
    out = oracle.half_l2_norm_squared(golden[f"half_l2_norm_{s}/X"])
    np.testing.assert_allclose(out, golden[f"half_l2_norm_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("case", ["reduce_centroids", "reduce_centroids_empty"])
@pytest.mark.parametrize("s,dt", DTYPES)
def test_reduce_centroids_data(golden, oracle, case, s, dt):
    p = f"{case}_{s}/"
    osz, oc, lst, ne = oracle.reduce_centroids(golden[p + "sizes_cp"], golden[p + "cent_cp"],
                                               n_empty_init=0, list_fill=10)
    assert ne == int(golden[p + "expected_n_empty"])
    np.testing.assert_array_equal(lst, golden[p + "expected_list"])
    np.testing.assert_allclose(oc, golden[p + "expected_sums"], rtol=res(dt))
    np.testing.assert_allclose(osz, golden[p + "expected_sizes"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_compute_threshold(golden, oracle, s, dt):
    x = golden[f"threshold_{s}/data"]
    assert oracle.compute_threshold(x, 1) == float(golden[f"threshold_{s}/expected_top1"])
    assert oracle.compute_threshold(x, 2) == float(golden[f"threshold_{s}/expected_top2"])


@pytest.mark.parametrize("s,dt", DTYPES)
def test_select_samples_far_from_centroid(golden, oracle, s, dt):
    x = golden[f"select_{s}/distance"]
    ne = int(golden[f"select_{s}/n_empty"])
    thr = oracle.compute_threshold(x, ne)
    sel, ng, nq = oracle.select_samples_far_from_centroid(ne, x, thr, fill=172, n_gt=0, n_eq=1)
    # tests/test_kernels.py:360-362
    assert ng + nq - 1 == ne
    assert np.all(x[sel[:ng]] > thr)
    assert np.all(x[sel[1 - nq:]] == thr)
    # defined order: sel[ng-1-r] is the r-th farthest
    order = np.lexsort((np.arange(x.size), -x))
    np.testing.assert_array_equal(sel[:ng][::-1], order[:ng])


@pytest.mark.parametrize("s,dt", DTYPES)
def test_relocate_empty_clusters(golden, oracle, s, dt):
    p = f"relocate_{s}/"
    X_t = golden[p + "X_t"]
    n = X_t.shape[1]
    C, sizes, inr = oracle.relocate_empty_clusters(
        1, X_t, np.ones(n, dt), golden[p + "labels"], golden[p + "empty_list"],
        golden[p + "sq_dist"], golden[p + "C_t"], golden[p + "sizes"], golden[p + "sq_dist"])
    np.testing.assert_allclose(sizes, golden[p + "expected_sizes"], rtol=res(dt))
    np.testing.assert_allclose(C, golden[p + "expected_C_t"], rtol=res(dt))
    np.testing.assert_allclose(inr, golden[p + "expected_inertia"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_centroid_shifts(golden, oracle, s, dt):
    out = oracle.centroid_shifts(golden[f"shifts_{s}/C1_t"], golden[f"shifts_{s}/C2_t"])
    np.testing.assert_allclose(out, golden[f"shifts_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt,f", [("f32", np.float32, 64), ("f64", np.float64, 1)])
def test_distances(golden, oracle, s, dt, f):
    out = oracle.distances(golden[f"distances_{s}/X_t"], golden[f"distances_{s}/C_t"])
    np.testing.assert_allclose(out, golden[f"distances_{s}/expected"], rtol=f * res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_assignment(golden, oracle, s, dt):
    lab = oracle.assignment(golden[f"assignment_{s}/X_t"], golden[f"assignment_{s}/C_t"])
    np.testing.assert_array_equal(lab, golden[f"assignment_{s}/expected"])


@pytest.mark.parametrize("s,dt", DTYPES)
def test_compute_inertia(golden, oracle, s, dt):
    X_t = golden[f"inertia_{s}/X_t"]
    out = oracle.compute_inertia(X_t, np.ones(X_t.shape[1], dt), golden[f"inertia_{s}/C_t"],
                                 golden[f"inertia_{s}/labels"])
    np.testing.assert_allclose(out, golden[f"inertia_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_reduce_vector(golden, oracle, s, dt):
    assert oracle.sum_ld(golden[f"reduce_vector_{s}/data"]) == float(golden[f"reduce_vector_{s}/expected"])


@pytest.mark.parametrize("s,dt", DTYPES)
def test_fused_lloyd_single_step(golden, oracle, s, dt):
    p = f"fused_step_{s}/"
    X_t = golden[p + "X_t"]
    lab, sums, sizes = oracle.fused_lloyd_single_step(X_t, np.ones(X_t.shape[1], dt), golden[p + "C_t"],
                                                      golden[p + "half_norm"])
    np.testing.assert_array_equal(lab, golden[p + "expected_labels"])
    np.testing.assert_allclose(sizes, golden[p + "expected_sizes"], rtol=res(dt))
    np.testing.assert_allclose(sums, golden[p + "expected_sums"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DTYPES)
def test_kmeans_lloyd_driver(golden, oracle, s, dt):
    p = f"driver_{s}/"
    X_t = golden[p + "X_t"]
    it, lab, C, inertia, rel = oracle.kmeans_lloyd_driver(
        X_t, np.ones(X_t.shape[1], dt), golden[p + "init_C_t"], float(golden[p + "tol"]),
        int(golden[p + "max_iter"]))
    np.testing.assert_array_equal(lab, golden[p + "expected_labels"])
    assert it < int(golden[p + "max_iter"])
    assert it == int(golden[p + "expected_n_iters"])


def test_oracle_relocation_multiple_empty(oracle):
    """n_empty >= 2: empty cluster r takes the r-th farthest sample (ties: lower index)."""
    rng = np.random.default_rng(7)
    n, d, k = 50, 2, 5
    X_t = rng.standard_normal((d, n))
    labels = rng.integers(0, 2, n)
    C = rng.standard_normal((d, k))
    sq = np.array([np.sum((X_t[:, i] - C[:, labels[i]]) ** 2) for i in range(n)])
    sq[10] = sq[20] = sq.max() + 1.0          # a tie at the top
    sizes = np.bincount(labels, minlength=k).astype(np.float64)
    sums = np.zeros((d, k))
    for i in range(n):
        sums[:, labels[i]] += X_t[:, i]
    empty = np.array([2, 3, 4, -1, -1])
    C2, sz2, inr2 = oracle.relocate_empty_clusters(3, X_t, np.ones(n), labels, empty, sq, sums, sizes, sq)
    order = np.lexsort((np.arange(n), -sq))[:3]
    assert list(order[:2]) == [10, 20]
    for r, cl in enumerate([2, 3, 4]):
        np.testing.assert_allclose(C2[:, cl], X_t[:, order[r]])
        assert sz2[cl] == 1.0
        assert inr2[order[r]] == 0.0
    assert sz2.sum() == n


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_oracle_iteration_chains_to_the_driver(oracle, dt):
    """lloyd_iteration is the driver's loop body: chained from the same start (one centroid
    forced empty, so the first pass relocates) it reaches the driver's centroids bit for bit,
    and its last labels are the assignment against its last input centroids."""
    import bench

    X, _, _ = bench.make_blobs(3000, 4, 6, (-10, 10), 1.0, 21, dtype=dt)
    C0 = bench.random_row_init(X, 6, 21, far_first=True)
    w = np.ones(X.shape[1], dt)
    it, _, C_drv, _, rel = oracle.kmeans_lloyd_driver(X, w, C0, 0.0, 4)
    assert it == 4 and rel >= 1
    C = C0.copy()
    relocated = []
    for _ in range(4):
        lab, C_next, shift, r = oracle.lloyd_iteration(X, w, C)
        np.testing.assert_array_equal(lab, oracle.assignment(X, C))
        relocated.append(r)
        C = C_next
    assert relocated[0]
    np.testing.assert_array_equal(C, C_drv)
    assert shift >= 0.0
