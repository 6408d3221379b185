"""The reference's known-answer tests (tests/test_kernels.py), run on the GB300
kernels through the drop-in Python surface, for every dtype/index combination.

Inputs and expected answers come from tests/golden/known_answers.npz; the
tolerances are the reference test's own.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DT = [("f32", np.float32), ("f64", np.float64)]
IT = [np.int32, np.int64]


def res(dt):
    return np.finfo(dt).resolution


def T(a, dtype=None):
    import torch

    # np.array(copy=True, order="C") keeps 0-d arrays 0-d
    a = np.array(a, dtype=dtype, copy=True, order="C")
    return torch.from_numpy(a).cuda()


def H(t):
    return t.cpu().numpy()


@pytest.mark.parametrize("s,dt", DT)
def test_broadcast_divide(golden, kdp, s, dt):
    X = T(golden[f"broadcast_divide_{s}/X"])
    y = T(golden[f"broadcast_divide_{s}/y"])
    ht, _ = kdp.broadcast_divide(X, y, work_group_size=32, sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(X), golden[f"broadcast_divide_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DT)
def test_half_l2_norm_squared(golden, kdp, s, dt):
    import torch

    X = T(golden[f"half_l2_norm_{s}/X"])
    y = torch.empty(X.shape[1], dtype=X.dtype, device=X.device)
    ht, _ = kdp.half_l2_norm_squared(X, y, work_group_size=32, sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(y), golden[f"half_l2_norm_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("case", ["reduce_centroids", "reduce_centroids_empty"])
@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_reduce_centroids_data(golden, kdp, case, s, dt, it):
    import torch

    p = f"{case}_{s}/"
    szc, cc = T(golden[p + "sizes_cp"]), T(golden[p + "cent_cp"])
    k, d = szc.shape[1], cc.shape[1]
    osz = torch.empty(k, dtype=szc.dtype, device="cuda")
    oc = torch.empty((d, k), dtype=szc.dtype, device="cuda")
    lst = T(np.full(k, 10), it)
    ne = T(np.zeros(1), it)
    ht, ev = kdp.reduce_centroids_data(szc, cc, osz, oc, lst, ne, work_group_size=32, sycl_queue=None)
    ht.wait()
    ev.wait()
    assert int(H(ne)[0]) == int(golden[p + "expected_n_empty"])
    np.testing.assert_array_equal(H(lst), golden[p + "expected_list"])
    np.testing.assert_allclose(H(oc), golden[p + "expected_sums"], rtol=res(dt))
    np.testing.assert_allclose(H(osz), golden[p + "expected_sizes"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("topk,key", [(1, "expected_top1"), (2, "expected_top2")])
def test_compute_threshold(golden, kdp, s, dt, topk, key):
    data = T(golden[f"threshold_{s}/data"])
    thr = T(np.full((), -127), dt)
    ht, _ = kdp.compute_threshold(data, topk, thr, sycl_queue=None)
    ht.wait()
    assert H(thr).item() == float(golden[f"threshold_{s}/{key}"])


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_select_samples_far_from_centroid(golden, kdp, s, dt, it):
    import torch

    x = golden[f"select_{s}/distance"]
    ne = int(golden[f"select_{s}/n_empty"])
    dist = T(x)
    thr = torch.empty((), dtype=dist.dtype, device="cuda")
    sel = T(np.full(x.size, 172), it)
    ngt = T(np.zeros(()), it)
    neq = T(np.ones(()), it)
    ht, c_ev = kdp.compute_threshold(dist, ne, thr, sycl_queue=None)
    ht2, _ = kdp.select_samples_far_from_centroid(ne, dist, thr, sel, ngt, neq, work_group_size=256,
                                                  sycl_queue=None, depends=[c_ev])
    ht2.wait()
    ht.wait()
    ng, nq, t = H(ngt).item(), H(neq).item(), H(thr).item()
    s_np = H(sel)
    assert ng + nq - 1 == ne
    assert np.all(x[s_np[:ng]] > t)
    assert np.all(x[s_np[1 - nq:]] == t)


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_relocate_empty_clusters(golden, kdp, s, dt, it):
    p = f"relocate_{s}/"
    X_t = T(golden[p + "X_t"])
    n = X_t.shape[1]
    w = T(np.ones(n), dt)
    C = T(golden[p + "C_t"])
    sizes = T(golden[p + "sizes"])
    sq = T(golden[p + "sq_dist"])
    inr = sq  # the reference test passes the same array for both
    ht, _ = kdp.relocate_empty_clusters(1, X_t, w, T(golden[p + "labels"], it),
                                        T(golden[p + "empty_list"], it), sq, C, sizes, inr,
                                        work_group_size=256, sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(sizes), golden[p + "expected_sizes"], rtol=res(dt))
    np.testing.assert_allclose(H(C), golden[p + "expected_C_t"], rtol=res(dt))
    np.testing.assert_allclose(H(inr), golden[p + "expected_inertia"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DT)
def test_centroid_shifts(golden, kdp, s, dt):
    import torch

    a, b = T(golden[f"shifts_{s}/C1_t"]), T(golden[f"shifts_{s}/C2_t"])
    cs = torch.empty(a.shape[1], dtype=a.dtype, device="cuda")
    ht, _ = kdp.compute_centroid_shifts_squared(a, b, cs, sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(cs), golden[f"shifts_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt,f", [("f32", np.float32, 64), ("f64", np.float64, 1)])
def test_compute_centroid_to_sample_distances(golden, kdp, s, dt, f):
    import torch

    X, C = T(golden[f"distances_{s}/X_t"]), T(golden[f"distances_{s}/C_t"])
    dm = torch.empty((C.shape[1], X.shape[1]), dtype=X.dtype, device="cuda")
    ht, _ = kdp.compute_centroid_to_sample_distances(X, C, dm, 256, 8, sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(dm), golden[f"distances_{s}/expected"], rtol=f * res(dt))


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_assignment(golden, kdp, s, dt, it):
    import torch

    X, C = T(golden[f"assignment_{s}/X_t"]), T(golden[f"assignment_{s}/C_t"])
    hl2n = torch.empty(C.shape[1], dtype=X.dtype, device="cuda")
    lab = torch.empty(X.shape[1], dtype=torch.from_numpy(np.zeros(1, it)).dtype, device="cuda")
    ht1, e_hl2n = kdp.half_l2_norm_squared(C, hl2n, work_group_size=256, sycl_queue=None)
    ht2, e_assign = kdp.assignment(X, C, hl2n, lab, centroids_window_height=8, work_group_size=256,
                                   sycl_queue=None, depends=[e_hl2n])
    ht1.wait()
    ht2.wait()
    np.testing.assert_array_equal(H(lab), golden[f"assignment_{s}/expected"])


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_compute_inertia(golden, kdp, s, dt, it):
    import torch

    X = T(golden[f"inertia_{s}/X_t"])
    n = X.shape[1]
    out = torch.empty(n, dtype=X.dtype, device="cuda")
    ht, _ = kdp.compute_inertia(X, T(np.ones(n), dt), T(golden[f"inertia_{s}/C_t"]),
                                T(golden[f"inertia_{s}/labels"], it), out, work_group_size=256,
                                sycl_queue=None)
    ht.wait()
    np.testing.assert_allclose(H(out), golden[f"inertia_{s}/expected"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DT)
def test_reduce_vector_blocking(golden, kdp, s, dt):
    r = kdp.reduce_vector_blocking(T(golden[f"reduce_vector_{s}/data"]), sycl_queue=None)
    assert r == 50 * 99


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_lloyd_single_step(golden, kdp, s, dt, it):
    import torch

    p = f"fused_step_{s}/"
    X, C, hn = T(golden[p + "X_t"]), T(golden[p + "C_t"]), T(golden[p + "half_norm"])
    d, n = X.shape
    k = C.shape[1]
    P = int(golden[p + "n_copies"])
    lab = T(np.empty(n), it)
    cc = torch.zeros((P, d, k), dtype=X.dtype, device="cuda")
    szc = torch.zeros((P, k), dtype=X.dtype, device="cuda")
    ht, _ = kdp.fused_lloyd_single_step(X, T(np.ones(n), dt), C, hn, lab, cc, szc, 8, 256, None)
    ht.wait()
    np.testing.assert_array_equal(H(lab), golden[p + "expected_labels"])
    np.testing.assert_allclose(H(szc).sum(axis=0), golden[p + "expected_sizes"], rtol=res(dt))
    np.testing.assert_allclose(H(cc).sum(axis=0), golden[p + "expected_sums"], rtol=res(dt))


@pytest.mark.parametrize("s,dt", DT)
@pytest.mark.parametrize("it", IT)
def test_kmeans_lloyd_driver(golden, kdp, s, dt, it):
    import torch

    p = f"driver_{s}/"
    X = T(golden[p + "X_t"])
    n = X.shape[1]
    init = T(golden[p + "init_C_t"])
    res_c = torch.empty_like(init)
    lab = T(np.empty(n), it)
    n_iters, inertia = kdp.kmeans_lloyd_driver(X, T(np.ones(n), dt), init, lab, res_c,
                                               float(golden[p + "tol"]), False,
                                               int(golden[p + "max_iter"]), 8, 128, 0.7,
                                               sycl_queue=None)
    np.testing.assert_array_equal(H(lab), golden[p + "expected_labels"])
    assert n_iters < int(golden[p + "max_iter"])
    assert n_iters == int(golden[p + "expected_n_iters"])
    assert inertia.shape == (1,) and inertia.dtype == dt


def test_torch_stream_and_depends(golden, kdp):
    """sycl_queue accepts a torch.cuda.Stream; depends orders work across streams."""
    import torch

    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    X = T(golden["half_l2_norm_f32/X"])
    y = torch.empty(X.shape[1], dtype=X.dtype, device="cuda")
    z = torch.empty_like(X)
    with torch.cuda.stream(s1):
        z.copy_(X)
    torch.cuda.synchronize()
    ht1, ev1 = kdp.broadcast_divide(z, T(np.full(6, 2.0), np.float32), 32, s1)
    ht2, ev2 = kdp.half_l2_norm_squared(z, y, 32, s2, depends=[ev1])
    ht2.wait()
    ht1.wait()
    np.testing.assert_allclose(H(y), golden["half_l2_norm_f32/expected"] / 4, rtol=1e-6)
