"""The drop-in boundary without a GPU: exported C symbols, the Python surface's
names and argument lists, host-side arithmetic and argument validation.

Validation is exercised with stand-in objects that expose
__cuda_array_interface__ with null data pointers, so every error path that
precedes device work runs on the CPU (the reference raises the same
ValueError messages from python_api/_kmeans_lloyd.cpp).
"""
import re

import numpy as np
import pytest

from kmeans_dpcpp_gb300 import capi

# Argument lists of the reference's module (python_api/_kmeans_lloyd.cpp:1277-1449).
REFERENCE_SIGNATURES = {
    "broadcast_divide": ["divident", "divisor", "work_group_size", "sycl_queue", "depends"],
    "half_l2_norm_squared": ["centroids", "centroids_half_l2_norm_squared", "work_group_size",
                             "sycl_queue", "depends"],
    "reduce_centroids_data": ["cluster_sizes_private_copies", "centroids_t_private_copies",
                              "out_cluster_sizes", "out_centroids_t", "out_empty_clusters_list",
                              "out_n_empty_clusters", "work_group_size", "sycl_queue", "depends"],
    "compute_threshold": ["data", "topk", "threshold", "sycl_queue", "depends"],
    "select_samples_far_from_centroid": ["n_selected", "distance_to_centroid", "threshold",
                                         "selected_samples_idx", "n_selected_gt_threshold",
                                         "n_selected_eq_threshold", "work_group_size",
                                         "sycl_queue", "depends"],
    "relocate_empty_clusters": ["n_empty_clusters", "X_t", "sample_weights", "assignment_id",
                                "empty_clusters_list", "sq_dist_to_nearest_centroid",
                                "centroid_t", "cluster_sizes", "per_sample_inertia",
                                "work_group_size", "sycl_queue", "depends"],
    "compute_centroid_shifts_squared": ["centroid_t", "new_centroid_t", "out_centroid_shifts",
                                        "sycl_queue", "depends"],
    "compute_centroid_to_sample_distances": ["X_t", "centroid_t", "euclidean_distances_t",
                                             "work_group_size", "centroids_window_height",
                                             "sycl_queue", "depends"],
    "assignment": ["X_t", "centroids_t", "centroids_half_l2_norm", "assignment_id",
                   "centroids_window_height", "work_group_size", "sycl_queue", "depends"],
    "compute_inertia": ["X_t", "sample_weight", "centroid_t", "assignment_id",
                        "out_per_sample_inertia", "work_group_size", "sycl_queue", "depends"],
    "reduce_vector_blocking": ["data", "sycl_queue", "depends"],
    "fused_lloyd_single_step": ["X_t", "sample_weight", "centroids_t", "centroids_half_l2_norm",
                                "assignments_idx", "new_centroids_t_private_copies",
                                "cluster_sizes_private_copies", "centroids_window_height",
                                "work_group_size", "sycl_queue", "depends"],
    "compute_number_of_private_copies": ["array", "n_samples", "n_features", "n_clusters",
                                         "centroids_private_copies_max_cache_occupancy",
                                         "work_group_size"],
    "kmeans_lloyd_driver": ["X_t", "sample_weight", "init_centroid_t", "assignments_id",
                            "res_centroids_t", "tol", "verbose", "max_iter",
                            "centroids_window_height", "work_group_size",
                            "centroids_private_copies_max_cache_occupancy", "sycl_queue",
                            "depends"],
}
# Trailing keyword arguments this engine adds after the reference's list.
EXTRA_KWARGS = {"kmeans_lloyd_driver": ["form"]}


def test_library_exports_every_declared_symbol():
    lib = capi.lib()
    protos = capi.parse_header()
    assert len(protos) >= 50
    missing = [name for name in protos if not hasattr(lib, name)]
    assert missing == []
    assert lib.kmc_abi_version() == 1


def test_module_surface_matches_reference():
    import kmeans_dpcpp_gb300 as kdp

    assert sorted(kdp.__all__) == sorted(REFERENCE_SIGNATURES)
    for name, args in REFERENCE_SIGNATURES.items():
        fn = getattr(kdp, name)
        sig = fn.__doc__.splitlines()[0]
        got = re.findall(r"(\w+): ", sig[sig.index("(") + 1:])
        assert got == args + EXTRA_KWARGS.get(name, []), (name, got)


def _py_private_copies(esize, n, d, k, occ, wgs, l2):
    # src/lloyd_single_step.hpp:12-35
    copies = int((l2 * occ) / (esize * k * (d + 1)))
    gsize = -(-n // wgs) * wgs
    return min(gsize // 8, copies)


@pytest.mark.parametrize("esize,n,d,k,occ,wgs", [
    (4, 256, 3, 8, 0.7, 128), (8, 10 ** 6, 14, 127, 0.5, 256), (4, 10 ** 7, 64, 1024, 0.9, 64),
    (4, 5, 3, 8, 0.7, 32)])
def test_number_of_private_copies_host_arithmetic(esize, n, d, k, occ, wgs):
    import ctypes

    out = ctypes.c_int64()
    l2 = 126 * 2 ** 20
    capi.check(capi.lib().kmc_compute_number_of_private_copies(esize, n, d, k, occ, wgs, l2,
                                                               ctypes.byref(out)))
    assert out.value == _py_private_copies(esize, n, d, k, occ, wgs, l2)


def test_c_abi_rejects_bad_arguments():
    import ctypes

    L = capi.lib()
    out = ctypes.c_int64()
    assert L.kmc_compute_number_of_private_copies(4, 10, 3, 8, 1.0, 128, 1 << 20,
                                                  ctypes.byref(out)) == 1
    assert "strictly between 0 and 1" in L.kmc_last_error().decode()
    assert L.kmc_select_samples_far_from_centroid_f32_i32(0, None, None, None, None, None, 10, 32,
                                                          None) == 1
    assert "must be positive" in L.kmc_last_error().decode()
    assert L.kmc_relocate_empty_clusters_f32_i32(0, None, None, None, None, None, None, None,
                                                 None, 8, 3, 2, 32, None) == 1
    assert L.kmc_compute_threshold_f32(None, 5, 6, None, None) == 1


class FakeCUDAArray:
    """__cuda_array_interface__ with a null pointer: passes the device check."""

    def __init__(self, shape, typestr="<f4", strides=None):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": typestr,
                                         "data": (0, False), "version": 3, "strides": strides}


class FakeStream:
    cuda_stream = 0

    class device:
        index = 0


F = lambda *s: FakeCUDAArray(s, "<f4")  # noqa: E731
D = lambda *s: FakeCUDAArray(s, "<f8")  # noqa: E731
I4 = lambda *s: FakeCUDAArray(s, "<i4")  # noqa: E731


@pytest.mark.parametrize("call,msg", [
    (lambda k, q: k.broadcast_divide(F(4, 5), F(5, 1), 32, q),
     "Arguments must be a matrix and a vector with C-contiguous layout"),
    (lambda k, q: k.broadcast_divide(F(4, 5), F(4), 32, q),
     "Array dimensions of arguments are not consistent, X.shape[1] != y.shape[0]"),
    (lambda k, q: k.broadcast_divide(F(4, 5), D(5), 32, q),
     "Arguments must have the same elemental data types."),
    (lambda k, q: k.broadcast_divide(FakeCUDAArray((4, 5), "<f4", strides=(4, 16)), F(5), 32, q),
     "Arguments must be a matrix and a vector with C-contiguous layout"),
    (lambda k, q: k.half_l2_norm_squared(I4(3, 4), I4(4), 32, q),
     "Unsupported elemental data type. Expecting single or double precision floating point numbers"),
    (lambda k, q: k.reduce_centroids_data(F(3, 4), F(3, 2, 5), F(4), F(2, 4), I4(4), I4(1), 32, q),
     "Dimensions mismatch"),
    (lambda k, q: k.reduce_centroids_data(F(3, 4), F(3, 2, 4), F(4), D(2, 4), I4(4), I4(1), 32, q),
     "Array element data types must be consisten"),
    (lambda k, q: k.compute_threshold(F(10, 2), 1, F(1), q),
     "Argument data must be a C-contiguous vector"),
    (lambda k, q: k.compute_threshold(F(10), 1, F(2), q),
     "Argument threshold must be 1-element array"),
    (lambda k, q: k.select_samples_far_from_centroid(0, F(10), F(1), I4(10), I4(1), I4(1), 32, q),
     "Argument `n_selected` must be positive"),
    (lambda k, q: k.select_samples_far_from_centroid(11, F(10), F(1), I4(10), I4(1), I4(1), 32, q),
     "Argument `n_select` is too large"),
    (lambda k, q: k.select_samples_far_from_centroid(3, F(10), F(1), I4(9), I4(1), I4(1), 32, q),
     "Vector `selected_samples_idx` must have size `n_samples`"),
    (lambda k, q: k.relocate_empty_clusters(0, F(3, 8), F(8), I4(8), I4(2), F(8), F(3, 2), F(2),
                                            F(8), 32, q),
     "n_empty_clusters must be non-zero."),
    (lambda k, q: k.relocate_empty_clusters(1, F(3, 8), F(7), I4(8), I4(2), F(8), F(3, 2), F(2),
                                            F(8), 32, q),
     "Input dimensions are inconsistent"),
    (lambda k, q: k.compute_centroid_shifts_squared(F(3, 4), F(3, 5), F(4), q),
     "Array dimensions are not consistent."),
    (lambda k, q: k.compute_centroid_to_sample_distances(F(3, 10), F(3, 4), F(4, 9), 32, 8, q),
     "Input array dimensions are not consistant"),
    (lambda k, q: k.assignment(F(3, 10), F(3, 4), F(5), I4(10), 8, 32, q),
     "Inputs have inconsistent dimensions."),
    (lambda k, q: k.compute_inertia(F(3, 10), F(10), F(3, 4), I4(10), D(10), 32, q),
     "Array elemental data types are not consistent"),
    (lambda k, q: k.reduce_vector_blocking(F(3, 3), q), "Expecting 1D contiguous vector."),
    (lambda k, q: k.fused_lloyd_single_step(F(3, 10), F(10), F(3, 4), F(4), I4(10), F(2, 3, 4),
                                            F(3, 4), 8, 32, q),
     "Unexpected array dimensions"),
    (lambda k, q: k.compute_number_of_private_copies(F(3), 10, 3, 4, 1.5, 32),
     "Expecting a fraction strictly between 0 and 1"),
    (lambda k, q: k.kmeans_lloyd_driver(F(3, 10), F(10), F(3, 4), I4(10), F(3, 4), 1e-4, False,
                                        10, 8, 32, 1.0, q),
     "Fraction `centroids_private_copies_max_cache_occupancy` is out of bounds"),
    (lambda k, q: k.kmeans_lloyd_driver(F(3, 10), F(10), F(3, 4), I4(10), F(3, 4), -1.0, False,
                                        10, 8, 32, 0.5, q),
     "Tolerance must be non-negative"),
    (lambda k, q: k.kmeans_lloyd_driver(F(3, 10), D(10), F(3, 4), I4(10), F(3, 4), 1e-4, False,
                                        10, 8, 32, 0.5, q),
     "Sample coordinates, weights and centroids must have the same elemental data types"),
])
def test_python_surface_validation_messages(call, msg):
    import kmeans_dpcpp_gb300 as kdp

    with pytest.raises(ValueError) as ei:
        call(kdp, FakeStream())
    assert str(ei.value) == msg


def test_driver_rejects_unknown_form():
    import kmeans_dpcpp_gb300 as kdp

    with pytest.raises(ValueError) as ei:
        kdp.kmeans_lloyd_driver(F(3, 10), F(10), F(3, 4), I4(10), F(3, 4), 1e-4, False, 10, 8, 32,
                                0.5, FakeStream(), form="int8")
    assert "form must be" in str(ei.value)


def test_compute_threshold_topk_zero_is_noop():
    import kmeans_dpcpp_gb300 as kdp

    ht, ev = kdp.compute_threshold(F(10), 0, F(1), FakeStream())
    ht.wait()
    ev.wait()
    assert ht.is_complete
