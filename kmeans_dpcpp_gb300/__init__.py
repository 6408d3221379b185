"""GB300 (sm_103a) Lloyd k-means engine with the Python surface of kmeans_dpcpp.

The fourteen functions below keep the names, arguments and error behaviour of
``kmeans_dpcpp`` (``kmeans_dpcpp/__init__.py`` / ``python_api/_kmeans_lloyd.cpp``
in the reference).  Arrays are CUDA arrays exposing ``__cuda_array_interface__``
(torch CUDA tensors, CuPy arrays ...); ``sycl_queue`` is a CUDA stream (``None``,
an ``int`` handle or a ``torch.cuda.Stream``).  Every function runs hand-written
sm_103a kernels from ``libkmeans_gb300.so``; there is no CPU fallback: importing
this package fails if the native extension has not been built
(``python -c "import __graft_entry__ as g; g.build()"``).
"""
try:
    from ._kmeans_dpcpp import (  # noqa: F401
        Event,
        broadcast_divide,
        half_l2_norm_squared,
        reduce_centroids_data,
        compute_threshold,
        select_samples_far_from_centroid,
        relocate_empty_clusters,
        compute_centroid_shifts_squared,
        compute_centroid_to_sample_distances,
        assignment,
        compute_inertia,
        reduce_vector_blocking,
        fused_lloyd_single_step,
        compute_number_of_private_copies,
        kmeans_lloyd_driver,
    )
except ImportError as exc:  # pragma: no cover - exercised only without a build
    raise ImportError(
        "kmeans_dpcpp_gb300 native extension is not built; run "
        "`python -c \"import __graft_entry__ as g; g.build()\"` first"
    ) from exc

__all__ = [
    "broadcast_divide",
    "half_l2_norm_squared",
    "reduce_centroids_data",
    "compute_threshold",
    "select_samples_far_from_centroid",
    "relocate_empty_clusters",
    "compute_centroid_shifts_squared",
    "compute_centroid_to_sample_distances",
    "assignment",
    "compute_inertia",
    "reduce_vector_blocking",
    "fused_lloyd_single_step",
    "compute_number_of_private_copies",
    "kmeans_lloyd_driver",
]

# scikit-learn-style estimator over the module (not part of the reference's
# surface, so it stays out of __all__)
from .estimator import KMeans  # noqa: E402,F401

__doc__ += """
This module implements GB300 offloading routines necessary for implementing
Lloyd's algorithm to solve the K-Means problem.
"""
