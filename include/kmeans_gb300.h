/*
 * kmeans_gb300.h -- C ABI of the GB300 (sm_103a) Lloyd k-means engine.
 *
 * This is the drop-in boundary for the pybind11 surface of kmeans_dpcpp
 * (python_api/_kmeans_lloyd.cpp).  Each entry point replaces one templated
 * SYCL host function that the reference's pybind11 wrappers dispatch to; the
 * comment above each group cites the wrapper (python_api/_kmeans_lloyd.cpp)
 * and the kernel header (a src/ .hpp file) it replaces.
 *
 * Conventions
 *  - All array arguments are device pointers to C-contiguous arrays, in the
 *    layouts of the reference: X_t is (n_features, n_samples), centroid
 *    matrices are (n_features, n_clusters), private copies are
 *    (n_copies, n_features, n_clusters) and (n_copies, n_clusters).
 *  - Suffix _f32/_f64 selects dataT (float/double), _i32/_i64 selects indT.
 *  - `stream` is a cudaStream_t (0 = legacy default stream).  Every call is
 *    asynchronous on that stream unless documented as blocking, exactly like
 *    the reference's submit-and-return-event pattern.
 *  - work_group_size and centroids_window_height are accepted for API
 *    compatibility; the engine picks its own tile shapes.
 *  - Every function returns KMC_OK (0) or a KMC_ERR_* code and never throws;
 *    kmc_last_error() returns a message for the calling thread.
 */
#ifndef KMEANS_GB300_H
#define KMEANS_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st *kmc_stream_t; /* ABI-identical to cudaStream_t */
typedef struct CUevent_st *kmc_event_t;   /* ABI-identical to cudaEvent_t  */

#define KMC_OK 0
#define KMC_ERR_INVALID_ARGUMENT 1
#define KMC_ERR_CUDA 2
#define KMC_ERR_OUT_OF_MEMORY 3
#define KMC_ERR_UNSUPPORTED 4
#define KMC_ERR_DEVICE_TIMEOUT 5
#define KMC_ERR_CANCELLED 6

/* Message describing the last failure on the calling thread. */
const char *kmc_last_error(void);
/* ABI version of this library. */
int kmc_abi_version(void);
/* No counterpart in the reference.  Device scratch (fits, batches, the
 * reference-shaped helpers) comes from a stream-ordered memory pool of this
 * library that keeps freed memory mapped, so the next fit reuses it instead
 * of mapping it again (~9 ms per 4 GB).  This returns the pool's unused memory
 * on every device to the system; memory of live fits is unaffected. */
int kmc_trim_cached_memory(void);
/* No counterpart in the reference.  Bytes of that pool in use by live work
 * on the current device (memory that is mapped but free is not counted). */
int kmc_scratch_bytes_in_use(int64_t *bytes_out);
/* No counterpart in the reference; a test hook of the out-of-memory paths.
 * After this call the (after + 1)-th scratch allocation of the library (any
 * thread, any device) fails as the device's allocator does when memory runs
 * out: the call that asked for it releases what it had taken and returns
 * KMC_ERR_OUT_OF_MEMORY.  The hook fires once; after < 0 disarms it. */
int kmc_debug_fail_allocation(int64_t after);

/* ---- broadcast_divide: X /= y column-wise --------------------------------
 * replaces py_broadcast_divide (_kmeans_lloyd.cpp:60-105) ->
 * broadcast_division_kernel (src/util_kernels.hpp:9-41).
 * divident is (n_rows, n_cols), divisor is (n_cols,). */
int kmc_broadcast_divide_f32(float *divident, const float *divisor, int64_t n_rows,
                             int64_t n_cols, int64_t work_group_size, kmc_stream_t stream);
int kmc_broadcast_divide_f64(double *divident, const double *divisor, int64_t n_rows,
                             int64_t n_cols, int64_t work_group_size, kmc_stream_t stream);

/* ---- half_l2_norm_squared: y[j] = sum_f X[f,j]^2 / 2 -----------------------
 * replaces py_half_l2_norm_squared (_kmeans_lloyd.cpp:108-152) ->
 * half_l2_norm_kernel (src/util_kernels.hpp:47-82). */
int kmc_half_l2_norm_squared_f32(const float *centroids, float *out, int64_t n_features,
                                 int64_t n_clusters, int64_t work_group_size,
                                 kmc_stream_t stream);
int kmc_half_l2_norm_squared_f64(const double *centroids, double *out, int64_t n_features,
                                 int64_t n_clusters, int64_t work_group_size,
                                 kmc_stream_t stream);

/* ---- reduce_centroids_data -------------------------------------------------
 * replaces py_reduce_centroids_data (_kmeans_lloyd.cpp:155-282) ->
 * reduce_centroid_data_kernel (src/util_kernels.hpp:87-161).
 * Empty clusters are appended to out_empty_clusters_list starting at the
 * current value of *out_n_empty_clusters, in ascending cluster order. */
int kmc_reduce_centroids_data_f32_i32(const float *cluster_sizes_private_copies,
                                      const float *centroids_t_private_copies,
                                      float *out_cluster_sizes, float *out_centroids_t,
                                      int32_t *out_empty_clusters_list,
                                      int32_t *out_n_empty_clusters, int64_t n_copies,
                                      int64_t n_features, int64_t n_clusters,
                                      int64_t work_group_size, kmc_stream_t stream);
int kmc_reduce_centroids_data_f32_i64(const float *cluster_sizes_private_copies,
                                      const float *centroids_t_private_copies,
                                      float *out_cluster_sizes, float *out_centroids_t,
                                      int64_t *out_empty_clusters_list,
                                      int64_t *out_n_empty_clusters, int64_t n_copies,
                                      int64_t n_features, int64_t n_clusters,
                                      int64_t work_group_size, kmc_stream_t stream);
int kmc_reduce_centroids_data_f64_i32(const double *cluster_sizes_private_copies,
                                      const double *centroids_t_private_copies,
                                      double *out_cluster_sizes, double *out_centroids_t,
                                      int32_t *out_empty_clusters_list,
                                      int32_t *out_n_empty_clusters, int64_t n_copies,
                                      int64_t n_features, int64_t n_clusters,
                                      int64_t work_group_size, kmc_stream_t stream);
int kmc_reduce_centroids_data_f64_i64(const double *cluster_sizes_private_copies,
                                      const double *centroids_t_private_copies,
                                      double *out_cluster_sizes, double *out_centroids_t,
                                      int64_t *out_empty_clusters_list,
                                      int64_t *out_n_empty_clusters, int64_t n_copies,
                                      int64_t n_features, int64_t n_clusters,
                                      int64_t work_group_size, kmc_stream_t stream);

/* ---- compute_threshold: topk-th largest element of data ---------------------
 * replaces py_compute_threshold (_kmeans_lloyd.cpp:284-337) ->
 * compute_threshold_kernel (src/util_kernels.hpp:163-206) and the
 * iterative_merge_sort it calls (src/iterative_merge_sort.hpp:204-368),
 * by a radix select.  topk == 0 is a no-op, as in the reference. */
int kmc_compute_threshold_f32(const float *data, int64_t n_samples, int64_t topk,
                              float *threshold, kmc_stream_t stream);
int kmc_compute_threshold_f64(const double *data, int64_t n_samples, int64_t topk,
                              double *threshold, kmc_stream_t stream);

/* ---- select_samples_far_from_centroid ---------------------------------------
 * replaces py_select_samples_far_from_centroid (_kmeans_lloyd.cpp:339-441) ->
 * select_samples_far_from_centroid_kernel (src/util_kernels.hpp:211-297).
 * Indices with distance > threshold go to the front (ordered so that
 * selected[n_gt-1-r] is the r-th farthest, ties by lowest index), indices with
 * distance == threshold go to the back (selected[n-1], selected[n-2], ... in
 * ascending index order).  The counters are incremented from their current
 * values, as in the reference. */
int kmc_select_samples_far_from_centroid_f32_i32(int64_t n_selected,
                                                 const float *distance_to_centroid,
                                                 const float *threshold,
                                                 int32_t *selected_samples_idx,
                                                 int32_t *n_selected_gt_threshold,
                                                 int32_t *n_selected_eq_threshold,
                                                 int64_t n_samples, int64_t work_group_size,
                                                 kmc_stream_t stream);
int kmc_select_samples_far_from_centroid_f32_i64(int64_t n_selected,
                                                 const float *distance_to_centroid,
                                                 const float *threshold,
                                                 int64_t *selected_samples_idx,
                                                 int64_t *n_selected_gt_threshold,
                                                 int64_t *n_selected_eq_threshold,
                                                 int64_t n_samples, int64_t work_group_size,
                                                 kmc_stream_t stream);
int kmc_select_samples_far_from_centroid_f64_i32(int64_t n_selected,
                                                 const double *distance_to_centroid,
                                                 const double *threshold,
                                                 int32_t *selected_samples_idx,
                                                 int32_t *n_selected_gt_threshold,
                                                 int32_t *n_selected_eq_threshold,
                                                 int64_t n_samples, int64_t work_group_size,
                                                 kmc_stream_t stream);
int kmc_select_samples_far_from_centroid_f64_i64(int64_t n_selected,
                                                 const double *distance_to_centroid,
                                                 const double *threshold,
                                                 int64_t *selected_samples_idx,
                                                 int64_t *n_selected_gt_threshold,
                                                 int64_t *n_selected_eq_threshold,
                                                 int64_t n_samples, int64_t work_group_size,
                                                 kmc_stream_t stream);

/* ---- allocation-free select_samples_far_from_centroid (float32 / int32) -----
 * No counterpart in the reference: an extra entry point of this library for
 * callers that must not allocate device memory during the call.  Same
 * arguments, results and errors as kmc_select_samples_far_from_centroid_f32_i32,
 * but its scratch is a static device array sized for n_selected <= 4096;
 * larger n_selected is rejected with KMC_ERR_INVALID_ARGUMENT.  It makes no
 * cudaMalloc / cudaFree or other allocating call.  Calls whose kernels overlap
 * on the same device (other streams or host threads) race on the shared
 * scratch.  The first call on a device looks the array up with
 * cudaGetSymbolAddress; make it before any stream capture.  The address is
 * kept per device and context, so after a device reset the next call looks
 * it up again (again before any capture). */
int kmc_select_samples_far_from_centroid_noalloc_f32_i32(int64_t n_selected,
                                                         const float *distance_to_centroid,
                                                         const float *threshold,
                                                         int32_t *selected_samples_idx,
                                                         int32_t *n_selected_gt_threshold,
                                                         int32_t *n_selected_eq_threshold,
                                                         int64_t n_samples,
                                                         int64_t work_group_size,
                                                         kmc_stream_t stream);

/* ---- relocate_empty_clusters --------------------------------------------------
 * replaces py_relocate_empty_clusters (_kmeans_lloyd.cpp:443-589) ->
 * relocate_empty_clusters (src/util_kernels.hpp:392-476): threshold, select,
 * relocate.  Empty cluster r (in list order) takes the r-th farthest sample by
 * sq_dist_to_nearest_centroid (ties by lowest sample index). */
int kmc_relocate_empty_clusters_f32_i32(int64_t n_empty_clusters, const float *X_t,
                                        const float *sample_weights,
                                        const int32_t *assignment_id,
                                        const int32_t *empty_clusters_list,
                                        const float *sq_dist_to_nearest_centroid,
                                        float *centroid_t, float *cluster_sizes,
                                        float *per_sample_inertia, int64_t n_samples,
                                        int64_t n_features, int64_t n_clusters,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_relocate_empty_clusters_f32_i64(int64_t n_empty_clusters, const float *X_t,
                                        const float *sample_weights,
                                        const int64_t *assignment_id,
                                        const int64_t *empty_clusters_list,
                                        const float *sq_dist_to_nearest_centroid,
                                        float *centroid_t, float *cluster_sizes,
                                        float *per_sample_inertia, int64_t n_samples,
                                        int64_t n_features, int64_t n_clusters,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_relocate_empty_clusters_f64_i32(int64_t n_empty_clusters, const double *X_t,
                                        const double *sample_weights,
                                        const int32_t *assignment_id,
                                        const int32_t *empty_clusters_list,
                                        const double *sq_dist_to_nearest_centroid,
                                        double *centroid_t, double *cluster_sizes,
                                        double *per_sample_inertia, int64_t n_samples,
                                        int64_t n_features, int64_t n_clusters,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_relocate_empty_clusters_f64_i64(int64_t n_empty_clusters, const double *X_t,
                                        const double *sample_weights,
                                        const int64_t *assignment_id,
                                        const int64_t *empty_clusters_list,
                                        const double *sq_dist_to_nearest_centroid,
                                        double *centroid_t, double *cluster_sizes,
                                        double *per_sample_inertia, int64_t n_samples,
                                        int64_t n_features, int64_t n_clusters,
                                        int64_t work_group_size, kmc_stream_t stream);

/* ---- compute_centroid_shifts_squared: out[j] = sum_f (old[f,j]-new[f,j])^2 ---
 * replaces py_compute_centroid_shifts_squared_kernel (_kmeans_lloyd.cpp:591-664)
 * -> compute_centroid_shifts_squared_kernel (src/util_kernels.hpp:481-516). */
int kmc_compute_centroid_shifts_squared_f32(const float *centroid_t,
                                            const float *new_centroid_t,
                                            float *out_centroid_shifts, int64_t n_features,
                                            int64_t n_clusters, kmc_stream_t stream);
int kmc_compute_centroid_shifts_squared_f64(const double *centroid_t,
                                            const double *new_centroid_t,
                                            double *out_centroid_shifts, int64_t n_features,
                                            int64_t n_clusters, kmc_stream_t stream);

/* ---- compute_centroid_to_sample_distances: (n_clusters, n_samples) ----------
 * replaces py_compute_distances (_kmeans_lloyd.cpp:666-745) ->
 * compute_distances (src/compute_euclidean_distance.hpp:12-114). */
int kmc_compute_centroid_to_sample_distances_f32(const float *X_t, const float *centroid_t,
                                                 float *euclidean_distances_t,
                                                 int64_t n_samples, int64_t n_features,
                                                 int64_t n_clusters, int64_t work_group_size,
                                                 int64_t centroids_window_height,
                                                 kmc_stream_t stream);
int kmc_compute_centroid_to_sample_distances_f64(const double *X_t, const double *centroid_t,
                                                 double *euclidean_distances_t,
                                                 int64_t n_samples, int64_t n_features,
                                                 int64_t n_clusters, int64_t work_group_size,
                                                 int64_t centroids_window_height,
                                                 kmc_stream_t stream);

/* ---- assignment: labels of the nearest centroid -------------------------------
 * replaces py_assignment (_kmeans_lloyd.cpp:747-839) -> assignment
 * (src/assignment.hpp:11-146). */
int kmc_assignment_f32_i32(const float *X_t, const float *centroids_t,
                           const float *centroids_half_l2_norm, int32_t *assignment_id,
                           int64_t n_samples, int64_t n_features, int64_t n_clusters,
                           int64_t centroids_window_height, int64_t work_group_size,
                           kmc_stream_t stream);
int kmc_assignment_f32_i64(const float *X_t, const float *centroids_t,
                           const float *centroids_half_l2_norm, int64_t *assignment_id,
                           int64_t n_samples, int64_t n_features, int64_t n_clusters,
                           int64_t centroids_window_height, int64_t work_group_size,
                           kmc_stream_t stream);
int kmc_assignment_f64_i32(const double *X_t, const double *centroids_t,
                           const double *centroids_half_l2_norm, int32_t *assignment_id,
                           int64_t n_samples, int64_t n_features, int64_t n_clusters,
                           int64_t centroids_window_height, int64_t work_group_size,
                           kmc_stream_t stream);
int kmc_assignment_f64_i64(const double *X_t, const double *centroids_t,
                           const double *centroids_half_l2_norm, int64_t *assignment_id,
                           int64_t n_samples, int64_t n_features, int64_t n_clusters,
                           int64_t centroids_window_height, int64_t work_group_size,
                           kmc_stream_t stream);

/* ---- compute_inertia: out[i] = w[i] * ||x_i - c_label(i)||^2 ----------------
 * replaces py_compute_inertia (_kmeans_lloyd.cpp:841-939) ->
 * compute_inertia_kernel (src/compute_inertia.hpp:11-53). */
int kmc_compute_inertia_f32_i32(const float *X_t, const float *sample_weight,
                                const float *centroid_t, const int32_t *assignment_id,
                                float *per_sample_inertia, int64_t n_samples,
                                int64_t n_features, int64_t n_clusters,
                                int64_t work_group_size, kmc_stream_t stream);
int kmc_compute_inertia_f32_i64(const float *X_t, const float *sample_weight,
                                const float *centroid_t, const int64_t *assignment_id,
                                float *per_sample_inertia, int64_t n_samples,
                                int64_t n_features, int64_t n_clusters,
                                int64_t work_group_size, kmc_stream_t stream);
int kmc_compute_inertia_f64_i32(const double *X_t, const double *sample_weight,
                                const double *centroid_t, const int32_t *assignment_id,
                                double *per_sample_inertia, int64_t n_samples,
                                int64_t n_features, int64_t n_clusters,
                                int64_t work_group_size, kmc_stream_t stream);
int kmc_compute_inertia_f64_i64(const double *X_t, const double *sample_weight,
                                const double *centroid_t, const int64_t *assignment_id,
                                double *per_sample_inertia, int64_t n_samples,
                                int64_t n_features, int64_t n_clusters,
                                int64_t work_group_size, kmc_stream_t stream);

/* ---- reduce_vector_blocking: blocking sum of a vector ------------------------
 * replaces py_reduce_vector_blocking (_kmeans_lloyd.cpp:941-976) ->
 * reduce_vector_kernel_blocking (src/compute_inertia.hpp:104-135).
 * The sum is accumulated in float64 and rounded once to dataT.  Blocks until
 * the result is on the host. */
int kmc_reduce_vector_blocking_f32(const float *data, int64_t n, kmc_stream_t stream,
                                   float *result);
int kmc_reduce_vector_blocking_f64(const double *data, int64_t n, kmc_stream_t stream,
                                   double *result);

/* ---- fused_lloyd_single_step ----------------------------------------------------
 * replaces py_fused_lloyd_single_step (_kmeans_lloyd.cpp:980-1109) ->
 * lloyd_single_step (src/lloyd_single_step.hpp:37-209).  Labels are written;
 * w*x and w are ADDED into the caller-zeroed private copies. */
int kmc_fused_lloyd_single_step_f32_i32(const float *X_t, const float *sample_weight,
                                        const float *centroids_t,
                                        const float *centroids_half_l2_norm,
                                        int32_t *assignments_idx,
                                        float *new_centroids_t_private_copies,
                                        float *cluster_sizes_private_copies,
                                        int64_t n_samples, int64_t n_features,
                                        int64_t n_clusters, int64_t n_copies,
                                        int64_t centroids_window_height,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_fused_lloyd_single_step_f32_i64(const float *X_t, const float *sample_weight,
                                        const float *centroids_t,
                                        const float *centroids_half_l2_norm,
                                        int64_t *assignments_idx,
                                        float *new_centroids_t_private_copies,
                                        float *cluster_sizes_private_copies,
                                        int64_t n_samples, int64_t n_features,
                                        int64_t n_clusters, int64_t n_copies,
                                        int64_t centroids_window_height,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_fused_lloyd_single_step_f64_i32(const double *X_t, const double *sample_weight,
                                        const double *centroids_t,
                                        const double *centroids_half_l2_norm,
                                        int32_t *assignments_idx,
                                        double *new_centroids_t_private_copies,
                                        double *cluster_sizes_private_copies,
                                        int64_t n_samples, int64_t n_features,
                                        int64_t n_clusters, int64_t n_copies,
                                        int64_t centroids_window_height,
                                        int64_t work_group_size, kmc_stream_t stream);
int kmc_fused_lloyd_single_step_f64_i64(const double *X_t, const double *sample_weight,
                                        const double *centroids_t,
                                        const double *centroids_half_l2_norm,
                                        int64_t *assignments_idx,
                                        double *new_centroids_t_private_copies,
                                        double *cluster_sizes_private_copies,
                                        int64_t n_samples, int64_t n_features,
                                        int64_t n_clusters, int64_t n_copies,
                                        int64_t centroids_window_height,
                                        int64_t work_group_size, kmc_stream_t stream);

/* ---- compute_number_of_private_copies ---------------------------------------------
 * replaces py_compute_number_of_private_copies (_kmeans_lloyd.cpp:1111-1147) ->
 * compute_number_of_private_copies (src/lloyd_single_step.hpp:12-35).
 * element_size is sizeof(dataT); l2_cache_bytes <= 0 queries the current
 * device.  Pure host arithmetic otherwise. */
int kmc_compute_number_of_private_copies(int64_t element_size, int64_t n_samples,
                                         int64_t n_features, int64_t n_clusters,
                                         double centroids_private_copies_max_cache_occupancy,
                                         int64_t work_group_size, int64_t l2_cache_bytes,
                                         int64_t *n_copies_out);

/* ---- kmeans_lloyd_driver -----------------------------------------------------------
 * replaces py_kmeans_lloyd_driver (_kmeans_lloyd.cpp:1149-1275) -> driver_lloyd
 * (src/kmeans_lloyd_driver.hpp:21-431).  Blocking.  init_centroids_t is
 * overwritten (the two centroid buffers ping-pong).  The convergence sum and
 * the returned inertia are accumulated in float64 and rounded to dataT.
 * print_fn receives the verbose per-iteration lines (may be NULL). */
typedef void (*kmc_print_fn)(const char *line, void *ctx);
int kmc_lloyd_driver_f32_i32(const float *X_t, const float *sample_weight,
                             float *init_centroids_t, int32_t *assignment_id,
                             float *res_centroids_t, int64_t n_samples, int64_t n_features,
                             int64_t n_clusters, double tol, int verbose, int64_t max_iter,
                             int64_t centroids_window_height, int64_t work_group_size,
                             double centroids_private_copies_max_cache_occupancy,
                             kmc_stream_t stream, kmc_print_fn print_fn, void *print_ctx,
                             int64_t *n_iters_out, float *total_inertia_out);
int kmc_lloyd_driver_f32_i64(const float *X_t, const float *sample_weight,
                             float *init_centroids_t, int64_t *assignment_id,
                             float *res_centroids_t, int64_t n_samples, int64_t n_features,
                             int64_t n_clusters, double tol, int verbose, int64_t max_iter,
                             int64_t centroids_window_height, int64_t work_group_size,
                             double centroids_private_copies_max_cache_occupancy,
                             kmc_stream_t stream, kmc_print_fn print_fn, void *print_ctx,
                             int64_t *n_iters_out, float *total_inertia_out);
int kmc_lloyd_driver_f64_i32(const double *X_t, const double *sample_weight,
                             double *init_centroids_t, int32_t *assignment_id,
                             double *res_centroids_t, int64_t n_samples, int64_t n_features,
                             int64_t n_clusters, double tol, int verbose, int64_t max_iter,
                             int64_t centroids_window_height, int64_t work_group_size,
                             double centroids_private_copies_max_cache_occupancy,
                             kmc_stream_t stream, kmc_print_fn print_fn, void *print_ctx,
                             int64_t *n_iters_out, double *total_inertia_out);
int kmc_lloyd_driver_f64_i64(const double *X_t, const double *sample_weight,
                             double *init_centroids_t, int64_t *assignment_id,
                             double *res_centroids_t, int64_t n_samples, int64_t n_features,
                             int64_t n_clusters, double tol, int verbose, int64_t max_iter,
                             int64_t centroids_window_height, int64_t work_group_size,
                             double centroids_private_copies_max_cache_occupancy,
                             kmc_stream_t stream, kmc_print_fn print_fn, void *print_ctx,
                             int64_t *n_iters_out, double *total_inertia_out);

/* ---- fit sessions: the driver loop of driver_lloyd (src/kmeans_lloyd_driver.hpp:
 * 83-354) as a resumable handle.  kmeans_lloyd_driver is create + run +
 * finalize + destroy.  A session keeps data, centroids and loop state on the
 * device; kmc_fit_step enqueues iterations without host synchronisation (the
 * GPU stops the loop itself once tol or max_iter is reached).
 * form: KMC_FORM_PLAIN (exact dataT arithmetic, the reference's) or a mixed
 * tensor-core form (float32 data, n_features <= 256, any n_clusters; the
 * labels are the exact float32 ones, KMC_ERR_UNSUPPORTED beyond 256 features). */
typedef struct kmc_fit_s *kmc_fit_t;
#define KMC_FORM_PLAIN 0
#define KMC_FORM_MIXED_BF16 1
#define KMC_FORM_MIXED_FP16 2
int kmc_fit_create_f32_i32(const float *X_t, const float *sample_weight, float *centroids_t,
                           int32_t *assignment_id, float *res_centroids_t, int64_t n_samples,
                           int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                           int form, kmc_stream_t stream, kmc_fit_t *fit_out);
int kmc_fit_create_f32_i64(const float *X_t, const float *sample_weight, float *centroids_t,
                           int64_t *assignment_id, float *res_centroids_t, int64_t n_samples,
                           int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                           int form, kmc_stream_t stream, kmc_fit_t *fit_out);
int kmc_fit_create_f64_i32(const double *X_t, const double *sample_weight, double *centroids_t,
                           int32_t *assignment_id, double *res_centroids_t, int64_t n_samples,
                           int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                           int form, kmc_stream_t stream, kmc_fit_t *fit_out);
int kmc_fit_create_f64_i64(const double *X_t, const double *sample_weight, double *centroids_t,
                           int64_t *assignment_id, double *res_centroids_t, int64_t n_samples,
                           int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                           int form, kmc_stream_t stream, kmc_fit_t *fit_out);
/* Row-major input.  No counterpart in the reference, whose entry points take
 * feature-major X_t (n_features, n_samples) only: the same fit session for X
 * given as (n_samples, n_features) C-contiguous, other arguments as above.
 * The mixed forms read it directly in their one-time operand conversion (no
 * transposed copy is made); the plain form makes one feature-major copy on
 * the device. */
int kmc_fit_create_rowmajor_f32_i32(const float *X, const float *sample_weight,
                                    float *centroids_t, int32_t *assignment_id,
                                    float *res_centroids_t, int64_t n_samples,
                                    int64_t n_features, int64_t n_clusters, double tol,
                                    int64_t max_iter, int form, kmc_stream_t stream,
                                    kmc_fit_t *fit_out);
int kmc_fit_create_rowmajor_f32_i64(const float *X, const float *sample_weight,
                                    float *centroids_t, int64_t *assignment_id,
                                    float *res_centroids_t, int64_t n_samples,
                                    int64_t n_features, int64_t n_clusters, double tol,
                                    int64_t max_iter, int form, kmc_stream_t stream,
                                    kmc_fit_t *fit_out);
int kmc_fit_create_rowmajor_f64_i32(const double *X, const double *sample_weight,
                                    double *centroids_t, int32_t *assignment_id,
                                    double *res_centroids_t, int64_t n_samples,
                                    int64_t n_features, int64_t n_clusters, double tol,
                                    int64_t max_iter, int form, kmc_stream_t stream,
                                    kmc_fit_t *fit_out);
int kmc_fit_create_rowmajor_f64_i64(const double *X, const double *sample_weight,
                                    double *centroids_t, int64_t *assignment_id,
                                    double *res_centroids_t, int64_t n_samples,
                                    int64_t n_features, int64_t n_clusters, double tol,
                                    int64_t max_iter, int form, kmc_stream_t stream,
                                    kmc_fit_t *fit_out);
/* Enqueue n_iterations iterations (asynchronous; no-ops once the loop stopped). */
int kmc_fit_step(kmc_fit_t fit, int64_t n_iterations);
/* Run to convergence (blocking). */
int kmc_fit_run(kmc_fit_t fit);
/* Blocking read of the loop state. */
int kmc_fit_status(kmc_fit_t fit, int64_t *n_iter_out, int *done_out, double *last_shift_out);
/* Final assignment + inertia against the current centroids (blocking). */
int kmc_fit_finalize(kmc_fit_t fit, int64_t *n_iter_out, double *total_inertia_out);
/* Per-phase CUDA-event timing (off by default): phase 0 is the assignment +
 * accumulation kernel of every iteration.  Times are summed over recorded
 * iterations; reading them synchronises the stream. */
int kmc_fit_set_profiling(kmc_fit_t fit, int enable);
int kmc_fit_phase_time(kmc_fit_t fit, int phase, double *total_ms_out, int64_t *count_out);
/* Mixed forms: samples whose tensor-core margin did not certify their label
 * and were re-evaluated in exact float32 (last pass and running total), and
 * the device-side error flag of the tensor-core kernel (1 after a bounded
 * wait timed out).  Plain form: zeros.  Blocking. */
int kmc_fit_rechecked(kmc_fit_t fit, int64_t *last_out, int64_t *total_out, int *device_error_out);
/* No counterpart in the reference.  Limit, in SM clocks, of every
 * device-side wait of the tensor-core kernels of a mixed-form session
 * (clocks <= 0 restores the default, 4e9 clocks or about two seconds).  A
 * wait that runs out makes the kernel wind down (it waits for the copies and
 * tensor-core operations it issued, frees its tensor memory) and stops the
 * loop; the next blocking call (kmc_fit_run, kmc_fit_status,
 * kmc_fit_finalize) returns KMC_ERR_DEVICE_TIMEOUT and kmc_fit_rechecked
 * reports device_error = 1.  stall_once = 1 makes the next assignment pass
 * first wait on a barrier that nothing completes, so that this wait runs out
 * after `clocks`: a test of the timeout path that faults and hangs nothing.
 * The plain form has no device-side waits and ignores both. */
int kmc_fit_set_wait_limit(kmc_fit_t fit, int64_t clocks, int stall_once);
/* No counterpart in the reference (whose kernels take a window height and a
 * work-group size as arguments).  The plain form's kernels choose their
 * centroid-tile width themselves: the first fit of a (n_features, power-of-two
 * bucket of n_clusters, dtype) times each width (128 / 64 / 32 centroids for
 * float32, 64 / 32 for float64) on a synthetic instance and caches the fastest
 * in memory and in $KMC_TILE_CACHE (default $XDG_CACHE_HOME or ~/.cache,
 * kmeans_gb300/tiles.txt); KMC_TUNE=0 turns the search off.  Every width gives
 * the same labels.  kmc_fit_tile_variant returns (tuning if needed) the choice
 * (0, 1, 2) for dtype_bytes 4 or 8; kmc_fit_set_tile_variant overrides a
 * session's. */
int kmc_fit_tile_variant(int64_t n_features, int64_t n_clusters, int dtype_bytes,
                         kmc_stream_t stream, int *variant_out);
int kmc_fit_set_tile_variant(kmc_fit_t fit, int variant);
/* Mixed forms: the session's kernel variant, 10 * ring stages + f, where f = 4
 * or 2 is the fixed-point cluster sums with that many columns per update
 * thread and f = 0 the float reductions (-1 for a plain session).  The
 * autotuner times the variants that fit shared memory on a synthetic fit once
 * per (n_features, power-of-two bucket of n_clusters, form, size class: at
 * least 32 128-sample tiles per SM or fewer), caches the fastest beside the
 * tile choices above (KMC_TUNE=0: the deepest ring with the widest
 * fixed-point sums).  Sessions of the request server use a cached choice or
 * that default and never time variants on a request's path.  Every variant gives the same labels.
 * kmc_debug_force_mixed_variant forces a variant for the fits created
 * afterwards (a test hook; -1 restores the tuner; a variant that does not fit
 * a shape fails that fit with KMC_ERR_INVALID_ARGUMENT).  No reference
 * counterpart. */
int kmc_fit_mixed_variant(kmc_fit_t fit, int *variant_out);
int kmc_debug_force_mixed_variant(int variant);
/* The packed fixed-point term the mixed forms use for the cluster sums up to
 * 32 features (host copy of the packing, for tests; no GPU involved): for
 * value = +-m 2^(E - 150) (E its exponent field, m its 24-bit mantissa) and
 * scale 2^shift, packed = (+-m) << 6 | (E - 150 + shift) << 1 when that shift
 * is 0..30 (then value 2^shift = +-m 2^(E - 150 + shift) exactly), 0 for a
 * zero, and the flag 1 otherwise (too small for the scale, denormal, infinite,
 * NaN).  No reference counterpart. */
int kmc_debug_pack_fixed(float value, int shift, int *packed_out);
/* Kernel launches enqueued so far by this session. */
int kmc_fit_launch_count(kmc_fit_t fit, int64_t *launches_out);
int kmc_fit_destroy(kmc_fit_t fit);

/* ---- input layout and initialisation -----------------------------------------------
 * No counterpart in the reference, which takes the feature-major X_t and the
 * initial centroids as given (_kmeans_lloyd.cpp:1153); these are the steps
 * before its path.  kmc_transpose_* turns row-major X (n_samples, n_features)
 * into X_t (n_features, n_samples).  kmc_gather_rows_* copies the given rows
 * of X_t into centroids_t (random-row initialisation; rows in [0, n)).
 * kmc_kmeans_plusplus_* seeds k centroids by D^2 sampling on the device,
 * deterministic for a seed (sample_weight may be NULL); chosen_rows receives
 * the k sample indices. */
int kmc_transpose_f32(const float *X, float *X_t, int64_t n_samples, int64_t n_features,
                      kmc_stream_t stream);
int kmc_transpose_f64(const double *X, double *X_t, int64_t n_samples, int64_t n_features,
                      kmc_stream_t stream);
int kmc_gather_rows_f32(const float *X_t, int64_t n_samples, int64_t n_features,
                        const int32_t *rows, int64_t n_clusters, float *centroids_t,
                        kmc_stream_t stream);
int kmc_gather_rows_f64(const double *X_t, int64_t n_samples, int64_t n_features,
                        const int32_t *rows, int64_t n_clusters, double *centroids_t,
                        kmc_stream_t stream);
/* Mean over features of each feature's population variance (float64; the
 * scale scikit-learn's Lloyd engine applies to tol). */
int kmc_mean_feature_variance_f32(const float *X_t, int64_t n_samples, int64_t n_features,
                                  double *mean_variance_out, kmc_stream_t stream);
int kmc_mean_feature_variance_f64(const double *X_t, int64_t n_samples, int64_t n_features,
                                  double *mean_variance_out, kmc_stream_t stream);
int kmc_kmeans_plusplus_f32(const float *X_t, const float *sample_weight, int64_t n_samples,
                            int64_t n_features, int64_t n_clusters, uint64_t seed,
                            float *centroids_t, int32_t *chosen_rows, kmc_stream_t stream);
int kmc_kmeans_plusplus_f64(const double *X_t, const double *sample_weight, int64_t n_samples,
                            int64_t n_features, int64_t n_clusters, uint64_t seed,
                            double *centroids_t, int32_t *chosen_rows, kmc_stream_t stream);

/* ---- batched fits ------------------------------------------------------------------
 * No counterpart in the reference.  Many independent float32 fits and
 * label-only predictions of uneven (n, d, k) advance together, one Lloyd
 * iteration per kmc_batch_step, through per-phase kernels fed by a device work
 * queue and replayed as CUDA graphs.
 * Each fit follows kmeans_lloyd_driver's semantics (stop rule, empty-cluster
 * relocation, final assignment and inertia) with the plain form's arithmetic:
 * labels equal a single plain fit's, centroids and inertia agree to float64
 * summation order.  The caller owns X_t, sample_weight, centroids_t (initial
 * centroids in, final centroids out) and labels until the instance is
 * removed.  d <= 1024, k <= 4096. */
typedef struct kmc_batch_s *kmc_batch_t;
int kmc_batch_create(int64_t max_instances, kmc_stream_t stream, kmc_batch_t *batch_out);
int kmc_batch_add_fit_f32(kmc_batch_t batch, const float *X_t, const float *sample_weight,
                          float *centroids_t, int32_t *labels, int64_t n_samples,
                          int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                          int64_t *instance_out);
int kmc_batch_add_predict_f32(kmc_batch_t batch, const float *X_t, const float *centroids_t,
                              int32_t *labels, int64_t n_samples, int64_t n_features,
                              int64_t n_clusters, int64_t *instance_out);
/* Batched transform: the (n_clusters, n_samples) Euclidean distances of
 * compute_centroid_to_sample_distances (compute_euclidean_distance.hpp:
 * 12-114, the intended full result) into `distances`, computed in the next
 * engine step by the same persistent tiles as the assignments (bit-equal to
 * kmc_compute_centroid_to_sample_distances_f32). */
int kmc_batch_add_transform_f32(kmc_batch_t batch, const float *X_t, const float *centroids_t,
                                float *distances, int64_t n_samples, int64_t n_features,
                                int64_t n_clusters, int64_t *instance_out);
/* One engine step; *n_active_out = instances still running afterwards. */
int kmc_batch_step(kmc_batch_t batch, int64_t *n_active_out);
/* Steps until every instance has finished. */
int kmc_batch_run(kmc_batch_t batch);
int kmc_batch_result(kmc_batch_t batch, int64_t instance, int *finished_out,
                     int64_t *n_iter_out, double *inertia_out);
int kmc_batch_remove(kmc_batch_t batch, int64_t instance);
int kmc_batch_stats(kmc_batch_t batch, int64_t *steps_out, int64_t *graph_builds_out,
                    int64_t *relocations_out);
int kmc_batch_destroy(kmc_batch_t batch);
/* Tile autotuner: centroid-window variant (0: 32, 1: 64, 2: 128 columns) the
 * batched assignment uses for (d, k, float32); measured once, cached. */
int kmc_tile_variant(int64_t n_features, int64_t n_clusters, kmc_stream_t stream,
                     int *variant_out);
/* Seeded synthetic Gaussian blobs written on the device, X_t (d, n). */
int kmc_generate_blobs_f32(float *X_t, int64_t n_samples, int64_t n_features,
                           int64_t n_centers, float box_lo, float box_hi, float std_lo,
                           float std_hi, uint64_t seed, kmc_stream_t stream);
/* Seeded distinct row indices for random-row initialisation (host). */
int kmc_seeded_rows(int64_t n_samples, int64_t n_clusters, uint64_t seed, int32_t *rows_out);
/* The batched engine's work items for instances of n_samples[q] samples, mode
 * modes[q] (0 fit, 1 assign, 2 transform) and tile variant variants[q] (host
 * planning only, for tests): runs of at most 8 128-sample tiles, listed by
 * group (kind * 3 + variant; kind 1 = transforms) in instance order.  Writes up
 * to `capacity` items and the total count.  No reference counterpart. */
int kmc_debug_batch_items(int64_t count, const int64_t *n_samples, const int *modes,
                          const int *variants, int64_t capacity, int32_t *instance_out,
                          int32_t *tiles_out, int64_t *first_tile_out, int32_t *group_out,
                          int64_t *n_items_out);

/* ---- serving loop ------------------------------------------------------------------
 * No counterpart in the reference.  Replays a stream of fit and predict
 * requests against the engine with continuous batching: a request is
 * admitted at its arrival time as soon as an instance slot is free and the
 * device bytes it needs fit the budget; running fits advance concurrently
 * (in the plain form together, one iteration per engine step); converged fits
 * retire mid-batch and free their memory.
 * Each request's data are seeded Gaussian blobs generated on the device at
 * admission.  form KMC_FORM_PLAIN runs the batched engine; the mixed forms run
 * one tensor-core fit session per request on a pool of streams, each session
 * replaying one captured iteration (a CUDA graph) and advancing on its own.
 * Times are seconds from the start of the replay. */
typedef struct {
    double arrival_s;
    int32_t kind;        /* 0 fit, 1 predict, 2 transform (distances; result.inertia = their float64 sum) */
    int32_t n_features;
    int64_t n_samples;
    int64_t n_clusters;
    int64_t n_centers;   /* blobs of the request's data */
    uint64_t seed;
    double tol;
    int64_t max_iter;
    int64_t model;       /* predict, transform: index of the fit request whose centroids it uses */
    float std_lo, std_hi;
} kmc_serve_request_t;
typedef struct {
    double admit_s;
    double finish_s;
    int64_t n_iter;
    double inertia;
    int32_t status;      /* KMC_OK or an error code */
    int32_t pad;
} kmc_serve_result_t;
/* ---- request server ------------------------------------------------------------------
 * No counterpart in the reference.  Each request is what the reference does per
 * call, on the caller's device buffers: a fit is kmeans_lloyd_driver
 * (_kmeans_lloyd.cpp:1427-1448 -> src/kmeans_lloyd_driver.hpp:21-431, without
 * overwriting the initial centroids), a prediction is assignment
 * (_kmeans_lloyd.cpp:1369-1380) against a fitted model, a transform is
 * compute_centroid_to_sample_distances (_kmeans_lloyd.cpp:1354-1367).
 *
 * kmc_server_open starts a server of one form (KMC_FORM_*) with an HBM budget for
 * the memory it allocates and a limit on running requests.  Submissions return
 * a ticket at once; requests are admitted in submission order while the running
 * count and the budget allow (a prediction waits, without blocking the queue,
 * for the fit whose model it names).  The inputs must have been written on the
 * stream given to kmc_server_open (or be complete before the submission) and
 * stay unchanged until the ticket finishes; the outputs are complete when the
 * ticket reports KMC_REQ_DONE.  A fit's final centroids stay on the device as
 * its model (predictions and transforms name the fit's ticket) until
 * kmc_server_release or kmc_server_close.  The plain form advances all running
 * requests together in the batched engine (bit-equal to single plain fits); the
 * mixed forms run one tensor-core session per request on a pool of streams.
 * A server is driven by its callers: submissions only queue, and
 * kmc_server_poll / kmc_server_wait admit requests and make progress (in the
 * plain form each such step runs one engine iteration of every running
 * request; in the mixed forms it launches work and returns).  Calls on one
 * server must not overlap (one host thread at a time).  A request's own failure is its status (KMC_ERR_OUT_OF_MEMORY when it
 * can never fit the budget, KMC_ERR_CANCELLED, KMC_ERR_DEVICE_TIMEOUT, ...); the
 * functions' return codes report invalid calls and CUDA errors. */
typedef struct kmc_server_s *kmc_server_t;
#define KMC_REQ_PENDING 0
#define KMC_REQ_RUNNING 1
#define KMC_REQ_DONE 2
#define KMC_REQ_FAILED 3
#define KMC_REQ_CANCELLED 4
int kmc_server_open(int form, int64_t hbm_budget_bytes, int64_t max_active, kmc_stream_t stream,
                    kmc_server_t *server_out);
/* X_t (d, n), sample_weight (n), init_centroids_t (d, k) are read; labels_out (n)
 * and centroids_out (d, k) are written. */
int kmc_server_submit_fit_f32(kmc_server_t server, const float *X_t, const float *sample_weight,
                              const float *init_centroids_t, int32_t *labels_out,
                              float *centroids_out, int64_t n_samples, int64_t n_features,
                              int64_t n_clusters, double tol, int64_t max_iter,
                              int64_t *ticket_out);
/* Labels of X_t (d, n) against the model of fit ticket model_ticket (d and k are
 * the model's).  The plain form reports inertia 0; the mixed forms report the
 * unit-weight inertia of the labels. */
int kmc_server_submit_predict_f32(kmc_server_t server, const float *X_t, int64_t model_ticket,
                                  int32_t *labels_out, int64_t n_samples, int64_t *ticket_out);
/* distances_out (k, n) = Euclidean distances to the model's centroids;
 * the result's inertia is their float64 sum. */
int kmc_server_submit_transform_f32(kmc_server_t server, const float *X_t, int64_t model_ticket,
                                    float *distances_out, int64_t n_samples,
                                    int64_t *ticket_out);
/* Makes one step of progress, then reports the ticket's state
 * (KMC_REQ_*) and, once it finished, its status, iterations and inertia. */
int kmc_server_poll(kmc_server_t server, int64_t ticket, int *state_out, int *status_out,
                    int64_t *n_iter_out, double *inertia_out);
/* Drives the server until the ticket finished. */
int kmc_server_wait(kmc_server_t server, int64_t ticket, int *status_out, int64_t *n_iter_out,
                    double *inertia_out);
/* A pending request is dropped; a running one stops after the work it has in
 * flight.  Either ends with status KMC_ERR_CANCELLED (its outputs are then
 * undefined); predictions waiting for a cancelled fit fail.  No effect on a
 * finished ticket. */
int kmc_server_cancel(kmc_server_t server, int64_t ticket);
/* Frees a finished ticket's record and, for a fit, its model. */
int kmc_server_release(kmc_server_t server, int64_t ticket);
int kmc_server_stats(kmc_server_t server, int64_t *pending_out, int64_t *running_out,
                     int64_t *bytes_in_use_out);
/* Cancels what has not finished, waits for the work in flight, frees everything. */
int kmc_server_close(kmc_server_t server);

int kmc_serve_bytes_needed(int32_t kind, int64_t n_samples, int64_t n_features,
                           int64_t n_clusters, int form, int64_t *bytes_out);
int kmc_serve_run(const kmc_serve_request_t *requests, int64_t n_requests, int form,
                  int64_t hbm_budget_bytes, int64_t max_active, kmc_stream_t stream,
                  kmc_serve_result_t *results_out, double *makespan_s_out);

/* ---- events: the (host_task_event, compute_event) pair of the reference ------------
 * The reference returns sycl::event pairs from every wrapper
 * (e.g. _kmeans_lloyd.cpp:102-103) and accepts `depends` lists.  These wrap
 * cudaEvent_t so a host binding can offer the same .wait() / depends. */
int kmc_event_create(kmc_event_t *event_out);
int kmc_event_record(kmc_event_t event, kmc_stream_t stream);
int kmc_event_synchronize(kmc_event_t event);
int kmc_event_query(kmc_event_t event, int *completed_out);
int kmc_stream_wait_event(kmc_stream_t stream, kmc_event_t event);
int kmc_event_destroy(kmc_event_t event);
int kmc_stream_synchronize(kmc_stream_t stream);
/* Device ordinal owning a pointer (-1 for host memory); replaces the
 * reference's queue-compatibility check (_kmeans_lloyd.cpp:46-56). */
int kmc_pointer_device(const void *ptr, int *device_out);
int kmc_current_device(int *device_out);

#ifdef __cplusplus
}
#endif

#endif /* KMEANS_GB300_H */
