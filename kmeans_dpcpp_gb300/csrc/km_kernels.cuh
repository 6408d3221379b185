// Host-side launchers for every kernel of the engine.  Each launcher returns a
// KMC_* status.  `guard`, when non-null, points to the device-resident loop
// state of the Lloyd driver: guarded kernels return immediately once the loop
// has stopped, so the driver can enqueue iterations ahead of the convergence
// test without a host round-trip.
#pragma once

#include "km_common.cuh"

namespace kmc {

// Device-resident control block of one Lloyd fit (see driver.cu).
struct LoopState {
    int done;              // 1 once the loop stopped (max_iter or shift <= tol)
    int relocations;       // number of iterations that relocated clusters
    long long n_iter;      // iterations executed
    long long max_iter;
    double tol;            // tol rounded to dataT, widened back to double
    double last_shift;     // float64 total of the last centroid shift
    double last_inertia;   // float64 total of the verbose inertia (if computed)
    unsigned int err;      // device-side error bits
    unsigned int pad;
};

// A kernel of the fit gave up a device-side wait (it then stopped the loop).
inline int check_device_error(const LoopState &s) {
    if (s.err != 0) {
        set_error("a tensor-core kernel of this fit gave up a device-side wait after its time "
                  "limit; the loop was stopped and its results are not valid");
        return KMC_ERR_DEVICE_TIMEOUT;
    }
    return KMC_OK;
}

// Lexicographic (value, index) minimum of each of the TM sample rows a thread
// holds over the 16 threads (lanes differing in bits 0-3, tx = lane & 15) that
// hold the same rows -- the first minimum of a sequential strict-< scan over
// ascending index.  Recursive halving: at offset o the lower thread of a pair
// keeps the first half of its remaining rows and the upper thread the second,
// each combining its own candidate with the partner's for the rows it keeps;
// once one row is left, partners combine it.  Returns the row (0..TM-1) whose
// result this thread ends with in v[0], j[0]; 16 / TM threads end with each
// row, the lowest of them has (tx & (16 / TM - 1)) == 0.  Values are never NaN
// (they come from strict-< updates of +inf).
template <typename T, int TM>
__device__ __forceinline__ int rowmin16(T (&v)[TM], int (&j)[TM], int tx) {
    int base = 0;
    int R = TM;
#pragma unroll
    for (int off = 8; off > 0; off >>= 1) {
        if (R >= 2) {
            const int H = R / 2;
            const bool upper = (tx & off) != 0;
#pragma unroll
            for (int r = 0; r < H; ++r) {
                const T sv = upper ? v[r] : v[r + H];
                const int sj = upper ? j[r] : j[r + H];
                T kv = upper ? v[r + H] : v[r];
                int kj = upper ? j[r + H] : j[r];
                const T ov = __shfl_xor_sync(0xffffffffu, sv, off);
                const int oj = __shfl_xor_sync(0xffffffffu, sj, off);
                if (ov < kv || (ov == kv && oj < kj)) {
                    kv = ov;
                    kj = oj;
                }
                v[r] = kv;
                j[r] = kj;
            }
            if (upper) base += H;
            R = H;
        } else {
            const T ov = __shfl_xor_sync(0xffffffffu, v[0], off);
            const int oj = __shfl_xor_sync(0xffffffffu, j[0], off);
            if (ov < v[0] || (ov == v[0] && oj < j[0])) {
                v[0] = ov;
                j[0] = oj;
            }
        }
    }
    return base;
}

// ---- kernels_util.cu ----
template <typename T>
int launch_broadcast_divide(T *X, const T *y, int64_t rows, int64_t cols, cudaStream_t s);
template <typename T>
int launch_half_norm(const T *C, T *out, int64_t d, int64_t k, cudaStream_t s,
                     const LoopState *guard = nullptr);
// A: accumulator type of the private copies (dataT or double).
template <typename T, typename I, typename A>
int launch_reduce_centroids(const A *sizes_cp, const A *cent_cp, T *out_sizes, T *out_cent,
                            I *empty_list, I *n_empty, int64_t P, int64_t d, int64_t k,
                            cudaStream_t s, const LoopState *guard = nullptr);
// Empty-cluster list in ascending order, appended from *n_empty.
template <typename T, typename I>
int launch_empty_list(const T *sizes, I *list, I *n_empty, int64_t k, cudaStream_t s,
                      const LoopState *guard = nullptr);
template <typename T>
int launch_shifts(const T *old_c, const T *new_c, T *out, int64_t d, int64_t k,
                  cudaStream_t s);
// new_c /= sizes (per cluster), then shifts[j] = sum_f (old_c - new_c)^2.
template <typename T>
int launch_divide_and_shift(const T *old_c, T *new_c, const T *sizes, T *shifts, int64_t d,
                            int64_t k, cudaStream_t s, const LoopState *guard);
// Loop control: float64 total of shifts, n_iter += 1, convergence test.
template <typename T>
int launch_loop_control(const T *shifts, int64_t k, LoopState *state, cudaStream_t s);
// w == nullptr selects the unit-weight variant.  X is feature-major (d, n)
// unless x_fstride > 0: then element (f, i) is X[f * x_fstride + i * x_sstride]
// (a row-major copy has x_fstride = 1, x_sstride = its row length).
template <typename T, typename I>
int launch_inertia(const T *X, const T *w, const T *C, const I *labels, T *out, int64_t n,
                   int64_t d, int64_t k, cudaStream_t s, const LoopState *guard = nullptr,
                   const int64_t *gate = nullptr, int64_t x_fstride = 0, int64_t x_sstride = 1);
// Deterministic float64 sum of n values into *out (device).  `partials` must
// hold sum_partials_size() doubles.
int64_t sum_partials_size();
template <typename T>
int launch_sum_f64(const T *data, int64_t n, double *partials, double *out, cudaStream_t s,
                   const LoopState *guard = nullptr);
template <typename T>
int launch_fill(T *p, T v, int64_t count, cudaStream_t s, const LoopState *guard = nullptr);

// ---- kernels_lloyd.cu : SIMT tiled distance kernels (exact FP32/FP64) ----
// variant: centroid-tile width of the autotuner (0: 16 x the default micro-
// tile width, 1: half of it, 2: 32 columns); every variant computes each
// (sample, centroid) score with the same arithmetic, so labels do not depend
// on it.  Variants 1 and 2 of the fused step exist for float64 accumulators.
template <typename T, typename I>
int launch_assignment(const T *X, const T *C, const T *hn, I *labels, int64_t n, int64_t d,
                      int64_t k, cudaStream_t s, const LoopState *guard = nullptr,
                      int variant = 0);
// A: accumulator type of the private copies (dataT for the public API,
// double inside the driver so sums are rounded to dataT once).
template <typename T, typename I, typename A>
int launch_fused_step(const T *X, const T *w, const T *C, const T *hn, I *labels, A *sums_cp,
                      A *sizes_cp, int64_t n, int64_t d, int64_t k, int64_t P, cudaStream_t s,
                      const LoopState *guard = nullptr, int variant = 0);
// Autotuner of the single-fit tile: times the fused step of each variant on a
// synthetic 65,536-sample instance of (d, power-of-two bucket of k) once and
// caches the fastest (in memory and in the tile cache file).  KMC_TUNE=0 in
// the environment turns it off (variant 0).
template <typename T>
int tune_fit_variant(int64_t d, int64_t k, cudaStream_t s, int *variant);
// The autotuner cache (batch_kernels.cu): choice for (d, k bucket, tag).
bool tune_lookup(int64_t d, int64_t k, const char *tag, int *variant);
void tune_record(int64_t d, int64_t k, const char *tag, int variant);
template <typename T>
int launch_distances(const T *X, const T *C, T *out, int64_t n, int64_t d, int64_t k,
                     cudaStream_t s);

// ---- kernels_reloc.cu : threshold (radix select), selection, relocation ----
// Scratch bytes needed by launch_threshold for n samples.
size_t threshold_scratch_bytes();
template <typename T>
int launch_threshold(const T *data, int64_t n, const int64_t *topk_dev, int64_t topk_host,
                     T *threshold, void *scratch, cudaStream_t s,
                     const LoopState *guard = nullptr);
// Scratch for launch_select; max_selected bounds n_selected.
size_t select_scratch_bytes(int64_t max_selected);
// Kernels launch_select enqueues for a given max_selected.
int64_t select_launches(int64_t max_selected);
// `scratch` holds select_scratch_bytes(max_selected) bytes; n_selected (on the
// device or the host) is at most max_selected.
template <typename T, typename I>
int launch_select(const int64_t *n_selected_dev, int64_t n_selected_host, const T *dist,
                  const T *threshold, I *selected, I *n_gt, I *n_eq, int64_t n, void *scratch,
                  int64_t max_selected, cudaStream_t s, const LoopState *guard = nullptr);
template <typename T, typename I>
int launch_relocate(const int64_t *n_empty_dev, int64_t n_empty_host, const T *X, const T *w,
                    const I *labels, const I *selected, const I *n_gt, const I *empty_list,
                    T *sums, T *sizes, T *inertia, int64_t n, int64_t d, int64_t k,
                    cudaStream_t s, const LoopState *guard = nullptr, int64_t x_fstride = 0,
                    int64_t x_sstride = 1);
// Copies *n_empty (indT) into an int64 device scalar (0 when the loop stopped).
template <typename I>
int launch_gate_from_count(const I *n_empty, int64_t *gate, cudaStream_t s,
                           const LoopState *guard);

}  // namespace kmc
