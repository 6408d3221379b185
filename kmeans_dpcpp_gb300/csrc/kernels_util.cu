// O(k*d) and O(n) kernels of the Lloyd engine: half norms, broadcast
// division, private-copy reduction with empty-cluster detection, centroid
// shifts, per-sample inertia and deterministic float64 sums.
//
// Arithmetic order follows the SYCL kernels cited on each function: sums over
// features run sequentially f = 0..d-1 with a fused multiply-add, exactly as
// `acc += a * b` is contracted by the reference's device compiler.
#include "km_kernels.cuh"

namespace kmc {

namespace {

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

__device__ __forceinline__ bool stopped(const LoopState *g) {
    return g != nullptr && *reinterpret_cast<const volatile int *>(&g->done) != 0;
}

// broadcast_division_kernel, src/util_kernels.hpp:9-41: X[r, c] /= y[c].
template <typename T>
__global__ void broadcast_divide_kernel(T *X, const T *y, int64_t rows, int64_t cols) {
    int64_t total = rows * cols;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = e % cols;
        X[e] = X[e] / y[c];
    }
}

// half_l2_norm_kernel, src/util_kernels.hpp:47-82: out[j] = (sum_f C[f,j]^2) / 2.
template <typename T>
__global__ void half_norm_kernel(const T *C, T *out, int64_t d, int64_t k,
                                 const LoopState *guard) {
    if (stopped(guard)) return;
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= k) return;
    T acc = T(0);
    for (int64_t f = 0; f < d; ++f) {
        T v = C[f * k + j];
        acc = fma_t(v, v, acc);
    }
    out[j] = acc / T(2);
}

// reduce_centroid_data_kernel, src/util_kernels.hpp:87-161, part 1: sums of
// the private copies in copy order 0..P-1 (sums and sizes).
// A is the accumulator type of the copies (dataT for the public API, float64
// inside the driver); the result is rounded once to dataT.
template <typename T, typename A>
__global__ void reduce_copies_kernel(const A *sizes_cp, const A *cent_cp, T *out_sizes,
                                     T *out_cent, int64_t P, int64_t d, int64_t k,
                                     const LoopState *guard) {
    if (stopped(guard)) return;
    int64_t dk = d * k;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < dk + k;
         e += (int64_t)gridDim.x * blockDim.x) {
        // copies added in index order; loads issued eight ahead of the adds
        const A *src = (e < dk) ? cent_cp + e : sizes_cp + (e - dk);
        const int64_t stride = (e < dk) ? dk : k;
        A s = A(0);
        int64_t p = 0;
        for (; p + 8 <= P; p += 8) {
            A v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = src[(p + u) * stride];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += v[u];
        }
        for (; p < P; ++p) s += src[p * stride];
        if (e < dk)
            out_cent[e] = (T)s;
        else
            out_sizes[e - dk] = (T)s;
    }
}

// Part 2: empty-cluster list.  The reference appends through an atomic
// counter in arbitrary order (util_kernels.hpp:143-153, marked FIXME there);
// here the list is built in ascending cluster order by one block, starting
// at the counter's current value.
template <typename T, typename I>
__global__ void empty_list_kernel(const T *sizes, I *list, I *n_empty, int64_t k,
                                  const LoopState *guard) {
    if (stopped(guard)) return;
    __shared__ int warp_counts[32];
    __shared__ long long base_sh;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) base_sh = (long long)(*n_empty);
    __syncthreads();
    for (int64_t j0 = 0; j0 < k; j0 += blockDim.x) {
        int64_t j = j0 + threadIdx.x;
        bool empty = (j < k) && (sizes[j] == T(0));
        unsigned ballot = __ballot_sync(0xffffffffu, empty);
        if (lane == 0) warp_counts[wid] = __popc(ballot);
        __syncthreads();
        long long before = 0, total = 0;
        for (int w = 0; w < nwarps; ++w) {
            if (w < wid) before += warp_counts[w];
            total += warp_counts[w];
        }
        if (empty) {
            long long pos = base_sh + before + __popc(ballot & ((1u << lane) - 1u));
            if (pos >= 0 && pos < k) list[pos] = (I)j;  // the counter is caller-initialised
        }
        __syncthreads();
        if (threadIdx.x == 0) base_sh += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *n_empty = (I)base_sh;
}

// compute_centroid_shifts_squared_kernel, src/util_kernels.hpp:481-516.
template <typename T>
__global__ void shifts_kernel(const T *old_c, const T *new_c, T *out, int64_t d, int64_t k) {
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= k) return;
    T acc = T(0);
    for (int64_t f = 0; f < d; ++f) {
        T diff = old_c[f * k + j] - new_c[f * k + j];
        acc = fma_t(diff, diff, acc);
    }
    out[j] = acc;
}

// Driver fusion of broadcast_division_kernel (util_kernels.hpp:9-41) and the
// shift kernel above: same per-element operations, one pass over (d, k).
template <typename T>
__global__ void divide_and_shift_kernel(const T *__restrict__ old_c, T *__restrict__ new_c,
                                        const T *__restrict__ sizes, T *__restrict__ shifts,
                                        int64_t d, int64_t k, const LoopState *guard) {
    if (stopped(guard)) return;
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= k) return;
    T sz = sizes[j];
    T acc = T(0);
    // features in groups of 8: the group's loads are all in flight before
    // its divisions and the (sequential, as the reference's) fma chain
    constexpr int kG = 8;
    for (int64_t f0 = 0; f0 < d; f0 += kG) {
        T nv[kG], ov[kG];
#pragma unroll
        for (int e = 0; e < kG; ++e) {
            const int64_t f = f0 + e;
            nv[e] = (f < d) ? new_c[f * k + j] : T(0);
            ov[e] = (f < d) ? old_c[f * k + j] : T(0);
        }
#pragma unroll
        for (int e = 0; e < kG; ++e) {
            const int64_t f = f0 + e;
            if (f < d) {
                T c = nv[e] / sz;
                new_c[f * k + j] = c;
                T diff = ov[e] - c;
                acc = fma_t(diff, diff, acc);
            }
        }
    }
    shifts[j] = acc;
}

// Fixed-order block reduction of doubles (deterministic for a given grid).
__device__ double block_sum(double v, double *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = (lane < (int)(blockDim.x >> 5)) ? sh[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    __syncthreads();
    return r;  // valid in thread 0
}

// Loop control of driver_lloyd (src/kmeans_lloyd_driver.hpp:83, 343-353):
// the total shift (float64 here) is compared with tol in dataT, n_iter += 1.
template <typename T>
__global__ void loop_control_kernel(const T *shifts, int64_t k, LoopState *st) {
    __shared__ double sh[32];
    if (*reinterpret_cast<volatile int *>(&st->done)) return;
    double acc = 0.0;
    for (int64_t j = threadIdx.x; j < k; j += blockDim.x) acc += (double)shifts[j];
    double tot = block_sum(acc, sh);
    if (threadIdx.x == 0) {
        st->last_shift = tot;
        st->n_iter += 1;
        T shift_t = (T)tot;
        T tol_t = (T)st->tol;
        bool go_on = (st->n_iter < st->max_iter) && (shift_t > tol_t);
        if (!go_on) st->done = 1;
    }
}

// compute_inertia_kernel / compute_uniform_weight_inertia_kernel,
// src/compute_inertia.hpp:11-99.  w == nullptr gives the unit-weight form.
template <typename T, typename I>
__global__ void inertia_kernel(const T *X, const T *w, const T *C, const I *labels, T *out,
                               int64_t n, int64_t d, int64_t k, const LoopState *guard,
                               const int64_t *gate, int64_t fs, int64_t ss) {
    if (stopped(guard)) return;
    if (gate != nullptr && *gate == 0) return;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        int64_t c = (int64_t)labels[i];
        if (c < 0 || c >= k) {  // caller-supplied label out of range
            out[i] = pos_inf<T>();
            continue;
        }
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) {
            T diff = X[f * fs + i * ss] - C[f * k + c];
            acc = fma_t(diff, diff, acc);
        }
        out[i] = (w != nullptr) ? mul_rn(acc, w[i]) : acc;
    }
}

constexpr int kSumGrid = 1024;
constexpr int kSumBlock = 256;

template <typename T>
__global__ void sum_stage1_kernel(const T *data, int64_t n, double *partials,
                                  const LoopState *guard) {
    __shared__ double sh[32];
    if (stopped(guard)) return;
    double acc = 0.0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        acc += (double)data[i];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) partials[blockIdx.x] = r;
}

__global__ void sum_stage2_kernel(const double *partials, int count, double *out,
                                  const LoopState *guard) {
    __shared__ double sh[32];
    if (stopped(guard)) return;
    double acc = 0.0;
    for (int i = threadIdx.x; i < count; i += blockDim.x) acc += partials[i];
    double r = block_sum(acc, sh);
    if (threadIdx.x == 0) *out = r;
}

template <typename T>
__global__ void fill_kernel(T *p, T v, int64_t count, const LoopState *guard) {
    if (stopped(guard)) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x)
        p[e] = v;
}

inline unsigned grid_for(int64_t work, int block, int max_blocks = 4096) {
    int64_t g = ceil_div<int64_t>(work, block);
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return (unsigned)g;
}

}  // namespace

template <typename T>
int launch_broadcast_divide(T *X, const T *y, int64_t rows, int64_t cols, cudaStream_t s) {
    if (rows * cols == 0) return KMC_OK;
    broadcast_divide_kernel<T><<<grid_for(rows * cols, 256, 8192), 256, 0, s>>>(X, y, rows, cols);
    return check_launch("broadcast_divide");
}

template <typename T>
int launch_half_norm(const T *C, T *out, int64_t d, int64_t k, cudaStream_t s,
                     const LoopState *guard) {
    if (k == 0) return KMC_OK;
    half_norm_kernel<T><<<grid_for(k, 128, 1 << 20), 128, 0, s>>>(C, out, d, k, guard);
    return check_launch("half_l2_norm");
}

template <typename T, typename I, typename A>
int launch_reduce_centroids(const A *sizes_cp, const A *cent_cp, T *out_sizes, T *out_cent,
                            I *empty_list, I *n_empty, int64_t P, int64_t d, int64_t k,
                            cudaStream_t s, const LoopState *guard) {
    if (k == 0) return KMC_OK;
    reduce_copies_kernel<T, A><<<grid_for(d * k + k, 256, 8192), 256, 0, s>>>(
        sizes_cp, cent_cp, out_sizes, out_cent, P, d, k, guard);
    KMC_TRY(check_launch("reduce_centroids_data"));
    empty_list_kernel<T, I><<<1, 1024, 0, s>>>(out_sizes, empty_list, n_empty, k, guard);
    return check_launch("empty_clusters_list");
}

template <typename T, typename I>
int launch_empty_list(const T *sizes, I *list, I *n_empty, int64_t k, cudaStream_t s,
                      const LoopState *guard) {
    if (k == 0) return KMC_OK;
    empty_list_kernel<T, I><<<1, 1024, 0, s>>>(sizes, list, n_empty, k, guard);
    return check_launch("empty_clusters_list");
}

template <typename T>
int launch_shifts(const T *old_c, const T *new_c, T *out, int64_t d, int64_t k,
                  cudaStream_t s) {
    if (k == 0) return KMC_OK;
    shifts_kernel<T><<<grid_for(k, 128, 1 << 20), 128, 0, s>>>(old_c, new_c, out, d, k);
    return check_launch("centroid_shifts");
}

template <typename T>
int launch_divide_and_shift(const T *old_c, T *new_c, const T *sizes, T *shifts, int64_t d,
                            int64_t k, cudaStream_t s, const LoopState *guard) {
    if (k == 0) return KMC_OK;
    divide_and_shift_kernel<T><<<grid_for(k, 128, 1 << 20), 128, 0, s>>>(old_c, new_c, sizes,
                                                                         shifts, d, k, guard);
    return check_launch("divide_and_shift");
}

template <typename T>
int launch_loop_control(const T *shifts, int64_t k, LoopState *state, cudaStream_t s) {
    loop_control_kernel<T><<<1, 1024, 0, s>>>(shifts, k, state);
    return check_launch("loop_control");
}

template <typename T, typename I>
int launch_inertia(const T *X, const T *w, const T *C, const I *labels, T *out, int64_t n,
                   int64_t d, int64_t k, cudaStream_t s, const LoopState *guard,
                   const int64_t *gate, int64_t x_fstride, int64_t x_sstride) {
    if (n == 0) return KMC_OK;
    const int64_t fs = x_fstride > 0 ? x_fstride : n, ss = x_fstride > 0 ? x_sstride : 1;
    inertia_kernel<T, I><<<grid_for(n, 256, 16384), 256, 0, s>>>(X, w, C, labels, out, n, d, k,
                                                                 guard, gate, fs, ss);
    return check_launch("compute_inertia");
}

int64_t sum_partials_size() { return kSumGrid; }

template <typename T>
int launch_sum_f64(const T *data, int64_t n, double *partials, double *out, cudaStream_t s,
                   const LoopState *guard) {
    sum_stage1_kernel<T><<<kSumGrid, kSumBlock, 0, s>>>(data, n, partials, guard);
    KMC_TRY(check_launch("sum_stage1"));
    sum_stage2_kernel<<<1, 1024, 0, s>>>(partials, kSumGrid, out, guard);
    return check_launch("sum_stage2");
}

template <typename T>
int launch_fill(T *p, T v, int64_t count, cudaStream_t s, const LoopState *guard) {
    if (count == 0) return KMC_OK;
    fill_kernel<T><<<grid_for(count, 256, 8192), 256, 0, s>>>(p, v, count, guard);
    return check_launch("fill");
}

#define KMC_INST_T(T)                                                                        \
    template int launch_broadcast_divide<T>(T *, const T *, int64_t, int64_t, cudaStream_t); \
    template int launch_half_norm<T>(const T *, T *, int64_t, int64_t, cudaStream_t,          \
                                     const LoopState *);                                      \
    template int launch_shifts<T>(const T *, const T *, T *, int64_t, int64_t, cudaStream_t); \
    template int launch_divide_and_shift<T>(const T *, T *, const T *, T *, int64_t, int64_t, \
                                            cudaStream_t, const LoopState *);                 \
    template int launch_loop_control<T>(const T *, int64_t, LoopState *, cudaStream_t);       \
    template int launch_sum_f64<T>(const T *, int64_t, double *, double *, cudaStream_t,      \
                                   const LoopState *);                                        \
    template int launch_fill<T>(T *, T, int64_t, cudaStream_t, const LoopState *);

#define KMC_INST_TI(T, I)                                                                     \
    template int launch_reduce_centroids<T, I, T>(const T *, const T *, T *, T *, I *, I *,   \
                                                  int64_t, int64_t, int64_t, cudaStream_t,    \
                                                  const LoopState *);                         \
    template int launch_empty_list<T, I>(const T *, I *, I *, int64_t, cudaStream_t,          \
                                         const LoopState *);                                  \
    template int launch_inertia<T, I>(const T *, const T *, const T *, const I *, T *,        \
                                      int64_t, int64_t, int64_t, cudaStream_t,                \
                                      const LoopState *, const int64_t *, int64_t, int64_t);

KMC_INST_T(float)
KMC_INST_T(double)
template int launch_fill<int32_t>(int32_t *, int32_t, int64_t, cudaStream_t, const LoopState *);
template int launch_fill<int64_t>(int64_t *, int64_t, int64_t, cudaStream_t, const LoopState *);
template int launch_reduce_centroids<float, int32_t, double>(
    const double *, const double *, float *, float *, int32_t *, int32_t *, int64_t, int64_t,
    int64_t, cudaStream_t, const LoopState *);
template int launch_reduce_centroids<float, int64_t, double>(
    const double *, const double *, float *, float *, int64_t *, int64_t *, int64_t, int64_t,
    int64_t, cudaStream_t, const LoopState *);
KMC_INST_TI(float, int32_t)
KMC_INST_TI(float, int64_t)
KMC_INST_TI(double, int32_t)
KMC_INST_TI(double, int64_t)

}  // namespace kmc
