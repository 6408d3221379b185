// Initialisation and input-layout kernels in front of the Lloyd path (the
// steps before the reference's driver, which takes X_t and initial centroids
// as given, python_api/_kmeans_lloyd.cpp:1153):
//   transpose     row-major X (n, d) -> the feature-major X_t (d, n) the
//                 engine reads, 32 x 32 tiles staged through shared memory so
//                 that both the reads and the writes are coalesced
//   gather_rows   C_t[:, j] = X_t[:, rows[j]] (random-row initialisation)
//   k-means++     D^2-weighted seeding (Arthur and Vassilvitskii, 2007), fully
//                 on the device and deterministic for a seed:
//                   draw u_t = SplitMix64(seed, t) / 2^64 in [0, 1)
//                   pick the first i whose running sum of v_i exceeds
//                   u_t * sum(v), with v_i = w_i (t = 0) or
//                   w_i * min_j ||x_i - c_j||^2 (t > 0) in float64, summed
//                   sequentially within fixed blocks of 4096 samples and then
//                   over the blocks in order
//                 so that a sequential CPU restatement selects the same rows.
//                 Squared distances use the engine's order: one fused
//                 multiply-add per feature, f = 0..d-1.
#include <cstdint>
#include <vector>

#include "km_kernels.cuh"
#include "kmeans_gb300.h"

namespace kmc {
namespace {

constexpr int kPPBlock = 4096;  // samples per partial sum of the k-means++ draw

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    // SplitMix64 output function (S. Vigna, public domain)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <typename T>
__global__ void transpose_kernel(const T *X, T *Xt, int64_t n, int64_t d) {
    __shared__ T tile[32][33];
    const int64_t i0 = (int64_t)blockIdx.x * 32, f0 = (int64_t)blockIdx.y * 32;
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t i = i0 + r, f = f0 + threadIdx.x;
        if (i < n && f < d) tile[r][threadIdx.x] = X[i * d + f];
    }
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += blockDim.y) {
        const int64_t f = f0 + r, i = i0 + threadIdx.x;
        if (i < n && f < d) Xt[f * n + i] = tile[threadIdx.x][r];
    }
}

template <typename T>
__global__ void gather_kernel(const T *Xt, int64_t n, int64_t d, const int32_t *rows, int64_t k,
                              T *Ct, int *bad) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d * k;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = e / k, j = e % k;
        const int64_t i = rows[j];
        if (i >= 0 && i < n) {
            Ct[e] = Xt[f * n + i];
        } else {
            Ct[e] = T(0);
            atomicOr(bad, 1);
        }
    }
}

template <typename T>
__device__ __forceinline__ T fma_k(T a, T b, T c);
template <>
__device__ __forceinline__ float fma_k(float a, float b, float c) { return __fmaf_rn(a, b, c); }
template <>
__device__ __forceinline__ double fma_k(double a, double b, double c) { return __fma_rn(a, b, c); }

// min_d2[i] = min(min_d2[i], ||x_i - c||^2) with c = X_t[:, *chosen] (first
// centre: min_d2 = the distance itself).
template <typename T>
__global__ void pp_update_kernel(const T *Xt, int64_t n, int64_t d, const int32_t *chosen,
                                 int first, T *min_d2) {
    const int64_t c = *chosen;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) {
            const T diff = Xt[f * n + i] - Xt[f * n + c];
            acc = fma_k(diff, diff, acc);
        }
        min_d2[i] = (first || acc < min_d2[i]) ? acc : min_d2[i];
    }
}

// One thread per block of kPPBlock samples: sequential float64 partial sum.
template <typename T>
__global__ void pp_partials_kernel(const T *w, const T *min_d2, int64_t n, int use_d2,
                                   double *partials) {
    const int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nb = (n + kPPBlock - 1) / kPPBlock;
    if (b >= nb) return;
    double s = 0.0;
    const int64_t hi = (b + 1) * kPPBlock < n ? (b + 1) * kPPBlock : n;
    for (int64_t i = b * kPPBlock; i < hi; ++i) {
        const double wi = w ? (double)w[i] : 1.0;
        s += use_d2 ? wi * (double)min_d2[i] : wi;
    }
    partials[b] = s;
}

// Draw of centre t (single block): pick the sample, record it, copy its row.
template <typename T>
__global__ void pp_select_kernel(const T *Xt, const T *w, const T *min_d2, int64_t n, int64_t d,
                                 int64_t k, int t, int use_d2, uint64_t seed,
                                 const double *partials, int32_t *chosen, T *Ct) {
    __shared__ int64_t pick;
    if (threadIdx.x == 0) {
        const int64_t nb = (n + kPPBlock - 1) / kPPBlock;
        double total = 0.0;
        for (int64_t b = 0; b < nb; ++b) total += partials[b];
        int64_t sel = -1;
        if (total > 0.0) {
            const double u = (double)(splitmix64(seed ^ splitmix64((uint64_t)t)) >> 11) * 0x1p-53;
            const double target = u * total;
            double run = 0.0;
            int64_t b = 0;
            for (; b < nb; ++b) {
                if (run + partials[b] > target) break;
                run += partials[b];
            }
            if (b == nb) b = nb - 1;  // rounding at the very end of the range
            const int64_t hi = (b + 1) * kPPBlock < n ? (b + 1) * kPPBlock : n;
            for (int64_t i = b * kPPBlock; i < hi; ++i) {
                const double wi = w ? (double)w[i] : 1.0;
                const double v = use_d2 ? wi * (double)min_d2[i] : wi;
                if (v > 0.0) sel = i;  // last positive sample if rounding overshoots
                run += v;
                if (run > target && v > 0.0) break;
            }
        }
        if (sel < 0) sel = t > 0 ? ((int64_t)chosen[t - 1] + 1) % n : 0;  // every weight is zero
        chosen[t] = (int32_t)sel;
        pick = sel;
    }
    __syncthreads();
    for (int64_t f = threadIdx.x; f < d; f += blockDim.x) Ct[f * k + t] = Xt[f * n + pick];
}

// Population variance of each feature (one block per feature, two passes in
// float64: the mean, then the mean squared deviation).
template <typename T>
__global__ void feature_var_kernel(const T *Xt, int64_t n, double *var) {
    __shared__ double sh[32];
    const int64_t f = blockIdx.x;
    const T *row = Xt + f * n;
    auto block_sum = [&](double v) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
        __syncthreads();
        double r = 0.0;
        if (threadIdx.x < 32) {
            r = (threadIdx.x < (blockDim.x >> 5)) ? sh[threadIdx.x] : 0.0;
            for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
            if (threadIdx.x == 0) sh[0] = r;
        }
        __syncthreads();
        const double out = sh[0];
        __syncthreads();
        return out;
    };
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += (double)row[i];
    const double mean = block_sum(s) / (double)n;
    double q = 0.0;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double dv = (double)row[i] - mean;
        q += dv * dv;
    }
    const double tot = block_sum(q);
    if (threadIdx.x == 0) var[f] = tot / (double)n;
}

template <typename T>
int mean_variance(const T *Xt, int64_t n, int64_t d, double *out, cudaStream_t s) {
    KMC_CHECK_ARG(n >= 1 && d >= 1, "invalid dimensions");
    KMC_CHECK_ARG(d <= (int64_t(1) << 31) - 1, "n_features too large");
    Scratch mem;
    KMC_TRY(mem.alloc(sizeof(double) * d, s));
    feature_var_kernel<T><<<(unsigned)d, 256, 0, s>>>(Xt, n, mem.as<double>());
    KMC_TRY(check_launch("feature_variance"));
    std::vector<double> h((size_t)d);
    KMC_CUDA_TRY(cudaMemcpyAsync(h.data(), mem.ptr, sizeof(double) * d, cudaMemcpyDeviceToHost, s));
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    double acc = 0.0;
    for (double v : h) acc += v;
    *out = acc / (double)d;
    return KMC_OK;
}

template <typename T>
int transpose(const T *X, T *Xt, int64_t n, int64_t d, cudaStream_t s) {
    KMC_CHECK_ARG(n >= 0 && d >= 0, "array dimensions must be non-negative");
    if (n == 0 || d == 0) return KMC_OK;
    KMC_CHECK_ARG(ceil_div<int64_t>(d, 32) <= 65535, "n_features too large");
    dim3 grid((unsigned)ceil_div<int64_t>(n, 32), (unsigned)ceil_div<int64_t>(d, 32));
    transpose_kernel<T><<<grid, dim3(32, 8), 0, s>>>(X, Xt, n, d);
    return check_launch("transpose");
}

template <typename T>
int gather(const T *Xt, int64_t n, int64_t d, const int32_t *rows, int64_t k, T *Ct,
           cudaStream_t s) {
    KMC_CHECK_ARG(n >= 1 && d >= 0 && k >= 0, "invalid dimensions");
    if (d * k == 0) return KMC_OK;
    Scratch flag;
    KMC_TRY(flag.alloc(sizeof(int), s));
    KMC_CUDA_TRY(cudaMemsetAsync(flag.ptr, 0, sizeof(int), s));
    const int64_t g = std::min<int64_t>(ceil_div<int64_t>(d * k, 256), 4096);
    gather_kernel<T><<<(unsigned)g, 256, 0, s>>>(Xt, n, d, rows, k, Ct, flag.as<int>());
    KMC_TRY(check_launch("gather_rows"));
    int bad = 0;
    KMC_CUDA_TRY(cudaMemcpyAsync(&bad, flag.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    KMC_CHECK_ARG(bad == 0, "row index out of range [0, n_samples)");
    return KMC_OK;
}

template <typename T>
int kmeanspp(const T *Xt, const T *w, int64_t n, int64_t d, int64_t k, uint64_t seed, T *Ct,
             int32_t *chosen, cudaStream_t s) {
    KMC_CHECK_ARG(n >= 1 && d >= 1 && k >= 1, "invalid dimensions");
    KMC_CHECK_ARG(k <= n, "n_clusters exceeds n_samples");
    KMC_CHECK_ARG(n < (int64_t(1) << 31), "n_samples must fit int32 indices");
    const int64_t nb = ceil_div<int64_t>(n, kPPBlock);
    Scratch mem;
    const size_t o_p = align256(sizeof(T) * n);
    KMC_TRY(mem.alloc(o_p + align256(sizeof(double) * nb), s));
    T *min_d2 = mem.as<T>();
    double *partials = reinterpret_cast<double *>(mem.as<char>() + o_p);
    const unsigned gp = (unsigned)ceil_div<int64_t>(nb, 128);
    const unsigned gu = (unsigned)std::min<int64_t>(ceil_div<int64_t>(n, 256), 8192);
    for (int64_t t = 0; t < k; ++t) {
        const int use_d2 = t > 0 ? 1 : 0;
        pp_partials_kernel<T><<<gp, 128, 0, s>>>(w, min_d2, n, use_d2, partials);
        KMC_TRY(check_launch("kmeanspp_partials"));
        pp_select_kernel<T><<<1, 128, 0, s>>>(Xt, w, min_d2, n, d, k, (int)t, use_d2, seed,
                                              partials, chosen, Ct);
        KMC_TRY(check_launch("kmeanspp_select"));
        if (t + 1 < k) {
            pp_update_kernel<T><<<gu, 256, 0, s>>>(Xt, n, d, chosen + t, t == 0 ? 1 : 0, min_d2);
            KMC_TRY(check_launch("kmeanspp_update"));
        }
    }
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    return KMC_OK;
}

}  // namespace
}  // namespace kmc

using namespace kmc;

extern "C" {

int kmc_transpose_f32(const float *X, float *X_t, int64_t n_samples, int64_t n_features,
                      kmc_stream_t stream) {
    return transpose<float>(X, X_t, n_samples, n_features, reinterpret_cast<cudaStream_t>(stream));
}

int kmc_transpose_f64(const double *X, double *X_t, int64_t n_samples, int64_t n_features,
                      kmc_stream_t stream) {
    return transpose<double>(X, X_t, n_samples, n_features,
                             reinterpret_cast<cudaStream_t>(stream));
}

int kmc_gather_rows_f32(const float *X_t, int64_t n_samples, int64_t n_features,
                        const int32_t *rows, int64_t n_clusters, float *centroids_t,
                        kmc_stream_t stream) {
    return gather<float>(X_t, n_samples, n_features, rows, n_clusters, centroids_t,
                         reinterpret_cast<cudaStream_t>(stream));
}

int kmc_gather_rows_f64(const double *X_t, int64_t n_samples, int64_t n_features,
                        const int32_t *rows, int64_t n_clusters, double *centroids_t,
                        kmc_stream_t stream) {
    return gather<double>(X_t, n_samples, n_features, rows, n_clusters, centroids_t,
                          reinterpret_cast<cudaStream_t>(stream));
}

int kmc_mean_feature_variance_f32(const float *X_t, int64_t n_samples, int64_t n_features,
                                  double *mean_variance_out, kmc_stream_t stream) {
    KMC_CHECK_ARG(mean_variance_out != nullptr, "null output");
    return mean_variance<float>(X_t, n_samples, n_features, mean_variance_out,
                                reinterpret_cast<cudaStream_t>(stream));
}

int kmc_mean_feature_variance_f64(const double *X_t, int64_t n_samples, int64_t n_features,
                                  double *mean_variance_out, kmc_stream_t stream) {
    KMC_CHECK_ARG(mean_variance_out != nullptr, "null output");
    return mean_variance<double>(X_t, n_samples, n_features, mean_variance_out,
                                 reinterpret_cast<cudaStream_t>(stream));
}

int kmc_kmeans_plusplus_f32(const float *X_t, const float *sample_weight, int64_t n_samples,
                            int64_t n_features, int64_t n_clusters, uint64_t seed,
                            float *centroids_t, int32_t *chosen_rows, kmc_stream_t stream) {
    return kmeanspp<float>(X_t, sample_weight, n_samples, n_features, n_clusters, seed,
                           centroids_t, chosen_rows, reinterpret_cast<cudaStream_t>(stream));
}

int kmc_kmeans_plusplus_f64(const double *X_t, const double *sample_weight, int64_t n_samples,
                            int64_t n_features, int64_t n_clusters, uint64_t seed,
                            double *centroids_t, int32_t *chosen_rows, kmc_stream_t stream) {
    return kmeanspp<double>(X_t, sample_weight, n_samples, n_features, n_clusters, seed,
                            centroids_t, chosen_rows, reinterpret_cast<cudaStream_t>(stream));
}

}  // extern "C"
