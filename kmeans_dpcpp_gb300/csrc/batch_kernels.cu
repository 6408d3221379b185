// Kernels of the batched Lloyd engine (km_batch.cuh), the device-side
// synthetic-data generator used by the serving loop, and the tile autotuner.
//
// Per engine step (every active instance advances one Lloyd iteration):
//   batch_prep    one CTA per instance: half norms of its centroids
//                 (src/util_kernels.hpp:47-82 order), zeroed float64 sums,
//                 reset work-queue counters
//   batch_assign  persistent CTAs pop (instance, run of 128-sample tiles)
//                 items from a device work queue.  Each (sample, centroid)
//                 pair gets the plain form's arithmetic -- sequential FMA dot
//                 over f = 0..d-1, D = hn - dot, strict < over ascending j
//                 (src/device_functions.hpp:106-162) -- so labels equal a
//                 single fit's bit for bit.  Fitting instances add w*x into
//                 float64 sums, privatised per item in shared memory when the
//                 instance's k*(d+1) doubles fit in 72 KB.  Three kernels
//                 differ in the centroid window (32, 64 or 128 columns per
//                 pass); the autotuner picks one per (d, k)
//   batch_reduce  one CTA per fitting instance: sums rounded once to float32,
//                 sizes, ascending empty-cluster list
//                 (src/util_kernels.hpp:87-161)
//   batch_update  one CTA per fitting instance: divide, per-cluster shifts,
//                 float64 total, the driver's stop rule
//                 (src/kmeans_lloyd_driver.hpp:317-353), copy-back
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <tuple>
#include <mutex>
#include <sstream>
#include <string>
#include <sys/stat.h>

#include "km_batch.cuh"

namespace kmc {

namespace {

constexpr int kThreadsB = 256;
constexpr int kBK = 16;
constexpr int kTM = 8;
constexpr size_t kPrivBytes = 72 * 1024;  // with the tiles: two CTAs per SM
constexpr int kSumCopies = 48;            // global copies of small instances' sums

// Deterministic block-wide float64 sum (same shape as the single-fit loop
// control: warp shuffles, then warp 0 over the warp totals).
__device__ double block_sum_b(double v, double *sh) {
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

__global__ void batch_prep_kernel(BInst *tab, const int *idx, int count, int *counters) {
    if (blockIdx.x == 0 && threadIdx.x < 2 * kBatchVariants) counters[threadIdx.x] = 0;
    if ((int)blockIdx.x >= count) return;
    BInst &in = tab[idx[blockIdx.x]];
    const int d = in.d, k = in.k;
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        float acc = 0.f;
        for (int f = 0; f < d; ++f) {
            const float v = in.C[(int64_t)f * k + j];
            acc = __fmaf_rn(v, v, acc);
        }
        in.hn[j] = acc / 2.f;
    }
    if (in.mode == B_FIT) {
        const int64_t total = ((int64_t)d * k + k) * in.copies;
        for (int64_t e = threadIdx.x; e < total; e += blockDim.x) in.sums[e] = 0.0;
        if (threadIdx.x == 0) in.empty_list[k] = 0;
    }
}

template <int HN>
__device__ __forceinline__ void vld(const float *p, float *o) {
    if constexpr (HN == 1) {
        o[0] = p[0];
    } else if constexpr (HN == 2) {
        const float2 v = *reinterpret_cast<const float2 *>(p);
        o[0] = v.x;
        o[1] = v.y;
    } else {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x;
        o[1] = v.y;
        o[2] = v.z;
        o[3] = v.w;
    }
}

template <int TN>
struct BTile {
    static constexpr int BM = 16 * kTM, BN = 16 * TN, HM = kTM / 2, HN = TN / 2;
    static constexpr int XR = kBK * BM / kThreadsB, CR = kBK * BN / kThreadsB;
    static constexpr size_t base_bytes =
        sizeof(float) * (2 * kBK * BM + 2 * kBK * BN + BN + BM) + sizeof(long long) * BM;
};

// DIST = 1: the items are B_TRANSFORM instances, whose (k, n) Euclidean
// distances sqrt(sum_f (c - x)^2) are written instead of labels (the plain
// form's MODE_DIST arithmetic, compute_euclidean_distance.hpp:12-114).
template <int TN, int DIST>
__global__ void __launch_bounds__(kThreadsB, 2)
    batch_assign_kernel(const BInst *tab, const BItem *items, int n_items, int *counter) {
    using G = BTile<TN>;
    constexpr int BM = G::BM, BN = G::BN, HM = G::HM, HN = G::HN, XR = G::XR, CR = G::CR;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *Xs = reinterpret_cast<float *>(smem_raw);
    float *Cs = Xs + 2 * kBK * BM;
    float *hs = Cs + 2 * kBK * BN;
    float *ws = hs + BN;
    long long *labs = reinterpret_cast<long long *>(ws + BM);
    double *psums = reinterpret_cast<double *>(labs + BM);
    __shared__ int item_sh;

    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    while (true) {
        if (tid == 0) item_sh = atomicAdd(counter, 1);
        __syncthreads();
        const int it = item_sh;
        __syncthreads();
        if (it >= n_items) break;
        const BItem item = items[it];
        const BInst &in = tab[item.inst];
        const float *X = in.X, *C = in.C, *hn = in.hn, *w = in.w;
        int32_t *labels = in.labels;
        const int64_t n = in.n;
        const int d = in.d, k = in.k;
        const bool fit = in.mode == B_FIT;
        const int64_t dk = (int64_t)d * k;
        const bool priv = fit && in.copies == 1 && (size_t)(dk + k) * sizeof(double) <= kPrivBytes;
        double *tsums = priv ? psums : in.sums + (int64_t)(blockIdx.x % (unsigned)in.copies) * (dk + k);
        double *tsizes = tsums + dk;
        if (priv) {
            for (int64_t e = tid; e < dk + k; e += kThreadsB) psums[e] = 0.0;
            __syncthreads();
        }
        const int nchunks = (d + kBK - 1) / kBK;
        const int64_t tile_end = item.tile0 + item.ntiles;
        // Feature chunk ch of samples li0.. and centroids lc0.. into registers;
        // chunk 0 of the item's next (tile, centroid window) step is loaded
        // while the current step's last chunk is multiplied (the widest
        // window has no registers to spare for it: it loads at the step).
        constexpr bool kAhead = TN <= 4;
        float xr[XR], cr[CR];
        auto load_regs = [&](int64_t li0, int lc0, int ch) {
            const int f0 = ch * kBK;
#pragma unroll
            for (int r = 0; r < XR; ++r) {
                const int e = tid + r * kThreadsB;
                const int kk = e / BM, s = e % BM;
                const int f = f0 + kk;
                const int64_t i = li0 + s;
                xr[r] = (f < d && i < n) ? X[(int64_t)f * n + i] : 0.f;
            }
#pragma unroll
            for (int r = 0; r < CR; ++r) {
                const int e = tid + r * kThreadsB;
                const int kk = e / BN, c = e % BN;
                const int f = f0 + kk, j = lc0 + c;
                cr[r] = (f < d && j < k) ? C[(int64_t)f * k + j] : 0.f;
            }
        };
        auto store_smem = [&](int buf) {
#pragma unroll
            for (int r = 0; r < XR; ++r) Xs[buf * kBK * BM + tid + r * kThreadsB] = xr[r];
#pragma unroll
            for (int r = 0; r < CR; ++r) Cs[buf * kBK * BN + tid + r * kThreadsB] = cr[r];
        };
        if (kAhead) load_regs(item.tile0 * BM, 0, 0);

        for (int64_t tile = item.tile0; tile < tile_end; ++tile) {
            const int64_t i0 = tile * BM;
            float best[kTM];
            int bidx[kTM];
#pragma unroll
            for (int m = 0; m < kTM; ++m) {
                best[m] = pos_inf<float>();
                bidx[m] = 0;
            }
            for (int c0 = 0; c0 < k; c0 += BN) {
                float acc[kTM][TN];
#pragma unroll
                for (int m = 0; m < kTM; ++m)
#pragma unroll
                    for (int q = 0; q < TN; ++q) acc[m][q] = 0.f;
                for (int c = tid; c < BN; c += kThreadsB)
                    hs[c] = (c0 + c < k) ? hn[c0 + c] : pos_inf<float>();

                if (!kAhead) load_regs(i0, c0, 0);
                store_smem(0);  // chunk 0 (loaded during the previous step when kAhead)
                __syncthreads();
                for (int ch = 0; ch < nchunks; ++ch) {
                    const int buf = ch & 1;
                    if (ch + 1 < nchunks)
                        load_regs(i0, c0, ch + 1);
                    else if (kAhead && c0 + BN < k)
                        load_regs(i0, c0 + BN, 0);
                    else if (kAhead && tile + 1 < tile_end)
                        load_regs(i0 + BM, 0, 0);
                    const float *xb = Xs + buf * kBK * BM;
                    const float *cb = Cs + buf * kBK * BN;
#pragma unroll
                    for (int kk = 0; kk < kBK; ++kk) {
                        float xv[kTM], cv[TN];
                        vld<HM>(xb + kk * BM + ty * HM, xv);
                        vld<HM>(xb + kk * BM + BM / 2 + ty * HM, xv + HM);
                        vld<HN>(cb + kk * BN + tx * HN, cv);
                        vld<HN>(cb + kk * BN + BN / 2 + tx * HN, cv + HN);
#pragma unroll
                        for (int m = 0; m < kTM; ++m)
#pragma unroll
                            for (int q = 0; q < TN; ++q) {
                                if (DIST) {
                                    const float diff = cv[q] - xv[m];
                                    acc[m][q] = __fmaf_rn(diff, diff, acc[m][q]);
                                } else {
                                    acc[m][q] = __fmaf_rn(xv[m], cv[q], acc[m][q]);
                                }
                            }
                    }
                    if (ch + 1 < nchunks) store_smem(buf ^ 1);
                    __syncthreads();
                }
                if (DIST) {
#pragma unroll
                    for (int m = 0; m < kTM; ++m) {
                        const int s = (m < HM) ? ty * HM + m : BM / 2 + ty * HM + (m - HM);
                        const int64_t i = i0 + s;
#pragma unroll
                        for (int q = 0; q < TN; ++q) {
                            const int cl = (q < HN) ? tx * HN + q : BN / 2 + tx * HN + (q - HN);
                            const int j = c0 + cl;
                            if (i < n && j < k) in.dist[(int64_t)j * n + i] = __fsqrt_rn(acc[m][q]);
                        }
                    }
                    continue;  // smem buffers are rewritten only after the next step's barrier
                }
                // ascending centroid order within this thread's columns
#pragma unroll
                for (int q = 0; q < TN; ++q) {
                    const int cl = (q < HN) ? tx * HN + q : BN / 2 + tx * HN + (q - HN);
                    const float h = hs[cl];
                    const int j = c0 + cl;
#pragma unroll
                    for (int m = 0; m < kTM; ++m) {
                        const float v = h - acc[m][q];
                        if (v < best[m]) {
                            best[m] = v;
                            bidx[m] = j;
                        }
                    }
                }
                __syncthreads();
            }
            if (DIST) continue;
            // (value, index) minimum over the 16 threads sharing these samples
            {
                const int m = rowmin16<float, kTM>(best, bidx, tx);
                if ((tx & (16 / kTM - 1)) == 0) {
                    const int s = (m < HM) ? ty * HM + m : BM / 2 + ty * HM + (m - HM);
                    const int64_t i = i0 + s;
                    if (i < n) labels[i] = bidx[0];
                    labs[s] = bidx[0];
                }
            }
            if (fit) {
                for (int s = tid; s < BM; s += kThreadsB) {
                    const int64_t i = i0 + s;
                    ws[s] = (i < n) ? w[i] : 0.f;
                }
                __syncthreads();
                for (int64_t e = tid; e < (int64_t)BM * d; e += kThreadsB) {
                    const int s = (int)(e % BM);
                    const int64_t f = e / BM;
                    const int64_t i = i0 + s;
                    if (i < n) {
                        // up to kBK features the samples are still in chunk buffer 0
                        const float x = (nchunks == 1) ? Xs[f * BM + s] : X[f * n + i];
                        const float v = __fmul_rn(x, ws[s]);
                        atomicAdd(&tsums[f * k + labs[s]], (double)v);
                    }
                }
                for (int s = tid; s < BM; s += kThreadsB) {
                    const int64_t i = i0 + s;
                    if (i < n) atomicAdd(&tsizes[labs[s]], (double)ws[s]);
                }
            }
            __syncthreads();
        }
        if (priv) {
            for (int64_t e = tid; e < dk + k; e += kThreadsB) {
                const double v = psums[e];
                if (v != 0.0) atomicAdd(&in.sums[e], v);
            }
        }
        __syncthreads();
    }
}

__global__ void batch_reduce_kernel(BInst *tab, const int *idx, int count, int *n_empty_out) {
    if ((int)blockIdx.x >= count) return;
    BInst &in = tab[idx[blockIdx.x]];
    const int d = in.d, k = in.k;
    const int64_t dk = (int64_t)d * k;
    for (int64_t e = threadIdx.x; e < dk + k; e += blockDim.x) {
        // copies added in index order; loads issued eight ahead of the adds
        const double *src = in.sums + e;
        double s = 0.0;
        int c = 0;
        for (; c + 8 <= in.copies; c += 8) {
            double v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = src[(int64_t)(c + u) * (dk + k)];
#pragma unroll
            for (int u = 0; u < 8; ++u) s += v[u];
        }
        for (; c < in.copies; ++c) s += src[(int64_t)c * (dk + k)];
        if (e < dk)
            in.Cn[e] = (float)s;
        else
            in.sizes[e - dk] = (float)s;
    }
    __syncthreads();
    // ascending empty-cluster list
    __shared__ int warp_counts[32];
    __shared__ int base_sh;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    if (threadIdx.x == 0) base_sh = 0;
    __syncthreads();
    for (int j0 = 0; j0 < k; j0 += blockDim.x) {
        const int j = j0 + threadIdx.x;
        const bool empty = (j < k) && (in.sizes[j] == 0.f);
        const unsigned ballot = __ballot_sync(0xffffffffu, empty);
        if (lane == 0) warp_counts[wid] = __popc(ballot);
        __syncthreads();
        int before = 0, total = 0;
        for (int q = 0; q < nwarps; ++q) {
            if (q < wid) before += warp_counts[q];
            total += warp_counts[q];
        }
        if (empty) {
            const int pos = base_sh + before + __popc(ballot & ((1u << lane) - 1u));
            if (pos >= 0 && pos < k) in.empty_list[pos] = j;
        }
        __syncthreads();
        if (threadIdx.x == 0) base_sh += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        in.empty_list[k] = base_sh;
        n_empty_out[blockIdx.x] = base_sh;
    }
}

__global__ void batch_update_kernel(BInst *tab, const int *idx, int count, int *done_out) {
    if ((int)blockIdx.x >= count) return;
    BInst &in = tab[idx[blockIdx.x]];
    __shared__ double sh[32];
    const int d = in.d, k = in.k;
    double part = 0.0;
    for (int j = threadIdx.x; j < k; j += blockDim.x) {
        const float sz = in.sizes[j];
        float acc = 0.f;
        for (int f = 0; f < d; ++f) {
            const int64_t e = (int64_t)f * k + j;
            const float c = in.Cn[e] / sz;
            in.Cn[e] = c;
            const float diff = in.C[e] - c;
            acc = __fmaf_rn(diff, diff, acc);
        }
        part += (double)acc;
    }
    const double tot = block_sum_b(part, sh);
    if (threadIdx.x == 0) {
        in.st.last_shift = tot;
        in.st.n_iter += 1;
        const float shift_t = (float)tot;
        const float tol_t = (float)in.st.tol;
        const bool go_on = (in.st.n_iter < in.st.max_iter) && (shift_t > tol_t);
        if (!go_on) in.st.done = 1;
        done_out[blockIdx.x] = in.st.done;
    }
    __syncthreads();
    for (int64_t e = threadIdx.x; e < (int64_t)d * k; e += blockDim.x) in.C[e] = in.Cn[e];
}

// SplitMix64 output function (S. Vigna, public domain).
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ float unit01(uint64_t h) {  // [0, 1), 24 bits
    return (float)(h >> 40) * 0x1p-24f;
}

// Gaussian blobs: sample i belongs to centre c(i) = hash(i) mod n_centers;
// centre coordinates uniform in [box_lo, box_hi), per-centre standard
// deviation uniform in [std_lo, std_hi], normal deviates by Box-Muller.
__global__ void blobs_kernel(float *X, int64_t n, int64_t d, int64_t n_centers, float box_lo,
                             float box_hi, float std_lo, float std_hi, uint64_t seed) {
    const uint64_t s_c = mix64(seed ^ 0x1111), s_m = mix64(seed ^ 0x2222),
                   s_s = mix64(seed ^ 0x3333), s_z = mix64(seed ^ 0x4444);
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * d;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = e / n, i = e % n;
        const int64_t c = (int64_t)(mix64(s_c ^ (uint64_t)i) % (uint64_t)n_centers);
        const float centre = box_lo + (box_hi - box_lo) * unit01(mix64(s_m ^ (uint64_t)(c * d + f)));
        const float sd = std_lo + (std_hi - std_lo) * unit01(mix64(s_s ^ (uint64_t)c));
        const uint64_t h = mix64(s_z ^ (uint64_t)e);
        const float u1 = ((float)(h >> 40) + 1.f) * 0x1p-24f;  // (0, 1]
        const float u2 = (float)(h & 0xFFFFFFull) * 0x1p-24f;
        const float z = sqrtf(-2.f * logf(u1)) * cospif(2.f * u2);
        X[e] = centre + sd * z;
    }
}

__global__ void gather_rows_kernel(const float *X, int64_t n, int64_t d, const int32_t *idx,
                                   int64_t k, float *C) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < d * k;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t f = e / k, j = e % k;
        const int64_t i = idx[j];
        C[e] = (i >= 0 && i < n) ? X[f * n + i] : 0.f;
    }
}

// Launch shape of each assign variant (shared memory attribute set once, so
// the launch itself can be captured into a graph).
struct AssignShape {
    size_t smem = 0;
    int grid = 0;
};
std::mutex g_shape_mu;
AssignShape g_shape[2][kBatchVariants][64];  // [dist][variant][device]

template <int TN, int DIST>
int assign_shape(int variant, AssignShape *out) {
    int dev = 0;
    KMC_CUDA_TRY(cudaGetDevice(&dev));
    KMC_CHECK_ARG(dev >= 0 && dev < 64, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_shape_mu);
    AssignShape &sh = g_shape[DIST][variant][dev];
    if (sh.grid == 0) {
        const size_t smem = BTile<TN>::base_bytes + kPrivBytes;
        auto kern = batch_assign_kernel<TN, DIST>;
        KMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        int per_sm = 0;
        KMC_CUDA_TRY(
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreadsB, smem));
        sh.smem = smem;
        sh.grid = num_sms() * (per_sm < 1 ? 1 : per_sm);
    }
    *out = sh;
    return KMC_OK;
}

template <int TN, int DIST>
int launch_assign_v(int variant, const BInst *tab, const BItem *items, int n_items,
                    int *counter, cudaStream_t s) {
    AssignShape sh;
    KMC_TRY((assign_shape<TN, DIST>(variant, &sh)));
    int grid = sh.grid;
    if (grid > n_items) grid = n_items;
    if (grid < 1) return KMC_OK;
    batch_assign_kernel<TN, DIST><<<grid, kThreadsB, sh.smem, s>>>(tab, items, n_items, counter);
    return check_launch("batch_assign");
}

std::mutex g_tune_mu;
// autotuner choices by (d, power-of-two bucket of k, tag); tag "f32" is the
// batched engine's centroid window, "fit-f32" / "fit-f64" the single-fit tile
std::map<std::tuple<int64_t, int64_t, std::string>, int> g_tune;
bool g_tune_loaded = false;

std::string tune_path() {
    if (const char *p = std::getenv("KMC_TILE_CACHE")) return p;
    std::string base;
    if (const char *x = std::getenv("XDG_CACHE_HOME"))
        base = x;
    else if (const char *h = std::getenv("HOME"))
        base = std::string(h) + "/.cache";
    else
        return "";
    return base + "/kmeans_gb300/tiles.txt";
}

// Lines "d k tag variant"; later lines win.
void tune_load() {
    const std::string p = tune_path();
    if (p.empty()) return;
    std::ifstream f(p);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        int64_t d = 0, k = 0;
        std::string tag;
        int v = -1;
        if (is >> d >> k >> tag >> v && v >= 0 && v < 8) g_tune[{d, k, tag}] = v;
    }
}

void tune_store(int64_t d, int64_t k, const std::string &tag, int v) {
    const std::string p = tune_path();
    if (p.empty()) return;
    const size_t slash = p.rfind('/');
    if (slash != std::string::npos) {
        // create the cache directory (and its parent) if needed
        const std::string dir = p.substr(0, slash);
        const size_t s2 = dir.rfind('/');
        if (s2 != std::string::npos && s2 > 0) mkdir(dir.substr(0, s2).c_str(), 0755);
        mkdir(dir.c_str(), 0755);
    }
    std::ofstream f(p, std::ios::app);
    if (f) f << d << " " << k << " " << tag << " " << v << "\n";
}

}  // namespace

int batch_variant_width(int v) { return v == 0 ? 32 : (v == 1 ? 64 : 128); }

int batch_sum_copies(int64_t d, int64_t k) {
    return ((d + 1) * k * (int64_t)sizeof(double) <= (int64_t)kPrivBytes) ? kSumCopies : 1;
}

size_t batch_assign_smem(int v) {
    const size_t b = v == 0 ? BTile<2>::base_bytes
                            : (v == 1 ? BTile<4>::base_bytes : BTile<8>::base_bytes);
    return b + kPrivBytes;
}

int launch_batch_prep(BInst *tab, const int *idx, int count, int *counters, cudaStream_t s) {
    batch_prep_kernel<<<count > 0 ? count : 1, 256, 0, s>>>(tab, idx, count, counters);
    return check_launch("batch_prep");
}

int prepare_batch_assign() {
    AssignShape sh;
    KMC_TRY((assign_shape<2, 0>(0, &sh)));
    KMC_TRY((assign_shape<4, 0>(1, &sh)));
    KMC_TRY((assign_shape<8, 0>(2, &sh)));
    KMC_TRY((assign_shape<2, 1>(0, &sh)));
    KMC_TRY((assign_shape<4, 1>(1, &sh)));
    return assign_shape<8, 1>(2, &sh);
}

int launch_batch_assign(int variant, int dist, const BInst *tab, const BItem *items,
                        int n_items, int *counter, cudaStream_t s) {
    if (n_items <= 0) return KMC_OK;
    if (dist) {
        if (variant == 0) return launch_assign_v<2, 1>(0, tab, items, n_items, counter, s);
        if (variant == 1) return launch_assign_v<4, 1>(1, tab, items, n_items, counter, s);
        return launch_assign_v<8, 1>(2, tab, items, n_items, counter, s);
    }
    if (variant == 0) return launch_assign_v<2, 0>(0, tab, items, n_items, counter, s);
    if (variant == 1) return launch_assign_v<4, 0>(1, tab, items, n_items, counter, s);
    return launch_assign_v<8, 0>(2, tab, items, n_items, counter, s);
}

int launch_batch_reduce(BInst *tab, const int *idx, int count, int *n_empty_out,
                        cudaStream_t s) {
    if (count <= 0) return KMC_OK;
    batch_reduce_kernel<<<count, 1024, 0, s>>>(tab, idx, count, n_empty_out);
    return check_launch("batch_reduce");
}

int launch_batch_update(BInst *tab, const int *idx, int count, int *done_out, cudaStream_t s) {
    if (count <= 0) return KMC_OK;
    batch_update_kernel<<<count, 1024, 0, s>>>(tab, idx, count, done_out);
    return check_launch("batch_update");
}

int launch_blobs(float *X, int64_t n, int64_t d, int64_t n_centers, float box_lo,
                 float box_hi, float std_lo, float std_hi, uint64_t seed, cudaStream_t s) {
    if (n * d == 0) return KMC_OK;
    KMC_CHECK_ARG(n_centers > 0, "n_centers must be positive");
    const int64_t g = std::min<int64_t>(ceil_div<int64_t>(n * d, 256), 65536);
    blobs_kernel<<<(unsigned)g, 256, 0, s>>>(X, n, d, n_centers, box_lo, box_hi, std_lo, std_hi,
                                             seed);
    return check_launch("blobs");
}

int launch_gather_rows(const float *X, int64_t n, int64_t d, const int32_t *idx, int64_t k,
                       float *C, cudaStream_t s) {
    if (d * k == 0) return KMC_OK;
    const int64_t g = std::min<int64_t>(ceil_div<int64_t>(d * k, 256), 4096);
    gather_rows_kernel<<<(unsigned)g, 256, 0, s>>>(X, n, d, idx, k, C);
    return check_launch("gather_rows");
}

void seeded_rows(int64_t n, int64_t k, uint64_t seed, std::vector<int32_t> *out) {
    out->resize((size_t)k);
    if (n <= 0) return;
    uint64_t a = (mix64(seed) % (uint64_t)n) | 1ull;
    auto gcd = [](uint64_t x, uint64_t y) {
        while (y) {
            const uint64_t t = x % y;
            x = y;
            y = t;
        }
        return x;
    };
    while (gcd(a, (uint64_t)n) != 1) a += 2;
    const uint64_t b = mix64(seed ^ 0x5555) % (uint64_t)n;
    for (int64_t j = 0; j < k; ++j)
        (*out)[(size_t)j] = (int32_t)((a % (uint64_t)n * (uint64_t)j + b) % (uint64_t)n);
}

bool tune_lookup(int64_t d, int64_t k, const char *tag, int *v) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    if (!g_tune_loaded) {
        tune_load();
        g_tune_loaded = true;
    }
    auto it = g_tune.find({d, k, std::string(tag)});
    if (it == g_tune.end()) return false;
    *v = it->second;
    return true;
}

void tune_record(int64_t d, int64_t k, const char *tag, int v) {
    std::lock_guard<std::mutex> lock(g_tune_mu);
    g_tune[{d, k, std::string(tag)}] = v;
    tune_store(d, k, tag, v);
}

int tune_variant(int64_t d, int64_t k_in, cudaStream_t s, int *variant) {
    // one measurement per (d, power-of-two bucket of k)
    int64_t k = 1;
    while (k < k_in) k <<= 1;
    if (tune_lookup(d, k, "f32", variant) && *variant < kBatchVariants) return KMC_OK;
    // Time the three assign kernels on a synthetic fitting instance of this
    // (d, k): 256 tiles of 128 samples, blobs around k centres.
    const int64_t n = 256 * kBatchTileM;
    Scratch mem;
    const size_t off_C = align256(sizeof(float) * d * n);
    const size_t off_hn = off_C + align256(sizeof(float) * d * k);
    const size_t off_w = off_hn + align256(sizeof(float) * k);
    const size_t off_lab = off_w + align256(sizeof(float) * n);
    const size_t off_sum = off_lab + align256(sizeof(int32_t) * n);
    const size_t off_tab = off_sum + align256(sizeof(double) * (d * k + k));
    const size_t off_item = off_tab + align256(sizeof(BInst));
    const size_t off_cnt = off_item + align256(sizeof(BItem) * 64);
    KMC_TRY(mem.alloc(off_cnt + 256, s));
    char *b = mem.as<char>();
    float *X = reinterpret_cast<float *>(b);
    float *C = reinterpret_cast<float *>(b + off_C);
    BInst h{};
    h.X = X;
    h.w = reinterpret_cast<float *>(b + off_w);
    h.C = C;
    h.hn = reinterpret_cast<float *>(b + off_hn);
    h.sums = reinterpret_cast<double *>(b + off_sum);
    h.copies = 1;
    h.labels = reinterpret_cast<int32_t *>(b + off_lab);
    h.n = n;
    h.d = (int)d;
    h.k = (int)k;
    h.mode = B_FIT;
    KMC_TRY(launch_blobs(X, n, d, k, -5.f, 5.f, 1.f, 1.f, 7, s));
    KMC_TRY(launch_blobs(C, k, d, k, -5.f, 5.f, 1.f, 1.f, 8, s));
    KMC_TRY(launch_fill<float>(const_cast<float *>(h.w), 1.f, n, s));
    KMC_TRY(launch_fill<float>(h.hn, 0.f, k, s));
    KMC_TRY(launch_fill<double>(h.sums, 0.0, d * k + k, s));
    BItem hi[64];
    for (int q = 0; q < 64; ++q) hi[q] = BItem{0, 4, (long long)q * 4};
    BInst *tab = reinterpret_cast<BInst *>(b + off_tab);
    BItem *items = reinterpret_cast<BItem *>(b + off_item);
    int *cnt = reinterpret_cast<int *>(b + off_cnt);
    KMC_CUDA_TRY(cudaMemcpyAsync(tab, &h, sizeof(h), cudaMemcpyHostToDevice, s));
    KMC_CUDA_TRY(cudaMemcpyAsync(items, hi, sizeof(hi), cudaMemcpyHostToDevice, s));
    cudaEvent_t e0, e1;
    KMC_CUDA_TRY(cudaEventCreate(&e0));
    KMC_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 0.f;
    int best = 2;
    for (int v = 0; v < kBatchVariants; ++v) {
        float tot = 0.f;
        for (int rep = 0; rep < 3; ++rep) {
            KMC_CUDA_TRY(cudaMemsetAsync(cnt, 0, sizeof(int), s));
            KMC_CUDA_TRY(cudaEventRecord(e0, s));
            KMC_TRY(launch_batch_assign(v, 0, tab, items, 64, cnt, s));
            KMC_CUDA_TRY(cudaEventRecord(e1, s));
            KMC_CUDA_TRY(cudaEventSynchronize(e1));
            float ms = 0.f;
            KMC_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
            if (rep > 0) tot += ms;  // first run warms up
        }
        if (v == 0 || tot < best_ms) {
            best_ms = tot;
            best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    tune_record(d, k, "f32", best);
    *variant = best;
    return KMC_OK;
}

}  // namespace kmc
