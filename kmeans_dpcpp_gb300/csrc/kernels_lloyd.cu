// Exact SIMT (FP32 / FP64) distance tiles: the fused Lloyd step, the
// assignment kernel and the centroid-to-sample distance matrix.
//
// Semantics (per sample i, centroid j), following the reference:
//   dot_j  = sum_f x[f] * c[f, j]   accumulated f = 0..d-1 with one fused
//            multiply-add per term (src/device_functions.hpp:106-137)
//   D_j    = half_norm[j] - dot_j    (src/device_functions.hpp:139-162)
//   label  = first j with the smallest D_j (strict `<` over ascending j,
//            starting from (+inf, 0))
// The fused step then adds w*x into the centroid sums of `label` and w into
// its size (src/lloyd_single_step.hpp:169-203).
//
// GB300 design: a 256-thread CTA owns a tile of BM samples and sweeps the
// centroids in tiles of BN; each thread keeps a TM x TN register micro-tile
// of dot products (outer products over the feature axis from shared memory),
// so every x and c element fetched from shared memory feeds TM or TN fused
// multiply-adds.  Feature chunks are double-buffered through registers.  The
// argmin of each sample is reduced across the 16 threads that share it with
// warp shuffles.  Centroid sums are privatised per CTA in shared memory when
// (d + 1) * k fits, and flushed once per CTA with atomics; otherwise they go
// straight to the global private copy with atomics.  float64 sums of float
// samples with one global copy per CTA take the global route: float64
// reductions to global memory are native (fire-and-forget), in shared memory
// they are compare-and-swap loops.
//
// float64 samples are summed in a deterministic order whenever every CTA has a
// copy of its own: thread t of a CTA owns clusters j = t (mod 256) and adds
// each tile's samples in ascending order with plain read-modify-writes (in
// shared memory when the sums fit there), and the copies are reduced in copy
// order.  A fit whose labels stop changing then reproduces its centroids bit
// for bit, so a zero tolerance stops it on the same iteration as a sequential
// implementation (atomics in arbitrary order leave last-bit noise in every
// centroid shift).
#include <cstdlib>
#include <type_traits>

#include "km_kernels.cuh"

namespace kmc {

namespace {

// Register micro-tile TM x TN per thread (BM = 16 TM samples x BN = 16 TN
// centroids per CTA tile).  TN is a template argument of the kernels: the
// autotuner picks the centroid-tile width per (d, k, dtype) (narrower tiles
// waste fewer padded columns when k is small); TileCfg holds the default.
template <typename T>
struct TileCfg;
template <>
struct TileCfg<float> {
    static constexpr int TM = 8, TN = 8, BK = 16;
};
template <>
struct TileCfg<double> {
    static constexpr int TM = 4, TN = 4, BK = 16;
};

// Micro-tile width of autotuner variant v (0 = TileCfg's, then halves).
template <typename T>
__host__ __device__ constexpr int variant_tn(int v) {
    return v <= 0 ? TileCfg<T>::TN : (v == 1 ? TileCfg<T>::TN / 2 : 2);
}

constexpr int kThreads = 256;
constexpr int MODE_ASSIGN = 0, MODE_FUSED = 1, MODE_DIST = 2;
constexpr size_t kPrivMaxBytes = 64 * 1024;

__device__ __forceinline__ float fma_t(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_t(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float sqrt_t(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ double sqrt_t(double a) { return __dsqrt_rn(a); }

template <typename T, typename I, typename A = T>
struct TileArgs {
    const T *X;
    const T *w;
    const T *C;
    const T *hn;
    I *labels;
    A *sums;
    A *sizes;
    T *dist;
    int64_t n, d, k, P;
    int priv;
    int owned;  // every CTA has a copy of its own (float64 samples: ordered sums)
    const LoopState *guard;
};

template <typename T, int V>
struct VecLd;
template <>
struct VecLd<float, 4> {
    __device__ static void ld(const float *p, float *o) {
        float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <>
struct VecLd<float, 2> {
    __device__ static void ld(const float *p, float *o) {
        float2 v = *reinterpret_cast<const float2 *>(p);
        o[0] = v.x; o[1] = v.y;
    }
};
template <>
struct VecLd<float, 1> {
    __device__ static void ld(const float *p, float *o) { o[0] = *p; }
};
template <>
struct VecLd<double, 2> {
    __device__ static void ld(const double *p, double *o) {
        double2 v = *reinterpret_cast<const double2 *>(p);
        o[0] = v.x; o[1] = v.y;
    }
};
template <>
struct VecLd<double, 1> {
    __device__ static void ld(const double *p, double *o) { o[0] = *p; }
};

template <typename T, int TN_ = TileCfg<T>::TN>
struct TileSmem {
    static constexpr int TM = TileCfg<T>::TM, TN = TN_, BK = TileCfg<T>::BK;
    static constexpr int BM = 16 * TM, BN = 16 * TN;
    static constexpr size_t base_bytes =
        sizeof(T) * (2 * BK * BM + 2 * BK * BN + BN + BM) + sizeof(long long) * BM;
};

template <typename T, typename I, int MODE, typename A, int TN>
__global__ void __launch_bounds__(kThreads, 2) tile_kernel(TileArgs<T, I, A> a) {
    if (a.guard != nullptr && *reinterpret_cast<const volatile int *>(&a.guard->done)) return;
    constexpr int TM = TileCfg<T>::TM, BK = TileCfg<T>::BK;
    constexpr int BM = 16 * TM, BN = 16 * TN;
    constexpr int HM = TM / 2, HN = TN / 2;
    constexpr int XR = BK * BM / kThreads, CR = BK * BN / kThreads;

    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Xs = reinterpret_cast<T *>(smem_raw);
    T *Cs = Xs + 2 * BK * BM;
    T *hs = Cs + 2 * BK * BN;
    T *ws = hs + BN;
    long long *labs = reinterpret_cast<long long *>(ws + BM);
    A *psums = reinterpret_cast<A *>(labs + BM);

    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    const int64_t n = a.n, d = a.d, k = a.k;
    const int64_t dk = d * k;
    A *psizes = psums + dk;
    const int64_t copy = (MODE == MODE_FUSED) ? (int64_t)(blockIdx.x % a.P) : 0;
    A *gsums = (MODE == MODE_FUSED) ? a.sums + copy * dk : nullptr;
    A *gsizes = (MODE == MODE_FUSED) ? a.sizes + copy * k : nullptr;

    if (MODE == MODE_FUSED && a.priv) {
        for (int64_t e = tid; e < dk + k; e += kThreads) psums[e] = A(0);
        __syncthreads();
    }

    const int64_t num_tiles = ceil_div<int64_t>(n, BM);
    const int nchunks = (int)ceil_div<int64_t>(d, BK);

    // Feature chunk ch of the samples i0.. and centroids c0.. into registers.
    // The CTA's (tile, centroid tile) steps run in order, and chunk 0 of the
    // next step is loaded while the last chunk of the current one is
    // multiplied, so global-memory latency is not paid at step boundaries
    // (the assignment-only mode loads it at the step itself: it has no
    // registers to spare across its epilogue).
    constexpr bool kAhead = MODE != MODE_ASSIGN;
    T xr[XR], cr[CR];
    auto load_regs = [&](int64_t li0, int64_t lc0, int ch) {
        const int64_t f0 = (int64_t)ch * BK;
#pragma unroll
        for (int r = 0; r < XR; ++r) {
            int e = tid + r * kThreads;
            int kk = e / BM, s = e % BM;
            int64_t f = f0 + kk, i = li0 + s;
            xr[r] = (f < d && i < n) ? a.X[f * n + i] : T(0);
        }
#pragma unroll
        for (int r = 0; r < CR; ++r) {
            int e = tid + r * kThreads;
            int kk = e / BN, c = e % BN;
            int64_t f = f0 + kk, j = lc0 + c;
            cr[r] = (f < d && j < k) ? a.C[f * k + j] : T(0);
        }
    };
    auto store_smem = [&](int buf) {
#pragma unroll
        for (int r = 0; r < XR; ++r) Xs[buf * BK * BM + tid + r * kThreads] = xr[r];
#pragma unroll
        for (int r = 0; r < CR; ++r) Cs[buf * BK * BN + tid + r * kThreads] = cr[r];
    };
    if (kAhead && (int64_t)blockIdx.x < num_tiles) load_regs((int64_t)blockIdx.x * BM, 0, 0);

    for (int64_t tile = blockIdx.x; tile < num_tiles; tile += gridDim.x) {
        const int64_t i0 = tile * BM;
        T best[TM];
        int bidx[TM];
#pragma unroll
        for (int m = 0; m < TM; ++m) {
            best[m] = pos_inf<T>();
            bidx[m] = 0;
        }

        for (int64_t c0 = 0; c0 < k; c0 += BN) {
            T acc[TM][TN];
#pragma unroll
            for (int m = 0; m < TM; ++m)
#pragma unroll
                for (int q = 0; q < TN; ++q) acc[m][q] = T(0);

            if (MODE != MODE_DIST) {
                for (int c = tid; c < BN; c += kThreads)
                    hs[c] = (c0 + c < k) ? a.hn[c0 + c] : pos_inf<T>();
            }

            if (!kAhead) load_regs(i0, c0, 0);
            store_smem(0);  // chunk 0 (loaded during the previous step when kAhead)
            __syncthreads();
            for (int ch = 0; ch < nchunks; ++ch) {
                const int buf = ch & 1;
                if (ch + 1 < nchunks) {
                    load_regs(i0, c0, ch + 1);
                } else if (kAhead && c0 + BN < k) {
                    load_regs(i0, c0 + BN, 0);
                } else if (kAhead && tile + gridDim.x < num_tiles) {
                    load_regs((tile + gridDim.x) * BM, 0, 0);
                }
                const T *xb = Xs + buf * BK * BM;
                const T *cb = Cs + buf * BK * BN;
#pragma unroll
                for (int kk = 0; kk < BK; ++kk) {
                    T xv[TM], cv[TN];
                    VecLd<T, HM>::ld(xb + kk * BM + ty * HM, xv);
                    VecLd<T, HM>::ld(xb + kk * BM + BM / 2 + ty * HM, xv + HM);
                    VecLd<T, HN>::ld(cb + kk * BN + tx * HN, cv);
                    VecLd<T, HN>::ld(cb + kk * BN + BN / 2 + tx * HN, cv + HN);
#pragma unroll
                    for (int m = 0; m < TM; ++m)
#pragma unroll
                        for (int q = 0; q < TN; ++q) {
                            if (MODE == MODE_DIST) {
                                T diff = cv[q] - xv[m];
                                acc[m][q] = fma_t(diff, diff, acc[m][q]);
                            } else {
                                acc[m][q] = fma_t(xv[m], cv[q], acc[m][q]);
                            }
                        }
                }
                if (ch + 1 < nchunks) store_smem(buf ^ 1);
                __syncthreads();
            }

            if (MODE == MODE_DIST) {
#pragma unroll
                for (int m = 0; m < TM; ++m) {
                    int s = (m < HM) ? ty * HM + m : BM / 2 + ty * HM + (m - HM);
                    int64_t i = i0 + s;
#pragma unroll
                    for (int q = 0; q < TN; ++q) {
                        int cl = (q < HN) ? tx * HN + q : BN / 2 + tx * HN + (q - HN);
                        int64_t j = c0 + cl;
                        if (i < n && j < k) a.dist[j * n + i] = sqrt_t(acc[m][q]);
                    }
                }
            } else {
                // Ascending centroid order within this thread's columns.
#pragma unroll
                for (int q = 0; q < TN; ++q) {
                    int cl = (q < HN) ? tx * HN + q : BN / 2 + tx * HN + (q - HN);
                    T h = hs[cl];
                    int j = (int)(c0 + cl);
#pragma unroll
                    for (int m = 0; m < TM; ++m) {
                        T v = h - acc[m][q];
                        if (v < best[m]) {
                            best[m] = v;
                            bidx[m] = j;
                        }
                    }
                }
            }
            __syncthreads();
        }

        if (MODE == MODE_DIST) continue;

        // Lexicographic (value, index) minimum over the 16 threads sharing
        // these samples == the first minimum of a sequential strict-< scan.
#pragma unroll
        for (int m = 0; m < TM; ++m) {
            T v = best[m];
            int j = bidx[m];
#pragma unroll
            for (int off = 8; off > 0; off >>= 1) {
                T ov = __shfl_xor_sync(0xffffffffu, v, off);
                int oj = __shfl_xor_sync(0xffffffffu, j, off);
                if (ov < v || (ov == v && oj < j)) {
                    v = ov;
                    j = oj;
                }
            }
            bidx[m] = j;
        }
#pragma unroll
        for (int m = 0; m < TM; ++m) {
            if (tx == m) {
                int s = (m < HM) ? ty * HM + m : BM / 2 + ty * HM + (m - HM);
                int64_t i = i0 + s;
                if (i < n) a.labels[i] = (I)bidx[m];
                if (MODE == MODE_FUSED) labs[s] = bidx[m];
            }
        }

        if (MODE == MODE_FUSED) {
            for (int s = tid; s < BM; s += kThreads) {
                int64_t i = i0 + s;
                ws[s] = (i < n) ? a.w[i] : T(0);
            }
            __syncthreads();
            A *tsums = a.priv ? psums : gsums;
            A *tsizes = a.priv ? psizes : gsizes;
            bool ordered = false;
            if constexpr (sizeof(T) == 8) {
                if (a.owned) {
                    ordered = true;
                    static_assert((kThreads & (kThreads - 1)) == 0, "power-of-two CTA");
                    for (int s = 0; s < BM; ++s) {
                        const int64_t j = labs[s];
                        if (i0 + s >= n || (int)(j & (kThreads - 1)) != tid) continue;
                        const T wv = ws[s];
                        for (int64_t f = 0; f < d; ++f) {
                            const T xv = (nchunks == 1) ? Xs[f * BM + s] : a.X[f * n + i0 + s];
                            tsums[f * k + j] += (A)mul_rn(xv, wv);
                        }
                        tsizes[j] += (A)wv;
                    }
                }
            }
            for (int64_t e = tid; !ordered && e < (int64_t)BM * d; e += kThreads) {
                int s = (int)(e % BM);
                int64_t f = e / BM;
                int64_t i = i0 + s;
                if (i < n) {
                    // up to BK features the tile's samples are still in chunk
                    // buffer 0 of shared memory
                    const T xv = (nchunks == 1) ? Xs[f * BM + s] : a.X[f * n + i];
                    T val = mul_rn(xv, ws[s]);
                    atomicAdd(&tsums[f * k + labs[s]], (A)val);
                }
            }
            for (int s = tid; !ordered && s < BM; s += kThreads) {
                int64_t i = i0 + s;
                if (i < n) atomicAdd(&tsizes[labs[s]], (A)ws[s]);
            }
            __syncthreads();
        }
    }

    if (MODE == MODE_FUSED && a.priv) {
        __syncthreads();
        for (int64_t e = tid; e < dk; e += kThreads) {
            A v = psums[e];
            if (v != A(0)) atomicAdd(&gsums[e], v);
        }
        for (int64_t j = tid; j < k; j += kThreads) {
            A v = psizes[j];
            if (v != A(0)) atomicAdd(&gsizes[j], v);
        }
    }
}

template <typename T, typename I, int MODE, typename A = T, int TN = TileCfg<T>::TN>
int launch_tile(TileArgs<T, I, A> args, cudaStream_t s) {
    if (args.n == 0) return KMC_OK;
    size_t smem = TileSmem<T, TN>::base_bytes;
    if (MODE == MODE_FUSED && args.priv) smem += sizeof(A) * (size_t)(args.d * args.k + args.k);
    auto kern = tile_kernel<T, I, MODE, A, TN>;
    if (smem > 48 * 1024) {
        KMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
    }
    int per_sm = 0;
    KMC_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kThreads, smem));
    if (per_sm < 1) per_sm = 1;
    int64_t tiles = ceil_div<int64_t>(args.n, TileSmem<T, TN>::BM);
    int64_t grid = (int64_t)num_sms() * per_sm;
    if (MODE == MODE_DIST) grid = tiles;  // output-bound: one tile per CTA
    if (grid > tiles) grid = tiles;
    if (grid > (1LL << 30)) grid = 1LL << 30;
    args.owned = (MODE == MODE_FUSED && sizeof(T) == 8 && args.P >= grid) ? 1 : 0;
    kern<<<(unsigned)grid, kThreads, smem, s>>>(args);
    return check_launch("tile_kernel");
}

}  // namespace

template <typename T, typename I>
int launch_assignment(const T *X, const T *C, const T *hn, I *labels, int64_t n, int64_t d,
                      int64_t k, cudaStream_t s, const LoopState *guard, int variant) {
    TileArgs<T, I> a{X, nullptr, C, hn, labels, nullptr, nullptr, nullptr, n, d, k, 1, 0, 0,
                     guard};
    if (variant == 1) return launch_tile<T, I, MODE_ASSIGN, T, variant_tn<T>(1)>(a, s);
    if (variant == 2) return launch_tile<T, I, MODE_ASSIGN, T, variant_tn<T>(2)>(a, s);
    return launch_tile<T, I, MODE_ASSIGN>(a, s);
}

template <typename T, typename I, typename A>
int launch_fused_step(const T *X, const T *w, const T *C, const T *hn, I *labels, A *sums_cp,
                      A *sizes_cp, int64_t n, int64_t d, int64_t k, int64_t P, cudaStream_t s,
                      const LoopState *guard, int variant) {
    // float64 sums of float samples with one copy per CTA go straight to
    // global memory (native reductions); otherwise small sums are privatised
    // in shared memory (float64 samples: ordered plain updates, no atomics)
    const bool fits = sizeof(A) * (size_t)(d * k + k) <= kPrivMaxBytes;
    int priv = (fits && (sizeof(T) == 8 || !(sizeof(A) == 8 && P > 1))) ? 1 : 0;
    TileArgs<T, I, A> a{X, w, C, hn, labels, sums_cp, sizes_cp, nullptr, n, d, k, P, priv, 0,
                        guard};
    // the variants are instantiated for the driver's float64 sums
    if constexpr (std::is_same<A, double>::value) {
        if (variant == 1) return launch_tile<T, I, MODE_FUSED, A, variant_tn<T>(1)>(a, s);
        if (variant == 2) return launch_tile<T, I, MODE_FUSED, A, variant_tn<T>(2)>(a, s);
    }
    return launch_tile<T, I, MODE_FUSED, A>(a, s);
}

template <typename T>
int launch_distances(const T *X, const T *C, T *out, int64_t n, int64_t d, int64_t k,
                     cudaStream_t s) {
    TileArgs<T, int32_t> a{X, nullptr, C, nullptr, nullptr, nullptr, nullptr, out,
                           n, d, k, 1, 0, 0, nullptr};
    return launch_tile<T, int32_t, MODE_DIST>(a, s);
}

namespace {

// Seeded uniform [-4, 4) samples for the autotuner's synthetic instance.
template <typename T>
__global__ void tune_fill_kernel(T *x, int64_t count, uint64_t seed) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x) {
        uint64_t z = (uint64_t)e * 0x9E3779B97F4A7C15ull + seed;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        x[e] = (T)((double)(z >> 11) * 0x1p-53 * 8.0 - 4.0);
    }
}

}  // namespace

template <typename T>
int tune_fit_variant(int64_t d, int64_t k_in, cudaStream_t s, int *variant) {
    Range range("kmc.tune_fit_variant");
    *variant = 0;
    if (const char *e = std::getenv("KMC_TUNE"))
        if (e[0] == '0') return KMC_OK;
    if (d < 1 || k_in < 1) return KMC_OK;
    int64_t k = 1;
    while (k < k_in) k <<= 1;
    const char *tag = sizeof(T) == 4 ? "fit-f32" : "fit-f64";
    if (tune_lookup(d, k, tag, variant)) return KMC_OK;
    const int n_var = sizeof(T) == 4 ? 3 : 2;
    const int64_t n = 65536;
    Scratch mem;
    const size_t oX = 0, oC = oX + align256(sizeof(T) * n * d), oh = oC + align256(sizeof(T) * d * k);
    const size_t ow = oh + align256(sizeof(T) * k), ol = ow + align256(sizeof(T) * n);
    const size_t os = ol + align256(sizeof(int32_t) * n);
    KMC_TRY(mem.alloc(os + align256(sizeof(double) * (d * k + k)), s));
    char *b = mem.as<char>();
    T *X = reinterpret_cast<T *>(b + oX), *C = reinterpret_cast<T *>(b + oC);
    T *hn = reinterpret_cast<T *>(b + oh), *w = reinterpret_cast<T *>(b + ow);
    int32_t *lab = reinterpret_cast<int32_t *>(b + ol);
    double *sums = reinterpret_cast<double *>(b + os);
    tune_fill_kernel<T><<<1024, 256, 0, s>>>(X, n * d, 11);
    tune_fill_kernel<T><<<64, 256, 0, s>>>(C, d * k, 12);
    KMC_TRY(check_launch("tune_fill"));
    KMC_TRY(launch_fill<T>(w, T(1), n, s));
    KMC_TRY(launch_half_norm<T>(C, hn, d, k, s));
    cudaEvent_t e0, e1;
    KMC_CUDA_TRY(cudaEventCreate(&e0));
    KMC_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 0.f;
    int best = 0, rc = KMC_OK;
    for (int v = 0; v < n_var && rc == KMC_OK; ++v) {
        float tot = 0.f;
        for (int rep = 0; rep < 4 && rc == KMC_OK; ++rep) {
            rc = launch_fill<double>(sums, 0.0, d * k + k, s);
            if (rc == KMC_OK) rc = cudaEventRecord(e0, s) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
            if (rc == KMC_OK)
                rc = launch_fused_step<T, int32_t, double>(X, w, C, hn, lab, sums, sums + d * k,
                                                           n, d, k, 1, s, nullptr, v);
            if (rc == KMC_OK) rc = cudaEventRecord(e1, s) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
            if (rc == KMC_OK) rc = cudaEventSynchronize(e1) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
            float ms = 0.f;
            if (rc == KMC_OK)
                rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
            if (rep > 0) tot += ms;  // the first run warms up
        }
        if (v == 0 || tot < best_ms) {
            best_ms = tot;
            best = v;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != KMC_OK) {
        set_error("tile autotuner: a timing launch failed");
        return rc;
    }
    tune_record(d, k, tag, best);
    *variant = best;
    return KMC_OK;
}

template int tune_fit_variant<float>(int64_t, int64_t, cudaStream_t, int *);
template int tune_fit_variant<double>(int64_t, int64_t, cudaStream_t, int *);

#define KMC_INST_LLOYD(T, I)                                                                 \
    template int launch_assignment<T, I>(const T *, const T *, const T *, I *, int64_t,      \
                                         int64_t, int64_t, cudaStream_t, const LoopState *,  \
                                         int);                                               \
    template int launch_fused_step<T, I, T>(const T *, const T *, const T *, const T *, I *,   \
                                            T *, T *, int64_t, int64_t, int64_t, int64_t,     \
                                            cudaStream_t, const LoopState *, int);            \


template int launch_fused_step<float, int32_t, double>(const float *, const float *,
                                                       const float *, const float *, int32_t *,
                                                       double *, double *, int64_t, int64_t,
                                                       int64_t, int64_t, cudaStream_t,
                                                       const LoopState *, int);
template int launch_fused_step<float, int64_t, double>(const float *, const float *,
                                                       const float *, const float *, int64_t *,
                                                       double *, double *, int64_t, int64_t,
                                                       int64_t, int64_t, cudaStream_t,
                                                       const LoopState *, int);
KMC_INST_LLOYD(float, int32_t)
KMC_INST_LLOYD(float, int64_t)
KMC_INST_LLOYD(double, int32_t)
KMC_INST_LLOYD(double, int64_t)
template int launch_distances<float>(const float *, const float *, float *, int64_t, int64_t,
                                     int64_t, cudaStream_t);
template int launch_distances<double>(const double *, const double *, double *, int64_t,
                                      int64_t, int64_t, cudaStream_t);

}  // namespace kmc
