// Empty-cluster relocation: threshold (topk-th largest value), selection of
// the samples farthest from their centroid, and the relocation itself.
//
// Reference: src/util_kernels.hpp:163-476 and src/iterative_merge_sort.hpp.
// The reference sorts all n distances (merge sort) to find the threshold when
// more than one cluster is empty; here a 4-pass (FP32) / 8-pass (FP64) radix
// select over order-preserving integer keys finds the same value in O(n)
// per pass.  The selection writes indices in a defined order (the reference's
// atomic order is arbitrary), and relocation processes empty clusters in list
// order, one thread per feature, so results are deterministic:
//   empty cluster r (r-th entry of the list) takes the r-th farthest sample,
//   farthest = larger sq_dist, ties broken by the lower sample index.
// For a single empty cluster this is exactly the reference's rule
// (util_kernels.hpp:353-357); for several it is the rule that code intends
// (its size_t index underflows when n_empty >= 2 and distances are distinct).
#include "km_kernels.cuh"

namespace kmc {

namespace {

__device__ __forceinline__ bool stopped(const LoopState *g) {
    return g != nullptr && *reinterpret_cast<const volatile int *>(&g->done) != 0;
}

__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }

// Order-preserving unsigned keys (larger value -> larger key).
template <typename T>
struct KeyOf;
template <>
struct KeyOf<float> {
    using U = uint32_t;
    static constexpr int kPasses = 4;
    __device__ static U key(float v) {
        U b = __float_as_uint(v);
        return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    }
    __device__ static float val(U k) {
        U b = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
        return __uint_as_float(b);
    }
};
template <>
struct KeyOf<double> {
    using U = unsigned long long;
    static constexpr int kPasses = 8;
    __device__ static U key(double v) {
        U b = (U)__double_as_longlong(v);
        return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
    }
    __device__ static double val(U k) {
        U b = (k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k;
        return __longlong_as_double((long long)b);
    }
};

// Radix-select scratch (device memory).
struct SelectState {
    unsigned long long hist[256];
    unsigned long long prefix;  // key bits fixed so far
    unsigned long long rank;    // rank (0-based, descending) still to find
    long long active;           // 0: nothing to do
    long long pad;
};

__global__ void threshold_init_kernel(SelectState *st, const int64_t *topk_dev,
                                      int64_t topk_host, int64_t n, const LoopState *guard) {
    int t = threadIdx.x;
    st->hist[t] = 0ull;
    if (t == 0) {
        int64_t topk = (topk_dev != nullptr) ? *topk_dev : topk_host;
        if (stopped(guard)) topk = 0;
        if (topk > n) topk = n;
        st->active = (topk > 0) ? 1 : 0;
        st->rank = (topk > 0) ? (unsigned long long)(topk - 1) : 0ull;
        st->prefix = 0ull;
    }
}

template <typename T>
__global__ void threshold_hist_kernel(const T *data, int64_t n, SelectState *st, int pass) {
    using K = KeyOf<T>;
    using U = typename K::U;
    if (st->active == 0) return;
    __shared__ unsigned int h[256];
    for (int b = threadIdx.x; b < 256; b += blockDim.x) h[b] = 0u;
    __syncthreads();
    constexpr int kBits = 8 * (int)sizeof(U);
    const int shift = kBits - 8 * (pass + 1);
    const U prefix = (U)st->prefix;
    const U hi_mask = (pass == 0) ? (U)0 : (U)(~(U)0) << (kBits - 8 * pass);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        U key = K::key(data[i]);
        if ((key & hi_mask) == prefix) atomicAdd(&h[(unsigned)(key >> shift) & 0xffu], 1u);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < 256; b += blockDim.x)
        if (h[b]) atomicAdd(&st->hist[b], (unsigned long long)h[b]);
}

template <typename T>
__global__ void threshold_digit_kernel(SelectState *st, int pass, T *threshold) {
    using K = KeyOf<T>;
    using U = typename K::U;
    if (st->active == 0) return;
    __shared__ unsigned long long h[256];
    int t = threadIdx.x;
    h[t] = st->hist[t];
    __syncthreads();
    if (t == 0) {
        constexpr int kBits = 8 * (int)sizeof(U);
        const int shift = kBits - 8 * (pass + 1);
        unsigned long long r = st->rank, cum = 0ull;
        int digit = 0;
        for (int b = 255; b >= 0; --b) {
            if (cum + h[b] > r) {
                digit = b;
                r -= cum;
                break;
            }
            cum += h[b];
        }
        st->rank = r;
        st->prefix |= ((unsigned long long)digit) << shift;
        if (pass == K::kPasses - 1) *threshold = K::val((U)st->prefix);
    }
    __syncthreads();
    st->hist[t] = 0ull;
}

// ---------------------------------------------------------------------------
// Ordered selection (select_samples_far_from_centroid_kernel,
// src/util_kernels.hpp:211-297).
// ---------------------------------------------------------------------------
constexpr int kSelGrid = 512;
constexpr int kSelBlock = 256;

struct SelHeader {
    long long total_gt, total_eq;
    long long gt_init, eq_init;
    long long need_eq;
    long long sorted;  // 1: gt elements are ranked, 0: written in index order
    long long n_sel;
    long long active;
    long long n_total;
};

// Up to this many selections the strictly-greater samples (fewer than
// n_selected) are ranked by counting all pairs; beyond it by a merge sort.
constexpr int64_t kRankAllPairs = 4096;

struct SelLayout {
    SelHeader *hdr;
    long long *cnt_gt, *cnt_eq;  // [kSelGrid]
    long long *gt_list;          // [max_selected] indices, used when ranking
    long long *gt_tmp;           // [max_selected] second merge buffer (max_selected > kRankAllPairs)
};

__host__ __device__ inline SelLayout sel_layout(void *base, int64_t max_selected) {
    char *p = static_cast<char *>(base);
    SelLayout L;
    L.hdr = reinterpret_cast<SelHeader *>(p);
    p += 256;
    L.cnt_gt = reinterpret_cast<long long *>(p);
    p += sizeof(long long) * kSelGrid;
    L.cnt_eq = reinterpret_cast<long long *>(p);
    p += sizeof(long long) * kSelGrid;
    L.gt_list = reinterpret_cast<long long *>(p);
    L.gt_tmp = L.gt_list + (max_selected > 0 ? max_selected : 1);
    return L;
}

__device__ __forceinline__ void block_range(int64_t n, int64_t &b0, int64_t &b1) {
    int64_t chunk = ceil_div<int64_t>(n, gridDim.x);
    b0 = blockIdx.x * chunk;
    b1 = b0 + chunk;
    if (b1 > n) b1 = n;
    if (b0 > n) b0 = n;
}

template <typename T>
__global__ void select_count_kernel(const T *dist, const T *thr, int64_t n, SelLayout L,
                                    const int64_t *gate, const LoopState *guard) {
    __shared__ long long sg[32], se[32];
    if (stopped(guard) || (gate != nullptr && *gate == 0)) return;
    int64_t b0, b1;
    block_range(n, b0, b1);
    const T th = *thr;
    long long g = 0, e = 0;
    for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        T v = dist[i];
        g += (v > th);
        e += (v == th);
    }
    for (int o = 16; o > 0; o >>= 1) {
        g += __shfl_down_sync(0xffffffffu, g, o);
        e += __shfl_down_sync(0xffffffffu, e, o);
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sg[wid] = g;
        se[wid] = e;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        long long G = 0, E = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            G += sg[w];
            E += se[w];
        }
        L.cnt_gt[blockIdx.x] = G;
        L.cnt_eq[blockIdx.x] = E;
    }
}

template <typename I>
__global__ void select_scan_kernel(SelLayout L, const int64_t *n_sel_dev, int64_t n_sel_host,
                                   I *n_gt, I *n_eq, int64_t n_total, const int64_t *gate,
                                   const LoopState *guard) {
    if (threadIdx.x != 0) return;
    SelHeader *h = L.hdr;
    if (stopped(guard) || (gate != nullptr && *gate == 0)) {
        h->active = 0;
        return;
    }
    long long sg = 0, se = 0;
    for (int b = 0; b < kSelGrid; ++b) {
        long long g = L.cnt_gt[b], e = L.cnt_eq[b];
        L.cnt_gt[b] = sg;
        L.cnt_eq[b] = se;
        sg += g;
        se += e;
    }
    long long n_sel = (n_sel_dev != nullptr) ? (long long)*n_sel_dev : (long long)n_sel_host;
    h->active = 1;
    h->n_sel = n_sel;
    h->n_total = n_total;
    h->total_gt = sg;
    h->total_eq = se;
    h->gt_init = (long long)*n_gt;
    h->eq_init = (long long)*n_eq;
    h->sorted = (sg < n_sel) ? 1 : 0;
    long long need = (sg < n_sel) ? (n_sel - sg) : 0;
    if (need > se) need = se;
    h->need_eq = need;
    *n_gt = (I)(h->gt_init + sg);
    *n_eq = (I)(h->eq_init + need);
}

template <typename T, typename I>
__global__ void select_write_kernel(const T *dist, const T *thr, int64_t n, SelLayout L,
                                    I *selected) {
    __shared__ int wg[32], we[32];
    __shared__ long long base_g, base_e;
    const SelHeader *h = L.hdr;
    if (h->active == 0) return;
    int64_t b0, b1;
    block_range(n, b0, b1);
    const T th = *thr;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) {
        base_g = L.cnt_gt[blockIdx.x];
        base_e = L.cnt_eq[blockIdx.x];
    }
    __syncthreads();
    const long long gt_init = h->gt_init, eq_init = h->eq_init, need_eq = h->need_eq;
    const bool sorted = h->sorted != 0;
    for (int64_t c0 = b0; c0 < b1; c0 += blockDim.x) {
        int64_t i = c0 + threadIdx.x;
        bool in = i < b1;
        T v = in ? dist[i] : T(0);
        bool isg = in && (v > th), ise = in && (v == th);
        unsigned bg = __ballot_sync(0xffffffffu, isg), be = __ballot_sync(0xffffffffu, ise);
        if (lane == 0) {
            wg[wid] = __popc(bg);
            we[wid] = __popc(be);
        }
        __syncthreads();
        long long pg = 0, pe = 0, tg = 0, te = 0;
        for (int w = 0; w < nw; ++w) {
            if (w < wid) {
                pg += wg[w];
                pe += we[w];
            }
            tg += wg[w];
            te += we[w];
        }
        unsigned lm = (1u << lane) - 1u;
        if (isg) {
            long long ord = base_g + pg + __popc(bg & lm);
            if (sorted) {
                L.gt_list[ord] = i;
            } else {
                long long pos = gt_init + ord;  // counters are caller-initialised
                if (pos >= 0 && pos < n) selected[pos] = (I)i;
            }
        }
        if (ise) {
            long long ord = base_e + pe + __popc(be & lm);
            long long pos = n - (eq_init + ord);
            if (ord < need_eq && pos >= 0 && pos < n) selected[pos] = (I)i;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            base_g += tg;
            base_e += te;
        }
        __syncthreads();
    }
}

// Ranks the (at most n_sel - 1 <= kRankAllPairs) strictly-greater samples by
// (distance desc, index asc), counting all pairs, and stores them so that
// selected[gt_init + m - 1 - r] holds the r-th farthest.
template <typename T, typename I>
__global__ void select_rank_kernel(const T *dist, SelLayout L, I *selected) {
    const SelHeader *h = L.hdr;
    if (h->active == 0 || h->sorted == 0) return;
    const long long m = h->total_gt;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        long long ie = L.gt_list[e];
        T ve = dist[ie];
        long long r = 0;
        for (long long q = 0; q < m; ++q) {
            long long iq = L.gt_list[q];
            T vq = dist[iq];
            r += (vq > ve) || (vq == ve && iq < ie);
        }
        long long pos = h->gt_init + m - 1 - r;
        if (pos >= 0 && pos < h->n_total) selected[pos] = (I)ie;
    }
}

// Sample a comes before sample b in the selection order: farther first,
// the lower index on equal distances (a strict total order: indices differ).
template <typename T>
__device__ __forceinline__ bool sel_before(const T *dist, long long a, long long b) {
    const T va = dist[a], vb = dist[b];
    return va > vb || (va == vb && a < b);
}

// Number of entries of the sorted run r[0, len) that come before sample e.
template <typename T>
__device__ __forceinline__ long long count_before(const T *dist, const long long *r, long long len,
                                                  long long e) {
    long long lo = 0, hi = len;
    while (lo < hi) {
        const long long mid = (lo + hi) >> 1;
        if (sel_before(dist, r[mid], e)) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One pass of the merge sort of the m strictly-greater samples (more than
// kRankAllPairs selections): runs of `len` sorted entries of src are merged
// pairwise into dst.  An entry's place in the merged run is its place in its
// own run plus the number of entries of the partner run before it, found by
// binary search (O(m log len) per pass).  gt_list holds the samples in
// ascending index order initially, so the first pass starts from runs of 1.
// A pass whose runs already cover all m entries does nothing.
template <typename T>
__global__ void select_merge_kernel(const T *dist, SelLayout L, int pass) {
    const SelHeader *h = L.hdr;
    if (h->active == 0 || h->sorted == 0) return;
    const long long m = h->total_gt, len = 1ll << pass;
    if (len >= m) return;
    const long long *src = (pass & 1) ? L.gt_tmp : L.gt_list;
    long long *dst = (pass & 1) ? L.gt_list : L.gt_tmp;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < m;
         e += (long long)gridDim.x * blockDim.x) {
        const long long base = (e / (2 * len)) * (2 * len);
        const long long a_len = (m - base < len) ? (m - base) : len;
        const long long b0 = base + a_len;
        const long long b_len = (m - b0 < len) ? (m - b0) : len;
        const long long v = src[e];
        long long pos;
        if (e < b0)
            pos = e + count_before(dist, src + b0, b_len, v);
        else
            pos = base + count_before(dist, src + base, a_len, v) + (e - b0);
        dst[pos] = v;
    }
}

// After the merge passes: the sorted list (in the buffer the last effective
// pass wrote) goes to selected[gt_init + m - 1 - r] for the r-th farthest.
template <typename T, typename I>
__global__ void select_place_kernel(SelLayout L, I *selected) {
    const SelHeader *h = L.hdr;
    if (h->active == 0 || h->sorted == 0) return;
    const long long m = h->total_gt;
    int passes = 0;
    while ((1ll << passes) < m) ++passes;
    const long long *srt = (passes & 1) ? L.gt_tmp : L.gt_list;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < m;
         r += (long long)gridDim.x * blockDim.x) {
        const long long pos = h->gt_init + m - 1 - r;
        if (pos >= 0 && pos < h->n_total) selected[pos] = (I)srt[r];
    }
}

// relocate_empty_clusters_kernel, src/util_kernels.hpp:302-390.
template <typename T, typename I>
__global__ void relocate_kernel(const int64_t *n_empty_dev, int64_t n_empty_host, const T *X,
                                const T *w, const I *labels, const I *selected, const I *n_gt,
                                const I *empty_list, T *sums, T *sizes, T *inertia, int64_t n,
                                int64_t d, int64_t k, const LoopState *guard, int64_t fs,
                                int64_t ss) {
    if (stopped(guard)) return;
    int64_t n_empty = (n_empty_dev != nullptr) ? *n_empty_dev : n_empty_host;
    if (n_empty <= 0) return;
    const int64_t gt = (int64_t)*n_gt;
    // Samples available: the gt ones plus the eq ones written at the back.
    if (n_empty > n) n_empty = n;
    int64_t f = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (f >= d) return;
    for (int64_t r = 0; r < n_empty; ++r) {
        int64_t pos = (r < gt) ? (gt - 1 - r) : (n - 1 - (r - gt));
        if (pos < 0 || pos >= n) continue;
        int64_t s = (int64_t)selected[pos];
        if (s < 0 || s >= n) continue;
        int64_t old = (int64_t)labels[s];
        int64_t cl = (int64_t)empty_list[r];
        // caller-supplied indices: never dereference out of range
        if (old < 0 || old >= k || cl < 0 || cl >= k) continue;
        T wv = w[s];
        T xw = mul_rn(X[f * fs + s * ss], wv);  // rounded product, as in the reference
        sums[f * k + old] -= xw;
        sums[f * k + cl] = xw;
        if (f == 0) {
            sizes[old] -= wv;
            sizes[cl] = wv;
            inertia[s] = T(0);
        }
    }
}

template <typename I>
__global__ void gate_kernel(const I *n_empty, int64_t *gate, const LoopState *guard) {
    if (threadIdx.x == 0) *gate = stopped(guard) ? 0 : (int64_t)*n_empty;
}

}  // namespace

size_t threshold_scratch_bytes() { return align256(sizeof(SelectState)); }

template <typename T>
int launch_threshold(const T *data, int64_t n, const int64_t *topk_dev, int64_t topk_host,
                     T *threshold, void *scratch, cudaStream_t s, const LoopState *guard) {
    SelectState *st = static_cast<SelectState *>(scratch);
    threshold_init_kernel<<<1, 256, 0, s>>>(st, topk_dev, topk_host, n, guard);
    KMC_TRY(check_launch("threshold_init"));
    int64_t g = ceil_div<int64_t>(n, 1024);
    int grid = (int)std::max<int64_t>(1, std::min<int64_t>(g, (int64_t)num_sms() * 4));
    for (int pass = 0; pass < KeyOf<T>::kPasses; ++pass) {
        threshold_hist_kernel<T><<<grid, 1024, 0, s>>>(data, n, st, pass);
        KMC_TRY(check_launch("threshold_hist"));
        threshold_digit_kernel<T><<<1, 256, 0, s>>>(st, pass, threshold);
        KMC_TRY(check_launch("threshold_digit"));
    }
    return KMC_OK;
}

size_t select_scratch_bytes(int64_t max_selected) {
    const size_t m = (size_t)(max_selected > 0 ? max_selected : 1);
    const size_t lists = (max_selected > kRankAllPairs) ? 2 : 1;
    return align256(256 + 2 * sizeof(long long) * kSelGrid + sizeof(long long) * m * lists);
}

int64_t select_launches(int64_t max_selected) {
    if (max_selected <= kRankAllPairs) return 4;
    int64_t passes = 0;
    while ((int64_t(1) << passes) < max_selected) ++passes;
    return 3 + passes + 1;
}

template <typename T, typename I>
int launch_select(const int64_t *n_selected_dev, int64_t n_selected_host, const T *dist,
                  const T *threshold, I *selected, I *n_gt, I *n_eq, int64_t n, void *scratch,
                  int64_t max_selected, cudaStream_t s, const LoopState *guard) {
    SelLayout L = sel_layout(scratch, max_selected);
    const int64_t *gate = n_selected_dev;
    select_count_kernel<T><<<kSelGrid, kSelBlock, 0, s>>>(dist, threshold, n, L, gate, guard);
    KMC_TRY(check_launch("select_count"));
    select_scan_kernel<I><<<1, 32, 0, s>>>(L, n_selected_dev, n_selected_host, n_gt, n_eq, n,
                                           gate, guard);
    KMC_TRY(check_launch("select_scan"));
    select_write_kernel<T, I><<<kSelGrid, kSelBlock, 0, s>>>(dist, threshold, n, L, selected);
    KMC_TRY(check_launch("select_write"));
    if (max_selected <= kRankAllPairs) {
        select_rank_kernel<T, I><<<64, 256, 0, s>>>(dist, L, selected);
        return check_launch("select_rank");
    }
    // at most max_selected - 1 entries: ceil(log2(max_selected)) passes cover them
    const unsigned grid =
        (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div<int64_t>(max_selected, 256),
                                                         (int64_t)num_sms() * 8));
    for (int pass = 0; (int64_t(1) << pass) < max_selected; ++pass) {
        select_merge_kernel<T><<<grid, 256, 0, s>>>(dist, L, pass);
        KMC_TRY(check_launch("select_merge"));
    }
    select_place_kernel<T, I><<<grid, 256, 0, s>>>(L, selected);
    return check_launch("select_place");
}

template <typename T, typename I>
int launch_relocate(const int64_t *n_empty_dev, int64_t n_empty_host, const T *X, const T *w,
                    const I *labels, const I *selected, const I *n_gt, const I *empty_list,
                    T *sums, T *sizes, T *inertia, int64_t n, int64_t d, int64_t k,
                    cudaStream_t s, const LoopState *guard, int64_t x_fstride,
                    int64_t x_sstride) {
    int grid = (int)ceil_div<int64_t>(std::max<int64_t>(d, 1), 128);
    const int64_t fs = x_fstride > 0 ? x_fstride : n, ss = x_fstride > 0 ? x_sstride : 1;
    relocate_kernel<T, I><<<grid, 128, 0, s>>>(n_empty_dev, n_empty_host, X, w, labels, selected,
                                               n_gt, empty_list, sums, sizes, inertia, n, d, k,
                                               guard, fs, ss);
    return check_launch("relocate");
}

template <typename I>
int launch_gate_from_count(const I *n_empty, int64_t *gate, cudaStream_t s,
                           const LoopState *guard) {
    gate_kernel<I><<<1, 32, 0, s>>>(n_empty, gate, guard);
    return check_launch("relocation_gate");
}

template int launch_threshold<float>(const float *, int64_t, const int64_t *, int64_t, float *,
                                     void *, cudaStream_t, const LoopState *);
template int launch_threshold<double>(const double *, int64_t, const int64_t *, int64_t,
                                      double *, void *, cudaStream_t, const LoopState *);
#define KMC_INST_RELOC(T, I)                                                                  \
    template int launch_select<T, I>(const int64_t *, int64_t, const T *, const T *, I *, I *, \
                                     I *, int64_t, void *, int64_t, cudaStream_t,             \
                                     const LoopState *);                                      \
    template int launch_relocate<T, I>(const int64_t *, int64_t, const T *, const T *,        \
                                       const I *, const I *, const I *, const I *, T *, T *,  \
                                       T *, int64_t, int64_t, int64_t, cudaStream_t,          \
                                       const LoopState *, int64_t, int64_t);
KMC_INST_RELOC(float, int32_t)
KMC_INST_RELOC(float, int64_t)
KMC_INST_RELOC(double, int32_t)
KMC_INST_RELOC(double, int64_t)
template int launch_gate_from_count<int32_t>(const int32_t *, int64_t *, cudaStream_t,
                                             const LoopState *);
template int launch_gate_from_count<int64_t>(const int64_t *, int64_t *, cudaStream_t,
                                             const LoopState *);

}  // namespace kmc
