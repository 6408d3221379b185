// extern "C" entry points declared in include/kmeans_gb300.h.
//
// Each entry point validates sizes, selects the dtype instantiation and calls
// the kernel launchers.  Array-shape validation of the Python surface lives in
// the pybind11 module, mirroring python_api/_kmeans_lloyd.cpp.
#include <cstdarg>
#include <cstring>
#include <memory>
#include <mutex>

#include "km_fit.cuh"
#include "km_kernels.cuh"

namespace kmc {

namespace {
thread_local char g_err[1024] = "";
}

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

const char *get_error() { return g_err; }

std::atomic<long long> g_fail_alloc_after{-1};

int num_sms() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 148;
    if (cache[dev] == 0) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 148;
    }
    return cache[dev];
}

namespace {
std::mutex g_pool_mu;
cudaMemPool_t g_pools[64] = {};
}  // namespace

cudaMemPool_t scratch_pool() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_pool_mu);
    if (g_pools[dev] == nullptr) {
        cudaMemPoolProps props;
        std::memset(&props, 0, sizeof(props));
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool = nullptr;
        if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;  // callers fall back to the device's default pool
        }
        uint64_t keep = ~uint64_t(0);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        g_pools[dev] = pool;
    }
    return g_pools[dev];
}

int trim_pools() {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    for (int d = 0; d < 64; ++d)
        if (g_pools[d] != nullptr) KMC_CUDA_TRY(cudaMemPoolTrimTo(g_pools[d], 0));
    return KMC_OK;
}

int64_t l2_bytes() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    cudaDeviceGetAttribute(&v, cudaDevAttrL2CacheSize, dev);
    return v;
}

}  // namespace kmc

using namespace kmc;

namespace {

inline cudaStream_t S(kmc_stream_t s) { return reinterpret_cast<cudaStream_t>(s); }

#define CHECK_DIMS(...)                                                              \
    do {                                                                             \
        int64_t _dims[] = {__VA_ARGS__};                                             \
        for (int64_t _v : _dims)                                                     \
            KMC_CHECK_ARG(_v >= 0, "array dimensions must be non-negative");         \
    } while (0)

template <typename T>
int broadcast_divide(T *X, const T *y, int64_t rows, int64_t cols, cudaStream_t s) {
    CHECK_DIMS(rows, cols);
    return launch_broadcast_divide<T>(X, y, rows, cols, s);
}

template <typename T>
int half_norm(const T *C, T *out, int64_t d, int64_t k, cudaStream_t s) {
    CHECK_DIMS(d, k);
    return launch_half_norm<T>(C, out, d, k, s);
}

template <typename T, typename I>
int reduce_centroids(const T *sz_cp, const T *c_cp, T *out_sz, T *out_c, I *list, I *n_empty,
                     int64_t P, int64_t d, int64_t k, cudaStream_t s) {
    CHECK_DIMS(P, d, k);
    return launch_reduce_centroids<T, I, T>(sz_cp, c_cp, out_sz, out_c, list, n_empty, P, d, k,
                                             s);
}

template <typename T>
int compute_threshold(const T *data, int64_t n, int64_t topk, T *thr, cudaStream_t s) {
    CHECK_DIMS(n, topk);
    if (topk == 0) return KMC_OK;  // _kmeans_lloyd.cpp:312-316
    KMC_CHECK_ARG(topk <= n, "topk (%lld) exceeds the number of elements (%lld)",
                  (long long)topk, (long long)n);
    Scratch sc;
    KMC_TRY(sc.alloc(threshold_scratch_bytes(), s));
    return launch_threshold<T>(data, n, nullptr, topk, thr, sc.ptr, s);
}

template <typename T, typename I>
int select_far(int64_t n_sel, const T *dist, const T *thr, I *sel, I *n_gt, I *n_eq, int64_t n,
               cudaStream_t s) {
    CHECK_DIMS(n_sel, n);
    KMC_CHECK_ARG(n_sel > 0, "Argument `n_selected` must be positive");
    KMC_CHECK_ARG(n_sel <= n, "Argument `n_select` is too large");
    Scratch sc;
    KMC_TRY(sc.alloc(select_scratch_bytes(n_sel), s));
    return launch_select<T, I>(nullptr, n_sel, dist, thr, sel, n_gt, n_eq, n, sc.ptr, n_sel, s);
}

template <typename T, typename I>
int relocate(int64_t n_empty, const T *X, const T *w, const I *labels, const I *list,
             const T *sq_dist, T *C, T *sizes, T *inertia, int64_t n, int64_t d, int64_t k,
             cudaStream_t s) {
    CHECK_DIMS(n_empty, n, d, k);
    KMC_CHECK_ARG(n_empty != 0, "n_empty_clusters must be non-zero.");
    KMC_CHECK_ARG(n_empty <= k, "n_empty_clusters exceeds n_clusters");
    KMC_CHECK_ARG(n_empty <= n, "n_empty_clusters exceeds n_samples");
    // relocate_empty_clusters, src/util_kernels.hpp:392-476
    size_t o_thr = 0, o_tsc = align256(sizeof(T)), o_cnt = o_tsc + threshold_scratch_bytes();
    size_t o_sel = o_cnt + align256(2 * sizeof(I));
    size_t o_ssc = o_sel + align256(sizeof(I) * n);
    size_t total = o_ssc + select_scratch_bytes(n_empty);
    Scratch sc;
    KMC_TRY(sc.alloc(total, s));
    char *b = sc.as<char>();
    T *thr = reinterpret_cast<T *>(b + o_thr);
    I *cnt = reinterpret_cast<I *>(b + o_cnt);
    I *sel = reinterpret_cast<I *>(b + o_sel);
    KMC_TRY(launch_threshold<T>(sq_dist, n, nullptr, n_empty, thr, b + o_tsc, s));
    KMC_TRY(launch_fill<I>(cnt, I(0), 1, s));
    KMC_TRY(launch_fill<I>(cnt + 1, I(1), 1, s));
    KMC_TRY(launch_select<T, I>(nullptr, n_empty, sq_dist, thr, sel, cnt, cnt + 1, n, b + o_ssc,
                                n_empty, s));
    return launch_relocate<T, I>(nullptr, n_empty, X, w, labels, sel, cnt, list, C, sizes,
                                 inertia, n, d, k, s);
}

template <typename T>
int shifts(const T *a, const T *b, T *out, int64_t d, int64_t k, cudaStream_t s) {
    CHECK_DIMS(d, k);
    return launch_shifts<T>(a, b, out, d, k, s);
}

template <typename T>
int distances(const T *X, const T *C, T *out, int64_t n, int64_t d, int64_t k, cudaStream_t s) {
    CHECK_DIMS(n, d, k);
    return launch_distances<T>(X, C, out, n, d, k, s);
}

template <typename T, typename I>
int assignment(const T *X, const T *C, const T *hn, I *out, int64_t n, int64_t d, int64_t k,
               cudaStream_t s) {
    CHECK_DIMS(n, d, k);
    KMC_CHECK_ARG(k > 0 || n == 0, "n_clusters must be positive");
    return launch_assignment<T, I>(X, C, hn, out, n, d, k, s);
}

template <typename T, typename I>
int inertia(const T *X, const T *w, const T *C, const I *lab, T *out, int64_t n, int64_t d,
            int64_t k, cudaStream_t s) {
    CHECK_DIMS(n, d, k);
    return launch_inertia<T, I>(X, w, C, lab, out, n, d, k, s);
}

template <typename T>
int reduce_vector(const T *data, int64_t n, cudaStream_t s, T *result) {
    CHECK_DIMS(n);
    KMC_CHECK_ARG(result != nullptr, "result pointer is null");
    Scratch sc;
    KMC_TRY(sc.alloc(sizeof(double) * (sum_partials_size() + 1), s));
    double *part = sc.as<double>();
    KMC_TRY(launch_sum_f64<T>(data, n, part, part + sum_partials_size(), s));
    double tot = 0.0;
    KMC_CUDA_TRY(cudaMemcpyAsync(&tot, part + sum_partials_size(), sizeof(double),
                                 cudaMemcpyDeviceToHost, s));
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    *result = (T)tot;
    return KMC_OK;
}

template <typename T, typename I>
int fused_step(const T *X, const T *w, const T *C, const T *hn, I *lab, T *sums, T *sizes,
               int64_t n, int64_t d, int64_t k, int64_t P, cudaStream_t s) {
    CHECK_DIMS(n, d, k, P);
    KMC_CHECK_ARG(P >= 1 || n == 0, "n_copies must be positive");
    KMC_CHECK_ARG(k > 0 || n == 0, "n_clusters must be positive");
    return launch_fused_step<T, I, T>(X, w, C, hn, lab, sums, sizes, n, d, k, P, s);
}

template <typename T, typename I>
int make_fit(const FitParams<T, I> &p, int form, std::unique_ptr<FitBase> *out) {
    Range range("kmc.fit_create");
    if (form == KMC_FORM_PLAIN) {
        auto f = std::make_unique<PlainFit<T, I>>();
        KMC_TRY(f->init(p));
        *out = std::move(f);
        return KMC_OK;
    }
    KMC_CHECK_ARG(form == KMC_FORM_MIXED_BF16 || form == KMC_FORM_MIXED_FP16,
                  "unknown form %d", form);
    return make_mixed_fit<T, I>(p, form, out);
}

template <typename T, typename I>
int driver(const T *X, const T *w, T *init_c, I *labels, T *res_c, int64_t n, int64_t d,
           int64_t k, double tol, int verbose, int64_t max_iter, double occ, cudaStream_t s,
           kmc_print_fn pf, void *pctx, int64_t *n_iter_out, T *inertia_out) {
    Range range("kmc.lloyd_driver");
    CHECK_DIMS(n, d, k, max_iter);
    KMC_CHECK_ARG(occ > 0.0 && occ < 1.0,
                  "Fraction `centroids_private_copies_max_cache_occupancy` is out of bounds");
    KMC_CHECK_ARG(tol >= 0.0, "Tolerance must be non-negative");
    KMC_CHECK_ARG(k > 0, "n_clusters must be positive");
    FitParams<T, I> p;
    p.X = X;
    p.w = w;
    p.centroids = init_c;
    p.new_centroids = res_c;
    p.labels = labels;
    p.n = n;
    p.d = d;
    p.k = k;
    p.tol = tol;
    p.max_iter = max_iter;
    p.verbose = verbose;
    p.print_fn = pf;
    p.print_ctx = pctx;
    p.stream = s;
    int64_t it = 0;
    double tot = 0.0;
    {
        std::unique_ptr<FitBase> fit;
        KMC_TRY(make_fit<T, I>(p, KMC_FORM_PLAIN, &fit));
        KMC_TRY(fit->run(0));
        KMC_TRY(fit->finalize(&it, &tot));
    }
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    if (n_iter_out) *n_iter_out = it;
    if (inertia_out) *inertia_out = (T)tot;
    return KMC_OK;
}

template <typename T, typename I>
int fit_create(const T *X, const T *w, T *c, I *labels, T *rc, int64_t n, int64_t d, int64_t k,
               double tol, int64_t max_iter, int form, cudaStream_t s, FitBase **out,
               int rowmajor = 0) {
    CHECK_DIMS(n, d, k, max_iter);
    KMC_CHECK_ARG(out != nullptr, "null output pointer");
    KMC_CHECK_ARG(k > 0, "n_clusters must be positive");
    KMC_CHECK_ARG(tol >= 0.0, "Tolerance must be non-negative");
    FitParams<T, I> p;
    p.X = X;
    p.w = w;
    p.centroids = c;
    p.new_centroids = rc;
    p.labels = labels;
    p.n = n;
    p.d = d;
    p.k = k;
    p.tol = tol;
    p.max_iter = max_iter;
    p.stream = s;
    p.x_rowmajor = rowmajor;
    std::unique_ptr<FitBase> fit;
    KMC_TRY(make_fit<T, I>(p, form, &fit));
    *out = fit.release();
    return KMC_OK;
}

}  // namespace

struct kmc_fit_s {
    kmc::FitBase *impl;
};

extern "C" {

const char *kmc_last_error(void) { return kmc::get_error(); }
int kmc_abi_version(void) { return 1; }
int kmc_trim_cached_memory(void) { return kmc::trim_pools(); }

int kmc_scratch_bytes_in_use(int64_t *bytes_out) {
    KMC_CHECK_ARG(bytes_out != nullptr, "null output pointer");
    *bytes_out = 0;
    cudaMemPool_t pool = kmc::scratch_pool();
    if (pool == nullptr) return KMC_OK;
    unsigned long long used = 0;  // the attribute is a 64-bit unsigned value
    KMC_CUDA_TRY(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used));
    *bytes_out = (int64_t)used;
    return KMC_OK;
}

int kmc_debug_fail_allocation(int64_t after) {
    kmc::g_fail_alloc_after.store(after < 0 ? -1 : after);
    return KMC_OK;
}

#define KMC_T_ENTRY(SUF, T)                                                                    \
    int kmc_broadcast_divide_##SUF(T *X, const T *y, int64_t r, int64_t c, int64_t,            \
                                   kmc_stream_t s) {                                           \
        return broadcast_divide<T>(X, y, r, c, S(s));                                          \
    }                                                                                          \
    int kmc_half_l2_norm_squared_##SUF(const T *C, T *o, int64_t d, int64_t k, int64_t,        \
                                       kmc_stream_t s) {                                       \
        return half_norm<T>(C, o, d, k, S(s));                                                 \
    }                                                                                          \
    int kmc_compute_threshold_##SUF(const T *x, int64_t n, int64_t topk, T *thr,               \
                                    kmc_stream_t s) {                                          \
        return compute_threshold<T>(x, n, topk, thr, S(s));                                    \
    }                                                                                          \
    int kmc_compute_centroid_shifts_squared_##SUF(const T *a, const T *b, T *o, int64_t d,     \
                                                  int64_t k, kmc_stream_t s) {                 \
        return shifts<T>(a, b, o, d, k, S(s));                                                 \
    }                                                                                          \
    int kmc_compute_centroid_to_sample_distances_##SUF(const T *X, const T *C, T *o,          \
                                                       int64_t n, int64_t d, int64_t k,        \
                                                       int64_t, int64_t, kmc_stream_t s) {     \
        return distances<T>(X, C, o, n, d, k, S(s));                                           \
    }                                                                                          \
    int kmc_reduce_vector_blocking_##SUF(const T *x, int64_t n, kmc_stream_t s, T *r) {        \
        return reduce_vector<T>(x, n, S(s), r);                                                \
    }

#define KMC_TI_ENTRY(SUF, T, I)                                                                \
    int kmc_reduce_centroids_data_##SUF(const T *zc, const T *cc, T *oz, T *oc, I *l, I *ne,   \
                                        int64_t P, int64_t d, int64_t k, int64_t,              \
                                        kmc_stream_t s) {                                      \
        return reduce_centroids<T, I>(zc, cc, oz, oc, l, ne, P, d, k, S(s));                   \
    }                                                                                          \
    int kmc_select_samples_far_from_centroid_##SUF(int64_t m, const T *dist, const T *thr,     \
                                                   I *sel, I *ng, I *nq, int64_t n, int64_t,   \
                                                   kmc_stream_t s) {                           \
        return select_far<T, I>(m, dist, thr, sel, ng, nq, n, S(s));                           \
    }                                                                                          \
    int kmc_relocate_empty_clusters_##SUF(int64_t ne, const T *X, const T *w, const I *lab,    \
                                          const I *list, const T *sq, T *C, T *sz, T *inr,     \
                                          int64_t n, int64_t d, int64_t k, int64_t,            \
                                          kmc_stream_t s) {                                    \
        return relocate<T, I>(ne, X, w, lab, list, sq, C, sz, inr, n, d, k, S(s));             \
    }                                                                                          \
    int kmc_assignment_##SUF(const T *X, const T *C, const T *hn, I *o, int64_t n, int64_t d,  \
                             int64_t k, int64_t, int64_t, kmc_stream_t s) {                    \
        return assignment<T, I>(X, C, hn, o, n, d, k, S(s));                                   \
    }                                                                                          \
    int kmc_compute_inertia_##SUF(const T *X, const T *w, const T *C, const I *lab, T *o,      \
                                  int64_t n, int64_t d, int64_t k, int64_t, kmc_stream_t s) {  \
        return inertia<T, I>(X, w, C, lab, o, n, d, k, S(s));                                  \
    }                                                                                          \
    int kmc_fused_lloyd_single_step_##SUF(const T *X, const T *w, const T *C, const T *hn,     \
                                          I *lab, T *sums, T *sizes, int64_t n, int64_t d,     \
                                          int64_t k, int64_t P, int64_t, int64_t,              \
                                          kmc_stream_t s) {                                    \
        return fused_step<T, I>(X, w, C, hn, lab, sums, sizes, n, d, k, P, S(s));              \
    }                                                                                          \
    int kmc_lloyd_driver_##SUF(const T *X, const T *w, T *ic, I *lab, T *rc, int64_t n,        \
                               int64_t d, int64_t k, double tol, int verbose,                  \
                               int64_t max_iter, int64_t, int64_t, double occ,                 \
                               kmc_stream_t s, kmc_print_fn pf, void *pctx, int64_t *it,       \
                               T *inr) {                                                       \
        return driver<T, I>(X, w, ic, lab, rc, n, d, k, tol, verbose, max_iter, occ, S(s), pf, \
                            pctx, it, inr);                                                    \
    }

KMC_T_ENTRY(f32, float)
KMC_T_ENTRY(f64, double)
KMC_TI_ENTRY(f32_i32, float, int32_t)
KMC_TI_ENTRY(f32_i64, float, int64_t)
KMC_TI_ENTRY(f64_i32, double, int32_t)
KMC_TI_ENTRY(f64_i64, double, int64_t)

// compute_number_of_private_copies, src/lloyd_single_step.hpp:12-35.
int kmc_compute_number_of_private_copies(int64_t element_size, int64_t n, int64_t d, int64_t k,
                                         double occ, int64_t wgs, int64_t l2, int64_t *out) {
    KMC_CHECK_ARG(out != nullptr, "output pointer is null");
    KMC_CHECK_ARG(occ > 0.0 && occ < 1.0, "Expecting a fraction strictly between 0 and 1");
    KMC_CHECK_ARG(element_size > 0 && n >= 0 && d >= 0 && k > 0 && wgs > 0,
                  "invalid sizes for compute_number_of_private_copies");
    if (l2 <= 0) l2 = kmc::l2_bytes();
    const uint64_t cluster_bytes = (uint64_t)element_size * (uint64_t)(k * (d + 1));
    uint64_t copies = (uint64_t)(((double)(uint64_t)l2 * occ) / (double)cluster_bytes);
    const uint64_t global_size = (uint64_t)kmc::ceil_div<int64_t>(n, wgs) * (uint64_t)wgs;
    const uint64_t n_subgroups = global_size / 8;  // preferred_work_group_size_multiple
    if (n_subgroups < copies) copies = n_subgroups;
    *out = (int64_t)copies;
    return KMC_OK;
}

#define KMC_FIT_CREATE(SUF, T, I)                                                             \
    int kmc_fit_create_##SUF(const T *X, const T *w, T *c, I *lab, T *rc, int64_t n, int64_t d, \
                             int64_t k, double tol, int64_t max_iter, int form, kmc_stream_t s, \
                             kmc_fit_t *out) {                                                 \
        KMC_CHECK_ARG(out != nullptr, "null output pointer");                                  \
        FitBase *f = nullptr;                                                                  \
        KMC_TRY(fit_create<T, I>(X, w, c, lab, rc, n, d, k, tol, max_iter, form, S(s), &f));   \
        *out = new kmc_fit_s{f};                                                               \
        return KMC_OK;                                                                         \
    }
KMC_FIT_CREATE(f32_i32, float, int32_t)
KMC_FIT_CREATE(f32_i64, float, int64_t)
KMC_FIT_CREATE(f64_i32, double, int32_t)
KMC_FIT_CREATE(f64_i64, double, int64_t)

#define KMC_FIT_CREATE_ROWMAJOR(SUF, T, I)                                                    \
    int kmc_fit_create_rowmajor_##SUF(const T *X, const T *w, T *c, I *lab, T *rc, int64_t n,  \
                                      int64_t d, int64_t k, double tol, int64_t max_iter,      \
                                      int form, kmc_stream_t s, kmc_fit_t *out) {              \
        KMC_CHECK_ARG(out != nullptr, "null output pointer");                                  \
        FitBase *f = nullptr;                                                                  \
        KMC_TRY(fit_create<T, I>(X, w, c, lab, rc, n, d, k, tol, max_iter, form, S(s), &f, 1)); \
        *out = new kmc_fit_s{f};                                                               \
        return KMC_OK;                                                                         \
    }
KMC_FIT_CREATE_ROWMAJOR(f32_i32, float, int32_t)
KMC_FIT_CREATE_ROWMAJOR(f32_i64, float, int64_t)
KMC_FIT_CREATE_ROWMAJOR(f64_i32, double, int32_t)
KMC_FIT_CREATE_ROWMAJOR(f64_i64, double, int64_t)

#define KMC_FIT_CHECK(fit) KMC_CHECK_ARG((fit) != nullptr && (fit)->impl != nullptr, "null fit")

int kmc_fit_step(kmc_fit_t fit, int64_t n_iterations) {
    kmc::Range range("kmc.fit_step");
    KMC_FIT_CHECK(fit);
    KMC_CHECK_ARG(n_iterations >= 0, "n_iterations must be non-negative");
    for (int64_t t = 0; t < n_iterations; ++t) KMC_TRY(fit->impl->enqueue_iteration());
    return KMC_OK;
}
int kmc_fit_run(kmc_fit_t fit) {
    kmc::Range range("kmc.fit_run");
    KMC_FIT_CHECK(fit);
    return fit->impl->run(0);
}
int kmc_fit_status(kmc_fit_t fit, int64_t *n_iter, int *done, double *last_shift) {
    KMC_FIT_CHECK(fit);
    LoopState h{};
    KMC_TRY(fit->impl->read_state(h));
    if (n_iter) *n_iter = h.n_iter;
    if (done) *done = h.done;
    if (last_shift) *last_shift = h.last_shift;
    return KMC_OK;
}
int kmc_fit_finalize(kmc_fit_t fit, int64_t *n_iter, double *inertia) {
    kmc::Range range("kmc.fit_finalize");
    KMC_FIT_CHECK(fit);
    return fit->impl->finalize(n_iter, inertia);
}
int kmc_fit_set_profiling(kmc_fit_t fit, int enable) {
    KMC_FIT_CHECK(fit);
    fit->impl->profiling = enable != 0;
    return KMC_OK;
}
int kmc_fit_phase_time(kmc_fit_t fit, int phase, double *total_ms, int64_t *count) {
    KMC_FIT_CHECK(fit);
    KMC_CHECK_ARG(phase == 0, "unknown phase %d", phase);
    KMC_CHECK_ARG(total_ms != nullptr && count != nullptr, "null output pointer");
    return fit->impl->phase_time(total_ms, count);
}
int kmc_fit_rechecked(kmc_fit_t fit, int64_t *last, int64_t *total, int *device_error) {
    KMC_FIT_CHECK(fit);
    return fit->impl->counters(last, total, device_error);
}
int kmc_fit_set_wait_limit(kmc_fit_t fit, int64_t clocks, int stall_once) {
    KMC_FIT_CHECK(fit);
    return fit->impl->set_wait_limit((long long)clocks, stall_once);
}
int kmc_fit_set_tile_variant(kmc_fit_t fit, int variant) {
    KMC_FIT_CHECK(fit);
    return fit->impl->set_tile_variant(variant);
}
int kmc_fit_tile_variant(int64_t n_features, int64_t n_clusters, int dtype_bytes,
                         kmc_stream_t stream, int *variant_out) {
    KMC_CHECK_ARG(variant_out != nullptr, "null output");
    KMC_CHECK_ARG(dtype_bytes == 4 || dtype_bytes == 8, "dtype_bytes must be 4 or 8");
    KMC_CHECK_ARG(n_features >= 1 && n_clusters >= 1, "invalid sizes");
    if (dtype_bytes == 4) return kmc::tune_fit_variant<float>(n_features, n_clusters, S(stream),
                                                              variant_out);
    return kmc::tune_fit_variant<double>(n_features, n_clusters, S(stream), variant_out);
}
int kmc_fit_mixed_variant(kmc_fit_t fit, int *variant_out) {
    KMC_FIT_CHECK(fit);
    KMC_CHECK_ARG(variant_out != nullptr, "null output pointer");
    return kmc::mixed_variant_of(fit->impl, variant_out);
}
int kmc_debug_force_mixed_variant(int variant) { return kmc::force_mixed_variant(variant); }
int kmc_debug_pack_fixed(float value, int shift, int *packed_out) {
    KMC_CHECK_ARG(packed_out != nullptr, "null output pointer");
    KMC_CHECK_ARG(shift >= -74 && shift <= 100, "shift out of range");
    *packed_out = kmc::pack_fixed_term(value, shift);
    return KMC_OK;
}
int kmc_fit_launch_count(kmc_fit_t fit, int64_t *out) {
    KMC_FIT_CHECK(fit);
    KMC_CHECK_ARG(out != nullptr, "null output pointer");
    *out = fit->impl->launches;
    return KMC_OK;
}
int kmc_fit_destroy(kmc_fit_t fit) {
    if (fit == nullptr) return KMC_OK;
    delete fit->impl;
    delete fit;
    return KMC_OK;
}

int kmc_event_create(kmc_event_t *ev) {
    KMC_CHECK_ARG(ev != nullptr, "null event pointer");
    cudaEvent_t e;
    KMC_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    *ev = reinterpret_cast<kmc_event_t>(e);
    return KMC_OK;
}
int kmc_event_record(kmc_event_t ev, kmc_stream_t s) {
    KMC_CUDA_TRY(cudaEventRecord(reinterpret_cast<cudaEvent_t>(ev), S(s)));
    return KMC_OK;
}
int kmc_event_synchronize(kmc_event_t ev) {
    KMC_CUDA_TRY(cudaEventSynchronize(reinterpret_cast<cudaEvent_t>(ev)));
    return KMC_OK;
}
int kmc_event_query(kmc_event_t ev, int *done) {
    cudaError_t e = cudaEventQuery(reinterpret_cast<cudaEvent_t>(ev));
    if (e == cudaErrorNotReady) {
        (void)cudaGetLastError();
        *done = 0;
        return KMC_OK;
    }
    KMC_CUDA_TRY(e);
    *done = 1;
    return KMC_OK;
}
int kmc_stream_wait_event(kmc_stream_t s, kmc_event_t ev) {
    KMC_CUDA_TRY(cudaStreamWaitEvent(S(s), reinterpret_cast<cudaEvent_t>(ev), 0));
    return KMC_OK;
}
int kmc_event_destroy(kmc_event_t ev) {
    KMC_CUDA_TRY(cudaEventDestroy(reinterpret_cast<cudaEvent_t>(ev)));
    return KMC_OK;
}
int kmc_stream_synchronize(kmc_stream_t s) {
    KMC_CUDA_TRY(cudaStreamSynchronize(S(s)));
    return KMC_OK;
}
int kmc_pointer_device(const void *p, int *dev) {
    KMC_CHECK_ARG(dev != nullptr, "null output pointer");
    cudaPointerAttributes a;
    cudaError_t e = cudaPointerGetAttributes(&a, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        *dev = -1;
        return KMC_OK;
    }
    *dev = (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) ? a.device : -1;
    return KMC_OK;
}
int kmc_current_device(int *dev) {
    KMC_CUDA_TRY(cudaGetDevice(dev));
    return KMC_OK;
}

}  // extern "C"
