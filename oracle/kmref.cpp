// kmref -- CPU restatement of the kmeans_dpcpp Lloyd path, used ONLY as the
// correctness oracle (tests, smoke check) and as the timed CPU baseline of
// bench.py.  It is never part of the product path.
//
// Parity status: pinned.  The restatement is checked against every
// known-answer test of the reference's tests/test_kernels.py (fixtures in
// tests/golden/, generated by tests/golden/make_golden.py); the reference
// itself (SYCL + dpctl) cannot be compiled or run here.
//
// Arithmetic ("mirror" mode) follows the reference kernels line by line:
//   * sums over features run f = 0..d-1 sequentially with one fused
//     multiply-add per term: `acc += a * b` in src/device_functions.hpp:
//     121-137, src/util_kernels.hpp:69-73, 504-509, src/compute_inertia.hpp:
//     41-46 (compiled with -ffp-contract=off, the fma is written explicitly);
//   * pseudo-distance D_j = half_norm[j] - dot_j and the first j with the
//     smallest D_j wins (strict `<`, start (+inf, 0)),
//     src/device_functions.hpp:139-162;
//   * products that the reference rounds before accumulating (w * x in
//     lloyd_single_step.hpp:201, util_kernels.hpp:361) are rounded here too.
// Where the reference is nondeterministic or undefined, the oracle defines:
//   * centroid sums: accumulated in long double, rounded once to dataT (the
//     reference's atomic order is arbitrary);
//   * empty-cluster list: ascending cluster id (util_kernels.hpp:143 FIXME);
//   * relocation with n_empty >= 2: empty cluster r takes the r-th farthest
//     sample (larger sq_dist first, ties by lower index) -- the reference's
//     index arithmetic underflows there (util_kernels.hpp:353);
//   * distance matrix: the intended full (k, n) result (the reference swaps
//     its two loop bounds, compute_euclidean_distance.hpp:56-107);
//   * convergence / inertia totals: long double, rounded to dataT for the
//     tol comparison (kmeans_lloyd_driver.hpp:343-348) and the result.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <numeric>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <typename T>
T fma_t(T a, T b, T c) { return std::fma(a, b, c); }

// src/util_kernels.hpp:47-82
template <typename T>
void half_norm(const T *C, T *out, int64_t d, int64_t k) {
    for (int64_t j = 0; j < k; ++j) {
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) acc = fma_t(C[f * k + j], C[f * k + j], acc);
        out[j] = acc / T(2);
    }
}

// src/util_kernels.hpp:9-41
template <typename T>
void broadcast_divide(T *X, const T *y, int64_t rows, int64_t cols) {
    for (int64_t r = 0; r < rows; ++r)
        for (int64_t c = 0; c < cols; ++c) X[r * cols + c] = X[r * cols + c] / y[c];
}

// src/util_kernels.hpp:87-161 (list order: ascending cluster id)
template <typename T, typename I>
void reduce_centroids(const T *szc, const T *cc, T *osz, T *oc, I *list, I *n_empty, int64_t P,
                      int64_t d, int64_t k) {
    for (int64_t e = 0; e < d * k; ++e) {
        T s = T(0);
        for (int64_t p = 0; p < P; ++p) s += cc[p * d * k + e];
        oc[e] = s;
    }
    I cnt = *n_empty;
    for (int64_t j = 0; j < k; ++j) {
        T s = T(0);
        for (int64_t p = 0; p < P; ++p) s += szc[p * k + j];
        osz[j] = s;
        if (s == T(0)) list[cnt++] = (I)j;
    }
    *n_empty = cnt;
}

// src/util_kernels.hpp:163-206: the topk-th largest value (sorted[n - topk]).
template <typename T>
T threshold(const T *data, int64_t n, int64_t topk) {
    std::vector<T> v(data, data + n);
    int64_t pos = n - topk;
    std::nth_element(v.begin(), v.begin() + pos, v.end());
    return v[pos];
}

// src/util_kernels.hpp:211-297 with a defined order: the strictly greater
// samples are ranked (distance desc, index asc) and stored so that
// sel[gt_init + m - 1 - r] is the r-th farthest; equal samples go to
// sel[n - eq_init - t] in ascending index order, as many as still needed.
template <typename T, typename I>
void select_far(int64_t n_sel, const T *dist, T thr, I *sel, I *n_gt, I *n_eq, int64_t n) {
    std::vector<int64_t> gt, eq;
    for (int64_t i = 0; i < n; ++i) {
        if (dist[i] > thr) gt.push_back(i);
        else if (dist[i] == thr) eq.push_back(i);
    }
    const int64_t gt_init = (int64_t)*n_gt, eq_init = (int64_t)*n_eq;
    const int64_t m = (int64_t)gt.size();
    if (m < n_sel) {
        std::vector<int64_t> order = gt;
        std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
            if (dist[a] != dist[b]) return dist[a] > dist[b];
            return a < b;
        });
        for (int64_t r = 0; r < m; ++r) sel[gt_init + m - 1 - r] = (I)order[r];
    } else {
        for (int64_t t = 0; t < m; ++t) sel[gt_init + t] = (I)gt[t];
    }
    int64_t need = (m < n_sel) ? (n_sel - m) : 0;
    need = std::min<int64_t>(need, (int64_t)eq.size());
    for (int64_t t = 0; t < need; ++t) sel[n - (eq_init + t)] = (I)eq[t];
    *n_gt = (I)(gt_init + m);
    *n_eq = (I)(eq_init + need);
}

// src/util_kernels.hpp:302-390 (sequential over the empty list).
template <typename T, typename I>
void relocate_kernel(int64_t n_empty, const T *X, const T *w, const I *labels, const I *sel,
                     int64_t gt, const I *list, T *C, T *sizes, T *inertia, int64_t n, int64_t d,
                     int64_t k) {
    if (n_empty > n) n_empty = n;
    for (int64_t r = 0; r < n_empty; ++r) {
        int64_t pos = (r < gt) ? (gt - 1 - r) : (n - 1 - (r - gt));
        int64_t s = (int64_t)sel[pos];
        int64_t old = (int64_t)labels[s];
        int64_t cl = (int64_t)list[r];
        T wv = w[s];
        for (int64_t f = 0; f < d; ++f) {
            volatile T xw = X[f * n + s] * wv;
            C[f * k + old] -= xw;
            C[f * k + cl] = xw;
        }
        sizes[old] -= wv;
        sizes[cl] = wv;
        inertia[s] = T(0);
    }
}

// src/util_kernels.hpp:392-476
template <typename T, typename I>
void relocate(int64_t n_empty, const T *X, const T *w, const I *labels, const I *list,
              const T *sq, T *C, T *sizes, T *inertia, int64_t n, int64_t d, int64_t k) {
    int64_t topk = std::min<int64_t>(n_empty, n);
    T thr = threshold<T>(sq, n, topk);
    std::vector<I> sel(n, I(0));
    I ng = 0, ne = 1;
    select_far<T, I>(topk, sq, thr, sel.data(), &ng, &ne, n);
    relocate_kernel<T, I>(n_empty, X, w, labels, sel.data(), (int64_t)ng, list, C, sizes, inertia,
                          n, d, k);
}

// src/util_kernels.hpp:481-516
template <typename T>
void shifts(const T *a, const T *b, T *out, int64_t d, int64_t k) {
    for (int64_t j = 0; j < k; ++j) {
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) {
            T diff = a[f * k + j] - b[f * k + j];
            acc = fma_t(diff, diff, acc);
        }
        out[j] = acc;
    }
}

// src/compute_euclidean_distance.hpp:12-114 (intended result)
template <typename T>
void distances(const T *X, const T *C, T *out, int64_t n, int64_t d, int64_t k) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i)
        for (int64_t j = 0; j < k; ++j) {
            T acc = T(0);
            for (int64_t f = 0; f < d; ++f) {
                T diff = C[f * k + j] - X[f * n + i];
                acc = fma_t(diff, diff, acc);
            }
            out[j * n + i] = std::sqrt(acc);
        }
}

// Labels of a block of samples; dots accumulated f = 0..d-1 (fma), four
// samples share each centroid row so the inner loop vectorises over j.
template <typename T, typename I>
void assign_block(const T *X, const T *C, const T *hn, I *labels, int64_t i0, int64_t i1,
                  int64_t n, int64_t d, int64_t k, std::vector<T> &dots) {
    dots.assign(4 * k, T(0));
    for (int64_t i = i0; i < i1; i += 4) {
        const int64_t cnt = std::min<int64_t>(4, i1 - i);
        T *d0 = dots.data(), *d1 = d0 + k, *d2 = d1 + k, *d3 = d2 + k;
        std::fill(dots.begin(), dots.end(), T(0));
        for (int64_t f = 0; f < d; ++f) {
            const T *cr = C + f * k;
            const T x0 = X[f * n + i];
            const T x1 = cnt > 1 ? X[f * n + i + 1] : T(0);
            const T x2 = cnt > 2 ? X[f * n + i + 2] : T(0);
            const T x3 = cnt > 3 ? X[f * n + i + 3] : T(0);
            for (int64_t j = 0; j < k; ++j) {
                const T c = cr[j];
                d0[j] = fma_t(x0, c, d0[j]);
                d1[j] = fma_t(x1, c, d1[j]);
                d2[j] = fma_t(x2, c, d2[j]);
                d3[j] = fma_t(x3, c, d3[j]);
            }
        }
        for (int64_t q = 0; q < cnt; ++q) {
            const T *dq = dots.data() + q * k;
            T best = std::numeric_limits<T>::infinity();
            int64_t bi = 0;
            for (int64_t j = 0; j < k; ++j) {
                T v = hn[j] - dq[j];
                if (v < best) {
                    best = v;
                    bi = j;
                }
            }
            labels[i + q] = (I)bi;
        }
    }
}

// src/assignment.hpp:11-146
template <typename T, typename I>
void assignment(const T *X, const T *C, const T *hn, I *labels, int64_t n, int64_t d,
                int64_t k) {
    const int64_t B = 256;
#pragma omp parallel
    {
        std::vector<T> dots;
#pragma omp for schedule(dynamic, 1)
        for (int64_t i0 = 0; i0 < n; i0 += B)
            assign_block<T, I>(X, C, hn, labels, i0, std::min(n, i0 + B), n, d, k, dots);
    }
}

// src/compute_inertia.hpp:11-99 (w == nullptr: unit weights)
template <typename T, typename I>
void inertia(const T *X, const T *w, const T *C, const I *labels, T *out, int64_t n, int64_t d,
             int64_t k) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = (int64_t)labels[i];
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) {
            T diff = X[f * n + i] - C[f * k + c];
            acc = fma_t(diff, diff, acc);
        }
        out[i] = w ? acc * w[i] : acc;
    }
}

template <typename T>
long double sum_ld(const T *x, int64_t n) {
    long double s = 0.0L;
    for (int64_t i = 0; i < n; ++i) s += (long double)x[i];
    return s;
}

// Centroid sums and sizes of one labelling (long double accumulation).
template <typename T, typename I>
void accumulate(const T *X, const T *w, const I *labels, T *sums, T *sizes, int64_t n, int64_t d,
                int64_t k) {
    std::vector<long double> acc((size_t)(d * k), 0.0L), sz((size_t)k, 0.0L);
    for (int64_t i = 0; i < n; ++i) {
        int64_t c = (int64_t)labels[i];
        sz[c] += (long double)w[i];
    }
#pragma omp parallel for schedule(static)
    for (int64_t f = 0; f < d; ++f) {
        long double *a = acc.data() + f * k;
        for (int64_t i = 0; i < n; ++i) {
            volatile T v = X[f * n + i] * w[i];
            a[labels[i]] += (long double)v;
        }
    }
    for (int64_t e = 0; e < d * k; ++e) sums[e] = (T)acc[e];
    for (int64_t j = 0; j < k; ++j) sizes[j] = (T)sz[j];
}

// One pass of the loop body of src/kmeans_lloyd_driver.hpp:86-353 from the
// centroids `cur`: labels against cur (fused step, :86-143), sums, sizes and
// the empty list (:155-170), relocation when a cluster is empty (:217-312),
// division and the centroid shifts (:317-341) into `newc`.  Returns the
// float64 total of the shifts cast to T (:343-348); *relocated is set when the
// pass relocated.
template <typename T, typename I>
T iteration(const T *X, const T *w, const T *cur, I *labels, T *newc, int64_t n, int64_t d,
            int64_t k, bool *relocated) {
    std::vector<T> hn(k), sizes(k), sh(k);
    std::vector<I> list(k);
    half_norm<T>(cur, hn.data(), d, k);
    assignment<T, I>(X, cur, hn.data(), labels, n, d, k);
    accumulate<T, I>(X, w, labels, newc, sizes.data(), n, d, k);
    I n_empty = 0;
    for (int64_t j = 0; j < k; ++j)
        if (sizes[j] == T(0)) list[n_empty++] = (I)j;
    *relocated = n_empty > 0;
    if (n_empty > 0) {
        std::vector<T> sq(n);
        inertia<T, I>(X, nullptr, cur, labels, sq.data(), n, d, k);
        relocate<T, I>((int64_t)n_empty, X, w, labels, list.data(), sq.data(), newc, sizes.data(),
                       sq.data(), n, d, k);
    }
    for (int64_t j = 0; j < k; ++j) {
        T acc = T(0);
        for (int64_t f = 0; f < d; ++f) {
            T c = newc[f * k + j] / sizes[j];
            newc[f * k + j] = c;
            T diff = cur[f * k + j] - c;
            acc = fma_t(diff, diff, acc);
        }
        sh[j] = acc;
    }
    long double tot = 0.0L;
    for (int64_t j = 0; j < k; ++j) tot += (long double)sh[j];
    return (T)(double)tot;
}

// src/kmeans_lloyd_driver.hpp:21-431
template <typename T, typename I>
int64_t driver(const T *X, const T *w, T *init_c, I *labels, T *res_c, int64_t n, int64_t d,
               int64_t k, double tol, int64_t max_iter, double *inertia_out,
               int64_t *relocations_out) {
    std::vector<T> hn(k), sq(n), newc(d * k);
    const T tol_t = (T)tol;
    T shift_t = std::numeric_limits<T>::infinity();
    int64_t it = 0, relocations = 0;
    T *cur = init_c;
    while (it < max_iter && shift_t > tol_t) {
        bool rel = false;
        shift_t = iteration<T, I>(X, w, cur, labels, newc.data(), n, d, k, &rel);
        if (rel) ++relocations;
        std::memcpy(cur, newc.data(), sizeof(T) * d * k);
        ++it;
    }
    half_norm<T>(cur, hn.data(), d, k);
    assignment<T, I>(X, cur, hn.data(), labels, n, d, k);
    inertia<T, I>(X, w, cur, labels, sq.data(), n, d, k);
    *inertia_out = (double)sum_ld<T>(sq.data(), n);
    if (res_c != cur) std::memcpy(res_c, cur, sizeof(T) * d * k);
    if (relocations_out) *relocations_out = relocations;
    return it;
}

// k-means++ seeding as the engine's kmc_kmeans_plusplus_* defines it (not a
// reference function: the reference takes initial centroids as given).  Draw
// u_t = SplitMix64(seed ^ SplitMix64(t)) >> 11 scaled to [0, 1); values v_i =
// w_i (t = 0) or w_i * min_j ||x_i - c_j||^2 (float64 products of the dataT
// distance); float64 sums run sequentially inside blocks of 4096 samples and
// then over the blocks; the pick is the first i whose running sum exceeds
// u_t * total (or the block's last positive sample if rounding overshoots).
uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

template <typename T>
void kmeanspp(const T *X, const T *w, int64_t n, int64_t d, int64_t k, uint64_t seed, T *C,
              int32_t *chosen) {
    const int64_t B = 4096, nb = (n + B - 1) / B;
    std::vector<T> md(n, T(0));
    std::vector<double> part(nb);
    for (int64_t t = 0; t < k; ++t) {
        const bool use_d2 = t > 0;
        auto val = [&](int64_t i) {
            const double wi = w ? (double)w[i] : 1.0;
            return use_d2 ? wi * (double)md[i] : wi;
        };
        for (int64_t b = 0; b < nb; ++b) {
            double s = 0.0;
            for (int64_t i = b * B; i < std::min(n, (b + 1) * B); ++i) s += val(i);
            part[b] = s;
        }
        double total = 0.0;
        for (int64_t b = 0; b < nb; ++b) total += part[b];
        int64_t sel = -1;
        if (total > 0.0) {
            const double u = (double)(splitmix64(seed ^ splitmix64((uint64_t)t)) >> 11) * 0x1p-53;
            const double target = u * total;
            double run = 0.0;
            int64_t b = 0;
            for (; b < nb; ++b) {
                if (run + part[b] > target) break;
                run += part[b];
            }
            if (b == nb) b = nb - 1;
            for (int64_t i = b * B; i < std::min(n, (b + 1) * B); ++i) {
                const double v = val(i);
                if (v > 0.0) sel = i;
                run += v;
                if (run > target && v > 0.0) break;
            }
        }
        if (sel < 0) sel = t > 0 ? ((int64_t)chosen[t - 1] + 1) % n : 0;
        chosen[t] = (int32_t)sel;
        for (int64_t f = 0; f < d; ++f) C[f * k + t] = X[f * n + sel];
        if (t + 1 < k) {
#pragma omp parallel for schedule(static)
            for (int64_t i = 0; i < n; ++i) {
                T acc = T(0);
                for (int64_t f = 0; f < d; ++f) {
                    const T diff = X[f * n + i] - X[f * n + sel];
                    acc = fma_t(diff, diff, acc);
                }
                md[i] = (t == 0 || acc < md[i]) ? acc : md[i];
            }
        }
    }
}

}  // namespace

extern "C" {

int kmref_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void kmref_set_num_threads(int t) {
#ifdef _OPENMP
    if (t > 0) omp_set_num_threads(t);
#else
    (void)t;
#endif
}

#define KMREF_T(SUF, T)                                                                       \
    void kmref_half_norm_##SUF(const T *C, T *o, int64_t d, int64_t k) {                     \
        half_norm<T>(C, o, d, k);                                                             \
    }                                                                                         \
    void kmref_broadcast_divide_##SUF(T *X, const T *y, int64_t r, int64_t c) {               \
        broadcast_divide<T>(X, y, r, c);                                                      \
    }                                                                                         \
    T kmref_threshold_##SUF(const T *x, int64_t n, int64_t topk) {                            \
        return threshold<T>(x, n, topk);                                                      \
    }                                                                                         \
    void kmref_shifts_##SUF(const T *a, const T *b, T *o, int64_t d, int64_t k) {             \
        shifts<T>(a, b, o, d, k);                                                             \
    }                                                                                         \
    void kmref_distances_##SUF(const T *X, const T *C, T *o, int64_t n, int64_t d, int64_t k) { \
        distances<T>(X, C, o, n, d, k);                                                       \
    }                                                                                         \
    double kmref_sum_##SUF(const T *x, int64_t n) { return (double)sum_ld<T>(x, n); }          \
    void kmref_reduce_centroids_##SUF(const T *szc, const T *cc, T *osz, T *oc, int64_t *l,    \
                                      int64_t *ne, int64_t P, int64_t d, int64_t k) {          \
        reduce_centroids<T, int64_t>(szc, cc, osz, oc, l, ne, P, d, k);                        \
    }                                                                                         \
    void kmref_select_##SUF(int64_t m, const T *dist, T thr, int64_t *sel, int64_t *ng,        \
                            int64_t *nq, int64_t n) {                                         \
        select_far<T, int64_t>(m, dist, thr, sel, ng, nq, n);                                 \
    }                                                                                         \
    void kmref_relocate_##SUF(int64_t ne, const T *X, const T *w, const int64_t *lab,          \
                              const int64_t *lst, const T *sq, T *C, T *sz, T *inr, int64_t n,  \
                              int64_t d, int64_t k) {                                         \
        relocate<T, int64_t>(ne, X, w, lab, lst, sq, C, sz, inr, n, d, k);                     \
    }                                                                                         \
    void kmref_assignment_##SUF(const T *X, const T *C, const T *hn, int64_t *lab, int64_t n,  \
                                int64_t d, int64_t k) {                                       \
        assignment<T, int64_t>(X, C, hn, lab, n, d, k);                                       \
    }                                                                                         \
    void kmref_inertia_##SUF(const T *X, const T *w, const T *C, const int64_t *lab, T *o,     \
                             int64_t n, int64_t d, int64_t k) {                               \
        inertia<T, int64_t>(X, w, C, lab, o, n, d, k);                                        \
    }                                                                                         \
    void kmref_fused_step_##SUF(const T *X, const T *w, const T *C, const T *hn, int64_t *lab, \
                                T *sums, T *sizes, int64_t n, int64_t d, int64_t k) {          \
        assignment<T, int64_t>(X, C, hn, lab, n, d, k);                                       \
        accumulate<T, int64_t>(X, w, lab, sums, sizes, n, d, k);                               \
    }                                                                                         \
    double kmref_iteration_##SUF(const T *X, const T *w, const T *cur, int64_t *lab, T *nxt,   \
                                 int64_t n, int64_t d, int64_t k, int64_t *relocated) {        \
        bool rel = false;                                                                     \
        const T sh = iteration<T, int64_t>(X, w, cur, lab, nxt, n, d, k, &rel);               \
        *relocated = rel ? 1 : 0;                                                             \
        return (double)sh;                                                                    \
    }                                                                                         \
    int64_t kmref_driver_##SUF(const T *X, const T *w, T *ic, int64_t *lab, T *rc, int64_t n,  \
                               int64_t d, int64_t k, double tol, int64_t max_iter,            \
                               double *inertia, int64_t *relocations) {                       \
        return driver<T, int64_t>(X, w, ic, lab, rc, n, d, k, tol, max_iter, inertia,          \
                                  relocations);                                               \
    }

KMREF_T(f32, float)
KMREF_T(f64, double)

void kmref_kmeanspp_f32(const float *X, const float *w, int64_t n, int64_t d, int64_t k,
                        uint64_t seed, float *C, int32_t *chosen) {
    kmeanspp<float>(X, w, n, d, k, seed, C, chosen);
}
void kmref_kmeanspp_f64(const double *X, const double *w, int64_t n, int64_t d, int64_t k,
                        uint64_t seed, double *C, int32_t *chosen) {
    kmeanspp<double>(X, w, n, d, k, seed, C, chosen);
}

}  // extern "C"
