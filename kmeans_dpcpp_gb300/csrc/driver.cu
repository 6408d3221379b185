// Lloyd driver: the host loop of driver_lloyd (src/kmeans_lloyd_driver.hpp:
// 21-431), re-designed so that the GPU decides when to stop.
//
// Reference loop, per iteration (kmeans_lloyd_driver.hpp:83-354):
//   half norms -> zero private copies -> fused step -> reduce copies (sums,
//   sizes, empty list) -> [verbose inertia print] -> host reads n_empty ->
//   [relocate empty clusters] -> divide -> shifts -> host reads shift sum ->
//   swap -> ++n_iter;   while (n_iter < max_iter && shift_sum > tol).
//
// Here every kernel of an iteration is guarded by a device-resident loop
// state: the loop-control kernel sets `done` once the reference's condition
// fails, after which the remaining enqueued kernels return immediately.  The
// relocation kernels are gated by the device value of n_empty.  The host
// therefore enqueues iterations in batches and reads the state once per batch
// instead of twice per iteration.  Centroid buffers do not ping-pong: new
// centroids are copied back into the current buffer after the shift test, so
// one iteration body works for every iteration (and can be captured once
// into a CUDA graph).  The convergence total and the final inertia are summed
// in float64.
#include <algorithm>
#include <cstdarg>
#include <memory>
#include <vector>

#include "km_kernels.cuh"
#include "km_fit.cuh"

namespace kmc {

template <typename T, typename I>
int PlainFit<T, I>::init(const FitParams<T, I> &p) {
    prm = p;
    const int64_t n = p.n, d = p.d, k = p.k;
    KMC_CHECK_ARG(n >= 0 && d >= 0 && k >= 0, "negative array dimension");
    // Small sums get one float64 copy per CTA of the fused step (two CTAs
    // per SM), filled with fire-and-forget global reductions; shared-memory
    // float64 atomics would be compare-and-swap loops on the critical path.
    // float64 samples get a copy per CTA up to 256 MiB of copies: each CTA
    // then sums its samples in a fixed order (bit-reproducible centroids).
    if (!uses_private_copies()) {
        P = 1;
    } else if (sizeof(T) == 8) {
        const int64_t per_copy = 8 * (d + 1) * std::max<int64_t>(k, 1);
        P = std::max<int64_t>(1, std::min<int64_t>(2 * (int64_t)num_sms(),
                                                   (int64_t(256) << 20) / per_copy));
    } else {
        P = ((d + 1) * k <= 8192) ? 2 * (int64_t)num_sms() : 1;
    }
    size_t off = 0;
    auto take = [&](size_t bytes) {
        size_t o = off;
        off += align256(bytes);
        return o;
    };
    const size_t o_state = take(sizeof(LoopState));
    const size_t o_hn = take(sizeof(T) * k);
    const size_t o_sizes = take(sizeof(T) * k);
    const size_t o_shifts = take(sizeof(T) * k);
    const size_t o_sq = take(sizeof(T) * n);
    const size_t o_scp = take(sizeof(double) * P * d * k);
    const size_t o_zcp = take(sizeof(double) * P * k);
    const size_t o_list = take(sizeof(I) * (k + 1));
    const size_t o_sel = take(sizeof(I) * (n + 2));
    const size_t o_gate = take(sizeof(int64_t));
    const size_t o_thr = take(sizeof(T));
    const size_t o_part = take(sizeof(double) * sum_partials_size());
    const size_t o_dsum = take(sizeof(double) * 2);
    const size_t o_tsc = take(threshold_scratch_bytes());
    const size_t o_ssc = take(select_scratch_bytes(k));
    KMC_TRY(ws.alloc(off, p.stream));
    // the plain kernels' centroid-tile width for this (d, k, dtype)
    if (uses_private_copies()) KMC_TRY(tune_fit_variant<T>(d, k, p.stream, &tile_variant));
    if (p.x_rowmajor && !reads_rowmajor()) {
        KMC_TRY(xt.alloc(sizeof(T) * (size_t)n * (size_t)d, p.stream));
        if (sizeof(T) == 4)
            KMC_TRY(kmc_transpose_f32(reinterpret_cast<const float *>(p.X), xt.as<float>(), n, d,
                                      reinterpret_cast<kmc_stream_t>(p.stream)));
        else
            KMC_TRY(kmc_transpose_f64(reinterpret_cast<const double *>(p.X), xt.as<double>(), n,
                                      d, reinterpret_cast<kmc_stream_t>(p.stream)));
        prm.X = xt.as<T>();
        prm.x_rowmajor = 0;
    }
    char *b = ws.as<char>();
    state = reinterpret_cast<LoopState *>(b + o_state);
    hn = reinterpret_cast<T *>(b + o_hn);
    sizes = reinterpret_cast<T *>(b + o_sizes);
    shifts = reinterpret_cast<T *>(b + o_shifts);
    sq_dist = reinterpret_cast<T *>(b + o_sq);
    sums_cp = reinterpret_cast<double *>(b + o_scp);
    sizes_cp = reinterpret_cast<double *>(b + o_zcp);
    empty_list = reinterpret_cast<I *>(b + o_list);
    n_empty = empty_list + k;
    selected = reinterpret_cast<I *>(b + o_sel);
    counters = selected + n;
    gate = reinterpret_cast<int64_t *>(b + o_gate);
    threshold = reinterpret_cast<T *>(b + o_thr);
    partials = reinterpret_cast<double *>(b + o_part);
    dsum = reinterpret_cast<double *>(b + o_dsum);
    thr_scratch = b + o_tsc;
    sel_scratch = b + o_ssc;

    LoopState h{};
    h.done = 0;
    h.n_iter = 0;
    h.max_iter = p.max_iter;
    const T tol_t = (T)p.tol;
    h.tol = (double)tol_t;
    // while (n_iter < max_iter && shift_sum > tol) with shift_sum = +inf
    // initially (kmeans_lloyd_driver.hpp:78, 83).
    if (!(0 < p.max_iter && pos_inf<T>() > tol_t)) h.done = 1;
    host_done = h.done;
    KMC_CUDA_TRY(cudaMemcpyAsync(state, &h, sizeof(h), cudaMemcpyHostToDevice, p.stream));
    return KMC_OK;
}

template <typename T, typename I>
int PlainFit<T, I>::enqueue_iteration() {
    const FitParams<T, I> &p = prm;
    const int64_t n = p.n, d = p.d, k = p.k;
    cudaStream_t s = p.stream;
    T *cur = p.centroids;       // this_centroids_t
    T *nxt = p.new_centroids;   // new_centroids_t
    const int64_t thr_launches = 1 + 2 * (sizeof(T) == 4 ? 4 : 8);
    const T *xv = nullptr;
    int64_t xfs = 0, xss = 0;
    x_view(&xv, &xfs, &xss);
    // kmeans_lloyd_driver.hpp:86-111
    KMC_TRY(launch_half_norm<T>(cur, hn, d, k, s, state));
    const bool copies = uses_private_copies();
    if (copies) {
        KMC_TRY(launch_fill<double>(sums_cp, 0.0, P * d * k, s, state));
        KMC_TRY(launch_fill<double>(sizes_cp, 0.0, P * k, s, state));
    }
    KMC_TRY(launch_fill<I>(n_empty, I(0), 1, s, state));
    // kmeans_lloyd_driver.hpp:124-143
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (profiling) {
        KMC_CUDA_TRY(cudaEventCreate(&e0));
        KMC_CUDA_TRY(cudaEventCreate(&e1));
        KMC_CUDA_TRY(cudaEventRecord(e0, s));
    }
    int64_t step_launches = 0;
    KMC_TRY(step_assign_and_accumulate(cur, &step_launches));
    if (profiling) {
        KMC_CUDA_TRY(cudaEventRecord(e1, s));
        phase_events.emplace_back(e0, e1);
    }
    // kmeans_lloyd_driver.hpp:155-170
    KMC_TRY(reduce_step(nxt));
    int64_t verbose_launches = 0;
    if (p.verbose) {
        // kmeans_lloyd_driver.hpp:179-197: inertia of the *undivided* sums.
        KMC_TRY(launch_inertia<T, I>(xv, p.w, nxt, p.labels, sq_dist, n, d, k, s, state, nullptr,
                                     xfs, xss));
        KMC_TRY(launch_sum_f64<T>(sq_dist, n, partials, dsum, s, state));
        verbose_launches = 3;
    }
    // kmeans_lloyd_driver.hpp:217-312, gated on the device value of n_empty.
    KMC_TRY(launch_gate_from_count<I>(n_empty, gate, s, state));
    KMC_TRY(launch_inertia<T, I>(xv, nullptr, cur, p.labels, sq_dist, n, d, k, s, state, gate,
                                 xfs, xss));
    KMC_TRY(launch_threshold<T>(sq_dist, n, gate, 0, threshold, thr_scratch, s, state));
    KMC_TRY(launch_fill<I>(counters, I(0), 1, s, state));
    KMC_TRY(launch_fill<I>(counters + 1, I(1), 1, s, state));
    KMC_TRY(launch_select<T, I>(gate, 0, sq_dist, threshold, selected, counters, counters + 1, n,
                                sel_scratch, k, s, state));
    KMC_TRY(launch_relocate<T, I>(gate, 0, xv, p.w, p.labels, selected, counters, empty_list,
                                  nxt, sizes, sq_dist, n, d, k, s, state, xfs, xss));
    // kmeans_lloyd_driver.hpp:317-353
    KMC_TRY(launch_divide_and_shift<T>(cur, nxt, sizes, shifts, d, k, s, state));
    KMC_TRY(launch_loop_control<T>(shifts, k, state, s));
    KMC_CUDA_TRY(cudaMemcpyAsync(cur, nxt, sizeof(T) * d * k, cudaMemcpyDeviceToDevice, s));
    // 4 (norm, fills) + step + 2 (reduce) + gate + inertia + threshold + 2 fills
    // + 4 (select) + relocate + divide/shift + control
    launches += (copies ? 4 : 2) + step_launches + 2 + verbose_launches + 1 + 1 + thr_launches + 2 +
                select_launches(k) + 1 + 1 + 1;
    ++issued;
    return KMC_OK;
}

template <typename T, typename I>
int PlainFit<T, I>::step_assign_and_accumulate(const T *cur, int64_t *n_launches) {
    const FitParams<T, I> &p = prm;
    *n_launches = 1;
    return launch_fused_step<T, I, double>(p.X, p.w, cur, hn, p.labels, sums_cp, sizes_cp, p.n,
                                           p.d, p.k, P, p.stream, state, tile_variant);
}

template <typename T, typename I>
int PlainFit<T, I>::read_state(LoopState &out) {
    KMC_CUDA_TRY(cudaMemcpyAsync(&out, state, sizeof(LoopState), cudaMemcpyDeviceToHost,
                                 prm.stream));
    KMC_CUDA_TRY(cudaStreamSynchronize(prm.stream));
    host_done = out.done;
    return check_device_error(out);
}

template <typename T, typename I>
int PlainFit<T, I>::run(int64_t max_batch) {
    const FitParams<T, I> &p = prm;
    LoopState h{};
    KMC_TRY(read_state(h));
    int64_t batch = 1;
    while (!h.done && issued < p.max_iter) {
        int64_t m = p.verbose ? 1 : std::min<int64_t>(batch, p.max_iter - issued);
        if (max_batch > 0) m = std::min<int64_t>(m, max_batch);
        for (int64_t t = 0; t < m; ++t) KMC_TRY(enqueue_iteration());
        KMC_TRY(read_state(h));
        if (p.verbose && p.print_fn != nullptr && h.n_iter > 0) {
            double tot = 0.0;
            KMC_CUDA_TRY(cudaMemcpy(&tot, dsum, sizeof(double), cudaMemcpyDeviceToHost));
            char line[128];
            // kmeans_lloyd_driver.hpp:199-204
            snprintf(line, sizeof(line), "Iteration: %lld Inertia: %.9g", (long long)(h.n_iter - 1),
                     (double)(T)tot);
            p.print_fn(line, p.print_ctx);
        }
        if (batch < 64) batch *= 2;
    }
    return KMC_OK;
}

template <typename T, typename I>
int PlainFit<T, I>::finalize_enqueue(LoopState *state_out, double *inertia_out) {
    const FitParams<T, I> &p = prm;
    const int64_t n = p.n, d = p.d, k = p.k;
    cudaStream_t s = p.stream;
    // kmeans_lloyd_driver.hpp:360-418: final assignment and inertia against
    // the final centroids.
    KMC_TRY(launch_half_norm<T>(p.centroids, hn, d, k, s));
    KMC_TRY(final_assignment());
    const T *xv = nullptr;
    int64_t xfs = 0, xss = 0;
    x_view(&xv, &xfs, &xss);
    KMC_TRY(launch_inertia<T, I>(xv, p.w, p.centroids, p.labels, sq_dist, n, d, k, s, nullptr,
                                 nullptr, xfs, xss));
    KMC_TRY(launch_sum_f64<T>(sq_dist, n, partials, dsum, s));
    launches += 5;
    if (p.new_centroids != p.centroids && d * k > 0)
        KMC_CUDA_TRY(cudaMemcpyAsync(p.new_centroids, p.centroids, sizeof(T) * d * k,
                                     cudaMemcpyDeviceToDevice, s));
    KMC_CUDA_TRY(cudaMemcpyAsync(inertia_out, dsum, sizeof(double), cudaMemcpyDeviceToHost, s));
    KMC_CUDA_TRY(cudaMemcpyAsync(state_out, state, sizeof(LoopState), cudaMemcpyDeviceToHost, s));
    return KMC_OK;
}

template <typename T, typename I>
int PlainFit<T, I>::finalize(int64_t *n_iter_out, double *inertia_out) {
    LoopState h{};
    double tot = 0.0;
    KMC_TRY(finalize_enqueue(&h, &tot));
    KMC_CUDA_TRY(cudaStreamSynchronize(prm.stream));
    host_done = h.done;
    KMC_TRY(check_device_error(h));
    if (n_iter_out) *n_iter_out = h.n_iter;
    if (inertia_out) *inertia_out = tot;
    return KMC_OK;
}

template <typename T, typename I>
int PlainFit<T, I>::reduce_step(T *nxt) {
    const FitParams<T, I> &p = prm;
    return launch_reduce_centroids<T, I, double>(sizes_cp, sums_cp, sizes, nxt, empty_list,
                                                 n_empty, P, p.d, p.k, p.stream, state);
}

template <typename T, typename I>
int PlainFit<T, I>::final_assignment() {
    const FitParams<T, I> &p = prm;
    return launch_assignment<T, I>(p.X, p.centroids, hn, p.labels, p.n, p.d, p.k, p.stream,
                                   nullptr, tile_variant);
}

template struct PlainFit<float, int32_t>;
template struct PlainFit<float, int64_t>;
template struct PlainFit<double, int32_t>;
template struct PlainFit<double, int64_t>;

}  // namespace kmc
