// One Lloyd fit: workspace, iteration body and device-resident loop state.
#pragma once

#include <memory>
#include <utility>
#include <vector>

#include "km_kernels.cuh"

namespace kmc {

template <typename T, typename I>
struct FitParams {
    const T *X = nullptr;         // (d, n) feature-major samples, or (n, d) if x_rowmajor
    const T *w = nullptr;         // (n,) sample weights
    T *centroids = nullptr;       // (d, k) current centroids; overwritten
    T *new_centroids = nullptr;   // (d, k) result buffer
    I *labels = nullptr;          // (n,)
    int64_t n = 0, d = 0, k = 0;
    double tol = 0.0;
    int64_t max_iter = 0;
    int verbose = 0;
    kmc_print_fn print_fn = nullptr;
    void *print_ctx = nullptr;
    cudaStream_t stream = nullptr;
    int x_rowmajor = 0;           // X given as (n, d) C-contiguous
};

struct FitBase {
    // Optional CUDA-event timing of the assignment + accumulation phase.
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> phase_events;
    int64_t launches = 0;

    virtual ~FitBase() {
        for (auto &e : phase_events) {
            cudaEventDestroy(e.first);
            cudaEventDestroy(e.second);
        }
    }
    int phase_time(double *total_ms, int64_t *count) {
        double tot = 0.0;
        for (auto &e : phase_events) {
            KMC_CUDA_TRY(cudaEventSynchronize(e.second));
            float ms = 0.f;
            KMC_CUDA_TRY(cudaEventElapsedTime(&ms, e.first, e.second));
            tot += ms;
        }
        *total_ms = tot;
        *count = (int64_t)phase_events.size();
        return KMC_OK;
    }
    // Enqueue iterations until the loop stops (batches of at most max_batch
    // iterations between host checks; <= 0 means unbounded growth).
    virtual int run(int64_t max_batch) = 0;
    // Enqueue exactly one iteration (no host synchronisation).
    virtual int enqueue_iteration() = 0;
    virtual int read_state(LoopState &out) = 0;
    // Device copy of the loop state (read by every kernel of an iteration).
    virtual const LoopState *device_state() const = 0;
    virtual int finalize(int64_t *n_iter_out, double *inertia_out) = 0;
    // The final pass without host synchronisation: the loop state and the
    // inertia total land in *state_out and *inertia_out (pinned host memory)
    // once the fit's stream reaches this point.
    virtual int finalize_enqueue(LoopState *state_out, double *inertia_out) = 0;
    // Limit (SM clocks) of the device-side waits of the tensor-core kernels;
    // with `stall`, the next assignment pass first waits on a barrier that
    // nothing completes, so that wait runs out (test of the timeout path).
    // The plain form has no device-side waits and ignores both.
    virtual int set_wait_limit(long long clocks, int stall) {
        (void)clocks;
        (void)stall;
        return KMC_OK;
    }
    // Centroid-tile variant of the plain form's kernels (the autotuner's
    // choice unless set here); the mixed forms ignore it.
    virtual int set_tile_variant(int v) {
        (void)v;
        return KMC_OK;
    }
    // Samples re-evaluated in exact arithmetic (mixed form): last pass and total.
    virtual int counters(int64_t *last, int64_t *total, int *device_error) {
        if (last) *last = 0;
        if (total) *total = 0;
        if (device_error) *device_error = 0;
        return KMC_OK;
    }
};

template <typename T, typename I>
struct PlainFit : FitBase {
    FitParams<T, I> prm;
    int64_t P = 1;  // private copies used internally
    Scratch ws;
    LoopState *state = nullptr;
    T *hn = nullptr, *sizes = nullptr, *shifts = nullptr, *sq_dist = nullptr;
    double *sums_cp = nullptr, *sizes_cp = nullptr;  // float64 accumulators
    T *threshold = nullptr;
    I *empty_list = nullptr, *n_empty = nullptr, *selected = nullptr, *counters = nullptr;
    int64_t *gate = nullptr;
    double *partials = nullptr, *dsum = nullptr;
    void *thr_scratch = nullptr, *sel_scratch = nullptr;
    int64_t issued = 0;
    int host_done = 0;
    int tile_variant = 0;  // autotuned centroid-tile width of the plain kernels
    Scratch xt;  // feature-major copy of a row-major X (forms that need one)

    int set_tile_variant(int v) override {
        KMC_CHECK_ARG(v >= 0 && v <= 2, "tile variant must be 0, 1 or 2");
        tile_variant = v;
        return KMC_OK;
    }

    int init(const FitParams<T, I> &p);
    int enqueue_iteration() override;
    int read_state(LoopState &out) override;
    int run(int64_t max_batch) override;
    int finalize(int64_t *n_iter_out, double *inertia_out) override;
    int finalize_enqueue(LoopState *state_out, double *inertia_out) override;
    const LoopState *device_state() const override { return state; }
    // Assignment + accumulation of one iteration (the fused Lloyd step);
    // reports the number of kernels it launched.
    virtual int step_assign_and_accumulate(const T *cur, int64_t *n_launches);
    // Labels against the final centroids (kmeans_lloyd_driver.hpp:372-386).
    virtual int final_assignment();
    // Private copies -> new centroid sums, sizes and the empty-cluster list
    // (kmeans_lloyd_driver.hpp:155-170).
    virtual int reduce_step(T *nxt);
    // Whether the step accumulates into the driver's float64 private copies
    // (the mixed forms keep their own sums).
    virtual bool uses_private_copies() const { return true; }
    // Whether the form reads a row-major X itself (else init makes a
    // feature-major copy).
    virtual bool reads_rowmajor() const { return false; }
    // The samples as the inertia and relocation kernels read them: element
    // (f, i) at x[f * fs + i * ss].
    virtual void x_view(const T **x, int64_t *fs, int64_t *ss) const {
        *x = prm.X;
        *fs = prm.n;
        *ss = 1;
    }
};

// Mixed tensor-core form (kernels_mixed.cu); float32 data only.
template <typename T, typename I>
int make_mixed_fit(const FitParams<T, I> &p, int form, std::unique_ptr<FitBase> *out);
// Whether the mixed form takes n_features = d and n_clusters = k.
bool mixed_fit_supported(int64_t d, int64_t k);
// Mixed-form variant (10 stages + fixed-point columns per update thread, 0 for
// float reductions): forced for every fit created afterwards (-1: the
// autotuner's choice again), and a session's choice (-1: not a mixed fit).
int force_mixed_variant(int code);
// Fits created on this thread while on use cached variant choices or the
// default and never time variants (the request server).
void mixed_tuning_lookup_only(bool on);
// The packed fixed-point term of v at scale 2^shift (host copy of the
// device's packing, for tests).
int pack_fixed_term(float v, int shift);
int mixed_variant_of(FitBase *fit, int *code);

}  // namespace kmc
