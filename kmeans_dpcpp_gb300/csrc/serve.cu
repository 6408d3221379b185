// Host side of the batched Lloyd engine (km_batch.cuh) and the serving loop,
// with their extern "C" entry points (include/kmeans_gb300.h).
//
// BatchEngine::step() advances every running instance by one iteration:
//   graph A   batch_prep -> batch_assign (one launch per centroid-window
//             variant in use, all fed from the device work queue) ->
//             batch_reduce
//   host      reads the empty-cluster counts of the fitting instances; those
//             with empty clusters run the single-fit relocation chain
//             (kmeans_lloyd_driver.hpp:217-312) on their own buffers
//   graph B   batch_update (divide, shifts, stop rule, copy-back)
//   host      reads the stop flags; finished fits get the driver's final pass
//             (half norms, assignment, weighted inertia, float64 total,
//             kmeans_lloyd_driver.hpp:360-418); predictions finish after
//             their assignment
// The two graphs are captured once per set of running instances and replayed
// until an instance joins or leaves.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <deque>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#include "km_batch.cuh"
#include "kmeans_gb300.h"

namespace kmc {

namespace {

constexpr int kItemTiles = 8;  // 128-sample tiles per work item

// Work items of one instance: runs of at most kItemTiles 128-sample tiles,
// appended to the list of its (kind, tile variant); kind 1 = distance
// (transform) instances, 0 = the rest.  The persistent assign kernels take
// items from a device counter (atomicAdd), so every tile is handled by one
// CTA exactly once.
void append_items(int q, int64_t n, int mode, int variant,
                  std::vector<BItem> (&items)[2][kBatchVariants]) {
    const int64_t tiles = ceil_div<int64_t>(n, kBatchTileM);
    const int kind = (mode == B_TRANSFORM) ? 1 : 0;
    for (int64_t t = 0; t < tiles; t += kItemTiles)
        items[kind][variant].push_back(
            BItem{q, (int)std::min<int64_t>(kItemTiles, tiles - t), (long long)t});
}

// Engine-owned device memory of one instance.
struct SlotMem {
    Scratch mem;
    float *Cn = nullptr, *hn = nullptr, *sizes = nullptr, *sq_dist = nullptr, *thr = nullptr;
    double *sums = nullptr, *partials = nullptr, *dsum = nullptr;
    int32_t *empty_list = nullptr, *selected = nullptr;
    void *thr_scratch = nullptr, *sel_scratch = nullptr;
};

size_t slot_bytes(int mode, int64_t n, int64_t d, int64_t k) {
    size_t b = align256(sizeof(float) * d * k) + 2 * align256(sizeof(float) * k);
    if (mode == B_FIT) {
        b += align256(sizeof(double) * (d * k + k) * batch_sum_copies(d, k)) +
             align256(sizeof(int32_t) * (k + 1)) +
             align256(sizeof(float) * n) + align256(sizeof(int32_t) * (n + 2)) +
             align256(sizeof(float)) + align256(threshold_scratch_bytes()) +
             align256(select_scratch_bytes(k)) + align256(sizeof(double) * sum_partials_size()) +
             align256(sizeof(double));
    }
    return b;
}

int alloc_slot(SlotMem &m, int mode, int64_t n, int64_t d, int64_t k, cudaStream_t s) {
    KMC_TRY(m.mem.alloc(slot_bytes(mode, n, d, k), s));
    char *b = m.mem.as<char>();
    size_t off = 0;
    auto take = [&](size_t bytes) {
        char *p = b + off;
        off += align256(bytes);
        return p;
    };
    m.Cn = reinterpret_cast<float *>(take(sizeof(float) * d * k));
    m.hn = reinterpret_cast<float *>(take(sizeof(float) * k));
    m.sizes = reinterpret_cast<float *>(take(sizeof(float) * k));
    if (mode == B_FIT) {
        m.sums = reinterpret_cast<double *>(take(sizeof(double) * (d * k + k) * batch_sum_copies(d, k)));
        m.empty_list = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * (k + 1)));
        m.sq_dist = reinterpret_cast<float *>(take(sizeof(float) * n));
        m.selected = reinterpret_cast<int32_t *>(take(sizeof(int32_t) * (n + 2)));
        m.thr = reinterpret_cast<float *>(take(sizeof(float)));
        m.thr_scratch = take(threshold_scratch_bytes());
        m.sel_scratch = take(select_scratch_bytes(k));
        m.partials = reinterpret_cast<double *>(take(sizeof(double) * sum_partials_size()));
        m.dsum = reinterpret_cast<double *>(take(sizeof(double)));
    }
    return KMC_OK;
}

struct GraphExec {
    cudaGraphExec_t exec = nullptr;
    ~GraphExec() { reset(); }
    void reset() {
        if (exec) cudaGraphExecDestroy(exec);
        exec = nullptr;
    }
};

}  // namespace

struct BatchEngine {
    enum SlotState { FREE = 0, RUNNING = 1, FINISHED = 2 };
    // The engine's work runs on its own stream (graphs cannot capture the
    // legacy default stream); events order it after the caller's stream when
    // instances are added and the caller's stream after each step.
    cudaStream_t user = nullptr;
    cudaStream_t s = nullptr;
    cudaEvent_t ev_in = nullptr, ev_out = nullptr;
    // the assign variants run as parallel branches of graph A, so each one's
    // tail overlaps the others instead of leaving SMs idle
    cudaStream_t side[kBatchVariants] = {nullptr, nullptr, nullptr};
    cudaEvent_t ev_fork = nullptr, ev_join[kBatchVariants] = {nullptr, nullptr, nullptr};
    int64_t cap = 0;
    Scratch dev;                    // table, lists, work queue, counters, status
    BInst *tab_d = nullptr;
    int *all_d = nullptr, *fit_d = nullptr, *counters_d = nullptr;
    int *nempty_d = nullptr, *done_d = nullptr;
    BItem *items_d = nullptr;
    int64_t items_cap = 0;
    Scratch items_mem;
    std::vector<BInst> tab;
    std::vector<int> state;
    std::vector<std::unique_ptr<SlotMem>> mem;
    std::vector<long long> res_iter;
    std::vector<double> res_inertia;
    // current step plan
    std::vector<int> all, fits;
    // [0][v]: assignment items of variant v, [1][v]: transform items
    int n_items[2][kBatchVariants] = {{0, 0, 0}, {0, 0, 0}};
    int64_t item_off[2][kBatchVariants] = {{0, 0, 0}, {0, 0, 0}};
    bool dirty = true;
    GraphExec gA, gB;
    int *host_i = nullptr;  // pinned: empty counts then done flags
    int64_t steps = 0, graph_builds = 0, relocations = 0;

    ~BatchEngine() {
        if (s) cudaStreamSynchronize(s);
        if (host_i) cudaFreeHost(host_i);
        // device memory is released (stream-ordered) before the stream goes
        gA.reset();
        gB.reset();
        mem.clear();
        items_mem.release();
        dev.release();
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_out) cudaEventDestroy(ev_out);
        if (ev_fork) cudaEventDestroy(ev_fork);
        for (int v = 0; v < kBatchVariants; ++v) {
            if (side[v]) cudaStreamDestroy(side[v]);
            if (ev_join[v]) cudaEventDestroy(ev_join[v]);
        }
    }

    int init(int64_t capacity, cudaStream_t stream) {
        KMC_CHECK_ARG(capacity > 0 && capacity <= (1 << 20), "max_instances out of range");
        user = stream;
        KMC_CUDA_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        KMC_CUDA_TRY(cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming));
        KMC_CUDA_TRY(cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming));
        KMC_CUDA_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming));
        for (int v = 0; v < kBatchVariants; ++v) {
            KMC_CUDA_TRY(cudaStreamCreateWithFlags(&side[v], cudaStreamNonBlocking));
            KMC_CUDA_TRY(cudaEventCreateWithFlags(&ev_join[v], cudaEventDisableTiming));
        }
        cap = capacity;
        const size_t o_tab = 0;
        const size_t o_all = o_tab + align256(sizeof(BInst) * cap);
        const size_t o_fit = o_all + align256(sizeof(int) * cap);
        const size_t o_cnt = o_fit + align256(sizeof(int) * cap);
        const size_t o_ne = o_cnt + align256(sizeof(int) * 2 * kBatchVariants);
        const size_t o_dn = o_ne + align256(sizeof(int) * cap);
        KMC_TRY(dev.alloc(o_dn + align256(sizeof(int) * cap), s));
        char *b = dev.as<char>();
        tab_d = reinterpret_cast<BInst *>(b + o_tab);
        all_d = reinterpret_cast<int *>(b + o_all);
        fit_d = reinterpret_cast<int *>(b + o_fit);
        counters_d = reinterpret_cast<int *>(b + o_cnt);
        nempty_d = reinterpret_cast<int *>(b + o_ne);
        done_d = reinterpret_cast<int *>(b + o_dn);
        KMC_CUDA_TRY(cudaMallocHost(&host_i, sizeof(int) * 2 * cap));
        tab.assign((size_t)cap, BInst{});
        state.assign((size_t)cap, FREE);
        mem.resize((size_t)cap);
        res_iter.assign((size_t)cap, 0);
        res_inertia.assign((size_t)cap, 0.0);
        return KMC_OK;
    }

    int free_slot(int64_t *slot) {
        for (int64_t q = 0; q < cap; ++q)
            if (state[(size_t)q] == FREE) {
                *slot = q;
                return KMC_OK;
            }
        set_error("all %lld instance slots are in use", (long long)cap);
        return KMC_ERR_UNSUPPORTED;
    }

    int upload(int64_t q) {
        KMC_CUDA_TRY(cudaMemcpyAsync(tab_d + q, &tab[(size_t)q], sizeof(BInst),
                                     cudaMemcpyHostToDevice, s));
        // the host copy may change before the copy runs: order it now
        KMC_CUDA_TRY(cudaStreamSynchronize(s));
        return KMC_OK;
    }

    int add(int mode, const float *X, const float *w, float *C, int32_t *labels, int64_t n,
            int64_t d, int64_t k, double tol, int64_t max_iter, int64_t *out,
            float *dist = nullptr) {
        KMC_CHECK_ARG(n >= 0 && d >= 1 && k >= 1, "invalid dimensions (n=%lld, d=%lld, k=%lld)",
                      (long long)n, (long long)d, (long long)k);
        KMC_CHECK_ARG(d <= 1024 && k <= 4096, "batched fits take d <= 1024 and k <= 4096");
        KMC_CHECK_ARG(n < (int64_t(1) << 31), "n_samples must fit int32 labels");
        KMC_CHECK_ARG(mode != B_FIT || k <= n, "n_clusters exceeds n_samples");
        KMC_CHECK_ARG(tol >= 0.0, "Tolerance must be non-negative");
        int64_t q = 0;
        KMC_TRY(free_slot(&q));
        // the caller's writes of X, w and C come first
        KMC_CUDA_TRY(cudaEventRecord(ev_in, user));
        KMC_CUDA_TRY(cudaStreamWaitEvent(s, ev_in, 0));
        auto m = std::make_unique<SlotMem>();
        KMC_TRY(alloc_slot(*m, mode, n, d, k, s));
        int variant = 2;
        KMC_TRY(tune_variant(d, k, s, &variant));
        BInst h{};
        h.X = X;
        h.w = w;
        h.C = C;
        h.Cn = m->Cn;
        h.hn = m->hn;
        h.sizes = m->sizes;
        h.sums = m->sums;
        h.copies = mode == B_FIT ? batch_sum_copies(d, k) : 1;
        h.labels = labels;
        h.dist = dist;
        h.empty_list = m->empty_list;
        h.n = n;
        h.d = (int)d;
        h.k = (int)k;
        h.mode = mode;
        h.variant = variant;
        h.st.max_iter = max_iter;
        const float tol_t = (float)tol;
        h.st.tol = (double)tol_t;
        // while (n_iter < max_iter && shift_sum > tol), shift_sum = +inf at
        // the start (kmeans_lloyd_driver.hpp:78, 83)
        h.st.done = (mode == B_FIT && !(0 < max_iter && pos_inf<float>() > tol_t)) ? 1 : 0;
        tab[(size_t)q] = h;
        mem[(size_t)q] = std::move(m);
        state[(size_t)q] = RUNNING;
        res_iter[(size_t)q] = 0;
        res_inertia[(size_t)q] = 0.0;
        KMC_TRY(upload(q));
        dirty = true;
        *out = q;
        if (h.st.done) KMC_TRY(finish_fit(q));
        return KMC_OK;
    }

    int remove(int64_t q) {
        KMC_CHECK_ARG(q >= 0 && q < cap && state[(size_t)q] != FREE, "no such instance");
        KMC_CUDA_TRY(cudaStreamSynchronize(s));
        mem[(size_t)q].reset();
        state[(size_t)q] = FREE;
        dirty = true;
        return KMC_OK;
    }

    int64_t running() const {
        int64_t c = 0;
        for (int v : state) c += (v == RUNNING);
        return c;
    }

    // Work lists, work queue and graphs for the current running set.
    int plan() {
        all.clear();
        fits.clear();
        std::vector<BItem> items[2][kBatchVariants];
        for (int64_t q = 0; q < cap; ++q) {
            if (state[(size_t)q] != RUNNING) continue;
            const BInst &h = tab[(size_t)q];
            all.push_back((int)q);
            if (h.mode == B_FIT) fits.push_back((int)q);
            append_items((int)q, h.n, h.mode, h.variant, items);
        }
        int64_t total = 0;
        for (int kind = 0; kind < 2; ++kind)
            for (int v = 0; v < kBatchVariants; ++v) {
                item_off[kind][v] = total;
                n_items[kind][v] = (int)items[kind][v].size();
                total += n_items[kind][v];
            }
        if (total > items_cap) {
            items_cap = std::max<int64_t>(total, 2 * items_cap);
            KMC_TRY(items_mem.alloc(sizeof(BItem) * (size_t)items_cap, s));
            items_d = items_mem.as<BItem>();
        }
        for (int kind = 0; kind < 2; ++kind)
            for (int v = 0; v < kBatchVariants; ++v)
                if (n_items[kind][v] > 0)
                    KMC_CUDA_TRY(cudaMemcpyAsync(items_d + item_off[kind][v],
                                                 items[kind][v].data(),
                                                 sizeof(BItem) * n_items[kind][v],
                                                 cudaMemcpyHostToDevice, s));
        if (!all.empty())
            KMC_CUDA_TRY(cudaMemcpyAsync(all_d, all.data(), sizeof(int) * all.size(),
                                         cudaMemcpyHostToDevice, s));
        if (!fits.empty())
            KMC_CUDA_TRY(cudaMemcpyAsync(fit_d, fits.data(), sizeof(int) * fits.size(),
                                         cudaMemcpyHostToDevice, s));
        KMC_CUDA_TRY(cudaStreamSynchronize(s));
        // kernel attributes are set outside the capture
        KMC_TRY(prepare_batch_assign());
        KMC_TRY(capture(&gA, [&]() -> int {
            KMC_TRY(launch_batch_prep(tab_d, all_d, (int)all.size(), counters_d, s));
            KMC_CUDA_TRY(cudaEventRecord(ev_fork, s));
            // one branch per centroid-window variant: its assignment items,
            // then its transform items
            for (int v = 0; v < kBatchVariants; ++v) {
                if (n_items[0][v] + n_items[1][v] == 0) continue;
                KMC_CUDA_TRY(cudaStreamWaitEvent(side[v], ev_fork, 0));
                for (int kind = 0; kind < 2; ++kind)
                    KMC_TRY(launch_batch_assign(v, kind, tab_d, items_d + item_off[kind][v],
                                                n_items[kind][v],
                                                counters_d + kind * kBatchVariants + v, side[v]));
                KMC_CUDA_TRY(cudaEventRecord(ev_join[v], side[v]));
                KMC_CUDA_TRY(cudaStreamWaitEvent(s, ev_join[v], 0));
            }
            return launch_batch_reduce(tab_d, fit_d, (int)fits.size(), nempty_d, s);
        }));
        KMC_TRY(capture(&gB, [&]() -> int {
            return launch_batch_update(tab_d, fit_d, (int)fits.size(), done_d, s);
        }));
        ++graph_builds;
        dirty = false;
        return KMC_OK;
    }

    template <typename F>
    int capture(GraphExec *g, F body) {
        g->reset();
        cudaGraph_t graph = nullptr;
        KMC_CUDA_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        const int rc = body();
        const cudaError_t e = cudaStreamEndCapture(s, &graph);
        if (rc != KMC_OK) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        KMC_CUDA_TRY(e);
        const cudaError_t ei = cudaGraphInstantiate(&g->exec, graph, 0);
        cudaGraphDestroy(graph);
        KMC_CUDA_TRY(ei);
        return KMC_OK;
    }

    // kmeans_lloyd_driver.hpp:217-312 for one instance with m empty clusters.
    int relocate(int64_t q, int m) {
        const BInst &h = tab[(size_t)q];
        SlotMem &sm = *mem[(size_t)q];
        int32_t *counters = sm.selected + h.n;
        KMC_TRY(launch_inertia<float, int32_t>(h.X, nullptr, h.C, h.labels, sm.sq_dist, h.n, h.d,
                                               h.k, s));
        KMC_TRY(launch_threshold<float>(sm.sq_dist, h.n, nullptr, m, sm.thr, sm.thr_scratch, s));
        KMC_TRY(launch_fill<int32_t>(counters, 0, 1, s));
        KMC_TRY(launch_fill<int32_t>(counters + 1, 1, 1, s));
        KMC_TRY(launch_select<float, int32_t>(nullptr, m, sm.sq_dist, sm.thr, sm.selected,
                                              counters, counters + 1, h.n, sm.sel_scratch, h.k,
                                              s));
        KMC_TRY(launch_relocate<float, int32_t>(nullptr, m, h.X, h.w, h.labels, sm.selected,
                                                counters, sm.empty_list, sm.Cn, sm.sizes,
                                                sm.sq_dist, h.n, h.d, h.k, s));
        ++relocations;
        return KMC_OK;
    }

    // kmeans_lloyd_driver.hpp:360-418: labels and weighted inertia against
    // the final centroids.
    int finish_fit(int64_t q) {
        const BInst &h = tab[(size_t)q];
        SlotMem &sm = *mem[(size_t)q];
        KMC_TRY(launch_half_norm<float>(h.C, sm.hn, h.d, h.k, s));
        KMC_TRY(launch_assignment<float, int32_t>(h.X, h.C, sm.hn, h.labels, h.n, h.d, h.k, s));
        KMC_TRY(launch_inertia<float, int32_t>(h.X, h.w, h.C, h.labels, sm.sq_dist, h.n, h.d,
                                               h.k, s));
        KMC_TRY(launch_sum_f64<float>(sm.sq_dist, h.n, sm.partials, sm.dsum, s));
        LoopState st{};
        double tot = 0.0;
        KMC_CUDA_TRY(cudaMemcpyAsync(&st, &tab_d[q].st, sizeof(st), cudaMemcpyDeviceToHost, s));
        KMC_CUDA_TRY(cudaMemcpyAsync(&tot, sm.dsum, sizeof(double), cudaMemcpyDeviceToHost, s));
        KMC_CUDA_TRY(cudaStreamSynchronize(s));
        res_iter[(size_t)q] = st.n_iter;
        res_inertia[(size_t)q] = tot;
        state[(size_t)q] = FINISHED;
        dirty = true;
        return KMC_OK;
    }

    int step(int64_t *n_active) {
        if (dirty) KMC_TRY(plan());
        if (!all.empty()) {
            KMC_CUDA_TRY(cudaGraphLaunch(gA.exec, s));
            const size_t nf = fits.size();
            if (nf > 0) {
                KMC_CUDA_TRY(cudaMemcpyAsync(host_i, nempty_d, sizeof(int) * nf,
                                             cudaMemcpyDeviceToHost, s));
                KMC_CUDA_TRY(cudaStreamSynchronize(s));
                for (size_t t = 0; t < nf; ++t)
                    if (host_i[t] > 0) KMC_TRY(relocate(fits[t], host_i[t]));
                KMC_CUDA_TRY(cudaGraphLaunch(gB.exec, s));
                KMC_CUDA_TRY(cudaMemcpyAsync(host_i + cap, done_d, sizeof(int) * nf,
                                             cudaMemcpyDeviceToHost, s));
            }
            KMC_CUDA_TRY(cudaStreamSynchronize(s));
            ++steps;
            for (size_t t = 0; t < nf; ++t)
                if (host_i[cap + t]) KMC_TRY(finish_fit(fits[t]));
            for (int q : all)
                if (tab[(size_t)q].mode != B_FIT) {
                    state[(size_t)q] = FINISHED;
                    res_iter[(size_t)q] = 0;
                    dirty = true;
                }
        }
        KMC_CUDA_TRY(cudaEventRecord(ev_out, s));
        KMC_CUDA_TRY(cudaStreamWaitEvent(user, ev_out, 0));
        if (n_active) *n_active = running();
        return KMC_OK;
    }
};

// ---------------------------------------------------------------------------
// Serving: a request server over caller buffers (kmc_server_*) and, built on
// it, the replay harness of a request stream (kmc_serve_run)
// ---------------------------------------------------------------------------
namespace serving {

// Bytes of a request's own data: samples, weights, centroids and labels, and
// for a transform its (k, n) distances.
int64_t data_bytes(int kind, int64_t n, int64_t d, int64_t k) {
    int64_t b = (int64_t)(align256(sizeof(float) * n * d) + align256(sizeof(float) * n) +
                          align256(sizeof(float) * d * k) + align256(sizeof(int32_t) * n));
    if (kind == 2) b += (int64_t)align256(sizeof(float) * n * k);
    return b;
}

// Device bytes the server allocates for a request while it runs: a fit's
// model (its working centroids, kept after the fit for predictions), a
// transform's checksum scratch, and the batched engine's slot or the
// tensor-core session's working memory.
int64_t work_bytes(int kind, int64_t n, int64_t d, int64_t k, int form) {
    const int64_t d4 = ceil_div<int64_t>(std::max<int64_t>(d, 1), 4) * 4;
    int64_t b = (int64_t)align256(sizeof(float) * d * k);
    if (kind == 2) {
        b += (int64_t)(align256(sizeof(double) * (sum_partials_size() + 1)) +
                       slot_bytes(B_ASSIGN, n, d, k));
    } else if (form == KMC_FORM_PLAIN) {
        b += (int64_t)slot_bytes(kind == 0 ? B_FIT : B_ASSIGN, n, d, k);
    } else {
        // plain-fit workspace plus the tensor-core operands: fp16/bf16 image,
        // fp32 row copy, norms, candidate masks, recheck list, cluster sums
        const int64_t nkb = ceil_div<int64_t>(std::max<int64_t>(d, 1), 64);
        const int64_t kp = ceil_div<int64_t>(k, 256) * 256;
        b += (int64_t)slot_bytes(B_FIT, n, d, k) +
             n * (nkb * 128 + 4 * d4 + 8 + 16 + 4) + kp * (nkb * 128 + 32 + 4 * d4) +
             152 * (kp * d4 + kp) * 8;
    }
    return b;
}

int64_t with_slack(int64_t b) { return b + (b >> 4) + (16 << 20); }

// What one replayed request holds while admitted: its data and the server's
// working memory, with allocator slack.
int64_t request_bytes(int kind, int64_t n, int64_t d, int64_t k, int form) {
    return with_slack(data_bytes(kind, n, d, k) + work_bytes(kind, n, d, k, form));
}

// A replayed request's data (generated on the device when it is admitted).
struct ReqMem {
    Scratch mem;
    float *X = nullptr, *w = nullptr, *C = nullptr, *Cres = nullptr;
    int32_t *labels = nullptr;
    float *dist = nullptr;  // transform: (k, n) distances
};

int alloc_request(ReqMem &m, int64_t n, int64_t d, int64_t k, int kind, cudaStream_t s) {
    const size_t bX = align256(sizeof(float) * n * d), bw = align256(sizeof(float) * n),
                 bC = align256(sizeof(float) * d * k), bl = align256(sizeof(int32_t) * n);
    const size_t bD = kind == 2 ? align256(sizeof(float) * n * k) : 0;
    KMC_TRY(m.mem.alloc(bX + bw + 2 * bC + bl + bD, s));
    char *b = m.mem.as<char>();
    m.X = reinterpret_cast<float *>(b);
    m.w = reinterpret_cast<float *>(b + bX);
    m.C = reinterpret_cast<float *>(b + bX + bw);
    m.Cres = reinterpret_cast<float *>(b + bX + bw + bC);
    m.labels = reinterpret_cast<int32_t *>(b + bX + bw + 2 * bC);
    if (kind == 2) m.dist = reinterpret_cast<float *>(b + bX + bw + 2 * bC + bl);
    return KMC_OK;
}

// State of a request while it runs.
struct Active {
    int64_t inst = -1;                 // plain: batch instance
    std::unique_ptr<FitBase> fit;      // mixed: tensor-core fit session
    cudaEvent_t ev = nullptr;          // mixed: a transform's distances are written
    cudaStream_t st = nullptr;         // the request's stream
    Scratch sums;                      // transform: float64 checksum scratch
    // mixed fits and predictions: one captured iteration (kernels + a copy of
    // the loop state to pinned host memory), the event that marks the end of
    // the session's last enqueued work, and its pinned result slot
    cudaGraphExec_t iter_graph = nullptr;
    cudaEvent_t step_ev = nullptr;
    int slot = -1;
    LoopState *hstate = nullptr;
    double *hinertia = nullptr;
    bool inflight = false;
    bool final_enqueued = false;
    ~Active() {
        if (iter_graph) cudaGraphExecDestroy(iter_graph);
        if (step_ev) cudaEventDestroy(step_ev);
        if (ev) cudaEventDestroy(ev);
    }
};

// Iterations a mixed session is given per visit of the serving loop: the loop
// state is checked between visits, and iterations enqueued past the stop are
// no-ops (every kernel reads the device loop state first).
constexpr int kItersPerVisit = 4;

// Captures one iteration of a session into a graph, followed by a copy of the
// loop state into the session's pinned slot.
int capture_iteration(Active &a) {
    cudaGraph_t g = nullptr;
    KMC_CUDA_TRY(cudaStreamBeginCapture(a.st, cudaStreamCaptureModeRelaxed));
    int rc = a.fit->enqueue_iteration();
    if (rc == KMC_OK) {
        const cudaError_t e = cudaMemcpyAsync(a.hstate, a.fit->device_state(), sizeof(LoopState),
                                              cudaMemcpyDeviceToHost, a.st);
        if (e != cudaSuccess) {
            set_error("CUDA error %s in capture_iteration", cudaGetErrorName(e));
            rc = KMC_ERR_CUDA;
        }
    }
    const cudaError_t ee = cudaStreamEndCapture(a.st, &g);
    if (rc != KMC_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    KMC_CUDA_TRY(ee);
    const cudaError_t ei = cudaGraphInstantiate(&a.iter_graph, g, 0);
    cudaGraphDestroy(g);
    KMC_CUDA_TRY(ei);
    return KMC_OK;
}


// A request server: fits, predictions and transforms of different sizes on
// caller buffers, admitted in submission order while the HBM budget and the
// number of running requests allow; predictions wait (without blocking the
// queue) for the fit whose model they use.  A fit's centroids stay on the
// device as its model until the ticket is released or the server closed.
//   plain form   every running request is an instance of one batched engine
//                (persistent kernels fed by a device work queue, replayed as
//                CUDA graphs); each progress call advances all of them by one
//                iteration and retires the finished ones
//   mixed forms  one tensor-core fit session per request on a pool of
//                streams; each session replays a captured iteration and
//                advances on its own (event queries, no host waits)
// The server is driven by its callers (submit, poll, wait): calls on one
// server must not overlap.
struct Server {
    struct Ticket {
        int64_t id = -1;
        int kind = 0;  // 0 fit, 1 predict, 2 transform
        int state = KMC_REQ_PENDING, status = KMC_OK;
        int64_t n = 0, d = 0, k = 0, max_iter = 0, model = -1;
        double tol = 0.0;
        const float *X = nullptr, *w = nullptr, *Cinit = nullptr;
        int32_t *labels = nullptr;
        float *Cout = nullptr, *dist = nullptr;
        Scratch model_mem;   // fit: working centroids, then the model
        float *mdl = nullptr;
        int64_t extra = 0;   // bytes the caller declares held while it runs
        int64_t bytes = 0;   // bytes admitted
        cudaEvent_t ready = nullptr;  // the caller's writes of the inputs
        // replay harness: makes the request's data when it is admitted
        std::function<int(Ticket &, cudaStream_t)> on_admit;
        std::unique_ptr<ReqMem> data;
        double admit_s = -1.0, finish_s = -1.0, inertia = 0.0;
        int64_t n_iter = 0;
        bool cancel = false, released = false;
        std::unique_ptr<Active> act;
        ~Ticket() {
            if (ready) cudaEventDestroy(ready);
        }
    };

    int form = KMC_FORM_PLAIN;
    bool plain = true;
    int64_t budget = 0, max_active = 1, in_use = 0;
    cudaStream_t user = nullptr;
    BatchEngine eng;
    static constexpr int kStreams = 8;
    std::vector<cudaStream_t> pool;
    int64_t rr = 0;
    static constexpr size_t kSlotBytes = 128;
    char *pinned = nullptr;
    std::vector<int> free_slots;
    std::vector<std::unique_ptr<Ticket>> tickets;
    std::deque<int64_t> pending;
    std::vector<int64_t> running;
    std::vector<int64_t> finished_log;  // tickets in the order they finished
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double elapsed() const {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }

    ~Server() {
        // requests still running are stopped; nothing may write memory that
        // is about to be freed
        for (int64_t id : running) {
            Ticket &t = *tickets[(size_t)id];
            if (t.act && t.act->st) cudaStreamSynchronize(t.act->st);
            t.act.reset();
        }
        if (plain && eng.s) cudaStreamSynchronize(eng.s);
        for (auto t : pool) cudaStreamSynchronize(t);
        tickets.clear();
        for (auto t : pool) {
            cudaStreamSynchronize(t);
            cudaStreamDestroy(t);
        }
        if (pinned) cudaFreeHost(pinned);
    }

    int init(int f, int64_t bud, int64_t max_act, cudaStream_t s) {
        KMC_CHECK_ARG(f == KMC_FORM_PLAIN || f == KMC_FORM_MIXED_BF16 || f == KMC_FORM_MIXED_FP16,
                      "unknown form %d", f);
        KMC_CHECK_ARG(bud > 0, "hbm_budget_bytes must be positive");
        KMC_CHECK_ARG(max_act >= 1 && max_act <= (1 << 16), "max_active out of range");
        form = f;
        plain = f == KMC_FORM_PLAIN;
        budget = bud;
        max_active = max_act;
        user = s;
        if (plain) {
            KMC_TRY(eng.init(max_act, s));
        } else {
            for (int q = 0; q < kStreams; ++q) {
                cudaStream_t t = nullptr;
                KMC_CUDA_TRY(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking));
                pool.push_back(t);
            }
            KMC_CUDA_TRY(cudaHostAlloc(&pinned, kSlotBytes * (size_t)max_act, cudaHostAllocDefault));
            for (int64_t q = max_act - 1; q >= 0; --q) free_slots.push_back((int)q);
        }
        return KMC_OK;
    }

    Ticket *get(int64_t id) {
        if (id < 0 || id >= (int64_t)tickets.size() || tickets[(size_t)id]->released)
            return nullptr;
        return tickets[(size_t)id].get();
    }

    // Queues a request; the caller's stream orders its input writes.
    int submit(std::unique_ptr<Ticket> t, int64_t *id_out) {
        KMC_CUDA_TRY(cudaEventCreateWithFlags(&t->ready, cudaEventDisableTiming));
        KMC_CUDA_TRY(cudaEventRecord(t->ready, user));
        const int64_t id = (int64_t)tickets.size();
        t->id = id;
        tickets.push_back(std::move(t));
        pending.push_back(id);
        *id_out = id;
        return KMC_OK;
    }

    static bool final_state(int s) { return s >= KMC_REQ_DONE; }

    void end(Ticket &t, int state, int status) {
        if (t.act) {
            if (t.act->slot >= 0) free_slots.push_back(t.act->slot);
            t.act.reset();
        }
        if (state != KMC_REQ_DONE || t.kind != 0) t.model_mem.release();
        if (state != KMC_REQ_DONE) t.mdl = nullptr;
        t.data.reset();
        in_use -= t.bytes;
        t.bytes = 0;
        t.state = state;
        t.status = status;
        t.finish_s = elapsed();
        finished_log.push_back(t.id);
    }

    // Starts an admitted request: its stream waits for the caller's writes,
    // the harness makes its data, a fit copies its initial centroids into its
    // model, and the work is handed to the engine or a fit session.
    int start(Ticket &t, const Ticket *m) {
        // owned by the ticket from here on, so a failure below is cleaned up
        // by end() (the session, the pinned slot)
        t.act = std::make_unique<Active>();
        Active *a = t.act.get();
        a->st = plain ? user : pool[(size_t)(rr++ % kStreams)];
        KMC_CUDA_TRY(cudaStreamWaitEvent(a->st, t.ready, 0));
        if (t.on_admit) KMC_TRY(t.on_admit(t, a->st));
        const float *model = (t.kind == 0) ? nullptr : m->mdl;
        if (t.kind == 0) {
            KMC_TRY(t.model_mem.alloc(sizeof(float) * t.d * t.k, a->st));
            t.mdl = t.model_mem.as<float>();
            KMC_CUDA_TRY(cudaMemcpyAsync(t.mdl, t.Cinit, sizeof(float) * t.d * t.k,
                                         cudaMemcpyDeviceToDevice, a->st));
        }
        if (t.kind == 2) KMC_TRY(a->sums.alloc(sizeof(double) * (sum_partials_size() + 1), a->st));
        if (plain) {
            // the engine's stream is ordered after `user` when an instance is added
            if (t.kind == 0)
                KMC_TRY(eng.add(B_FIT, t.X, t.w, t.mdl, t.labels, t.n, t.d, t.k, t.tol,
                                t.max_iter, &a->inst));
            else if (t.kind == 1)
                KMC_TRY(eng.add(B_ASSIGN, t.X, nullptr, const_cast<float *>(model), t.labels, t.n,
                                t.d, t.k, 0.0, 0, &a->inst));
            else
                KMC_TRY(eng.add(B_TRANSFORM, t.X, nullptr, const_cast<float *>(model), nullptr,
                                t.n, t.d, t.k, 0.0, 0, &a->inst, t.dist));
        } else if (t.kind == 2) {
            // exact float32 distances (no tensor-core form of the distance matrix)
            KMC_TRY(launch_distances<float>(t.X, model, t.dist, t.n, t.d, t.k, a->st));
            KMC_CUDA_TRY(cudaEventCreateWithFlags(&a->ev, cudaEventDisableTiming));
            KMC_CUDA_TRY(cudaEventRecord(a->ev, a->st));
        } else {
            FitParams<float, int32_t> p;
            p.X = t.X;
            p.w = t.kind == 0 ? t.w : nullptr;
            // a prediction reads the model and writes nothing but labels
            p.centroids = t.kind == 0 ? t.mdl : const_cast<float *>(model);
            p.new_centroids = t.kind == 0 ? t.Cout : const_cast<float *>(model);
            p.labels = t.labels;
            p.n = t.n;
            p.d = t.d;
            p.k = t.k;
            p.tol = t.kind == 0 ? t.tol : 0.0;
            p.max_iter = t.kind == 0 ? t.max_iter : 0;
            p.stream = a->st;
            // a cached variant choice or the default: no timing on a request's path
            mixed_tuning_lookup_only(true);
            const int mrc = make_mixed_fit<float, int32_t>(p, form, &a->fit);
            mixed_tuning_lookup_only(false);
            KMC_TRY(mrc);
            a->slot = free_slots.back();
            free_slots.pop_back();
            a->hstate = reinterpret_cast<LoopState *>(pinned + kSlotBytes * (size_t)a->slot);
            a->hinertia = reinterpret_cast<double *>(pinned + kSlotBytes * (size_t)a->slot + 64);
            // the slot's previous session has retired: nothing writes it now
            *reinterpret_cast<volatile int *>(&a->hstate->done) = 0;
            *reinterpret_cast<volatile unsigned *>(&a->hstate->err) = 0u;
            KMC_CUDA_TRY(cudaEventCreateWithFlags(&a->step_ev, cudaEventDisableTiming));
            if (p.max_iter > 0) KMC_TRY(capture_iteration(*a));
        }
        return KMC_OK;
    }

    // Admission in submission order while the budget and the running count
    // allow; a prediction whose model is not ready yet waits without
    // blocking the requests behind it.
    int admit(bool *moved) {
        for (auto it = pending.begin(); it != pending.end();) {
            const int64_t id = *it;
            Ticket &t = *tickets[(size_t)id];
            if (t.cancel) {
                end(t, KMC_REQ_CANCELLED, KMC_ERR_CANCELLED);
                it = pending.erase(it);
                *moved = true;
                continue;
            }
            const Ticket *m = nullptr;
            if (t.kind != 0) {
                m = tickets[(size_t)t.model].get();
                if (m->state == KMC_REQ_PENDING || m->state == KMC_REQ_RUNNING) {
                    ++it;
                    continue;
                }
                if (m->state != KMC_REQ_DONE || m->released) {
                    set_error("request %lld: its model (request %lld) did not complete",
                              (long long)id, (long long)t.model);
                    end(t, KMC_REQ_FAILED, KMC_ERR_INVALID_ARGUMENT);
                    it = pending.erase(it);
                    *moved = true;
                    continue;
                }
            }
            const int64_t need = with_slack(work_bytes(t.kind, t.n, t.d, t.k, form) + t.extra);
            if (need > budget) {  // can never be admitted
                end(t, KMC_REQ_FAILED, KMC_ERR_OUT_OF_MEMORY);
                it = pending.erase(it);
                *moved = true;
                continue;
            }
            if ((int64_t)running.size() >= max_active || in_use + need > budget) break;
            it = pending.erase(it);
            t.bytes = need;
            in_use += need;
            t.state = KMC_REQ_RUNNING;
            t.admit_s = elapsed();
            const int rc = start(t, m);
            *moved = true;
            if (rc != KMC_OK) {
                // a request that cannot start fails alone; the server goes on
                if (t.act && t.act->st) cudaStreamSynchronize(t.act->st);
                if (plain && t.act && t.act->inst >= 0) eng.remove(t.act->inst);
                end(t, KMC_REQ_FAILED, rc);
                continue;
            }
            running.push_back(id);
        }
        return KMC_OK;
    }

    // Float64 total of a transform's distances (deterministic order).
    int dist_checksum(Ticket &t, cudaStream_t s, double *out) {
        double *part = t.act->sums.as<double>();
        KMC_TRY(launch_sum_f64<float>(t.dist, t.n * t.k, part, part + sum_partials_size(), s));
        KMC_CUDA_TRY(cudaMemcpyAsync(out, part + sum_partials_size(), sizeof(double),
                                     cudaMemcpyDeviceToHost, s));
        KMC_CUDA_TRY(cudaStreamSynchronize(s));
        return KMC_OK;
    }

    // Plain form: one engine iteration for every running request.
    int advance_plain(bool *moved) {
        if (running.empty()) return KMC_OK;
        KMC_TRY(eng.step(nullptr));
        *moved = true;
        for (size_t r = 0; r < running.size();) {
            Ticket &t = *tickets[(size_t)running[r]];
            const int64_t q = t.act->inst;
            int state = -1, status = KMC_OK;
            if (t.cancel) {
                state = KMC_REQ_CANCELLED;
                status = KMC_ERR_CANCELLED;
            } else if (eng.state[(size_t)q] == BatchEngine::FINISHED) {
                state = KMC_REQ_DONE;
                t.n_iter = eng.res_iter[(size_t)q];
                t.inertia = eng.res_inertia[(size_t)q];
                if (t.kind == 0 && t.Cout != nullptr)
                    KMC_CUDA_TRY(cudaMemcpyAsync(t.Cout, t.mdl, sizeof(float) * t.d * t.k,
                                                 cudaMemcpyDeviceToDevice, eng.s));
                if (t.kind == 2) KMC_TRY(dist_checksum(t, eng.s, &t.inertia));
                KMC_CUDA_TRY(cudaStreamSynchronize(eng.s));
            }
            if (state < 0) {
                ++r;
                continue;
            }
            KMC_TRY(eng.remove(q));
            end(t, state, status);
            running.erase(running.begin() + (int64_t)r);
        }
        return KMC_OK;
    }

    // Mixed forms: each session advances on its own.  Once its last enqueued
    // work is done it gets kItersPerVisit more iterations (one graph launch
    // each) or, when its loop has stopped, the final pass, and it retires when
    // that is done.  No session waits for another, and the host neither
    // launches kernels one by one nor waits on a stream.
    int advance_mixed(bool *moved) {
        for (size_t r = 0; r < running.size();) {
            Ticket &t = *tickets[(size_t)running[r]];
            Active &a = *t.act;
            auto retire = [&](int state, int status) {
                end(t, state, status);
                running.erase(running.begin() + (int64_t)r);
                *moved = true;
            };
            if (!a.fit) {  // a transform in flight
                const cudaError_t q = cudaEventQuery(a.ev);
                if (q == cudaErrorNotReady) {
                    ++r;
                    continue;
                }
                KMC_CUDA_TRY(q);
                if (!t.cancel) KMC_TRY(dist_checksum(t, a.st, &t.inertia));
                retire(t.cancel ? KMC_REQ_CANCELLED : KMC_REQ_DONE,
                       t.cancel ? KMC_ERR_CANCELLED : KMC_OK);
                continue;
            }
            if (a.inflight) {
                const cudaError_t q = cudaEventQuery(a.step_ev);
                if (q == cudaErrorNotReady) {
                    ++r;
                    continue;
                }
                KMC_CUDA_TRY(q);
                a.inflight = false;
            }
            if (t.cancel) {
                retire(KMC_REQ_CANCELLED, KMC_ERR_CANCELLED);
                continue;
            }
            const volatile LoopState *hs = a.hstate;
            if (a.final_enqueued) {
                t.n_iter = (int64_t)hs->n_iter;
                t.inertia = *(const volatile double *)a.hinertia;
                // a tensor-core kernel that gave up a wait fails the request
                if (hs->err != 0)
                    retire(KMC_REQ_FAILED, KMC_ERR_DEVICE_TIMEOUT);
                else
                    retire(KMC_REQ_DONE, KMC_OK);
                continue;
            }
            if (a.iter_graph == nullptr || hs->done) {
                KMC_TRY(a.fit->finalize_enqueue(a.hstate, a.hinertia));
                a.final_enqueued = true;
            } else {
                for (int i = 0; i < kItersPerVisit; ++i)
                    KMC_CUDA_TRY(cudaGraphLaunch(a.iter_graph, a.st));
            }
            KMC_CUDA_TRY(cudaEventRecord(a.step_ev, a.st));
            a.inflight = true;
            *moved = true;
            ++r;
        }
        return KMC_OK;
    }

    int progress(bool *moved) {
        Range range("kmc.server_progress");
        *moved = false;
        KMC_TRY(admit(moved));
        if (plain)
            KMC_TRY(advance_plain(moved));
        else
            KMC_TRY(advance_mixed(moved));
        // retirements free budget: admit again without waiting for the next call
        if (*moved) KMC_TRY(admit(moved));
        return KMC_OK;
    }

    int wait(int64_t id) {
        Ticket *t = get(id);
        KMC_CHECK_ARG(t != nullptr, "no such ticket %lld", (long long)id);
        while (!final_state(t->state)) {
            bool moved = false;
            KMC_TRY(progress(&moved));
            if (!moved) std::this_thread::sleep_for(std::chrono::microseconds(20));
        }
        return KMC_OK;
    }

    int cancel(int64_t id) {
        Ticket *t = get(id);
        KMC_CHECK_ARG(t != nullptr, "no such ticket %lld", (long long)id);
        if (!final_state(t->state)) t->cancel = true;
        bool moved = false;
        return progress(&moved);
    }

    // Drops a finished request's record and, for a fit, its model.
    int release(int64_t id) {
        Ticket *t = get(id);
        KMC_CHECK_ARG(t != nullptr, "no such ticket %lld", (long long)id);
        KMC_CHECK_ARG(final_state(t->state), "ticket %lld has not finished", (long long)id);
        t->model_mem.release();
        t->mdl = nullptr;
        t->released = true;
        return KMC_OK;
    }
};


// Shapes a form can serve: the batched engine takes d <= 1024 and k <= 4096;
// the tensor-core sessions take what the mixed fit supports.
int check_shape(int form, int64_t d, int64_t k) {
    if (form == KMC_FORM_PLAIN) {
        KMC_CHECK_ARG(d <= 1024 && k <= 4096, "the plain server takes d <= 1024 and k <= 4096");
        return KMC_OK;
    }
    if (!mixed_fit_supported(d, k)) {
        set_error("the mixed forms do not support d=%lld, k=%lld", (long long)d, (long long)k);
        return KMC_ERR_UNSUPPORTED;
    }
    return KMC_OK;
}

// Replays a request stream on a Server: each request is submitted at its
// arrival time and its data (seeded blobs, a seeded-row initialisation) is
// generated on the device when it is admitted, so the budget covers it.
int serve_run(const kmc_serve_request_t *rq, int64_t n_req, int form, int64_t budget,
              int64_t max_active, cudaStream_t s, kmc_serve_result_t *out, double *makespan) {
    KMC_CHECK_ARG(n_req >= 0 && (n_req == 0 || (rq != nullptr && out != nullptr)),
                  "null request or result array");
    KMC_CHECK_ARG(max_active >= 1, "max_active must be positive");
    KMC_CHECK_ARG(form == KMC_FORM_PLAIN || form == KMC_FORM_MIXED_BF16 ||
                      form == KMC_FORM_MIXED_FP16,
                  "unknown form %d", form);
    for (int64_t r = 0; r < n_req; ++r) {
        const kmc_serve_request_t &q = rq[r];
        KMC_CHECK_ARG(q.kind >= 0 && q.kind <= 2, "request %lld: kind must be 0, 1 or 2",
                      (long long)r);
        KMC_CHECK_ARG(q.n_samples >= 1 && q.n_features >= 1 && q.n_clusters >= 1 &&
                          (q.kind != 0 || q.n_clusters <= q.n_samples) && q.n_centers >= 1,
                      "request %lld: invalid sizes", (long long)r);
        KMC_CHECK_ARG(r == 0 || q.arrival_s >= rq[r - 1].arrival_s,
                      "requests must be sorted by arrival time");
        KMC_CHECK_ARG(q.kind == 0 || (q.model >= 0 && q.model < r && rq[q.model].kind == 0 &&
                                      rq[q.model].n_features == q.n_features &&
                                      rq[q.model].n_clusters == q.n_clusters),
                      "request %lld: a prediction or transform must name an earlier fit of "
                      "the same d, k",
                      (long long)r);
        out[r] = kmc_serve_result_t{-1.0, -1.0, 0, 0.0, KMC_OK, 0};
    }
    Server srv;
    KMC_TRY(srv.init(form, budget, max_active, s));
    std::vector<int64_t> ticket(n_req, -1), req_of;
    int64_t next = 0, finished = 0;
    size_t seen = 0;
    while (finished < n_req) {
        const double now = srv.elapsed();
        while (next < n_req && rq[next].arrival_s <= now) {
            const kmc_serve_request_t &q = rq[next];
            auto t = std::make_unique<Server::Ticket>();
            t->kind = q.kind;
            t->n = q.n_samples;
            t->d = q.n_features;
            t->k = q.n_clusters;
            t->tol = q.kind == 0 ? q.tol : 0.0;
            t->max_iter = q.kind == 0 ? q.max_iter : 0;
            t->model = q.kind == 0 ? -1 : ticket[(size_t)q.model];
            t->extra = data_bytes(q.kind, q.n_samples, q.n_features, q.n_clusters);
            t->on_admit = [q](Server::Ticket &tk, cudaStream_t st) -> int {
                tk.data = std::make_unique<ReqMem>();
                ReqMem &m = *tk.data;
                KMC_TRY(alloc_request(m, tk.n, tk.d, tk.k, q.kind, st));
                KMC_TRY(launch_blobs(m.X, tk.n, tk.d, q.n_centers, -10.f, 10.f, q.std_lo,
                                     q.std_hi, q.seed, st));
                KMC_TRY(launch_fill<float>(m.w, 1.f, tk.n, st));
                if (q.kind == 0) {
                    std::vector<int32_t> rows;
                    seeded_rows(tk.n, tk.k, q.seed ^ 0x9999ull, &rows);
                    Scratch idx;
                    KMC_TRY(idx.alloc(sizeof(int32_t) * rows.size(), st));
                    // a pageable upload returns once its source is staged, and
                    // the index buffer is freed in stream order
                    KMC_CUDA_TRY(cudaMemcpyAsync(idx.ptr, rows.data(),
                                                 sizeof(int32_t) * rows.size(),
                                                 cudaMemcpyHostToDevice, st));
                    KMC_TRY(launch_gather_rows(m.X, tk.n, tk.d, idx.as<int32_t>(), tk.k, m.C, st));
                }
                tk.X = m.X;
                tk.w = m.w;
                tk.Cinit = m.C;
                tk.labels = m.labels;
                tk.Cout = m.Cres;
                tk.dist = m.dist;
                return KMC_OK;
            };
            int64_t id = -1;
            KMC_TRY(srv.submit(std::move(t), &id));
            ticket[(size_t)next] = id;
            if ((int64_t)req_of.size() <= id) req_of.resize((size_t)id + 1, -1);
            req_of[(size_t)id] = next;
            ++next;
        }
        bool moved = false;
        KMC_TRY(srv.progress(&moved));
        for (; seen < srv.finished_log.size(); ++seen) {
            const int64_t id = srv.finished_log[seen];
            const Server::Ticket &t = *srv.tickets[(size_t)id];
            kmc_serve_result_t &o = out[(size_t)req_of[(size_t)id]];
            o.admit_s = t.admit_s;
            o.finish_s = t.finish_s;
            o.n_iter = t.n_iter;
            o.inertia = t.inertia;
            o.status = t.status;
            ++finished;
        }
        if (!moved && finished < n_req) {
            double wait = 20e-6;
            if (srv.running.empty() && srv.pending.empty() && next < n_req)
                wait = std::min(std::max(rq[next].arrival_s - srv.elapsed(), 0.0), 0.001);
            if (wait > 0)
                std::this_thread::sleep_for(std::chrono::microseconds((int64_t)(wait * 1e6)));
        }
    }
    if (makespan) *makespan = srv.elapsed();
    return KMC_OK;
}

}  // namespace serving


}  // namespace kmc

using namespace kmc;

struct kmc_batch_s {
    BatchEngine eng;
};

struct kmc_server_s {
    serving::Server srv;
};

extern "C" {

int kmc_batch_create(int64_t max_instances, kmc_stream_t stream, kmc_batch_t *batch_out) {
    KMC_CHECK_ARG(batch_out != nullptr, "null output handle");
    auto b = std::make_unique<kmc_batch_s>();
    KMC_TRY(b->eng.init(max_instances, reinterpret_cast<cudaStream_t>(stream)));
    *batch_out = b.release();
    return KMC_OK;
}

int kmc_batch_add_fit_f32(kmc_batch_t batch, const float *X_t, const float *sample_weight,
                          float *centroids_t, int32_t *labels, int64_t n_samples,
                          int64_t n_features, int64_t n_clusters, double tol, int64_t max_iter,
                          int64_t *instance_out) {
    KMC_CHECK_ARG(batch != nullptr && instance_out != nullptr, "null argument");
    KMC_CHECK_ARG(max_iter >= 0, "max_iter must be non-negative");
    return batch->eng.add(B_FIT, X_t, sample_weight, centroids_t, labels, n_samples, n_features,
                          n_clusters, tol, max_iter, instance_out);
}

int kmc_batch_add_predict_f32(kmc_batch_t batch, const float *X_t, const float *centroids_t,
                              int32_t *labels, int64_t n_samples, int64_t n_features,
                              int64_t n_clusters, int64_t *instance_out) {
    KMC_CHECK_ARG(batch != nullptr && instance_out != nullptr, "null argument");
    return batch->eng.add(B_ASSIGN, X_t, nullptr, const_cast<float *>(centroids_t), labels,
                          n_samples, n_features, n_clusters, 0.0, 0, instance_out);
}

int kmc_batch_add_transform_f32(kmc_batch_t batch, const float *X_t, const float *centroids_t,
                                float *distances, int64_t n_samples, int64_t n_features,
                                int64_t n_clusters, int64_t *instance_out) {
    KMC_CHECK_ARG(batch != nullptr && instance_out != nullptr, "null argument");
    KMC_CHECK_ARG(distances != nullptr || n_samples == 0, "null distances");
    return batch->eng.add(B_TRANSFORM, X_t, nullptr, const_cast<float *>(centroids_t), nullptr,
                          n_samples, n_features, n_clusters, 0.0, 0, instance_out, distances);
}

int kmc_batch_step(kmc_batch_t batch, int64_t *n_active_out) {
    KMC_CHECK_ARG(batch != nullptr, "null batch");
    return batch->eng.step(n_active_out);
}

int kmc_batch_run(kmc_batch_t batch) {
    kmc::Range range("kmc.batch_run");
    KMC_CHECK_ARG(batch != nullptr, "null batch");
    int64_t active = 1;
    while (active > 0) KMC_TRY(batch->eng.step(&active));
    return KMC_OK;
}

int kmc_batch_result(kmc_batch_t batch, int64_t instance, int *finished_out,
                     int64_t *n_iter_out, double *inertia_out) {
    KMC_CHECK_ARG(batch != nullptr, "null batch");
    BatchEngine &e = batch->eng;
    KMC_CHECK_ARG(instance >= 0 && instance < e.cap && e.state[(size_t)instance] != 0,
                  "no such instance");
    if (finished_out) *finished_out = e.state[(size_t)instance] == BatchEngine::FINISHED;
    if (n_iter_out) *n_iter_out = e.res_iter[(size_t)instance];
    if (inertia_out) *inertia_out = e.res_inertia[(size_t)instance];
    return KMC_OK;
}

int kmc_batch_remove(kmc_batch_t batch, int64_t instance) {
    KMC_CHECK_ARG(batch != nullptr, "null batch");
    return batch->eng.remove(instance);
}

int kmc_batch_stats(kmc_batch_t batch, int64_t *steps_out, int64_t *graph_builds_out,
                    int64_t *relocations_out) {
    KMC_CHECK_ARG(batch != nullptr, "null batch");
    if (steps_out) *steps_out = batch->eng.steps;
    if (graph_builds_out) *graph_builds_out = batch->eng.graph_builds;
    if (relocations_out) *relocations_out = batch->eng.relocations;
    return KMC_OK;
}

int kmc_batch_destroy(kmc_batch_t batch) {
    if (batch == nullptr) return KMC_OK;
    cudaStreamSynchronize(batch->eng.s);
    delete batch;
    return KMC_OK;
}

int kmc_tile_variant(int64_t n_features, int64_t n_clusters, kmc_stream_t stream,
                     int *variant_out) {
    KMC_CHECK_ARG(variant_out != nullptr, "null output");
    KMC_CHECK_ARG(n_features >= 1 && n_features <= 1024 && n_clusters >= 1 && n_clusters <= 4096,
                  "n_features / n_clusters out of range");
    return tune_variant(n_features, n_clusters, reinterpret_cast<cudaStream_t>(stream),
                        variant_out);
}

int kmc_generate_blobs_f32(float *X_t, int64_t n_samples, int64_t n_features,
                           int64_t n_centers, float box_lo, float box_hi, float std_lo,
                           float std_hi, uint64_t seed, kmc_stream_t stream) {
    KMC_CHECK_ARG(n_samples >= 0 && n_features >= 0, "negative dimension");
    return launch_blobs(X_t, n_samples, n_features, n_centers, box_lo, box_hi, std_lo, std_hi,
                        seed, reinterpret_cast<cudaStream_t>(stream));
}

int kmc_debug_batch_items(int64_t count, const int64_t *n_samples, const int *modes,
                          const int *variants, int64_t capacity, int32_t *instance_out,
                          int32_t *tiles_out, int64_t *first_tile_out, int32_t *group_out,
                          int64_t *n_items_out) {
    KMC_CHECK_ARG(count >= 0 && n_items_out != nullptr, "invalid arguments");
    KMC_CHECK_ARG(count == 0 || (n_samples && modes && variants), "null input");
    std::vector<kmc::BItem> items[2][kmc::kBatchVariants];
    for (int64_t q = 0; q < count; ++q) {
        KMC_CHECK_ARG(n_samples[q] >= 0 && variants[q] >= 0 && variants[q] < kmc::kBatchVariants &&
                          modes[q] >= kmc::B_FIT && modes[q] <= kmc::B_TRANSFORM,
                      "invalid instance %lld", (long long)q);
        kmc::append_items((int)q, n_samples[q], modes[q], variants[q], items);
    }
    int64_t total = 0;
    for (int kind = 0; kind < 2; ++kind)
        for (int v = 0; v < kmc::kBatchVariants; ++v) {
            for (const kmc::BItem &it : items[kind][v]) {
                if (total < capacity) {
                    instance_out[total] = it.inst;
                    tiles_out[total] = it.ntiles;
                    first_tile_out[total] = it.tile0;
                    group_out[total] = kind * kmc::kBatchVariants + v;
                }
                ++total;
            }
        }
    *n_items_out = total;
    return KMC_OK;
}

int kmc_seeded_rows(int64_t n_samples, int64_t n_clusters, uint64_t seed, int32_t *rows_out) {
    KMC_CHECK_ARG(rows_out != nullptr, "null output");
    KMC_CHECK_ARG(n_clusters >= 0 && n_clusters <= n_samples, "n_clusters exceeds n_samples");
    std::vector<int32_t> r;
    seeded_rows(n_samples, n_clusters, seed, &r);
    std::memcpy(rows_out, r.data(), sizeof(int32_t) * r.size());
    return KMC_OK;
}

int kmc_serve_bytes_needed(int32_t kind, int64_t n_samples, int64_t n_features,
                           int64_t n_clusters, int form, int64_t *bytes_out) {
    KMC_CHECK_ARG(bytes_out != nullptr, "null output");
    KMC_CHECK_ARG(kind >= 0 && kind <= 2, "kind must be 0 (fit), 1 (predict) or 2 (transform)");
    KMC_CHECK_ARG(n_samples >= 0 && n_features >= 1 && n_clusters >= 1, "invalid sizes");
    *bytes_out = serving::request_bytes(kind, n_samples, n_features, n_clusters, form);
    return KMC_OK;
}

int kmc_server_open(int form, int64_t hbm_budget_bytes, int64_t max_active, kmc_stream_t stream,
                    kmc_server_t *server_out) {
    KMC_CHECK_ARG(server_out != nullptr, "null output handle");
    auto srv = std::make_unique<kmc_server_s>();
    KMC_TRY(srv->srv.init(form, hbm_budget_bytes, max_active,
                          reinterpret_cast<cudaStream_t>(stream)));
    *server_out = srv.release();
    return KMC_OK;
}

int kmc_server_submit_fit_f32(kmc_server_t server, const float *X_t, const float *sample_weight,
                              const float *init_centroids_t, int32_t *labels_out,
                              float *centroids_out, int64_t n_samples, int64_t n_features,
                              int64_t n_clusters, double tol, int64_t max_iter,
                              int64_t *ticket_out) {
    KMC_CHECK_ARG(server != nullptr && ticket_out != nullptr, "null argument");
    KMC_CHECK_ARG(n_samples >= 1 && n_features >= 1 && n_clusters >= 1,
                  "invalid sizes (n=%lld, d=%lld, k=%lld)", (long long)n_samples,
                  (long long)n_features, (long long)n_clusters);
    KMC_CHECK_ARG(n_clusters <= n_samples, "n_clusters exceeds n_samples");
    KMC_CHECK_ARG(n_samples < (int64_t(1) << 31), "n_samples must fit int32 labels");
    KMC_CHECK_ARG(tol >= 0.0, "Tolerance must be non-negative");
    KMC_CHECK_ARG(max_iter >= 0, "max_iter must be non-negative");
    KMC_CHECK_ARG(X_t != nullptr && sample_weight != nullptr && init_centroids_t != nullptr &&
                      labels_out != nullptr && centroids_out != nullptr,
                  "null buffer");
    KMC_TRY(serving::check_shape(server->srv.form, n_features, n_clusters));
    auto t = std::make_unique<serving::Server::Ticket>();
    t->kind = 0;
    t->n = n_samples;
    t->d = n_features;
    t->k = n_clusters;
    t->tol = tol;
    t->max_iter = max_iter;
    t->X = X_t;
    t->w = sample_weight;
    t->Cinit = init_centroids_t;
    t->labels = labels_out;
    t->Cout = centroids_out;
    return server->srv.submit(std::move(t), ticket_out);
}

// Predictions and transforms against the model of an earlier fit ticket.
static int submit_with_model(kmc_server_t server, int kind, const float *X_t,
                             int64_t model_ticket, int32_t *labels_out, float *distances_out,
                             int64_t n_samples, int64_t *ticket_out) {
    KMC_CHECK_ARG(server != nullptr && ticket_out != nullptr, "null argument");
    KMC_CHECK_ARG(n_samples >= 1 && n_samples < (int64_t(1) << 31), "invalid n_samples");
    KMC_CHECK_ARG(X_t != nullptr, "null buffer");
    const serving::Server::Ticket *m = server->srv.get(model_ticket);
    KMC_CHECK_ARG(m != nullptr && m->kind == 0, "model_ticket %lld is not a fit of this server",
                  (long long)model_ticket);
    auto t = std::make_unique<serving::Server::Ticket>();
    t->kind = kind;
    t->n = n_samples;
    t->d = m->d;
    t->k = m->k;
    t->model = model_ticket;
    t->X = X_t;
    t->labels = labels_out;
    t->dist = distances_out;
    return server->srv.submit(std::move(t), ticket_out);
}

int kmc_server_submit_predict_f32(kmc_server_t server, const float *X_t, int64_t model_ticket,
                                  int32_t *labels_out, int64_t n_samples, int64_t *ticket_out) {
    KMC_CHECK_ARG(labels_out != nullptr, "null labels");
    return submit_with_model(server, 1, X_t, model_ticket, labels_out, nullptr, n_samples,
                             ticket_out);
}

int kmc_server_submit_transform_f32(kmc_server_t server, const float *X_t, int64_t model_ticket,
                                    float *distances_out, int64_t n_samples,
                                    int64_t *ticket_out) {
    KMC_CHECK_ARG(distances_out != nullptr, "null distances");
    return submit_with_model(server, 2, X_t, model_ticket, nullptr, distances_out, n_samples,
                             ticket_out);
}

static void ticket_result(const serving::Server::Ticket &t, int *status_out, int64_t *n_iter_out,
                          double *inertia_out) {
    if (status_out) *status_out = t.status;
    if (n_iter_out) *n_iter_out = t.n_iter;
    if (inertia_out) *inertia_out = t.inertia;
}

int kmc_server_poll(kmc_server_t server, int64_t ticket, int *state_out, int *status_out,
                    int64_t *n_iter_out, double *inertia_out) {
    KMC_CHECK_ARG(server != nullptr, "null server");
    KMC_CHECK_ARG(server->srv.get(ticket) != nullptr, "no such ticket %lld", (long long)ticket);
    bool moved = false;
    KMC_TRY(server->srv.progress(&moved));
    const serving::Server::Ticket &t = *server->srv.get(ticket);
    if (state_out) *state_out = t.state;
    ticket_result(t, status_out, n_iter_out, inertia_out);
    return KMC_OK;
}

int kmc_server_wait(kmc_server_t server, int64_t ticket, int *status_out, int64_t *n_iter_out,
                    double *inertia_out) {
    KMC_CHECK_ARG(server != nullptr, "null server");
    KMC_TRY(server->srv.wait(ticket));
    ticket_result(*server->srv.get(ticket), status_out, n_iter_out, inertia_out);
    return KMC_OK;
}

int kmc_server_cancel(kmc_server_t server, int64_t ticket) {
    KMC_CHECK_ARG(server != nullptr, "null server");
    return server->srv.cancel(ticket);
}

int kmc_server_release(kmc_server_t server, int64_t ticket) {
    KMC_CHECK_ARG(server != nullptr, "null server");
    return server->srv.release(ticket);
}

int kmc_server_stats(kmc_server_t server, int64_t *pending_out, int64_t *running_out,
                     int64_t *bytes_in_use_out) {
    KMC_CHECK_ARG(server != nullptr, "null server");
    if (pending_out) *pending_out = (int64_t)server->srv.pending.size();
    if (running_out) *running_out = (int64_t)server->srv.running.size();
    if (bytes_in_use_out) *bytes_in_use_out = server->srv.in_use;
    return KMC_OK;
}

int kmc_server_close(kmc_server_t server) {
    if (server == nullptr) return KMC_OK;
    int rc = KMC_OK;
    // requests not yet finished are cancelled; running ones stop after the
    // work they have in flight
    for (auto &t : server->srv.tickets)
        if (!serving::Server::final_state(t->state)) t->cancel = true;
    while (rc == KMC_OK && (!server->srv.running.empty() || !server->srv.pending.empty())) {
        bool moved = false;
        rc = server->srv.progress(&moved);
        if (!moved) std::this_thread::sleep_for(std::chrono::microseconds(20));
    }
    delete server;
    return rc;
}

int kmc_serve_run(const kmc_serve_request_t *requests, int64_t n_requests, int form,
                  int64_t hbm_budget_bytes, int64_t max_active, kmc_stream_t stream,
                  kmc_serve_result_t *results_out, double *makespan_s_out) {
    return serving::serve_run(requests, n_requests, form, hbm_budget_bytes, max_active,
                     reinterpret_cast<cudaStream_t>(stream), results_out, makespan_s_out);
}

}  // extern "C"
