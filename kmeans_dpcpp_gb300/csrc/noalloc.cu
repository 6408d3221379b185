// Allocation-free variant of select_samples_far_from_centroid (float32
// distances, int32 indices).
//
// The ordered selection needs scratch: a header, per-block counts and the
// list of strictly-greater samples that gets ranked, 256 + 2 * 8 * 512 +
// 8 * n_selected bytes.  kmc_select_samples_far_from_centroid_f32_i32 takes
// it from the stream-ordered allocator on every call; this variant keeps it
// in one file-scope device array sized for n_selected <= 4096 (41,216 bytes),
// so a call makes no allocation of any kind.  Nothing in the scratch has to
// start at zero: every word a kernel reads was written earlier in the same
// call (block counts by the count kernel, the header by the scan kernel, the
// list entries by the write kernel).
//
// The array is one per device and shared by every call on that device: two
// calls whose kernels overlap (different streams, or different host threads)
// race on it.  The first call on a device looks up the array's address with
// cudaGetSymbolAddress (which may load this module onto the device); make
// that first call before capturing a stream into a graph.  The address is
// kept together with the unique id of the context it belongs to: after a
// device reset (a new primary context, the module loaded again) the next call
// looks the address up again instead of using the old one.
#include <mutex>

#include "km_kernels.cuh"
#include "kmeans_gb300.h"

namespace kmc {
namespace {

constexpr int64_t kNoAllocMaxSelected = 4096;
constexpr size_t kNoAllocScratchBytes = 41216;  // 256 + 2*8*512 + 8*4096, 256-aligned

static __device__ __align__(256) unsigned char g_select_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
struct ScratchAddr {
    unsigned long long ctx_id;  // context the address belongs to
    void *ptr;
};
ScratchAddr g_scratch[kMaxDevices] = {};

// Unique id (over the life of the process) of the calling thread's current
// context, through the driver entry points the runtime exposes; 0 if unknown.
unsigned long long current_context_id() {
    using GetCurrentFn = int (*)(void **);
    using GetIdFn = int (*)(void *, unsigned long long *);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(f);
        (void)cudaGetLastError();
    });
    void *ctx = nullptr;
    unsigned long long id = 0;
    if (get_current == nullptr || get_id == nullptr || get_current(&ctx) != 0 || ctx == nullptr ||
        get_id(ctx, &id) != 0)
        return 0;
    return id;
}

// Address of this device's scratch array; the device must be current.  It is
// looked up once per device and context.
int scratch_for_current_device(void **out) {
    int dev = -1;
    KMC_CUDA_TRY(cudaGetDevice(&dev));
    KMC_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "device ordinal %d is out of range", dev);
    // 0 when no context is current on this thread yet: the lookup below then
    // makes the device's primary context current
    const unsigned long long ctx = current_context_id();
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    ScratchAddr &a = g_scratch[dev];
    if (a.ptr == nullptr || ctx == 0 || a.ctx_id != ctx) {
        void *p = nullptr;
        KMC_CUDA_TRY(cudaGetSymbolAddress(&p, g_select_scratch));
        a.ptr = p;
        a.ctx_id = current_context_id();
    }
    *out = a.ptr;
    return KMC_OK;
}

}  // namespace
}  // namespace kmc

extern "C" int kmc_select_samples_far_from_centroid_noalloc_f32_i32(
    int64_t n_selected, const float *distance_to_centroid, const float *threshold,
    int32_t *selected_samples_idx, int32_t *n_selected_gt_threshold,
    int32_t *n_selected_eq_threshold, int64_t n_samples, int64_t work_group_size,
    kmc_stream_t stream) {
    using namespace kmc;
    (void)work_group_size;
    KMC_CHECK_ARG(n_samples >= 0, "array dimensions must be non-negative");
    KMC_CHECK_ARG(n_selected > 0, "Argument `n_selected` must be positive");
    KMC_CHECK_ARG(n_selected <= n_samples, "Argument `n_select` is too large");
    KMC_CHECK_ARG(n_selected <= kNoAllocMaxSelected,
                  "n_selected (%lld) exceeds %lld, the most the allocation-free selection "
                  "holds in its static scratch; use "
                  "kmc_select_samples_far_from_centroid_f32_i32",
                  (long long)n_selected, (long long)kNoAllocMaxSelected);
    KMC_CHECK_ARG(select_scratch_bytes(n_selected) <= kNoAllocScratchBytes,
                  "static selection scratch is too small");
    void *scratch = nullptr;
    KMC_TRY(scratch_for_current_device(&scratch));
    return launch_select<float, int32_t>(nullptr, n_selected, distance_to_centroid, threshold,
                                         selected_samples_idx, n_selected_gt_threshold,
                                         n_selected_eq_threshold, n_samples, scratch, n_selected,
                                         reinterpret_cast<cudaStream_t>(stream));
}
