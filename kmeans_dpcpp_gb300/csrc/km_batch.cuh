// Batched Lloyd engine: many independent float32 fits and label-only
// predictions of uneven (n, d, k) advanced together, one iteration per step.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "km_fit.cuh"
#include "km_kernels.cuh"

namespace kmc {

enum BatchMode : int { B_FIT = 0, B_ASSIGN = 1, B_TRANSFORM = 2 };

// Device table entry of one instance.  X, w, C and labels are the caller's
// arrays (C is the caller's initial-centroid buffer and is overwritten, as in
// the driver); everything else is owned by the engine.
struct BInst {
    const float *X;        // (d, n) feature-major
    const float *w;        // (n,)
    float *C;              // (d, k) current centroids
    float *Cn;             // (d, k) float32 sums, then the next centroids
    float *hn;             // (k,) half squared norms of C
    float *sizes;          // (k,) float32 cluster sizes
    double *sums;          // (d*k + k,) float64 sums (f*k + j), then sizes
    int32_t *labels;       // (n,)
    float *dist;           // (k, n) distances (B_TRANSFORM)
    int32_t *empty_list;   // (k + 1,) ascending list, count at [k]
    long long n;
    int d, k;
    int mode;              // B_FIT or B_ASSIGN
    int variant;           // centroid-window width: 0 -> 32, 1 -> 64, 2 -> 128
    int copies;            // private copies of sums (CTA b adds into copy b % copies)
    LoopState st;          // done / n_iter / max_iter / tol / last_shift
};

// One work item: a run of 128-sample tiles of one instance.
struct BItem {
    int inst;
    int ntiles;
    long long tile0;
};

constexpr int kBatchVariants = 3;
constexpr int kBatchTileM = 128;

int batch_variant_width(int v);
// Private global copies of an instance's float64 sums: small sums get several
// (their few addresses would serialise the reductions of many CTAs).
int batch_sum_copies(int64_t d, int64_t k);
// Dynamic shared memory of one assign CTA of variant v.
size_t batch_assign_smem(int v);

// ---- launchers (batch.cu) ----
int launch_batch_prep(BInst *tab, const int *idx, int count, int *counters, cudaStream_t s);
// Sets the assign kernels' shared-memory attributes (outside graph capture).
int prepare_batch_assign();
// dist != 0: the transform kernel (items of B_TRANSFORM instances only).
int launch_batch_assign(int variant, int dist, const BInst *tab, const BItem *items,
                        int n_items, int *counter, cudaStream_t s);
int launch_batch_reduce(BInst *tab, const int *idx, int count, int *n_empty_out,
                        cudaStream_t s);
int launch_batch_update(BInst *tab, const int *idx, int count, int *done_out, cudaStream_t s);
int launch_blobs(float *X, int64_t n, int64_t d, int64_t n_centers, float box_lo,
                 float box_hi, float std_lo, float std_hi, uint64_t seed, cudaStream_t s);
int launch_gather_rows(const float *X, int64_t n, int64_t d, const int32_t *idx, int64_t k,
                       float *C, cudaStream_t s);

// Seeded distinct row indices (k <= n): (a*j + b) mod n with gcd(a, n) = 1.
void seeded_rows(int64_t n, int64_t k, uint64_t seed, std::vector<int32_t> *out);

// Tile autotuner: the fastest assign variant for (d, k, float32), measured on
// a synthetic instance of (d, k rounded up to a power of two) and cached in
// memory and in a text file
// (KMC_TILE_CACHE, else $XDG_CACHE_HOME or $HOME/.cache/kmeans_gb300/tiles.txt).
int tune_variant(int64_t d, int64_t k, cudaStream_t s, int *variant);

}  // namespace kmc
