// Mixed-precision Lloyd step on the sm_103a tensor cores (tcgen05 + TMEM).
//
// The assignment needs, for each sample x and centroid c_j, the reference's
// pseudo-distance D_j = half_norm[j] - x.c_j (src/device_functions.hpp:
// 106-162).  Here the score s_j = sigma^2 (x.c_j - hn_j) is produced entirely
// by the tensor cores: the contraction over the features runs with fp16 (or
// bf16) operands and fp32 accumulation, and one more K=16 MMA per chunk adds
// -hn_j, split into three 16-bit parts against constant columns
// (-2^10, -1, -2^-10), so TMEM holds finished scores.  For every sample the
// epilogue finds the best score M and an exact bound on the runner-up R
// without sorting (see "runner-up" below).  A sample whose margin M - R
// exceeds twice its error bound E_i is certified: no rounding of the
// operands, of the tensor-core accumulation or of the reference's own fp32
// evaluation can change its winner, so its label equals the reference's.
// Every other sample is re-evaluated in exact fp32 reference arithmetic over
// the few centroids that can still win (recheck kernel), so labels never
// drift from the plain form.
//
// Error bound (unscaled units; operands scaled by a global power of two
// sigma and rounded to 16 bits: sigma x + dX_i and sigma c_j + dC_j, where the
// rounding errors dX_i, dC_j are exact in fp32 and measured, subnormals
// included; u = 2^-11 for fp16, 2^-8 for bf16; d features):
//   E_i = ||x_i|| alpha + ||dX_i|| / sigma beta1 + beta0
//   alpha = dCmax + 2^-16 (Cmax + dCmax) + (d + 4) 2^-23 Cmax
//   beta1 = (Cmax + dCmax)(1 + 2^-16)
//   beta0 = Hmax (u^3 + 2^-16 + 2^-23) + hfloor
// with Cmax = max_j ||c_j||, dCmax = max_j ||dC_j|| / sigma, Hmax = max_j
// |hn_j|.  By Cauchy-Schwarz |(sigma x + dX).(sigma c + dC) - sigma^2 x.c| <=
// ||dX|| (||sigma c|| + ||dC||) + ||sigma x|| ||dC||: the measured rounding
// errors (about 0.4 u ||.|| for random data) replace the worst case u ||.||
// of each operand.  The bound also covers the three-part split of the half
// norms (u^3, plus subnormal parts hfloor), tensor-core fp32 accumulation
// (<= 2^-17 relative to the sum of magnitudes, allowing truncation), and the
// reference's sequential fp32 dot (d 2^-24) and final subtraction; for bf16,
// whose subnormal inputs the tensor cores may flush, 2^-126 sqrt(d) (1 + u)
// is added to alpha and that times Cmax to beta0.  All norms are rounded up.
// sigma keeps |x sigma| <= 2^14 and sigma^2 * hn <= 2^25 so every 16-bit part
// is finite.
//
// Runner-up without sorting: per sample, P1[s] = max over 32-column
// sub-chunk s and P2[t] = max over columns j = t (mod 32).  Two distinct
// columns in the same sub-chunk lie in different classes, so
//   runner-up = max(second largest P1, second largest P2),
// and the winner is (argmax P1) * 32 + argmax P2 whenever the maximum is
// unique (otherwise the margin is zero and the sample is rechecked).
//
// Kernel roles (one CTA of 384 threads per SM, persistent over 128-sample
// tiles; 12 warps leave 168 registers per thread, so nothing spills):
//   warp 0      bulk copies: the centroid image once, X tiles into a 2-4 stage ring
//   warp 1      TMEM allocation; one thread issues tcgen05.mma (M=128, N=256,
//               K=16) into two 256-column TMEM accumulators
//   warps 2-9   epilogue: tcgen05.ld of score pairs, P1/P2, certification, labels
//   warps 10-11 update: w*x of certified samples into cluster-major sums.
//               d > 32: fire-and-forget red.global.add.v4.f32 into the
//               private copy of this CTA (copy blockIdx % n_copies), summed in
//               copy order afterwards.  d <= 32: integer (fixed-point) sums
//               in shared memory from terms packed once per fit, added at the
//               end into order-independent integer totals (fixed_sums_role);
//               when those sums do not fit shared memory,
//               red.global.add.f64 per feature into the CTA's copy
// Samples that fail certification are accumulated by the recheck kernel.
// Waits poll mbarrier.test_wait (no suspension: with tensor-core kernels of
// several streams at once, suspended waiters sometimes slept for seconds).
//
// Every wait is bounded.  A wait that runs out raises the CTA's error flag;
// the other roles see it and stop, the producer and the MMA issuer then wait
// (ignoring the flag) for the copies and tensor-core operations they already
// issued, TMEM is freed, and the fit's loop state records the error and stops
// the loop, so the host gets KMC_ERR_DEVICE_TIMEOUT and the context stays
// usable.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "km_batch.cuh"
#include "km_fit.cuh"
#include "km_mixed.cuh"

namespace kmc {

namespace {

using namespace tc;

constexpr int kTileM = 128;
constexpr int kChunkN = 256;
constexpr uint32_t kNormRowBytes = 32;  // K=16 block holding the half-norm parts
constexpr int kEpiWarps = 8;
constexpr int kUpdWarps = 2;
constexpr int kUpdThreads = 32 * kUpdWarps;  // each handles rows u and u + 64 of a tile
constexpr int kThreadsMixed = 32 * (2 + kEpiWarps + kUpdWarps);
constexpr int kMaxChunks = 4;   // 256-column chunks per pass (k <= 1024)
constexpr uint32_t kTileBytes = kTileM * 128;  // one 64-wide K block of a tile
constexpr size_t kSmemLimit = 232448;

struct MixedConsts {
    float s2;       // sigma^2 (scores in TMEM are sigma^2 (x.c - hn))
    float alpha;    // E_i = nx_i * alpha + ndx_i * beta1 + beta0
    float beta1;
    float beta0;
    float sigma;
    unsigned int xmax_bits;  // max |x| (fp32 bits)
    int overflow;            // an operand left the 16-bit range this pass
    unsigned int wmax_bits;  // max |w| (fp32 bits; fixed-point sums only)
    int fx_shift;            // w x and w are summed as the integers w x 2^fx_shift, w 2^fx_shift
    int fx_ok;               // the fixed-point sums may be used (finite bounds)
};

// Order-independent totals of the fixed-point sums (d <= 32): element e
// (cluster-major [k][d4] sums, then the k sizes) of copy c is
// hi[c stride + e] 2^32 + lo[c stride + e]; contributions q are added as
// (q >> 32) into hi and (q mod 2^32) into lo with 64-bit integer atomics (the
// copies, CTA b into copy b mod copies, spread the contention), and the copies
// are added as integers, so every order gives the same bits.  xq: the packed
// terms ([n][d4 + 4]); null when not in use.
struct FxAcc {
    const int *xq;
    long long *hi;
    unsigned long long *lo;
    int64_t stride;  // elements per copy
    int copies;
    // the copy of block b
    __device__ __forceinline__ FxAcc copy_of(unsigned b) const {
        FxAcc r = *this;
        if (hi != nullptr) {
            const int64_t o = (int64_t)(b % (unsigned)copies) * stride;
            r.hi += o;
            r.lo += o;
        }
        return r;
    }
};

__device__ __forceinline__ void fx_add(const FxAcc &fx, int64_t e, long long q) {
    atomicAdd(reinterpret_cast<unsigned long long *>(fx.hi + e), (unsigned long long)(q >> 32));
    atomicAdd(fx.lo + e, (unsigned long long)(q & 0xffffffffll));
}

// Sample i (label c) into the integer totals of fx (this block's copy): its
// packed terms w x_j (j < d4) and w; a flagged term (not representable) goes
// as its exact float value into the float64 copy acc64 ([k_pad][d4] sums,
// then k_pad sizes).
__device__ __forceinline__ void add_packed_row(const FxAcc &fx, double *acc64, int64_t k_pad,
                                               int64_t k, int64_t d4, const float *xrow,
                                               const float *w, int64_t i, int64_t c) {
    const int64_t ds = d4 + 4;
    const float wv = w[i];
    for (int64_t j = 0; j <= d4; ++j) {
        const int pk = fx.xq[i * ds + j];
        if (pk == 1) {
            const float v = j < d4 ? __fmul_rn(xrow[i * d4 + j], wv) : wv;
            atomicAdd(j < d4 ? acc64 + c * d4 + j : acc64 + k_pad * d4 + c, (double)v);
        } else if (pk != 0) {
            fx_add(fx, j < d4 ? c * d4 + j : k * d4 + c,
                   (long long)(pk >> 6) * (1ll << ((pk >> 1) & 31)));
        }
    }
}

struct MixedArgs {
    const uint8_t *ximg;
    const uint8_t *cimg;
    const float *nx;
    const float *ndx;   // ||operand rounding error of x_i|| / sigma, rounded up
    const MixedConsts *consts;
    const float *X;
    const float *w;
    void *labels;
    // Cluster sums in n_copies private copies ([copy][k_pad*d4 + k_pad]:
    // cluster-major sums, then sizes; CTA b uses copy b % n_copies), reduced
    // in a fixed order afterwards.
    float *sums32;     // fp32 copies (vector-red path)
    double *acc64;     // fp64 copies (acc_f64 path)
    int n_copies;
    const float *xrow; // [n][d4] row-major fp32 copy of X (update and recheck)
    uint4 *cand;
    int *flagged;
    int *n_flagged;
    int *err_global;
    const LoopState *guard;
    int64_t n, d, k, k_pad, d4;
    int update;
    int label64;
    int acc_f64;       // red.global.add.f64 per feature (else red.global.add.v4.f32)
    int stages;        // depth of the X-tile ring
    long long wait_limit;  // SM clocks after which a wait gives up
    int stall;         // test of the timeout path: the epilogue first waits on a
                       // barrier that nothing completes
    LoopState *state;  // receives the error bit and stops the loop (nullable)
    // Column passes (n_clusters beyond what one launch holds in shared
    // memory): this launch covers columns col0 .. col0 + NCH*256 - 1 of a
    // global centroid image of k_img rows.  With multi set it writes, per
    // sample, its best score of the pass (pmax) and full candidate masks of
    // the pass (cand) instead of labels; a combine kernel decides.
    int64_t k_img, col0;
    int multi;
    float *pmax;
    // > 0: the sums of own_k clusters are accumulated per CTA in shared memory
    // (fixed point), own_f packed columns per update thread
    int64_t own_k;
    int own_f;
    const int *xq;  // [n][d4 + 4] packed fixed-point terms (w x, then w, 0, 0, 0)
    FxAcc fx;       // their order-independent totals
};

// Fixed-point sums: each of the 64 update threads adds own_f consecutive
// columns of its rows, w columns / own_f threads per row, so the rows are
// split into (and the sums kept in) this many groups.
__host__ __device__ constexpr int fx_copies(int64_t w, int own_f) {
    return (int)(kUpdThreads / (w / own_f));
}

struct SmemLayout {
    size_t c, hnb, aon, x, xch, lab, bar, p1, osum, ostage, ocode, ow, total;
};

// Sub-chunk maxima stay in registers up to two chunks; beyond that they go
// to shared memory (registers would spill).
__host__ __device__ constexpr bool p1_in_smem(int64_t nch) { return nch >= 3; }

// c:    centroid image, NKB blocks of k_pad x 128 bytes (128-byte swizzle)
// hnb:  half-norm parts, k_pad x 32 bytes (32-byte swizzle); c and hnb are
//       one contiguous copy of the global centroid image
// aon:  constant A block (128 x 32 bytes): columns 0..2 = -2^10, -1, -2^-10
// x:    X-tile ring (stages x NKB x 16 KB)
// xch:  per-row maxima of the two column halves (two tiles in flight)
// lab:  labels / recheck slots handed to the update warps (two tiles)
// p1:   sub-chunk maxima, [sub-chunk][256 epilogue threads] (3+ chunks)
// osum: the CTA's fixed-point cluster sums and sizes, R copies of
//       [own_k + 1][d4 + 4] (int64), R = fx_copies(d4 + 4, own_f); ostage /
//       ocode: a tile's packed rows and labels handed between the two update
//       warps (fixed-point sums only)
__host__ __device__ inline SmemLayout smem_layout(int nkb, int64_t k_pad, int64_t d4,
                                                  int stages, int64_t own_k = 0,
                                                  int own_f = 1) {
    SmemLayout L;
    size_t off = 0;
    L.c = off;
    off += (size_t)nkb * k_pad * 128;
    L.hnb = off;
    off += (size_t)k_pad * kNormRowBytes;
    off = (off + 1023) & ~size_t(1023);
    L.aon = off;
    off += (size_t)kTileM * kNormRowBytes;
    off = (off + 1023) & ~size_t(1023);
    L.x = off;
    off += (size_t)stages * nkb * kTileBytes;
    L.xch = off;
    off += sizeof(float) * 2 * 2 * kTileM;
    L.lab = off;
    off += sizeof(int) * 2 * kTileM;
    off = (off + 15) & ~size_t(15);
    L.bar = off;
    off += 8 * 19 + 16;
    off = (off + 15) & ~size_t(15);
    L.p1 = off;
    if (p1_in_smem(k_pad / kChunkN)) off += sizeof(float) * 32 * kEpiWarps * (size_t)(k_pad / 64);
    off = (off + 15) & ~size_t(15);
    L.osum = off;
    L.ostage = L.ocode = L.ow = off;
    if (own_k > 0) {
        // R copies of [own_k + 1][d4 + 4] (the last cluster row takes rows
        // without a certified label)
        off += sizeof(long long) * (size_t)fx_copies(d4 + 4, own_f) * (size_t)(own_k + 1) *
               (size_t)(d4 + 4);
        L.ostage = off;
        off += sizeof(int) * kTileM * (size_t)(d4 + 4);
        L.ocode = off;
        off += sizeof(int) * kTileM;
        L.ow = off;
    }
    L.total = off + 1024;  // slack for aligning the dynamic shared memory base
    return L;
}

// Bytes of the global centroid image (128-byte-swizzled blocks + norm parts).
__host__ __device__ inline size_t cimg_bytes(int nkb, int64_t k_pad) {
    return (size_t)nkb * k_pad * 128 + (size_t)k_pad * kNormRowBytes;
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

__device__ __forceinline__ float u2f(uint32_t v) { return __uint_as_float(v); }

// Maximum of 32 scores (16 three-input max operations).
__device__ __forceinline__ float max32(const uint32_t (&r)[32]) {
    float m[11];
#pragma unroll
    for (int u = 0; u < 10; ++u) m[u] = max3f(u2f(r[3 * u]), u2f(r[3 * u + 1]), u2f(r[3 * u + 2]));
    m[10] = fmaxf(u2f(r[30]), u2f(r[31]));
    const float a = max3f(m[0], m[1], m[2]);
    const float b = max3f(m[3], m[4], m[5]);
    const float c = max3f(m[6], m[7], m[8]);
    return fmaxf(max3f(a, b, c), fmaxf(m[9], m[10]));
}

// tcgen05.ld writes its registers asynchronously; after tcgen05.wait::ld the
// empty asm statements (ordered after the wait like every volatile asm) make
// each later use of the registers depend on the wait.
__device__ __forceinline__ void tmem_ld_wait_regs(uint32_t (&r0)[32], uint32_t (&r1)[32]) {
    tmem_ld_wait();
#pragma unroll
    for (int t = 0; t < 32; ++t) asm volatile("" : "+r"(r0[t]), "+r"(r1[t]));
}

// Columns at or beyond k (padding) never win.
__device__ __forceinline__ void mask_tail(uint32_t (&r)[32], int64_t j0, int64_t k) {
    if (j0 + 32 > k) {
#pragma unroll
        for (int t = 0; t < 32; ++t)
            if (j0 + t >= k) r[t] = __float_as_uint(-pos_inf<float>());
    }
}

// The test v >= thr as a fused multiply-add with saturation, which runs on
// the FMA pipe instead of the ALU pipe the compares and selects use.  thrp is
// the float just below thr and K = 2 / ulp(thrp), a power of two: for every
// float v > thrp (equivalently v >= thr), v - thrp >= ulp(thrp) / 2 (v lies
// in thrp's binade or above, or at most one binade below it, where floats are
// spaced ulp(thrp) / 2), so the exact K (v - thrp) is >= 1 and saturates to
// exactly 1; for v <= thrp it is <= 0 and saturates to 0 (a NaN score also
// gives 0, as a NaN compare is false).  thrp K is exact.  Products that
// overflow give +-inf, which saturate to the right side as well.  Thresholds
// whose neighbour's exponent is too small for K to be finite (|thr| below
// about 2^-88), zero, infinite or NaN thresholds take the compare path.
struct HotTest {
    float K, nK;
    bool ok;
    __device__ __forceinline__ float hot(float v) const { return __saturatef(fmaf(v, K, nK)); }
};

__device__ __forceinline__ HotTest hot_test(float thr) {
    HotTest h;
    const uint32_t b = __float_as_uint(thr);
    const uint32_t e = (b >> 23) & 0xffu;
    h.ok = e >= 40u && e < 255u;
    // the float just below thr (|thr| >= 2^-87 here, so it is normal)
    const uint32_t pb = (b & 0x80000000u) ? b + 1u : b - 1u;
    const uint32_t ep = (pb >> 23) & 0xffu;
    h.K = __uint_as_float(h.ok ? (278u - ep) << 23 : 0x3f800000u);  // 2^(151 - ep)
    h.nK = -__uint_as_float(pb) * h.K;
    return h;
}

// OR over the 64 epilogue threads of TMEM lane quadrant q (the two warps that
// scan the two column halves of the same rows), named barrier 8 + q.  Only
// these two warps exchange data, so the other quadrants are not held back.
__device__ __forceinline__ bool pair_any(bool v, int q) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, %2, 64, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(8 + q)
        : "memory");
    return r != 0;
}

// Barrier of the two update warps (named barrier 12, 64 threads); upd_any
// also returns the OR of v over them.
__device__ __forceinline__ void upd_sync() {
    asm volatile("bar.sync 12, 64;" ::: "memory");
}
__device__ __forceinline__ bool upd_any(bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "barrier.red.or.pred q, 12, 64, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)v)
        : "memory");
    return r != 0;
}

// 2^e as a float (e in [-126, 127]).
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((127 + e) << 23); }

// Packed fixed-point term of a float v = +-m 2^(E - 150) (E its exponent
// field, m its 24-bit mantissa) at scale 2^s, emin = 150 - s: when
// 0 <= E - emin <= 30, v 2^s = +-m 2^(E - emin) is an integer, stored as
// (+-m) << 6 | (E - emin) << 1; zero is 0; every other v (below the scale's
// resolution, denormal, infinite, NaN; the field 255 lies more than 30 above
// any emin <= 224) is the flag 1, which adds nothing.
__host__ __device__ inline int pack_fixed(float v, int emin) {
    uint32_t b;
    memcpy(&b, &v, 4);
    if ((b & 0x7fffffffu) == 0u) return 0;
    const uint32_t sh = (uint32_t)((int)((b >> 23) & 0xffu) - emin);
    if (sh > 30u) return 1;
    const int m = (int)((b & 0x7fffffu) | 0x800000u);
    const int ms = (b >> 31) ? -m : m;
    return (int)(((uint32_t)ms << 6) | (sh << 1));
}

// sum += the integer a packed term stands for (one 32 x 32 -> 64-bit
// multiply-add).
__device__ __forceinline__ void add_packed(unsigned long long &sum, int p) {
    const int ms = p >> 6;
    const int pw = 1 << ((p >> 1) & 31);
    asm("mad.wide.s32 %0, %1, %2, %0;" : "+l"(sum) : "r"(ms), "r"(pw));
}

// own_f (2 or 4) consecutive 64-bit sums at a 16-byte aligned shared-window
// address (volatile: kept in program order with each other).
template <int F>
__device__ __forceinline__ void lds_sums(uint32_t addr, unsigned long long (&q)[F]) {
    static_assert(F == 2 || F == 4, "two or four columns per thread");
#pragma unroll
    for (int j = 0; j < F; j += 2)
        asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(q[j]), "=l"(q[j + 1]) : "r"(addr + 8u * j));
}
template <int F>
__device__ __forceinline__ void sts_sums(uint32_t addr, const unsigned long long (&q)[F]) {
    static_assert(F == 2 || F == 4, "two or four columns per thread");
#pragma unroll
    for (int j = 0; j < F; j += 2)
        asm volatile("st.shared.v2.u64 [%0], {%1, %2};" ::"r"(addr + 8u * j), "l"(q[j]), "l"(q[j + 1]));
}

// Second pass over a tile's terms that the fixed-point sums cannot hold
// (flag 1: below the scale's resolution, or NaN): their exact float values
// straight into the float64 sums.  Kept out of line so that no float64
// instruction enters the first pass.  Columns c0 .. c0 + nc - 1 of rows
// grp, grp + R, ... of the tile whose first sample is i0.
__device__ __noinline__ void rare_terms(const MixedArgs &a, double *acc64, int64_t ks, int64_t i0,
                                        const int *code, const int *stage, int grp, int R, int c0,
                                        int nc) {
    const int64_t d4 = a.d4, ds = d4 + 4;
    for (int r = grp; r < kTileM; r += R) {
        const int c = code[r];
        if (c < 0 || c >= a.k) continue;
        for (int j = c0; j < c0 + nc; ++j) {
            if (stage[r * ds + j] != 1) continue;
            const float w = a.w[i0 + r];
            if (j < d4) {
                const float v = __fmul_rn(a.xrow[(i0 + r) * d4 + j], w);
                if (v != 0.f) atomicAdd(acc64 + (int64_t)c * d4 + j, (double)v);
            } else if (j == d4) {
                atomicAdd(acc64 + ks * d4 + c, (double)w);
            }
        }
    }
}

// The update role of the tensor-core kernel with fixed-point sums (d <= 32,
// one column pass): the CTA adds the features and weights of its certified
// rows into integer sums in shared memory and adds them to the fit's
// order-independent integer totals (FxAcc) once at the end.  Every term w x (and w) is prepared once per
// fit as the packed integer w x 2^fx_shift (the shift keeps every CTA's sums
// below 2^61), so a term costs one multiply-add on the integer pipe per
// iteration.  No float64 instruction runs per tile: on this part even a
// predicated-off float64 conversion costs the issue slots of a whole row.
// Terms below the scale's resolution, and NaNs, are rare: a tile that has
// some adds them to the float64 copy in a second pass.
//
// Rows are d4 + 4 packed columns (w x_0 .. w x_{d4-1}, w, 0, 0, 0).  Thread
// u adds columns j0 .. j0 + F - 1, j0 = F (u mod T), T = (d4 + 4) / F, of
// rows r = g (mod R), g = u / T, R = fx_copies(d4 + 4, F), into its group's
// copy [g][cluster][column]; rows without a certified label go to the spare
// cluster row own_k.  The two update warps copy each tile's packed rows and
// labels into shared memory (named barrier 12) and load the next tile's rows
// while they add this one's.
template <int F>
__device__ __forceinline__ void fixed_sums_role(const MixedArgs &a, const MixedConsts &cst,
                                                uint8_t *smem, const SmemLayout &L, int *lab_s,
                                                uint64_t *ufull, uint64_t *uempty, volatile int *err,
                                                long long lim, double *acc64, int64_t ks) {
    const int u = threadIdx.x - 32 * (2 + kEpiWarps);
    const int64_t n = a.n, k = a.k, d4 = a.d4, ok = a.own_k;
    const int ds = (int)d4 + 4, dq = ds / 4;  // packed columns, uint4 per row
    const int64_t ntiles = ceil_div<int64_t>(n, kTileM);
    const int T = ds / F, R = fx_copies(ds, F);
    const int grp = u / T, j0 = F * (u - grp * T);
    long long *osum = reinterpret_cast<long long *>(smem + L.osum);
    int *ostage = reinterpret_cast<int *>(smem + L.ostage);
    int *ocode = reinterpret_cast<int *>(smem + L.ocode);
    const uint32_t mine = smem_u32(osum + (int64_t)grp * (ok + 1) * ds + j0);
    const uint32_t cstride = 8u * (uint32_t)ds;

    for (int64_t e = u; e < (int64_t)R * (ok + 1) * ds; e += kUpdThreads) osum[e] = 0;
    // rows u and u + 64 of a tile, loaded one tile ahead
    uint4 ra[9], rb[9];
    auto load_rows = [&](int64_t tile) {
        const int64_t i0 = tile * kTileM + u, i1 = i0 + 64;
        const uint4 *pa = reinterpret_cast<const uint4 *>(a.xq + i0 * ds);
        const uint4 *pb = reinterpret_cast<const uint4 *>(a.xq + i1 * ds);
#pragma unroll
        for (int g = 0; g < 9; ++g) {
            const bool in = g < dq && tile < ntiles;
            ra[g] = (in && i0 < n) ? __ldg(pa + g) : make_uint4(0u, 0u, 0u, 0u);
            rb[g] = (in && i1 < n) ? __ldg(pb + g) : make_uint4(0u, 0u, 0u, 0u);
        }
    };
    load_rows(blockIdx.x);
    int tl = 0;
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++tl) {
        const int tb = tl & 1;
        const bool got = mbar_wait(&ufull[tb], ((uint32_t)tl >> 1) & 1u, err, lim);
        int c0 = -1, c1 = -1;
        if (got) {
            c0 = lab_s[tb * kTileM + u];
            c1 = lab_s[tb * kTileM + u + 64];
            mbar_arrive(&uempty[tb]);
        }
        // both warps stop together (this barrier also orders the previous
        // tile's reads of the stage before the writes below)
        if (upd_any(!got)) break;
        uint4 *sa = reinterpret_cast<uint4 *>(ostage + u * ds);
        uint4 *sb = reinterpret_cast<uint4 *>(ostage + (u + 64) * ds);
#pragma unroll
        for (int g = 0; g < 9; ++g)
            if (g < dq) {
                sa[g] = ra[g];
                sb[g] = rb[g];
            }
        // labels of rows the kernel did not certify (and padding) go to the
        // spare cluster row
        ocode[u] = (c0 >= 0 && c0 < k) ? c0 : (int)ok;
        ocode[u + 64] = (c1 >= 0 && c1 < k) ? c1 : (int)ok;
        upd_sync();
        load_rows(tile + gridDim.x);
        if (grp < R) {
            int flags = 0;
            for (int r = grp; r < kTileM; r += R) {
                const int c = ocode[r];
                const int *t = ostage + r * ds + j0;
                int v[F];
                if constexpr (F == 4) {
                    const int4 q = *reinterpret_cast<const int4 *>(t);
                    v[0] = q.x, v[1] = q.y, v[2] = q.z, v[3] = q.w;
                } else {
                    const int2 q = *reinterpret_cast<const int2 *>(t);
                    v[0] = q.x, v[1] = q.y;
                }
                const uint32_t addr = mine + (uint32_t)c * cstride;
                unsigned long long sum[F];
                lds_sums<F>(addr, sum);
                int rf = 0;
#pragma unroll
                for (int j = 0; j < F; ++j) {
                    add_packed(sum[j], v[j]);
                    rf |= v[j];
                }
                sts_sums<F>(addr, sum);
                // flagged terms of the spare row never count
                flags |= c != (int)ok ? rf : 0;
            }
            if (flags & 1)
                rare_terms(a, acc64, ks, tile * kTileM, ocode, ostage, grp, R, j0, F);
        }
    }
    upd_sync();
    // this CTA's sums (its R copies added exactly) into the order-independent
    // integer totals
    const FxAcc fxc = a.fx.copy_of(blockIdx.x);
    for (int64_t e = u; e < ok * (d4 + 1); e += kUpdThreads) {
        const int64_t c = e < ok * d4 ? e / d4 : e - ok * d4;
        const int64_t j = e < ok * d4 ? e - c * d4 : d4;
        long long q = 0;
        for (int g = 0; g < R; ++g) q += osum[((int64_t)g * (ok + 1) + c) * ds + j];
        if (q != 0) fx_add(fxc, e, q);
    }
}

// Packed fixed-point terms of every sample: w x_j for j < d4 (rounded
// products, as the reference forms them), then w, 0, 0, 0.
__global__ void fx_pack_kernel(const float *xrow, const float *w, int64_t n, int64_t d4,
                               const MixedConsts *c, int *xq) {
    const int64_t ds = d4 + 4;
    const int emin = 150 - c->fx_shift;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n * ds;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i = e / ds, j = e - i * ds;
        const float wi = w[i];
        float v = 0.f;
        if (j < d4)
            v = __fmul_rn(xrow[i * d4 + j], wi);
        else if (j == d4)
            v = wi;
        xq[e] = pack_fixed(v, emin);
    }
}

template <int BF16>
__device__ __forceinline__ uint32_t pack2(float a, float b) {
    if (BF16) {
        __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    } else {
        __half2 h = __floats2half2_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&h);
    }
}

// Constant columns of the half-norm block: the score receives
// -(c0 h0 + c1 h1 + c2 h2) with (h0, h1, h2) the 16-bit parts of sigma^2 hn.
__host__ __device__ constexpr float norm_coef(int bf16, int part) {
    return bf16 ? -1.f : (part == 0 ? -1024.f : (part == 1 ? -1.f : -0x1p-10f));
}

template <int BF16, int NKB, int NCH, bool MULTI>
__global__ void __launch_bounds__(kThreadsMixed, 1) mixed_assign_kernel(MixedArgs a) {
    if (a.guard != nullptr && *reinterpret_cast<const volatile int *>(&a.guard->done)) return;
    extern __shared__ __align__(1024) uint8_t smem_raw[];
    // the swizzles are functions of absolute shared-memory address bits, so
    // every operand image starts on a 1024-byte boundary
    uint8_t *smem = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
    constexpr int64_t k_pad = (int64_t)NCH * kChunkN;
    const int stages = a.stages;
    const SmemLayout L = smem_layout(NKB, k_pad, a.d4, stages, a.own_k, a.own_f);
    uint8_t *cimg_s = smem + L.c;
    uint8_t *aon_s = smem + L.aon;
    uint8_t *xring = smem + L.x;
    float *xch = reinterpret_cast<float *>(smem + L.xch);
    int *lab_s = reinterpret_cast<int *>(smem + L.lab);
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem + L.bar);
    uint64_t *full = bars, *empty = bars + 4, *tfull = bars + 8, *tempty = bars + 10;
    uint64_t *ufull = bars + 12, *uempty = bars + 14, *cbar = bars + 16, *tdone = bars + 17;
    uint64_t *never = bars + 18;  // completed by no role (timeout test only)
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bars + 19);
    volatile int *err = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // k: columns from this pass's first on (the padding beyond never wins)
    const int64_t n = a.n, k = a.k - a.col0;
    const long long lim = a.wait_limit;
    const int64_t ntiles = ceil_div<int64_t>(n, kTileM);
    const uint32_t cbytes = (uint32_t)cimg_bytes(NKB, k_pad);

    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 32 * kEpiWarps);
            mbar_init(&ufull[b], kTileM);
            mbar_init(&uempty[b], kUpdThreads);
        }
        mbar_init(cbar, 1);
        mbar_init(tdone, 1);
        mbar_init(never, 1);
        *err = 0;
        fence_barrier_init();
    }
    // constant A block of the half-norm MMA: row r = (c0, c1, c2, 0, ..., 0)
    for (int t = threadIdx.x; t < 2 * kTileM; t += blockDim.x) {
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if ((t & 1) == 0) {
            v.x = pack2<BF16>(norm_coef(BF16, 0), norm_coef(BF16, 1));
            v.y = pack2<BF16>(norm_coef(BF16, 2), 0.f);
        }
        *reinterpret_cast<uint4 *>(aon_s + sw32_offset((uint32_t)(t >> 1), (uint32_t)(t & 1) * 8)) = v;
    }
    fence_proxy_async();  // generic-proxy writes -> tensor-core operand reads
    if (warp == 1) {
        tmem_alloc(tmem_slot, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const MixedConsts cst = *a.consts;

    if (warp == 0) {
        // ------------------------------ producer ------------------------------
        if (lane == 0) {
            mbar_arrive_expect_tx(cbar, cbytes);
            // rows col0 .. col0 + k_pad - 1 of every feature block and of the
            // half-norm block of the global image
            for (int kb = 0; kb <= NKB; ++kb) {
                const uint32_t row = kb < NKB ? 128u : kNormRowBytes;
                const uint32_t bytes = (uint32_t)k_pad * row;
                const uint8_t *src = a.cimg + (size_t)kb * a.k_img * 128 + (size_t)a.col0 * row;
                uint8_t *dst = cimg_s + (size_t)kb * k_pad * 128;
                for (uint32_t off = 0; off < bytes; off += 32768u)
                    bulk_g2s(dst + off, src + off, min(32768u, bytes - off), cbar);
            }
            int s = 0;
            uint32_t ph = 0, issued = 0u, last_ph = 0u;
            for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
                if (!mbar_wait(&empty[s], ph ^ 1u, err, lim)) break;
                mbar_arrive_expect_tx(&full[s], NKB * kTileBytes);
                bulk_g2s(xring + (size_t)s * NKB * kTileBytes,
                         a.ximg + (size_t)tile * NKB * kTileBytes, NKB * kTileBytes, &full[s]);
                issued |= 1u << s;
                last_ph = (last_ph & ~(1u << s)) | (ph << s);
                if (++s == stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
            // never leave a copy in flight into this CTA's shared memory: the
            // centroid image and the last copy into each ring stage (a stage
            // holds at most one copy in flight) are waited for even after an
            // error
            mbar_wait_drain(cbar, 0, err);
            for (int q = 0; q < stages; ++q)
                if ((issued >> q) & 1u) mbar_wait_drain(&full[q], (last_ph >> q) & 1u, err);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------ MMA issuer ----------------------------
        if (lane == 0) {
            const uint32_t idesc = idesc_f16(BF16, kTileM, kChunkN);
            const uint32_t cbase = smem_u32(cimg_s);
            const uint32_t hbase = cbase + (uint32_t)(NKB * k_pad * 128);
            const uint64_t adesc_norm = desc_sw32(smem_u32(aon_s));
            bool ok = mbar_wait(cbar, 0, err, lim);
            int s = 0;
            uint32_t ph = 0, cnt = 0;
            for (int64_t tile = blockIdx.x; ok && tile < ntiles; tile += gridDim.x) {
                if (!mbar_wait(&full[s], ph, err, lim)) break;
                tc_fence_after();
                const uint32_t xbase = smem_u32(xring + (size_t)s * NKB * kTileBytes);
                for (int c = 0; c < NCH; ++c) {
                    const uint32_t b = cnt & 1u, bph = (cnt >> 1) & 1u;
                    if (!mbar_wait(&tempty[b], bph ^ 1u, err, lim)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dt = tmem + b * kChunkN;
#pragma unroll
                    for (int kb = 0; kb < NKB; ++kb)
#pragma unroll
                        for (int kk = 0; kk < 4; ++kk) {
                            const uint64_t ad = desc_sw128(xbase + kb * kTileBytes + kk * 32);
                            const uint64_t bd = desc_sw128(cbase + (uint32_t)(kb * k_pad * 128) +
                                                           (uint32_t)(c * kChunkN * 128) + kk * 32);
                            mma_f16(dt, ad, bd, idesc, (kb | kk) != 0 ? 1u : 0u);
                        }
                    // - sigma^2 hn_j for the 256 columns of this chunk
                    mma_f16(dt, adesc_norm,
                            desc_sw32(hbase + (uint32_t)(c * kChunkN) * kNormRowBytes), idesc, 1u);
                    mma_commit(&tfull[b]);
                    ++cnt;
                }
                mma_commit(&empty[s]);
                if (++s == stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
            // all issued MMAs must have finished before TMEM is released,
            // error or not
            mma_commit(tdone);
            mbar_wait_drain(tdone, 0, err);
        }
        __syncwarp();
    } else if (warp < 2 + kEpiWarps) {
        // ------------------------------ epilogue ------------------------------
        // Thread (row, h) scans columns h*128 .. h*128+127 of every chunk for
        // tile row `row`: P2[t] = max over its columns j = t (mod 32), P1[s] =
        // max over its 32-column sub-chunk s (4 per chunk).
        constexpr int kSub = 4 * NCH;
        constexpr uint32_t kAll1 = (kSub == 32) ? ~0u : ((1u << kSub) - 1u);
        constexpr bool kP1s = p1_in_smem(NCH);
        constexpr int kChunkUnroll = kP1s ? 1 : NCH;
        const int ew = warp - 2;
        float *my_p1 = reinterpret_cast<float *>(smem + L.p1) + (ew * 32 + lane);
        const int q = warp & 3;   // TMEM lane quadrant accessible to this warp
        const int h = ew >> 2;    // column half of each 256-wide chunk
        const int row = 32 * q + lane;
        const uint32_t lane_addr = (uint32_t)(32 * q) << 16;
        uint32_t cnt = 0;
        int tl = 0;
        // test of the timeout path: this wait runs out after `lim` clocks
        if (a.stall) mbar_wait(never, 0, err, lim);
        // per-sample norms of the next tile are loaded one tile ahead
        float nx_next = 0.f, dx_next = 0.f;
        {
            const int64_t i0 = (int64_t)blockIdx.x * kTileM + row;
            if (i0 < n) {
                nx_next = a.nx[i0];
                dx_next = a.ndx[i0];
            }
        }
        for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++tl) {
            const int64_t i = tile * kTileM + row;
            float E2 = 0.f;
            if (i < n) {
                const float e = fmaf(nx_next, cst.alpha, fmaf(dx_next, cst.beta1, cst.beta0));
                E2 = 2.f * e * 1.000001f;
            }
            {
                const int64_t inext = (tile + gridDim.x) * kTileM + row;
                if (inext < n) {
                    nx_next = a.nx[inext];
                    dx_next = a.ndx[inext];
                }
            }
            float P2[32], P1[kP1s ? 1 : kSub];
            float Mh = -pos_inf<float>();
            // sub-chunk maximum m of sub-chunk sc (register or shared copy)
            auto put = [&](int sc, float m) {
                Mh = fmaxf(Mh, m);
                if constexpr (kP1s)
                    my_p1[sc * 32 * kEpiWarps] = m;
                else
                    P1[sc] = m;
            };
#pragma unroll
            for (int t = 0; t < 32; ++t) P2[t] = -pos_inf<float>();
            bool bad = false;
            // unrolled when the maxima live in registers (static indices)
#pragma unroll kChunkUnroll
            for (int c = 0; c < NCH; ++c) {
                const uint32_t b = cnt & 1u, bph = (cnt >> 1) & 1u;
                if (!mbar_wait(&tfull[b], bph, err, lim)) bad = true;
                // tcgen05.ld is warp-collective: re-converge after the spin-wait
                if (__any_sync(0xffffffffu, bad)) {
                    bad = true;
                    break;
                }
                tc_fence_after();
                const uint32_t cb = tmem + lane_addr + b * kChunkN + h * 128;
                const int64_t j0 = (int64_t)c * kChunkN + h * 128;
                uint32_t ra[32], rb[32];
                // sub-chunks 0 and 1
                tmem_ld32(cb, ra);
                tmem_ld32(cb + 32, rb);
                tmem_ld_wait_regs(ra, rb);
                // padding columns (at or beyond k) never win; a pass's padding
                // may span several chunks
                const bool pad = MULTI ? (int64_t)(c + 1) * kChunkN > k : c == NCH - 1;
                if (pad) {
                    mask_tail(ra, j0, k);
                    mask_tail(rb, j0 + 32, k);
                }
#pragma unroll
                for (int t = 0; t < 32; ++t) P2[t] = max3f(P2[t], u2f(ra[t]), u2f(rb[t]));
                const float m0 = max32(ra);
                // the loads below reuse ra / rb: finish every read of them first
#pragma unroll
                for (int t = 0; t < 32; ++t) asm volatile("" : "+f"(P2[t]));
                asm volatile("" ::"f"(m0));
                tmem_ld32(cb + 64, ra);
                const float m1 = max32(rb);
                asm volatile("" ::"f"(m1));
                tmem_ld32(cb + 96, rb);
                put(4 * c, m0);
                put(4 * c + 1, m1);
                // sub-chunks 2 and 3
                tmem_ld_wait_regs(ra, rb);
                tc_fence_before();
                mbar_arrive(&tempty[b]);  // the accumulator may be overwritten now
                if (pad) {
                    mask_tail(ra, j0 + 64, k);
                    mask_tail(rb, j0 + 96, k);
                }
#pragma unroll
                for (int t = 0; t < 32; ++t) P2[t] = max3f(P2[t], u2f(ra[t]), u2f(rb[t]));
                put(4 * c + 2, max32(ra));
                put(4 * c + 3, max32(rb));
                ++cnt;
            }

            // best score of this half, exchanged with the other half
            float *xb = xch + (size_t)(tl & 1) * (2 * kTileM);
            xb[h * kTileM + row] = Mh;
            // one pair barrier per tile: publishes the exchange and agrees on errors
            if (pair_any(bad || *err != 0, q)) break;
            const float Mo = xb[(h ^ 1) * kTileM + row];
            // Columns whose score reaches thr = M - E2 can hold the reference's
            // winner (every score is within E2 / 2 of its exact value).  The
            // winner is certified when exactly one column can: no column of
            // the other half reaches thr, and exactly one sub-chunk and one
            // class of the winning half do (two distinct columns of one
            // sub-chunk lie in distinct classes).
            const float thr = fmaxf(Mh, Mo) - E2;
            // exactly one of the pair wins, whatever the maxima (a NaN loses
            // every comparison: the first half then wins); only the winner
            // hands the row over, and ufull counts one arrival per row
            const bool win = (Mh > Mo) || (h == 0 && !(Mo > Mh));
            uint32_t hot1 = 0u, hot2 = 0u;
            const HotTest ht = hot_test(thr);
            if (ht.ok) {
                // the masks on the FMA pipe: 0 / 1 per maximum, summed as
                // exact powers of two in two 16-bit float halves
                float l1 = 0.f, l2 = 0.f, h2 = 0.f;
#pragma unroll
                for (int t = 0; t < kSub; ++t) {
                    const float m = kP1s ? my_p1[t * 32 * kEpiWarps] : P1[kP1s ? 0 : t];
                    l1 = fmaf(ht.hot(m), (float)(1u << t), l1);
                }
#pragma unroll
                for (int t = 0; t < 16; ++t) {
                    l2 = fmaf(ht.hot(P2[t]), (float)(1u << t), l2);
                    h2 = fmaf(ht.hot(P2[16 + t]), (float)(1u << t), h2);
                }
                hot1 = __float2uint_rz(l1);
                hot2 = __float2uint_rz(l2) | (__float2uint_rz(h2) << 16);
            } else {
#pragma unroll
                for (int t = 0; t < kSub; ++t) {
                    const float m = kP1s ? my_p1[t * 32 * kEpiWarps] : P1[kP1s ? 0 : t];
                    hot1 |= (m >= thr) ? (1u << t) : 0u;
                }
#pragma unroll
                for (int t = 0; t < 32; ++t) hot2 |= (P2[t] >= thr) ? (1u << t) : 0u;
            }
            bool loser_hot = fminf(Mh, Mo) >= thr;
            if (!(thr == thr)) {  // cannot happen with finite operands; recheck all
                hot1 = kAll1;
                hot2 = ~0u;
                loser_hot = true;
            }
            int code = -1;  // handoff to the update warps: >= 0 label, <= -2 recheck slot
            if (MULTI && i < n) {
                // column pass: the pass's best score and both halves' masks
                // (single bits for a unique winner), decided by the combine
                uint32_t *cw = reinterpret_cast<uint32_t *>(a.cand + i);
                if (win) {
                    cw[h] = hot1;
                    cw[2 + h] = hot2;
                    if (!loser_hot) {
                        cw[h ^ 1] = 0u;
                        cw[2 + (h ^ 1)] = 0u;
                    }
                    a.pmax[i] = fmaxf(Mh, Mo);
                } else if (loser_hot) {
                    cw[h] = hot1;
                    cw[2 + h] = hot2;
                }
            } else if (i < n) {
                uint32_t *cw = reinterpret_cast<uint32_t *>(a.cand + i);
                if (win) {
                    if (!loser_hot && __popc(hot1) == 1 && __popc(hot2) == 1) {
                        const int sc = __ffs(hot1) - 1, t = __ffs(hot2) - 1;
                        code = (sc >> 2) * kChunkN + h * 128 + (sc & 3) * 32 + t;
                        if (a.label64)
                            reinterpret_cast<int64_t *>(a.labels)[i] = code;
                        else
                            reinterpret_cast<int32_t *>(a.labels)[i] = code;
                    } else {
                        cw[h] = hot1;
                        cw[2 + h] = hot2;
                        if (!loser_hot) {
                            cw[h ^ 1] = 0u;
                            cw[2 + (h ^ 1)] = 0u;
                        }
                        const int pos = atomicAdd(a.n_flagged, 1);
                        if (pos >= 0 && pos < n) {
                            a.flagged[pos] = (int)i;
                            code = -2 - pos;
                        }
                    }
                } else if (loser_hot) {
                    cw[h] = hot1;
                    cw[2 + h] = hot2;
                }
            }
            const int tb = tl & 1;
            if (mbar_wait(&uempty[tb], (((uint32_t)tl >> 1) & 1u) ^ 1u, err, lim) && win) {
                lab_s[tb * kTileM + row] = code;
                mbar_arrive(&ufull[tb]);
            }
        }
    } else {
        // ------------------------------ update --------------------------------
        // Thread u handles rows u and u + 64 of every tile.  The rows (from
        // the row-major fp32 copy of X) and weights are loaded before their
        // labels are known, so the loads overlap the epilogue of the tile.
        // Uncertified rows are left to the recheck kernel.
        const int u = threadIdx.x - 32 * (2 + kEpiWarps);
        const int64_t d4 = a.d4;
        const int64_t ks = MULTI ? a.k_img : k_pad;  // rows of the cluster sums (all columns)
        const int64_t cstride = ks * d4 + ks;
        float *sums32 = a.sums32 + (int64_t)(blockIdx.x % (unsigned)a.n_copies) * cstride;
        double *acc64 = a.acc64 + (int64_t)(blockIdx.x % (unsigned)a.n_copies) * cstride;
        auto consume = [&](int code, const float4 (&xv)[16], float wv, int pass) {
            if (code < 0 || code >= k || !a.update) return;
            if (a.acc_f64) {
                // small d: float64 sums keep the trajectory on the reference's
                double *dst = acc64 + (int64_t)code * d4 + pass * 64;
#pragma unroll
                for (int g = 0; g < 16; ++g) {
                    if ((int64_t)pass * 64 + 4 * g < d4) {
                        atomicAdd(dst + 4 * g + 0, (double)__fmul_rn(xv[g].x, wv));
                        atomicAdd(dst + 4 * g + 1, (double)__fmul_rn(xv[g].y, wv));
                        atomicAdd(dst + 4 * g + 2, (double)__fmul_rn(xv[g].z, wv));
                        atomicAdd(dst + 4 * g + 3, (double)__fmul_rn(xv[g].w, wv));
                    }
                }
                if (pass == 0) atomicAdd(acc64 + ks * d4 + code, (double)wv);
            } else {
                float4 *dst = reinterpret_cast<float4 *>(sums32 + (int64_t)code * d4 + pass * 64);
#pragma unroll
                for (int g = 0; g < 16; ++g) {
                    if ((int64_t)pass * 64 + 4 * g < d4) {
                        float4 v;
                        v.x = __fmul_rn(xv[g].x, wv);
                        v.y = __fmul_rn(xv[g].y, wv);
                        v.z = __fmul_rn(xv[g].z, wv);
                        v.w = __fmul_rn(xv[g].w, wv);
                        atomicAdd(dst + g, v);
                    }
                }
                if (pass == 0) atomicAdd(sums32 + ks * d4 + code, wv);
            }
        };
        bool owned_done = false;
        if constexpr (NKB == 1 && !MULTI) {
            if (a.update && a.own_k > 0 && cst.fx_ok) {
                if (a.own_f == 4)
                    fixed_sums_role<4>(a, cst, smem, L, lab_s, ufull, uempty, err, lim, acc64, ks);
                else
                    fixed_sums_role<2>(a, cst, smem, L, lab_s, ufull, uempty, err, lim, acc64, ks);
                owned_done = true;
            }
        }
        int tl = 0;
        for (int64_t tile = blockIdx.x; !owned_done && tile < ntiles; tile += gridDim.x, ++tl) {
            const int tb = tl & 1;
            const int64_t i0 = tile * kTileM + u, i1 = i0 + 64;
            const float w0 = (a.update && i0 < n) ? __ldg(a.w + i0) : 0.f;
            const float w1 = (a.update && i1 < n) ? __ldg(a.w + i1) : 0.f;
            int c0 = -1, c1 = -1;
            bool have_code = false;
#pragma unroll 1
            for (int pass = 0; pass < NKB; ++pass) {
                float4 xa[16], xb[16];
                const float4 *ra = reinterpret_cast<const float4 *>(a.xrow + i0 * d4 + pass * 64);
                const float4 *rb = reinterpret_cast<const float4 *>(a.xrow + i1 * d4 + pass * 64);
#pragma unroll
                for (int g = 0; g < 16; ++g) {
                    const bool in = (int64_t)pass * 64 + 4 * g < d4;
                    xa[g] = (a.update && in && i0 < n) ? __ldg(ra + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                    xb[g] = (a.update && in && i1 < n) ? __ldg(rb + g) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
                if (!have_code) {
                    if (!mbar_wait(&ufull[tb], ((uint32_t)tl >> 1) & 1u, err, lim)) break;
                    c0 = lab_s[tb * kTileM + u];
                    c1 = lab_s[tb * kTileM + u + 64];
                    mbar_arrive(&uempty[tb]);
                    have_code = true;
                }
                consume(c0, xa, w0, pass);
                consume(c1, xb, w1, pass);
            }
            if (!have_code) break;
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem, 512);
    }
    if (threadIdx.x == 0 && *err) {
        atomicExch(a.err_global, 1);
        if (a.state != nullptr) {
            // the remaining kernels of the iteration and the host loop stop
            atomicOr(&a.state->err, 1u);
            atomicExch(&a.state->done, 1);
        }
    }
}

// ---------------------------------------------------------------------------
// preparation kernels
// ---------------------------------------------------------------------------
__global__ void absmax_kernel(const float *X, int64_t count, unsigned int *out_bits) {
    float m = 0.f;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(X[e]));
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m == m) atomicMax(out_bits, __float_as_uint(m));
}

// fp16 operands: sigma is the largest power of two in [2^-60, 2^60] with
// max|x| sigma <= 2^14 and sigma^2 d max|x|^2 / 2 <= 2^25, so that every
// scaled sample, every scaled centroid inside the data's range and the
// largest part of sigma^2 hn stay finite in fp16 with room to spare.  bf16
// shares fp32's exponent range and is never scaled.
__global__ void sigma_kernel(MixedConsts *c, int bf16, int64_t d) {
    const double xmax = (double)__uint_as_float(c->xmax_bits);

    double sigma = 1.0;
    if (!bf16 && xmax > 0.0 && xmax < 1e300) {
        const double hx = 0.5 * (double)d * xmax * xmax;
        auto fits = [&](double s) { return xmax * s <= 0x1p14 && s * s * hx <= 0x1p25; };
        while (sigma < 0x1p60 && fits(sigma * 2.0)) sigma *= 2.0;
        while (sigma > 0x1p-60 && !fits(sigma)) sigma *= 0.5;
    }
    c->sigma = (float)sigma;
    c->s2 = (float)(sigma * sigma);
    c->overflow = 0;
}

// Shift of the fixed-point cluster sums: a CTA adds at most `rows` (>= 128)
// values w x per feature (|w x| <= max|x| max|w|) and `rows` weights, so with
// bound = rows max(max|x| max|w|, max|w|) < 2^e the shift 61 - e keeps every
// sum below 2^61 and every term below 2^54 (all-zero data gives 0).
__global__ void fixed_scale_kernel(MixedConsts *c, double rows) {
    const double xm = (double)__uint_as_float(c->xmax_bits);
    const double wm = (double)__uint_as_float(c->wmax_bits);
    auto shift_for = [](double bound) {
        int sh = 0;
        if (bound > 0.0 && bound < 1e300) {
            int e = 0;
            frexp(bound, &e);
            sh = min(100, 61 - e);
        }
        return sh;
    };
    const int sx = shift_for(rows * fmax(xm * wm, wm));
    // products w x that may overflow fp32, and scales whose resolution field
    // 150 - shift would come within 30 of the infinity / NaN field, keep the
    // float64 reductions
    c->fx_ok = (xm * wm < 1e37 && sx >= -70) ? 1 : 0;
    c->fx_shift = sx;
}

// Round to the 16-bit operand type and back (exact in fp32).
template <int BF16>
__device__ __forceinline__ float round16(float v) {
    if (BF16) return __bfloat162float(__float2bfloat16_rn(v));
    return __half2float(__float2half_rn(v));
}

// One CTA per 128-sample tile (including the zero rows that pad the last
// tile): the tile's features are staged in shared memory (coalesced reads of
// each feature's 128 samples from a feature-major X, or of each sample's d
// features from a row-major one), then written out as the 128-byte-swizzled
// K-major image of (x * sigma) and the row-major fp32 copy of x (features
// d..d4-1 zero), both as contiguous 16-byte chunks, and per sample ||x|| and
// the norm of the image's rounding error ||round16(x sigma) - x sigma|| /
// sigma, both rounded up.
constexpr int kXImageThreads = 256;
constexpr int kXsPitch = kTileM + 1;  // floats per staged feature (bank offset)

__host__ __device__ inline size_t x_image_smem(int nkb) {
    return sizeof(float) * (size_t)nkb * 64 * kXsPitch;
}

template <int BF16>
__global__ void __launch_bounds__(kXImageThreads) x_image_kernel(
    const float *X, int64_t n, int64_t d, int64_t d4, int nkb, int64_t ntiles,
    const MixedConsts *c, uint8_t *img, float *xrow, float *nx, float *ndx, int rowmajor) {
    extern __shared__ float xs[];  // [feature][kXsPitch]
    const float sigma = c->sigma;
    const int F = nkb * 64;
    const int g4 = (int)(d4 / 4);
    for (int64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int64_t i0 = tile * kTileM;
        if (rowmajor) {
            for (int e = threadIdx.x; e < F * kTileM; e += kXImageThreads) {
                const int r = e / F, f = e - r * F;
                const int64_t i = i0 + r;
                xs[f * kXsPitch + r] = (f < d && i < n) ? X[i * d + f] : 0.f;
            }
        } else {
            for (int e = threadIdx.x; e < F * kTileM; e += kXImageThreads) {
                const int f = e >> 7, r = e & (kTileM - 1);
                const int64_t i = i0 + r;
                xs[f * kXsPitch + r] = (f < d && i < n) ? X[(int64_t)f * n + i] : 0.f;
            }
        }
        __syncthreads();
        // image: 16-byte chunk q of feature block kb holds row r, features
        // 8 ch .. 8 ch + 7 with ch = (q mod 8) xor (r mod 8) (128-byte swizzle)
        for (int q = threadIdx.x; q < nkb * 1024; q += kXImageThreads) {
            const int kb = q >> 10, qq = q & 1023;
            const int r = (qq >> 6) * 8 + ((qq >> 3) & 7);
            const int ch = (qq & 7) ^ (r & 7);
            const float *src = xs + (kb * 64 + ch * 8) * kXsPitch + r;
            uint4 pk;
            pk.x = pack2<BF16>(src[0 * kXsPitch] * sigma, src[1 * kXsPitch] * sigma);
            pk.y = pack2<BF16>(src[2 * kXsPitch] * sigma, src[3 * kXsPitch] * sigma);
            pk.z = pack2<BF16>(src[4 * kXsPitch] * sigma, src[5 * kXsPitch] * sigma);
            pk.w = pack2<BF16>(src[6 * kXsPitch] * sigma, src[7 * kXsPitch] * sigma);
            *reinterpret_cast<uint4 *>(img + ((size_t)tile * nkb + kb) * kTileBytes +
                                       (size_t)qq * 16) = pk;
        }
        // row-major fp32 rows: the tile's block of xrow is contiguous
        const int rows_here = (n - i0 < (int64_t)kTileM) ? (int)(n - i0) : kTileM;
        for (int e = threadIdx.x; e < rows_here * g4; e += kXImageThreads) {
            const int r = e / g4, g = e - r * g4;
            const float *src = xs + (4 * g) * kXsPitch + r;
            reinterpret_cast<float4 *>(xrow + (i0 + r) * d4)[g] =
                make_float4(src[0], src[kXsPitch], src[2 * kXsPitch], src[3 * kXsPitch]);
        }
        if (threadIdx.x < kTileM && threadIdx.x < rows_here) {
            const int r = threadIdx.x;
            float s2 = 0.f, sd = 0.f;  // float32 sums, bounded from above below
            for (int f = 0; f < F; ++f) {
                const float x = xs[f * kXsPitch + r];
                s2 = __fmaf_rn(x, x, s2);
                const float v = x * sigma;
                const float dv = round16<BF16>(v) - v;  // exact
                sd = __fmaf_rn(dv, dv, sd);
            }
            // A float32 sum of m non-negative terms (each rounded once) is at
            // least (1 - 2^-24)^m times the exact sum; m <= 128 here, so the
            // factor 1 + (m + 2) 2^-23 applied with upward rounding (and an
            // upward square root) gives upper bounds of both norms (1 / sigma
            // is a power of two).
            const float grow = 1.f + (float)(nkb * 64 + 2) * 0x1p-23f;
            nx[i0 + r] = __fsqrt_ru(__fmul_ru(s2, grow));
            ndx[i0 + r] = __fmul_ru(__fsqrt_ru(__fmul_ru(sd, grow)), 1.f / sigma);
        }
        __syncthreads();
    }
}

// Largest finite operand value: fp16 65504, bf16 (1 - 2^-8) 2^128.
template <int BF16>
__device__ __forceinline__ float max16() {
    return BF16 ? 3.3895313892515355e38f : 65504.f;
}

// Centroid image (rows j < k_pad, zero padding), the half-norm block and the
// per-centroid norms ||c_j|| and ||round16(c_j sigma) - c_j sigma|| / sigma
// (both rounded up).  Row j of the half-norm block holds (h0, h1, h2) with
//   c0 h0 + c1 h1 + c2 h2 = -sigma^2 hn_j   (c = norm_coef)
// up to sigma^2 |hn_j| u^3 (u = 2^-11 fp16, 2^-8 bf16; plus 2^-35 for fp16
// subnormal parts): h0 is the rounded leading part and each following part
// the rounded remainder, formed exactly in fp64.  A value that would leave the
// operand range is clamped and raises consts->overflow, which disables
// certification for the pass (every sample is then re-evaluated exactly).
template <int BF16>
__global__ void c_image_kernel(const float *C, const float *hn, int64_t d, int64_t k,
                               int64_t k_pad, int nkb, MixedConsts *c, uint8_t *img, float *cn2,
                               float *dcn, float *ct, int64_t d4, const LoopState *guard) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    const float sigma = c->sigma;
    const double s2 = (double)sigma * (double)sigma;
    const float lim = max16<BF16>();
    bool ovf = false;
    // One thread per (centroid row j, 8-feature chunk): G = 8 nkb rounded up
    // to a power of two consecutive lanes hold one row, the ones past its 8 nkb
    // chunks idle (k_pad G is a multiple of 32, so every warp is either
    // entirely inside the range or entirely past it, and a row's lanes never
    // straddle two warps).
    const int G = (nkb <= 1) ? 8 : (nkb == 2 ? 16 : 32);
    const int64_t total = k_pad * G;
    for (int64_t tt = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; tt < total;
         tt += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = tt / G;
        const int qc = (int)(tt % G), kb = qc >> 3, ch = qc & 7;
        const bool lane_used = kb < nkb;
        const int64_t f0 = (int64_t)kb * 64 + ch * 8;
        double q2 = 0.0, qd = 0.0;
        float v[8], xr[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) {
            const int64_t f = f0 + e;
            const float x = (lane_used && j < k && f < d) ? C[f * k + j] : 0.f;
            q2 += (double)x * (double)x;
            float sv = x * sigma;
            if (!(fabsf(sv) <= lim)) {
                ovf = true;
                sv = (sv > 0.f) ? lim : ((sv < 0.f) ? -lim : 0.f);
            }
            const double dv = (double)round16<BF16>(sv) - (double)sv;
            qd += dv * dv;
            v[e] = sv;
            xr[e] = x;
        }
        if (lane_used) {
            // d4 is a multiple of 4 and f0 of 8: whole float4 stores
            float4 *cdst = reinterpret_cast<float4 *>(ct + j * d4 + f0);
            if (f0 < d4) cdst[0] = make_float4(xr[0], xr[1], xr[2], xr[3]);
            if (f0 + 4 < d4) cdst[1] = make_float4(xr[4], xr[5], xr[6], xr[7]);
            uint4 pk;
            pk.x = pack2<BF16>(v[0], v[1]);
            pk.y = pack2<BF16>(v[2], v[3]);
            pk.z = pack2<BF16>(v[4], v[5]);
            pk.w = pack2<BF16>(v[6], v[7]);
            *reinterpret_cast<uint4 *>(img + (size_t)kb * k_pad * 128 +
                                       sw128_offset((uint32_t)j, (uint32_t)ch * 8)) = pk;
        }
        // the row's squared norms over its G chunk lanes
        for (int o = G >> 1; o > 0; o >>= 1) {
            q2 += __shfl_xor_sync(0xffffffffu, q2, o);
            qd += __shfl_xor_sync(0xffffffffu, qd, o);
        }
        if (qc != 0) continue;
        float h0 = 0.f, h1 = 0.f, h2 = 0.f;
        if (j < k) {
            const double H = (double)hn[j] * s2;
            const double c0 = -(double)norm_coef(BF16, 0), c1 = -(double)norm_coef(BF16, 1),
                         c2 = -(double)norm_coef(BF16, 2);
            h0 = round16<BF16>((float)(H / c0));
            if (!(fabsf(h0) <= lim)) {
                ovf = true;
                h0 = (H > 0.0) ? lim : -lim;
            }
            const double r1 = H - c0 * (double)h0;
            h1 = round16<BF16>((float)(r1 / c1));
            const double r2 = r1 - c1 * (double)h1;
            h2 = round16<BF16>((float)(r2 / c2));
            if (!(fabsf(h1) <= lim) || !(fabsf(h2) <= lim)) {
                ovf = true;
                h1 = 0.f;
                h2 = 0.f;
            }
            cn2[j] = __double2float_ru(sqrt(q2) * (1.0 + 1e-12));
            dcn[j] = __double2float_ru(sqrt(qd) / (double)sigma * (1.0 + 1e-12));
        }
        uint8_t *nb = img + (size_t)nkb * k_pad * 128;
        uint4 p0 = make_uint4(pack2<BF16>(h0, h1), pack2<BF16>(h2, 0.f), 0u, 0u);
        *reinterpret_cast<uint4 *>(nb + sw32_offset((uint32_t)j, 0)) = p0;
        *reinterpret_cast<uint4 *>(nb + sw32_offset((uint32_t)j, 8)) = make_uint4(0u, 0u, 0u, 0u);
    }
    if (ovf) atomicOr(&c->overflow, 1);
}

// Per-iteration bound constants (one block), in the scaled units of the
// scores (sigma^2).  Resets the overflow flag raised by c_image_kernel.
__global__ void bound_kernel(const float *cn2, const float *dcn, const float *hn, int64_t d,
                             int64_t k, int bf16, MixedConsts *c, const LoopState *guard) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    __shared__ float sh[3][32];
    float m2 = 0.f, m1 = 0.f, mh = 0.f;
    for (int64_t j = threadIdx.x; j < k; j += blockDim.x) {
        m2 = fmaxf(m2, cn2[j]);
        m1 = fmaxf(m1, dcn[j]);
        mh = fmaxf(mh, fabsf(hn[j]));
    }
    for (int o = 16; o > 0; o >>= 1) {
        m2 = fmaxf(m2, __shfl_xor_sync(0xffffffffu, m2, o));
        m1 = fmaxf(m1, __shfl_xor_sync(0xffffffffu, m1, o));
        mh = fmaxf(mh, __shfl_xor_sync(0xffffffffu, mh, o));
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) {
        sh[0][wid] = m2;
        sh[1][wid] = m1;
        sh[2][wid] = mh;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            m2 = fmaxf(m2, sh[0][w]);
            m1 = fmaxf(m1, sh[1][w]);
            mh = fmaxf(mh, sh[2][w]);
        }
        const double sigma = (double)c->sigma, s2 = sigma * sigma;
        const double u = bf16 ? 0x1p-8 : 0x1p-11;
        const double cmax = (double)m2, dcmax = (double)m1;
        // bf16 subnormal inputs may be flushed by the tensor cores (fp16
        // subnormals are part of the measured rounding errors)
        const double flush = bf16 ? 0x1p-126 * sqrt((double)d) * (1 + u) : 0.0;
        const double alpha =
            dcmax + 0x1p-16 * (cmax + dcmax) + (double)(d + 4) * 0x1p-23 * cmax + flush;
        const double beta1 = (cmax + dcmax) * (1 + 0x1p-16);
        const double hfloor = (bf16 ? 0x1p-126 : 0x1p-34) / s2;
        const double beta0 =
            (double)mh * (u * u * u + 0x1p-16 + 0x1p-23) + hfloor + flush * cmax;
        c->alpha = __double2float_ru(alpha * s2 * (1 + 1e-6));
        c->beta1 = __double2float_ru(beta1 * s2 * (1 + 1e-6));
        c->beta0 = c->overflow ? pos_inf<float>()
                               : __double2float_ru(beta0 * s2 * (1 + 1e-6) + 1e-37);
        c->overflow = 0;
    }
}

// Exact fp32 re-evaluation of samples whose margin did not certify them: the
// reference's arithmetic (sequential fma dot over f = 0..d-1, hn - dot,
// strict < with the lowest index on ties) over the candidate set (hot
// sub-chunks x hot classes of each column half).  A warp takes 32 flagged
// samples and spreads their (sample, candidate) pairs evenly over its lanes,
// so one sample with many candidates does not hold its warp back; each pair's
// result goes into the sample's 64-bit (distance, index) key with a
// shared-memory atomic minimum, which is exactly the lexicographic minimum a
// strict-< scan in ascending index finds.  The sample's features come from the
// row-major fp32 copy of X (cached in L1 across its candidates) and the
// centroids from their transposed fp32 copy (one contiguous row each).
constexpr int kRecheckThreads = 256;

// Order-preserving map of a float to an unsigned key (NaN never compared).
__device__ __forceinline__ uint32_t order_key(float v) {
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Candidates of a flagged sample: per column pass p (cand[p * n + i], columns
// offset by p * pass_cols; one pass unless n_clusters needed several), hot
// sub-chunks x hot classes of each column half.
__device__ __forceinline__ int pass_count(const uint4 &m) {
    return __popc(m.x) * __popc(m.z) + __popc(m.y) * __popc(m.w);
}

__global__ void __launch_bounds__(kRecheckThreads) recheck_kernel(
    const float *xrow, const float *ct, const float *hn, const float *w, const uint4 *cand,
    const int *flagged, const int *n_flagged, int64_t n, int64_t d, int64_t k, int64_t d4,
    void *labels, int label64, int update, int acc_f64, float *sums32, double *acc64,
    int64_t k_pad, int n_copies, const LoopState *guard, int passes, int64_t pass_cols, FxAcc fx,
    const MixedConsts *consts) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    constexpr int kWarps = kRecheckThreads / 32;
    const bool use_fx = fx.xq != nullptr && consts->fx_ok;
    fx = fx.copy_of(blockIdx.x);
    __shared__ unsigned long long key_s[kWarps][32];
    __shared__ int incl_s[kWarps][32];
    __shared__ int row_s[kWarps][32];
    __shared__ uint4 cm_s[kWarps][32];
    {
        // this block's share of the per-CTA copies of the cluster sums
        const int64_t copy = (int64_t)(blockIdx.x % (unsigned)n_copies) * (k_pad * d4 + k_pad);
        sums32 += copy;
        acc64 += copy;
    }
    const int lane = threadIdx.x & 31, wq = threadIdx.x >> 5;
    const int64_t nf = (int64_t)*n_flagged;
    const int64_t total = nf < n ? nf : n;
    const int64_t g4 = d4 / 4;
    const unsigned long long kNone = ((unsigned long long)order_key(pos_inf<float>()) << 32);
    const int64_t wstride = (int64_t)gridDim.x * kWarps * 32;
    for (int64_t base = ((int64_t)blockIdx.x * kWarps + wq) * 32; base < total; base += wstride) {
        const int64_t e = base + lane;
        int64_t i = -1;
        uint4 cm = make_uint4(0u, 0u, 0u, 0u);
        int cnt = 0;
        if (e < total) {
            i = flagged[e];
            if (i >= 0 && i < n) {
                cm = cand[i];
                cnt = pass_count(cm);
                for (int p = 1; p < passes; ++p) cnt += pass_count(cand[(int64_t)p * n + i]);
            } else {
                i = -1;
            }
        }
        // candidates of this lane's sample: per column half, hot sub-chunks x hot classes
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        const int tot = __shfl_sync(0xffffffffu, incl, 31);
        key_s[wq][lane] = kNone;
        incl_s[wq][lane] = incl;
        row_s[wq][lane] = (int)i;
        cm_s[wq][lane] = cm;
        __syncwarp();
        for (int pr = lane; pr < tot; pr += 32) {
            // owner: the first lane whose inclusive count exceeds pr
            int lo = 0, hi = 31;
            while (lo < hi) {
                const int mid = (lo + hi) >> 1;
                if (incl_s[wq][mid] > pr) hi = mid; else lo = mid + 1;
            }
            const int owner = lo;
            int r = pr - (owner ? incl_s[wq][owner - 1] : 0);
            const int64_t oi = row_s[wq][owner];
            uint4 om = cm_s[wq][owner];
            int64_t jbase = 0;
            for (int p = 1; p < passes && r >= pass_count(om); ++p) {
                r -= pass_count(om);
                om = cand[(int64_t)p * n + oi];
                jbase += pass_cols;
            }
            const int oc0 = __popc(om.x) * __popc(om.z);
            int h = 0;
            uint32_t m1 = om.x, m2 = om.z;
            if (r >= oc0) {
                h = 1;
                r -= oc0;
                m1 = om.y;
                m2 = om.w;
            }
            // the (r / n2)-th hot sub-chunk and the (r % n2)-th hot class
            const int n2 = __popc(m2);
            for (int q = r / n2; q > 0; --q) m1 &= m1 - 1u;
            for (int q = r % n2; q > 0; --q) m2 &= m2 - 1u;
            const int sc = __ffs(m1) - 1, t = __ffs(m2) - 1;
            const int64_t j = jbase + (int64_t)(sc >> 2) * kChunkN + h * 128 + (sc & 3) * 32 + t;
            if (j >= k) continue;
            const float4 *xr = reinterpret_cast<const float4 *>(xrow + oi * d4);
            const float4 *cr = reinterpret_cast<const float4 *>(ct + j * d4);
            float dot = 0.f;
            // unrolled so that a candidate's row loads are in flight
            // before its fma chain needs them
#pragma unroll 8
            for (int64_t g = 0; g < g4; ++g) {
                const float4 xv = __ldg(xr + g), cv = __ldg(cr + g);
                dot = __fmaf_rn(xv.x, cv.x, dot);
                if (4 * g + 1 < d) dot = __fmaf_rn(xv.y, cv.y, dot);
                if (4 * g + 2 < d) dot = __fmaf_rn(xv.z, cv.z, dot);
                if (4 * g + 3 < d) dot = __fmaf_rn(xv.w, cv.w, dot);
            }
            const float D = hn[j] - dot;
            if (D == D)
                atomicMin(&key_s[wq][owner],
                          ((unsigned long long)order_key(D) << 32) | (unsigned long long)j);
        }
        __syncwarp();
        if (i >= 0) {
            const int bj = (int)(key_s[wq][lane] & 0xffffffffull);
            if (label64)
                reinterpret_cast<int64_t *>(labels)[i] = bj;
            else
                reinterpret_cast<int32_t *>(labels)[i] = bj;
            if (update && use_fx) {
                add_packed_row(fx, acc64, k_pad, k, d4, xrow, w, i, bj);
            } else if (update) {
                const float4 *xr = reinterpret_cast<const float4 *>(xrow + i * d4);
                const float wv = w[i];
                if (acc_f64) {
                    double *dst = acc64 + (int64_t)bj * d4;
                    for (int64_t g = 0; g < g4; ++g) {
                        const float4 xv = __ldg(xr + g);
                        atomicAdd(dst + 4 * g + 0, (double)__fmul_rn(xv.x, wv));
                        atomicAdd(dst + 4 * g + 1, (double)__fmul_rn(xv.y, wv));
                        atomicAdd(dst + 4 * g + 2, (double)__fmul_rn(xv.z, wv));
                        atomicAdd(dst + 4 * g + 3, (double)__fmul_rn(xv.w, wv));
                    }
                    atomicAdd(acc64 + k_pad * d4 + bj, (double)wv);
                } else {
                    float4 *dst = reinterpret_cast<float4 *>(sums32 + (int64_t)bj * d4);
                    for (int64_t g = 0; g < g4; ++g) {
                        const float4 xv = __ldg(xr + g);
                        atomicAdd(dst + g, make_float4(__fmul_rn(xv.x, wv), __fmul_rn(xv.y, wv),
                                                       __fmul_rn(xv.z, wv), __fmul_rn(xv.w, wv)));
                    }
                    atomicAdd(sums32 + k_pad * d4 + bj, wv);
                }
            }
        }
        __syncwarp();  // this batch's keys and masks are read before the next batch
    }
}

// After the column passes of one assignment: per sample the best score M
// over the passes and thr = M - E2 (the bound the passes used).  Every
// score within E2 / 2 of its exact value, a pass whose best score is below
// thr holds no candidate; the pass masks were made against the pass's own
// best score minus E2, which is at most thr, so a hot pass's masks hold a
// superset of its candidates.  The sample is certified when exactly one pass
// reaches thr and that pass has a unique winner (single bits in one half,
// nothing in the other): its label is written and w x added to its cluster's
// sums.  Otherwise the masks of the passes below thr are cleared and the
// sample goes to the recheck list.
__global__ void __launch_bounds__(256) combine_kernel(
    const float *pmax, uint4 *cand, int passes, int64_t pass_cols, const float *nx,
    const float *ndx, const MixedConsts *consts, const float *xrow, const float *w, void *labels,
    int label64, int update, int acc_f64, float *sums32, double *acc64, int64_t k_pad,
    int64_t d4, int n_copies, int *flagged, int *n_flagged, int64_t n, int64_t k,
    const LoopState *guard, FxAcc fx) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    const MixedConsts cst = *consts;
    const bool use_fx = fx.xq != nullptr && cst.fx_ok;
    fx = fx.copy_of(blockIdx.x);
    {
        const int64_t copy = (int64_t)(blockIdx.x % (unsigned)n_copies) * (k_pad * d4 + k_pad);
        sums32 += copy;
        acc64 += copy;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const float e = fmaf(nx[i], cst.alpha, fmaf(ndx[i], cst.beta1, cst.beta0));
        const float E2 = 2.f * e * 1.000001f;
        float M = -pos_inf<float>();
        bool nan = false;
        for (int p = 0; p < passes; ++p) {
            const float v = pmax[(int64_t)p * n + i];
            nan |= !(v == v);
            M = fmaxf(M, v);
        }
        const float thr = M - E2;
        nan |= !(thr == thr);
        int hot = 0, ph = -1;
        for (int p = 0; p < passes; ++p)
            if (nan || pmax[(int64_t)p * n + i] >= thr) {
                ++hot;
                ph = p;
            }
        int64_t label = -1;
        if (!nan && hot == 1) {
            const uint4 m = cand[(int64_t)ph * n + i];
            const bool a0 = (m.x | m.z) != 0u, a1 = (m.y | m.w) != 0u;
            if (a0 != a1) {
                const int h = a1 ? 1 : 0;
                const uint32_t h1 = h ? m.y : m.x, h2 = h ? m.w : m.z;
                if (__popc(h1) == 1 && __popc(h2) == 1) {
                    const int sc = __ffs(h1) - 1, t = __ffs(h2) - 1;
                    label = (int64_t)ph * pass_cols + (int64_t)(sc >> 2) * kChunkN + h * 128 +
                            (sc & 3) * 32 + t;
                    if (label >= k) label = -1;
                }
            }
        }
        if (label >= 0) {
            if (label64)
                reinterpret_cast<int64_t *>(labels)[i] = label;
            else
                reinterpret_cast<int32_t *>(labels)[i] = (int32_t)label;
            if (update && use_fx) {
                add_packed_row(fx, acc64, k_pad, k, d4, xrow, w, i, label);
            } else if (update) {
                const float4 *xr = reinterpret_cast<const float4 *>(xrow + i * d4);
                const float wv = w[i];
                if (acc_f64) {
                    double *dst = acc64 + label * d4;
                    for (int64_t g = 0; g < d4 / 4; ++g) {
                        const float4 xv = __ldg(xr + g);
                        atomicAdd(dst + 4 * g + 0, (double)__fmul_rn(xv.x, wv));
                        atomicAdd(dst + 4 * g + 1, (double)__fmul_rn(xv.y, wv));
                        atomicAdd(dst + 4 * g + 2, (double)__fmul_rn(xv.z, wv));
                        atomicAdd(dst + 4 * g + 3, (double)__fmul_rn(xv.w, wv));
                    }
                    atomicAdd(acc64 + k_pad * d4 + label, (double)wv);
                } else {
                    float4 *dst = reinterpret_cast<float4 *>(sums32 + label * d4);
                    for (int64_t g = 0; g < d4 / 4; ++g) {
                        const float4 xv = __ldg(xr + g);
                        atomicAdd(dst + g, make_float4(__fmul_rn(xv.x, wv), __fmul_rn(xv.y, wv),
                                                       __fmul_rn(xv.z, wv), __fmul_rn(xv.w, wv)));
                    }
                    atomicAdd(sums32 + k_pad * d4 + label, wv);
                }
            }
        } else {
            if (!nan)
                for (int p = 0; p < passes; ++p)
                    if (!(pmax[(int64_t)p * n + i] >= thr))
                        cand[(int64_t)p * n + i] = make_uint4(0u, 0u, 0u, 0u);
            const int pos = atomicAdd(n_flagged, 1);
            if (pos >= 0 && pos < n) flagged[pos] = (int)i;
        }
    }
}

// Per-CTA copies of the cluster-major sums (fp32 or fp64) -> (d, k) centroid
// sums and sizes in dataT: copies added in index order in fp64, rounded once.
template <typename A>
__global__ void km_to_dk_kernel(const A *copies, int n_copies, float *out_c, float *out_sizes,
                                int64_t d, int64_t k, int64_t k_pad, int64_t d4, FxAcc fx,
                                const MixedConsts *consts, const LoopState *guard) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    const int64_t cs = k_pad * d4 + k_pad;
    // consecutive threads read consecutive words of every copy
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < k * d4 + k;
         e += (int64_t)gridDim.x * blockDim.x) {
        const bool is_size = e >= k * d4;
        const int64_t off = is_size ? k_pad * d4 + (e - k * d4) : e;
        const int64_t j = e / d4, f = e % d4;
        if (!is_size && f >= d) continue;
        // the integer totals (exact to one rounding), then the copies added
        // in index order; loads issued eight ahead of the adds
        double acc = 0.0;
        if (fx.hi != nullptr && consts->fx_ok) {
            long long h = 0;
            unsigned long long l = 0;
            for (int c = 0; c < fx.copies; ++c) {
                h += fx.hi[(int64_t)c * fx.stride + e];
                l += fx.lo[(int64_t)c * fx.stride + e];
            }
            acc = ((double)h * 4294967296.0 + (double)l) * (1.0 / (double)pow2f(consts->fx_shift));
        }
        int c = 0;
        for (; c + 8 <= n_copies; c += 8) {
            A v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = copies[(int64_t)(c + u) * cs + off];
#pragma unroll
            for (int u = 0; u < 8; ++u) acc += (double)v[u];
        }
        for (; c < n_copies; ++c) acc += (double)copies[(int64_t)c * cs + off];
        if (is_size)
            out_sizes[e - k * d4] = (float)acc;
        else
            out_c[f * k + j] = (float)acc;
    }
}

__global__ void reset_kernel(float *sums32, double *acc64, int64_t count, int acc_f64,
                             int *n_flagged, FxAcc fx, int64_t fx_count, const LoopState *guard) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < count;
         e += (int64_t)gridDim.x * blockDim.x) {
        if (acc_f64)
            acc64[e] = 0.0;
        else
            sums32[e] = 0.f;
    }
    if (fx.hi != nullptr)
        for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
             e < fx_count * fx.copies; e += (int64_t)gridDim.x * blockDim.x) {
            fx.hi[e] = 0;
            fx.lo[e] = 0ull;
        }
    if (blockIdx.x == 0 && threadIdx.x == 0) *n_flagged = 0;
}

// Copies the flagged count of this pass into the per-fit statistics.
__global__ void stats_kernel(const int *n_flagged, long long *last, long long *total,
                             const LoopState *guard) {
    if (guard != nullptr && *reinterpret_cast<const volatile int *>(&guard->done)) return;
    *last = *n_flagged;
    *total += *n_flagged;
}

using MixedKernel = void (*)(MixedArgs);

// The widest pass each feature-block count takes (shared memory); column
// passes always use it, so only those shapes have a multi-pass kernel.
constexpr int max_chunks(int nkb) { return nkb == 1 ? 4 : (nkb == 2 ? 2 : 1); }

template <int BF16, int NKB>
MixedKernel pick_chunks(int nch, bool multi) {
    constexpr int W = max_chunks(NKB);
    if (multi) return nch == W ? mixed_assign_kernel<BF16, NKB, W, true> : nullptr;
    switch (nch) {
        case 1: return mixed_assign_kernel<BF16, NKB, 1, false>;
        case 2: return W >= 2 ? mixed_assign_kernel<BF16, NKB, (W >= 2 ? 2 : 1), false> : nullptr;
        case 3: return W >= 3 ? mixed_assign_kernel<BF16, NKB, (W >= 3 ? 3 : 1), false> : nullptr;
        case 4: return W >= 4 ? mixed_assign_kernel<BF16, NKB, (W >= 4 ? 4 : 1), false> : nullptr;
        default: return nullptr;
    }
}

// Kernel for (operand type, 64-feature blocks, 256-column chunks per pass,
// column passes or one).
MixedKernel pick_kernel(int bf16, int nkb, int nch, bool multi = false) {
    switch (nkb) {
        case 1: return bf16 ? pick_chunks<1, 1>(nch, multi) : pick_chunks<0, 1>(nch, multi);
        case 2: return bf16 ? pick_chunks<1, 2>(nch, multi) : pick_chunks<0, 2>(nch, multi);
        case 3: return bf16 ? pick_chunks<1, 3>(nch, multi) : pick_chunks<0, 3>(nch, multi);
        case 4: return bf16 ? pick_chunks<1, 4>(nch, multi) : pick_chunks<0, 4>(nch, multi);
        default: return nullptr;
    }
}

// Up to 4 feature blocks (d <= 256) fit next to one 256-column chunk.
constexpr int kMaxFeatureBlocks = 4;

// Column chunks per pass and X-ring depth for nkb feature blocks: the widest
// pass (at most kMaxChunks chunks, and no wider than needed for kp columns)
// that fits shared memory with a ring of at least two stages, else one stage.
bool pass_plan(int nkb, int64_t kp, int64_t d4, int *nch_out, int *stages_out) {
    const int want = (int)std::min<int64_t>(max_chunks(nkb), kp / kChunkN);
    for (int nch = want; nch >= 1; --nch) {
        if (pick_kernel(0, nkb, nch) == nullptr) continue;
        for (int st = 4; st >= 1; --st)
            if (smem_layout(nkb, (int64_t)nch * kChunkN, d4, st).total <= kSmemLimit) {
                if (st == 1 && nch > 1) break;  // a narrower pass keeps a two-stage ring
                *nch_out = nch;
                *stages_out = st;
                return true;
            }
    }
    return false;
}

unsigned grid1d(int64_t work, int block, int cap = 8192) {
    int64_t g = ceil_div<int64_t>(work, block);
    return (unsigned)std::max<int64_t>(1, std::min<int64_t>(g, cap));
}

}  // namespace

// ---------------------------------------------------------------------------
// Mixed-form variant choice.  A variant forced process-wide (a test hook) or
// for the fits the autotuner creates on this thread overrides the tuner.
std::atomic<int> g_force_mixed_variant{-1};
thread_local int tl_force_mixed_variant = -1;
// Fits created while this is set use a cached choice or the default, never
// time variants (the request server: no measurement on a request's path).
thread_local bool tl_mixed_lookup_only = false;

int forced_variant() {
    const int g = g_force_mixed_variant.load();
    return g >= 0 ? g : tl_force_mixed_variant;
}

int64_t pow2_at_least(int64_t v) {
    int64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

template <typename I>
int make_mixed_fit_impl(const FitParams<float, I> &p, int form, std::unique_ptr<FitBase> *out);

// Times each candidate variant on a synthetic fit (Gaussian blobs of d
// features, k clusters) for four iterations after one warm-up, and caches the
// fastest per (d, k, form, size class).  Fits of at least 32 tiles per SM
// ("large") are timed with 48 tiles per SM, smaller ones with 8: the
// per-CTA costs of the fixed-point sums (zeroing and adding the shared-memory
// copies) weigh on few tiles, not on many.  KMC_TUNE=0 keeps the default (the
// first candidate).
int tune_mixed_variant(int64_t d, int64_t k, int form, bool large, const std::vector<int> &cand,
                       cudaStream_t s, int *code) {
    Range range("kmc.tune_mixed_variant");
    *code = cand.front();
    if (const char *e = std::getenv("KMC_TUNE"))
        if (e[0] == '0') return KMC_OK;
    const char *tag = form == KMC_FORM_MIXED_BF16 ? (large ? "mixed-bf16-large" : "mixed-bf16")
                                                  : (large ? "mixed-fp16-large" : "mixed-fp16");
    int cached = -1;
    if (tune_lookup(d, k, tag, &cached) &&
        std::find(cand.begin(), cand.end(), cached) != cand.end()) {
        *code = cached;
        return KMC_OK;
    }
    if (tl_mixed_lookup_only) return KMC_OK;
    const int64_t n = (int64_t)num_sms() * kTileM * (large ? 48 : 8);
    Scratch mem;
    const size_t oX = 0, oC0 = oX + align256(sizeof(float) * n * d);
    const size_t oC = oC0 + align256(sizeof(float) * d * k), oCn = oC + align256(sizeof(float) * d * k);
    const size_t ow = oCn + align256(sizeof(float) * d * k), ol = ow + align256(sizeof(float) * n);
    const size_t oi = ol + align256(sizeof(int32_t) * n);
    KMC_TRY(mem.alloc(oi + align256(sizeof(int32_t) * k), s));
    char *b = mem.as<char>();
    float *X = reinterpret_cast<float *>(b + oX), *C0 = reinterpret_cast<float *>(b + oC0);
    float *C = reinterpret_cast<float *>(b + oC), *Cn = reinterpret_cast<float *>(b + oCn);
    float *w = reinterpret_cast<float *>(b + ow);
    int32_t *lab = reinterpret_cast<int32_t *>(b + ol), *idx = reinterpret_cast<int32_t *>(b + oi);
    KMC_TRY(launch_blobs(X, n, d, k, -10.f, 10.f, 1.f, 1.f, 77, s));
    KMC_TRY(launch_fill<float>(w, 1.f, n, s));
    std::vector<int32_t> rows;
    seeded_rows(n, k, 78, &rows);
    KMC_CUDA_TRY(cudaMemcpyAsync(idx, rows.data(), sizeof(int32_t) * k, cudaMemcpyHostToDevice, s));
    KMC_TRY(launch_gather_rows(X, n, d, idx, k, C0, s));
    KMC_CUDA_TRY(cudaStreamSynchronize(s));  // rows (host vector) copied
    cudaEvent_t e0, e1;
    KMC_CUDA_TRY(cudaEventCreate(&e0));
    KMC_CUDA_TRY(cudaEventCreate(&e1));
    float best_ms = 0.f;
    int best = -1;
    for (int c : cand) {
        FitParams<float, int32_t> q;
        q.X = X;
        q.w = w;
        q.centroids = C;
        q.new_centroids = Cn;
        q.labels = lab;
        q.n = n;
        q.d = d;
        q.k = k;
        q.tol = 0.0;
        q.max_iter = 1000;
        q.stream = s;
        if (cudaMemcpyAsync(C, C0, sizeof(float) * d * k, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
            continue;
        tl_force_mixed_variant = c;
        std::unique_ptr<FitBase> fit;
        int rc = make_mixed_fit_impl<int32_t>(q, form, &fit);
        tl_force_mixed_variant = -1;
        if (rc != KMC_OK) continue;
        float ms = 0.f;
        rc = fit->enqueue_iteration();
        if (rc == KMC_OK) rc = cudaEventRecord(e0, s) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
        for (int it = 0; it < 4 && rc == KMC_OK; ++it) rc = fit->enqueue_iteration();
        if (rc == KMC_OK) rc = cudaEventRecord(e1, s) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
        if (rc == KMC_OK) rc = cudaEventSynchronize(e1) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
        if (rc == KMC_OK) rc = cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess ? KMC_OK : KMC_ERR_CUDA;
        if (rc == KMC_OK && (best < 0 || ms < best_ms)) {
            best_ms = ms;
            best = c;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    KMC_CUDA_TRY(cudaStreamSynchronize(s));
    if (best >= 0) {
        tune_record(d, k, tag, best);
        *code = best;
    }
    return KMC_OK;
}

template <typename I>
struct MixedFit : PlainFit<float, I> {
    using Base = PlainFit<float, I>;
    int bf16 = 0;
    int nkb = 1;
    int acc_f64 = 0;
    int stages = 2;
    int64_t k_pad = 0, d4 = 0, ntiles = 0;
    Scratch mws;
    uint8_t *ximg = nullptr, *cimg = nullptr;
    float *nx = nullptr, *ndx = nullptr, *ct = nullptr, *xrow = nullptr;
    float *sums32 = nullptr;
    double *acc64 = nullptr;
    int n_copies = 1;  // private copies of the cluster sums (one per CTA)
    float *cn2 = nullptr, *dcn = nullptr;
    MixedConsts *consts = nullptr;
    uint4 *cand = nullptr;
    int *flagged = nullptr, *n_flagged = nullptr, *err_dev = nullptr;
    long long *stats = nullptr;  // [0] last pass, [1] total
    long long wait_limit = kWaitClocks;
    int stall_once = 0;

    int set_wait_limit(long long clocks, int stall) override {
        wait_limit = clocks > 0 ? clocks : kWaitClocks;
        stall_once = stall != 0;
        return KMC_OK;
    }

    // The one-time conversion reads X in either layout; afterwards every
    // kernel reads the row-major fp32 copy.
    bool reads_rowmajor() const override { return true; }
    bool uses_private_copies() const override { return false; }
    void x_view(const float **x, int64_t *fs, int64_t *ss) const override {
        *x = xrow;
        *fs = 1;
        *ss = d4;
    }

    int nch = 1;     // 256-column chunks per pass
    int passes = 1;  // column passes per assignment (n_clusters beyond one pass)
    float *pmax = nullptr;
    int variant = 0;    // 10 stages + fixed-point columns per thread (0: none)
    int64_t own_k = 0;  // > 0: fixed-point sums accumulated per CTA in shared memory
    int own_f = 1;      // packed columns per update thread in those sums
    int *xq = nullptr;  // [n][d4 + 4] packed fixed-point terms
    long long *fxhi = nullptr;           // their integer totals (high words)
    unsigned long long *fxlo = nullptr;  // (low words)
    // Up to 32 features (fits with weights): packed terms and integer totals
    // for every accumulating kernel -- the assignment's fixed-point sums when
    // its variant has them, the recheck and the column passes' combine.
    bool fx_on = false;
    FxAcc fx_acc() const {
        return fx_on ? FxAcc{xq, fxhi, fxlo, this->prm.k * d4 + this->prm.k, n_copies}
                     : FxAcc{nullptr, nullptr, nullptr, 0, 1};
    }

    static bool supported(int64_t d, int64_t k) {
        const int nk = (int)ceil_div<int64_t>(std::max<int64_t>(d, 1), 64);
        if (nk > kMaxFeatureBlocks || k < 1) return false;
        const int64_t kp = ceil_div<int64_t>(k, kChunkN) * kChunkN;
        const int64_t dd = ceil_div<int64_t>(std::max<int64_t>(d, 1), 4) * 4;
        int c = 0, st = 0;
        return pass_plan(nk, kp, dd, &c, &st);
    }

    int init_mixed(int form) {
        const FitParams<float, I> &p = this->prm;
        cudaStream_t s = p.stream;
        bf16 = (form == KMC_FORM_MIXED_BF16) ? 1 : 0;
        nkb = (int)ceil_div<int64_t>(std::max<int64_t>(p.d, 1), 64);
        d4 = ceil_div<int64_t>(std::max<int64_t>(p.d, 1), 4) * 4;
        ntiles = ceil_div<int64_t>(p.n, kTileM);
        if (!pass_plan(nkb, ceil_div<int64_t>(p.k, kChunkN) * kChunkN, d4, &nch, &stages)) {
            set_error("mixed form: operands do not fit in shared memory");
            return KMC_ERR_UNSUPPORTED;
        }
        // the centroid image has whole passes of rows (zero padding)
        passes = (int)ceil_div<int64_t>(p.k, (int64_t)nch * kChunkN);
        k_pad = (int64_t)passes * nch * kChunkN;
        // Cluster sums: up to 32 features, float64 reductions per feature
        // (a few per sample; they keep the trajectory on the float64
        // reference's), beyond that float32 four-wide reductions.
        acc_f64 = d4 <= 32 ? 1 : 0;
        // float64 sums that fit shared memory next to the operands (keeping a
        // ring of at least two stages) are formed per CTA in fixed point: the
        // deepest ring that fits, then as many columns per update thread as
        // fit beside it.  One column per thread leaves a single copy, whose
        // read-modify-write chain (one row after another) is slower than the
        // float64 reductions.  Fits only: a prediction has no weights and no
        // sums.
        //
        // The choice (ring depth, and for these sums fixed point with 4 or 2
        // columns per thread or float64 reductions) is a variant code
        // 10 stages + f (f = 0: no fixed point).  The autotuner times the
        // variants that fit on a synthetic fit once per (d, power-of-two
        // bucket of k, form, size class) and caches the fastest; the rule
        // above is the default when tuning is off.
        {
            std::vector<int> cand;
            const int64_t kb = std::min<int64_t>(k_pad, std::max<int64_t>(pow2_at_least(p.k), 1));
            const bool fx_shape = acc_f64 && passes == 1 && p.w != nullptr;
            for (int st = stages; st >= 2; --st) {
                if (fx_shape)
                    for (int f : {4, 2})
                        if (smem_layout(nkb, k_pad, d4, st, kb, f).total <= kSmemLimit)
                            cand.push_back(10 * st + f);
                if (smem_layout(nkb, k_pad, d4, st).total <= kSmemLimit) cand.push_back(10 * st);
            }
            if (cand.empty()) cand.push_back(10 * stages);
            int code = cand.front();  // deepest ring, widest fixed-point sums
            const int forced = forced_variant();
            if (forced >= 0) {
                if (std::find(cand.begin(), cand.end(), forced) == cand.end()) {
                    set_error("mixed form: variant %d does not fit this shape", forced);
                    return KMC_ERR_INVALID_ARGUMENT;
                }
                code = forced;
            } else if (cand.size() > 1) {
                // a measurement that cannot run (out of memory, say) leaves the
                // default: tuning never fails a fit
                const bool large = ntiles >= 32 * (int64_t)num_sms();
                if (tune_mixed_variant(p.d, kb, form, large, cand, s, &code) != KMC_OK)
                    code = cand.front();
            }
            variant = code;
            stages = code / 10;
            if (code % 10 != 0) {
                own_k = p.k;
                own_f = code % 10;
            }
        }
        size_t off = 0;
        auto take = [&](size_t bytes) {
            size_t o = off;
            off += align256(bytes);
            return o;
        };
        const size_t o_x = take((size_t)std::max<int64_t>(ntiles, 1) * nkb * kTileBytes);
        const size_t o_c = take(cimg_bytes(nkb, k_pad));
        const size_t o_ct = take(sizeof(float) * k_pad * d4);
        const size_t o_nx = take(sizeof(float) * p.n);
        const size_t o_ndx = take(sizeof(float) * p.n);
        // Small sums get private copies, one per CTA of the assignment for
        // large n: their few addresses would otherwise serialise the
        // reductions of all SMs.  Every iteration zeroes and reduces every
        // copy, so small fits get one copy per eight tiles instead (a
        // 50K-sample fit spent more time there than in its assignment).
        // Large sums (c3-sized, 266 KB) stay single: per-CTA copies would
        // crowd L2 for less contention than they remove.
        n_copies = (k_pad * d4 <= 32768)
                       ? (int)std::max<int64_t>(1, std::min<int64_t>(ntiles / 8, num_sms()))
                       : 1;
        const int64_t csz = (int64_t)n_copies * (k_pad * d4 + k_pad);
        const size_t o_s32 = take(acc_f64 ? 16 : sizeof(float) * csz);
        const size_t o_a64 = take(acc_f64 ? sizeof(double) * csz : 16);
        const size_t o_xf = take(sizeof(float) * std::max<int64_t>(p.n, 1) * d4);
        fx_on = acc_f64 && p.w != nullptr;
        const size_t o_xq = take(fx_on ? sizeof(int) * std::max<int64_t>(p.n, 1) * (d4 + 4) : 16);
        const size_t o_fx = take(fx_on ? 2 * sizeof(long long) * (size_t)n_copies *
                                                 (size_t)(p.k * d4 + p.k)
                                           : 16);
        const size_t o_cn2 = take(sizeof(float) * p.k);
        const size_t o_dcn = take(sizeof(float) * p.k);
        const size_t o_cst = take(sizeof(MixedConsts));
        // candidate masks (and best scores) of every column pass
        const size_t o_cand = take(sizeof(uint4) * (size_t)p.n * passes);
        const size_t o_pmax = take(passes > 1 ? sizeof(float) * (size_t)p.n * passes : 16);
        const size_t o_flg = take(sizeof(int) * p.n);
        const size_t o_cnt = take(sizeof(int) * 4);
        const size_t o_st = take(sizeof(long long) * 2);
        KMC_TRY(mws.alloc(off, s));
        char *b = mws.as<char>();
        ximg = reinterpret_cast<uint8_t *>(b + o_x);
        cimg = reinterpret_cast<uint8_t *>(b + o_c);
        ct = reinterpret_cast<float *>(b + o_ct);
        nx = reinterpret_cast<float *>(b + o_nx);
        ndx = reinterpret_cast<float *>(b + o_ndx);
        sums32 = reinterpret_cast<float *>(b + o_s32);
        acc64 = reinterpret_cast<double *>(b + o_a64);
        xrow = reinterpret_cast<float *>(b + o_xf);
        xq = reinterpret_cast<int *>(b + o_xq);
        if (fx_on) {
            fxhi = reinterpret_cast<long long *>(b + o_fx);
            fxlo = reinterpret_cast<unsigned long long *>(fxhi + n_copies * (p.k * d4 + p.k));
        }
        cn2 = reinterpret_cast<float *>(b + o_cn2);
        dcn = reinterpret_cast<float *>(b + o_dcn);
        consts = reinterpret_cast<MixedConsts *>(b + o_cst);
        cand = reinterpret_cast<uint4 *>(b + o_cand);
        pmax = reinterpret_cast<float *>(b + o_pmax);
        flagged = reinterpret_cast<int *>(b + o_flg);
        n_flagged = reinterpret_cast<int *>(b + o_cnt);
        err_dev = n_flagged + 1;
        stats = reinterpret_cast<long long *>(b + o_st);
        KMC_CUDA_TRY(cudaMemsetAsync(consts, 0, sizeof(MixedConsts), s));
        KMC_CUDA_TRY(cudaMemsetAsync(n_flagged, 0, sizeof(int) * 4, s));
        KMC_CUDA_TRY(cudaMemsetAsync(stats, 0, sizeof(long long) * 2, s));
        // one-time conversion of X (charged to the fit, reported separately)
        absmax_kernel<<<grid1d(p.n * p.d, 256, 4096), 256, 0, s>>>(p.X, p.n * p.d,
                                                                    &consts->xmax_bits);
        KMC_TRY(check_launch("absmax"));
        sigma_kernel<<<1, 1, 0, s>>>(consts, bf16, p.d);
        KMC_TRY(check_launch("sigma"));
        if (fx_on) {
            absmax_kernel<<<grid1d(p.n, 256, 4096), 256, 0, s>>>(p.w, p.n, &consts->wmax_bits);
            KMC_TRY(check_launch("absmax_w"));
            // rows one CTA of the assignment handles at most
            const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ntiles, num_sms()));
            const double rows = (double)ceil_div<int64_t>(std::max<int64_t>(ntiles, 1), grid) * kTileM;
            fixed_scale_kernel<<<1, 1, 0, s>>>(consts, rows);
            KMC_TRY(check_launch("fixed_scale"));
            this->launches += 2;
        }
        {
            auto xk = bf16 ? x_image_kernel<1> : x_image_kernel<0>;
            const size_t xsm = x_image_smem(nkb);
            if (xsm > 48 * 1024)
                KMC_CUDA_TRY(cudaFuncSetAttribute(xk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                  (int)xsm));
            const int64_t xg = std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)num_sms() * 8));
            xk<<<(unsigned)xg, kXImageThreads, xsm, s>>>(p.X, p.n, p.d, d4, nkb, ntiles, consts,
                                                         ximg, xrow, nx, ndx, p.x_rowmajor);
        }
        KMC_TRY(check_launch("x_image"));
        this->launches += 3;
        if (fx_on) {
            fx_pack_kernel<<<grid1d(p.n * (d4 + 4), 256, 8192), 256, 0, s>>>(xrow, p.w, p.n, d4,
                                                                           consts, xq);
            KMC_TRY(check_launch("fx_pack"));
            this->launches += 1;
        }
        return KMC_OK;
    }

    int centroid_prep(const float *cur, const LoopState *guard) {
        const FitParams<float, I> &p = this->prm;
        cudaStream_t s = p.stream;
        const int64_t lanes = k_pad * (nkb <= 1 ? 8 : (nkb == 2 ? 16 : 32));  // c_image's G
        if (bf16)
            c_image_kernel<1><<<grid1d(lanes, 128, 4096), 128, 0, s>>>(
                cur, this->hn, p.d, p.k, k_pad, nkb, consts, cimg, cn2, dcn, ct, d4, guard);
        else
            c_image_kernel<0><<<grid1d(lanes, 128, 4096), 128, 0, s>>>(
                cur, this->hn, p.d, p.k, k_pad, nkb, consts, cimg, cn2, dcn, ct, d4, guard);
        KMC_TRY(check_launch("c_image"));
        bound_kernel<<<1, 1024, 0, s>>>(cn2, dcn, this->hn, p.d, p.k, bf16, consts, guard);
        return check_launch("bound");
    }

    int assign_pass(const float *cur, int update, const LoopState *guard) {
        const FitParams<float, I> &p = this->prm;
        cudaStream_t s = p.stream;
        KMC_TRY(centroid_prep(cur, guard));
        const int64_t csz = (int64_t)n_copies * (k_pad * d4 + k_pad);
        reset_kernel<<<grid1d(csz, 256, 4096), 256, 0, s>>>(sums32, acc64, csz, acc_f64,
                                                           n_flagged, fx_acc(), p.k * d4 + p.k,
                                                           guard);
        KMC_TRY(check_launch("mixed_reset"));
        MixedArgs a;
        a.ximg = ximg;
        a.cimg = cimg;
        a.nx = nx;
        a.ndx = ndx;
        a.consts = consts;
        a.X = p.X;
        a.w = p.w;
        a.labels = p.labels;
        a.sums32 = sums32;
        a.acc64 = acc64;
        a.n_copies = n_copies;
        a.xrow = xrow;
        a.cand = cand;
        a.flagged = flagged;
        a.n_flagged = n_flagged;
        a.err_global = err_dev;
        a.guard = guard;
        a.n = p.n;
        a.d = p.d;
        a.k = p.k;
        a.k_pad = k_pad;
        a.d4 = d4;
        a.update = update;
        a.label64 = sizeof(I) == 8 ? 1 : 0;
        a.acc_f64 = acc_f64;
        a.stages = stages;
        a.wait_limit = wait_limit;
        a.stall = stall_once;
        a.state = this->state;
        stall_once = 0;
        const int64_t pass_cols = (int64_t)nch * kChunkN;
        a.k_pad = pass_cols;
        a.k_img = k_pad;
        a.multi = passes > 1 ? 1 : 0;
        if (a.multi) a.update = 0;  // the combine accumulates the certified samples
        a.own_k = a.multi ? 0 : own_k;
        a.own_f = own_f;
        a.xq = xq;
        a.fx = fx_acc();
        const SmemLayout L = smem_layout(nkb, pass_cols, d4, stages, a.own_k, a.own_f);
        if ((L.ostage & 15) != 0 || (L.osum & 15) != 0) {
            set_error("mixed form: misaligned shared-memory sums layout");
            return KMC_ERR_CUDA;
        }
        auto kern = pick_kernel(bf16, nkb, nch, a.multi != 0);
        if (kern == nullptr) {
            set_error("mixed form: no kernel for %d feature blocks and %d chunks", nkb, nch);
            return KMC_ERR_UNSUPPORTED;
        }
        KMC_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)L.total));
        const int64_t grid = std::max<int64_t>(1, std::min<int64_t>(ntiles, num_sms()));
        if (p.n > 0) {
            for (int ps = 0; ps < passes; ++ps) {
                a.col0 = (int64_t)ps * pass_cols;
                a.cand = cand + (int64_t)ps * p.n;
                a.pmax = pmax + (a.multi ? (int64_t)ps * p.n : 0);
                kern<<<(unsigned)grid, kThreadsMixed, L.total, s>>>(a);
                KMC_TRY(check_launch("mixed_assign"));
                a.stall = 0;
            }
            if (a.multi) {
                combine_kernel<<<grid1d(p.n, 256, num_sms() * 8), 256, 0, s>>>(
                    pmax, cand, passes, pass_cols, nx, ndx, consts, xrow, p.w, p.labels, a.label64,
                    update, acc_f64, sums32, acc64, k_pad, d4, n_copies, flagged, n_flagged, p.n,
                    p.k, guard, fx_acc());
                KMC_TRY(check_launch("mixed_combine"));
            }
        }
        // enough CTAs for every sample flagged (8 warps of 32 per CTA round),
        // at most 8 per SM
        const int64_t rgrid = std::max<int64_t>(
            1, std::min<int64_t>((int64_t)num_sms() * 8, ceil_div<int64_t>(p.n, kRecheckThreads)));
        recheck_kernel<<<(unsigned)rgrid, kRecheckThreads, 0, s>>>(
            xrow, ct, this->hn, p.w, cand, flagged, n_flagged, p.n, p.d, p.k, d4, p.labels,
            a.label64, update, acc_f64, sums32, acc64, k_pad, n_copies, guard, passes, pass_cols,
            fx_acc(), consts);
        KMC_TRY(check_launch("mixed_recheck"));
        stats_kernel<<<1, 1, 0, s>>>(n_flagged, stats, stats + 1, guard);
        return check_launch("mixed_stats");
    }

    int step_assign_and_accumulate(const float *cur, int64_t *n_launches) override {
        *n_launches = 6 + (passes > 1 ? passes : 0);
        return assign_pass(cur, 1, this->state);
    }

    int reduce_step(float *nxt) override {
        const FitParams<float, I> &p = this->prm;
        cudaStream_t s = p.stream;
        if (acc_f64)
            km_to_dk_kernel<double><<<grid1d(p.k * d4 + p.k, 256, 4096), 256, 0, s>>>(
                acc64, n_copies, nxt, this->sizes, p.d, p.k, k_pad, d4, fx_acc(), consts,
                this->state);
        else
            km_to_dk_kernel<float><<<grid1d(p.k * d4 + p.k, 256, 4096), 256, 0, s>>>(
                sums32, n_copies, nxt, this->sizes, p.d, p.k, k_pad, d4,
                FxAcc{nullptr, nullptr, nullptr, 0, 1}, consts, this->state);
        KMC_TRY(check_launch("km_to_dk"));
        return launch_empty_list<float, I>(this->sizes, this->empty_list, this->n_empty, p.k, s,
                                           this->state);
    }

    int final_assignment() override { return assign_pass(this->prm.centroids, 0, nullptr); }

    int counters(int64_t *last, int64_t *total, int *device_error) override {
        long long h[2] = {0, 0};
        int e = 0;
        KMC_CUDA_TRY(cudaMemcpyAsync(h, stats, sizeof(h), cudaMemcpyDeviceToHost,
                                     this->prm.stream));
        KMC_CUDA_TRY(cudaMemcpyAsync(&e, err_dev, sizeof(int), cudaMemcpyDeviceToHost,
                                     this->prm.stream));
        KMC_CUDA_TRY(cudaStreamSynchronize(this->prm.stream));
        if (last) *last = h[0];
        if (total) *total = h[1];
        if (device_error) *device_error = e;
        return KMC_OK;
    }
};

template <typename I>
int make_mixed_fit_impl(const FitParams<float, I> &p, int form, std::unique_ptr<FitBase> *out) {
    if (!MixedFit<I>::supported(p.d, p.k)) {
        set_error("mixed form supports n_features <= %d (got d=%lld, k=%lld)",
                  64 * kMaxFeatureBlocks, (long long)p.d, (long long)p.k);
        return KMC_ERR_UNSUPPORTED;
    }
    auto f = std::make_unique<MixedFit<I>>();
    KMC_TRY(f->init(p));
    KMC_TRY(f->init_mixed(form));
    *out = std::move(f);
    return KMC_OK;
}

template <typename T, typename I>
int make_mixed_fit(const FitParams<T, I> &p, int form, std::unique_ptr<FitBase> *out) {
    if constexpr (!std::is_same<T, float>::value) {
        set_error("the mixed tensor-core form needs float32 data");
        return KMC_ERR_UNSUPPORTED;
    } else {
        return make_mixed_fit_impl<I>(p, form, out);
    }
}

void mixed_tuning_lookup_only(bool on) { tl_mixed_lookup_only = on; }

int force_mixed_variant(int code) {
    KMC_CHECK_ARG(code == -1 || (code >= 10 && code <= 44), "variant must be -1 or 10 s + f");
    g_force_mixed_variant.store(code);
    return KMC_OK;
}

int mixed_variant_of(FitBase *fit, int *code) {
    auto *m32 = dynamic_cast<MixedFit<int32_t> *>(fit);
    auto *m64 = dynamic_cast<MixedFit<int64_t> *>(fit);
    *code = m32 ? m32->variant : (m64 ? m64->variant : -1);
    return KMC_OK;
}

bool mixed_fit_supported(int64_t d, int64_t k) { return MixedFit<int32_t>::supported(d, k); }

int pack_fixed_term(float v, int shift) { return pack_fixed(v, 150 - shift); }

template int make_mixed_fit<float, int32_t>(const FitParams<float, int32_t> &, int,
                                            std::unique_ptr<FitBase> *);
template int make_mixed_fit<float, int64_t>(const FitParams<float, int64_t> &, int,
                                            std::unique_ptr<FitBase> *);
template int make_mixed_fit<double, int32_t>(const FitParams<double, int32_t> &, int,
                                             std::unique_ptr<FitBase> *);
template int make_mixed_fit<double, int64_t>(const FitParams<double, int64_t> &, int,
                                             std::unique_ptr<FitBase> *);

}  // namespace kmc
