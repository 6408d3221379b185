// Inline-PTX building blocks for the sm_103a tensor-core (tcgen05) Lloyd step:
// mbarriers with bounded waits, bulk global->shared copies, TMEM allocation,
// UMMA shared-memory / instruction descriptors, tcgen05.mma / commit / ld.
#pragma once

#include <cstdint>

namespace kmc {
namespace tc {

// A wait that has not completed after this many SM clocks (~2 s at 2 GHz) is
// treated as a hang: the waiter sets the CTA's error flag and gives up, and
// every other role sees the flag and winds down.
constexpr long long kWaitClocks = 4000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// Non-blocking test of the phase with the given parity.  The waits below poll
// it with a short sleep between polls.  The suspending form
// (mbarrier.try_wait with a suspend-time hint) is not used: with tensor-core
// kernels of several streams running at once, a thread suspended in it
// sometimes stayed asleep for seconds after the phase had completed (fits of
// the request server gave up their waits after the 2 s limit; with polling
// none did).
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.test_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase with the given parity.  Returns false (and raises the
// CTA error flag) after `limit` SM clocks, or as soon as another role has
// raised the flag.  After a few polls the waiter sleeps ~0.1 us between
// polls, so waiting warps leave the issue slots to the working ones.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *err,
                                          long long limit = kWaitClocks) {
    if (mbar_test(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_test(bar, parity)) return true;
        if (*err) return false;
        if (clock64() - t0 > limit) {
            *err = 1;
            return false;
        }
    }
}

// Wait used while winding down: it ignores the error flag and returns only
// when the phase completes (true) or after kWaitClocks (false).  It waits for
// work that was already issued -- bulk copies into this CTA's shared memory,
// committed tensor-core operations -- which always completes, so a CTA never
// frees TMEM or exits with such work still writing.
__device__ __forceinline__ bool mbar_wait_drain(uint64_t *bar, uint32_t parity, volatile int *err) {
    if (mbar_test(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_test(bar, parity)) return true;
        if (clock64() - t0 > kWaitClocks) {
            *err = 1;
            return false;
        }
    }
}

// 1-D bulk copy global -> shared, completion reported as tx bytes on `bar`.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
        "[%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// ---- tensor memory ----
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, kind::f16 (fp16 or bf16 inputs, fp32 accumulate).
__device__ __forceinline__ void mma_f16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                        uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every tcgen05 operation issued so far by this thread
// has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 32 lanes x 32 consecutive 32-bit columns -> 32 registers per thread.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, "
        "[%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ---- descriptors ----
// Shared-memory matrix descriptor, K-major operand in the 128-byte swizzled
// canonical layout: rows of 128 bytes (64 16-bit elements), 8-row groups of
// 1024 bytes stacked along M/N (stride byte offset 1024), swizzle mode 2.
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                    // leading byte offset (unused here)
    d |= (uint64_t)(1024u >> 4) << 32;         // stride byte offset
    d |= (uint64_t)1 << 46;                    // descriptor version
    d |= (uint64_t)2 << 61;                    // 128-byte swizzle
    return d;
}

// Same for a K extent of 16 16-bit elements (32-byte rows): 32-byte
// swizzle, 8-row groups of 256 bytes (stride byte offset 256), mode 6.
__device__ __forceinline__ uint64_t desc_sw32(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(256u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)6 << 61;  // 32-byte swizzle
    return d;
}

// Instruction descriptor, kind::f16: fp32 accumulator, A and B both fp16
// (bf16 = 0) or both bf16 (bf16 = 1), both K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int bf16, int M, int N) {
    return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) |
           ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// Byte offset of element (r, k) (k < 64) inside a 128-byte-swizzled K-major
// image whose base is 1024-byte aligned.
__host__ __device__ constexpr uint32_t sw128_offset(uint32_t r, uint32_t k) {
    return (r >> 3) * 1024u + (r & 7u) * 128u + ((((k >> 3) ^ (r & 7u)) & 7u) << 4) +
           (k & 7u) * 2u;
}

// Byte offset of element (r, k) (k < 16) inside a 32-byte-swizzled K-major
// image (8-row atoms of 256 bytes; the 16-byte halves of rows 4-7 of each
// atom are swapped), base 1024-byte aligned.
__host__ __device__ constexpr uint32_t sw32_offset(uint32_t r, uint32_t k) {
    return (r >> 3) * 256u + (r & 7u) * 32u + ((((k >> 3) ^ ((r & 7u) >> 2)) & 1u) << 4) +
           (k & 7u) * 2u;
}

}  // namespace tc
}  // namespace kmc
