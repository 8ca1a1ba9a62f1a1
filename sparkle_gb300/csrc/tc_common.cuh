// tc_common.cuh -- sm_103a building blocks for the tensor-core kernels of the denoiser: mbarriers with
// time-bounded waits, TMA tiled loads, tcgen05 TMEM allocation / MMA issue / commit / loads, and the
// shared-memory and instruction descriptors of tcgen05.mma kind::f16 (BF16 in, FP32 accumulate).
//
// Layout conventions (operands K-major unless stated, 64-byte swizzle):
//   * an operand tile is R rows x 32 BF16 (64 B per row) written by TMA with CU_TENSOR_MAP_SWIZZLE_64B or
//     by threads applying the same XOR pattern (16-byte chunk c of row r lands at chunk c ^ ((r >> 1) & 3));
//   * 8 rows form a 512-byte swizzle atom, so the descriptor's stride byte offset is 512 and every tile
//     starts on a 1024-byte boundary;
//   * one kind::f16 MMA consumes K = 16 (32 bytes of each row); the second K step of a tile starts 32 bytes
//     further;
//   * an MN-major operand (the weight gradient's) is the same 64-byte-row atom with the roles swapped: a row
//     is 32 consecutive M (or N) elements, rows run along K, and one MMA's K = 16 rows span two atoms.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace spk {
namespace tc {

// Error bits reported by the tensor-core kernels (OR-ed into a device word the host reads back).
enum : uint32_t {
    kErrWaitTimeout = 1u << 0,   // an mbarrier wait gave up (1 s)
    kErrBadShape = 1u << 1,      // a launch shape the kernel does not support
};

constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// ---------------------------------------------------------------------------------------------
// mbarrier
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the phase of `bar` with the given parity to complete. Gives up after kWaitLimitNs, sets
// kErrWaitTimeout in *err and returns false; the caller then skips the rest of its work.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, uint32_t *err) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (;;) {
        for (int k = 0; k < 64; ++k)
            if (mbar_try_wait(bar, parity)) return true;
        if (global_ns() - t0 > kWaitLimitNs) {
            atomicOr(err, kErrWaitTimeout);
            return false;
        }
    }
}

// ---------------------------------------------------------------------------------------------
// TMA (tiled, global -> shared, completion on an mbarrier)
// ---------------------------------------------------------------------------------------------
__device__ __forceinline__ void tma_load_2d(void *dst, const void *tmap, uint64_t *bar, int c0, int c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::
            "r"(smem_u32(dst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_load_4d(void *dst, const void *tmap, uint64_t *bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// Tiled store shared -> global (bulk-group completion). Elements of the box outside the tensor are not
// written. The source must stay unchanged until tma_store_wait_read() returns.
__device__ __forceinline__ void tma_store_4d(const void *tmap, const void *src, int c0, int c1, int c2, int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.global.shared::cta.bulk_group [%0, {%2, %3, %4, %5}], [%1];" ::"l"(tmap),
        "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
        : "memory");
}

__device__ __forceinline__ void tma_store_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }

// Waits until every committed bulk store of this thread has finished reading shared memory.
__device__ __forceinline__ void tma_store_wait_read() {
    asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const void *tmap) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(tmap) : "memory");
}

// Generic-proxy shared-memory writes made visible to the async proxy (tcgen05.mma reads).
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ---------------------------------------------------------------------------------------------
// tcgen05
// ---------------------------------------------------------------------------------------------
// Whole warp: allocates `ncols` TMEM columns (power of two >= 32) and writes the base address to *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// D[tmem] (+)= A[smem] * B[smem]^T, one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrives once on `bar` when every MMA this thread issued before has completed.
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread `lane` of the warp receives row (lane base + lane). The
// load and its wait are one asm statement, so no use of the registers can be scheduled before the wait.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
}

// Shared-memory matrix descriptor: K-major, 64-byte swizzle, 8-row atoms 512 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw64(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);      // start address
    d |= static_cast<uint64_t>(1u) << 16;                      // leading byte offset (unused when swizzled)
    d |= static_cast<uint64_t>(512u >> 4) << 32;               // stride byte offset
    d |= static_cast<uint64_t>(1u) << 46;                      // descriptor version
    d |= static_cast<uint64_t>(4u) << 61;                      // SWIZZLE_64B
    return d;
}

// Shared-memory matrix descriptor of an MN-major operand, 64-byte swizzle: the tile is rows of 64 bytes
// (32 consecutive BF16 of the M or N dimension), one row per K index; 8 consecutive K rows form a 512-byte
// swizzle atom (stride byte offset = 512 between 8-row K groups) and 32-element M/N spans sit `span_bytes`
// apart (leading byte offset). This is the layout a 64-byte-swizzled TMA box {32 channels, pixels} lands
// in, with K = pixels.
__device__ __forceinline__ uint64_t smem_desc_mn_sw64(uint32_t saddr, uint32_t span_bytes) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);              // start address
    d |= static_cast<uint64_t>((span_bytes >> 4) & 0x3FFFu) << 16;   // leading byte offset: next M/N span
    d |= static_cast<uint64_t>(512u >> 4) << 32;                     // stride byte offset: next 8 K rows
    d |= static_cast<uint64_t>(1u) << 46;                            // descriptor version
    d |= static_cast<uint64_t>(4u) << 61;                            // SWIZZLE_64B
    return d;
}

// Instruction descriptor of kind::f16: BF16 A and B, FP32 D, M x N; A and B K-major unless `a_mn` /
// `b_mn` select the MN-major (transposed) reading of that operand.
__host__ __device__ constexpr uint32_t idesc_bf16(uint32_t m, uint32_t n, bool a_mn = false, bool b_mn = false) {
    return (1u << 4)                  // D format F32
           | (1u << 7)                // A format BF16
           | (1u << 10)               // B format BF16
           | ((a_mn ? 1u : 0u) << 15)  // A major: MN
           | ((b_mn ? 1u : 0u) << 16)  // B major: MN
           | ((n >> 3) << 17)         // N / 8
           | ((m >> 4) << 24);        // M / 16
}

// Byte offset of 16-byte chunk `chunk` (0..3) of row `row` in a 64-byte-swizzled K-major tile.
__host__ __device__ constexpr uint32_t sw64_offset(uint32_t row, uint32_t chunk) {
    return row * 64u + ((chunk ^ ((row >> 1) & 3u)) << 4);
}

}  // namespace tc
}  // namespace spk
