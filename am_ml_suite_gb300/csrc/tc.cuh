// tc.cuh -- the Blackwell tensor-core primitives used by the convolution
// kernels: tensor-memory (TMEM) allocation and loads, tcgen05.mma issue and
// completion, shared-memory matrix descriptors, and tiled tensor copies
// (cp.async.bulk.tensor) that complete on an mbarrier.
//
// Operand layout without swizzle (K-major): a "core matrix" is 8 rows
// of 16 bytes (8 BF16 values of K) stored contiguously (128 bytes).  A tile of R
// rows and 16 values of K is two planes of R x 16 bytes -- K values 0-7 of every
// row, then K values 8-15 -- so consecutive 8-row groups are 128 bytes apart
// (the stride-dimension byte offset, SBO) and the two K halves R x 16 bytes
// apart (the leading-dimension byte offset, LBO).  A tiled tensor copy whose box
// is 8 channels wide lands in exactly this layout.  With swizzling (32, 64 or
// 128-byte rows) a copy whose box is 16, 32 or 64 channels wide lands in the
// matching swizzled layout (smem_desc_sw).
#pragma once
#include <cuda.h>
#include <stdint.h>

#include "bulk.cuh"

namespace amk {
namespace tc {

using bulk::smem_addr;

// ---- tiled tensor copies -------------------------------------------------------
__device__ __forceinline__ void prefetch_map(const CUtensorMap *m) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(m)) : "memory");
}
__device__ __forceinline__ void load_3d(void *dst, const CUtensorMap *m, int c0, int c1, int c2, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_addr(bar))
        : "memory");
}
__device__ __forceinline__ void load_5d(void *dst, const CUtensorMap *m, int c0, int c1, int c2, int c3, int c4,
                                        uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
        "%5, %6}], [%7];" ::"r"(smem_addr(dst)),
        "l"(reinterpret_cast<uint64_t>(m)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_addr(bar))
        : "memory");
}

// ---- tensor memory ---------------------------------------------------------------
// One full warp allocates `cols` columns (a power of two >= 32); the TMEM address
// is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// one plain arrival on an mbarrier
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 16 consecutive 32-bit columns of the warp's 32 lanes: thread i receives lane
// (lane quadrant of the warp) + i, columns col..col+15 of taddr.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---- MMA ----------------------------------------------------------------------------
// Shared-memory matrix descriptor, K-major without swizzle: start address, the
// leading (K-half) and stride (8-row group) byte offsets, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(const void *p, uint32_t lbo, uint32_t sbo) {
    const uint64_t a = smem_addr(p);
    return ((a >> 4) & 0x3FFFull) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}
// Swizzled K-major descriptor: rows of `row_bytes` (32, 64 or 128 bytes = the
// swizzle span, the K extent of one staged chunk), 8-row atoms row_bytes * 8 apart
// (SBO); the leading offset is unused.  The tile's base must sit on a 1024-byte
// boundary; a K step of 16 BF16 values inside a row advances the start by 32 bytes.
__device__ __forceinline__ uint64_t smem_desc_sw(const void *p, uint32_t row_bytes) {
    const uint64_t a = smem_addr(p);
    const uint64_t layout = row_bytes == 128 ? 2ull : row_bytes == 64 ? 4ull : 6ull;
    return ((a >> 4) & 0x3FFFull) | (1ull << 16) | ((uint64_t)(((row_bytes * 8) >> 4) & 0x3FFF) << 32) |
           (1ull << 46) | (layout << 61);
}
// Instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D (TMEM) (+)= A (smem) * B (smem)^T, issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(
            d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// The mbarrier receives one arrival once every MMA this thread issued so far has
// completed (their shared-memory operands may then be overwritten).
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

}  // namespace tc
}  // namespace amk
