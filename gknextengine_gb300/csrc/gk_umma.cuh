// gk_umma.cuh — 5th-generation tensor core (tcgen05) building blocks for sm_103a.
//
// Tensor memory allocation, single-thread MMA issue with shared-memory operand descriptors,
// MMA completion through mbarriers, and tensor-memory loads for the epilogue. Operands are
// bf16, K-major, in the 64-byte-swizzled layout that a TMA load with SWIZZLE_64B writes:
// rows of 64 bytes (32 bf16 along K), 8-row atoms of 512 bytes, the 16-byte chunk c of row r
// stored at chunk c ^ ((r >> 1) & 3). One MMA consumes K = 16 (32 bytes of each row); the
// second half of a 32-wide K chunk is addressed by advancing the descriptor's start address
// by 32 bytes, as the swizzle is a function of the address bits.
#pragma once
#include <cstdint>

#include "gk_tma.cuh"

namespace gk {

// Shared-memory matrix descriptor (tcgen05): start address, leading/stride byte offsets
// (16-byte units), descriptor version 1 at bits 46-47, layout type at bits 61-63
// (4 = 64-byte swizzle).
__device__ __forceinline__ uint64_t umma_desc_sw64(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;                 // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(512u >> 4) << 32;        // stride byte offset: 8-row atoms are 512 bytes apart
    d |= (uint64_t)1u << 46;                 // version
    d |= (uint64_t)4u << 61;                 // SWIZZLE_64B
    return d;
}

// Descriptor of a K-major operand without swizzle: core matrices of 8 rows x 16 bytes, each
// stored as 128 contiguous bytes; lbo: bytes between core matrices adjacent along K, sbo: bytes
// between core matrices adjacent along M (or N). Start, lbo and sbo are multiples of 16.
__device__ __forceinline__ uint64_t umma_desc_dense(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;                 // version; layout type 0 (no swizzle) at bits 61-63
    return d;
}

// Descriptor of a K-major operand with 32- or 64-byte swizzle: rows of rb bytes (16 or 32
// bf16 along K), 8-row groups sbo bytes apart (512 / 256 for dense atoms; any multiple of 16).
// The tensor core applies the swizzle on the absolute address bits, as the TMA does when it
// writes a box, so the operand may start at any row of a box (base offset 0).
__device__ __forceinline__ uint64_t umma_desc_swz(uint32_t saddr, uint32_t rb, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1u << 16;                      // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;                      // version
    d |= (uint64_t)(rb == 64u ? 4u : 6u) << 61;   // SWIZZLE_64B or SWIZZLE_32B
    return d;
}

// Instruction descriptor, kind::f16: D f32 (bits 4-5 = 1), A and B bf16 (bits 7-9, 10-12 = 1),
// both K-major, N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_bf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {   // whole warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {   // whole warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued so far has completed.
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 lanes x 16 consecutive 32-bit columns: thread t of the warp gets lane (warp's quarter + t).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace gk
