// gk_tma.cuh — 2D TMA tile loads into shared memory for the image passes (sm_103a).
//
// One elected thread arms an mbarrier with the expected byte count and issues
// cp.async.bulk.tensor.2d loads; the block waits on the barrier's phase. Every wait is
// bounded: if the barrier does not complete within the limit the kernel records
// kErrTmaWait in the device error word and the block skips its tile instead of hanging.
// Images are viewed as 2D arrays of 32-bit elements (a float4 pixel is 4 elements), so the
// innermost coordinate of every copy is a multiple of 16 bytes; loads starting outside the
// image read zeros, which is the out-of-range rule of the passes.
#pragma once
#include <cuda.h>
#include <cstdint>
#include <cuda_runtime.h>

namespace gk {

constexpr uint32_t kErrTmaWait = 4u;
constexpr int kTmaWaitLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0u;
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Bounded wait for phase `parity`; false (and kErrTmaWait recorded) when it does not complete.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t* err) {
    for (int i = 0; i < kTmaWaitLimit; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    atomicOr(err, kErrTmaWait);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace gk

// Host side: encode a 2D tensor map over an image of `elems_x` 32-bit elements per row,
// `rows` rows and `row_bytes` between rows (a multiple of 16), copied in boxes of
// box_x x box_y elements; elements outside the image read as zero.
cudaError_t gkrt_encode_tmap_2d(CUtensorMap* map, const void* base, uint32_t elems_x, uint32_t rows,
                                uint32_t row_bytes, uint32_t box_x, uint32_t box_y, bool is_float);
