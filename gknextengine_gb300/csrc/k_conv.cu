// k_conv.cu — 3x3 "same" convolution as an implicit GEMM on the tcgen05 tensor cores.
//
// Building block of the learned denoiser (no counterpart in the reference, whose learned
// denoiser is the closed OIDN library). Activations are NHWC bf16 with channel counts that
// are multiples of 32; weights are [Cout][3][3][Cin] bf16; accumulation is FP32 in tensor
// memory.
//
// One CTA computes a tile of 8 x 16 pixels (M = 128) times all Cout (N <= 256) of one image:
//   K loop   9 taps x Cin / 32 chunks. For tap (dy, dx) and chunk c the A operand is the
//            4D TMA box {32 channels, 16 x, 8 y, 1 image} of the input shifted by the tap;
//            coordinates outside the image read zeros, which is the zero padding. The B
//            operand is the 2D box {32, Cout} of the weights at column tap * Cin + 32 c.
//            Both land 64-byte swizzled, the K-major layout of gk_umma.cuh.
//   stages   4 shared-memory stages; one thread issues the TMA loads (full barriers with
//            transaction counts), one thread issues two K = 16 MMAs per stage and frees
//            the stage with tcgen05.commit (empty barriers), then commits the accumulator.
//   epilogue all four warps read their 32 TMEM lanes (pixels) 16 columns at a time, add the
//            bias, apply ReLU, and store bf16 (or fp32) NHWC at a channel offset of a wider
//            tensor, which is how skip connections are concatenated without copies.
// Every barrier wait is bounded; a wait that runs out records the wait error bit in the
// device error word and the CTA skips its stores.
#include <algorithm>

#include <cuda_bf16.h>

#include "gk_umma.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kConvThreads = 128;
constexpr int kConvStages = 4;
constexpr int kTileX = 16, kTileY = 8;

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(kConvThreads) k_conv3x3(const __grid_constant__ CUtensorMap mx,
                                                             const __grid_constant__ CUtensorMap mw, ConvArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int a_bytes = kTileX * kTileY * 64;
    const int b_bytes = a.cout * 64;
    const int stage_bytes = (a_bytes + b_bytes + 1023) & ~1023;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kConvStages * stage_bytes);
    uint64_t* empty = full + kConvStages;
    uint64_t* accb = empty + kConvStages;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int x0 = blockIdx.x * kTileX, y0 = blockIdx.y * kTileY, img = blockIdx.z;
    const int kc = a.cin / 32, nk = 9 * kc;
    const uint32_t ncols = a.cout <= 32 ? 32u : a.cout <= 64 ? 64u : a.cout <= 128 ? 128u : 256u;

    if (tid == 0) {
        for (int s = 0; s < kConvStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accb, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 0) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0) {
        // producer: TMA loads of the A (shifted input) and B (weights) chunks
        int issued = 0;
        for (int k = 0; k < nk; ++k) {
            const int s = k % kConvStages;
            const uint32_t it = (uint32_t)(k / kConvStages);
            if (k >= kConvStages && !mbar_wait_bounded(&empty[s], (it - 1u) & 1u, a.err)) {
                *abort_flag = 1;
                break;
            }
            if (*abort_flag) break;
            const int tap = k / kc, c = k % kc;
            uint8_t* sa = smem + s * stage_bytes;
            mbar_expect_tx(&full[s], (uint32_t)(a_bytes + b_bytes));
            tma_load_4d(sa, &mx, c * 32, x0 + tap % 3 - 1, y0 + tap / 3 - 1, img, &full[s]);
            tma_load_2d(sa + a_bytes, &mw, tap * a.cin + c * 32, 0, &full[s]);
            ++issued;
        }
        // on an abort, let the loads already issued land before the CTA's memory goes away
        for (int k = std::max(0, issued - kConvStages); k < issued && *abort_flag; ++k)
            mbar_wait_bounded(&full[k % kConvStages], (uint32_t)(k / kConvStages) & 1u, a.err);
    } else if (warp == 1 && lane == 0) {
        // MMA issuer
        const uint32_t idesc = umma_idesc_bf16(128u, (uint32_t)a.cout);
        bool ok = true;
        for (int k = 0; k < nk; ++k) {
            const int s = k % kConvStages;
            if (!mbar_wait_bounded(&full[s], (uint32_t)(k / kConvStages) & 1u, a.err)) {
                *abort_flag = 1;
                ok = false;
                break;
            }
            tc_fence_after();
            const uint32_t sa = smem_u32(smem + s * stage_bytes), sb = sa + (uint32_t)a_bytes;
            umma_bf16(tmem, umma_desc_sw64(sa), umma_desc_sw64(sb), idesc, k != 0 ? 1u : 0u);
            umma_bf16(tmem, umma_desc_sw64(sa + 32u), umma_desc_sw64(sb + 32u), idesc, 1u);
            umma_commit(&empty[s]);
        }
        (void)ok;
        umma_commit(accb);   // arrives once every MMA issued above has completed
    }
    __syncwarp();

    // epilogue: TMEM lanes 32 w .. 32 w + 31 are the tile's pixels 32 w .. 32 w + 31
    const bool ready = mbar_wait_bounded(accb, 0u, a.err);
    __syncwarp();
    tc_fence_after();
    const int p = warp * 32 + lane;
    const int y = y0 + p / kTileX, x = x0 + p % kTileX;
    const bool inside = ready && !*abort_flag && y < a.H && x < a.W;
    const size_t pix = ((size_t)img * a.H + y) * a.W + x;
    for (int c0 = 0; c0 < a.cout; c0 += 16) {
        uint32_t r[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, r);
        tmem_ld_wait();
        if (!inside) continue;
        float v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            v[j] = __uint_as_float(r[j]) + (a.bias ? __ldg(&a.bias[c0 + j]) : 0.0f);
            if (a.flags & kConvRelu) v[j] = fmaxf(v[j], 0.0f);
        }
        if (a.flags & kConvF32Out) {
            float* o = reinterpret_cast<float*>(a.out) + pix * a.out_c + a.out_off + c0;
            for (int j = 0; j < 16 && c0 + j < a.n_store; ++j) o[j] = v[j];
        } else {
            uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.out) + pix * a.out_c + a.out_off + c0);
            o[0] = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]),
                              pack_bf16x2(v[6], v[7]));
            o[1] = make_uint4(pack_bf16x2(v[8], v[9]), pack_bf16x2(v[10], v[11]), pack_bf16x2(v[12], v[13]),
                              pack_bf16x2(v[14], v[15]));
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
}

}  // namespace

}  // namespace gk

using namespace gk;

cudaError_t gkrt_encode_tmap_bf16(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                  const uint64_t* strides_bytes, const uint32_t* box);

size_t gkrt_conv_smem_bytes(int cout) {
    const int stage = (kTileX * kTileY * 64 + cout * 64 + 1023) & ~1023;
    return (size_t)kConvStages * stage + 2 * kConvStages * 8 + 8 + 8 + 1024;
}

cudaError_t gkrt_launch_conv3x3(const void* x, const void* w, const ConvArgs& args, cudaStream_t st) {
    const bool f32 = (args.flags & kConvF32Out) != 0;
    if (args.cin % 32 || args.cin < 32 || args.cout % 16 || args.cout < 16 || args.cout > 256 || args.B < 1 ||
        args.H < 1 || args.W < 1 || (!f32 && (args.out_c % 16 || args.out_off % 16)) ||
        args.out_off + (f32 ? args.n_store : args.cout) > args.out_c || (f32 && args.n_store > args.cout) ||
        ((uintptr_t)x & 15u) || ((uintptr_t)w & 15u) || ((uintptr_t)args.out & 15u) || args.x_off % 8 ||
        (args.x_c > 0 && (args.x_c % 8 || args.x_off + args.cin > args.x_c)))
        return cudaErrorInvalidValue;
    CUtensorMap mx, mw;
    const uint64_t xc = (uint64_t)(args.x_c > 0 ? args.x_c : args.cin);
    const uint64_t xd[4] = {(uint64_t)args.cin, (uint64_t)args.W, (uint64_t)args.H, (uint64_t)args.B};
    const uint64_t xs[3] = {xc * 2, (uint64_t)args.W * xc * 2, (uint64_t)args.H * args.W * xc * 2};
    const uint32_t xb[4] = {32, kTileX, kTileY, 1};
    const void* xbase = static_cast<const uint8_t*>(x) + (size_t)args.x_off * 2;
    cudaError_t e = gkrt_encode_tmap_bf16(&mx, xbase, 4, xd, xs, xb);
    if (e != cudaSuccess) return e;
    const uint64_t wd[2] = {(uint64_t)9 * args.cin, (uint64_t)args.cout};
    const uint64_t ws[1] = {(uint64_t)9 * args.cin * 2};
    const uint32_t wb[2] = {32, (uint32_t)args.cout};
    e = gkrt_encode_tmap_bf16(&mw, w, 2, wd, ws, wb);
    if (e != cudaSuccess) return e;
    const size_t smem = gkrt_conv_smem_bytes(args.cout);
    e = cudaFuncSetAttribute(k_conv3x3, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const dim3 grid((args.W + kTileX - 1) / kTileX, (args.H + kTileY - 1) / kTileY, args.B);
    k_conv3x3<<<grid, kConvThreads, smem, st>>>(mx, mw, args);
    return cudaGetLastError();
}
