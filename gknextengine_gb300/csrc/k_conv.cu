// k_conv.cu — 3x3 "same" convolution as an implicit GEMM on the tcgen05 tensor cores.
//
// Building block of the learned denoiser (no counterpart in the reference, whose learned
// denoiser is the closed OIDN library). Activations are NHWC bf16 with channel counts that
// are multiples of 32; weights are [Cout][3][3][Cin] bf16; accumulation is FP32 in tensor
// memory.
//
// Persistent, warp-specialised CTAs loop over tiles of 16 x 8 pixels (x by y, M = 128) times
// all Cout (N <= 256) of one image (outputs of up to 32 channels use the halo-tile kernel below):
//   K loop   9 taps x Cin / 32 chunks. For tap (dy, dx) and chunk c the A operand is the
//            4D TMA box {32 channels, 16 x, 8 y, 1 image} of the input shifted by the tap;
//            coordinates outside the image read zeros, which is the zero padding. The B
//            operand is the 2D box {32, Cout} of the weights at column tap * Cin + 32 c.
//            Both land 64-byte swizzled, the K-major layout of gk_umma.cuh.
//   rows     for outputs of up to 128 channels (the full-resolution layers especially, whose few
//            MMAs per loaded byte leave them bound by L2 reads of the nine shifted boxes) one stage
//            holds the box {32, 16 x, 10 y, 1} at horizontal shift dx and the three weight
//            boxes of taps (0..2, dx): the three vertical taps are the windows starting 0, 1
//            and 2 image rows (1024 bytes, a whole number of 64-byte swizzle atoms) into the
//            box, so each input chunk is read 3 times instead of 9.
//   stages   warp 0 issues the TMA loads into a ring of shared-memory stages (full barriers
//            with transaction counts) across tile boundaries; warp 1 issues two K = 16 MMAs per
//            stage, frees the stage with tcgen05.commit (empty barriers) and commits each
//            tile's accumulator; two accumulators in TMEM alternate between tiles, so the
//            epilogue of one tile runs under the MMAs of the next.
//   epilogue warps 2-5 (one per TMEM lane quarter) read their 32 lanes (pixels) 16 columns at
//            a time, add the bias (and an optional half-resolution parity addend), apply ReLU,
//            store bf16 (or fp32) NHWC at a channel offset of a wider tensor (skip connections
//            are concatenated without copies; bf16 through the warp's shared-memory exchange,
//            whole 32-byte sectors per store), optionally with the 2 x 2 average and the
//            nearest upsampling, and release the accumulator.
// The grid holds as many CTAs per SM as shared memory and the 512 TMEM columns allow.
// Every barrier wait is bounded; a wait that runs out records the wait error bit in the
// device error word and the CTA skips its stores.
#include <algorithm>

#include <cuda_bf16.h>

#include "gk_umma.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kConvThreads = 192;   // warp 0 TMA, warp 1 MMA, warps 2-5 epilogue
constexpr int kEpiThreads = 128;
constexpr int kTileX = 16, kTileY = 8;

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// Shared memory of the bf16 epilogue: 1 KB per epilogue warp (16-byte aligned).
constexpr int kEpiBuf = 4 * 1024 + 16;

__device__ __forceinline__ size_t shfl_size(size_t v, int src) {
    const uint32_t lo = __shfl_sync(0xFFFFFFFFu, (uint32_t)v, src);
    const uint32_t hi = __shfl_sync(0xFFFFFFFFu, (uint32_t)((uint64_t)v >> 32), src);
    return (size_t)(((uint64_t)hi << 32) | lo);
}

// The bf16 epilogue of 16 channels (c0 .. c0 + 15) of pixel (x, y) of image img: the plain
// store, and the optional pooled and upsampled outputs. Called by every lane of the warp
// (the pool's 2 x 2 block is four lanes of one warp: x-neighbour lane ^ 1, y-neighbour lane ^
// yl); the pooled average is (((0 + v(x, y)) + v(x + 1, y)) + v(x, y + 1)) + v(x + 1, y + 1) of
// the stored (bf16-rounded) values, times 1/4, rounded to bf16. The warp's 32 pixels pass their
// 32 bytes through ebuf (this warp's 1 KB of shared memory; 16-byte chunks swizzled by lane bit
// 2, so that neither side has bank conflicts), and each 32-byte sector of the output is then
// written whole by two lanes of one store instruction: lane-per-pixel stores wrote every sector
// in two 16-byte halves from separate instructions, twice the L2 write requests.
// Where a lane's stores of one tile go, the same for every channel group (computed once per
// tile): the two pixels whose 16-byte halves it stores (element offsets into out and, for the
// nearest upsampling, of the top-left of the 2 x 2 block in up), and the pooled pixel whose
// four channels it stores.
struct EpiDst {
    size_t o[2], u[2], p;
    bool in[2], pin;
};
__device__ __forceinline__ EpiDst epi_dst(const ConvArgs& a, int img, int x, int y, bool inside, int yl) {
    const int lane = threadIdx.x & 31, h = lane & 1;
    const size_t pix = ((size_t)img * a.H + y) * a.W + x;
    const size_t uq = ((size_t)img * 2 * a.H + 2 * (size_t)y) * (2 * (size_t)a.W) + 2 * (size_t)x;
    EpiDst d;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int src = (lane >> 1) + 16 * i;
        d.o[i] = shfl_size(pix, src) * a.out_c + a.out_off + 8 * h;
        d.in[i] = __shfl_sync(0xFFFFFFFFu, inside ? 1 : 0, src) != 0;
        d.u[i] = a.up_out ? shfl_size(uq, src) * a.up_c + a.up_off + 8 * h : 0;
    }
    d.p = 0;
    d.pin = false;
    if (a.pool_out) {
        const int h2 = a.H / 2, w2 = a.W / 2;
        const int b = yl == 16 ? 4 : 3;
        const int k = lane >> 2;
        const int tl = ((k >> (b - 1)) << (b + 1)) | ((k & ((1 << (b - 1)) - 1)) << 1);   // top-left lane
        const size_t pp = ((size_t)img * h2 + y / 2) * w2 + x / 2;
        const bool pvalid = !(x & 1) && !(y & 1) && x / 2 < w2 && y / 2 < h2;
        d.p = shfl_size(pp, tl) * a.pool_c + a.pool_off + 4 * (lane & 3);
        d.pin = __shfl_sync(0xFFFFFFFFu, pvalid ? 1 : 0, tl) != 0;
    }
    return d;
}

// The bf16 epilogue of 16 channels (c0 .. c0 + 15) of the warp's 32 pixels: the plain store,
// and the optional pooled and upsampled outputs. Called by every lane of the warp (the pool's
// 2 x 2 block is four lanes of one warp: x-neighbour lane ^ 1, y-neighbour lane ^ yl); the
// pooled average is (((0 + v(x, y)) + v(x + 1, y)) + v(x, y + 1)) + v(x + 1, y + 1) of the
// stored (bf16-rounded) values, times 1/4, rounded to bf16. The warp's 32 pixels pass their
// 32 bytes through ebuf (this warp's 1 KB of shared memory; 16-byte chunks swizzled by lane bit
// 2, so that neither side has bank conflicts), and each 32-byte sector of the output is then
// written whole by two lanes of one store instruction: lane-per-pixel stores wrote every sector
// in two 16-byte halves from separate instructions, twice the L2 write requests.
__device__ __forceinline__ void epilogue_bf16(const ConvArgs& a, const float (&v)[16], const EpiDst& d, int c0,
                                              int yl, uint4* ebuf) {
    const int lane = threadIdx.x & 31;
    const int sw = (lane >> 2) & 1;
    ebuf[2 * lane + sw] = make_uint4(pack_bf16x2(v[0], v[1]), pack_bf16x2(v[2], v[3]), pack_bf16x2(v[4], v[5]),
                                     pack_bf16x2(v[6], v[7]));
    ebuf[2 * lane + (sw ^ 1)] = make_uint4(pack_bf16x2(v[8], v[9]), pack_bf16x2(v[10], v[11]),
                                           pack_bf16x2(v[12], v[13]), pack_bf16x2(v[14], v[15]));
    __syncwarp();
    const size_t W2 = 2 * (size_t)a.W;
    const int h = lane & 1;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const int src = (lane >> 1) + 16 * i;
        const uint4 val = ebuf[2 * src + (h ^ ((src >> 2) & 1))];
        if (d.in[i]) *reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(a.out) + d.o[i] + c0) = val;
        if (a.up_out && d.in[i]) {
            __nv_bfloat16* up = reinterpret_cast<__nv_bfloat16*>(a.up_out) + d.u[i] + c0;
            for (int k = 0; k < 4; ++k)
                *reinterpret_cast<uint4*>(up + ((k >> 1) * W2 + (k & 1)) * a.up_c) = val;
        }
    }
    __syncwarp();   // the next group rewrites ebuf
    if (a.pool_out) {
        // The warp's 8 pooled pixels x 16 channels: lane l averages channels 4 (l & 3) .. + 3 of
        // pooled pixel l >> 2 from the block's four stored values in ebuf (the block's top-left
        // lane, even x and even y, has lane bits 0 and log2(yl) clear; then its x-, y- and
        // diagonal neighbours, in that order) and stores them: 4 lanes per 32-byte sector.
        const int b = yl == 16 ? 4 : 3;
        const int k = lane >> 2, qd = lane & 3;
        const int tl = ((k >> (b - 1)) << (b + 1)) | ((k & ((1 << (b - 1)) - 1)) << 1);   // top-left lane
        float s4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
            const int nl = tl ^ (t & 1) ^ (t & 2 ? yl : 0);
            const uint2 w = *reinterpret_cast<const uint2*>(reinterpret_cast<const uint8_t*>(ebuf) +
                                                            (2 * nl + ((qd >> 1) ^ ((nl >> 2) & 1))) * 16 +
                                                            (qd & 1) * 8);
            s4[0] = s4[0] + __uint_as_float(w.x << 16);
            s4[1] = s4[1] + __uint_as_float(w.x & 0xFFFF0000u);
            s4[2] = s4[2] + __uint_as_float(w.y << 16);
            s4[3] = s4[3] + __uint_as_float(w.y & 0xFFFF0000u);
        }
        if (d.pin)
            *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(a.pool_out) + d.p + c0) =
                make_uint2(pack_bf16x2(s4[0] * 0.25f, s4[1] * 0.25f), pack_bf16x2(s4[2] * 0.25f, s4[3] * 0.25f));
        __syncwarp();   // the next group rewrites ebuf
    }
}

// v[j] += bias[c0 + j] (bias null: nothing) as four 16-byte loads (the bias is 16-byte aligned).
__device__ __forceinline__ void add_bias16(const float* bias, int c0, float (&v)[16]) {
    if (!bias) return;
    const float4* b4 = reinterpret_cast<const float4*>(bias + c0);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float4 b = __ldg(b4 + k);
        v[4 * k] += b.x; v[4 * k + 1] += b.y; v[4 * k + 2] += b.z; v[4 * k + 3] += b.w;
    }
}

// The addend's 16 channels for output channels c0 .. c0 + 15 of pixel (x, y) (add_par): q is
// the element index of the half-resolution pixel's parity group.
__device__ __forceinline__ size_t pix_add(const ConvArgs& a, int img, int x, int y) {
    const size_t hp = ((size_t)img * (a.H >> 1) + (y >> 1)) * (a.W >> 1) + (x >> 1);
    return hp * a.add_c + (size_t)(((y & 1) << 1) | (x & 1)) * a.cout;
}
__device__ __forceinline__ void add_parity(const ConvArgs& a, float (&v)[16], size_t q, int c0) {
    const uint4* s = reinterpret_cast<const uint4*>(reinterpret_cast<const __nv_bfloat16*>(a.add_par) + q + c0);
    const uint4 lo = __ldg(s), hi = __ldg(s + 1);
    const uint32_t w[8] = {lo.x, lo.y, lo.z, lo.w, hi.x, hi.y, hi.z, hi.w};
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        v[2 * j] += __uint_as_float(w[j] << 16);
        v[2 * j + 1] += __uint_as_float(w[j] & 0xFFFF0000u);
    }
}

// fp32 output of channels c0 .. c0 + n - 1 (n <= 16) at o: 16-byte stores where o allows.
// Unrolled with constant indices, so that v stays in registers.
__device__ __forceinline__ void store_f32(float* o, const float (&v)[16], int n) {
    const bool al = !(reinterpret_cast<uintptr_t>(o) & 15u);
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        if (al && 4 * q + 4 <= n) {
            *reinterpret_cast<float4*>(o + 4 * q) = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
        } else {
#pragma unroll
            for (int j = 4 * q; j < 4 * q + 4; ++j)
                if (j < n) o[j] = v[j];
        }
    }
}

__device__ __forceinline__ void tile_origin(int t, int tiles_x, int tiles_y, int& x0, int& y0, int& img) {
    const int per_img = tiles_x * tiles_y;
    img = t / per_img;
    const int r = t - img * per_img;
    y0 = (r / tiles_x) * kTileY;
    x0 = (r % tiles_x) * kTileX;
}

// kRows: row-box stages (three vertical taps per stage) or one tap per stage. The MMA issuer
// adds each operand's offset to the descriptors' start fields as a constant.
template <bool kRows>
__global__ void __launch_bounds__(kConvThreads) k_conv3x3(const __grid_constant__ CUtensorMap mx,
                                                          const __grid_constant__ CUtensorMap mw, ConvArgs a,
                                                          int tiles_x, int tiles_y, int ntiles, int stages) {
    constexpr bool rows = kRows;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int a_bytes = kTileX * (rows ? kTileY + 2 : kTileY) * 64;
    const int b_bytes = a.cout * 64;
    constexpr int nb = rows ? 3 : 1;   // weight boxes per stage
    const int stage_bytes = (a_bytes + nb * b_bytes + 1023) & ~1023;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + stages * stage_bytes);
    uint64_t* empty = full + stages;
    uint64_t* accf = empty + stages;   // accumulator ready (MMA commit)
    uint64_t* acce = accf + 2;         // accumulator drained (128 epilogue arrivals)
    uint64_t* fin = acce + 2;          // every MMA of this CTA completed
    uint32_t* tslot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    uint4* ebuf = reinterpret_cast<uint4*>((reinterpret_cast<uintptr_t>(tslot + 2) + 15) & ~(uintptr_t)15);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kc = a.cin / 32, nk = (rows ? 3 : 9) * kc;
    const uint32_t ncols1 = a.cout <= 32 ? 32u : a.cout <= 64 ? 64u : a.cout <= 128 ? 128u : 256u;
    const uint32_t ncols = 2u * ncols1;

    if (tid == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&accf[0], 1);
        mbar_init(&accf[1], 1);
        mbar_init(&acce[0], kEpiThreads);
        mbar_init(&acce[1], kEpiThreads);
        mbar_init(fin, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 1) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        if (lane == 0) {   // producer
            int kg = 0;
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                int x0, y0, img;
                tile_origin(t, tiles_x, tiles_y, x0, y0, img);
                for (int k = 0; k < nk; ++k, ++kg) {
                    const int s = kg % stages;
                    const uint32_t use = (uint32_t)(kg / stages);
                    if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1u) & 1u, a.err)) {
                        *abort_flag = 1;
                        break;
                    }
                    uint8_t* sa = smem + s * stage_bytes;
                    mbar_expect_tx(&full[s], (uint32_t)(a_bytes + nb * b_bytes));
                    if (rows) {
                        const int dx = k / kc, c = k - dx * kc;
                        tma_load_4d(sa, &mx, c * 32, x0 + dx - 1, y0 - 1, img, &full[s]);
                        for (int dy = 0; dy < 3; ++dy)
                            tma_load_2d(sa + a_bytes + dy * b_bytes, &mw, (dy * 3 + dx) * a.cin + c * 32, 0, &full[s]);
                    } else {
                        const int tap = k / kc, c = k - tap * kc;
                        tma_load_4d(sa, &mx, c * 32, x0 + tap % 3 - 1, y0 + tap / 3 - 1, img, &full[s]);
                        tma_load_2d(sa + a_bytes, &mw, tap * a.cin + c * 32, 0, &full[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            const uint32_t idesc = umma_idesc_bf16(128u, (uint32_t)a.cout);
            const int b_step = b_bytes >> 4;   // one weight box in 16-byte units
            int kg = 0, i = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++i) {
                const int acc = i & 1;
                const uint32_t use = (uint32_t)(i >> 1);
                if (use > 0 && !mbar_wait_bounded(&acce[acc], (use - 1u) & 1u, a.err)) {
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)acc * ncols1;
                for (int k = 0; k < nk; ++k, ++kg) {
                    const int s = kg % stages;
                    if (!mbar_wait_bounded(&full[s], (uint32_t)(kg / stages) & 1u, a.err)) {
                        *abort_flag = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(smem + s * stage_bytes);
                    // start fields (16-byte units) stay below 2^14: shared memory < 256 KB
                    const uint64_t a0 = umma_desc_sw64(sa), b0 = umma_desc_sw64(sa + (uint32_t)a_bytes);
#pragma unroll
                    for (int dy = 0; dy < nb; ++dy) {
                        const uint64_t ta = a0 + (uint64_t)(dy * kTileX * 4), tb = b0 + (uint64_t)(dy * b_step);
                        umma_bf16(d, ta, tb, idesc, (k | dy) != 0 ? 1u : 0u);
                        umma_bf16(d, ta + 2u, tb + 2u, idesc, 1u);
                    }
                    umma_commit(&empty[s]);
                }
                if (ok) umma_commit(&accf[acc]);
            }
            umma_commit(fin);
            mbar_wait_bounded(fin, 0u, a.err);   // nothing may be in flight when TMEM is freed
        }
    } else {
        // epilogue: warp w reads TMEM lanes 32 (w % 4) .. +31, the tile's pixels of that quarter
        const int q = warp & 3;
        const int p = q * 32 + lane;
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
            const int acc = i & 1;
            const bool ready = mbar_wait_bounded(&accf[acc], (uint32_t)(i >> 1) & 1u, a.err);
            __syncwarp();
            tc_fence_after();
            if (!__all_sync(0xFFFFFFFFu, ready) || *abort_flag) break;
            int x0, y0, img;
            tile_origin(t, tiles_x, tiles_y, x0, y0, img);
            const int y = y0 + p / kTileX, x = x0 + p % kTileX;
            const bool inside = y < a.H && x < a.W;
            const size_t pix = ((size_t)img * a.H + y) * a.W + x;
            const uint32_t base = tmem + (uint32_t)acc * ncols1 + ((uint32_t)(q * 32) << 16);
            const EpiDst dst = epi_dst(a, img, x, y, inside, 16);   // y-neighbour: lane ^ 16 (16-pixel rows)
            for (int c0 = 0; c0 < a.cout; c0 += 16) {
                uint32_t r[16];
                tmem_ld16(base + (uint32_t)c0, r);
                tmem_ld_wait();
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
                add_bias16(a.bias, c0, v);
                if (a.add_par && inside) add_parity(a, v, pix_add(a, img, x, y), c0);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (a.flags & kConvRelu) v[j] = fmaxf(v[j], 0.0f);
                if (a.flags & kConvF32Out) {
                    if (!inside) continue;
                    store_f32(reinterpret_cast<float*>(a.out) + pix * a.out_c + a.out_off + c0, v,
                              min(16, a.n_store - c0));
                } else {
                    epilogue_bf16(a, v, dst, c0, 16, ebuf + 64 * q);
                }
            }
            tc_fence_before();
            mbar_arrive(&acce[acc]);
        }
    }
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, ncols);
}

// ---------------------------------------------------------------------------------------------
// Halo tiles: outputs of up to 32 channels whose weights fit in shared memory (the
// full-resolution layers). Tiles of 8 x 16 pixels (x by y, M = 128). The CTA loads all weights
// once ({32 Cin, Cout} boxes per tap and input chunk, 64-byte swizzled) and keeps them; per
// 32-channel input chunk a stage holds the chunk's 10 x 18-pixel halo box (180 pixel rows), so
// that the A operand of tap (dy, dx) is that box at start offset (10 dy + dx) rows, 8-row groups
// (one tile row) 10 rows apart. Each input chunk is read once per tile (with its halo, 1.4x),
// and no weights per tile. Two layouts of the box, chosen by the input's pixel stride:
//  * rows (rb = 64, or 32 for an input of 16 channels), when the chunk is the whole pixel: one
//    TMA box of rb-byte pixel rows in the K-major layout with rb-byte swizzle. The tensor core
//    applies the swizzle on the absolute shared-memory address bits, as the TMA does when it
//    writes the box, so an operand may start at any row of it (descriptor base offset 0).
//  * planes (rb = 16), when the chunk is part of a wider pixel: four 8-channel planes without
//    swizzle (180 rows of 16 bytes each, planes 2944 bytes apart: a TMA destination must be
//    128-byte aligned), core matrices of 8 pixels 160 bytes apart, K halves one plane pair apart.
// Measured on the 1080p denoiser layers (ncu, cold): 32 -> 32 layers 110 -> 95 us with rows;
// the 96-channel input (192-byte pixels read 64 bytes at a time) 211 us with planes, 281 with
// rows; the 16-channel input 111 -> 85 us (rows of 32 bytes: half the MMAs).

constexpr int kHaloX = 8, kHaloY = 16;
constexpr int kHaloBoxX = kHaloX + 2, kHaloBoxY = kHaloY + 2;
constexpr int kHaloRows = kHaloBoxX * kHaloBoxY;                   // 180 pixel rows
constexpr int kHaloPlane = kHaloRows * 16;                         // 8 channels: 2880 bytes
constexpr int kHaloPlaneStride = (kHaloPlane + 127) & ~127;        // 2944
constexpr int kHaloStage = (4 * kHaloPlaneStride + 1023) & ~1023;  // 12288 (>= 180 x 64): 1024-byte aligned
constexpr int kHaloStages = 4;
constexpr int kHaloWeightMax = 96 * 1024;

// kRb: 16 (planes), 32 or 64 (rows of that many bytes). The MMA issuer's loop over the nine taps
// is unrolled with the operand offsets as constants added to the descriptors' start fields: with
// up to 54 MMAs per tile a single issuing thread must not fall behind the tensor core.
template <int kRb>
__global__ void __launch_bounds__(kConvThreads) k_conv3x3_halo(const __grid_constant__ CUtensorMap mx,
                                                               const __grid_constant__ CUtensorMap mw, ConvArgs a,
                                                               int tiles_x, int tiles_y, int ntiles) {
    constexpr int rb = kRb;
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int kc = a.cin / 32;
    const int b_bytes = a.cout * 64;   // one weight box: a multiple of 1024 bytes
    const int w_bytes = 9 * kc * b_bytes;
    uint8_t* wsm = smem;               // box (chunk c, tap) at (9 c + tap) * b_bytes
    uint8_t* stage0 = smem + w_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(stage0 + kHaloStages * kHaloStage);
    uint64_t* empty = full + kHaloStages;
    uint64_t* wbar = empty + kHaloStages;
    uint64_t* accf = wbar + 1;
    uint64_t* acce = accf + 2;
    uint64_t* fin = acce + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(fin + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    uint4* ebuf = reinterpret_cast<uint4*>((reinterpret_cast<uintptr_t>(tslot + 2) + 15) & ~(uintptr_t)15);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t ncols1 = a.cout <= 32 ? 32u : 64u;
    const uint32_t ncols = 2u * ncols1;

    if (tid == 0) {
        for (int s = 0; s < kHaloStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(wbar, 1);
        mbar_init(&accf[0], 1);
        mbar_init(&accf[1], 1);
        mbar_init(&acce[0], kEpiThreads);
        mbar_init(&acce[1], kEpiThreads);
        mbar_init(fin, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    if (warp == 1) {
        tmem_alloc(tslot, ncols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tslot;

    if (warp == 0) {
        if (lane == 0) {   // producer: the weights once, then one halo box per tile and chunk
            mbar_expect_tx(wbar, (uint32_t)w_bytes);
            for (int c = 0; c < kc; ++c)
                for (int tap = 0; tap < 9; ++tap)
                    tma_load_2d(wsm + (9 * c + tap) * b_bytes, &mw, tap * a.cin + c * 32, 0, wbar);
            int kg = 0;
            for (int t = blockIdx.x; t < ntiles && !*abort_flag; t += gridDim.x) {
                const int per_img = tiles_x * tiles_y, img = t / per_img, r = t - img * per_img;
                const int y0 = (r / tiles_x) * kHaloY, x0 = (r % tiles_x) * kHaloX;
                for (int c = 0; c < kc; ++c, ++kg) {
                    const int s = kg % kHaloStages;
                    const uint32_t use = (uint32_t)(kg / kHaloStages);
                    if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1u) & 1u, a.err)) {
                        *abort_flag = 1;
                        break;
                    }
                    uint8_t* sa = stage0 + s * kHaloStage;
                    if (smem_u32(sa) & 1023u) {   // stages start 1024-byte aligned (weights: 1024-byte boxes)
                        // (planes then start 128-byte aligned)
                        atomicOr(a.err, kErrTmaWait);
                        *abort_flag = 1;
                        break;
                    }
                    if (kRb == 16) {
                        mbar_expect_tx(&full[s], (uint32_t)(4 * kHaloPlane));
                        for (int j = 0; j < 4; ++j)
                            tma_load_4d(sa + j * kHaloPlaneStride, &mx, c * 32 + j * 8, x0 - 1, y0 - 1, img,
                                        &full[s]);
                    } else {
                        mbar_expect_tx(&full[s], (uint32_t)(kHaloRows * rb));
                        tma_load_4d(sa, &mx, c * 32, x0 - 1, y0 - 1, img, &full[s]);
                    }
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            const uint32_t idesc = umma_idesc_bf16(128u, (uint32_t)a.cout);
            bool ok = mbar_wait_bounded(wbar, 0u, a.err);
            if (!ok) *abort_flag = 1;
            tc_fence_after();
            const uint32_t wb0 = smem_u32(wsm);
            const int b_step = b_bytes >> 4;   // one tap's weight box in 16-byte units
            int kg = 0, i = 0;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x, ++i) {
                const int acc = i & 1;
                const uint32_t use = (uint32_t)(i >> 1);
                if (use > 0 && !mbar_wait_bounded(&acce[acc], (use - 1u) & 1u, a.err)) {
                    *abort_flag = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + (uint32_t)acc * ncols1;
                for (int c = 0; c < kc; ++c, ++kg) {
                    const int s = kg % kHaloStages;
                    if (!mbar_wait_bounded(&full[s], (uint32_t)(kg / kHaloStages) & 1u, a.err)) {
                        *abort_flag = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(stage0 + s * kHaloStage);
                    // descriptors of the tap-(0, 0) operands; a tap adds its offset (16-byte
                    // units) to the start field, which stays below 2^14 (shared memory < 256 KB)
                    const uint64_t a0 = kRb == 16 ? umma_desc_dense(sa, (uint32_t)kHaloPlaneStride, kHaloBoxX * 16u)
                                                  : umma_desc_swz(sa, (uint32_t)kRb, (uint32_t)(kHaloBoxX * kRb));
                    const uint64_t b0 = umma_desc_sw64(wb0 + (uint32_t)(9 * c * b_bytes));
                    constexpr int nkk = kRb == 32 ? 1 : 2;
#pragma unroll
                    for (int tap = 0; tap < 9; ++tap) {
                        const int off = ((tap / 3) * kHaloBoxX + tap % 3) * kRb;
#pragma unroll
                        for (int kk = 0; kk < nkk; ++kk) {
                            const int aoff = kRb == 16 ? 2 * kk * kHaloPlaneStride + off : off + kk * 32;
                            umma_bf16(d, a0 + (uint64_t)(aoff >> 4), b0 + (uint64_t)(tap * b_step + kk * 2), idesc,
                                      (c | tap | kk) != 0 ? 1u : 0u);
                        }
                    }
                    umma_commit(&empty[s]);
                }
                if (ok) umma_commit(&accf[acc]);
            }
            umma_commit(fin);
            mbar_wait_bounded(fin, 0u, a.err);   // nothing may be in flight when TMEM is freed
        }
    } else {
        const int q = warp & 3;
        const int p = q * 32 + lane;
        int i = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++i) {
            const int acc = i & 1;
            const bool ready = mbar_wait_bounded(&accf[acc], (uint32_t)(i >> 1) & 1u, a.err);
            __syncwarp();
            tc_fence_after();
            if (!__all_sync(0xFFFFFFFFu, ready) || *abort_flag) break;
            const int per_img = tiles_x * tiles_y, img = t / per_img, r = t - img * per_img;
            const int y = (r / tiles_x) * kHaloY + p / kHaloX, x = (r % tiles_x) * kHaloX + p % kHaloX;
            const bool inside = y < a.H && x < a.W;
            const size_t pix = ((size_t)img * a.H + y) * a.W + x;
            const uint32_t base = tmem + (uint32_t)acc * ncols1 + ((uint32_t)(q * 32) << 16);
            const EpiDst dst = epi_dst(a, img, x, y, inside, 8);   // y-neighbour: lane ^ 8 (8-pixel rows)
            for (int c0 = 0; c0 < a.cout; c0 += 16) {
                uint32_t rr[16];
                tmem_ld16(base + (uint32_t)c0, rr);
                tmem_ld_wait();
                float v[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(rr[j]);
                add_bias16(a.bias, c0, v);
                if (a.add_par && inside) add_parity(a, v, pix_add(a, img, x, y), c0);
#pragma unroll
                for (int j = 0; j < 16; ++j)
                    if (a.flags & kConvRelu) v[j] = fmaxf(v[j], 0.0f);
                if (a.flags & kConvF32Out) {
                    if (!inside) continue;
                    store_f32(reinterpret_cast<float*>(a.out) + pix * a.out_c + a.out_off + c0, v,
                              min(16, a.n_store - c0));
                } else {
                    epilogue_bf16(a, v, dst, c0, 8, ebuf + 64 * q);
                }
            }
            tc_fence_before();
            mbar_arrive(&acce[acc]);
        }
    }
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, ncols);
}

}  // namespace

}  // namespace gk

using namespace gk;

cudaError_t gkrt_encode_tmap_bf16(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                  const uint64_t* strides_bytes, const uint32_t* box);
cudaError_t gkrt_encode_tmap_bf16_sw32(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                       const uint64_t* strides_bytes, const uint32_t* box);
cudaError_t gkrt_encode_tmap_bf16_dense(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                        const uint64_t* strides_bytes, const uint32_t* box);

// Halo tiles for outputs of up to 32 channels whose weights (9 Cin Cout bf16) fit in 96 KB.
// The 1080p forward (event-timed, one box): row-box stages everywhere 1.560 ms; halo tiles for
// Cout <= 32 1.503 ms; also for Cout <= 64 with weights <= 40 KB 1.504 ms, <= 96 KB 1.556 ms
// (the 64 -> 64 layers then run one CTA per SM behind 72 KB of weights).
static bool conv_halo(int cin, int cout) { return cout <= 32 && 9 * cin * cout * 2 <= kHaloWeightMax; }
static size_t conv_halo_smem(int cin, int cout) {
    return (size_t)9 * cin * cout * 2 + kHaloStages * kHaloStage + (2 * kHaloStages + 6) * 8 + 8 + kEpiBuf + 1024;
}

// Outputs of up to 128 channels use the row-box stages (three vertical taps per box); the
// 1080p forward: none 1.94 ms, up to 64 channels 1.67 ms, up to 128 channels 1.58 ms.
static bool conv_rows(int cout) { return cout <= 128; }

// Four stages per CTA (three for row-box stages, which carry three taps each), so that several
// CTAs share an SM (as many as shared memory and the 512 TMEM columns allow): independent
// load/MMA/epilogue streams hide L2 latency better than deeper rings in fewer CTAs (measured
// on the level-0 layers: 1.74 -> 1.67 ms for the 1080p forward with three row-box stages).
static int conv_stages(int cout) { return conv_rows(cout) ? 3 : 4; }

size_t gkrt_conv_smem_bytes(int cout) {
    const bool rows = conv_rows(cout);
    const int stage = (kTileX * (rows ? kTileY + 2 : kTileY) * 64 + (rows ? 3 : 1) * cout * 64 + 1023) & ~1023;
    return (size_t)conv_stages(cout) * stage + 2 * conv_stages(cout) * 8 + 5 * 8 + 8 + kEpiBuf + 1024;
}

static size_t conv_smem_max() {
    size_t m = 0;
    for (int c = 16; c <= 256; c += 16) m = std::max(m, gkrt_conv_smem_bytes(c));
    return m;
}

cudaError_t gkrt_launch_conv3x3(const void* x, const void* w, const ConvArgs& args, cudaStream_t st) {
    const bool f32 = (args.flags & kConvF32Out) != 0;
    if (args.cin % 32 || args.cin < 32 || args.cout % 16 || args.cout < 16 || args.cout > 256 || args.B < 1 ||
        args.H < 1 || args.W < 1 || (!f32 && (args.out_c % 16 || args.out_off % 16)) ||
        args.out_off + (f32 ? args.n_store : args.cout) > args.out_c || (f32 && args.n_store > args.cout) ||
        ((uintptr_t)x & 15u) || ((uintptr_t)w & 15u) || ((uintptr_t)args.out & 15u) ||
        ((uintptr_t)args.bias & 15u) || args.x_off % 8 ||
        args.x_valid < 0 || args.x_valid > args.cin || (args.x_valid % 32 && args.x_valid != 16))
        return cudaErrorInvalidValue;
    const int xv = args.x_valid > 0 ? args.x_valid : args.cin;   // channels present; the rest are zeros
    // the 32-channel boxes end inside the map, except 16 channels of a 32-channel input (halo
    // tiles with 32-byte rows)
    const bool halo = conv_halo(args.cin, args.cout);
    if (xv % 32 && !(halo && args.cin == 32)) return cudaErrorInvalidValue;
    if (args.x_c > 0 && (args.x_c % 8 || args.x_off + xv > args.x_c)) return cudaErrorInvalidValue;
    if ((args.pool_out || args.up_out || args.add_par) && f32) return cudaErrorInvalidValue;
    if (args.add_par && ((args.H | args.W) & 1 || args.add_c % 8 || args.add_c < 4 * args.cout ||
                         ((uintptr_t)args.add_par & 15u)))
        return cudaErrorInvalidValue;
    if (args.pool_out && (args.pool_c % 8 || args.pool_off % 8 || args.pool_off + args.cout > args.pool_c ||
                          ((uintptr_t)args.pool_out & 15u)))
        return cudaErrorInvalidValue;
    if (args.up_out && (args.up_c % 8 || args.up_off % 8 || args.up_off + args.cout > args.up_c ||
                        ((uintptr_t)args.up_out & 15u)))
        return cudaErrorInvalidValue;
    CUtensorMap mx, mw;
    const uint64_t xc = (uint64_t)(args.x_c > 0 ? args.x_c : xv);
    // per device: SM count, the attributes set, resident CTAs per output width
    static int sms_dev[kMaxDevices] = {};
    static bool halo_attr[kMaxDevices] = {};
    static size_t smem_set[kMaxDevices] = {};
    static int per_sm_cache[kMaxDevices][257] = {};
    const int dev = current_device_slot();
    if (dev < 0) return cudaErrorInvalidDevice;
    if (!sms_dev[dev]) {
        const cudaError_t e0 = cudaDeviceGetAttribute(&sms_dev[dev], cudaDevAttrMultiProcessorCount, dev);
        if (e0 != cudaSuccess) return e0;
    }
    const int sms = sms_dev[dev];
    if (halo) {
        // rows when a chunk is the whole pixel (64 bytes, or 32 for an input of 16 channels),
        // planes when the pixel is wider than the chunk
        const int rb = (int)xc * 2 == std::min(xv, 32) * 2 ? (xv == 16 ? 32 : 64) : 16;
        if (rb == 16 && xv % 32) return cudaErrorInvalidValue;
        const uint64_t xd[4] = {(uint64_t)xv, (uint64_t)args.W, (uint64_t)args.H, (uint64_t)args.B};
        const uint64_t xs[3] = {xc * 2, (uint64_t)args.W * xc * 2, (uint64_t)args.H * args.W * xc * 2};
        const uint32_t xb[4] = {(uint32_t)(rb == 16 ? 8 : rb / 2), kHaloBoxX, kHaloBoxY, 1};
        const void* xbase = static_cast<const uint8_t*>(x) + (size_t)args.x_off * 2;
        cudaError_t e = rb == 64   ? gkrt_encode_tmap_bf16(&mx, xbase, 4, xd, xs, xb)
                        : rb == 32 ? gkrt_encode_tmap_bf16_sw32(&mx, xbase, 4, xd, xs, xb)
                                   : gkrt_encode_tmap_bf16_dense(&mx, xbase, 4, xd, xs, xb);
        if (e != cudaSuccess) return e;
        const uint64_t wd[2] = {(uint64_t)9 * args.cin, (uint64_t)args.cout};
        const uint64_t ws[1] = {(uint64_t)9 * args.cin * 2};
        const uint32_t wb[2] = {32, (uint32_t)args.cout};
        if ((e = gkrt_encode_tmap_bf16(&mw, w, 2, wd, ws, wb)) != cudaSuccess) return e;
        const size_t smem = conv_halo_smem(args.cin, args.cout);
        if (!halo_attr[dev]) {
            const int mx_smem = (int)(kHaloWeightMax + kHaloStages * kHaloStage + 2048 + kEpiBuf);
            for (const void* f : {(const void*)k_conv3x3_halo<16>, (const void*)k_conv3x3_halo<32>,
                                  (const void*)k_conv3x3_halo<64>}) {
                if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, mx_smem)) != cudaSuccess)
                    return e;
                if ((e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                              (int)cudaSharedmemCarveoutMaxShared)) != cudaSuccess)
                    return e;
            }
            halo_attr[dev] = true;
        }
        const int ncols = 2 * (args.cout <= 32 ? 32 : 64);
        const int per_sm = std::max(1, std::min({(int)((227 * 1024) / (smem + 1024)), 512 / ncols,
                                                 2048 / kConvThreads}));
        const int tiles_x = (args.W + kHaloX - 1) / kHaloX, tiles_y = (args.H + kHaloY - 1) / kHaloY;
        const int ntiles = tiles_x * tiles_y * args.B;
        const int grid = std::min(ntiles, sms * per_sm);
        if (rb == 64)
            k_conv3x3_halo<64><<<grid, kConvThreads, smem, st>>>(mx, mw, args, tiles_x, tiles_y, ntiles);
        else if (rb == 32)
            k_conv3x3_halo<32><<<grid, kConvThreads, smem, st>>>(mx, mw, args, tiles_x, tiles_y, ntiles);
        else
            k_conv3x3_halo<16><<<grid, kConvThreads, smem, st>>>(mx, mw, args, tiles_x, tiles_y, ntiles);
        return cudaGetLastError();
    }
    const uint64_t xd[4] = {(uint64_t)xv, (uint64_t)args.W, (uint64_t)args.H, (uint64_t)args.B};
    const uint64_t xs[3] = {xc * 2, (uint64_t)args.W * xc * 2, (uint64_t)args.H * args.W * xc * 2};
    const bool rows = conv_rows(args.cout);
    const uint32_t xb[4] = {32, kTileX, (uint32_t)(rows ? kTileY + 2 : kTileY), 1};
    const void* xbase = static_cast<const uint8_t*>(x) + (size_t)args.x_off * 2;
    cudaError_t e = gkrt_encode_tmap_bf16(&mx, xbase, 4, xd, xs, xb);
    if (e != cudaSuccess) return e;
    const uint64_t wd[2] = {(uint64_t)9 * args.cin, (uint64_t)args.cout};
    const uint64_t ws[1] = {(uint64_t)9 * args.cin * 2};
    const uint32_t wb[2] = {32, (uint32_t)args.cout};
    e = gkrt_encode_tmap_bf16(&mw, w, 2, wd, ws, wb);
    if (e != cudaSuccess) return e;
    const size_t smem = gkrt_conv_smem_bytes(args.cout);
    // launch geometry per output width, computed once per device (host calls kept off the
    // per-launch path)
    if (smem > smem_set[dev]) {
        for (const void* f : {(const void*)k_conv3x3<true>, (const void*)k_conv3x3<false>}) {
            if ((e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)conv_smem_max())) !=
                cudaSuccess)
                return e;
            if ((e = cudaFuncSetAttribute(f, cudaFuncAttributePreferredSharedMemoryCarveout,
                                          (int)cudaSharedmemCarveoutMaxShared)) != cudaSuccess)
                return e;
        }
        smem_set[dev] = conv_smem_max();
    }
    int per_sm = per_sm_cache[dev][args.cout];
    if (!per_sm) {
        // resident CTAs per SM: shared memory (227 KB per SM, 1 KB reserved per CTA), the 512
        // TMEM columns (two accumulators per CTA) and 2048 threads
        const int ncols = 2 * (args.cout <= 32 ? 32 : args.cout <= 64 ? 64 : args.cout <= 128 ? 128 : 256);
        per_sm = std::min({(int)((227 * 1024) / (smem + 1024)), 512 / ncols, 2048 / kConvThreads});
        per_sm = std::max(1, per_sm);
        per_sm_cache[dev][args.cout] = per_sm;
    }
    const int tiles_x = (args.W + kTileX - 1) / kTileX, tiles_y = (args.H + kTileY - 1) / kTileY;
    const int ntiles = tiles_x * tiles_y * args.B;
    const int grid = std::min(ntiles, sms * per_sm);
    if (rows)
        k_conv3x3<true><<<grid, kConvThreads, smem, st>>>(mx, mw, args, tiles_x, tiles_y, ntiles, conv_stages(args.cout));
    else
        k_conv3x3<false><<<grid, kConvThreads, smem, st>>>(mx, mw, args, tiles_x, tiles_y, ntiles,
                                                           conv_stages(args.cout));
    return cudaGetLastError();
}
