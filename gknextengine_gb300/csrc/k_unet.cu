// k_unet.cu — the learned denoiser's training and inference kernels besides the forward
// convolution (k_conv.cu): weight gradients on the tensor cores, and the element-wise,
// pooling, loss and optimiser kernels.
//
// The weight gradient of a 3x3 convolution, dW[cout][tap][cin] = sum over pixels of
// dP[p][cout] * X[p + tap offset][cin], is a GEMM with K = pixels whose operands TMA loads
// straight from the NHWC tensors in the MN-major layout (k_conv_wgrad_tma, below).
#include <algorithm>

#include "gk_umma.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

// ---- weight gradient with TMA-fed MN-major operands ----
// The same GEMM, dW[cout][tap][cin] = sum over pixels of dP[p][cout] X[p + tap][cin], with K =
// pixels: NHWC rows hold the channels of one pixel contiguously, which is the MN-major layout
// of both operands for K along pixels, so TMA loads them unchanged. A K step is a run of
// kWtK pixels of one image row; per 64-channel group one box {64 channels, kWtK pixels} lands
// 128-byte swizzled (an atom of 8 pixel rows x 128 bytes, atoms 1024 bytes apart along K). X's
// box starts at the tap's shift, and TMA's zero fill outside the tensor is the padding. The CTA
// takes one tap and a run of image rows: warp 0 issues the loads into a ring of stages, warp 1
// the MMAs (M = 128 rows of dP's channels, zero past cout; N = cin), and all four warps the
// epilogue (atomics into dW). Every wait is bounded.

constexpr int kWtThreads = 128;
constexpr int kWtK = 32;                        // pixels per K step
constexpr int kWtAtom = kWtK * 128;             // one 64-channel box of a step: 4096 bytes
constexpr int kWtStages = 4;
constexpr int kWtGuard = 4096;                  // shared memory after the last stage, never written

// Descriptor of an MN-major, 128-byte-swizzled operand: the leading byte offset is the stride
// between 64-channel atoms along M (or N), 4096 bytes here, and the stride byte offset the one
// between 8-row groups along K, 1024 bytes (the weight-gradient test against torch holds this
// assignment; the swapped one gives wrong sums).
__device__ __forceinline__ uint64_t wt_desc(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)(((uint32_t)kWtAtom >> 4) & 0x3FFFu) << 16;   // leading byte offset
    d |= (uint64_t)((1024u >> 4) & 0x3FFFu) << 32;               // stride byte offset
    d |= (uint64_t)1u << 46;   // version
    d |= (uint64_t)2u << 61;   // SWIZZLE_128B
    return d;
}

// kTaps = 1: one tap per CTA (blockIdx.y), N = cin in nb atoms. kTaps = 9: all nine taps in one
// CTA for cin <= 32 (one B atom per tap, nine accumulators of 32 columns in 512 TMEM columns),
// so that dP is loaded once per step instead of once per tap.
template <int kTaps>
__global__ void __launch_bounds__(kWtThreads) k_conv_wgrad_tma(const __grid_constant__ CUtensorMap mdp,
                                                               const __grid_constant__ CUtensorMap mx, WgradArgs a,
                                                               int rows_per_cta, int nb) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int nbt = kTaps == 1 ? nb : 9;           // B atoms per stage
    const int stage_bytes = (2 + nbt) * kWtAtom;   // A: 2 atoms (M = 128), then the B atoms
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + kWtStages * stage_bytes + kWtGuard);
    uint64_t* empty = full + kWtStages;
    uint64_t* accb = empty + kWtStages;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap0 = kTaps == 1 ? (int)blockIdx.y : 0;
    const int rows = a.B * a.H;
    const int r0 = blockIdx.x * rows_per_cta, r1 = min(r0 + rows_per_cta, rows);
    const int xsteps = (a.W + kWtK - 1) / kWtK;
    const int nk = r1 > r0 ? (r1 - r0) * xsteps : 0;
    const bool a_two = a.cout > 64;   // dP's second 64-channel atom is loaded, else it stays zero
    const uint32_t ncols = kTaps == 9 ? 512u : a.cin <= 32 ? 32u : a.cin <= 64 ? 64u : a.cin <= 128 ? 128u : 256u;

    if (!a_two)   // the second A atom of every stage: zero rows of M
        for (int st = 0; st < kWtStages; ++st)
            for (int i = tid; i < kWtAtom / 16; i += kWtThreads)
                reinterpret_cast<uint4*>(smem + st * stage_bytes + kWtAtom)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        for (int st = 0; st < kWtStages; ++st) {
            mbar_init(&full[st], 1);
            mbar_init(&empty[st], 1);
        }
        mbar_init(accb, 1);
        *abort_flag = 0;
        mbar_fence_init();
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");   // the zeroed atoms, for the tensor core
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
            const uint32_t bytes = (uint32_t)((a_two ? 2 : 1) + nbt) * (uint32_t)kWtAtom;
            for (int k = 0; k < nk && !*abort_flag; ++k) {
                const int s = k % kWtStages;
                const uint32_t use = (uint32_t)(k / kWtStages);
                if (use > 0 && !mbar_wait_bounded(&empty[s], (use - 1u) & 1u, a.err)) {
                    *abort_flag = 1;
                    break;
                }
                const int row = r0 + k / xsteps, x0 = (k % xsteps) * kWtK;
                const int img = row / a.H, y = row - img * a.H;
                uint8_t* st = smem + s * stage_bytes;
                mbar_expect_tx(&full[s], bytes);
                tma_load_4d(st, &mdp, 0, x0, y, img, &full[s]);
                if (a_two) tma_load_4d(st + kWtAtom, &mdp, 64, x0, y, img, &full[s]);
                if (kTaps == 1) {
                    const int dy = tap0 / 3 - 1, dx = tap0 % 3 - 1;
                    for (int j = 0; j < nb; ++j)
                        tma_load_4d(st + (2 + j) * kWtAtom, &mx, 64 * j, x0 + dx, y + dy, img, &full[s]);
                } else {
                    for (int t = 0; t < 9; ++t)
                        tma_load_4d(st + (2 + t) * kWtAtom, &mx, 0, x0 + t % 3 - 1, y + t / 3 - 1, img, &full[s]);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {   // MMA issuer
            const uint32_t idesc = umma_idesc_bf16(128u, (uint32_t)a.cin) | (1u << 15) | (1u << 16);   // MN-major A, B
            bool ok = true;
            for (int k = 0; k < nk && ok; ++k) {
                const int s = k % kWtStages;
                if (!mbar_wait_bounded(&full[s], (uint32_t)(k / kWtStages) & 1u, a.err)) {
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t sa = smem_u32(smem + s * stage_bytes), sb = sa + 2u * (uint32_t)kWtAtom;
                for (int t = 0; t < (kTaps == 1 ? 1 : 9); ++t)
                    for (int kk = 0; kk < kWtK / 16; ++kk)   // 16 pixels (two 8-row groups) per MMA
                        umma_bf16(tmem + (uint32_t)(t * 32), wt_desc(sa + 2048u * kk),
                                  wt_desc(sb + (uint32_t)(t * kWtAtom) + 2048u * kk), idesc, (k | kk) != 0 ? 1u : 0u);
                umma_commit(&empty[s]);
            }
        }
        if (lane == 0) umma_commit(accb);
    }
    __syncwarp();
    const bool ready = mbar_wait_bounded(accb, 0u, a.err) && nk > 0 && !*abort_flag;
    __syncwarp();
    tc_fence_after();
    const int r = warp * 32 + lane;   // TMEM lane = cout row
    for (int t = 0; t < (kTaps == 1 ? 1 : 9); ++t)
        for (int c0 = 0; c0 < a.cin; c0 += 16) {
            uint32_t v[16];
            tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(t * 32 + c0), v);
            tmem_ld_wait();
            if (!ready || r >= a.cout) continue;
            float* d = a.dw + ((size_t)r * 9 + (kTaps == 1 ? tap0 : t)) * a.cin + c0;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float f = __uint_as_float(v[j]);
                if (f != 0.0f) atomicAdd(d + j, f);
            }
        }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) tmem_dealloc(tmem, ncols);
}

// ---- element-wise kernels (NHWC bf16 with channel stride/offset) ----
// One thread per pixel and group of 8 channels (16-byte loads and stores); channel counts,
// strides and offsets are multiples of 8. Pixel counts fit 32-bit indices.

__device__ __forceinline__ void ld8(const __nv_bfloat16* p, float* v) {
    const uint4 u = *reinterpret_cast<const uint4*>(p);
    const __nv_bfloat162* h = reinterpret_cast<const __nv_bfloat162*>(&u);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 f = __bfloat1622float2(h[k]);
        v[2 * k] = f.x;
        v[2 * k + 1] = f.y;
    }
}
__device__ __forceinline__ void st8(__nv_bfloat16* p, const float* v) {
    uint4 u;
    __nv_bfloat162* h = reinterpret_cast<__nv_bfloat162*>(&u);
#pragma unroll
    for (int k = 0; k < 4; ++k) h[k] = __floats2bfloat162_rn(v[2 * k], v[2 * k + 1]);
    *reinterpret_cast<uint4*>(p) = u;
}

// d_in (+)= d_out / 4 for each of the 2x2 inputs (accumulate: add to what is there)
__global__ void k_avgpool2_bwd(const __nv_bfloat16* dout, int dout_c, int dout_off, __nv_bfloat16* din, int din_c,
                               int din_off, int B, int H, int W, int C, int accumulate) {   // H, W: input size
    const int g8 = C / 8;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * H * W * g8) return;
    const int g = i % g8, p = i / g8;
    const int x = p % W, y = (p / W) % H, b = p / (W * H);
    const size_t q = (size_t)(b * (H / 2) + y / 2) * (W / 2) + x / 2;
    float v[8], d[8];
    ld8(dout + q * dout_c + dout_off + 8 * g, v);
    __nv_bfloat16* dst = din + (size_t)p * din_c + din_off + 8 * g;
    if (accumulate) ld8(dst, d);
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = 0.25f * v[j] + (accumulate ? d[j] : 0.0f);
    st8(dst, v);
}

// d_in = sum of the 2x2 output gradients it was copied to
__global__ void k_upsample2_bwd(const __nv_bfloat16* dout, int dout_c, int dout_off, __nv_bfloat16* din, int din_c,
                                int din_off, int B, int h, int w, int C) {   // h, w: input size
    const int g8 = C / 8;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B * h * w * g8) return;
    const int g = i % g8, p = i / g8;
    const int x = p % w, y = (p / w) % h, b = p / (w * h);
    const int W = 2 * w, H = 2 * h;
    float s[8] = {0, 0, 0, 0, 0, 0, 0, 0}, v[8];
    for (int k = 0; k < 4; ++k) {
        const size_t q = (size_t)(b * H + 2 * y + (k >> 1)) * W + 2 * x + (k & 1);
        ld8(dout + q * dout_c + dout_off + 8 * g, v);
#pragma unroll
        for (int j = 0; j < 8; ++j) s[j] += v[j];
    }
    st8(din + (size_t)p * din_c + din_off + 8 * g, s);
}

// dP = dY * (Y > 0) (ReLU), written in place of dY
__global__ void k_relu_bwd(__nv_bfloat16* dy, int dy_c, int dy_off, const __nv_bfloat16* y, int y_c, int y_off,
                           int npix, int C) {
    const int g8 = C / 8;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= npix * g8) return;
    const int g = i % g8, p = i / g8;
    float a[8], b[8];
    __nv_bfloat16* d = dy + (size_t)p * dy_c + dy_off + 8 * g;
    ld8(d, a);
    ld8(y + (size_t)p * y_c + y_off + 8 * g, b);
#pragma unroll
    for (int j = 0; j < 8; ++j)
        if (!(b[j] > 0.0f)) a[j] = 0.0f;
    st8(d, a);
}

// db[c] += sum over pixels of dP[p][c]; one block per run of pixels. Thread t owns the 8
// channels 8 (t % G) .. +7 (G = C / 8, one 16-byte load per pixel) of every (256 / G)-th pixel
// of the run and sums them in registers; the threads of each channel group are then reduced
// in shared memory and each channel gets one atomic per block.
__global__ void __launch_bounds__(256) k_bias_grad(const __nv_bfloat16* dp, int dp_c, int dp_off, long long npix,
                                                   int C, int run, float* db) {
    __shared__ float part[256 * 8];
    const int G = C / 8, per = 256 / G;
    const int g = threadIdx.x % G, k = threadIdx.x / G;
    float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (k < per) {
        const long long p0 = (long long)blockIdx.x * run;
        const long long p1 = p0 + run < npix ? p0 + run : npix;
        for (long long p = p0 + k; p < p1; p += per) {
            float v[8];
            ld8(dp + p * dp_c + dp_off + 8 * g, v);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += v[j];
        }
    }
#pragma unroll
    for (int j = 0; j < 8; ++j) part[threadIdx.x * 8 + j] = acc[j];
    __syncthreads();
    if (threadIdx.x < C) {
        const int c = threadIdx.x, cg = c / 8, cj = c % 8;
        float sum = 0.0f;
        for (int i = 0; i < per; ++i) sum += part[(i * G + cg) * 8 + cj];
        if (sum != 0.0f) atomicAdd(&db[c], sum);
    }
}

}  // namespace

}  // namespace gk

using namespace gk;

cudaError_t gkrt_encode_tmap_bf16_sw128(CUtensorMap* map, const void* base, uint32_t rank, const uint64_t* dims,
                                        const uint64_t* strides_bytes, const uint32_t* box);

static size_t wgrad_tma_smem(int nbt) {   // nbt: B atoms per stage
    return (size_t)kWtStages * (size_t)(2 + nbt) * kWtAtom + kWtGuard + 256 + 1024;
}

cudaError_t gkrt_launch_conv_wgrad(const WgradArgs& a, cudaStream_t st) {
    const int xv = a.x_valid > 0 ? a.x_valid : a.cin;   // X's channels present; the rest are zeros
    if (a.cin % 16 || a.cin < 16 || a.cin > 256 || a.cout % 8 || a.cout < 8 || a.cout > 128 || a.dp_c % 8 ||
        a.dp_off % 8 || a.x_c % 8 || a.x_off % 8 || a.dp_off + a.cout > a.dp_c || a.x_valid < 0 ||
        a.x_valid > a.cin || a.x_valid % 8 || a.x_off + xv > a.x_c || ((uintptr_t)a.dp & 15u) ||
        ((uintptr_t)a.x & 15u) || a.B < 1 || a.H < 1 || a.W < 1)
        return cudaErrorInvalidValue;
    static int sms_dev[kMaxDevices] = {};
    static bool attr_set[kMaxDevices] = {};   // set once per device for the largest stage
    const int dev = current_device_slot();
    if (dev < 0) return cudaErrorInvalidDevice;
    if (!sms_dev[dev]) {
        cudaError_t e = cudaDeviceGetAttribute(&sms_dev[dev], cudaDevAttrMultiProcessorCount, dev);
        if (e != cudaSuccess) return e;
    }
    if (!attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad_tma<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)wgrad_tma_smem(4));
        if (e == cudaSuccess)
            e = cudaFuncSetAttribute(k_conv_wgrad_tma<9>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)wgrad_tma_smem(9));
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    const uint64_t W = (uint64_t)a.W, H = (uint64_t)a.H, B = (uint64_t)a.B;
    const uint32_t box[4] = {64u, (uint32_t)kWtK, 1u, 1u};
    CUtensorMap mdp, mx;
    const uint64_t dd[4] = {(uint64_t)a.cout, W, H, B};
    const uint64_t ds[3] = {(uint64_t)a.dp_c * 2, W * a.dp_c * 2, H * W * a.dp_c * 2};
    cudaError_t e = gkrt_encode_tmap_bf16_sw128(&mdp, a.dp + a.dp_off, 4, dd, ds, box);
    if (e != cudaSuccess) return e;
    const uint64_t xd[4] = {(uint64_t)xv, W, H, B};   // channels past xv: TMA's zero fill
    const uint64_t xs[3] = {(uint64_t)a.x_c * 2, W * a.x_c * 2, H * W * a.x_c * 2};
    if ((e = gkrt_encode_tmap_bf16_sw128(&mx, a.x + a.x_off, 4, xd, xs, box)) != cudaSuccess) return e;
    const int nb = (a.cin + 63) / 64;
    const long long rows = (long long)a.B * a.H;
    if (a.cin <= 32) {   // all taps per CTA (512 TMEM columns: one CTA per SM), a run of image rows each
        const long long target = sms_dev[dev];
        const int rows_per_cta = (int)std::max(1LL, (rows + target - 1) / target);
        const dim3 grid((unsigned)((rows + rows_per_cta - 1) / rows_per_cta), 1);
        k_conv_wgrad_tma<9><<<grid, kWtThreads, wgrad_tma_smem(9), st>>>(mdp, mx, a, rows_per_cta, 1);
        return cudaGetLastError();
    }
    // about two CTAs per SM over the nine taps, each a run of image rows
    const long long target = 2LL * sms_dev[dev];
    const int rows_per_cta = (int)std::max(1LL, (rows * 9 + target - 1) / target);
    const dim3 grid((unsigned)((rows + rows_per_cta - 1) / rows_per_cta), 9);
    k_conv_wgrad_tma<1><<<grid, kWtThreads, wgrad_tma_smem(nb), st>>>(mdp, mx, a, rows_per_cta, nb);
    return cudaGetLastError();
}

static inline unsigned nblk(long long n) { return (unsigned)((n + 255) / 256); }

cudaError_t gkrt_launch_avgpool2_bwd(const void* dout, int dout_c, int dout_off, void* din, int din_c, int din_off,
                                     int B, int H, int W, int C, int accumulate, cudaStream_t st) {
    k_avgpool2_bwd<<<nblk((long long)B * H * W * (C / 8)), 256, 0, st>>>((const __nv_bfloat16*)dout, dout_c, dout_off,
                                                                   (__nv_bfloat16*)din, din_c, din_off, B, H, W, C,
                                                                   accumulate);
    return cudaGetLastError();
}
cudaError_t gkrt_launch_upsample2_bwd(const void* dout, int dout_c, int dout_off, void* din, int din_c, int din_off,
                                      int B, int h, int w, int C, cudaStream_t st) {
    k_upsample2_bwd<<<nblk((long long)B * h * w * (C / 8)), 256, 0, st>>>((const __nv_bfloat16*)dout, dout_c, dout_off,
                                                                    (__nv_bfloat16*)din, din_c, din_off, B, h, w, C);
    return cudaGetLastError();
}
cudaError_t gkrt_launch_relu_bwd(void* dy, int dy_c, int dy_off, const void* y, int y_c, int y_off, long long npix,
                                 int C, cudaStream_t st) {
    k_relu_bwd<<<nblk(npix * (C / 8)), 256, 0, st>>>((__nv_bfloat16*)dy, dy_c, dy_off, (const __nv_bfloat16*)y, y_c,
                                                     y_off, (int)npix, C);
    return cudaGetLastError();
}
cudaError_t gkrt_launch_bias_grad(const void* dp, int dp_c, int dp_off, long long npix, int C, float* db,
                                  cudaStream_t st) {
    if (C > 256 || C % 8 || dp_c % 8 || dp_off % 8 || ((uintptr_t)dp & 15u)) return cudaErrorInvalidValue;
    const int run = 1024;
    k_bias_grad<<<(unsigned)((npix + run - 1) / run), 256, 0, st>>>((const __nv_bfloat16*)dp, dp_c, dp_off, npix, C,
                                                                   run, db);
    return cudaGetLastError();
}
