// k_unet.cu — the learned denoiser's training and inference kernels besides the forward
// convolution (k_conv.cu): weight gradients on the tensor cores, and the element-wise,
// pooling, loss and optimiser kernels.
//
// Weight gradient of a 3x3 convolution, dW[cout][tap][cin] = sum over pixels of
// dP[p][cout] * X[p + tap offset][cin], is a GEMM with M = cout (padded to 128 rows of
// zeros), N = cin and K = pixels. One CTA takes one tap and a run of pixels; both operands
// are staged by the CTA's threads into the 64-byte-swizzled K-major layout (pixels along K)
// straight from the NHWC tensors, made visible to the tensor core with a proxy fence, and
// multiplied by one thread while the next pixels are staged (two buffers); a thread stages an
// 8-pixel x 8-channel block with eight 16-byte loads and stores it transposed (byte permutes)
// as eight 16-byte rows. The FP32
// accumulator is added to dW with atomics. Every wait is bounded.
#include "gk_umma.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kWgThreads = 128;
constexpr int kWgStep = 32;   // pixels per K step

__device__ __forceinline__ uint32_t sw64_offset(int r, int k) {   // byte offset of element (row r, k) in a tile
    return (uint32_t)((r >> 3) * 512 + (r & 7) * 64 + ((((k >> 3) ^ (r >> 1)) & 3) << 4) + (k & 7) * 2);
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ uint32_t word_of(const uint4& v, int i) {
    return i == 0 ? v.x : i == 1 ? v.y : i == 2 ? v.z : v.w;
}

// Stores the 8 x 8 block v (v[i]: 8 channels of pixel i) transposed: row r0 + c of the
// 64-byte-swizzled K-major tile gets the 8 pixels' channel c as one 16-byte chunk at K
// offset k0 (a multiple of 8).
__device__ __forceinline__ void store_block_t(uint8_t* tile, int r0, int k0, const uint4* v) {
#pragma unroll
    for (int c = 0; c < 8; ++c) {
        uint32_t w[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const uint32_t lo = word_of(v[2 * h], c >> 1), hi = word_of(v[2 * h + 1], c >> 1);
            w[h] = (c & 1) ? __byte_perm(lo, hi, 0x7632) : __byte_perm(lo, hi, 0x5410);
        }
        *reinterpret_cast<uint4*>(tile + sw64_offset(r0 + c, k0)) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

__global__ void __launch_bounds__(kWgThreads) k_conv_wgrad(WgradArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
    const int a_bytes = 128 * 64;
    const int b_bytes = ((a.cin * 64) + 1023) & ~1023;
    const int stage_bytes = a_bytes + b_bytes;
    uint64_t* done = reinterpret_cast<uint64_t*>(smem + 2 * stage_bytes);
    uint64_t* accb = done + 2;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accb + 1);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tap = blockIdx.y, dy = tap / 3 - 1, dx = tap % 3 - 1;
    const long long npix = (long long)a.B * a.H * a.W;
    const long long p0 = (long long)blockIdx.x * a.chunk;
    const long long pend = min(p0 + (long long)a.chunk, npix);   // pixels of this CTA: [p0, pend)
    const int nk = (int)((min((long long)a.chunk, npix - p0) + kWgStep - 1) / kWgStep);
    const uint32_t ncols = a.cin <= 32 ? 32u : a.cin <= 64 ? 64u : a.cin <= 128 ? 128u : 256u;

    for (int i = tid; i < 2 * stage_bytes / 16; i += kWgThreads)   // zero rows stay zero (M padding)
        reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    if (tid == 0) {
        mbar_init(&done[0], 1);
        mbar_init(&done[1], 1);
        mbar_init(accb, 1);
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
    const uint32_t idesc = umma_idesc_bf16(128u, (uint32_t)a.cin);
    bool ok = true;
    const int ga = a.cout / 8, gb = a.cin / 8;
    // A[cout][pixel] = dP[pixel][cout] and B[cin][pixel] = X[pixel shifted by the tap][cin]
    // (zero outside the image): per K step, one thread per block of 8 pixels x 8 channels
    // (eight 16-byte loads, consecutive threads on consecutive channel groups), stored
    // transposed as eight 16-byte rows. A thread has at most two blocks per step
    // (4 (cout / 8 + cin / 8) <= 192); it loads its next step's blocks into registers before
    // the barrier of the current one, so the loads are in flight during the barrier and the MMA.
    const int na = (kWgStep / 8) * ga, nb = (kWgStep / 8) * gb;
    uint4 v[2][8];
    auto load_step = [&](int k) {
        const long long qk = p0 + (long long)k * kWgStep;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int it = tid + m * kWgThreads;
            if (it >= na + nb) continue;
            const bool is_a = it < na;
            const int j = is_a ? it : it - na, gn = is_a ? ga : gb;
            const int g = j % gn, jb = j / gn;
            const long long q0 = qk + 8 * jb;
            if (is_a) {
#pragma unroll
                for (int i = 0; i < 8; ++i)
                    v[m][i] = q0 + i < pend
                                  ? *reinterpret_cast<const uint4*>(a.dp + (q0 + i) * a.dp_c + a.dp_off + 8 * g)
                                  : make_uint4(0u, 0u, 0u, 0u);
            } else {
                // coordinates of the block's first pixel, then stepped along the row
                int x = 0, y = 0;
                long long b = 0;
                if (q0 < pend) {
                    const long long row = q0 / a.W;
                    x = (int)(q0 - row * a.W);
                    y = (int)(row % a.H);
                    b = row / a.H;
                }
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    v[m][i] = make_uint4(0u, 0u, 0u, 0u);
                    if (q0 + i < pend) {
                        const int xs = x + dx, ys = y + dy;
                        if (xs >= 0 && xs < a.W && ys >= 0 && ys < a.H)
                            v[m][i] = *reinterpret_cast<const uint4*>(a.x + ((b * a.H + ys) * a.W + xs) * a.x_c +
                                                                      a.x_off + 8 * g);
                    }
                    if (++x == a.W) {
                        x = 0;
                        if (++y == a.H) { y = 0; ++b; }
                    }
                }
            }
        }
    };
    if (nk > 0) load_step(0);
    for (int k = 0; k < nk && ok; ++k) {
        const int s = k & 1;
        if (k >= 2 && !mbar_wait_bounded(&done[s], (uint32_t)((k >> 1) - 1) & 1u, a.err)) ok = false;
        if (__syncthreads_or(!ok)) { ok = false; break; }
        uint8_t* sa = smem + s * stage_bytes;
        uint8_t* sb = sa + a_bytes;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            const int it = tid + m * kWgThreads;
            if (it >= na + nb) continue;
            const bool is_a = it < na;
            const int j = is_a ? it : it - na, gn = is_a ? ga : gb;
            store_block_t(is_a ? sa : sb, 8 * (j % gn), 8 * (j / gn), v[m]);
        }
        if (k + 1 < nk) load_step(k + 1);
        fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            tc_fence_after();
            const uint32_t ua = smem_u32(sa), ub = smem_u32(sb);
            umma_bf16(tmem, umma_desc_sw64(ua), umma_desc_sw64(ub), idesc, k != 0 ? 1u : 0u);
            umma_bf16(tmem, umma_desc_sw64(ua + 32u), umma_desc_sw64(ub + 32u), idesc, 1u);
            umma_commit(&done[s]);
        }
    }
    if (tid == 0) umma_commit(accb);
    const bool ready = mbar_wait_bounded(accb, 0u, a.err) && ok && nk > 0;
    __syncwarp();
    tc_fence_after();
    const int r = warp * 32 + lane;   // TMEM lane = cout row
    for (int c0 = 0; c0 < a.cin; c0 += 16) {
        uint32_t v[16];
        tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
        tmem_ld_wait();
        if (!ready || r >= a.cout) continue;
        float* d = a.dw + ((size_t)r * 9 + tap) * a.cin + c0;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const float f = __uint_as_float(v[j]);
            if (f != 0.0f) atomicAdd(d + j, f);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, ncols);
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

size_t gkrt_wgrad_smem_bytes(int cin) {
    return 2 * (size_t)(128 * 64 + (((cin * 64) + 1023) & ~1023)) + 64 + 1024;
}

cudaError_t gkrt_launch_conv_wgrad(const WgradArgs& a, cudaStream_t st) {
    if (a.cin % 16 || a.cin < 16 || a.cin > 256 || a.cout % 8 || a.cout > 128 || a.chunk % kWgStep || a.chunk <= 0 ||
        a.dp_c % 8 || a.dp_off % 8 || a.x_c % 8 || a.x_off % 8 || ((uintptr_t)a.dp & 15u) || ((uintptr_t)a.x & 15u))
        return cudaErrorInvalidValue;
    const long long npix = (long long)a.B * a.H * a.W;
    const size_t smem = gkrt_wgrad_smem_bytes(a.cin);
    static bool attr_set[kMaxDevices] = {};   // set once per device for the largest operand (cin = 256)
    const int dev = current_device_slot();
    if (dev < 0) return cudaErrorInvalidDevice;
    if (!attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k_conv_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)gkrt_wgrad_smem_bytes(256));
        if (e != cudaSuccess) return e;
        attr_set[dev] = true;
    }
    const dim3 grid((unsigned)((npix + a.chunk - 1) / a.chunk), 9);
    k_conv_wgrad<<<grid, kWgThreads, smem, st>>>(a);
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
