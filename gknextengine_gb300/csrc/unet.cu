// unet.cu — the learned denoiser: a 4-level convolutional U-Net in bf16 on the tensor cores,
// trained and run by this library's own kernels (no counterpart in the reference: its learned
// denoiser is the closed OIDN library, PathTracingRenderer.cpp:33-64, 234-269).
//
// Inputs, 10 channels per pixel: 1-spp linear radiance (as log(1 + x)), albedo, normal,
// depth (NDC, clamped to [0, 1]: camera misses carry 100000); stored as 16 channels (zeros
// after the 10), the first layer reads 32 (the rest as zeros). Output: log(1 + radiance), 3
// channels, stored with a fourth (an unused network output) so that each pixel is one 16-byte
// store.
//   level 0 (full)   enc0a 32->32, enc0b 32->32 ............ dec0a 96->32, dec0b 32->32, out 32->3
//   level 1 (1/2)    enc1a 32->64, enc1b 64->64 ............ dec1a 160->64, dec1b 64->64
//   level 2 (1/4)    enc2a 64->96, enc2b 96->96 ............ dec2a 224->96, dec2b 96->96
//   level 3 (1/8)    enc3a 96->128, enc3b 128->128
// 3x3 convolutions with ReLU (none on the output), 2x2 average pooling down, nearest 2x
// upsampling up, skips concatenated in place: each decoder input tensor holds the upsampled
// deeper features in its first channels and the encoder output (written there directly by
// the encoder's convolution) in the rest. Training: loss = mean squared error in
// log(1 + radiance) against the target, Adam on FP32 master weights, bf16 copies of the
// weights in the forward layout [cout][tap][cin] and in the transposed, tap-mirrored layout
// [cin][8 - tap][cout] that turns the input gradient into a forward convolution.
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "gk_device.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

struct LayerDef {
    int cin, cout, relu, n_store;
};
// enc0a enc0b enc1a enc1b enc2a enc2b enc3a enc3b dec2a dec2b dec1a dec1b dec0a dec0b out
constexpr LayerDef kLayers[kUnetLayers] = {
    {32, 32, 1, 32},   {32, 32, 1, 32},   {32, 64, 1, 64},  {64, 64, 1, 64},  {64, 96, 1, 96},
    {96, 96, 1, 96},   {96, 128, 1, 128}, {128, 128, 1, 128}, {224, 96, 1, 96}, {96, 96, 1, 96},
    {160, 64, 1, 64},  {64, 64, 1, 64},   {96, 32, 1, 32},  {32, 32, 1, 32},  {32, 32, 0, 4}};
enum { E0A, E0B, E1A, E1B, E2A, E2B, E3A, E3B, D2A, D2B, D1A, D1B, D0A, D0B, OUT };

// The network input x0: kXc channels per pixel (the 10 inputs, then zeros); the first layer's
// 32 input channels read the ones past kXc as zeros (its tensor map ends there).
constexpr int kXc = 16;

// 256 pixels per block: their 10 KB of input are read as whole 16-byte words into shared
// memory (pixel-per-thread loads of 40-byte records touch every line ten times).
__global__ void __launch_bounds__(256) k_pack_input(const float* in, long long npix, __nv_bfloat16* x0) {
    __shared__ __align__(16) float rec[256 * 10];
    const long long p0 = blockIdx.x * 256LL;
    const int n = (int)(npix - p0 < 256 ? npix - p0 : 256);
    const float* src = in + p0 * 10;
    if (n == 256 && !(reinterpret_cast<uintptr_t>(src) & 15u)) {
        for (int i = threadIdx.x; i < 640; i += 256)
            reinterpret_cast<float4*>(rec)[i] = __ldcs(reinterpret_cast<const float4*>(src) + i);
    } else {
        for (int i = threadIdx.x; i < n * 10; i += 256) rec[i] = src[i];
    }
    __syncthreads();
    float v[kXc];
#pragma unroll
    for (int c = 0; c < kXc; ++c) v[c] = 0.0f;
    if ((int)threadIdx.x < n) {   // one pixel
#pragma unroll
        for (int c = 0; c < 10; ++c) v[c] = rec[threadIdx.x * 10 + c];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) v[c] = log1pf(fmaxf(v[c], 0.0f));
    v[9] = fminf(fmaxf(v[9], 0.0f), 1.0f);   // depth; misses carry 100000
    __syncthreads();   // rec now holds the packed pixels (32 bytes each), stored as whole lines
    uint4* packed = reinterpret_cast<uint4*>(rec);
#pragma unroll
    for (int k = 0; k < kXc / 8; ++k) {
        __nv_bfloat162 h[4];
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(v[8 * k + 2 * j], v[8 * k + 2 * j + 1]);
        packed[threadIdx.x * (kXc / 8) + k] = *reinterpret_cast<uint4*>(h);
    }
    __syncthreads();
    uint4* o = reinterpret_cast<uint4*>(x0 + p0 * kXc);
    for (int i = threadIdx.x; i < n * (kXc / 8); i += 256) o[i] = packed[i];
}

// From the pass's images (pitched float4 / float): composed 1-spp radiance
// (diffuse x albedo + specular), albedo, normal, depth.
// (256 pixels per block, their packed 32-byte records stored as whole lines through shared memory)
__global__ void __launch_bounds__(256) k_pack_frame(const float4* sd, const float4* ss, const float4* alb,
                                                    const float4* nrm, const float* depth, int W, int H, int P,
                                                    __nv_bfloat16* x0) {
    __shared__ __align__(16) uint4 packed[256 * (kXc / 8)];
    const long long i0 = blockIdx.x * 256LL, i = i0 + threadIdx.x;
    const long long npix = (long long)W * H;
    const int n = (int)(npix - i0 < 256 ? npix - i0 : 256);
    float v[kXc];
#pragma unroll
    for (int c = 0; c < kXc; ++c) v[c] = 0.0f;
    if (i < npix) {
        const int x = (int)(i % W), y = (int)(i / W);
        const size_t q = (size_t)y * P + x;
        const float4 d = sd[q], s = ss[q], a = alb[q], n4 = nrm[q];
        v[0] = log1pf(fmaxf(fmaf(d.x, a.x, s.x), 0.0f));
        v[1] = log1pf(fmaxf(fmaf(d.y, a.y, s.y), 0.0f));
        v[2] = log1pf(fmaxf(fmaf(d.z, a.z, s.z), 0.0f));
        v[3] = a.x; v[4] = a.y; v[5] = a.z;
        v[6] = n4.x; v[7] = n4.y; v[8] = n4.z;
        v[9] = fminf(fmaxf(depth[q], 0.0f), 1.0f);   // misses carry 100000
    }
#pragma unroll
    for (int k = 0; k < kXc / 8; ++k) {
        __nv_bfloat162 h[4];
        for (int j = 0; j < 4; ++j) h[j] = __floats2bfloat162_rn(v[8 * k + 2 * j], v[8 * k + 2 * j + 1]);
        packed[threadIdx.x * (kXc / 8) + k] = *reinterpret_cast<uint4*>(h);
    }
    __syncthreads();
    uint4* o = reinterpret_cast<uint4*>(x0 + i0 * kXc);
    for (int j = threadIdx.x; j < n * (kXc / 8); j += 256) o[j] = packed[j];
}

// gradient of the loss in log space; loss sum in FP64
__global__ void k_loss(const float* y, const float* target, long long npix, float gscale, __nv_bfloat16* gy,
                       double* loss) {
    __shared__ double part[8];
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    double l = 0.0;
    if (p < npix) {
        __nv_bfloat16* g = gy + p * 32;
        for (int c = 0; c < 3; ++c) {
            const float e = y[p * 4 + c] - log1pf(fmaxf(target[p * 3 + c], 0.0f));
            l += (double)e * e;
            g[c] = __float2bfloat16_rn(2.0f * e * gscale);
        }
        for (int c = 3; c < 32; ++c) g[c] = __float2bfloat16_rn(0.0f);
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_down_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += part[k];
        atomicAdd(loss, s);
    }
}

// caller-supplied gradient of the raw output (f32, 4 channels) to the bf16 32-channel layout
__global__ void k_grad_in(const float* d, long long npix, __nv_bfloat16* gy) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= npix * 32) return;
    const int c = (int)(i % 32);
    gy[i] = __float2bfloat16_rn(c < 3 ? d[(i / 32) * 4 + c] : 0.0f);
}

__global__ void k_out_linear(const float* y, long long npix, float* out) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= npix) return;
    for (int c = 0; c < 3; ++c) out[p * 4 + c] = fmaxf(expm1f(fminf(y[p * 4 + c], kUnetMaxLog)), 0.0f);
    out[p * 4 + 3] = 1.0f;
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, long long n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// bf16 weights in both layouts: wb[co][tap][ci] and wf[ci][8 - tap][co]
__global__ void k_weights_bf16(const float* w, int cin, int cout, __nv_bfloat16* wb, __nv_bfloat16* wf) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= 9LL * cin * cout) return;
    const int ci = (int)(i % cin);
    const int tap = (int)((i / cin) % 9);
    const int co = (int)(i / (9LL * cin));
    const __nv_bfloat16 h = __float2bfloat16_rn(w[i]);
    wb[i] = h;
    wf[((long long)ci * 9 + (8 - tap)) * cout + co] = h;
}

// dec0a's weights (fp32 [32][9][96]; input channels 0-63 the nearest-upsampled dec1b, 64-95
// enc0b) as the inference forward's two convolutions. A 3x3 tap (dy, dx) of output pixel
// (2i + a, 2j + b) reads the upsampled input at half-resolution offset (floor((a + dy) / 2),
// floor((b + dx) / 2)), so over the upsampled channels the layer is, per parity (a, b), a 3x3
// convolution at half resolution whose tap weights are the sums of the full-resolution taps
// reading that offset (zero padding agrees, H and W being even):
//   wup[(2a + b) 32 + co][3 (dyl + 1) + dxl + 1][ci] = sum of w[co][3 (dy + 1) + dx + 1][ci]
//     over dy, dx in -1..1 (ascending) with floor((a + dy) / 2) = dyl, floor((b + dx) / 2) = dxl,
// summed in FP32 and rounded to bf16; we0b[co][tap][ci] = w[co][tap][64 + ci].
__device__ __forceinline__ int floor_half(int v) { return (v + 2) / 2 - 1; }   // v in -1..2
__global__ void k_weights_subpixel(const float* w, __nv_bfloat16* wup, __nv_bfloat16* we0b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 128 * 9 * 64) {
        const int ci = i % 64, lt = (i / 64) % 9, n = i / (64 * 9);
        const int a = (n / 32) >> 1, b = (n / 32) & 1, co = n % 32;
        const int dyl = lt / 3 - 1, dxl = lt % 3 - 1;
        float acc = 0.0f;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx)
                if (floor_half(a + dy) == dyl && floor_half(b + dx) == dxl)
                    acc = acc + w[((size_t)co * 9 + 3 * (dy + 1) + dx + 1) * 96 + ci];
        wup[i] = __float2bfloat16_rn(acc);
    }
    if (i < 32 * 9 * 32) {
        const int ci = i % 32, tap = (i / 32) % 9, co = i / (32 * 9);
        we0b[i] = __float2bfloat16_rn(w[((size_t)co * 9 + tap) * 96 + 64 + ci]);
    }
}

inline unsigned nb(long long n) { return (unsigned)((n + 255) / 256); }

}  // namespace

struct Unet {
    size_t woff[kUnetLayers], boff[kUnetLayers], wb_off[kUnetLayers];
    size_t nparams = 0, nweights_bf16 = 0;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wb = nullptr, *wf = nullptr;
    __nv_bfloat16 *wup = nullptr, *we0b = nullptr;   // dec0a as the inference forward's convolutions
    bool train_acts = false;   // the activations are the training forward's (backward may run)
    int step = 0;
    int B = 0, H = 0, W = 0;
    void* arena = nullptr;
    size_t arena_bytes = 0;
    // activations (bf16 NHWC) and their gradients
    __nv_bfloat16 *x0, *e0a, *cat0, *p0, *e1a, *cat1, *p1, *e2a, *cat2, *p2, *e3a, *e3b, *d2a, *d2b, *d1a, *d1b, *d0a,
        *d0b;
    __nv_bfloat16 *gy, *g_d0b, *g_d0a, *g_cat0, *g_d1b, *g_d1a, *g_cat1, *g_d2b, *g_d2a, *g_cat2, *g_e3b, *g_e3a, *g_p2,
        *g_e2a, *g_p1, *g_e1a, *g_p0, *g_e0a;
    float* y = nullptr;
    double* d_loss = nullptr;
    uint32_t* err = nullptr;

    Unet() {
        size_t off = 0, wo = 0;
        for (int l = 0; l < kUnetLayers; ++l) {
            woff[l] = off;
            off += 9ull * kLayers[l].cin * kLayers[l].cout;
            boff[l] = off;
            off += kLayers[l].cout;
            wb_off[l] = wo;
            wo += 9ull * kLayers[l].cin * kLayers[l].cout;
        }
        nparams = off;
        nweights_bf16 = wo;
    }
    ~Unet() {
        for (void* q : {(void*)p, (void*)g, (void*)m, (void*)v, (void*)wb, (void*)wf, (void*)wup, (void*)we0b, arena,
                        (void*)d_loss, (void*)err})
            if (q) cudaFree(q);
    }

    cudaError_t alloc_params() {
        cudaError_t e;
        for (float** q : {&p, &g, &m, &v})
            if ((e = cudaMalloc((void**)q, nparams * sizeof(float))) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&wb, nweights_bf16 * 2)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&wf, nweights_bf16 * 2)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&wup, 128 * 9 * 64 * 2)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&we0b, 32 * 9 * 32 * 2)) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&d_loss, sizeof(double))) != cudaSuccess) return e;
        if ((e = cudaMalloc((void**)&err, 4)) != cudaSuccess) return e;
        return cudaMemset(err, 0, 4);
    }

    // bf16 copies of the weights from the FP32 masters
    cudaError_t refresh_bf16(cudaStream_t st) {
        for (int l = 0; l < kUnetLayers; ++l) {
            const long long n = 9LL * kLayers[l].cin * kLayers[l].cout;
            k_weights_bf16<<<nb(n), 256, 0, st>>>(p + woff[l], kLayers[l].cin, kLayers[l].cout, wb + wb_off[l],
                                                  wf + wb_off[l]);
        }
        k_weights_subpixel<<<nb(128 * 9 * 64), 256, 0, st>>>(p + woff[D0A], wup, we0b);
        return cudaGetLastError();
    }

    cudaError_t ensure_size(int b, int h, int w) {
        if (b == B && h == H && w == W && arena) return cudaSuccess;
        if (arena) cudaFree(arena);
        arena = nullptr;
        B = H = W = 0;
        struct Req {
            __nv_bfloat16** ptr;
            int level, ch;
        };
        const Req reqs[] = {{&x0, 0, kXc},    {&e0a, 0, 32},   {&cat0, 0, 96},   {&p0, 1, 32},    {&e1a, 1, 64},
                            {&cat1, 1, 160}, {&p1, 2, 64},    {&e2a, 2, 96},    {&cat2, 2, 224}, {&p2, 3, 96},
                            {&e3a, 3, 128},  {&e3b, 3, 128},  {&d2a, 2, 96},    {&d2b, 2, 96},   {&d1a, 1, 64},
                            {&d1b, 1, 64},   {&d0a, 0, 32},   {&d0b, 0, 32},    {&gy, 0, 32},    {&g_d0b, 0, 32},
                            {&g_d0a, 0, 32}, {&g_cat0, 0, 96}, {&g_d1b, 1, 64}, {&g_d1a, 1, 64}, {&g_cat1, 1, 160},
                            {&g_d2b, 2, 96}, {&g_d2a, 2, 96}, {&g_cat2, 2, 224}, {&g_e3b, 3, 128}, {&g_e3a, 3, 128},
                            {&g_p2, 3, 96},  {&g_e2a, 2, 96}, {&g_p1, 2, 64},   {&g_e1a, 1, 64}, {&g_p0, 1, 32},
                            {&g_e0a, 0, 32}};
        size_t total = 0;
        std::vector<size_t> offs;
        for (const Req& r : reqs) {
            offs.push_back(total);
            const size_t px = (size_t)b * (h >> r.level) * (w >> r.level);
            total += (px * r.ch * 2 + 255) & ~(size_t)255;
        }
        const size_t ybytes = ((size_t)b * h * w * 16 + 255) & ~(size_t)255;
        cudaError_t e = cudaMalloc(&arena, total + ybytes);
        if (e != cudaSuccess) return e;
        e = cudaMemset(arena, 0, total + ybytes);
        if (e != cudaSuccess) return e;
        for (size_t i = 0; i < offs.size(); ++i)
            *reqs[i].ptr = reinterpret_cast<__nv_bfloat16*>(static_cast<uint8_t*>(arena) + offs[i]);
        y = reinterpret_cast<float*>(static_cast<uint8_t*>(arena) + total);
        B = b;
        H = h;
        W = w;
        arena_bytes = total + ybytes;
        return cudaSuccess;
    }

    // pool / up (optional): the epilogue also writes the 2 x 2 average of the output at half
    // resolution, or the output at double resolution (nearest), at channel offset *_off of a
    // tensor of *_c channels
    cudaError_t conv(int l, const __nv_bfloat16* in, int in_c, int in_off, void* out, int out_c, int out_off, int level,
                     cudaStream_t st, __nv_bfloat16* pool = nullptr, int pool_c = 0, int pool_off = 0,
                     __nv_bfloat16* up = nullptr, int up_c = 0, int up_off = 0) {
        ConvArgs a{};
        a.B = B; a.H = H >> level; a.W = W >> level;
        a.cin = kLayers[l].cin; a.cout = kLayers[l].cout;
        // the output layer stores 4 of its 32 channels: its first 16 weight rows (an MMA of
        // N = 16) compute them; the gradients of the others are zero (their loss gradient is)
        if (l == OUT) a.cout = 16;
        a.x_c = in_c; a.x_off = in_off;
        a.x_valid = in_c - in_off < a.cin ? in_c - in_off : 0;   // x0 holds fewer channels than E0A's 32
        a.bias = p + boff[l];
        a.out = out; a.out_c = out_c; a.out_off = out_off;
        a.n_store = kLayers[l].n_store;
        a.flags = (kLayers[l].relu ? kConvRelu : 0) | (l == OUT ? kConvF32Out : 0);
        a.err = err;
        a.pool_out = pool; a.pool_c = pool_c; a.pool_off = pool_off;
        a.up_out = up; a.up_c = up_c; a.up_off = up_off;
        return gkrt_launch_conv3x3(in, wb + wb_off[l], a, st);
    }

    // train: the forward whose activations the backward reads (the upsampled copies in the
    // concatenations). Otherwise dec1b's upsampled copy is not written: dec0a runs as the
    // sub-pixel convolution of dec1b at half resolution (the four parities, 128 channels, into
    // the unused gradient buffer g_cat0) and a convolution over enc0b (dense in g_e0a) that adds
    // them.
    cudaError_t forward(cudaStream_t st, bool train) {
        cudaError_t e;
        train_acts = train;
#define GK_T(x) if ((e = (x)) != cudaSuccess) return e
        GK_T(conv(E0A, x0, kXc, 0, e0a, 32, 0, 0, st));
        // the 2 x 2 pools and nearest upsamplings ride in the epilogues of the convolutions that
        // produce their inputs: 2 x 2 means of the stored values, nearest copies
        // inference: enc0b dense in the unused gradient buffer g_e0a (the sub-pixel dec0a reads it
        // alone); training: into its concatenation
        __nv_bfloat16* e0b = train ? cat0 : g_e0a;
        const int e0b_c = train ? 96 : 32, e0b_off = train ? 64 : 0;
        GK_T(conv(E0B, e0a, 32, 0, e0b, e0b_c, e0b_off, 0, st, p0, 32, 0));
        GK_T(conv(E1A, p0, 32, 0, e1a, 64, 0, 1, st));
        GK_T(conv(E1B, e1a, 64, 0, cat1, 160, 96, 1, st, p1, 64, 0));
        GK_T(conv(E2A, p1, 64, 0, e2a, 96, 0, 2, st));
        GK_T(conv(E2B, e2a, 96, 0, cat2, 224, 128, 2, st, p2, 96, 0));
        GK_T(conv(E3A, p2, 96, 0, e3a, 128, 0, 3, st));
        GK_T(conv(E3B, e3a, 128, 0, e3b, 128, 0, 3, st, nullptr, 0, 0, cat2, 224, 0));
        GK_T(conv(D2A, cat2, 224, 0, d2a, 96, 0, 2, st));
        GK_T(conv(D2B, d2a, 96, 0, d2b, 96, 0, 2, st, nullptr, 0, 0, cat1, 160, 0));
        GK_T(conv(D1A, cat1, 160, 0, d1a, 64, 0, 1, st));
        if (train) {
            GK_T(conv(D1B, d1a, 64, 0, d1b, 64, 0, 1, st, nullptr, 0, 0, cat0, 96, 0));
            GK_T(conv(D0A, cat0, 96, 0, d0a, 32, 0, 0, st));
        } else {
            GK_T(conv(D1B, d1a, 64, 0, d1b, 64, 0, 1, st));
            __nv_bfloat16* par = g_cat0;   // B x H/2 x W/2 x 128 fits in B x H x W x 96
            ConvArgs a{};
            a.B = B; a.H = H >> 1; a.W = W >> 1; a.cin = 64; a.cout = 128;
            a.x_c = 64;
            a.out = par; a.out_c = 128; a.n_store = 128;
            a.err = err;
            GK_T(gkrt_launch_conv3x3(d1b, wup, a, st));
            ConvArgs c{};
            c.B = B; c.H = H; c.W = W; c.cin = 32; c.cout = 32;
            c.x_c = e0b_c; c.x_off = e0b_off;
            c.bias = p + boff[D0A];
            c.out = d0a; c.out_c = 32; c.n_store = 32;
            c.flags = kConvRelu;
            c.err = err;
            c.add_par = par; c.add_c = 128;
            GK_T(gkrt_launch_conv3x3(e0b, we0b, c, st));
        }
        GK_T(conv(D0B, d0a, 32, 0, d0b, 32, 0, 0, st));
        GK_T(conv(OUT, d0b, 32, 0, y, 4, 0, 0, st));
        return cudaSuccess;
    }

    // One layer's backward: dP (in place of dY) = dY * relu', weight and bias gradients, and
    // (if din) the input gradient through the mirrored weights.
    cudaError_t layer_bwd(int l, __nv_bfloat16* dy, int dy_c, int dy_off, const __nv_bfloat16* y_act, int y_c,
                          int y_off, const __nv_bfloat16* x, int x_c, int x_off, __nv_bfloat16* din, int level,
                          cudaStream_t st) {
        cudaError_t e;
        const int h = H >> level, w = W >> level;
        const long long npix = (long long)B * h * w;
        const LayerDef& L = kLayers[l];
        if (L.relu) GK_T(gkrt_launch_relu_bwd(dy, dy_c, dy_off, y_act, y_c, y_off, npix, L.cout, st));
        WgradArgs wa{};
        wa.B = B; wa.H = h; wa.W = w;
        wa.dp = dy; wa.dp_c = dy_c; wa.dp_off = dy_off; wa.cout = L.cout;
        wa.x = x; wa.x_c = x_c; wa.x_off = x_off; wa.cin = L.cin;
        wa.x_valid = x_c - x_off < L.cin ? x_c - x_off : 0;
        wa.dw = g + woff[l];
        wa.err = err;
        GK_T(gkrt_launch_conv_wgrad(wa, st));
        GK_T(gkrt_launch_bias_grad(dy, dy_c, dy_off, npix, L.cout, g + boff[l], st));
        if (din) {
            ConvArgs a{};
            a.B = B; a.H = h; a.W = w;
            a.cin = L.cout; a.cout = L.cin;
            a.x_c = dy_c; a.x_off = dy_off;
            a.bias = nullptr;
            a.out = din; a.out_c = L.cin; a.out_off = 0;
            a.n_store = L.cin;
            a.flags = 0;
            a.err = err;
            GK_T(gkrt_launch_conv3x3(dy, wf + wb_off[l], a, st));
        }
        return cudaSuccess;
    }

    cudaError_t backward(cudaStream_t st) {   // gy holds d loss / d output (bf16, 32 channels)
        cudaError_t e;
        GK_T(layer_bwd(OUT, gy, 32, 0, nullptr, 0, 0, d0b, 32, 0, g_d0b, 0, st));
        GK_T(layer_bwd(D0B, g_d0b, 32, 0, d0b, 32, 0, d0a, 32, 0, g_d0a, 0, st));
        GK_T(layer_bwd(D0A, g_d0a, 32, 0, d0a, 32, 0, cat0, 96, 0, g_cat0, 0, st));
        GK_T(gkrt_launch_upsample2_bwd(g_cat0, 96, 0, g_d1b, 64, 0, B, H >> 1, W >> 1, 64, st));
        GK_T(layer_bwd(D1B, g_d1b, 64, 0, d1b, 64, 0, d1a, 64, 0, g_d1a, 1, st));
        GK_T(layer_bwd(D1A, g_d1a, 64, 0, d1a, 64, 0, cat1, 160, 0, g_cat1, 1, st));
        GK_T(gkrt_launch_upsample2_bwd(g_cat1, 160, 0, g_d2b, 96, 0, B, H >> 2, W >> 2, 96, st));
        GK_T(layer_bwd(D2B, g_d2b, 96, 0, d2b, 96, 0, d2a, 96, 0, g_d2a, 2, st));
        GK_T(layer_bwd(D2A, g_d2a, 96, 0, d2a, 96, 0, cat2, 224, 0, g_cat2, 2, st));
        GK_T(gkrt_launch_upsample2_bwd(g_cat2, 224, 0, g_e3b, 128, 0, B, H >> 3, W >> 3, 128, st));
        GK_T(layer_bwd(E3B, g_e3b, 128, 0, e3b, 128, 0, e3a, 128, 0, g_e3a, 3, st));
        GK_T(layer_bwd(E3A, g_e3a, 128, 0, e3a, 128, 0, p2, 96, 0, g_p2, 3, st));
        // the encoder output of level 2 feeds both the pool and the skip
        GK_T(gkrt_launch_avgpool2_bwd(g_p2, 96, 0, g_cat2, 224, 128, B, H >> 2, W >> 2, 96, 1, st));
        GK_T(layer_bwd(E2B, g_cat2, 224, 128, cat2, 224, 128, e2a, 96, 0, g_e2a, 2, st));
        GK_T(layer_bwd(E2A, g_e2a, 96, 0, e2a, 96, 0, p1, 64, 0, g_p1, 2, st));
        GK_T(gkrt_launch_avgpool2_bwd(g_p1, 64, 0, g_cat1, 160, 96, B, H >> 1, W >> 1, 64, 1, st));
        GK_T(layer_bwd(E1B, g_cat1, 160, 96, cat1, 160, 96, e1a, 64, 0, g_e1a, 1, st));
        GK_T(layer_bwd(E1A, g_e1a, 64, 0, e1a, 64, 0, p0, 32, 0, g_p0, 1, st));
        GK_T(gkrt_launch_avgpool2_bwd(g_p0, 32, 0, g_cat0, 96, 64, B, H, W, 32, 1, st));
        GK_T(layer_bwd(E0B, g_cat0, 96, 64, cat0, 96, 64, e0a, 32, 0, g_e0a, 0, st));
        GK_T(layer_bwd(E0A, g_e0a, 32, 0, e0a, 32, 0, x0, kXc, 0, nullptr, 0, st));
        return cudaSuccess;
    }
#undef GK_T
};

}  // namespace gk

using namespace gk;

// ---- host entry points used by gkrt_api.cu ----
Unet* gkrt_unet_new() { return new (std::nothrow) Unet(); }
void gkrt_unet_delete(Unet* u) { delete u; }
size_t gkrt_unet_nparams(const Unet* u) { return u->nparams; }

cudaError_t gkrt_unet_init_params(Unet* u, uint64_t seed) {
    cudaError_t e = u->p ? cudaSuccess : u->alloc_params();
    if (e != cudaSuccess) return e;
    std::vector<float> h(u->nparams, 0.0f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < kUnetLayers; ++l) {
        const double sd = std::sqrt(2.0 / (9.0 * kLayers[l].cin)) * (l == OUT ? 0.1 : 1.0);
        std::normal_distribution<double> nd(0.0, sd);
        for (size_t i = 0; i < 9ull * kLayers[l].cin * kLayers[l].cout; ++i) h[u->woff[l] + i] = (float)nd(rng);
    }
    return gkrt_unet_set_params_host(u, h.data());
}

cudaError_t gkrt_unet_set_params_host(Unet* u, const float* h) {
    cudaError_t e = u->p ? cudaSuccess : u->alloc_params();
    if (e != cudaSuccess) return e;
    if ((e = cudaMemcpy(u->p, h, u->nparams * 4, cudaMemcpyHostToDevice)) != cudaSuccess) return e;
    for (float* q : {u->g, u->m, u->v})
        if ((e = cudaMemset(q, 0, u->nparams * 4)) != cudaSuccess) return e;
    u->step = 0;
    if ((e = u->refresh_bf16(0)) != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}

cudaError_t gkrt_unet_get_params_host(Unet* u, float* params, float* grads) {
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess && params) e = cudaMemcpy(params, u->p, u->nparams * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && grads) e = cudaMemcpy(grads, u->g, u->nparams * 4, cudaMemcpyDeviceToHost);
    return e;
}

// Adam's moments and step count, for checkpoints (set_params resets them).
cudaError_t gkrt_unet_get_state_host(Unet* u, float* m, float* v, uint64_t* step) {
    if (!u->p) return cudaErrorInvalidValue;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess && m) e = cudaMemcpy(m, u->m, u->nparams * 4, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && v) e = cudaMemcpy(v, u->v, u->nparams * 4, cudaMemcpyDeviceToHost);
    if (step) *step = (uint64_t)u->step;
    return e;
}
cudaError_t gkrt_unet_set_state_host(Unet* u, const float* m, const float* v, uint64_t step) {
    if (!u->p || step > 0x7FFFFFFFull) return cudaErrorInvalidValue;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(u->m, m, u->nparams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(u->v, v, u->nparams * 4, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) u->step = (int)step;
    return e;
}

cudaError_t gkrt_unet_zero_grad(Unet* u, cudaStream_t st) { return cudaMemsetAsync(u->g, 0, u->nparams * 4, st); }

static cudaError_t forward_dev(Unet* u, const float* input, int b, int h, int w, float* out_linear, float* out_raw,
                               bool train, cudaStream_t st) {
    cudaError_t e = u->ensure_size(b, h, w);
    if (e != cudaSuccess) return e;
    const long long npix = (long long)b * h * w;
    if (input) k_pack_input<<<nb(npix), 256, 0, st>>>(input, npix, u->x0);
    if ((e = u->forward(st, train)) != cudaSuccess) return e;
    if (out_linear) k_out_linear<<<nb(npix), 256, 0, st>>>(u->y, npix, out_linear);
    if (out_raw) e = cudaMemcpyAsync(out_raw, u->y, npix * 16, cudaMemcpyDeviceToDevice, st);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

// Inference: the sub-pixel form of dec0a. A backward after it runs the training forward again
// on the same packed input (x0) for the activations it reads.
cudaError_t gkrt_unet_forward_dev(Unet* u, const float* input, int b, int h, int w, float* out_linear, float* out_raw,
                                  cudaStream_t st) {
    return forward_dev(u, input, b, h, w, out_linear, out_raw, false, st);
}

cudaError_t gkrt_unet_backward_dev(Unet* u, const float* d_raw, cudaStream_t st) {
    const long long npix = (long long)u->B * u->H * u->W;
    cudaError_t e;
    if (!u->train_acts && (e = u->forward(st, true)) != cudaSuccess) return e;
    k_grad_in<<<nb(npix * 32), 256, 0, st>>>(d_raw, npix, u->gy);
    return u->backward(st);
}

cudaError_t gkrt_unet_train_step_dev(Unet* u, const float* input, const float* target, int b, int h, int w, float lr,
                                     double* loss_host, cudaStream_t st) {
    cudaError_t e = forward_dev(u, input, b, h, w, nullptr, nullptr, true, st);
    if (e != cudaSuccess) return e;
    const long long npix = (long long)b * h * w;
    if ((e = cudaMemsetAsync(u->d_loss, 0, sizeof(double), st)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(u->g, 0, u->nparams * 4, st)) != cudaSuccess) return e;
    // gradients of the per-image sum of squared log errors (Adam does not see the scale)
    k_loss<<<nb(npix), 256, 0, st>>>(u->y, target, npix, 1.0f, u->gy, u->d_loss);
    if ((e = u->backward(st)) != cudaSuccess) return e;
    u->step += 1;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, u->step)));
    const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, u->step)));
    k_adam<<<nb((long long)u->nparams), 256, 0, st>>>(u->p, u->g, u->m, u->v, (long long)u->nparams, lr, b1, b2, 1e-8f,
                                                     c1, c2);
    if ((e = u->refresh_bf16(st)) != cudaSuccess) return e;
    if (loss_host) {
        double l = 0.0;
        if ((e = cudaMemcpyAsync(&l, u->d_loss, sizeof(double), cudaMemcpyDeviceToHost, st)) != cudaSuccess) return e;
        if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return e;
        *loss_host = l / (double)(npix * 3);
    }
    return cudaGetLastError();
}

// Denoise the pass's current 1-spp images; writes linear radiance (float4, pitched) to
// out_linear via the compose writer's arguments.
cudaError_t gkrt_unet_denoise_frame(Unet* u, const float4* sd, const float4* ss, const float4* alb, const float4* nrm,
                                    const float* depth, int W, int H, int P, float* y_out_raw, cudaStream_t st) {
    cudaError_t e = u->ensure_size(1, H, W);
    if (e != cudaSuccess) return e;
    k_pack_frame<<<nb((long long)W * H), 256, 0, st>>>(sd, ss, alb, nrm, depth, W, H, P, u->x0);
    if ((e = u->forward(st, false)) != cudaSuccess) return e;
    (void)y_out_raw;
    return cudaGetLastError();
}

const float* gkrt_unet_output(const Unet* u) { return u->y; }
bool gkrt_unet_has_forward(const Unet* u) { return u->B > 0; }
uint32_t* gkrt_unet_error_word(const Unet* u) { return u->err; }
