// k_output.cu — the output stage: the rendered image (RT_DENOISED, tone mapped) into the
// presentation image, which here is a headless device buffer of 8-bit BGRA pixels standing in
// for the reference's B8G8R8A8_UNORM swapchain image.
//
// * resolve: the resolve pass of VulkanBaseRenderer::Render (VulkanBaseRenderer.cpp:1036-1068),
//   a vkCmdBlitImage of the render extent onto the output rectangle with VK_FILTER_LINEAR;
// * FSR compose: Process.UpScaleFSR.comp.slang, the EASU upscale (:23-248) and its main
//   (:264-299), dispatched by the split-view compose (VulkanBaseRenderer.cpp:958-986);
// * screenshot: ScreenShot::SaveSwapChainToFileFast (ScreenShot.cpp:18-79), a crop of the
//   presentation image read back as 8-bit RGB.
//
// Stores convert as a UNORM attachment does: clamp to [0, 1] (NaN to 0), scale by 255, round to
// nearest even. All three passes are gathers from an L2-resident source with one 4-byte store per
// output pixel; they are bound by the stores' HBM bandwidth at any useful size.
#include <algorithm>

#include "gk_device.cuh"
#include "gkrt_internal.h"

namespace gk {
namespace {

struct Src {
    const float4* p;
    int W, H, P;   // width, height, pitch in pixels
};

__device__ __forceinline__ float4 texel(const Src& s, int x, int y) { return __ldg(&s.p[(size_t)y * s.P + x]); }

__device__ __forceinline__ uint32_t unorm8(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);   // fmaxf(NaN, 0) = 0
    return __float2uint_rn(v * 255.0f);
}
__device__ __forceinline__ uint32_t pack_bgra(float4 c) {
    return unorm8(c.z) | (unorm8(c.y) << 8) | (unorm8(c.x) << 16) | (unorm8(c.w) << 24);
}

// ---------------------------------------------------------------------------------------------
// resolve: linear-filtered blit. Destination texel centre x + 0.5 maps to source coordinate
// u = (x - ox + 0.5) * W / ow; the filter reads texels floor(u - 0.5) and the next one with
// weights 1 - a and a, a = frac(u - 0.5), indices clamped to the edge (the blit rules of the
// Vulkan specification, "Copying Data Between Images" with scaling).

__global__ void k_resolve_blit(Src s, uint32_t* out, int OW, int x0, int y0, int nx, int ny, int ox, int oy,
                               float su, float sv) {
    const int tx = blockIdx.x * blockDim.x + threadIdx.x, ty = blockIdx.y * blockDim.y + threadIdx.y;
    if (tx >= nx || ty >= ny) return;
    const int x = x0 + tx, y = y0 + ty;
    const float u = ((float)(x - ox) + 0.5f) * su - 0.5f;
    const float v = ((float)(y - oy) + 0.5f) * sv - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float a = u - fu, b = v - fv;
    const int i0 = (int)fu, j0 = (int)fv;
    const int ia = min(max(i0, 0), s.W - 1), ib = min(max(i0 + 1, 0), s.W - 1);
    const int ja = min(max(j0, 0), s.H - 1), jb = min(max(j0 + 1, 0), s.H - 1);
    const float4 t00 = texel(s, ia, ja), t10 = texel(s, ib, ja), t01 = texel(s, ia, jb), t11 = texel(s, ib, jb);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    float4 c;
    c.x = ((t00.x * w00 + t10.x * w10) + t01.x * w01) + t11.x * w11;
    c.y = ((t00.y * w00 + t10.y * w10) + t01.y * w01) + t11.y * w11;
    c.z = ((t00.z * w00 + t10.z * w10) + t01.z * w01) + t11.z * w11;
    c.w = ((t00.w * w00 + t10.w * w10) + t01.w * w01) + t11.w * w11;
    out[(size_t)y * OW + x] = pack_bgra(c);
}

// ---------------------------------------------------------------------------------------------
// FSR EASU (Process.UpScaleFSR.comp.slang). Expression order follows the shader; rsqrt is a
// correctly rounded 1 / sqrt.

struct F2 { float x, y; };

// FsrEasuCF (:23-29): the texel under normalized position p, clamped to the image.
__device__ __forceinline__ float4 easu_cf(const Src& s, float px, float py) {
    int cx = (int)(px * (float)s.W), cy = (int)(py * (float)s.H);
    cx = min(max(cx, 0), s.W - 1);
    cy = min(max(cy, 0), s.H - 1);
    return texel(s, cx, cy);
}
__device__ __forceinline__ float easu_luma(float4 c) { return c.y + 0.5f * (c.x + c.z); }
__device__ __forceinline__ float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }

// FsrEasuSetF (:105-132)
__device__ __forceinline__ void easu_set(F2& dir, float& len, float w, float lA, float lB, float lC, float lD,
                                         float lE) {
    float lenX = fmaxf(fabsf(lD - lC), fabsf(lC - lB));
    const float dirX = lD - lB;
    dir.x += dirX * w;
    lenX = clamp01(fabsf(dirX) / lenX);
    lenX *= lenX;
    len += lenX * w;
    float lenY = fmaxf(fabsf(lE - lC), fabsf(lC - lA));
    const float dirY = lE - lA;
    dir.y += dirY * w;
    lenY = clamp01(fabsf(dirY) / lenY);
    lenY *= lenY;
    len += lenY * w;
}

// FsrEasuTapF (:74-101)
__device__ __forceinline__ void easu_tap(float4& aC, float& aW, float offx, float offy, F2 dir, F2 len, float lob,
                                         float clp, float4 c) {
    F2 v;
    v.x = offx * dir.x + offy * dir.y;
    v.y = offx * (-dir.y) + offy * dir.x;
    v.x *= len.x;
    v.y *= len.y;
    const float d2 = fminf(v.x * v.x + v.y * v.y, clp);
    float wB = 0.4f * d2 - 1.0f;
    float wA = lob * d2 - 1.0f;
    wB *= wB;
    wA *= wA;
    wB = 1.5625f * wB - 0.5625f;
    const float w = wB * wA;
    aC.x += c.x * w;
    aC.y += c.y * w;
    aC.z += c.z * w;
    aC.w += c.w * w;
    aW += w;
}

__device__ __forceinline__ float4 min4f(float4 a, float4 b) {
    return make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), fminf(a.w, b.w));
}
__device__ __forceinline__ float4 max4f(float4 a, float4 b) {
    return make_float4(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z), fmaxf(a.w, b.w));
}

// FsrEasuCon (:32-72) with the viewport and the input both W x H, output OW x OH; then FsrEasuF
// (:135-248) at output position (ipx, ipy).
__device__ float4 easu(const Src& s, float OWf, float OHf, float ipx, float ipy) {
    const float Wf = (float)s.W, Hf = (float)s.H;
    const float c0x = Wf / OWf, c0y = Hf / OHf, c0z = 0.5f * Wf / OWf - 0.5f, c0w = 0.5f * Hf / OHf - 0.5f;
    const float c1x = 1.0f / Wf, c1y = 1.0f / Hf, c1z = 1.0f / Wf, c1w = -1.0f / Hf;
    const float c2x = -1.0f / Wf, c2y = 2.0f / Hf, c2z = 1.0f / Wf, c2w = 2.0f / Hf;
    const float c3x = 0.0f / Wf, c3y = 4.0f / Hf;
    F2 pp = {ipx * c0x + c0z, ipy * c0y + c0w};
    const F2 fp = {floorf(pp.x), floorf(pp.y)};
    pp.x -= fp.x;
    pp.y -= fp.y;
    const F2 p0 = {fp.x * c1x + c1z, fp.y * c1y + c1w};
    const F2 p1 = {p0.x + c2x, p0.y + c2y}, p2 = {p0.x + c2z, p0.y + c2w}, p3 = {p0.x + c3x, p0.y + c3y};
    const float ox = -0.5f * c1x, oy = 0.5f * c1x, oz = -0.5f * c1y, ow = 0.5f * c1y;
    const float4 bC = easu_cf(s, p0.x + ox, p0.y + ow), cC = easu_cf(s, p0.x + oy, p0.y + ow);
    const float4 iC = easu_cf(s, p1.x + ox, p1.y + ow), jC = easu_cf(s, p1.x + oy, p1.y + ow);
    const float4 fC = easu_cf(s, p1.x + oy, p1.y + oz), eC = easu_cf(s, p1.x + ox, p1.y + oz);
    const float4 kC = easu_cf(s, p2.x + ox, p2.y + ow), lC = easu_cf(s, p2.x + oy, p2.y + ow);
    const float4 hC = easu_cf(s, p2.x + oy, p2.y + oz), gC = easu_cf(s, p2.x + ox, p2.y + oz);
    const float4 oC = easu_cf(s, p3.x + oy, p3.y + oz), nC = easu_cf(s, p3.x + ox, p3.y + oz);
    const float bL = easu_luma(bC), cL = easu_luma(cC), iL = easu_luma(iC), jL = easu_luma(jC);
    const float fL = easu_luma(fC), eL = easu_luma(eC), kL = easu_luma(kC), lL = easu_luma(lC);
    const float hL = easu_luma(hC), gL = easu_luma(gC), oL = easu_luma(oC), nL = easu_luma(nC);
    F2 dir = {0.0f, 0.0f};
    float len = 0.0f;
    easu_set(dir, len, (1.0f - pp.x) * (1.0f - pp.y), bL, eL, fL, gL, jL);
    easu_set(dir, len, pp.x * (1.0f - pp.y), cL, fL, gL, hL, kL);
    easu_set(dir, len, (1.0f - pp.x) * pp.y, fL, iL, jL, kL, nL);
    easu_set(dir, len, pp.x * pp.y, gL, jL, kL, lL, oL);
    const F2 dir2 = {dir.x * dir.x, dir.y * dir.y};
    float dirR = dir2.x + dir2.y;
    const bool zro = dirR < (1.0f / 32768.0f);
    dirR = 1.0f / sqrtf(dirR);
    dirR = zro ? 1.0f : dirR;
    dir.x = zro ? 1.0f : dir.x;
    dir.x *= dirR;
    dir.y *= dirR;
    len = len * 0.5f;
    len *= len;
    const float stretch = (dir.x * dir.x + dir.y * dir.y) / fmaxf(fabsf(dir.x), fabsf(dir.y));
    const F2 len2 = {1.0f + (stretch - 1.0f) * len, 1.0f - 0.5f * len};
    const float lob = 0.5f - 0.29f * len;
    const float clp = 1.0f / lob;
    const float4 mn = min4f(min4f(fC, gC), min4f(jC, kC));
    const float4 mx = max4f(max4f(fC, gC), max4f(jC, kC));
    float4 aC = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    float aW = 0.0f;
    easu_tap(aC, aW, 0.0f - pp.x, -1.0f - pp.y, dir, len2, lob, clp, bC);
    easu_tap(aC, aW, 1.0f - pp.x, -1.0f - pp.y, dir, len2, lob, clp, cC);
    easu_tap(aC, aW, -1.0f - pp.x, 1.0f - pp.y, dir, len2, lob, clp, iC);
    easu_tap(aC, aW, 0.0f - pp.x, 1.0f - pp.y, dir, len2, lob, clp, jC);
    easu_tap(aC, aW, 0.0f - pp.x, 0.0f - pp.y, dir, len2, lob, clp, fC);
    easu_tap(aC, aW, -1.0f - pp.x, 0.0f - pp.y, dir, len2, lob, clp, eC);
    easu_tap(aC, aW, 1.0f - pp.x, 1.0f - pp.y, dir, len2, lob, clp, kC);
    easu_tap(aC, aW, 2.0f - pp.x, 1.0f - pp.y, dir, len2, lob, clp, lC);
    easu_tap(aC, aW, 2.0f - pp.x, 0.0f - pp.y, dir, len2, lob, clp, hC);
    easu_tap(aC, aW, 1.0f - pp.x, 0.0f - pp.y, dir, len2, lob, clp, gC);
    easu_tap(aC, aW, 1.0f - pp.x, 2.0f - pp.y, dir, len2, lob, clp, oC);
    easu_tap(aC, aW, 0.0f - pp.x, 2.0f - pp.y, dir, len2, lob, clp, nC);
    const float4 q = make_float4(aC.x / aW, aC.y / aW, aC.z / aW, aC.w / aW);
    return min4f(mx, max4f(mn, q));
}

// main (:264-299) for the pixels [0, gw) x [0, gh) of the dispatch (output_w / 8 by output_h / 8
// groups of 8 x 8), written at ipos + offset when inside the OW x OH presentation image.
__global__ void k_upscale_fsr(Src s, uint32_t* out, int OW, int OH, int gw, int gh, int offx, int offy, int outw,
                              int outh) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= gw || y >= gh) return;
    float4 c;
    if (OW != s.W || OH != s.H) {
        const float uvx = (float)x / (float)outw, uvy = (float)y / (float)outh;
        c = easu(s, (float)OW, (float)OH, uvx * (float)OW, uvy * (float)OH);
    } else {
        int sx = (int)((float)x * (float)OW / (float)outw), sy = (int)((float)y * (float)OH / (float)outh);
        sx = min(max(sx, 0), s.W - 1);
        sy = min(max(sy, 0), s.H - 1);
        c = texel(s, sx, sy);
    }
    const long long dx = (long long)x + offx, dy = (long long)y + offy;
    if (dx < 0 || dy < 0 || dx >= OW || dy >= OH) return;
    out[(size_t)dy * OW + (size_t)dx] = pack_bgra(c);
}

// ---------------------------------------------------------------------------------------------
// screenshot: bytes R, G, B of each pixel of the crop (bits 16, 8, 0 of the BGRA word)

__global__ void k_screenshot(const uint32_t* img, int OW, int x0, int y0, int w, int h, uint8_t* rgb) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const uint32_t p = __ldg(&img[(size_t)(y0 + y) * OW + (x0 + x)]);
    uint8_t* d = rgb + 3 * ((size_t)y * w + x);
    d[0] = (uint8_t)((p >> 16) & 0xFFu);
    d[1] = (uint8_t)((p >> 8) & 0xFFu);
    d[2] = (uint8_t)(p & 0xFFu);
}

}  // namespace
}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_output_resolve(const float4* src, int W, int H, int P, uint32_t* out, int OW, int OH, int ox,
                                       int oy, int ow, int oh, cudaStream_t st) {
    const long long x0 = std::max<long long>(ox, 0), y0 = std::max<long long>(oy, 0);
    const long long x1 = std::min<long long>((long long)ox + ow, OW), y1 = std::min<long long>((long long)oy + oh, OH);
    if (x1 <= x0 || y1 <= y0) return cudaSuccess;
    const int nx = (int)(x1 - x0), ny = (int)(y1 - y0);
    const dim3 b(32, 8), g((nx + 31) / 32, (ny + 7) / 8);
    k_resolve_blit<<<g, b, 0, st>>>(Src{src, W, H, P}, out, OW, (int)x0, (int)y0, nx, ny, ox, oy,
                                    (float)W / (float)ow, (float)H / (float)oh);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_output_fsr(const float4* src, int W, int H, int P, uint32_t* out, int OW, int OH, int offx,
                                   int offy, int outw, int outh, cudaStream_t st) {
    const int gw = (outw / 8) * 8, gh = (outh / 8) * 8;
    if (gw == 0 || gh == 0) return cudaSuccess;
    const dim3 b(32, 8), g((gw + 31) / 32, (gh + 7) / 8);
    k_upscale_fsr<<<g, b, 0, st>>>(Src{src, W, H, P}, out, OW, OH, gw, gh, offx, offy, outw, outh);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_screenshot(const uint32_t* img, int OW, int x0, int y0, int w, int h, uint8_t* rgb,
                                   cudaStream_t st) {
    if (w <= 0 || h <= 0) return cudaSuccess;
    const dim3 b(32, 8), g((w + 31) / 32, (h + 7) / 8);
    k_screenshot<<<g, b, 0, st>>>(img, OW, x0, y0, w, h, rgb);
    return cudaGetLastError();
}
