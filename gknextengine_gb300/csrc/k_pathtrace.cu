// k_pathtrace.cu — the "rt pass" (Core.PathTracing) and ray-query kernels for sm_103a.
#include "gk_shade.cuh"
#include "gkrt_internal.h"

namespace gk {

constexpr int kPtBlockX = 16, kPtBlockY = 8, kPtThreads = kPtBlockX * kPtBlockY;

// Warp-aggregated flush: one atomic per counter per warp. Slots 0-4 are per pass
// (rays, FP64 fallbacks, exact re-traces, node visits, triangle tests); slot 5 counts rays
// since the context was created.
__device__ __forceinline__ void flush_counters(const Counters& c, unsigned long long* out) {
    unsigned long long v[5] = {c.rays, c.fallbacks, c.retraces, c.nodes, c.tris};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 5; ++k) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], o);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 5; ++k)
            if (v[k]) atomicAdd(&out[k], v[k]);
        if (v[0]) atomicAdd(&out[5], v[0]);
    }
}

__global__ void __launch_bounds__(kPtThreads) k_trace_pass(ShadeScene sc, GkrtFrameConstants fc, int W, int H,
                                                           PixelImages im, unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kPtThreads];
    const int tid = threadIdx.x;
    const int x = blockIdx.x * kPtBlockX + (tid % kPtBlockX);
    const int y = blockIdx.y * kPtBlockY + (tid / kPtBlockX);
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0;
    if (x < W && y < H) shade_pixel(sc, fc, W, H, x, y, im, stack + tid, kPtThreads, cn);
    flush_counters(cn, counters);
}

constexpr int kRqThreads = 128;

__global__ void __launch_bounds__(kRqThreads) k_trace_rays(SceneView S, const GkrtRay* rays, GkrtHit* hits,
                                                           uint32_t n, uint32_t mode,
                                                           unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kRqThreads];
    const uint32_t i = blockIdx.x * kRqThreads + threadIdx.x;
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0;
    if (i < n) {
        GkrtRay r = rays[i];
        f3 o = F3(r.origin[0], r.origin[1], r.origin[2]), d = F3(r.dir[0], r.dir[1], r.dir[2]);
        GkrtHit h;
        h.t = -1.0f; h.b1 = 0.0f; h.b2 = 0.0f; h.inst = 0xFFFFFFFFu; h.prim = 0xFFFFFFFFu;
        h.pad[0] = h.pad[1] = h.pad[2] = 0u;
        cn.rays = 1;
        if (mode == GKRT_TRACE_ANY) {
            TraceOut t = traverse<kAny>(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kRqThreads, cn);
            if (t.hit) {
                HitShade s = hit_shade(S, o, d, t.inst, t.tri);
                h.t = s.t; h.inst = t.inst; h.prim = t.prim;
            }
        } else {
            TraceOut t = trace_closest(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kRqThreads, cn);
            if (t.hit) {
                HitShade s = hit_shade(S, o, d, t.inst, t.tri);
                h.t = s.t; h.b1 = s.b1; h.b2 = s.b2; h.inst = t.inst; h.prim = t.prim;
            }
        }
        hits[i] = h;
    }
    flush_counters(cn, counters);
}

}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_trace_pass(const ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H,
                                   const PixelImages& im, unsigned long long* counters, cudaStream_t st) {
    dim3 grid((W + kPtBlockX - 1) / kPtBlockX, (H + kPtBlockY - 1) / kPtBlockY);
    k_trace_pass<<<grid, kPtThreads, 0, st>>>(sc, fc, W, H, im, counters);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_trace_rays(const SceneView& S, const GkrtRay* rays, GkrtHit* hits, uint32_t n,
                                   uint32_t mode, unsigned long long* counters, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_trace_rays<<<(n + kRqThreads - 1) / kRqThreads, kRqThreads, 0, st>>>(S, rays, hits, n, mode, counters);
    return cudaGetLastError();
}
