// k_noalloc.cu — ray queries for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc when they issue work: an engine whose device memory is
// owned by its own pool allocator (every allocation must come from that pool), or a process
// that is close to its memory budget and must not grow. gkrt_trace_rays_noalloc serves them. It answers the same ray queries as gkrt_trace_rays,
// on the context's scene and BVH, into the caller's ray and hit buffers, and allocates
// nothing. Its scratch memory (per-block partial sums of the query statistics) is a
// file-scope __device__ array of fixed size: 32768 blocks x 8 counters x 8 bytes = 2 MiB,
// which every GPU that loads the library holds until the process exits. The size caps one
// call at 32768 blocks of 128 rays = 4,194,304 rays; larger counts are rejected.
//
// All calls share the one array. Every block writes all 8 of its slots on each call, so
// nothing has to be cleared first, and the last call's values stay in it. Two calls that
// overlap on the GPU (issued on different streams without ordering) race on the array; issue
// them on one stream or order them with events.
//
// Set-up: the first call on a device, with that device current, looks up the array's device
// address (cudaGetSymbolAddress) and keeps it for the process; make that first call before any
// stream capture. A cudaDeviceReset ends every context of this library and this address with
// them: do not use the library across a device reset.
#include <mutex>

#include "gk_shade.cuh"
#include "gkrt_internal.h"

namespace gk {
namespace {

constexpr uint32_t kNaThreads = 128;
constexpr uint32_t kNaMaxBlocks = 32768;
constexpr uint32_t kNaSlots = 8;   // rays, fp64 fallbacks, resolved pairs, nodes, triangles, hits, 2 unused
constexpr uint32_t kNaMaxRays = kNaMaxBlocks * kNaThreads;

}  // namespace
}  // namespace gk

// The scratch array (2 MiB per device, see the top of this file).
static __device__ __align__(256) unsigned long long g_noalloc_scratch[gk::kNaMaxBlocks * gk::kNaSlots];

namespace gk {
namespace {

__global__ void __launch_bounds__(kNaThreads) k_trace_rays_noalloc(SceneView S, const GkrtRay* rays, GkrtHit* hits,
                                                                   uint32_t n, uint32_t mode,
                                                                   unsigned long long* partials) {
    __shared__ uint32_t stack[kStackSize * kNaThreads];
    __shared__ unsigned long long red[kNaThreads / 32][6];
    const uint32_t i = blockIdx.x * kNaThreads + threadIdx.x;
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    if (i < n) {
        const GkrtRay r = rays[i];
        const f3 o = F3(r.origin[0], r.origin[1], r.origin[2]), d = F3(r.dir[0], r.dir[1], r.dir[2]);
        GkrtHit h;
        h.t = -1.0f; h.b1 = 0.0f; h.b2 = 0.0f; h.inst = 0xFFFFFFFFu; h.prim = 0xFFFFFFFFu;
        h.pad[0] = h.pad[1] = h.pad[2] = 0u;
        cn.rays = 1;
        const TraceOut t = mode == GKRT_TRACE_ANY
                               ? traverse<kAny, true>(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kNaThreads, cn)
                               : traverse<kClosest, true>(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kNaThreads, cn);
        if (t.hit) {
            ++cn.hits;
            const HitShade s = hit_shade(S, o, d, t.inst, t.tri);
            h.t = s.t; h.inst = t.inst; h.prim = t.prim;
            if (mode != GKRT_TRACE_ANY) { h.b1 = s.b1; h.b2 = s.b2; }
        }
        hits[i] = h;
    }
    unsigned long long v[6] = {cn.rays, cn.fallbacks, cn.retraces, cn.nodes, cn.tris, cn.hits};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) red[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x < kNaSlots) {
        unsigned long long s = 0;
        if (threadIdx.x < 6)
            for (uint32_t w = 0; w < kNaThreads / 32; ++w) s += red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * kNaSlots + threadIdx.x] = s;   // every slot of the block, every call
    }
}

// Sums the per-block partials into the context's statistics (slots 0-5 overwritten,
// slot 6 accumulates rays since creation).
__global__ void __launch_bounds__(256) k_noalloc_reduce(const unsigned long long* partials, uint32_t blocks,
                                                         unsigned long long* counters) {
    __shared__ unsigned long long red[256 / 32][6];
    unsigned long long v[6] = {0, 0, 0, 0, 0, 0};
    for (uint32_t b = threadIdx.x; b < blocks; b += 256)
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] += partials[(size_t)b * kNaSlots + k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], o);
    if ((threadIdx.x & 31) == 0)
#pragma unroll
        for (int k = 0; k < 6; ++k) red[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 6) {
        unsigned long long s = 0;
        for (int w = 0; w < 256 / 32; ++w) s += red[w][threadIdx.x];
        counters[threadIdx.x] = s;
        if (threadIdx.x == 0) counters[6] += s;
    }
}

// Device address of the scratch array, looked up once per device (with that device
// current) and cached; the host-side name of a __device__ variable is not a device address.
// The cache holds until process exit (a device reset invalidates it, as it does every context).
constexpr int kMaxDevices = 64;
std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

cudaError_t scratch_address(int device, void** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = p;
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace
}  // namespace gk

using namespace gk;

extern "C" int gkrt_trace_rays_noalloc(GkrtContext* ctx, const GkrtRay* rays, GkrtHit* hits, uint32_t count,
                                       uint32_t mode, void* stream) {
    if (!ctx) return GKRT_ERR_INVALID_ARG;
    if (count && (!rays || !hits))
        return gkrt_internal_fail(ctx, GKRT_ERR_INVALID_ARG, "null ray or hit buffer");
    if (mode > GKRT_TRACE_ANY) return gkrt_internal_fail(ctx, GKRT_ERR_INVALID_ARG, "unknown trace mode");
    if (count > kNaMaxRays)
        return gkrt_internal_fail(ctx, GKRT_ERR_INVALID_ARG,
                                  "gkrt_trace_rays_noalloc: count exceeds the static scratch limit of 4194304 rays "
                                  "per call; split the batch");
    SceneView S;
    unsigned long long* counters = nullptr;
    int device = 0;
    int rc = gkrt_internal_ready_view(ctx, &S, &counters, &device);
    if (rc != GKRT_OK) return rc;
    DeviceGuard device_guard(device);
    cudaError_t e = device_guard.status;
    void* scratch = nullptr;
    if (e == cudaSuccess) e = scratch_address(device, &scratch);
    if (e != cudaSuccess)
        return gkrt_internal_fail(ctx, GKRT_ERR_CUDA,
                                  std::string("gkrt_trace_rays_noalloc: scratch address: ") + cudaGetErrorString(e));
    const uint32_t blocks = (count + kNaThreads - 1) / kNaThreads;
    cudaStream_t st = (cudaStream_t)stream;
    if (blocks)
        k_trace_rays_noalloc<<<blocks, kNaThreads, 0, st>>>(S, rays, hits, count, mode,
                                                             (unsigned long long*)scratch);
    // an empty batch still resets the per-call statistics (zero blocks sum to zero), as
    // gkrt_trace_rays does
    k_noalloc_reduce<<<1, 256, 0, st>>>((const unsigned long long*)scratch, blocks, counters);
    e = cudaGetLastError();
    if (e != cudaSuccess)
        return gkrt_internal_fail(ctx, GKRT_ERR_CUDA, std::string("gkrt_trace_rays_noalloc: ") + cudaGetErrorString(e));
    return GKRT_OK;
}
