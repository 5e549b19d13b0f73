// bvh_gpu.cu — binned-SAH BVH construction on the GPU (sm_103a).
//
// Replaces the Vulkan acceleration-structure builds of the reference
// (RayTraceBaseRenderer::CreateBottomLevelStructures / CreateTopLevelStructures,
// src/Rendering/RayTraceBaseRenderer.cpp:276-386, and the per-frame TLAS rebuild of
// AfterUpdateScene / TLAS Update, :165-218) with the split rule of the host builder
// (binned SAH, 16 bins per axis, median split when all centroids share a bin).
//
// Top-down and breadth first. Every range of more than kSmall primitives is a "big task";
// one level of big tasks is processed per round:
//   bounds    per work item (<= 1024 primitives of one task): box and centroid bounds,
//             reduced in the block and merged with ordered-integer atomics;
//   bin       per work item: 3 x 16 bins in shared memory, merged into the task's bins;
//   split     one thread per task: SAH over the 3 x 15 bin boundaries; the task writes its
//             box and node ref into its parent's node (a node's fields are written by its
//             two children, so no node is written twice);
//   partition left counts, exclusive scan over work items, stable scatter, copy back;
//   emit      children with more than kSmall primitives become the next round's big tasks
//             (with their work items); the others become small tasks with a reserved run of
//             m - 1 node slots (the most a subtree of m primitives can use).
// For the mesh level the host reads back one group of counts per round; the instance level
// runs the same steps in one cooperative launch (k_inst_level, below). Small tasks are finished
// at the end by one thread each (one warp each at the instance level), sequentially and with
// the host builder's leaf rule (SAH leaf test for up to max_leaf triangles). Node indices are deterministic; reserved slots that a small
// subtree does not use stay zero and are never referenced.
// Node layout and leaf encoding are those of gk_trace.cuh.
#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "gk_trace.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kBins = 16;
constexpr uint32_t kChunk = 1024;
constexpr int kBt = 256;
constexpr uint32_t kSmall = 32;
constexpr int kSmallStack = 40;
constexpr int kBinWords = 3 * kBins * 7;   // per task: 3 axes x 16 bins x (6 ordered bounds + count)
constexpr int kScanB = 1024;
constexpr float kFar = 1e30f;
constexpr uint32_t kBuildErrStack = 1u;     // small-task stack full
constexpr uint32_t kBuildErrRange = 2u;     // a write would leave its task's range or reservation

struct BigTask {
    int node;       // relative node index of this task
    int parent;     // relative node index of the parent, or -1 - root for a root task
    int side;
    int depth;
    uint32_t begin, end;
};

struct SmallTask {
    int parent, side, depth;
    int root_node;  // relative node index for a root task, -1 otherwise
    uint32_t begin, end;
    uint32_t res0;  // first reserved node slot
    uint32_t pad;
};

struct Split {
    int axis, bin;  // axis -1: split by position
    uint32_t nleft;
    float clo, scale;
};

struct MeshRange {
    uint32_t tri_base, index_offset, vertex_offset, pad;
};

struct Geo {
    const float* box;   // 6 per primitive: lo xyz, hi xyz
    const float* cent;  // 3 per primitive
};

__host__ __device__ inline int f2o(float f) {   // order-preserving float -> int
    int i;
    memcpy(&i, &f, 4);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__host__ __device__ inline float o2f(int i) {
    const int j = i >= 0 ? i : i ^ 0x7FFFFFFF;
    float f;
    memcpy(&f, &j, 4);
    return f;
}

__device__ __forceinline__ float area6(const float* b) {
    const float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
    if (!(dx >= 0.0f && dy >= 0.0f && dz >= 0.0f)) return 0.0f;
    return 2.0f * (dx * dy + dy * dz + dz * dx);
}

__device__ __forceinline__ int bin_of(float c, float clo, float scale) {
    const int b = (int)((c - clo) * scale);
    return min(max(b, 0), kBins - 1);
}

// Child `side` of node `parent` gets box (widened as node boxes are stored) and ref; a root's
// box goes to root_box instead, unwidened.
__device__ void write_child(BvhNode* nodes, float* root_box, int parent, int side, const float* box, int ref) {
    if (parent < 0) {
        float* rb = root_box + 6 * (-1 - parent);
        for (int j = 0; j < 6; ++j) rb[j] = box[j];
        return;
    }
    float* f = reinterpret_cast<float*>(nodes + parent);
    for (int j = 0; j < 3; ++j) {
        f[6 * side + j] = widen_lo(box[j]);
        f[6 * side + 3 + j] = widen_hi(box[3 + j]);
    }
    reinterpret_cast<int*>(nodes + parent)[12 + side] = ref;
}

// ---------------------------------------------------------------------------------------------
// primitive boxes

__device__ __forceinline__ uint32_t find_range(const MeshRange* mr, uint32_t nmr, uint32_t t) {
    uint32_t lo = 0, hi = nmr;   // last range whose tri_base <= t
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (mr[mid].tri_base <= t) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void k_tri_boxes(const float4* pos, const uint32_t* ind, const MeshRange* mr, uint32_t nmr, uint32_t ntri,
                            float* box, float* cent) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntri) return;
    const MeshRange m = mr[find_range(mr, nmr, t)];
    const uint32_t lt = t - m.tri_base;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = 0; v < 3; ++v) {
        const float4 p = pos[ind[m.index_offset + 3u * lt + v] + m.vertex_offset];
        const float c[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; ++k) { lo[k] = fminf(lo[k], c[k]); hi[k] = fmaxf(hi[k], c[k]); }
    }
    for (int k = 0; k < 3; ++k) {
        box[6 * (size_t)t + k] = lo[k];
        box[6 * (size_t)t + 3 + k] = hi[k];
        cent[3 * (size_t)t + k] = 0.5f * (lo[k] + hi[k]);
    }
}

// Triangles in leaf order, 3 float4 each; the first vertex's w holds the mesh-local index.
__global__ void k_gather_tris(const float4* pos, const uint32_t* ind, const MeshRange* mr, uint32_t nmr,
                              const uint32_t* order, uint32_t ntri, float4* tris) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= ntri) return;
    const uint32_t p = order[k];
    const MeshRange m = mr[find_range(mr, nmr, p)];
    const uint32_t lt = p - m.tri_base;
    for (int v = 0; v < 3; ++v) {
        const float4 q = pos[ind[m.index_offset + 3u * lt + v] + m.vertex_offset];
        tris[3 * (size_t)k + v] = make_float4(q.x, q.y, q.z, v == 0 ? __uint_as_float(lt) : 0.0f);
    }
}

// World boxes of instances: the mesh box's 8 corners through the 3x4 world matrix in FP64,
// widened because the mesh level traverses the FP32 object-space ray.
// World box of an instance: the mesh root box's corners through its transform in FP64, padded
// as the mesh level traverses the FP32-transformed ray, whose points sit within rounding of the
// world ray's. Shared by the instance-level build and its refit.
__device__ void inst_box(const GpuInstBox& I, const float* mesh_box, float* out) {
    const float* rb = mesh_box + 6 * (size_t)I.mesh;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int c = 0; c < 8; ++c) {
        const double p[3] = {(c & 1) ? rb[3] : rb[0], (c & 2) ? rb[4] : rb[1], (c & 4) ? rb[5] : rb[2]};
        for (int r = 0; r < 3; ++r) {
            const double v = (double)I.world[4 * r] * p[0] + (double)I.world[4 * r + 1] * p[1] +
                             (double)I.world[4 * r + 2] * p[2] + (double)I.world[4 * r + 3];
            lo[r] = fmin(lo[r], v);
            hi[r] = fmax(hi[r], v);
        }
    }
    for (int r = 0; r < 3; ++r) {
        const double pad = 1e-5 * (fabs(lo[r]) + fabs(hi[r]) + (hi[r] - lo[r])) + 1e-7;
        out[r] = (float)(lo[r] - pad);
        out[3 + r] = (float)(hi[r] + pad);
    }
}

__global__ void k_inst_boxes(const GpuInstBox* in, uint32_t n, const float* mesh_box, float* box, float* cent) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float b[6];
    inst_box(in[i], mesh_box, b);
    for (int r = 0; r < 3; ++r) {
        box[6 * (size_t)i + r] = b[r];
        box[6 * (size_t)i + 3 + r] = b[3 + r];
        cent[3 * (size_t)i + r] = 0.5f * (b[r] + b[3 + r]);
    }
}

// ---------------------------------------------------------------------------------------------
// one round of big tasks

__global__ void k_init_idx(uint32_t* idx, uint32_t n) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) idx[t] = t;
}

// Each device function below does one kernel's work for one item (a work item, a task, ...):
// the per-round kernels call them once per block or thread, the instance-level build of
// k_inst_level loops over them inside one cooperative launch.

__device__ void clear_bins(int* bins, int* tb, uint32_t ntask, uint32_t first, uint32_t stride) {
    const uint32_t nb = ntask * (uint32_t)kBinWords, nt = ntask * 12u;
    const int pinf = f2o(INFINITY), ninf = f2o(-INFINITY);
    for (uint32_t i = first; i < nb + nt; i += stride) {
        if (i < nb) {
            const uint32_t q = i % 7u;
            bins[i] = q == 6u ? 0 : (q < 3u ? pinf : ninf);
        } else {
            const uint32_t j = (i - nb) % 6u;
            tb[i - nb] = j < 3u ? pinf : ninf;
        }
    }
}
__global__ void k_clear(int* bins, int* tb, uint32_t ntask) {
    clear_bins(bins, tb, ntask, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// (block of kBt threads) box and centroid bounds of work item w, merged into its task's
__device__ void bounds_item(const Geo& g, const uint32_t* idx, const uint32_t* wtask, const uint32_t* wbeg,
                            const uint32_t* wend, int* tb, uint32_t w) {
    __shared__ int s[12];
    if (threadIdx.x < 12) s[threadIdx.x] = (threadIdx.x % 6) < 3 ? f2o(INFINITY) : f2o(-INFINITY);
    __syncthreads();
    float v[12];
    for (int k = 0; k < 3; ++k) {
        v[k] = INFINITY; v[3 + k] = -INFINITY; v[6 + k] = INFINITY; v[9 + k] = -INFINITY;
    }
    for (uint32_t i = wbeg[w] + threadIdx.x; i < wend[w]; i += kBt) {
        const uint32_t p = idx[i];
        for (int k = 0; k < 3; ++k) {
            v[k] = fminf(v[k], g.box[6 * (size_t)p + k]);
            v[3 + k] = fmaxf(v[3 + k], g.box[6 * (size_t)p + 3 + k]);
            const float c = g.cent[3 * (size_t)p + k];
            v[6 + k] = fminf(v[6 + k], c);
            v[9 + k] = fmaxf(v[9 + k], c);
        }
    }
    for (int k = 0; k < 12; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            const float u = __shfl_xor_sync(0xFFFFFFFFu, v[k], o);
            v[k] = (k % 6) < 3 ? fminf(v[k], u) : fmaxf(v[k], u);
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 12; ++k) {
            if ((k % 6) < 3) atomicMin(&s[k], f2o(v[k]));
            else atomicMax(&s[k], f2o(v[k]));
        }
    __syncthreads();
    if (threadIdx.x < 12) {
        int* d = &tb[12 * (size_t)wtask[w] + threadIdx.x];
        if ((threadIdx.x % 6) < 3) atomicMin(d, s[threadIdx.x]);
        else atomicMax(d, s[threadIdx.x]);
    }
}
__global__ void __launch_bounds__(kBt) k_bounds(Geo g, const uint32_t* idx, const uint32_t* wtask,
                                                const uint32_t* wbeg, const uint32_t* wend, int* tb) {
    bounds_item(g, idx, wtask, wbeg, wend, tb, blockIdx.x);
}

__device__ __forceinline__ void axis_scale(const int* tbt, int k, float* clo, float* scale) {
    *clo = o2f(tbt[6 + k]);
    const float ext = o2f(tbt[9 + k]) - *clo;
    *scale = ext > 0.0f ? (float)kBins / ext : 0.0f;
}

// (block of kBt threads) the 3 x 16 bins of work item w, merged into its task's
__device__ void bin_item(const Geo& g, const uint32_t* idx, const int* tb, const uint32_t* wtask,
                         const uint32_t* wbeg, const uint32_t* wend, int* bins, uint32_t w) {
    __shared__ int sb[kBinWords];
    const uint32_t t = wtask[w];
    const int pinf = f2o(INFINITY), ninf = f2o(-INFINITY);
    for (int i = threadIdx.x; i < kBinWords; i += kBt) {
        const int q = i % 7;
        sb[i] = q == 6 ? 0 : (q < 3 ? pinf : ninf);
    }
    __syncthreads();
    float clo[3], scale[3];
    for (int k = 0; k < 3; ++k) axis_scale(tb + 12 * (size_t)t, k, &clo[k], &scale[k]);
    for (uint32_t i = wbeg[w] + threadIdx.x; i < wend[w]; i += kBt) {
        const uint32_t p = idx[i];
        int b6[6];
        for (int j = 0; j < 6; ++j) b6[j] = f2o(g.box[6 * (size_t)p + j]);
        for (int k = 0; k < 3; ++k) {
            int* s = &sb[(k * kBins + bin_of(g.cent[3 * (size_t)p + k], clo[k], scale[k])) * 7];
            for (int j = 0; j < 3; ++j) {
                atomicMin(&s[j], b6[j]);
                atomicMax(&s[3 + j], b6[3 + j]);
            }
            atomicAdd(&s[6], 1);
        }
    }
    __syncthreads();
    int* gb = bins + (size_t)t * kBinWords;
    for (int i = threadIdx.x; i < kBinWords; i += kBt) {
        const int q = i % 7;
        if (sb[i - q + 6] == 0) continue;   // empty bin: nothing to merge
        if (q == 6) atomicAdd(&gb[i], sb[i]);
        else if (q < 3) atomicMin(&gb[i], sb[i]);
        else atomicMax(&gb[i], sb[i]);
    }
}
__global__ void __launch_bounds__(kBt) k_bin(Geo g, const uint32_t* idx, const int* tb, const uint32_t* wtask,
                                             const uint32_t* wbeg, const uint32_t* wend, int* bins) {
    bin_item(g, idx, tb, wtask, wbeg, wend, bins, blockIdx.x);
}

// SAH over one axis's bins (the host builder's sweep): best cost, boundary and left count.
__device__ void sah_axis(const float (*bb)[6], const uint32_t* bc, int axis, float* best, int* best_axis,
                         int* best_bin, uint32_t* best_left) {
    float ra[kBins];
    uint32_t rc[kBins];
    float acc[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    uint32_t cnt = 0;
    for (int i = kBins - 1; i > 0; --i) {
        for (int j = 0; j < 3; ++j) { acc[j] = fminf(acc[j], bb[i][j]); acc[3 + j] = fmaxf(acc[3 + j], bb[i][3 + j]); }
        cnt += bc[i];
        ra[i] = area6(acc);
        rc[i] = cnt;
    }
    for (int j = 0; j < 3; ++j) { acc[j] = INFINITY; acc[3 + j] = -INFINITY; }
    cnt = 0;
    for (int i = 0; i < kBins - 1; ++i) {
        for (int j = 0; j < 3; ++j) { acc[j] = fminf(acc[j], bb[i][j]); acc[3 + j] = fmaxf(acc[3 + j], bb[i][3 + j]); }
        cnt += bc[i];
        if (cnt == 0 || rc[i + 1] == 0) continue;
        const float cost = area6(acc) * (float)cnt + ra[i + 1] * (float)rc[i + 1];
        if (cost < *best) { *best = cost; *best_axis = axis; *best_bin = i + 1; *best_left = cnt; }
    }
}

// task t: writes its box into its parent and picks the SAH split
__device__ void split_task(const BigTask* tasks, uint32_t t, const int* bins, const int* tb, Split* split,
                           BvhNode* nodes, float* root_box, uint32_t node_base) {
    const BigTask T = tasks[t];
    const int* tbt = tb + 12 * (size_t)t;
    float box[6];
    for (int j = 0; j < 6; ++j) box[j] = o2f(tbt[j]);
    write_child(nodes, root_box, T.parent, T.side, box, (int)node_base + T.node);
    const int* b = bins + (size_t)t * kBinWords;
    Split s;
    s.axis = -1; s.bin = 0; s.nleft = (T.end - T.begin) / 2u; s.clo = 0.0f; s.scale = 0.0f;
    float best = INFINITY;
    float clo[3], scale[3];
    for (int k = 0; k < 3; ++k) {
        axis_scale(tbt, k, &clo[k], &scale[k]);
        if (!(scale[k] > 0.0f)) continue;
        float bb[kBins][6];
        uint32_t bc[kBins];
        for (int i = 0; i < kBins; ++i) {
            const int* q = &b[(k * kBins + i) * 7];
            for (int j = 0; j < 6; ++j) bb[i][j] = o2f(q[j]);
            bc[i] = (uint32_t)q[6];
        }
        sah_axis(bb, bc, k, &best, &s.axis, &s.bin, &s.nleft);
    }
    if (s.axis >= 0) { s.clo = clo[s.axis]; s.scale = scale[s.axis]; }
    split[t] = s;
}
__global__ void k_split(const BigTask* tasks, uint32_t ntask, const int* bins, const int* tb, Split* split,
                        BvhNode* nodes, float* root_box, uint32_t node_base) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntask) split_task(tasks, t, bins, tb, split, nodes, root_box, node_base);
}

__device__ __forceinline__ bool goes_left(const Geo& g, uint32_t p, uint32_t pos, const Split& s, uint32_t begin) {
    if (s.axis < 0) return pos - begin < s.nleft;
    return bin_of(g.cent[3 * (size_t)p + s.axis], s.clo, s.scale) < s.bin;
}

// (block of kBt threads) how many primitives of work item w go left
__device__ void count_left_item(const Geo& g, const uint32_t* idx, const Split* split, const BigTask* tasks,
                                const uint32_t* wtask, const uint32_t* wbeg, const uint32_t* wend, uint32_t* wleft,
                                uint32_t w) {
    __shared__ uint32_t red[kBt / 32];
    const uint32_t t = wtask[w];
    const Split s = split[t];
    const uint32_t begin = tasks[t].begin;
    uint32_t c = 0;
    for (uint32_t i = wbeg[w] + threadIdx.x; i < wend[w]; i += kBt) c += goes_left(g, idx[i], i, s, begin) ? 1u : 0u;
    for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t tot = 0;
        for (int i = 0; i < kBt / 32; ++i) tot += red[i];
        wleft[w] = tot;
    }
}
__global__ void __launch_bounds__(kBt) k_count_left(Geo g, const uint32_t* idx, const Split* split,
                                                    const BigTask* tasks, const uint32_t* wtask, const uint32_t* wbeg,
                                                    const uint32_t* wend, uint32_t* wleft) {
    count_left_item(g, idx, split, tasks, wtask, wbeg, wend, wleft, blockIdx.x);
}

// Stable scatter into tmp: left side first. wleft_scan: exclusive scan of left counts over
// work items; a task's work items are consecutive, the first being task_w0[t].
__device__ void scatter_item(const Geo& g, const uint32_t* idx, uint32_t* tmp, const Split* split,
                             const BigTask* tasks, const uint32_t* wtask, const uint32_t* wbeg, const uint32_t* wend,
                             const uint32_t* wleft_scan, const uint32_t* task_w0, uint32_t* info, uint32_t w) {
    __shared__ uint32_t wsum[kBt / 32];
    const uint32_t t = wtask[w];
    const BigTask T = tasks[t];
    const Split s = split[t];
    const uint32_t left_before = wleft_scan[w] - wleft_scan[task_w0[t]];
    const uint32_t right_before = (wbeg[w] - T.begin) - left_before;
    const uint32_t lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const unsigned below = (1u << lane) - 1u;
    uint32_t lrun = 0, rrun = 0;
    for (uint32_t base = wbeg[w]; base < wend[w]; base += kBt) {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < wend[w];
        uint32_t p = 0;
        bool left = false;
        if (valid) {
            p = idx[i];
            left = goes_left(g, p, i, s, T.begin);
        }
        const unsigned ml = __ballot_sync(0xFFFFFFFFu, valid && left);
        const unsigned mr = __ballot_sync(0xFFFFFFFFu, valid && !left);
        if (lane == 0) wsum[wid] = (uint32_t)__popc(ml) | ((uint32_t)__popc(mr) << 16);
        __syncthreads();
        uint32_t lw = 0, rw = 0, lt = 0, rt = 0;
        for (uint32_t j = 0; j < kBt / 32; ++j) {
            const uint32_t v = wsum[j];
            if (j < wid) { lw += v & 0xFFFFu; rw += v >> 16; }
            lt += v & 0xFFFFu;
            rt += v >> 16;
        }
        if (valid) {
            const uint32_t dst = left ? T.begin + left_before + lrun + lw + (uint32_t)__popc(ml & below)
                                      : T.begin + s.nleft + right_before + rrun + rw + (uint32_t)__popc(mr & below);
            if (dst >= T.begin && dst < T.end) tmp[dst] = p;
            else atomicOr(&info[2], kBuildErrRange);
        }
        lrun += lt;
        rrun += rt;
        __syncthreads();
    }
}
__global__ void __launch_bounds__(kBt) k_scatter(Geo g, const uint32_t* idx, uint32_t* tmp, const Split* split,
                                                 const BigTask* tasks, const uint32_t* wtask, const uint32_t* wbeg,
                                                 const uint32_t* wend, const uint32_t* wleft_scan,
                                                 const uint32_t* task_w0, uint32_t* info) {
    scatter_item(g, idx, tmp, split, tasks, wtask, wbeg, wend, wleft_scan, task_w0, info, blockIdx.x);
}

__device__ void copy_back_item(const uint32_t* tmp, uint32_t* idx, const uint32_t* wbeg, const uint32_t* wend,
                               uint32_t w) {
    for (uint32_t i = wbeg[w] + threadIdx.x; i < wend[w]; i += kBt) idx[i] = tmp[i];
}
__global__ void __launch_bounds__(kBt) k_copy_back(const uint32_t* tmp, uint32_t* idx, const uint32_t* wbeg,
                                                   const uint32_t* wend) {
    copy_back_item(tmp, idx, wbeg, wend, blockIdx.x);
}

// Per task: (big children, their work items, small children, node slots they reserve).
__device__ void child_counts_task(const BigTask* tasks, uint32_t t, const Split* split, uint4* cc) {
    const BigTask T = tasks[t];
    const uint32_t m[2] = {split[t].nleft, (T.end - T.begin) - split[t].nleft};
    uint4 c = make_uint4(0u, 0u, 0u, 0u);
    for (int k = 0; k < 2; ++k) {
        if (m[k] > kSmall) { c.x += 1u; c.y += (m[k] + kChunk - 1u) / kChunk; }
        else { c.z += 1u; c.w += m[k] - 1u; }
    }
    cc[t] = c;
}
__global__ void k_child_counts(const BigTask* tasks, uint32_t ntask, const Split* split, uint4* cc) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntask) child_counts_task(tasks, t, split, cc);
}

__device__ void emit_task(const BigTask* tasks, uint32_t t, const Split* split, const uint4* off, uint32_t node0,
                          uint32_t res0, uint32_t small0, BigTask* next, uint32_t* nwtask, uint32_t* nwbeg,
                          uint32_t* nwend, uint32_t* next_w0, SmallTask* small) {
    const BigTask T = tasks[t];
    uint4 o = off[t];
    const uint32_t mid = T.begin + split[t].nleft;
    for (int c = 0; c < 2; ++c) {
        const uint32_t b = c ? mid : T.begin, e = c ? T.end : mid, m = e - b;
        if (m > kSmall) {
            const uint32_t j = o.x++;
            BigTask nt;
            nt.node = (int)(node0 + j);
            nt.parent = T.node;
            nt.side = c;
            nt.depth = T.depth + 1;
            nt.begin = b;
            nt.end = e;
            next[j] = nt;
            next_w0[j] = o.y;
            for (uint32_t cb = b; cb < e; cb += kChunk) {
                const uint32_t w = o.y++;
                nwtask[w] = j;
                nwbeg[w] = cb;
                nwend[w] = min(cb + kChunk, e);
            }
        } else {
            SmallTask st;
            st.parent = T.node;
            st.side = c;
            st.depth = T.depth + 1;
            st.root_node = -1;
            st.begin = b;
            st.end = e;
            st.res0 = res0 + o.w;
            st.pad = 0;
            small[small0 + o.z++] = st;
            o.w += m - 1u;
        }
    }
}
__global__ void k_emit(const BigTask* tasks, uint32_t ntask, const Split* split, const uint4* off, uint32_t node0,
                       uint32_t res0, uint32_t small0, BigTask* next, uint32_t* nwtask, uint32_t* nwbeg,
                       uint32_t* nwend, uint32_t* next_w0, SmallTask* small) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < ntask)
        emit_task(tasks, t, split, off, node0, res0, small0, next, nwtask, nwbeg, nwend, next_w0, small);
}

// One thread per small task: the rest of the subtree, depth first, with the host builder's
// rules (triangle ranges of up to 2 are leaves, up to max_leaf when the SAH prefers a leaf;
// instance leaves hold one instance). info[0] += nodes used, info[1] = max depth, info[2]
// error bits.
__device__ void small_task(const Geo& g, uint32_t* idx, const SmallTask* st, uint32_t i, BvhNode* nodes,
                           float* root_box, uint32_t max_leaf, int inst_leaf, const uint32_t* prim_map,
                           uint32_t node_base, uint32_t* info) {
    const SmallTask S = st[i];
    struct Item {
        uint32_t b, e;
        int parent, side, depth;
    };
    Item stk[kSmallStack];
    int sp = 0;
    stk[sp++] = Item{S.begin, S.end, S.parent, S.side, S.depth};
    uint32_t res = S.res0, used = 0;
    int maxd = 0;
    bool first = true;
    while (sp > 0) {
        const Item it = stk[--sp];
        const uint32_t n = it.e - it.b;
        float box[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t q = it.b; q < it.e; ++q) {
            const uint32_t p = idx[q];
            for (int k = 0; k < 3; ++k) {
                box[k] = fminf(box[k], g.box[6 * (size_t)p + k]);
                box[3 + k] = fmaxf(box[3 + k], g.box[6 * (size_t)p + 3 + k]);
                const float c = g.cent[3 * (size_t)p + k];
                clo[k] = fminf(clo[k], c);
                chi[k] = fmaxf(chi[k], c);
            }
        }
        maxd = max(maxd, it.depth);
        bool leaf = inst_leaf ? n == 1u : n <= 2u;
        int best_axis = -1, best_bin = 0;
        uint32_t best_left = 0;
        float best = INFINITY, bclo = 0.0f, bscale = 0.0f;
        if (!leaf) {
            for (int k = 0; k < 3; ++k) {
                const float ext = chi[k] - clo[k];
                if (!(ext > 0.0f)) continue;
                const float scale = (float)kBins / ext;
                float bb[kBins][6];
                uint32_t bc[kBins];
                for (int j = 0; j < kBins; ++j) {
                    bc[j] = 0;
                    for (int c = 0; c < 3; ++c) { bb[j][c] = INFINITY; bb[j][3 + c] = -INFINITY; }
                }
                for (uint32_t q = it.b; q < it.e; ++q) {
                    const uint32_t p = idx[q];
                    const int bi = bin_of(g.cent[3 * (size_t)p + k], clo[k], scale);
                    bc[bi]++;
                    for (int c = 0; c < 3; ++c) {
                        bb[bi][c] = fminf(bb[bi][c], g.box[6 * (size_t)p + c]);
                        bb[bi][3 + c] = fmaxf(bb[bi][3 + c], g.box[6 * (size_t)p + 3 + c]);
                    }
                }
                const int prev_axis = best_axis;
                sah_axis(bb, bc, k, &best, &best_axis, &best_bin, &best_left);
                if (best_axis != prev_axis) { bclo = clo[k]; bscale = scale; }
            }
            const float area = area6(box);
            if (!inst_leaf && n <= max_leaf && (best_axis < 0 || area * (float)n <= best + 1.0f * area)) leaf = true;
        }
        if (leaf) {
            const uint32_t payload = inst_leaf ? (prim_map[idx[it.b]] << 3) : ((it.b << 3) | (n - 1u));
            const int ref = (int)(~payload);
            if (it.parent >= 0) {
                write_child(nodes, root_box, it.parent, it.side, box, ref);
            } else {
                // a root that is a single leaf: interior root whose second child never intersects
                write_child(nodes, root_box, it.parent, it.side, box, 0);
                BvhNode nd;
                nd.a = make_float4(widen_lo(box[0]), widen_lo(box[1]), widen_lo(box[2]), widen_hi(box[3]));
                nd.b = make_float4(widen_hi(box[4]), widen_hi(box[5]), kFar, kFar);
                nd.c = make_float4(kFar, kFar, kFar, kFar);
                nd.d = make_int4(ref, kRefPop, 0, 0);
                nodes[S.root_node] = nd;
                ++used;
            }
            first = false;
            continue;
        }
        if (!(first && S.root_node >= 0) && res >= S.res0 + (S.end - S.begin - 1u)) {
            atomicOr(&info[2], kBuildErrRange);
            break;
        }
        const int me = (first && S.root_node >= 0) ? S.root_node : (int)(res++);
        first = false;
        ++used;
        write_child(nodes, root_box, it.parent, it.side, box, (int)node_base + me);
        uint32_t mid;
        if (best_axis < 0) {
            mid = it.b + n / 2u;
        } else {
            uint32_t lo = it.b, hi = it.e;   // in-place partition: bins below best_bin first
            while (lo < hi) {
                const uint32_t p = idx[lo];
                if (bin_of(g.cent[3 * (size_t)p + best_axis], bclo, bscale) < best_bin) {
                    ++lo;
                } else {
                    --hi;
                    idx[lo] = idx[hi];
                    idx[hi] = p;
                }
            }
            mid = lo;
            if (mid == it.b || mid == it.e) mid = it.b + n / 2u;
        }
        if (sp + 2 > kSmallStack) {
            atomicOr(&info[2], kBuildErrStack);
            break;
        }
        stk[sp++] = Item{mid, it.e, me, 1, it.depth + 1};
        stk[sp++] = Item{it.b, mid, me, 0, it.depth + 1};
    }
    atomicAdd(&info[0], used);
    atomicMax(&info[1], (uint32_t)maxd);
}
__global__ void k_small(Geo g, uint32_t* idx, const SmallTask* st, uint32_t ns, BvhNode* nodes, float* root_box,
                        uint32_t max_leaf, int inst_leaf, const uint32_t* prim_map, uint32_t node_base,
                        uint32_t* info) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ns) small_task(g, idx, st, i, nodes, root_box, max_leaf, inst_leaf, prim_map, node_base, info);
}

// ---------------------------------------------------------------------------------------------
// collapse into compressed 8-wide nodes (WideNode, gk_trace.cuh)
//
// Top-down and breadth first over the two-child trees: a wide node starts from the children
// of one binary interior node and repeatedly replaces its interior child of largest surface
// area by that child's two children, up to 8 (Ylitie, Karras, Laine, HPG 2017, collapse by
// greedy expansion). Its interior children become the next level's wide nodes; indices come
// from an exclusive scan of the per-node interior counts, so the layout is deterministic.

struct WEnt {
    int ref;
    int slot;   // 2 * binary node + side: where the box and ref come from
    float b[6];
};

// Children of binary node `node`: the first replaces e[at], the second is appended at e[n].
// Returns false for a node without children (not produced by the builders). With links, each
// child's slot is recorded as its parent (interior child) or its instance's leaf (leaf child).
__device__ bool wide_children(const BvhNode* bin, int node, WEnt* e, int& n, int at, const RefitLinks* lk) {
    const float* f = reinterpret_cast<const float*>(bin + node);
    const int* r = reinterpret_cast<const int*>(bin + node) + 12;
    bool first = true;
    for (int side = 0; side < 2; ++side) {
        if (r[side] == kRefPop) continue;   // the empty half of a single-leaf root
        WEnt& d = first ? e[at] : e[n++];
        first = false;
        d.ref = r[side];
        d.slot = 2 * node + side;
        for (int j = 0; j < 6; ++j) d.b[j] = f[6 * side + j];
        if (lk) {
            if (d.ref >= 0) {
                const uint32_t k = (uint32_t)(d.ref - (int)lk->nbase);
                if (k < lk->ncap) lk->parent[k] = d.slot;
            } else {
                const uint32_t k = ~(uint32_t)d.ref >> 3;   // instance leaves hold one instance
                if (k < lk->ninst) lk->leaf[k] = d.slot;
            }
        }
    }
    return !first;
}

// Greedy expansion of binary node `root` into at most 8 children; -1 on a malformed tree.
__device__ int wide_expand(const BvhNode* bin, int root, WEnt* e, const RefitLinks* lk = nullptr) {
    int n = 1;
    if (!wide_children(bin, root, e, n, 0, lk)) return -1;
    while (n < 8) {
        int best = -1;
        float ba = -1.0f;
        for (int i = 0; i < n; ++i) {
            if (e[i].ref < 0) continue;
            const float a = area6(e[i].b);
            if (a > ba) { ba = a; best = i; }
        }
        if (best < 0) break;
        if (!wide_children(bin, e[best].ref, e, n, best, lk)) return -1;
    }
    return n;
}

// floor and ceil of the exact product x 2^-ex (rs = 2^-ex, -100 <= ex <= 38) in float: a
// product of magnitude >= 1 is a normal float and exact; below 1 only the sign of x matters
// (a product that underflowed to a subnormal or to zero keeps the answer exact).
__device__ __forceinline__ float floor_scaled(float x, float rs) {
    const float y = x * rs;
    if (fabsf(y) < 1.0f) return x < 0.0f ? -1.0f : 0.0f;
    return floorf(y);
}
__device__ __forceinline__ float ceil_scaled(float x, float rs) {
    const float y = x * rs;
    if (fabsf(y) < 1.0f) return x > 0.0f ? 1.0f : 0.0f;
    return ceilf(y);
}

// Per-axis scale 2^ex and origin k for the children's boxes, one step of margin on each side.
// Exact: x / 2^ex of a float is floored or ceiled exactly (floor_scaled), and every count
// below stays under 2^24, so the float arithmetic is that of exact integers. The exponent is
// capped at 38 so that 2^23 s |inv| stays finite for |inv| <= 1e20. Fails on non-finite or
// out-of-range boxes.
__device__ bool wide_axis(const WEnt* e, int n, int ax, float& origin, uint32_t& ebyte, uint32_t* qlo,
                          uint32_t* qhi) {
    float lo = INFINITY, hi = -INFINITY;
    for (int i = 0; i < n; ++i) {
        lo = fminf(lo, e[i].b[ax]);
        hi = fmaxf(hi, e[i].b[3 + ax]);
    }
    if (!(isfinite(lo) && isfinite(hi) && hi >= lo)) return false;
    int ex = -100;
    const double range = (double)hi - (double)lo;
    if (range > 0.0) ex = max(ex, ilogb(range / 253.0));
    if (lo != 0.0f) ex = max(ex, ilogb(fabs((double)lo)) - 21);
    for (; ex <= 38; ++ex) {
        const float s = __int_as_float((127 + ex) << 23), rs = __int_as_float((127 - ex) << 23);   // 2^ex, 2^-ex
        const float k = floor_scaled(lo, rs) - 1.0f;
        if (fabsf(k) >= 4194304.0f) continue;   // |k| < 2^22
        bool ok = true;
        for (int i = 0; i < n; ++i) ok = ok && (ceil_scaled(e[i].b[3 + ax], rs) + 1.0f - k <= 255.0f);
        if (!ok) continue;
        for (int i = 0; i < n; ++i) {
            qlo[i] = (uint32_t)(floor_scaled(e[i].b[ax], rs) - 1.0f - k);
            qhi[i] = (uint32_t)(ceil_scaled(e[i].b[3 + ax], rs) + 1.0f - k);
        }
        origin = k * s;
        ebyte = (uint32_t)(ex + 127);
        return true;
    }
    return false;
}

// items: x binary node, y wide index, z depth (1 at the roots)
__device__ void wide_count_item(const BvhNode* bin, const int4* items, uint32_t i, uint32_t* cnt) {
    WEnt e[8];
    const int m = wide_expand(bin, items[i].x, e);
    uint32_t c = 0;
    for (int j = 0; j < m; ++j) c += e[j].ref >= 0 ? 1u : 0u;
    cnt[i] = c;   // 0 for a malformed node: k_wide_emit reports it
}
__global__ void k_wide_count(const BvhNode* bin, const int4* items, uint32_t n, uint32_t* cnt) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wide_count_item(bin, items, i, cnt);
}

// links (optional, links.parent null for none): refit links of the trees being collapsed
// Wide node it.y from the m entries e: quantized boxes, refs (interior children become the
// next level's items at next_base + off_i + rank), and the refit's source slots with links.
__device__ void wide_write(const WEnt* e, int m, const int4& it, uint32_t off_i, uint32_t next_base, WideNode* out,
                           int4* next, uint32_t* err, const RefitLinks* lk) {
    if (lk) {
        const uint32_t w = (uint32_t)it.y - lk->wbase;
        if (w < lk->wcap)
            for (int j = 0; j < 8; ++j) lk->wsrc[8 * (size_t)w + j] = j < m ? e[j].slot : -1;
        else
            atomicOr(err, kBuildErrRange);
    }
    uint32_t qw[3][4] = {{0u, 0u, 0u, 0u}, {0u, 0u, 0u, 0u}, {0u, 0u, 0u, 0u}};
    float origin[3] = {0.0f, 0.0f, 0.0f};
    uint32_t meta = m > 0 ? ((1u << m) - 1u) << 24 : 0u;
    for (int ax = 0; ax < 3; ++ax) {
        uint32_t qlo[8], qhi[8], eb = 127u;
        if (m > 0 && !wide_axis(e, m, ax, origin[ax], eb, qlo, qhi)) {
            atomicOr(err, kBuildErrRange);   // the build fails; the node is written without slots
            meta = 0u;
            break;
        }
        meta |= eb << (8 * ax);
        for (int j = 0; j < m; ++j) {
            qw[ax][j >> 2] |= qlo[j] << (8 * (j & 3));
            qw[ax][2 + (j >> 2)] |= qhi[j] << (8 * (j & 3));
        }
    }
    int ref[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    uint32_t rank = 0;
    for (int j = 0; j < m; ++j) {   // interior children are still counted: the scan expects them
        if (e[j].ref >= 0) {
            const uint32_t wi = next_base + off_i + rank;
            next[off_i + rank] = make_int4(e[j].ref, (int)wi, it.z + 1, 0);
            ref[j] = (int)wi;
            ++rank;
        } else {
            ref[j] = e[j].ref;
        }
    }
    WideNode w;
    w.h = make_float4(origin[0], origin[1], origin[2], __uint_as_float(meta));
    for (int ax = 0; ax < 3; ++ax) w.q[ax] = make_uint4(qw[ax][0], qw[ax][1], qw[ax][2], qw[ax][3]);
    w.ref[0] = make_int4(ref[0], ref[1], ref[2], ref[3]);
    w.ref[1] = make_int4(ref[4], ref[5], ref[6], ref[7]);
    out[it.y] = w;
}
__device__ void wide_emit_item(const BvhNode* bin, const int4* items, uint32_t i, const uint32_t* off,
                               uint32_t next_base, WideNode* out, int4* next, uint32_t* err, const RefitLinks& links) {
    const int4 it = items[i];
    const RefitLinks* lk = links.parent ? &links : nullptr;
    WEnt e[8];
    int m = wide_expand(bin, it.x, e, lk);
    if (m < 0) {
        atomicOr(err, kBuildErrRange);
        m = 0;
    }
    wide_write(e, m, it, off[i], next_base, out, next, err, lk);
}
__global__ void k_wide_emit(const BvhNode* bin, const int4* items, uint32_t n, const uint32_t* off, uint32_t next_base,
                            WideNode* out, int4* next, uint32_t* err, RefitLinks links) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) wide_emit_item(bin, items, i, off, next_base, out, next, err, links);
}

// ---------------------------------------------------------------------------------------------
// refit of the instance level, topology kept
//
// One thread per instance climbs from its leaf: it writes its box into its slot (widened, as
// node boxes are stored; unwidened into ubox, 12 floats per node), and at a node with two
// children only the second arrival goes on, with the union of both children's boxes (Karras,
// HPG 2012, bottom-up boxes). The second arrival resets the node's counter for the next refit.
// Nothing waits: the first arrival stops. The union of exact boxes is exact, so every node
// gets the box a build of the same topology would give it.

__global__ void __launch_bounds__(128) k_refit_boxes(RefitLinks lk, const GpuInstBox* inst, const float* mesh_box,
                                                     BvhNode* nodes, float* ubox, uint32_t* arrive) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lk.ninst) return;
    int s = lk.leaf[i];
    if (s < 0) return;   // not in the tree (invisible, or an empty mesh)
    float b[6];
    inst_box(inst[i], mesh_box, b);
    for (int hop = 0; hop < 128; ++hop) {   // the builders stop at 64 levels
        const int node = s >> 1, side = s & 1;
        const uint32_t k = (uint32_t)(node - (int)lk.nbase);
        if (k >= lk.ncap) return;
        float* f = reinterpret_cast<float*>(nodes + node);
        float* u = ubox + 12 * (size_t)k;
        for (int j = 0; j < 3; ++j) {
            f[6 * side + j] = widen_lo(b[j]);
            f[6 * side + 3 + j] = widen_hi(b[3 + j]);
            u[6 * side + j] = b[j];
            u[6 * side + 3 + j] = b[3 + j];
        }
        const int* r = reinterpret_cast<const int*>(nodes + node) + 12;
        if (r[1] != kRefPop) {
            __threadfence();
            if (atomicAdd(&arrive[k], 1u) == 0u) return;   // the sibling's thread finishes the node
            __threadfence();
            arrive[k] = 0u;
            const float* o = u + 6 * (1 - side);
            for (int j = 0; j < 3; ++j) {
                b[j] = fminf(b[j], __ldcg(o + j));
                b[3 + j] = fmaxf(b[3 + j], __ldcg(o + 3 + j));
            }
        }
        s = lk.parent[k];
        if (s < 0) return;   // the root: its box sits in no slot
    }
}

// The wide nodes re-quantized from the refit slot boxes; their children, refs and slot masks
// stay as the collapse wrote them.
__global__ void __launch_bounds__(128) k_refit_wide(RefitLinks lk, const BvhNode* nodes, WideNode* wide, uint32_t nw,
                                                    uint32_t* err, uint32_t err_bit) {
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nw || j >= lk.wcap) return;
    WEnt e[8];
    int m = 0;
    for (int c = 0; c < 8; ++c) {
        const int s = lk.wsrc[8 * (size_t)j + c];
        if (s < 0) break;
        const float* f = reinterpret_cast<const float*>(nodes + (s >> 1)) + 6 * (s & 1);
        for (int q = 0; q < 6; ++q) e[m].b[q] = f[q];
        ++m;
    }
    uint32_t qw[3][4] = {{0u, 0u, 0u, 0u}, {0u, 0u, 0u, 0u}, {0u, 0u, 0u, 0u}};
    float origin[3] = {0.0f, 0.0f, 0.0f};
    uint32_t meta = m > 0 ? ((1u << m) - 1u) << 24 : 0u;
    for (int ax = 0; ax < 3; ++ax) {
        uint32_t qlo[8], qhi[8], eb = 127u;
        if (m > 0 && !wide_axis(e, m, ax, origin[ax], eb, qlo, qhi)) {
            atomicOr(err, err_bit);   // the node loses its slots; the error word reports it
            meta = 0u;
            break;
        }
        meta |= eb << (8 * ax);
        for (int c = 0; c < m; ++c) {
            qw[ax][c >> 2] |= qlo[c] << (8 * (c & 3));
            qw[ax][2 + (c >> 2)] |= qhi[c] << (8 * (c & 3));
        }
    }
    WideNode& w = wide[lk.wbase + j];
    w.h = make_float4(origin[0], origin[1], origin[2], __uint_as_float(meta));
    for (int ax = 0; ax < 3; ++ax) w.q[ax] = make_uint4(qw[ax][0], qw[ax][1], qw[ax][2], qw[ax][3]);
}

// ---------------------------------------------------------------------------------------------
// exclusive scans of uint32 / uint4: in-block inclusive scans, a scan of the block sums, a fix-up

__device__ __forceinline__ uint32_t add_(uint32_t a, uint32_t b) { return a + b; }
__device__ __forceinline__ uint4 add_(uint4 a, uint4 b) { return make_uint4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ uint32_t sub_(uint32_t a, uint32_t b) { return a - b; }
__device__ __forceinline__ uint4 sub_(uint4 a, uint4 b) { return make_uint4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
template <class T> __device__ __forceinline__ T zero_();
template <> __device__ __forceinline__ uint32_t zero_<uint32_t>() { return 0u; }
template <> __device__ __forceinline__ uint4 zero_<uint4>() { return make_uint4(0u, 0u, 0u, 0u); }

template <class T>
__device__ T block_scan_incl(T v, T* s) {   // inclusive scan over the kScanB threads
    s[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < kScanB; o <<= 1) {
        const T u = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : zero_<T>();
        __syncthreads();
        s[threadIdx.x] = add_(s[threadIdx.x], u);
        __syncthreads();
    }
    return s[threadIdx.x];
}

template <class T>
__global__ void __launch_bounds__(kScanB) k_scan_blocks(const T* in, uint32_t n, T* out, T* bsum) {
    __shared__ T s[kScanB];
    const uint32_t i = blockIdx.x * kScanB + threadIdx.x;
    const T incl = block_scan_incl(i < n ? in[i] : zero_<T>(), s);
    if (i < n) out[i] = incl;
    if (threadIdx.x == kScanB - 1) bsum[blockIdx.x] = incl;
}

template <class T>
__global__ void __launch_bounds__(kScanB) k_scan_sums(T* bsum, uint32_t nb, T* total) {
    __shared__ T s[kScanB];
    T carry = zero_<T>();
    for (uint32_t base = 0; base < nb; base += kScanB) {
        const uint32_t i = base + threadIdx.x;
        const T incl = block_scan_incl(i < nb ? bsum[i] : zero_<T>(), s);
        const T blk = s[kScanB - 1];
        if (i < nb) bsum[i] = add_(carry, incl);   // inclusive prefix of the block sums
        __syncthreads();
        carry = add_(carry, blk);
    }
    if (threadIdx.x == 0) *total = carry;
}

template <class T>
__global__ void __launch_bounds__(kScanB) k_scan_fix(const T* in, uint32_t n, T* out, const T* bsum_incl) {
    const uint32_t i = blockIdx.x * kScanB + threadIdx.x;
    if (i >= n) return;
    const T before = blockIdx.x ? bsum_incl[blockIdx.x - 1] : zero_<T>();
    out[i] = add_(sub_(out[i], in[i]), before);
}

// ---------------------------------------------------------------------------------------------
// the instance level in one cooperative launch
//
// The same rounds, small tasks and collapse levels as the per-round kernels (so the same
// trees), run by one persistent grid whose blocks are all resident (cooperative launch) and
// meet at grid_sync between the steps of a round. Counts that the host reads back between
// rounds elsewhere stay on the device: block 0 scans, every thread reads the totals after
// the next barrier and updates its own copy of the round state, so every thread takes the
// same branches. Buffers are sized from the instance count beforehand (a tree of n
// single-instance leaves has n - 1 interior nodes), so nothing grows during the build. The
// host waits once, for the result record.

constexpr long long kSyncCycles = 1ll << 31;   // ~1 s at 2 GHz: a barrier gives up after this
constexpr uint32_t kBuildErrSync = 4u;          // a barrier gave up
constexpr uint32_t kBuildErrCap = 8u;           // a count exceeded the buffers sized beforehand
constexpr uint32_t kBuildErrRounds = 16u;       // more than 64 rounds or collapse levels

// Grid-wide barrier of the cooperative launch: sync[0] arrivals, sync[1] generation, sync[2]
// error. Thread 0 of each block arrives; the last arrival resets the count and bumps the
// generation, the others wait for the bump with a bounded wait. Returns false (for the whole
// block) once any block gave up, so that every block leaves its loops.
__device__ bool grid_sync(uint32_t* sync) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile uint32_t* vs = sync;
        int good = vs[2] == 0u;
        if (good) {
            const uint32_t gen = vs[1];
            __threadfence();
            if (atomicAdd(&sync[0], 1u) == gridDim.x - 1u) {
                atomicExch(&sync[0], 0u);
                __threadfence();
                atomicAdd(&sync[1], 1u);
            } else {
                const long long t0 = clock64();
                while (vs[1] == gen) {
                    if (vs[2] != 0u) { good = 0; break; }
                    if (clock64() - t0 > kSyncCycles) { atomicOr(&sync[2], kBuildErrSync); good = 0; break; }
                    __nanosleep(64);
                }
            }
            __threadfence();
        }
        ok = good;
    }
    __syncthreads();
    return ok != 0;
}

// Exclusive scan of in[0, n) into out by one block of kBt threads; *total = the sum.
template <class T>
__device__ void block_scan_excl(const T* in, uint32_t n, T* out, T* total) {
    __shared__ T s[kBt];
    T carry = zero_<T>();
    for (uint32_t base = 0; base < n; base += kBt) {
        const uint32_t i = base + threadIdx.x;
        const T v = i < n ? __ldcg(in + i) : zero_<T>();
        s[threadIdx.x] = v;
        __syncthreads();
        for (int o = 1; o < kBt; o <<= 1) {
            const T u = threadIdx.x >= (unsigned)o ? s[threadIdx.x - o] : zero_<T>();
            __syncthreads();
            s[threadIdx.x] = add_(s[threadIdx.x], u);
            __syncthreads();
        }
        if (i < n) out[i] = add_(carry, sub_(s[threadIdx.x], v));
        carry = add_(carry, s[kBt - 1]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

// ---- warp-wide forms for the instance level (few tasks, each on a 32-lane warp) ----

struct WBox {
    float b[6];   // lo xyz, hi xyz
    uint32_t c;   // primitives
};
__device__ __forceinline__ WBox wbox_join(const WBox& x, const WBox& y) {
    WBox r;
    for (int j = 0; j < 3; ++j) { r.b[j] = fminf(x.b[j], y.b[j]); r.b[3 + j] = fmaxf(x.b[3 + j], y.b[3 + j]); }
    r.c = x.c + y.c;
    return r;
}
__device__ __forceinline__ WBox wbox_shfl_up(const WBox& x, int o) {
    WBox r;
    for (int j = 0; j < 6; ++j) r.b[j] = __shfl_up_sync(0xFFFFFFFFu, x.b[j], o, 16);
    r.c = __shfl_up_sync(0xFFFFFFFFu, x.c, o, 16);
    return r;
}
__device__ __forceinline__ WBox wbox_shfl_down(const WBox& x, int o) {
    WBox r;
    for (int j = 0; j < 6; ++j) r.b[j] = __shfl_down_sync(0xFFFFFFFFu, x.b[j], o, 16);
    r.c = __shfl_down_sync(0xFFFFFFFFu, x.c, o, 16);
    return r;
}

// sah_axis over two axes at once: lanes 0..15 hold the bins of axis `a0`, lanes 16..31 those
// of axis `a1` (bin = lane & 15; an axis < 0 takes no part). Each half computes the cost at
// its 15 bin boundaries from prefix and suffix unions; the warp keeps the candidate the
// serial sweep over the axes in order would keep: the smallest cost, then the smaller axis,
// then the first boundary, if that cost is below *best (NaN costs never win). Every lane
// returns the same answer.
__device__ void sah_pair_warp(const WBox& bin, int a0, int a1, float* best, int* best_axis, int* best_bin,
                              uint32_t* best_left) {
    const int lane = threadIdx.x & 31, l16 = lane & 15;
    const int axis = lane < 16 ? a0 : a1;
    WBox pre = bin, suf = bin;
    for (int o = 1; o < 16; o <<= 1) {
        const WBox u = wbox_shfl_up(pre, o), d = wbox_shfl_down(suf, o);
        if (l16 >= o) pre = wbox_join(pre, u);
        if (l16 + o < 16) suf = wbox_join(suf, d);
    }
    const WBox right = wbox_shfl_down(suf, 1);   // bins l16 + 1 .. 15 of the same half
    bool ok = axis >= 0 && l16 < kBins - 1 && pre.c != 0u && right.c != 0u;
    float cost = 0.0f;
    if (ok) cost = area6(pre.b) * (float)pre.c + area6(right.b) * (float)right.c;
    ok = ok && cost < *best;
    float bc = ok ? cost : INFINITY;
    int bk = ok ? (axis << 4) | l16 : 0x7FFFFFFF;   // (axis, boundary) order key
    int bl = lane;
    for (int o = 16; o > 0; o >>= 1) {
        const float oc = __shfl_xor_sync(0xFFFFFFFFu, bc, o);
        const int ok2 = __shfl_xor_sync(0xFFFFFFFFu, bk, o);
        const int ol = __shfl_xor_sync(0xFFFFFFFFu, bl, o);
        if (ok2 != 0x7FFFFFFF && (bk == 0x7FFFFFFF || oc < bc || (oc == bc && ok2 < bk))) { bc = oc; bk = ok2; bl = ol; }
    }
    const uint32_t left = __shfl_sync(0xFFFFFFFFu, pre.c, bl);
    if (bk != 0x7FFFFFFF) {
        *best = bc;
        *best_axis = bk >> 4;
        *best_bin = (bk & 15) + 1;
        *best_left = left;
    }
}

// The bins of axis k (lanes 0..15 or 16..31 of a warp) from the task's global bins.
__device__ __forceinline__ WBox load_bins(const int* b, int k, int l16) {
    WBox w;
    const int* q = &b[(k * kBins + l16) * 7];
    for (int j = 0; j < 6; ++j) w.b[j] = o2f(q[j]);
    w.c = (uint32_t)q[6];
    return w;
}
__device__ __forceinline__ WBox empty_wbox() {
    WBox w;
    for (int j = 0; j < 3; ++j) { w.b[j] = INFINITY; w.b[3 + j] = -INFINITY; }
    w.c = 0u;
    return w;
}

// split_task with one warp per task: the same split (axes 0 and 1 in one pass, then axis 2).
__device__ void split_task_warp(const BigTask* tasks, uint32_t t, const int* bins, const int* tb, Split* split,
                                BvhNode* nodes, float* root_box, uint32_t node_base) {
    const int lane = threadIdx.x & 31, l16 = lane & 15;
    const BigTask T = tasks[t];
    const int* tbt = tb + 12 * (size_t)t;
    if (lane == 0) {
        float box[6];
        for (int j = 0; j < 6; ++j) box[j] = o2f(tbt[j]);
        write_child(nodes, root_box, T.parent, T.side, box, (int)node_base + T.node);
    }
    const int* b = bins + (size_t)t * kBinWords;
    Split sp;
    sp.axis = -1; sp.bin = 0; sp.nleft = (T.end - T.begin) / 2u; sp.clo = 0.0f; sp.scale = 0.0f;
    float best = INFINITY;
    float clo[3], scale[3];
    int use[3];
    for (int k = 0; k < 3; ++k) {
        axis_scale(tbt, k, &clo[k], &scale[k]);
        use[k] = scale[k] > 0.0f ? k : -1;
    }
    {
        const int k = lane < 16 ? use[0] : use[1];
        sah_pair_warp(k >= 0 ? load_bins(b, k, l16) : empty_wbox(), use[0], use[1], &best, &sp.axis, &sp.bin,
                      &sp.nleft);
    }
    if (use[2] >= 0)
        sah_pair_warp(lane < 16 ? load_bins(b, 2, l16) : empty_wbox(), 2, -1, &best, &sp.axis, &sp.bin, &sp.nleft);
    if (sp.axis >= 0) { sp.clo = clo[sp.axis]; sp.scale = scale[sp.axis]; }
    if (lane == 0) split[t] = sp;
}

// small_task for instance leaves (one instance per leaf) with one warp per task. The task's
// instances (at most kSmall = 32: lane q holds the range's q-th) are staged once in the warp's
// shared memory with their boxes and centroids; per range: bounds by warp reductions, the bins
// of all three axes in shared memory, the same binned-SAH choice as the serial sweep, and a
// stable partition by ballots (the rounds' order) of the staged entries. The range stack is
// warp-uniform.
__device__ void small_task_warp(const Geo& g, uint32_t* idx, const SmallTask* st, uint32_t i, BvhNode* nodes,
                                float* root_box, const uint32_t* prim_map, uint32_t node_base, uint32_t* info) {
    constexpr int kW = kBt / 32;
    __shared__ int sbins[kW][3][kBins * 7];
    __shared__ float sbox[kW][9][32];   // lo xyz, hi xyz, centroid xyz of each staged entry
    __shared__ uint32_t sprim[kW][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const SmallTask S = st[i];
    const uint32_t m = S.end - S.begin;
    if (m > 32u) {   // not produced by the rounds (ranges of more than kSmall are big tasks)
        if (lane == 0) atomicOr(&info[2], kBuildErrRange);
        return;
    }
    if ((uint32_t)lane < m) {
        const uint32_t p = idx[S.begin + lane];
        sprim[wid][lane] = p;
        for (int k = 0; k < 6; ++k) sbox[wid][k][lane] = g.box[6 * (size_t)p + k];
        for (int k = 0; k < 3; ++k) sbox[wid][6 + k][lane] = g.cent[3 * (size_t)p + k];
    }
    __syncwarp();
    struct Item {
        uint32_t b, e;   // positions relative to S.begin
        int parent, side, depth;
    };
    Item stk[kSmallStack];
    int sp = 0;
    stk[sp++] = Item{0u, m, S.parent, S.side, S.depth};
    uint32_t res = S.res0, used = 0;
    int maxd = 0;
    bool first = true;
    const int pinf = f2o(INFINITY), ninf = f2o(-INFINITY);
    while (sp > 0) {
        const Item it = stk[--sp];
        const uint32_t n = it.e - it.b;
        const bool valid = (uint32_t)lane < n;
        const uint32_t pos = it.b + (valid ? (uint32_t)lane : 0u);
        const uint32_t p = sprim[wid][pos];
        float box[6], cen[3], clo[3], chi[3], ubox[6];
        for (int k = 0; k < 3; ++k) {
            box[k] = valid ? sbox[wid][k][pos] : INFINITY;
            box[3 + k] = valid ? sbox[wid][3 + k][pos] : -INFINITY;
            cen[k] = sbox[wid][6 + k][pos];
            clo[k] = valid ? cen[k] : INFINITY;
            chi[k] = valid ? cen[k] : -INFINITY;
        }
        for (int k = 0; k < 6; ++k) ubox[k] = box[k];
        for (int o = 16; o > 0; o >>= 1)
            for (int k = 0; k < 3; ++k) {
                ubox[k] = fminf(ubox[k], __shfl_xor_sync(0xFFFFFFFFu, ubox[k], o));
                ubox[3 + k] = fmaxf(ubox[3 + k], __shfl_xor_sync(0xFFFFFFFFu, ubox[3 + k], o));
                clo[k] = fminf(clo[k], __shfl_xor_sync(0xFFFFFFFFu, clo[k], o));
                chi[k] = fmaxf(chi[k], __shfl_xor_sync(0xFFFFFFFFu, chi[k], o));
            }
        maxd = max(maxd, it.depth);
        const bool leaf = n == 1u;
        int best_axis = -1, best_bin = 0;
        uint32_t best_left = 0;
        float best = INFINITY, scale[3];
        if (!leaf) {
            int use[3];
            for (int k = 0; k < 3; ++k) {
                const float ext = chi[k] - clo[k];
                use[k] = ext > 0.0f ? k : -1;
                scale[k] = ext > 0.0f ? (float)kBins / ext : 0.0f;
            }
            for (int j = lane; j < 3 * kBins * 7; j += 32) {
                const int q = j % 7;
                (&sbins[wid][0][0])[j] = q == 6 ? 0 : (q < 3 ? pinf : ninf);
            }
            __syncwarp();
            if (valid)
                for (int k = 0; k < 3; ++k) {
                    if (use[k] < 0) continue;
                    int* c = &sbins[wid][k][bin_of(cen[k], clo[k], scale[k]) * 7];
                    for (int j = 0; j < 3; ++j) {
                        atomicMin(&c[j], f2o(box[j]));
                        atomicMax(&c[3 + j], f2o(box[3 + j]));
                    }
                    atomicAdd(&c[6], 1);
                }
            __syncwarp();
            WBox w = empty_wbox();
            const int k01 = lane < 16 ? use[0] : use[1];
            if (k01 >= 0) {
                const int* q = &sbins[wid][k01][(lane & 15) * 7];
                for (int j = 0; j < 6; ++j) w.b[j] = o2f(q[j]);
                w.c = (uint32_t)q[6];
            }
            WBox w2 = empty_wbox();
            if (lane < 16 && use[2] >= 0) {
                const int* q = &sbins[wid][2][lane * 7];
                for (int j = 0; j < 6; ++j) w2.b[j] = o2f(q[j]);
                w2.c = (uint32_t)q[6];
            }
            __syncwarp();
            sah_pair_warp(w, use[0], use[1], &best, &best_axis, &best_bin, &best_left);
            if (use[2] >= 0) sah_pair_warp(w2, 2, -1, &best, &best_axis, &best_bin, &best_left);
        }
        if (leaf) {
            if (lane == 0) {
                const uint32_t payload = prim_map[p] << 3;
                const int ref = (int)(~payload);
                if (it.parent >= 0) {
                    write_child(nodes, root_box, it.parent, it.side, ubox, ref);
                } else {
                    // a root that is a single leaf: interior root whose second child never intersects
                    write_child(nodes, root_box, it.parent, it.side, ubox, 0);
                    BvhNode nd;
                    nd.a = make_float4(widen_lo(ubox[0]), widen_lo(ubox[1]), widen_lo(ubox[2]), widen_hi(ubox[3]));
                    nd.b = make_float4(widen_hi(ubox[4]), widen_hi(ubox[5]), kFar, kFar);
                    nd.c = make_float4(kFar, kFar, kFar, kFar);
                    nd.d = make_int4(ref, kRefPop, 0, 0);
                    nodes[S.root_node] = nd;
                }
            }
            if (it.parent < 0) ++used;
            first = false;
            continue;
        }
        if (!(first && S.root_node >= 0) && res >= S.res0 + (m - 1u)) {
            if (lane == 0) atomicOr(&info[2], kBuildErrRange);
            break;
        }
        const int me = (first && S.root_node >= 0) ? S.root_node : (int)(res++);
        first = false;
        ++used;
        if (lane == 0) write_child(nodes, root_box, it.parent, it.side, ubox, (int)node_base + me);
        uint32_t mid;
        if (best_axis < 0) {
            mid = it.b + n / 2u;
        } else {
            const bool left = valid && bin_of(cen[best_axis], clo[best_axis], scale[best_axis]) < best_bin;
            const unsigned ml = __ballot_sync(0xFFFFFFFFu, left), mv = __ballot_sync(0xFFFFFFFFu, valid);
            const unsigned below = (1u << lane) - 1u;
            const uint32_t nl = (uint32_t)__popc(ml);
            const uint32_t to = it.b + (left ? (uint32_t)__popc(ml & below) : nl + (uint32_t)__popc(mv & ~ml & below));
            __syncwarp();
            if (valid) {
                sprim[wid][to] = p;
                for (int k = 0; k < 3; ++k) {
                    sbox[wid][k][to] = box[k];
                    sbox[wid][3 + k][to] = box[3 + k];
                    sbox[wid][6 + k][to] = cen[k];
                }
            }
            __syncwarp();
            mid = it.b + nl;
            if (mid == it.b || mid == it.e) mid = it.b + n / 2u;
        }
        if (sp + 2 > kSmallStack) {
            if (lane == 0) atomicOr(&info[2], kBuildErrStack);
            break;
        }
        stk[sp++] = Item{mid, it.e, me, 1, it.depth + 1};
        stk[sp++] = Item{it.b, mid, me, 0, it.depth + 1};
    }
    if (lane == 0) {
        atomicAdd(&info[0], used);
        atomicMax(&info[1], (uint32_t)maxd);
    }
}

// The collapse of the instance level with the expansion cached: the count step expands a
// node (recording the refit links as it goes) and keeps its at most 8 entries, the emit step
// quantizes and writes them without walking the two-child nodes again.
__device__ void wide_count_cache_item(const BvhNode* bin, const int4* items, uint32_t i, uint32_t* cnt, WEnt* cache,
                                      int* cache_n, const RefitLinks& links) {
    const RefitLinks* lk = links.parent ? &links : nullptr;
    WEnt e[8];
    const int m = wide_expand(bin, items[i].x, e, lk);
    uint32_t c = 0;
    for (int j = 0; j < m; ++j) {
        c += e[j].ref >= 0 ? 1u : 0u;
        cache[8 * (size_t)i + j] = e[j];
    }
    cache_n[i] = m;
    cnt[i] = c;   // 0 for a malformed node (m < 0): the emit step reports it
}
__device__ void wide_emit_cached_item(const WEnt* cache, const int* cache_n, const int4* items, uint32_t i,
                                      const uint32_t* off, uint32_t next_base, WideNode* out, int4* next, uint32_t* err,
                                      const RefitLinks& links) {
    const int4 it = items[i];
    const RefitLinks* lk = links.parent ? &links : nullptr;
    WEnt e[8];
    int m = cache_n[i];
    if (m < 0 || m > 8) {
        atomicOr(err, kBuildErrRange);
        m = 0;
    }
    for (int j = 0; j < m; ++j) e[j] = cache[8 * (size_t)i + j];
    wide_write(e, m, it, off[i], next_base, out, next, err, lk);
}

struct InstLevelArgs {
    const GpuInstBox* inst;      // n instances of the tree (device)
    uint32_t n;
    const float* mesh_box;       // 6 per mesh
    float *box, *cent;           // 6 / 3 per instance
    uint32_t *idx, *tmp, *map;   // n each; map: instance index of each primitive
    BigTask* tasks[2];
    uint32_t *w0[2], *wtask[2], *wbeg[2], *wend[2];
    int *bins, *tb;
    Split* split;
    uint32_t *wleft, *wleft_scan;
    uint4 *cc, *cc_scan;
    SmallTask* small;
    uint32_t cap_t, cap_w, cap_s;   // task, work-item and small-task capacities
    BvhNode* nodes;              // the two-child slots, relative index (bin + node_base)
    const BvhNode* bin;          // the whole node array, for the collapse
    uint32_t node_base, node_cap;
    float* root_box;             // 6 floats
    uint32_t* info;              // [0] nodes used by small tasks, [1] their depth, [2] build errors, [3] collapse errors
    int4* witems[2];
    uint32_t *wcnt, *woff, item_cap;
    WEnt* wcache;                // 8 entries per collapse item of the level
    int* wcache_n;
    WideNode* wide;
    uint32_t wide_base, wide_cap;
    RefitLinks lk;
    uint32_t* sync;              // grid_sync state, 3 words, zero at launch
    uint4* tot4;
    uint32_t* tot32;
    uint32_t* result;            // node slots, nodes used, depth, wide nodes, wide levels, error bits
};

__global__ void __launch_bounds__(kBt) k_inst_level(InstLevelArgs a) {
    const uint32_t gtid = blockIdx.x * kBt + threadIdx.x, gthreads = gridDim.x * kBt;
    const uint32_t gwarp = gtid >> 5, gwarps = gthreads >> 5;
    const Geo g{a.box, a.cent};
    const uint32_t n = a.n;
    uint32_t err = 0;
    // instance boxes, the identity order and the root task
    for (uint32_t i = gtid; i < n; i += gthreads) {
        const GpuInstBox ib = a.inst[i];
        float b[6];
        inst_box(ib, a.mesh_box, b);
        for (int r = 0; r < 3; ++r) {
            a.box[6 * (size_t)i + r] = b[r];
            a.box[6 * (size_t)i + 3 + r] = b[3 + r];
            a.cent[3 * (size_t)i + r] = 0.5f * (b[r] + b[3 + r]);
        }
        a.idx[i] = i;
        a.map[i] = ib.inst;
    }
    uint32_t ntask = 0, nwork = 0, nsmall = 0, next_node = 0, nodes_used = 0, rounds = 0;
    int cur = 0;
    if (n > kSmall) {
        ntask = 1;
        nwork = (n + kChunk - 1) / kChunk;
        next_node = 1;
        if (gtid == 0) {
            a.tasks[0][0] = BigTask{0, -1, 0, 0, 0u, n};
            a.w0[0][0] = 0;
        }
        for (uint32_t k = gtid; k < nwork; k += gthreads) {
            a.wtask[0][k] = 0;
            a.wbeg[0][k] = k * kChunk;
            a.wend[0][k] = min((k + 1) * kChunk, n);
        }
        clear_bins(a.bins, a.tb, 1, gtid, gthreads);
    } else if (n > 0) {
        nsmall = 1;
        next_node = n;   // the root and its n - 1 reserved slots
        if (gtid == 0) a.small[0] = SmallTask{-1, 0, 0, 0, 0u, n, 1u, 0u};
    }
    if (gtid == 0)
        for (int k = 0; k < 3; ++k) { a.root_box[k] = INFINITY; a.root_box[3 + k] = -INFINITY; }
    bool live = grid_sync(a.sync);
    while (live && ntask > 0) {
        if (++rounds > 64) { err |= kBuildErrRounds; break; }
        for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
            bounds_item(g, a.idx, a.wtask[cur], a.wbeg[cur], a.wend[cur], a.tb, w);
            __syncthreads();
        }
        if (!(live = grid_sync(a.sync))) break;
        for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
            bin_item(g, a.idx, a.tb, a.wtask[cur], a.wbeg[cur], a.wend[cur], a.bins, w);
            __syncthreads();
        }
        if (!(live = grid_sync(a.sync))) break;
        for (uint32_t t = gwarp; t < ntask; t += gwarps)
            split_task_warp(a.tasks[cur], t, a.bins, a.tb, a.split, a.nodes, a.root_box, a.node_base);
        if (!(live = grid_sync(a.sync))) break;
        for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
            count_left_item(g, a.idx, a.split, a.tasks[cur], a.wtask[cur], a.wbeg[cur], a.wend[cur], a.wleft, w);
            __syncthreads();
        }
        for (uint32_t t = gtid; t < ntask; t += gthreads) child_counts_task(a.tasks[cur], t, a.split, a.cc);
        if (!(live = grid_sync(a.sync))) break;
        if (blockIdx.x == 0) block_scan_excl<uint32_t>(a.wleft, nwork, a.wleft_scan, a.tot32);
        if (blockIdx.x == (gridDim.x > 1u ? 1u : 0u)) block_scan_excl<uint4>(a.cc, ntask, a.cc_scan, a.tot4);
        if (!(live = grid_sync(a.sync))) break;
        const uint4 tot = __ldcg(a.tot4);
        const uint32_t nbig = tot.x, nwork_next = tot.y, nsm = tot.z, nres = tot.w;
        if (nbig > a.cap_t || nwork_next > a.cap_w || nsmall + nsm > a.cap_s ||
            (uint64_t)next_node + nbig + nres > a.node_cap) {
            err |= kBuildErrCap;
            break;
        }
        const uint32_t node0 = next_node, res0 = next_node + nbig;
        const int nx = cur ^ 1;
        for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) {
            scatter_item(g, a.idx, a.tmp, a.split, a.tasks[cur], a.wtask[cur], a.wbeg[cur], a.wend[cur],
                         a.wleft_scan, a.w0[cur], a.info, w);
            __syncthreads();
        }
        for (uint32_t t = gtid; t < ntask; t += gthreads)
            emit_task(a.tasks[cur], t, a.split, a.cc_scan, node0, res0, nsmall, a.tasks[nx], a.wtask[nx], a.wbeg[nx],
                      a.wend[nx], a.w0[nx], a.small);
        if (!(live = grid_sync(a.sync))) break;
        for (uint32_t w = blockIdx.x; w < nwork; w += gridDim.x) copy_back_item(a.tmp, a.idx, a.wbeg[cur], a.wend[cur], w);
        clear_bins(a.bins, a.tb, nbig, gtid, gthreads);
        nodes_used += ntask;
        nsmall += nsm;
        next_node += nbig + nres;
        ntask = nbig;
        nwork = nwork_next;
        cur = nx;
        live = grid_sync(a.sync);
    }
    if (live && err == 0u) {
        for (uint32_t i = gwarp; i < nsmall; i += gwarps)
            small_task_warp(g, a.idx, a.small, i, a.nodes, a.root_box, a.map, a.node_base, a.info);
        live = grid_sync(a.sync);
    }
    // the collapse of the one tree into wide nodes [wide_base, ...)
    uint32_t wn = 0, wnext = a.wide_base, levels = 0;
    int wc = 0;
    if (live && err == 0u && n > 0) {
        if ((uint64_t)a.wide_base + 1u > a.wide_cap || a.item_cap < 1u) {
            err |= kBuildErrCap;
        } else {
            wn = 1;
            wnext = a.wide_base + 1u;
            if (gtid == 0) a.witems[0][0] = make_int4((int)a.node_base, (int)a.wide_base, 1, 0);
            live = grid_sync(a.sync);
        }
    }
    while (live && err == 0u && wn > 0) {
        if (++levels > 64) { err |= kBuildErrRounds; break; }
        for (uint32_t i = gtid; i < wn; i += gthreads)
            wide_count_cache_item(a.bin, a.witems[wc], i, a.wcnt, a.wcache, a.wcache_n, a.lk);
        if (!(live = grid_sync(a.sync))) break;
        if (blockIdx.x == 0) block_scan_excl<uint32_t>(a.wcnt, wn, a.woff, a.tot32);
        if (!(live = grid_sync(a.sync))) break;
        const uint32_t tot = __ldcg(a.tot32);
        if ((uint64_t)wnext + tot > a.wide_cap || tot > a.item_cap) { err |= kBuildErrCap; break; }
        for (uint32_t i = gtid; i < wn; i += gthreads)
            wide_emit_cached_item(a.wcache, a.wcache_n, a.witems[wc], i, a.woff, wnext, a.wide, a.witems[wc ^ 1],
                                  a.info + 3, a.lk);
        if (!(live = grid_sync(a.sync))) break;
        wnext += tot;
        wn = tot;
        wc ^= 1;
    }
    // every thread has the same err (it follows from values all threads read); the last
    // barrier makes the small tasks' and the collapse's error words complete
    if (live) live = grid_sync(a.sync);
    if (gtid == 0) {
        const uint32_t used_small = __ldcg(a.info), depth_small = __ldcg(a.info + 1);
        a.result[0] = next_node;
        a.result[1] = nodes_used + used_small;
        a.result[2] = max(rounds, depth_small);
        a.result[3] = wnext - a.wide_base;
        a.result[4] = levels;
        a.result[5] = err | __ldcg(a.info + 2) | __ldcg(a.info + 3) | __ldcg(a.sync + 2) | (live ? 0u : kBuildErrSync);
    }
}

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t cap = 0;
    cudaError_t need(size_t n) {
        if (n <= cap) return cudaSuccess;
        release();
        const size_t want = std::max<size_t>(n + n / 4, 16);
        cudaError_t e = cudaMalloc((void**)&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        else p = nullptr;
        return e;
    }
    // grow keeping the first `keep` entries; the rest is zero
    cudaError_t grow_keep(size_t n, size_t keep, cudaStream_t st) {
        if (n <= cap) return cudaSuccess;
        const size_t want = std::max<size_t>(n + n / 2, 16);
        T* q = nullptr;
        cudaError_t e = cudaMalloc((void**)&q, want * sizeof(T));
        if (e != cudaSuccess) return e;
        e = cudaMemsetAsync(q, 0, want * sizeof(T), st);
        if (e == cudaSuccess && keep && p) e = cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            cudaFree(q);
            return e;
        }
        release();
        p = q;
        cap = want;
        return cudaSuccess;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

#define GK_TRY(x)                         \
    do {                                  \
        cudaError_t e_ = (x);             \
        if (e_ != cudaSuccess) return e_; \
    } while (0)

}  // namespace

struct GpuBvh {
    DBuf<float> box, cent, root_box;
    DBuf<uint32_t> idx, tmp, wtask[2], wbeg[2], wend[2], w0[2], wleft, wleft_scan, bsum32, tot32, info, map;
    DBuf<uint4> cc, cc_scan, bsum4, tot4;
    DBuf<int> bins, tb;
    DBuf<BigTask> tasks[2];
    DBuf<Split> split;
    DBuf<SmallTask> small;
    DBuf<BvhNode> nodes;
    DBuf<MeshRange> ranges;
    DBuf<int4> witems[2];
    DBuf<uint32_t> wcnt, woff, werr, sync, result;
    DBuf<WEnt> wcache;
    DBuf<int> wcache_n;
    uint32_t* result_host = nullptr;   // page-locked copy of the instance level's result record
    uint32_t inst_level_n = 0;         // instances of the instance-level build in flight
    uint32_t launches = 0;   // kernels launched by all builds so far

    ~GpuBvh() {
        box.release(); cent.release(); root_box.release(); idx.release(); tmp.release();
        for (int k = 0; k < 2; ++k) {
            wtask[k].release(); wbeg[k].release(); wend[k].release(); w0[k].release(); tasks[k].release();
        }
        wleft.release(); wleft_scan.release(); bsum32.release(); tot32.release(); info.release(); map.release();
        cc.release(); cc_scan.release(); bsum4.release(); tot4.release(); bins.release(); tb.release();
        split.release(); small.release(); nodes.release(); ranges.release();
        witems[0].release(); witems[1].release(); wcnt.release(); woff.release(); werr.release();
        sync.release(); result.release(); wcache.release(); wcache_n.release();
        if (result_host) cudaFreeHost(result_host);
    }

    template <class T>
    cudaError_t scan(const T* in, uint32_t n, T* out, DBuf<T>& bsum, DBuf<T>& tot, cudaStream_t st) {
        const uint32_t nb = std::max<uint32_t>((n + kScanB - 1) / kScanB, 1u);
        GK_TRY(bsum.need(nb));
        GK_TRY(tot.need(1));
        if (n) k_scan_blocks<T><<<nb, kScanB, 0, st>>>(in, n, out, bsum.p);
        else GK_TRY(cudaMemsetAsync(bsum.p, 0, sizeof(T), st));
        k_scan_sums<T><<<1, kScanB, 0, st>>>(bsum.p, nb, tot.p);
        if (n) k_scan_fix<T><<<nb, kScanB, 0, st>>>(in, n, out, bsum.p);
        launches += n ? 3u : 1u;
        return cudaGetLastError();
    }

    // Builds over the n primitives whose boxes and centroids are in box/cent, one tree per
    // root range [root_begin[r], root_end[r]). Triangle leaves hold ranges of the final
    // order (idx); instance leaves hold prim_map[primitive]. Refs are node_base + relative
    // node index.
    cudaError_t build(uint32_t n, const std::vector<uint32_t>& root_begin, const std::vector<uint32_t>& root_end,
                      uint32_t max_leaf, bool inst_leaf, const uint32_t* prim_map, uint32_t node_base,
                      GpuBvhResult* out, cudaStream_t st) {
        const uint32_t nroots = (uint32_t)root_begin.size();
        out->root_node.assign(nroots, -1);
        out->node_count = 0;
        out->nodes_used = 0;
        out->depth = 0;
        GK_TRY(idx.need(std::max<uint32_t>(n, 1u)));
        GK_TRY(tmp.need(std::max<uint32_t>(n, 1u)));
        GK_TRY(root_box.need(6 * (size_t)std::max<uint32_t>(nroots, 1u)));
        GK_TRY(info.need(4));
        GK_TRY(cudaMemsetAsync(info.p, 0, 16, st));
        if (n) {
            k_init_idx<<<(n + 255) / 256, 256, 0, st>>>(idx.p, n);
            ++launches;
        }
        // roots: node slots [0, nroots); small roots reserve m - 1 slots after them
        std::vector<float> rbox(6 * (size_t)std::max<uint32_t>(nroots, 1u));
        for (uint32_t r = 0; r < nroots; ++r)
            for (int k = 0; k < 3; ++k) { rbox[6 * r + k] = INFINITY; rbox[6 * r + 3 + k] = -INFINITY; }
        std::vector<BigTask> big;
        std::vector<SmallTask> smalls;
        std::vector<uint32_t> hw[3], hw0;
        uint32_t next_node = nroots;
        for (uint32_t r = 0; r < nroots; ++r) {
            const uint32_t b = root_begin[r], e = root_end[r];
            if (e <= b) continue;
            out->root_node[r] = (int)(node_base + r);
            if (e - b > kSmall) {
                hw0.push_back((uint32_t)hw[0].size());
                for (uint32_t cb = b; cb < e; cb += kChunk) {
                    hw[0].push_back((uint32_t)big.size());
                    hw[1].push_back(cb);
                    hw[2].push_back(std::min(cb + kChunk, e));
                }
                big.push_back(BigTask{(int)r, -1 - (int)r, 0, 0, b, e});
            } else {
                smalls.push_back(SmallTask{-1 - (int)r, 0, 0, (int)r, b, e, next_node, 0u});
                next_node += e - b - 1u;
            }
        }
        uint32_t ntask = (uint32_t)big.size(), nwork = (uint32_t)hw[0].size(), nsmall = (uint32_t)smalls.size();
        GK_TRY(nodes.grow_keep(std::max<uint32_t>(next_node, 1u), 0, st));
        GK_TRY(cudaMemsetAsync(nodes.p, 0, nodes.cap * sizeof(BvhNode), st));
        GK_TRY(small.grow_keep(std::max<uint32_t>(nsmall, 1u), 0, st));
        GK_TRY(cudaMemcpyAsync(root_box.p, rbox.data(), rbox.size() * 4, cudaMemcpyHostToDevice, st));
        if (nsmall)
            GK_TRY(cudaMemcpyAsync(small.p, smalls.data(), nsmall * sizeof(SmallTask), cudaMemcpyHostToDevice, st));
        int cur = 0;
        if (ntask) {
            GK_TRY(tasks[0].need(ntask));
            GK_TRY(w0[0].need(ntask));
            GK_TRY(wtask[0].need(nwork));
            GK_TRY(wbeg[0].need(nwork));
            GK_TRY(wend[0].need(nwork));
            GK_TRY(cudaMemcpyAsync(wtask[0].p, hw[0].data(), nwork * 4ull, cudaMemcpyHostToDevice, st));
            GK_TRY(cudaMemcpyAsync(wbeg[0].p, hw[1].data(), nwork * 4ull, cudaMemcpyHostToDevice, st));
            GK_TRY(cudaMemcpyAsync(wend[0].p, hw[2].data(), nwork * 4ull, cudaMemcpyHostToDevice, st));
            GK_TRY(cudaMemcpyAsync(tasks[0].p, big.data(), ntask * sizeof(BigTask), cudaMemcpyHostToDevice, st));
            GK_TRY(cudaMemcpyAsync(w0[0].p, hw0.data(), ntask * 4ull, cudaMemcpyHostToDevice, st));
        }
        GK_TRY(cudaStreamSynchronize(st));   // the host staging vectors are reused below
        const Geo g{box.p, cent.p};
        int rounds = 0;
        while (ntask > 0) {
            if (++rounds > 64) return cudaErrorInvalidValue;
            const uint32_t gt = (ntask + 255) / 256;
            GK_TRY(bins.need((size_t)ntask * kBinWords));
            GK_TRY(tb.need((size_t)ntask * 12));
            GK_TRY(split.need(ntask));
            GK_TRY(wleft.need(nwork));
            GK_TRY(wleft_scan.need(nwork));
            GK_TRY(cc.need(ntask));
            GK_TRY(cc_scan.need(ntask));
            const uint32_t nclear = ntask * (uint32_t)(kBinWords + 12);
            k_clear<<<std::min<uint32_t>((nclear + 255) / 256, 4096u), 256, 0, st>>>(bins.p, tb.p, ntask);
            k_bounds<<<nwork, kBt, 0, st>>>(g, idx.p, wtask[cur].p, wbeg[cur].p, wend[cur].p, tb.p);
            k_bin<<<nwork, kBt, 0, st>>>(g, idx.p, tb.p, wtask[cur].p, wbeg[cur].p, wend[cur].p, bins.p);
            k_split<<<gt, 256, 0, st>>>(tasks[cur].p, ntask, bins.p, tb.p, split.p, nodes.p, root_box.p, node_base);
            k_count_left<<<nwork, kBt, 0, st>>>(g, idx.p, split.p, tasks[cur].p, wtask[cur].p, wbeg[cur].p,
                                                wend[cur].p, wleft.p);
            GK_TRY(scan<uint32_t>(wleft.p, nwork, wleft_scan.p, bsum32, tot32, st));
            k_scatter<<<nwork, kBt, 0, st>>>(g, idx.p, tmp.p, split.p, tasks[cur].p, wtask[cur].p, wbeg[cur].p,
                                             wend[cur].p, wleft_scan.p, w0[cur].p, info.p);
            k_copy_back<<<nwork, kBt, 0, st>>>(tmp.p, idx.p, wbeg[cur].p, wend[cur].p);
            k_child_counts<<<gt, 256, 0, st>>>(tasks[cur].p, ntask, split.p, cc.p);
            GK_TRY(scan<uint4>(cc.p, ntask, cc_scan.p, bsum4, tot4, st));
            uint4 tot;
            GK_TRY(cudaMemcpyAsync(&tot, tot4.p, sizeof(uint4), cudaMemcpyDeviceToHost, st));
            GK_TRY(cudaStreamSynchronize(st));
            const uint32_t nbig = tot.x, nwork_next = tot.y, nsm = tot.z, nres = tot.w;
            const uint32_t node0 = next_node, res0 = next_node + nbig;
            GK_TRY(nodes.grow_keep(next_node + nbig + nres, next_node, st));
            next_node += nbig + nres;
            GK_TRY(small.grow_keep(nsmall + nsm, nsmall, st));
            const int nx = cur ^ 1;
            GK_TRY(tasks[nx].need(std::max<uint32_t>(nbig, 1u)));
            GK_TRY(w0[nx].need(std::max<uint32_t>(nbig, 1u)));
            GK_TRY(wtask[nx].need(std::max<uint32_t>(nwork_next, 1u)));
            GK_TRY(wbeg[nx].need(std::max<uint32_t>(nwork_next, 1u)));
            GK_TRY(wend[nx].need(std::max<uint32_t>(nwork_next, 1u)));
            k_emit<<<gt, 256, 0, st>>>(tasks[cur].p, ntask, split.p, cc_scan.p, node0, res0, nsmall, tasks[nx].p,
                                       wtask[nx].p, wbeg[nx].p, wend[nx].p, w0[nx].p, small.p);
            GK_TRY(cudaGetLastError());
            launches += 9u;   // clear, bounds, bin, split, count_left, scatter, copy_back, child_counts, emit
            out->nodes_used += ntask;
            nsmall += nsm;
            ntask = nbig;
            nwork = nwork_next;
            cur = nx;
        }
        if (nsmall) {
            k_small<<<(nsmall + 127) / 128, 128, 0, st>>>(g, idx.p, small.p, nsmall, nodes.p, root_box.p, max_leaf,
                                                          inst_leaf ? 1 : 0, prim_map, node_base, info.p);
            ++launches;
        }
        GK_TRY(cudaGetLastError());
        uint32_t hinfo[4];
        GK_TRY(cudaMemcpyAsync(hinfo, info.p, 16, cudaMemcpyDeviceToHost, st));
        GK_TRY(cudaStreamSynchronize(st));
        if (hinfo[2]) return cudaErrorInvalidValue;
        out->nodes_used += hinfo[0];
        out->depth = std::max<int>(rounds, (int)hinfo[1]);
        out->node_count = next_node;
        out->nodes = nodes.p;
        out->order = idx.p;
        out->root_box = root_box.p;
        return cudaSuccess;
    }

    // Collapses the two-child trees rooted at roots[r] (refs into bin; -1: none) into wide
    // nodes out[wide_base, wide_base + count), out holding out_cap nodes in all. The root of
    // tree r becomes wide node wroots[r] = wide_base + (its position among the valid roots).
    cudaError_t collapse(const BvhNode* bin, const std::vector<int>& roots, uint32_t wide_base, WideNode* out,
                         size_t out_cap, std::vector<int>& wroots, uint32_t* count, int* depth, cudaStream_t st,
                         const RefitLinks* links) {
        const RefitLinks lk = links ? *links : RefitLinks();
        wroots.assign(roots.size(), -1);
        std::vector<int4> it0;
        uint32_t next = wide_base;
        for (size_t r = 0; r < roots.size(); ++r) {
            if (roots[r] < 0) continue;
            wroots[r] = (int)next;
            it0.push_back(make_int4(roots[r], (int)next, 1, 0));
            ++next;
        }
        *count = 0;
        *depth = 0;
        uint32_t n = (uint32_t)it0.size();
        if (n == 0) return cudaSuccess;
        if (next > out_cap) return cudaErrorInvalidValue;
        GK_TRY(witems[0].need(n));
        GK_TRY(werr.need(1));
        GK_TRY(cudaMemsetAsync(werr.p, 0, 4, st));
        GK_TRY(cudaMemcpyAsync(witems[0].p, it0.data(), n * sizeof(int4), cudaMemcpyHostToDevice, st));
        int cur = 0, levels = 0;
        while (n > 0) {
            if (++levels > 64) return cudaErrorInvalidValue;
            GK_TRY(wcnt.need(n));
            GK_TRY(woff.need(n));
            const uint32_t g = (n + 127) / 128;
            k_wide_count<<<g, 128, 0, st>>>(bin, witems[cur].p, n, wcnt.p);
            ++launches;
            GK_TRY(scan<uint32_t>(wcnt.p, n, woff.p, bsum32, tot32, st));
            uint32_t tot = 0;
            GK_TRY(cudaMemcpyAsync(&tot, tot32.p, 4, cudaMemcpyDeviceToHost, st));
            GK_TRY(cudaStreamSynchronize(st));
            if ((size_t)next + tot > out_cap) return cudaErrorInvalidValue;
            GK_TRY(witems[cur ^ 1].need(std::max<uint32_t>(tot, 1u)));
            k_wide_emit<<<g, 128, 0, st>>>(bin, witems[cur].p, n, woff.p, next, out, witems[cur ^ 1].p, werr.p, lk);
            ++launches;
            GK_TRY(cudaGetLastError());
            next += tot;
            n = tot;
            cur ^= 1;
        }
        uint32_t herr = 0;
        GK_TRY(cudaMemcpyAsync(&herr, werr.p, 4, cudaMemcpyDeviceToHost, st));
        GK_TRY(cudaStreamSynchronize(st));
        if (herr) return cudaErrorInvalidValue;
        *count = next - wide_base;
        *depth = levels;
        return cudaSuccess;
    }
};

GpuBvh* gpu_bvh_new() { return new (std::nothrow) GpuBvh(); }
uint32_t gpu_bvh_launches(const GpuBvh* b) { return b ? b->launches : 0u; }
void gpu_bvh_free(GpuBvh* b) { delete b; }

cudaError_t gpu_bvh_build_meshes(GpuBvh* B, const float4* pos, const uint32_t* ind, const GkrtMesh* meshes,
                                 uint32_t nmesh, uint32_t node_base, float4* tris_out, GpuBvhResult* out,
                                 cudaStream_t st) {
    std::vector<MeshRange> mr(std::max<uint32_t>(nmesh, 1u), MeshRange{0u, 0u, 0u, 0u});
    std::vector<uint32_t> rb(nmesh), re(nmesh);
    uint32_t ntri = 0;
    for (uint32_t m = 0; m < nmesh; ++m) {
        mr[m] = MeshRange{ntri, meshes[m].index_offset, meshes[m].vertex_offset, 0u};
        rb[m] = ntri;
        ntri += meshes[m].index_count / 3u;
        re[m] = ntri;
    }
    GK_TRY(B->ranges.need(mr.size()));
    GK_TRY(cudaMemcpyAsync(B->ranges.p, mr.data(), mr.size() * sizeof(MeshRange), cudaMemcpyHostToDevice, st));
    GK_TRY(B->box.need(6 * (size_t)std::max<uint32_t>(ntri, 1u)));
    GK_TRY(B->cent.need(3 * (size_t)std::max<uint32_t>(ntri, 1u)));
    const uint32_t nmr = std::max<uint32_t>(nmesh, 1u);
    if (ntri) {
        k_tri_boxes<<<(ntri + 255) / 256, 256, 0, st>>>(pos, ind, B->ranges.p, nmr, ntri, B->box.p, B->cent.p);
        ++B->launches;
    }
    GK_TRY(cudaGetLastError());
    GK_TRY(B->build(ntri, rb, re, 4, false, nullptr, node_base, out, st));
    if (ntri) {
        k_gather_tris<<<(ntri + 255) / 256, 256, 0, st>>>(pos, ind, B->ranges.p, nmr, B->idx.p, ntri, tris_out);
        ++B->launches;
    }
    GK_TRY(cudaGetLastError());
    return cudaStreamSynchronize(st);
}

cudaError_t gpu_bvh_build_instance_level_launch(GpuBvh* B, const GpuInstBox* inst, uint32_t n, const float* mesh_box,
                                               BvhNode* nodes, uint32_t node_base, uint32_t node_cap, WideNode* wide,
                                               uint32_t wide_base, uint32_t wide_cap, const RefitLinks* links,
                                               cudaStream_t st) {
    B->inst_level_n = n;
    if (n == 0) return cudaSuccess;
    if ((uint64_t)node_cap < (uint64_t)n + 1u) return cudaErrorInvalidValue;
    const uint32_t cap_t = n / (kSmall + 1u) + 2u, cap_w = cap_t + n / kChunk + 2u, cap_s = n + 1u;
    GK_TRY(B->map.need(n));
    GK_TRY(B->box.need(6 * (size_t)n));
    GK_TRY(B->cent.need(3 * (size_t)n));
    GK_TRY(B->idx.need(n));
    GK_TRY(B->tmp.need(n));
    for (int k = 0; k < 2; ++k) {
        GK_TRY(B->tasks[k].need(cap_t));
        GK_TRY(B->w0[k].need(cap_t));
        GK_TRY(B->wtask[k].need(cap_w));
        GK_TRY(B->wbeg[k].need(cap_w));
        GK_TRY(B->wend[k].need(cap_w));
        GK_TRY(B->witems[k].need(cap_s));
    }
    GK_TRY(B->bins.need((size_t)cap_t * kBinWords));
    GK_TRY(B->tb.need((size_t)cap_t * 12));
    GK_TRY(B->split.need(cap_t));
    GK_TRY(B->wleft.need(cap_w));
    GK_TRY(B->wleft_scan.need(cap_w));
    GK_TRY(B->cc.need(cap_t));
    GK_TRY(B->cc_scan.need(cap_t));
    GK_TRY(B->small.need(cap_s));
    GK_TRY(B->root_box.need(6));
    GK_TRY(B->info.need(4));
    GK_TRY(B->wcnt.need(cap_s));
    GK_TRY(B->woff.need(cap_s));
    GK_TRY(B->wcache.need(8 * (size_t)cap_s));
    GK_TRY(B->wcache_n.need(cap_s));
    GK_TRY(B->tot4.need(1));
    GK_TRY(B->tot32.need(1));
    GK_TRY(B->sync.need(3));
    GK_TRY(B->result.need(8));
    if (!B->result_host) GK_TRY(cudaMallocHost((void**)&B->result_host, 8 * sizeof(uint32_t)));
    GK_TRY(cudaMemsetAsync(B->info.p, 0, 16, st));
    GK_TRY(cudaMemsetAsync(B->sync.p, 0, 12, st));
    GK_TRY(cudaMemsetAsync(nodes + node_base, 0, (size_t)node_cap * sizeof(BvhNode), st));
    InstLevelArgs a;
    std::memset(&a, 0, sizeof(a));
    a.inst = inst; a.n = n; a.mesh_box = mesh_box;
    a.box = B->box.p; a.cent = B->cent.p; a.idx = B->idx.p; a.tmp = B->tmp.p; a.map = B->map.p;
    for (int k = 0; k < 2; ++k) {
        a.tasks[k] = B->tasks[k].p; a.w0[k] = B->w0[k].p; a.wtask[k] = B->wtask[k].p;
        a.wbeg[k] = B->wbeg[k].p; a.wend[k] = B->wend[k].p; a.witems[k] = B->witems[k].p;
    }
    a.bins = B->bins.p; a.tb = B->tb.p; a.split = B->split.p; a.wleft = B->wleft.p; a.wleft_scan = B->wleft_scan.p;
    a.cc = B->cc.p; a.cc_scan = B->cc_scan.p; a.small = B->small.p;
    a.cap_t = cap_t; a.cap_w = cap_w; a.cap_s = cap_s;
    a.nodes = nodes + node_base; a.bin = nodes; a.node_base = node_base; a.node_cap = node_cap;
    a.root_box = B->root_box.p; a.info = B->info.p;
    a.wcnt = B->wcnt.p; a.woff = B->woff.p; a.item_cap = cap_s;
    a.wcache = B->wcache.p; a.wcache_n = B->wcache_n.p;
    a.wide = wide; a.wide_base = wide_base; a.wide_cap = wide_cap;
    if (links) a.lk = *links;
    a.sync = B->sync.p; a.tot4 = B->tot4.p; a.tot32 = B->tot32.p; a.result = B->result.p;
    // one block per 256 instances, at most one per SM: every block is resident (cooperative
    // launch), and a barrier costs one arrival per block
    int dev = 0, sms = 1, per = 0;
    GK_TRY(cudaGetDevice(&dev));
    GK_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GK_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_inst_level, kBt, 0));
    if (per < 1) return cudaErrorLaunchOutOfResources;
    const uint32_t grid = std::max<uint32_t>(1u, std::min<uint32_t>((n + kBt - 1) / kBt, (uint32_t)sms));
    void* params[] = {&a};
    GK_TRY(cudaLaunchCooperativeKernel((const void*)k_inst_level, dim3(grid), dim3(kBt), params, 0, st));
    ++B->launches;
    return cudaMemcpyAsync(B->result_host, B->result.p, 6 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
}

cudaError_t gpu_bvh_build_instance_level_finish(GpuBvh* B, InstLevelResult* res, cudaStream_t st) {
    *res = InstLevelResult();
    if (B->inst_level_n == 0) return cudaSuccess;
    GK_TRY(cudaStreamSynchronize(st));
    const uint32_t* r = B->result_host;
    res->node_count = r[0];
    res->nodes_used = r[1];
    res->depth = (int)r[2];
    res->wide_count = r[3];
    res->wide_depth = (int)r[4];
    res->error = r[5];
    return cudaSuccess;
}

bool gpu_bvh_cooperative_supported() {
    int dev = 0, coop = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess) return false;
    return coop != 0;
}

cudaError_t gpu_bvh_collapse(GpuBvh* B, const BvhNode* bin, const std::vector<int>& roots, uint32_t wide_base,
                             WideNode* out, size_t out_cap, std::vector<int>& wroots, uint32_t* count, int* depth,
                             cudaStream_t st, const RefitLinks* links) {
    return B->collapse(bin, roots, wide_base, out, out_cap, wroots, count, depth, st, links);
}

cudaError_t gpu_bvh_refit_instances(const RefitLinks& lk, const GpuInstBox* inst, const float* mesh_box,
                                    BvhNode* nodes, float* ubox, uint32_t* arrive, WideNode* wide, uint32_t nw,
                                    uint32_t* err, uint32_t err_bit, cudaStream_t st) {
    if (lk.ninst) k_refit_boxes<<<(lk.ninst + 127) / 128, 128, 0, st>>>(lk, inst, mesh_box, nodes, ubox, arrive);
    // a few thousand nodes: 32-thread blocks spread them over the SMs (FP64 latency-bound)
    if (nw) k_refit_wide<<<(nw + 31) / 32, 32, 0, st>>>(lk, nodes, wide, nw, err, err_bit);
    return cudaGetLastError();
}

}  // namespace gk
