// bvh_host.cu — binned-SAH BVH builder on the host (scene-load path).
//
// Replaces the Vulkan BLAS/TLAS builds of RayTraceBaseRenderer::CreateBottomLevelStructures
// / CreateTopLevelStructures (src/Rendering/RayTraceBaseRenderer.cpp:276-386), which use
// VK_BUILD_ACCELERATION_STRUCTURE_PREFER_FAST_TRACE (src/Vulkan/RayTracing/
// AccelerationStructure.cpp:21). Like the reference's CPU BVH (tinybvh::BVH::Build, binned
// SAH), it bins centroids; it emits the two-child 64-byte nodes the kernels traverse.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "gk_trace.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

struct Aabb {
    float lo[3], hi[3];
    void reset() { lo[0] = lo[1] = lo[2] = INFINITY; hi[0] = hi[1] = hi[2] = -INFINITY; }
    void grow(const Aabb& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    float area() const {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        if (dx < 0.0f || dy < 0.0f || dz < 0.0f) return 0.0f;
        return 2.0f * (dx * dy + dy * dz + dz * dx);
    }
};

struct Builder {
    const float* boxes;
    uint32_t max_leaf;
    uint32_t node_base, prim_base;
    bool inst_leaf;
    std::vector<uint32_t> idx;
    std::vector<float> cent;
    HostBvh* out;

    Aabb box_of(uint32_t p) const {
        Aabb b;
        for (int k = 0; k < 3; ++k) { b.lo[k] = boxes[6 * p + k]; b.hi[k] = boxes[6 * p + 3 + k]; }
        return b;
    }

    int leaf_ref(uint32_t first, uint32_t cnt) const {
        uint32_t payload;
        if (inst_leaf) payload = (idx[first] << 3);
        else payload = ((prim_base + first) << 3) | (cnt - 1u);
        return (int)(~payload);
    }

    // Returns a node ref for the subtree over idx[b, e); fills box.
    int build(uint32_t b, uint32_t e, Aabb& box, int depth) {
        out->depth = std::max(out->depth, depth);
        box.reset();
        Aabb cb;
        cb.reset();
        for (uint32_t i = b; i < e; ++i) {
            box.grow(box_of(idx[i]));
            for (int k = 0; k < 3; ++k) {
                cb.lo[k] = std::min(cb.lo[k], cent[3 * idx[i] + k]);
                cb.hi[k] = std::max(cb.hi[k], cent[3 * idx[i] + k]);
            }
        }
        const uint32_t n = e - b;
        if (inst_leaf ? n == 1 : n <= 2) return leaf_ref(b, n);
        // binned SAH over 16 bins on each axis
        const int kBins = 16;
        float best_cost = INFINITY;
        int best_axis = -1, best_split = 0;
        for (int ax = 0; ax < 3; ++ax) {
            float ext = cb.hi[ax] - cb.lo[ax];
            if (!(ext > 0.0f)) continue;
            Aabb bb[kBins];
            uint32_t bc[kBins] = {0};
            for (int i = 0; i < kBins; ++i) bb[i].reset();
            float scale = kBins / ext;
            for (uint32_t i = b; i < e; ++i) {
                int bi = (int)((cent[3 * idx[i] + ax] - cb.lo[ax]) * scale);
                bi = std::min(std::max(bi, 0), kBins - 1);
                bc[bi]++;
                bb[bi].grow(box_of(idx[i]));
            }
            float ra[kBins];
            uint32_t rc[kBins];
            Aabb acc;
            acc.reset();
            uint32_t cnt = 0;
            for (int i = kBins - 1; i > 0; --i) {
                acc.grow(bb[i]);
                cnt += bc[i];
                ra[i] = acc.area();
                rc[i] = cnt;
            }
            acc.reset();
            cnt = 0;
            for (int i = 0; i < kBins - 1; ++i) {
                acc.grow(bb[i]);
                cnt += bc[i];
                if (cnt == 0 || rc[i + 1] == 0) continue;
                float cost = acc.area() * cnt + ra[i + 1] * rc[i + 1];
                if (cost < best_cost) { best_cost = cost; best_axis = ax; best_split = i + 1; }
            }
        }
        const float leaf_cost = box.area() * n;
        if (n <= max_leaf && !inst_leaf && (best_axis < 0 || leaf_cost <= best_cost + 1.0f * box.area()))
            return leaf_ref(b, n);
        uint32_t mid;
        if (best_axis < 0) {
            mid = b + n / 2;   // coincident centroids: split by order
        } else {
            float ext = cb.hi[best_axis] - cb.lo[best_axis];
            float scale = kBins / ext;
            auto it = std::partition(idx.begin() + b, idx.begin() + e, [&](uint32_t p) {
                int bi = (int)((cent[3 * p + best_axis] - cb.lo[best_axis]) * scale);
                bi = std::min(std::max(bi, 0), kBins - 1);
                return bi < best_split;
            });
            mid = (uint32_t)(it - idx.begin());
            if (mid == b || mid == e) mid = b + n / 2;
        }
        const int me = (int)out->nodes.size();
        out->nodes.push_back(BvhNode{});
        Aabb lb, rb;
        int lref = build(b, mid, lb, depth + 1);
        int rref = build(mid, e, rb, depth + 1);
        BvhNode& nd = out->nodes[me];
        nd.a = make_float4(widen_lo(lb.lo[0]), widen_lo(lb.lo[1]), widen_lo(lb.lo[2]), widen_hi(lb.hi[0]));
        nd.b = make_float4(widen_hi(lb.hi[1]), widen_hi(lb.hi[2]), widen_lo(rb.lo[0]), widen_lo(rb.lo[1]));
        nd.c = make_float4(widen_lo(rb.lo[2]), widen_hi(rb.hi[0]), widen_hi(rb.hi[1]), widen_hi(rb.hi[2]));
        nd.d = make_int4(lref, rref, 0, 0);
        return (int)node_base + me;
    }
};

}  // namespace

void build_bvh_host(const float* boxes, uint32_t n, uint32_t max_leaf, uint32_t node_base, uint32_t prim_base,
                    bool leaf_is_instance, HostBvh& out) {
    out.nodes.clear();
    out.order.clear();
    out.root = -1;
    out.depth = 0;
    if (n == 0) return;
    Builder B;
    B.boxes = boxes;
    B.max_leaf = leaf_is_instance ? 1u : std::max(1u, std::min(max_leaf, 8u));
    B.node_base = node_base;
    B.prim_base = prim_base;
    B.inst_leaf = leaf_is_instance;
    B.idx.resize(n);
    B.cent.resize(3 * (size_t)n);
    for (uint32_t i = 0; i < n; ++i) {
        B.idx[i] = i;
        for (int k = 0; k < 3; ++k) B.cent[3 * i + k] = 0.5f * (boxes[6 * i + k] + boxes[6 * i + 3 + k]);
    }
    B.out = &out;
    Aabb box;
    int ref = B.build(0, n, box, 0);
    if (ref < 0) {
        // a single leaf: wrap it in an interior root whose second child never intersects
        BvhNode nd;
        const float far = 1e30f;
        nd.a = make_float4(widen_lo(box.lo[0]), widen_lo(box.lo[1]), widen_lo(box.lo[2]), widen_hi(box.hi[0]));
        nd.b = make_float4(widen_hi(box.hi[1]), widen_hi(box.hi[2]), far, far);
        nd.c = make_float4(far, far, far, far);
        nd.d = make_int4(ref, kRefPop, 0, 0);
        out.nodes.insert(out.nodes.begin(), nd);
        // no other nodes exist in this case, so no index shifts are needed
        out.root = (int)node_base;
    } else {
        out.root = ref;
    }
    out.order = B.idx;
}

}  // namespace gk
