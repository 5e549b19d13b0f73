// emitters.cu — the emissive-triangle table and its alias table (host side, per instance update).
//
// Used by GKRT_NEE_EMISSIVE (no counterpart in the built reference path; the reference's only
// area-light sampling is the legacy uniform light pick of RTCommon.glsl:50 with the
// parallelogram sample of Scatter.glsl:55-76). Every visible instance contributes the
// triangles whose vertex-0 material slot maps to a diffuse-light material of non-zero
// luminance, in the order: instance, slot 0..15, triangle. Each entry is picked with
// probability power / total power (power = area x luminance) through Walker's alias method
// as built by Vose (stable worklists, double-precision bookkeeping), so that the pick costs
// one table read and one comparison on the GPU.
//
// All float arithmetic is written out operation by operation and the library's host code is
// compiled without contraction, so the table is bit-identical to the oracle's restatement.
#include <cmath>
#include <cstring>
#include <vector>

#include "gkrt_internal.h"

namespace gk {

namespace {

struct V3 {
    float x, y, z;
};

inline V3 xform(const float* w, const float* p) {
    V3 r;
    r.x = ((w[0] * p[0] + w[1] * p[1]) + w[2] * p[2]) + w[3];
    r.y = ((w[4] * p[0] + w[5] * p[1]) + w[6] * p[2]) + w[7];
    r.z = ((w[8] * p[0] + w[9] * p[1]) + w[10] * p[2]) + w[11];
    return r;
}

}  // namespace

float emitter_luminance(const float* rgb) { return (0.2126f * rgb[0] + 0.7152f * rgb[1]) + 0.0722f * rgb[2]; }

void mesh_slot_triangles(const GkrtMesh* meshes, uint32_t nmesh, const uint32_t* indices, const uint32_t* slots,
                         std::vector<std::vector<uint32_t>>& out) {
    out.assign(16 * (size_t)nmesh, std::vector<uint32_t>());
    for (uint32_t m = 0; m < nmesh; ++m) {
        const GkrtMesh& ms = meshes[m];
        for (uint32_t t = 0; t < ms.index_count / 3; ++t) {
            const uint32_t s = slots[indices[ms.index_offset + 3 * t] + ms.vertex_offset] & 15u;
            out[16 * (size_t)m + s].push_back(t);
        }
    }
}

void build_emitter_table(const GkrtInstance* inst, uint32_t ninst, const GkrtMesh* meshes, const float* pos,
                         const uint32_t* indices, const std::vector<std::vector<uint32_t>>& slot_tris,
                         const GkrtMaterial* mats, uint32_t nmat, EmitterTable& out) {
    out.geo.clear();
    out.alias.clear();
    std::vector<float> power, lum;
    for (uint32_t i = 0; i < ninst; ++i) {
        const GkrtInstance& in = inst[i];
        if (!in.visible) continue;
        const GkrtMesh& ms = meshes[in.mesh_id];
        for (int s = 0; s < 16; ++s) {
            const uint32_t mi = in.mat_id[s];
            if (mi >= nmat) continue;
            const GkrtMaterial& mt = mats[mi];
            if (mt.material_model != GKRT_MAT_DIFFUSE_LIGHT) continue;
            const float l = emitter_luminance(mt.diffuse);
            if (!(l > 0.0f)) continue;
            for (uint32_t t : slot_tris[16 * (size_t)in.mesh_id + s]) {
                V3 p[3];
                for (int v = 0; v < 3; ++v)
                    p[v] = xform(in.world, pos + 4 * (size_t)(indices[ms.index_offset + 3 * t + v] + ms.vertex_offset));
                const V3 e1{p[1].x - p[0].x, p[1].y - p[0].y, p[1].z - p[0].z};
                const V3 e2{p[2].x - p[0].x, p[2].y - p[0].y, p[2].z - p[0].z};
                const V3 c{e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                const float len = std::sqrt((c.x * c.x + c.y * c.y) + c.z * c.z);
                const float area = 0.5f * len;
                if (!(area > 0.0f) || !std::isfinite(area)) continue;
                const float inv = 1.0f / len;
                out.geo.push_back(make_float4(p[0].x, p[0].y, p[0].z, 0.0f));   // w: area / pick probability
                out.geo.push_back(make_float4(e1.x, e1.y, e1.z, 0.0f));
                out.geo.push_back(make_float4(e2.x, e2.y, e2.z, 0.0f));
                out.geo.push_back(make_float4(c.x * inv, c.y * inv, c.z * inv, 0.0f));
                out.geo.push_back(make_float4(mt.diffuse[0], mt.diffuse[1], mt.diffuse[2], mt.diffuse[3]));
                power.push_back(area * l);
                lum.push_back(l);
            }
        }
    }
    const size_t n = power.size();
    if (n == 0) return;
    double total = 0.0;
    for (float p : power) total += (double)p;
    // area / (power / total) = total / luminance
    for (size_t j = 0; j < n; ++j) out.geo[5 * j].w = (float)(total / (double)lum[j]);
    std::vector<double> q(n);
    std::vector<size_t> small, large;
    for (size_t j = 0; j < n; ++j) {
        q[j] = (double)power[j] * (double)n / total;
        (q[j] < 1.0 ? small : large).push_back(j);
    }
    std::vector<float> thr(n, 1.0f);
    std::vector<uint32_t> ali(n);
    for (size_t j = 0; j < n; ++j) ali[j] = (uint32_t)j;
    while (!small.empty() && !large.empty()) {
        const size_t l = small.back();
        small.pop_back();
        const size_t g = large.back();
        large.pop_back();
        thr[l] = (float)q[l];
        ali[l] = (uint32_t)g;
        q[g] = (q[g] + q[l]) - 1.0;
        (q[g] < 1.0 ? small : large).push_back(g);
    }
    out.alias.resize(n);
    for (size_t j = 0; j < n; ++j) {
        float a;
        std::memcpy(&a, &ali[j], 4);
        out.alias[j] = make_float2(thr[j], a);
    }
}

}  // namespace gk
