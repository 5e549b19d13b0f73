// gk_oracle.cpp — CPU restatement of gkNextRenderer's ray-tracing pass.
//
// TEST INFRASTRUCTURE ONLY: this library is the oracle the GB300 kernels are checked
// against (tests/, __graft_entry__.smoke(), and the CPU-baseline leg of bench.py). The
// product library never links, loads or calls it.
//
// What it restates (reference files, paths within gkNextEngine):
//   RNG ................ assets/shaders/common/Const_Func.slang:227-258 (pcg4d, uint_to_float)
//   samplers ........... Const_Func.slang:8-49 (Schlick, ONB, AlignWithNormal), 260-340
//                        (concentric disk, cone, cosine hemisphere, bounded VNDF GGX)
//   camera ray ......... assets/shaders/common/Shading.slang:283-334 (FHardwarePrimaryRayCaster)
//   closest/any hit .... Shading.slang:737-826 (FHardwareRayTracerV2) with the FP64 closest-hit
//                        definition of oracle_isect.h in place of RT-core RayQuery
//   bounce/shading ..... Shading.slang:1003-1082 (GetRayColor), 1084-1184 (Render)
//   primary outputs .... Shading.slang:1186-1241 (PrimaryHit, Init), 50-72 (motion vector),
//                        82-112 (FetchGBufferV2), Util.BufferClear.comp.slang:6-13 (clears)
//   sun NEE ............ Shading.slang:886-908, 1135-1144
//   probe termination .. assets/shaders/common/AmbientCube.slang:71-78, 178-223, 290-382
//   sample multiplier .. assets/shaders/Core.PathTracing.comp.slang:16-30
//   reprojection ....... assets/shaders/Process.ReProject.comp.slang:32-223
//   bilateral denoise .. assets/shaders/Process.DenoiseJBF.comp.slang:14-184, tonemap
//                        Const_Func.slang:51-126
// Deviations that both sides share (documented with the product): FP32 vertices instead of
// FP16; sin/cos of 2*pi*u and of |x|<=pi/4 from the polynomial in oracle_math.h; a constant
// sky colour instead of the HDR texture; out-of-range image reads return zero; the
// accumulation alpha keeps last frame's value (the reference writes only .rgb).
#include "oracle_math.h"
#include "oracle_isect.h"
#include "../include/gkrt.h"

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

using namespace gko;

namespace {

const float kEPS = 1e-3f;                 // PreProcessor.slang:13
const float kPT_MAX = 1000.0f;            // Shading.slang:15
const float kM_1_PI = 0.318309886183790671538f;
const float kCosQuarterDeg = 0.999990482f;  // cos(0.25 deg), Shading.slang:897
const float kHalton[8][2] = {{0.5f, 0.3333f}, {0.25f, 0.6667f}, {0.75f, 0.1111f}, {0.125f, 0.4444f},
                             {0.625f, 0.7778f}, {0.375f, 0.2222f}, {0.875f, 0.5556f}, {0.0625f, 0.8889f}};
const int kCubeXY = 192, kCubeZ = 48;
const float kCubeUnit = 0.25f;
const float kCubeOff[3] = {-24.0f, -0.34375f, -24.0f};

struct BNode {
    float lo[3], hi[3];
    int left;    // interior: left child; leaf: first prim
    int count;   // 0 interior (right = left + 1 is not assumed; right stored below)
    int right;
};

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<uint32_t> prims;
};

struct Box { float lo[3], hi[3]; };

void build_rec(Bvh& bvh, std::vector<Box>& boxes, std::vector<float>& cent, uint32_t* idx, int n, int node) {
    Box b{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = 0; i < n; ++i) {
        const Box& p = boxes[idx[i]];
        for (int k = 0; k < 3; ++k) {
            b.lo[k] = std::min(b.lo[k], p.lo[k]);
            b.hi[k] = std::max(b.hi[k], p.hi[k]);
            clo[k] = std::min(clo[k], cent[idx[i] * 3 + k]);
            chi[k] = std::max(chi[k], cent[idx[i] * 3 + k]);
        }
    }
    for (int k = 0; k < 3; ++k) { bvh.nodes[node].lo[k] = b.lo[k]; bvh.nodes[node].hi[k] = b.hi[k]; }
    if (n <= 4) {
        bvh.nodes[node].left = (int)(idx - bvh.prims.data());
        bvh.nodes[node].count = n;
        return;
    }
    int axis = 0;
    float ext = chi[0] - clo[0];
    for (int k = 1; k < 3; ++k) if (chi[k] - clo[k] > ext) { ext = chi[k] - clo[k]; axis = k; }
    int mid = n / 2;
    std::nth_element(idx, idx + mid, idx + n, [&](uint32_t a, uint32_t c) {
        float ca = cent[a * 3 + axis], cc = cent[c * 3 + axis];
        return ca < cc || (ca == cc && a < c);
    });
    int l = (int)bvh.nodes.size();
    bvh.nodes.push_back(BNode{});
    bvh.nodes.push_back(BNode{});
    bvh.nodes[node].left = l;
    bvh.nodes[node].right = l + 1;
    bvh.nodes[node].count = 0;
    build_rec(bvh, boxes, cent, idx, mid, l);
    build_rec(bvh, boxes, cent, idx + mid, n - mid, l + 1);
}

void build_bvh(Bvh& bvh, std::vector<Box>& boxes) {
    int n = (int)boxes.size();
    bvh.nodes.clear();
    bvh.prims.resize(n);
    for (int i = 0; i < n; ++i) bvh.prims[i] = (uint32_t)i;
    std::vector<float> cent(3 * (size_t)std::max(n, 1));
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) cent[i * 3 + k] = 0.5f * (boxes[i].lo[k] + boxes[i].hi[k]);
    bvh.nodes.push_back(BNode{});
    if (n == 0) {
        for (int k = 0; k < 3; ++k) { bvh.nodes[0].lo[k] = 1.0f; bvh.nodes[0].hi[k] = -1.0f; }
        bvh.nodes[0].left = 0; bvh.nodes[0].count = 0; bvh.nodes[0].right = -1;
        return;
    }
    build_rec(bvh, boxes, cent, bvh.prims.data(), n, 0);
}

// Conservative double slab test (culling only; the triangle test decides hits).
bool box_hit(const float lo[3], const float hi[3], const double o[3], const double invd[3], const bool zero[3],
             double tmin, double tmax) {
    double tn = -INFINITY, tf = INFINITY;
    for (int k = 0; k < 3; ++k) {
        if (zero[k]) {
            double pad = 1e-9 * (std::fabs((double)lo[k]) + std::fabs((double)hi[k]) + 1e-30);
            if (o[k] < (double)lo[k] - pad || o[k] > (double)hi[k] + pad) return false;
            continue;
        }
        double t0 = ((double)lo[k] - o[k]) * invd[k];
        double t1 = ((double)hi[k] - o[k]) * invd[k];
        if (t0 > t1) std::swap(t0, t1);
        tn = std::max(tn, t0);
        tf = std::min(tf, t1);
    }
    double m = 1e-9 * (std::fabs(tn) + std::fabs(tf)) + 1e-12;
    if (tn > tf + m) return false;
    if (tf < tmin - m) return false;
    if (tn > tmax + m) return false;
    return true;
}

struct OScene {
    std::vector<f3> pos, nrm;
    std::vector<uint32_t> slot, idx;
    std::vector<GkrtMesh> meshes;
    std::vector<GkrtMaterial> mats;
    std::vector<GkrtInstance> inst;
    std::vector<GkrtLight> lights;
    std::vector<uint32_t> cubes, voxels;
    bool has_probes = false;
    std::vector<Bvh> blas;
    Bvh tlas;
    // emissive-triangle table (GKRT_NEE_EMISSIVE): 20 floats per emitter
    // (p0, w | p1-p0, 0 | p2-p0, 0 | normal, 0 | emission rgba) and its alias table
    std::vector<float> emit;
    std::vector<float> emit_thr;
    std::vector<uint32_t> emit_alias;
    // textured materials: per-vertex texture coordinates and tangents (empty: all zero), and the
    // texture pool by id (RGBA float texels as the sampler returns them)
    std::vector<f2> uv;
    std::vector<f4> tan;
    struct Tex {
        uint32_t w = 0, h = 0;
        std::vector<f4> t;
        float sh[27] = {0.0f};   // spherical-harmonic projection of an RGBA32F texture, else zero
    };
    std::vector<Tex> tex;
};

// 0: every candidate triangle is decided by the FP64 test (the definition itself).
// 1: the FP32 test with certified bounds rejects certain misses first; the outcome is the
//    same, only faster (used for the timed CPU baseline).
int g_fast = 0;

struct HitRec {
    bool hit;
    uint32_t inst, prim;
    double td;
};

struct LocalRay {
    f3 o, d;
    RayShear s;
};

LocalRay to_object(const GkrtInstance& in, f3 o, f3 d) {
    LocalRay r;
    r.o = xform_point(in.world_inv, o);
    r.d = xform_vector(in.world_inv, d);
    r.s = make_shear(r.d);
    return r;
}

void tri_verts(const OScene& S, const GkrtMesh& m, uint32_t prim, f3& v0, f3& v1, f3& v2, uint32_t* vi = nullptr) {
    uint32_t i0 = S.idx[m.index_offset + 3 * prim + 0] + m.vertex_offset;
    uint32_t i1 = S.idx[m.index_offset + 3 * prim + 1] + m.vertex_offset;
    uint32_t i2 = S.idx[m.index_offset + 3 * prim + 2] + m.vertex_offset;
    v0 = S.pos[i0]; v1 = S.pos[i1]; v2 = S.pos[i2];
    if (vi) { vi[0] = i0; vi[1] = i1; vi[2] = i2; }
}

inline bool key_less(double t, uint32_t inst, uint32_t prim, const HitRec& b) {
    if (!b.hit) return true;
    if (t != b.td) return t < b.td;
    if (inst != b.inst) return inst < b.inst;
    return prim < b.prim;
}

// Closest (any=false) or any (any=true) hit of a world ray under the FP64 definition.
HitRec trace(const OScene& S, f3 o, f3 d, float tminf, float tmaxf, bool any, bool brute, uint64_t* tests) {
    HitRec best{false, 0xFFFFFFFFu, 0xFFFFFFFFu, INFINITY};
    const double tmin = tminf, tmax0 = tmaxf;
    auto do_instance = [&](uint32_t ii) -> bool {
        const GkrtInstance& in = S.inst[ii];
        if (!in.visible) return false;
        const GkrtMesh& m = S.meshes[in.mesh_id];
        LocalRay lr = to_object(in, o, d);
        double od[3] = {lr.o.x, lr.o.y, lr.o.z};
        double dd[3] = {lr.d.x, lr.d.y, lr.d.z};
        double inv[3];
        bool zero[3];
        for (int k = 0; k < 3; ++k) { zero[k] = dd[k] == 0.0; inv[k] = zero[k] ? 0.0 : 1.0 / dd[k]; }
        auto test_tri = [&](uint32_t prim) -> bool {
            f3 v0, v1, v2;
            tri_verts(S, m, prim, v0, v1, v2);
            if (tests) ++*tests;
            if (g_fast && fp32_test(lr.o, lr.s, v0, v1, v2).kind == 0) return false;
            ExactHit x = exact_test(lr.o, lr.s, v0, v1, v2);
            if (!x.hit || !(x.t >= tmin && x.t <= tmax0)) return false;
            if (any) { best = HitRec{true, ii, prim, x.t}; return true; }
            if (key_less(x.t, ii, prim, best)) best = HitRec{true, ii, prim, x.t};
            return false;
        };
        uint32_t ntri = m.index_count / 3;
        if (brute) {
            for (uint32_t p = 0; p < ntri; ++p) if (test_tri(p)) return true;
            return false;
        }
        const Bvh& bv = S.blas[in.mesh_id];
        int stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp) {
            const BNode& nd = bv.nodes[stack[--sp]];
            double tcut = best.hit ? best.td : tmax0;
            if (!box_hit(nd.lo, nd.hi, od, inv, zero, tmin, tcut)) continue;
            if (nd.count > 0) {
                for (int i = 0; i < nd.count; ++i)
                    if (test_tri(bv.prims[nd.left + i])) return true;
            } else if (nd.right >= 0) {
                stack[sp++] = nd.left;
                stack[sp++] = nd.right;
            }
        }
        return false;
    };
    if (brute) {
        for (uint32_t ii = 0; ii < S.inst.size(); ++ii)
            if (do_instance(ii)) return best;
        return best;
    }
    double od[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z}, inv[3];
    bool zero[3];
    for (int k = 0; k < 3; ++k) { zero[k] = dd[k] == 0.0; inv[k] = zero[k] ? 0.0 : 1.0 / dd[k]; }
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
        const BNode& nd = S.tlas.nodes[stack[--sp]];
        double tcut = best.hit ? best.td : tmax0;
        if (!box_hit(nd.lo, nd.hi, od, inv, zero, tmin, tcut)) continue;
        if (nd.count > 0) {
            for (int i = 0; i < nd.count; ++i)
                if (do_instance(S.tlas.prims[nd.left + i])) return best;
        } else if (nd.right >= 0) {
            stack[sp++] = nd.left;
            stack[sp++] = nd.right;
        }
    }
    return best;
}

struct Vtx {
    f3 P, N;
    uint32_t mat;
    uint32_t inst;   // instance index
    f2 uv;           // texture coordinates at the hit
    f3 ln;           // object-space normal mix (the LocalNormal of the texture path)
    f4 lt;           // object-space tangent mix, w the packed handedness (LocalTangent)
};

const GkrtMaterial& get_mat(const OScene& S, uint32_t i) {
    uint32_t n = (uint32_t)S.mats.size();
    return S.mats[i < n ? i : n - 1];
}

// FHardwareRayTracerV2::TraceRay (Shading.slang:784-826) on top of trace().
bool trace_ray(const OScene& S, f3 o, f3 d, float tmax, Vtx& out, uint32_t* out_prim, uint64_t* rays) {
    if (rays) ++*rays;
    HitRec h = trace(S, o, d, kEPS, tmax, false, false, nullptr);
    if (!h.hit) return false;
    const GkrtInstance& in = S.inst[h.inst];
    const GkrtMesh& m = S.meshes[in.mesh_id];
    LocalRay lr = to_object(in, o, d);
    f3 v0, v1, v2;
    uint32_t vi[3];
    tri_verts(S, m, h.prim, v0, v1, v2, vi);
    HybridHit hh = hybrid_eval(lr.o, lr.s, v0, v1, v2);
    f3 n0 = S.nrm[vi[0]], n1 = S.nrm[vi[1]], n2 = S.nrm[vi[2]];
    // Mix(n0, n1, n2, bary) = n0 + (n1 - n0) b1 + (n2 - n0) b2
    f3 e1 = sub(n1, n0), e2 = sub(n2, n0);
    f3 nobj = f3{fma_(e2.x, hh.b2, fma_(e1.x, hh.b1, n0.x)), fma_(e2.y, hh.b2, fma_(e1.y, hh.b1, n0.y)),
                 fma_(e2.z, hh.b2, fma_(e1.z, hh.b1, n0.z))};
    out.N = normalize3(xform_normal(in.world_inv, nobj));
    out.P = fma3(d, hh.t, o);
    out.mat = in.mat_id[S.slot[vi[0]] & 15u];
    out.inst = h.inst;
    // the texture path's vertex attributes, each the same barycentric mix
    out.ln = nobj;
    out.uv = f2{0.0f, 0.0f};
    out.lt = f4{0.0f, 0.0f, 0.0f, 0.0f};
    if (!S.uv.empty()) {
        const f2 a = S.uv[vi[0]], b = S.uv[vi[1]], c = S.uv[vi[2]];
        out.uv = f2{fma_(c.x - a.x, hh.b2, fma_(b.x - a.x, hh.b1, a.x)), fma_(c.y - a.y, hh.b2, fma_(b.y - a.y, hh.b1, a.y))};
    }
    if (!S.tan.empty()) {
        f4 a = S.tan[vi[0]], b = S.tan[vi[1]], c = S.tan[vi[2]];
        // the vertex packing of the handedness (MakeVertex, Vertex.hpp:97): 2 when positive, else 0
        a.w = a.w > 0.0f ? 2.0f : 0.0f;
        b.w = b.w > 0.0f ? 2.0f : 0.0f;
        c.w = c.w > 0.0f ? 2.0f : 0.0f;
        out.lt = f4{fma_(c.x - a.x, hh.b2, fma_(b.x - a.x, hh.b1, a.x)), fma_(c.y - a.y, hh.b2, fma_(b.y - a.y, hh.b1, a.y)),
                    fma_(c.z - a.z, hh.b2, fma_(b.z - a.z, hh.b1, a.z)), fma_(c.w - a.w, hh.b2, fma_(b.w - a.w, hh.b1, a.w))};
    }
    if (out_prim) *out_prim = h.prim;
    return true;
}

// ---- textures: the pool's sampler at level 0 (Sampler.hpp:9-27, TextureImage.cpp:24-31):
// Vulkan's linear filter with repeat addressing; weights in FP32 in one fixed order ----
uint32_t wrap_repeat(float f, uint32_t n) {
    float m = std::fmod(f, (float)n);
    if (m < 0.0f) m = m + (float)n;
    const uint32_t i = (uint32_t)m;
    return i < n ? i : 0u;
}
f4 tex_sample(const OScene& S, int id, float u, float v) {
    const f4 white{1.0f, 1.0f, 1.0f, 1.0f};
    if (id < 0 || (size_t)id >= S.tex.size() || S.tex[id].t.empty()) return white;
    const OScene::Tex& t = S.tex[id];
    float x = fma_(u, (float)t.w, -0.5f), y = fma_(v, (float)t.h, -0.5f);
    if (!(std::fabs(x) < 1e30f)) x = -0.5f;
    if (!(std::fabs(y) < 1e30f)) y = -0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float a = x - fx, b = y - fy;
    const uint32_t x0 = wrap_repeat(fx, t.w), x1 = wrap_repeat(fx + 1.0f, t.w);
    const uint32_t y0 = wrap_repeat(fy, t.h), y1 = wrap_repeat(fy + 1.0f, t.h);
    const float ia = 1.0f - a, ib = 1.0f - b;
    const float w00 = ia * ib, w10 = a * ib, w01 = ia * b, w11 = a * b;
    const f4 t00 = t.t[(size_t)y0 * t.w + x0], t10 = t.t[(size_t)y0 * t.w + x1];
    const f4 t01 = t.t[(size_t)y1 * t.w + x0], t11 = t.t[(size_t)y1 * t.w + x1];
    return f4{fma_(t11.x, w11, fma_(t01.x, w01, fma_(t10.x, w10, t00.x * w00))),
              fma_(t11.y, w11, fma_(t01.y, w01, fma_(t10.y, w10, t00.y * w00))),
              fma_(t11.z, w11, fma_(t01.z, w01, fma_(t10.z, w10, t00.z * w00))),
              fma_(t11.w, w11, fma_(t01.w, w01, fma_(t10.w, w10, t00.w * w00)))};
}

bool trace_occlusion(const OScene& S, f3 o, f3 d, uint64_t* rays) {
    if (rays) ++*rays;
    return trace(S, o, d, kEPS, kPT_MAX, true, false, nullptr).hit;
}

// Any hit over [EPS, tmax] (TraceSegment, Shading.slang:759-782).
bool trace_segment(const OScene& S, f3 o, f3 d, float tmax, uint64_t* rays) {
    if (rays) ++*rays;
    return trace(S, o, d, kEPS, tmax, true, false, nullptr).hit;
}

// ---- samplers (Const_Func.slang) ----
void onb(f3 n, f3& b1, f3& b2) {
    float signZ = n.z < 0.0f ? -1.0f : 1.0f;
    float a = -1.0f / (signZ + n.z);
    b2 = f3{(n.x * n.y) * a, fma_(n.y * n.y, a, signZ), -n.y};
    b1 = f3{fma_((signZ * n.x) * n.x, a, 1.0f), signZ * b2.x, -signZ * n.x};
}
// to_world(v, T, B, N) = v.x T + v.y B + v.z N
f3 to_world(f3 v, f3 T, f3 B, f3 N) {
    return f3{fma_(v.z, N.x, fma_(v.y, B.x, v.x * T.x)), fma_(v.z, N.y, fma_(v.y, B.y, v.x * T.y)),
              fma_(v.z, N.z, fma_(v.y, B.z, v.x * T.z))};
}
f3 align_with_normal(f3 ray, f3 n) {
    f3 T, B;
    onb(n, T, B);
    return to_world(ray, T, B, n);
}
f3 hemi1(uint32_t seed[4]) {
    f2 u = rand2(seed);
    float s, c;
    sincos_2pi(u.x, &s, &c);
    float r = std::sqrt(u.y);
    return f3{r * c, r * s, std::sqrt(1.0f - u.y)};
}
f3 cone(uint32_t seed[4], float cos_theta) {
    f2 u = rand2(seed);
    float s, c;
    sincos_2pi(u.x, &s, &c);
    float ct = fma_(u.y, cos_theta - 1.0f, 1.0f);
    float r = std::sqrt(fma_(-ct, ct, 1.0f));
    return f3{r * c, r * s, ct};
}
f2 unit_disk(uint32_t seed[4]) {
    f2 u = rand2(seed);
    float ox = u.x + (u.x - 1.0f), oy = u.y + (u.y - 1.0f);
    const float nz = 1e-35f;
    if ((ox > -nz && ox < nz) && (oy > -nz && oy < nz)) return f2{0.0f, 0.0f};
    const float pi4 = 0.785398163397448309616f;
    float s, c;
    if (std::fabs(ox) > std::fabs(oy)) {
        float th = (pi4 * oy) / ox;
        sincos_poly(th, &s, &c);
        return f2{ox * c, ox * s};
    }
    float th = (pi4 * ox) / oy;
    sincos_poly(th, &s, &c);
    float ct = s;
    return f2{oy * ct, oy * std::sqrt(fma_(-ct, ct, 1.0f))};
}
f3 ggx_vndf(float alpha, f3 wi_, f2 uv) {
    f3 wi = normalize3(f3{wi_.x * alpha, wi_.y * alpha, wi_.z});
    float b = wi.z;
    if (wi_.z > 0.0f) {
        float a = saturate(alpha);
        float lxy = std::sqrt(fma_(wi_.y, wi_.y, wi_.x * wi_.x));
        float awiz_s = (a * wi_.z) / (1.0f + lxy);
        b = b * ((fma_(-a, a, 1.0f)) / fma_(awiz_s, awiz_s, 1.0f));
    }
    float z = fma_(1.0f - uv.y, 1.0f + b, -b);
    float s, c;
    sincos_2pi(uv.x, &s, &c);
    float r = std::sqrt(saturate(fma_(-z, z, 1.0f)));
    f3 o_std = f3{r * c, r * s, z};
    f3 m = add(wi, o_std);
    return normalize3(f3{m.x * alpha, m.y * alpha, m.z});
}
f3 ggx_sampling(uint32_t seed[4], float roughness, f3 n) {
    f3 T, B;
    onb(n, T, B);
    f3 loc = f3{dot3(T, n), dot3(B, n), dot3(n, n)};
    f2 uv = rand2(seed);
    f3 wm = ggx_vndf(roughness * roughness, loc, uv);
    return to_world(wm, T, B, n);
}
float schlick(float cosine, float ri) {
    float r0 = (1.0f - ri) / (1.0f + ri);
    r0 = r0 * r0;
    float x = 1.0f - cosine;
    float p5 = (((x * x) * x) * x) * x;
    return fma_(1.0f - r0, p5, r0);
}

// ---- ambient cube probes (AmbientCube.slang) ----
f4 unpack_rgb10a2(uint32_t p) {
    float r = (float)(p & 0x3FFu) / 1023.0f;
    float g = (float)((p >> 10) & 0x3FFu) / 1023.0f;
    float b = (float)((p >> 20) & 0x3FFu) / 1023.0f;
    return f4{r * 512.0f, g * 512.0f, b * 512.0f, 0.0f * 512.0f};
}
f4 sample_cube_full(const uint32_t* cube, f3 n) {
    float wx = fmax_(n.x, 0.0f), wnx = fmax_(-n.x, 0.0f);
    float wy = fmax_(n.y, 0.0f), wny = fmax_(-n.y, 0.0f);
    float wz = fmax_(n.z, 0.0f), wnz = fmax_(-n.z, 0.0f);
    float sum = ((((wx + wnx) + wy) + wny) + wz) + wnz;
    uint32_t s0 = cube[12], s1 = cube[13];
    float sky = 0.0f;
    sky = sky + (float)(s0 & 0xFFu) * wz;
    sky = sky + (float)((s0 >> 8) & 0xFFu) * wnz;
    sky = sky + (float)((s0 >> 16) & 0xFFu) * wy;
    sky = sky + (float)((s0 >> 24) & 0xFFu) * wny;
    sky = sky + (float)(s1 & 0xFFu) * wx;
    sky = sky + (float)((s1 >> 8) & 0xFFu) * wnx;
    f4 col{0.0f, 0.0f, 0.0f, 0.0f};
    const int order[12] = {10, 11, 8, 9, 6, 7, 4, 5, 2, 3, 0, 1};
    const float w[12] = {wx, wnx, wy, wny, wz, wnz, wx, wnx, wy, wny, wz, wnz};
    for (int i = 0; i < 12; ++i) col = add4(col, scale4(unpack_rgb10a2(cube[order[i]]), w[i]));
    float k = sum > 0.0f ? 1.0f / sum : 1.0f;
    col.x = col.x * k; col.y = col.y * k; col.z = col.z * k;
    sky = sky * k;
    col.w = sky / 255.0f;
    return col;
}
f4 probe_term(const OScene& S, f3 p, f3 n) {
    float npx = (p.x - kCubeOff[0]) / kCubeUnit;
    float npy = (p.y - kCubeOff[1]) / kCubeUnit;
    float npz = (p.z - kCubeOff[2]) / kCubeUnit;
    // !(>=): a NaN position takes the early out (the shader would read undefined probes)
    if (!(npx >= 0.0f) || !(npy >= 0.0f) || !(npz >= 0.0f) || npx > (float)(kCubeXY - 2) || npy > (float)(kCubeZ - 2) ||
        npz > (float)(kCubeXY - 2))
        return f4{0.0f, 0.0f, 0.0f, 1.0f};
    if (!S.has_probes) return f4{0.0f, 0.0f, 0.0f, 0.0f};
    float fx = std::floor(npx), fy = std::floor(npy), fz = std::floor(npz);
    int bx = (int)fx, by = (int)fy, bz = (int)fz;
    float frx = npx - fx, fry = npy - fy, frz = npz - fz;
    float tw = 0.0f;
    f4 res{0.0f, 0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 8; ++i) {
        int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        int px = bx + ox, py = by + oy, pz = bz + oz;
        size_t id = (size_t)py * kCubeXY * kCubeXY + (size_t)pz * kCubeXY + (size_t)px;
        const uint32_t* cube = &S.cubes[id * 14];
        const uint32_t* vox = &S.voxels[id * 4];
        uint32_t u0 = vox[2], u1 = vox[3];
        float d0y = (float)((u0 >> 8) & 0xFFu) / 255.0f;
        float d0z = (float)((u0 >> 16) & 0xFFu) / 255.0f;
        float d0w = (float)((u0 >> 24) & 0xFFu) / 255.0f;
        float d1x = (float)(u1 & 0xFFu) / 255.0f;
        float d1y = (float)((u1 >> 8) & 0xFFu) / 255.0f;
        float d1z = (float)((u1 >> 16) & 0xFFu) / 255.0f;
        float d1w = (float)((u1 >> 24) & 0xFFu) / 255.0f;
        if (d0y < 0.01f) continue;
        f3 pl = f3{frx - (float)ox, fry - (float)oy, frz - (float)oz};
        float dist = length3(pl);
        f3 dir = normalize3(pl);
        float wxp = std::sqrt(fmax_(dir.x, 0.0f)), wxn = std::sqrt(fmax_(-dir.x, 0.0f));
        float wyp = std::sqrt(fmax_(dir.y, 0.0f)), wyn = std::sqrt(fmax_(-dir.y, 0.0f));
        float wzp = std::sqrt(fmax_(dir.z, 0.0f)), wzn = std::sqrt(fmax_(-dir.z, 0.0f));
        float hl = wxp * d1x;
        hl = hl + wxn * d1y;
        hl = hl + wyp * d1z;
        hl = hl + wyn * d1w;
        hl = hl + wzp * d0z;
        hl = hl + wzn * d0w;
        if (dist > hl + 0.05f) continue;
        float wx = ox == 0 ? 1.0f - frx : frx;
        float wy = oy == 0 ? 1.0f - fry : fry;
        float wz = oz == 0 ? 1.0f - frz : frz;
        float wgt = (wx * wy) * wz;
        f4 sc = sample_cube_full(cube, n);
        res = add4(res, scale4(sc, wgt));
        tw = tw + wgt;
    }
    if (tw > 0.0f) return f4{res.x / tw, res.y / tw, res.z / tw, res.w / tw};
    return f4{0.0f, 0.0f, 0.0f, 0.0f};
}

f4 sky_color(const GkrtFrameConstants& fc) {
    if (!fc.has_sky) return f4{0.0f, 0.0f, 0.0f, 0.0f};
    f4 c{fmin_(10.0f, fc.sky_color[0]), fmin_(10.0f, fc.sky_color[1]), fmin_(10.0f, fc.sky_color[2]),
         fmin_(1.0f, fc.sky_color[3])};
    return scale4(c, fc.sky_intensity);
}

// SampleIBLRough (Shading.slang:188-192): EvaluateSH (Shading.slang:150-186) of the sky
// texture's projection at direction n, rotated about y by (1 - SkyRotation) pi, as (rgb, 1)
// times (HasSky ? SkyIntensity : 0). A texture without a projection (8-bit or absent) gives 0.
f4 sky_rough(const OScene& S, const GkrtFrameConstants& fc, f3 n) {
    static const float zero[27] = {0.0f};
    const float* c = fc.sky_index < S.tex.size() ? S.tex[fc.sky_index].sh : zero;
    float sn, cs;
    sincos_2pi((1.0f - fc.sky_rotation) * 0.5f, &sn, &cs);
    const float rx = n.x * cs + n.z * sn, ry = n.y, rz = -n.x * sn + n.z * cs;
    const float b[9] = {0.282095f,
                        -0.488603f * ry,
                        0.488603f * rz,
                        -0.488603f * rx,
                        (1.092548f * rx) * ry,
                        (-1.092548f * ry) * rz,
                        0.315392f * ((3.0f * ry) * ry - 1.0f),
                        (-1.092548f * rx) * rz,
                        0.546274f * (rx * rx - rz * rz)};
    float r = 0.0f, g = 0.0f, bl = 0.0f;
    for (int i = 0; i < 9; ++i) {
        r = r + c[i] * b[i];
        g = g + c[9 + i] * b[i];
        bl = bl + c[18 + i] * b[i];
    }
    return scale4(f4{r, g, bl, 1.0f}, fc.has_sky ? fc.sky_intensity : 0.0f);
}

// A sky miss in direction dir: SampleIBLV2 (Shading.slang:194-199) on texture sky_index when
// the frame asks for it (d = normalize(dir), t = ((atan2(d.x, d.z) + pi rotate) / 2pi,
// acos(d.y) / pi), min((10, 10, 10, 1), sample) x SkyIntensity), else the constant colour.
f4 sky_dir(const OScene& S, const GkrtFrameConstants& fc, f3 dir) {
    if (!fc.has_sky || !(fc.flags & GKRT_FRAME_SKY_TEXTURE)) return sky_color(fc);
    const f3 d = normalize3(dir);
    const float u = (atan2_(d.x, d.z) + 3.14159274f * fc.sky_rotation) * 0.159154937f;
    const float v = acos_(d.y) * 0.318309873f;
    const f4 c = tex_sample(S, (int)fc.sky_index, u, v);
    return scale4(f4{fmin_(10.0f, c.x), fmin_(10.0f, c.y), fmin_(10.0f, c.z), fmin_(1.0f, c.w)}, fc.sky_intensity);
}

// FetchGBufferV2 (Shading.slang:82-112) for the primary vertex: albedo = diffuse x diffuse
// texture, roughness = fuzziness x the MRA texture's green channel, and the normal map through
// mikkTSpace (:74-80) on the vertex's local normal and tangent (the barycentric mixes the
// visibility-buffer caster computes, GeneralFunc.slang:49-51), carried to world space by the
// instance transform and normalized.
void fetch_gbuffer(const OScene& S, const GkrtMaterial& m, Vtx& v, f4& albedo, float& rough) {
    albedo = f4{m.diffuse[0], m.diffuse[1], m.diffuse[2], m.diffuse[3]};
    if (m.diffuse_texture_id >= 0) albedo = mul4(albedo, tex_sample(S, m.diffuse_texture_id, v.uv.x, v.uv.y));
    rough = m.fuzziness;
    if (m.mra_texture_id >= 0) rough = rough * tex_sample(S, m.mra_texture_id, v.uv.x, v.uv.y).y;
    if (m.normal_texture_id >= 0) {
        const f4 t = tex_sample(S, m.normal_texture_id, v.uv.x, v.uv.y);
        const f3 vn{fma_(t.x, 2.0f, -1.0f), fma_(t.y, 2.0f, -1.0f), fma_(t.z, 2.0f, -1.0f)};
        const f3 T{v.lt.x, v.lt.y, v.lt.z};
        const f3 B = mul(cross3(v.ln, T), v.lt.w);
        const f3 nl = normalize3(f3{fma_(vn.z, v.ln.x, fma_(vn.y, B.x, vn.x * T.x)),
                                    fma_(vn.z, v.ln.y, fma_(vn.y, B.y, vn.x * T.y)),
                                    fma_(vn.z, v.ln.z, fma_(vn.y, B.z, vn.x * T.z))});
        v.N = normalize3(xform_vector(S.inst[v.inst].world, nl));
    }
}

// Emissive-triangle NEE (GKRT_NEE_EMISSIVE, no counterpart in the built reference path; the
// estimator of the legacy area-light branch, Scatter.glsl:55-76, with the alias-table pick
// of the light). Samples one point for vertex (P, N) with throughput rc; false when the
// sample cannot contribute (no shadow ray then).
bool nee_sample(const OScene& S, uint32_t seed[4], f3 P, f3 N, f4 rc, f3& o, f3& dir, float& tmax, f4& contrib) {
    const uint32_t n = (uint32_t)S.emit_thr.size();
    const float x = rand1(seed) * (float)n;
    uint32_t i = (uint32_t)x;
    if (i > n - 1u) i = n - 1u;
    const float frac = x - (float)i;
    const uint32_t j = frac < S.emit_thr[i] ? i : S.emit_alias[i];
    const f2 r = rand2(seed);
    const float* g = &S.emit[20 * (size_t)j];
    const float su = std::sqrt(r.x), bs = su * (1.0f - r.y), bt = su * r.y;
    const f3 q{(g[0] + g[4] * bs) + g[8] * bt, (g[1] + g[5] * bs) + g[9] * bt, (g[2] + g[6] * bs) + g[10] * bt};
    o = fma3(N, 0.001f, P);
    const f3 lv = sub(q, o);
    const float d2 = dot3(lv, lv);
    const float dist = std::sqrt(d2);
    if (!(dist > 2e-3f)) return false;
    const float inv = 1.0f / dist;
    dir = f3{lv.x * inv, lv.y * inv, lv.z * inv};
    const float cs = dot3(N, dir);
    if (!(cs > 0.0f)) return false;
    const float cl = std::fabs(dot3(f3{g[12], g[13], g[14]}, dir));
    if (!(cl > 0.0f)) return false;
    const float gm = ((cs * cl) * g[3]) / (d2 * 3.14159265358979323846f);
    const f4 le{g[16], g[17], g[18], g[19]};
    const f4 c = mul4(rc, le);
    contrib = f4{c.x * gm, c.y * gm, c.z * gm, c.w * gm};
    tmax = dist - 1e-3f;
    return true;
}

// Where a vertex's NEE samples go: the sample's accumulator, times the primary albedo when
// the sample's first bounce was metallic (Shading.slang:1159-1171).
struct NeeAcc {
    f4* acc;
    bool metal;
    f4 palb;
};

// FPathTracingRendererV2::GetRayColor (Shading.slang:1003-1082), plus the emissive-triangle
// NEE of its diffuse-lobe vertices when nee is given.
bool get_ray_color(const OScene& S, const GkrtFrameConstants& fc, Vtx& v, f3& dir, f4& color, uint32_t seed[4],
                   bool& hitReflect, bool& hitMetal, uint64_t* rays, const NeeAcc* nee = nullptr) {
    const GkrtMaterial& mat = get_mat(S, v.mat);
    const bool diel = mat.material_model == GKRT_MAT_DIELECTRIC;
    const float startPosOffset = diel ? 0.0f : 1.0f;
    const float roughness = mat.fuzziness;
    const float dotValue = dot3(dir, v.N);
    const bool back = dotValue > 0.0f;
    const f3 outward = back ? neg(v.N) : v.N;
    const float niOverNt = back ? mat.refraction_index2 : (1.0f / mat.refraction_index2);
    const float cosine = dotValue > 0.0f ? mat.refraction_index * dotValue : -dotValue;
    const float reflectProb = schlick(cosine, mat.refraction_index);
    const float metalProb = mat.metalness;
    bool chanceReflect = rand1(seed) < reflectProb;
    bool chanceMetal = rand1(seed) < metalProb;
    bool chanceGGX = chanceReflect || chanceMetal;
    f3 next = chanceGGX ? reflect3(dir, outward) : outward;
    f3 tdir = chanceGGX ? ggx_sampling(seed, std::sqrt(roughness), next) : align_with_normal(hemi1(seed), next);
    hitReflect = chanceGGX;
    hitMetal = chanceMetal;
    if (diel && !chanceReflect) tdir = refract3(dir, outward, niOverNt);
    dir = tdir;
    const bool neeLobe = nee && !S.emit_thr.empty() && !back && !diel && !chanceGGX;
    if (neeLobe) {
        f3 so, sd;
        float stmax;
        f4 contrib;
        if (nee_sample(S, seed, v.P, v.N, color, so, sd, stmax, contrib)) {
            if (nee->metal) contrib = mul4(contrib, nee->palb);
            if (!trace_segment(S, so, sd, stmax, rays)) *nee->acc = add4(*nee->acc, contrib);
        }
    }
    f3 org = fma3(v.N, 0.001f * startPosOffset, v.P);
    Vtx nv;
    if (trace_ray(S, org, tdir, kPT_MAX, nv, nullptr, rays)) {
        v = nv;
        const GkrtMaterial& hm = get_mat(S, v.mat);
        if (neeLobe && hm.material_model == GKRT_MAT_DIFFUSE_LIGHT) {
            color = f4{0.0f, 0.0f, 0.0f, 0.0f};   // this emitter is the NEE's to count
            return true;
        }
        f4 alb{hm.diffuse[0], hm.diffuse[1], hm.diffuse[2], hm.diffuse[3]};
        if (hm.diffuse_texture_id >= 0) alb = mul4(alb, tex_sample(S, hm.diffuse_texture_id, v.uv.x, v.uv.y));
        if (hm.material_model == GKRT_MAT_DIFFUSE_LIGHT || !chanceReflect) color = mul4(color, alb);
        if (back && !diel) {
            color = f4{0.5f, 0.5f, 0.5f, 0.0f};
            return true;
        }
        if (hm.material_model == GKRT_MAT_DIFFUSE_LIGHT) return true;
        return false;
    }
    color = mul4(color, sky_dir(S, fc, tdir));
    return true;
}

inline float* img_f4(void** im, int id, size_t i) { return ((float*)im[id]) + 4 * i; }

struct PixelOut {
    uint64_t rays;
};

// One pixel of Core.PathTracing (Core.PathTracing.comp.slang:7-31).
void shade_pixel(const OScene& S, const GkrtFrameConstants& fc, int W, int H, int x, int y, void** im,
                 uint64_t* rays) {
    const size_t pix = (size_t)y * W + x;
    uint32_t seed[4] = {(uint32_t)x, (uint32_t)y, fc.total_frames, 0u};
    // Util.BufferClear: single-frame targets start at 0 / 100000
    float* sd = img_f4(im, GKRT_IMG_SINGLE_DIFFUSE, pix);
    float* ss = img_f4(im, GKRT_IMG_SINGLE_SPECULAR, pix);
    ss[0] = ss[1] = ss[2] = ss[3] = 0.0f;
    ((float*)im[GKRT_IMG_PREV_DEPTH])[pix] = 100000.0f;
    if (im[GKRT_IMG_HIT_INST]) ((uint32_t*)im[GKRT_IMG_HIT_INST])[pix] = 0xFFFFFFFFu;
    if (im[GKRT_IMG_HIT_PRIM]) ((uint32_t*)im[GKRT_IMG_HIT_PRIM])[pix] = 0xFFFFFFFFu;

    // FHardwarePrimaryRayCaster::TracePrimaryRay
    float uvx = fma_((float)x / (float)W, 2.0f, -1.0f);
    float uvy = fma_((float)y / (float)H, 2.0f, -1.0f);
    if (fc.taa) {
        const float* h = kHalton[fc.total_frames % 8];
        uvx = uvx + (h[0] - 0.5f) / (float)W;
        uvy = uvy + (h[1] - 0.5f) / (float)H;
    }
    f2 disk = unit_disk(seed);
    float ha = fc.aperture / 2.0f;
    f2 off{ha * disk.x, ha * disk.y};
    f4 origin = mat4_mul(fc.model_view_inverse, f4{off.x, off.y, 0.0f, 1.0f});
    f4 target = mat4_mul(fc.projection_inverse, f4{uvx, uvy, 1.0f, 1.0f});
    f3 tv = f3{fma_(target.x, fc.focus_distance, -off.x), fma_(target.y, fc.focus_distance, -off.y),
               target.z * fc.focus_distance};
    f3 tn = normalize3(tv);
    f4 direction = mat4_mul(fc.model_view_inverse, f4{tn.x, tn.y, tn.z, 0.0f});
    f3 o3 = xyz(origin), d3 = xyz(direction);
    f3 primDir = normalize3(d3);
    Vtx pv;
    uint32_t pprim = 0;
    bool hit = trace_ray(S, o3, d3, kPT_MAX, pv, &pprim, rays);

    float* alb = img_f4(im, GKRT_IMG_ALBEDO, pix);
    float* nrm = img_f4(im, GKRT_IMG_NORMAL, pix);
    float* mot = ((float*)im[GKRT_IMG_MOTION]) + 2 * pix;
    uint32_t* oid = (uint32_t*)im[GKRT_IMG_OBJECT_ID];
    uint32_t* mom = (uint32_t*)im[GKRT_IMG_MOTION_MOMENT];
    if (!hit) {
        f4 sky = sky_dir(S, fc, primDir);
        sd[0] = sky.x; sd[1] = sky.y; sd[2] = sky.z; sd[3] = sky.w;
        mot[0] = 0.0f; mot[1] = 0.0f;
        alb[0] = alb[1] = alb[2] = alb[3] = 1.0f;
        nrm[0] = 0.0f; nrm[1] = 1.0f; nrm[2] = 0.0f; nrm[3] = 1.0f;
        oid[pix] = 65535u;
        return;
    }
    if (im[GKRT_IMG_HIT_INST]) ((uint32_t*)im[GKRT_IMG_HIT_INST])[pix] = pv.inst;
    if (im[GKRT_IMG_HIT_PRIM]) ((uint32_t*)im[GKRT_IMG_HIT_PRIM])[pix] = pprim;
    const GkrtInstance& pin = S.inst[pv.inst];
    // PrimaryHit (Shading.slang:1204-1220)
    f4 P4{pv.P.x, pv.P.y, pv.P.z, 1.0f};
    f4 clip = mat4_mul(fc.view_projection, P4);
    float ndcDepth = clip.z / clip.w;
    // CalculateMotionVectorV2 (Shading.slang:50-72)
    f4 ch = mat4_mul(fc.view_projection_unjit, P4);
    float cfx = (ch.x / ch.w) * 0.5f, cfy = (ch.y / ch.w) * 0.5f;
    f3 prevP = xform_point(pin.combined_prev, pv.P);
    f4 ph = mat4_mul(fc.prev_view_projection_unjit, f4{prevP.x, prevP.y, prevP.z, 1.0f});
    float pfx = (ph.x / ph.w) * 0.5f, pfy = (ph.y / ph.w) * 0.5f;
    if (length3(sub(pv.P, prevP)) > 0.02f) mom[pix] = fc.temporal_frames;
    else mom[pix] = mom[pix] > 0u ? mom[pix] - 1u : 0u;
    float mx = pfx - cfx, my = pfy - cfy;
    const GkrtMaterial& pmat = get_mat(S, pv.mat);
    f4 primaryAlbedo;
    float proughness;
    fetch_gbuffer(S, pmat, pv, primaryAlbedo, proughness);
    alb[0] = primaryAlbedo.x; alb[1] = primaryAlbedo.y; alb[2] = primaryAlbedo.z; alb[3] = primaryAlbedo.w;
    nrm[0] = pv.N.x; nrm[1] = pv.N.y; nrm[2] = pv.N.z; nrm[3] = proughness;
    oid[pix] = pin.instance_id;
    mot[0] = mx * (float)W; mot[1] = my * (float)H;
    ((float*)im[GKRT_IMG_PREV_DEPTH])[pix] = ndcDepth;
    if (pmat.material_model != GKRT_MAT_DIELECTRIC) pv.P = fma3(primDir, -0.03f, pv.P);

    // Render (Shading.slang:1084-1184)
    const int mult = mom[pix] > 0u ? 4 : 1;
    f4 fcol{0.0f, 0.0f, 0.0f, 0.0f}, frefl{0.0f, 0.0f, 0.0f, 0.0f};
    if (pmat.material_model == GKRT_MAT_DIFFUSE_LIGHT) {
        sd[0] = pmat.diffuse[0]; sd[1] = pmat.diffuse[1]; sd[2] = pmat.diffuse[2]; sd[3] = pmat.diffuse[3];
        return;
    }
    const bool pdiel = pmat.material_model == GKRT_MAT_DIELECTRIC;
    int samples = (int)fc.number_of_samples * mult;
    if (samples < 1) samples = 1;
    f4 eye = mat4_mul(fc.model_view_inverse, f4{0.0f, 0.0f, 0.0f, 1.0f});
    const uint32_t maxB = pdiel ? fc.max_number_of_bounces : fc.number_of_bounces;
    for (int i = 0; i < samples; ++i) {
        f4 rc{1.0f, 1.0f, 1.0f, 1.0f};
        f3 dir = normalize3(sub(pv.P, xyz(eye)));
        Vtx vs = pv;
        bool hitReflect = false, hitMetal = false;
        const bool nee_on = fc.nee_mode == GKRT_NEE_EMISSIVE;
        // a first-vertex NEE sample exists only for a diffuse first bounce: accumulator fcol
        const NeeAcc nee_first{&fcol, false, primaryAlbedo};
        bool exitFirst = get_ray_color(S, fc, vs, dir, rc, seed, hitReflect, hitMetal, rays,
                                       nee_on ? &nee_first : nullptr);
        const NeeAcc nee_rest{hitReflect ? &frefl : &fcol, hitMetal, primaryAlbedo};
        if (!exitFirst) {
            if (fc.fast_gather && !pdiel) {
                rc = mul4(rc, probe_term(S, vs.P, vs.N));
            } else {
                for (uint32_t b = 1; b < maxB; ++b) {
                    bool dc = false;
                    if (get_ray_color(S, fc, vs, dir, rc, seed, dc, dc, rays, nee_on ? &nee_rest : nullptr)) break;
                    if (fc.has_sun && rand1(seed) < 0.5f) {
                        f3 sun = f3{fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]};
                        f3 cd = align_with_normal(cone(seed, kCosQuarterDeg), sun);
                        if (!trace_occlusion(S, vs.P, cd, rays)) {
                            rc = mul4(rc, f4{fc.sun_color[0], fc.sun_color[1], fc.sun_color[2], fc.sun_color[3]});
                            break;
                        }
                    }
                    const bool early = !pdiel && rand1(seed) < 0.5f;
                    if (b == maxB - 1 || early) {
                        rc = mul4(rc, probe_term(S, vs.P, vs.N));
                        break;
                    }
                }
            }
        }
        if (hitMetal) rc = mul4(rc, primaryAlbedo);
        if (hitReflect) frefl = add4(frefl, rc);
        else fcol = add4(fcol, rc);
    }
    const float fs = (float)samples;
    fcol = f4{fcol.x / fs, fcol.y / fs, fcol.z / fs, fcol.w / fs};
    frefl = f4{frefl.x / fs, frefl.y / fs, frefl.z / fs, frefl.w / fs};
    // FHardwareDirectIlluminatorV2 (Shading.slang:886-908)
    f3 sun = f3{fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]};
    float dd = fmax_(dot3(sun, normalize3(pv.N)), 0.0f) * kM_1_PI;
    float shadow = 0.0f;
    if (fc.has_sun) {
        f3 cd = align_with_normal(cone(seed, kCosQuarterDeg), sun);
        shadow = 1.0f;
        if (trace_occlusion(S, pv.P, cd, rays)) shadow = 0.0f;
    }
    f4 dc{(fc.sun_color[0] * dd) * shadow, (fc.sun_color[1] * dd) * shadow, (fc.sun_color[2] * dd) * shadow,
          (fc.sun_color[3] * dd) * shadow};
    fcol = add4(fcol, dc);
    sd[0] = fcol.x; sd[1] = fcol.y; sd[2] = fcol.z; sd[3] = fcol.w;
    ss[0] = frefl.x; ss[1] = frefl.y; ss[2] = frefl.z; ss[3] = frefl.w;
}

// ---- reprojection (Process.ReProject.comp.slang) ----
struct Img {
    int W, H;
    bool in(int x, int y) const { return x >= 0 && y >= 0 && x < W && y < H; }
};
inline f4 ld4(const float* p, const Img& g, int x, int y) {
    if (!g.in(x, y)) return f4{0.0f, 0.0f, 0.0f, 0.0f};
    const float* q = p + 4 * ((size_t)y * g.W + x);
    return f4{q[0], q[1], q[2], q[3]};
}
inline f2 ld2(const float* p, const Img& g, int x, int y) {
    if (!g.in(x, y)) return f2{0.0f, 0.0f};
    const float* q = p + 2 * ((size_t)y * g.W + x);
    return f2{q[0], q[1]};
}
inline uint32_t ldu(const uint32_t* p, const Img& g, int x, int y) {
    if (!g.in(x, y)) return 0u;
    return p[(size_t)y * g.W + x];
}
inline float lerp_(float a, float b, float t) { return fma_(t, b - a, a); }
inline f3 lerp3(f3 a, f3 b, float t) { return f3{lerp_(a.x, b.x, t), lerp_(a.y, b.y, t), lerp_(a.z, b.z, t)}; }
inline f4 lerp4(f4 a, f4 b, float t) {
    return f4{lerp_(a.x, b.x, t), lerp_(a.y, b.y, t), lerp_(a.z, b.z, t), lerp_(a.w, b.w, t)};
}

float calc_weight(float cd, bool same, bool center, f3 n, f3 cn) {
    if (center) return 0.4f;
    if (!same) return 0.0f;
    float nd = saturate(dot3(n, cn));
    const float th = 0.98f;
    if (nd < th) return 0.0f;
    float nw = (nd - th) / (1.0f - th);
    return (nw * 2.0f) / fma_(cd, 1.5f, 4.0f);
}

f3 filter_history(const float* prev, const Img& g, f2 sub, int px, int py, uint32_t cur, uint32_t p0, uint32_t p1,
                  uint32_t p2, uint32_t p3, f4 cs) {
    f3 c = xyz(cs);
    f3 h0 = cur == p0 ? xyz(ld4(prev, g, px, py)) : c;
    f3 h1 = cur == p1 ? xyz(ld4(prev, g, px + 1, py)) : c;
    f3 h2 = cur == p2 ? xyz(ld4(prev, g, px, py + 1)) : c;
    f3 h3 = cur == p3 ? xyz(ld4(prev, g, px + 1, py + 1)) : c;
    f3 h = lerp3(lerp3(h0, h1, sub.x), lerp3(h2, h3, sub.x), sub.y);
    auto cl = [](float v) { return v < 0.0f ? 0.0f : (v > 1600.0f ? 1600.0f : v); };
    return f3{cl(h.x), cl(h.y), cl(h.z)};
}

void reproject_pixel(const GkrtFrameConstants& fc, int W, int H, int x, int y, void** im) {
    Img g{W, H};
    const size_t pix = (size_t)y * W + x;
    const float* SD = (const float*)im[GKRT_IMG_SINGLE_DIFFUSE];
    const float* SS = (const float*)im[GKRT_IMG_SINGLE_SPECULAR];
    const float* SA = (const float*)im[GKRT_IMG_ALBEDO];
    const float* PD = (const float*)im[GKRT_IMG_PREV_DIFFUSE];
    const float* PS = (const float*)im[GKRT_IMG_PREV_SPECULAR];
    const float* PA = (const float*)im[GKRT_IMG_PREV_ALBEDO];
    float* AD = (float*)im[GKRT_IMG_ACCUM_DIFFUSE];
    float* AS = (float*)im[GKRT_IMG_ACCUM_SPECULAR];
    float* AA = (float*)im[GKRT_IMG_ACCUM_ALBEDO];
    const uint32_t* ID0 = (const uint32_t*)im[GKRT_IMG_OBJECT_ID];
    const uint32_t* ID1 = (const uint32_t*)im[GKRT_IMG_OBJECT_ID_PREV];
    const float* MV = (const float*)im[GKRT_IMG_MOTION];
    const float* NB = (const float*)im[GKRT_IMG_NORMAL];
    const uint32_t* MM = (const uint32_t*)im[GKRT_IMG_MOTION_MOMENT];
    auto st = [&](float* dst, f4 v) { float* q = dst + 4 * pix; q[0] = v.x; q[1] = v.y; q[2] = v.z; q[3] = v.w; };
    if (fc.progressive_render) {
        const float k = 1.0f / 512.0f;
        st(AD, lerp4(ld4(PD, g, x, y), ld4(SD, g, x, y), k));
        st(AS, lerp4(ld4(PS, g, x, y), ld4(SS, g, x, y), k));
        st(AA, lerp4(ld4(PA, g, x, y), ld4(SA, g, x, y), k));
        return;
    }
    f4 cd = ld4(SD, g, x, y), cs = ld4(SS, g, x, y), ca = ld4(SA, g, x, y);
    f2 mv = ld2(MV, g, x, y);
    float fxm = (float)x + mv.x, fym = (float)y + mv.y;
    float flx = std::floor(fxm), fly = std::floor(fym);
    int px = (int)flx, py = (int)fly;
    bool inside = px < W && py < H && px >= -1 && py >= -1;
    uint32_t cur = ldu(ID0, g, x, y);
    uint32_t p0 = ldu(ID1, g, px, py);
    bool miss = cur == 65535u;
    uint32_t moment = ldu(MM, g, x, y);
    bool use = !(miss || !inside || moment > 0u);
    if (!use) {
        st(AD, cd); st(AS, cs); st(AA, ca);
        return;
    }
    f3 cn = xyz(ld4(NB, g, x, y));
    f4 sdiff{0, 0, 0, 0}, sspec{0, 0, 0, 0};
    float tw = 0.0f, mir = 0.0f;
    for (int oy = -2; oy <= 2; ++oy) {
        for (int ox = -2; ox <= 2; ++ox) {
            int sx = x + ox, sy = y + oy;
            uint32_t pid = ldu(ID0, g, sx, sy);
            f3 wn = xyz(ld4(NB, g, sx, sy));
            bool center = ox == 0 && oy == 0;
            bool same = pid == cur;
            float fox = (float)ox, foy = (float)oy;
            float cdist = std::sqrt(fma_(foy, foy, fox * fox));
            float w = calc_weight(cdist, same, center, wn, cn);
            sdiff = add4(sdiff, scale4(ld4(SD, g, sx, sy), w));
            sspec = add4(sspec, scale4(ld4(SS, g, sx, sy), w));
            tw = tw + w;
            f2 m2 = ld2(MV, g, x + 2 * ox, y + 2 * oy);
            mir = mir + std::sqrt(fma_(m2.y, m2.y, m2.x * m2.x));
        }
    }
    sdiff = f4{sdiff.x / tw, sdiff.y / tw, sdiff.z / tw, sdiff.w / tw};
    sspec = f4{sspec.x / tw, sspec.y / tw, sspec.z / tw, sspec.w / tw};
    uint32_t p1 = ldu(ID1, g, px + 1, py), p2 = ldu(ID1, g, px, py + 1), p3 = ldu(ID1, g, px + 1, py + 1);
    if (std::fabs(mir) < 0.1f) { p0 = cur; p1 = cur; p2 = cur; p3 = cur; }
    f2 sub{fxm - flx, fym - fly};
    f3 hd = filter_history(PD, g, sub, px, py, cur, p0, p1, p2, p3, sdiff);
    f3 hs = filter_history(PS, g, sub, px, py, cur, p0, p1, p2, p3, sspec);
    f3 ha = filter_history(PA, g, sub, px, py, cur, p0, p1, p2, p3, ca);
    float tf = (float)(fc.temporal_frames > 1u ? fc.temporal_frames : 1u);
    float keep = saturate(1.0f / tf);
    f3 od = lerp3(hd, xyz(cd), keep), os = lerp3(hs, xyz(cs), keep), oa = lerp3(ha, xyz(ca), keep);
    st(AD, f4{od.x, od.y, od.z, ld4(PD, g, x, y).w});
    st(AS, f4{os.x, os.y, os.z, ld4(PS, g, x, y).w});
    st(AA, f4{oa.x, oa.y, oa.z, ld4(PA, g, x, y).w});
}

// ---- compose / denoise (Process.DenoiseJBF.comp.slang, tonemaps Const_Func.slang:51-126) ----
float gt_tonemap(float x) {
    const float P = 1.0f, a = 0.7f, m = 0.22f, l = 0.4f, c = 1.33f, b = 0.0f;
    const float e = 2.71828f;
    float l0 = ((P - m) * l) / a;
    float L0 = m - m / a;
    (void)L0;
    float L_x = m + a * (x - m);
    float T_x = m * std::pow(x / m, c) + b;
    float S0 = m + l0;
    float S1 = m + a * l0;
    float C2 = (a * P) / (P - S1);
    float S_x = P - (P - S1) * std::pow(e, -((C2 * (x - S0)) / P));
    auto Wf = [](float v, float e0, float e1) {
        if (v <= e0) return 0.0f;
        if (v >= e1) return 1.0f;
        float q = (v - e0) / (e1 - e0);
        return (q * q) * (3.0f - 2.0f * q);
    };
    auto Hf = [](float v, float e0, float e1) {
        if (v <= e0) return 0.0f;
        if (v >= e1) return 1.0f;
        return (v - e0) / (e1 - e0);
    };
    float w0 = 1.0f - Wf(x, 0.0f, m);
    float w2 = Hf(x, m + l0, m + l0);
    float w1 = (1.0f - w0) - w2;
    return (T_x * w0 + L_x * w1) + S_x * w2;
}
f3 pq_encode(f3 lin) {
    const float m1 = 0.1593017578125f, m2 = 78.84375f, c1 = 0.8359375f, c2 = 18.8515625f, c3 = 18.6875f;
    const float C = 10000.0f;
    float in[3] = {lin.x / C, lin.y / C, lin.z / C}, out[3];
    for (int k = 0; k < 3; ++k) {
        float Lm = std::pow(in[k], m1);
        float N1 = c1 + c2 * Lm;
        float N2 = 1.0f + c3 * Lm;
        float N = N1 * (1.0f / N2);
        out[k] = std::pow(N, m2);
    }
    return f3{out[0], out[1], out[2]};
}

const f3 kLumW{0.212671f, 0.715160f, 0.072169f};

// Compose tail shared by both denoisers: linear output and the tone map
// (Process.DenoiseJBF.comp.slang:170-181).
void write_composed(const GkrtFrameConstants& fc, size_t pix, f3 total, void** im) {
    float* lin = img_f4(im, GKRT_IMG_DENOISED_LINEAR, pix);
    lin[0] = total.x; lin[1] = total.y; lin[2] = total.z; lin[3] = 1.0f;
    float* out = img_f4(im, GKRT_IMG_DENOISED, pix);
    if (fc.hdr) {
        f3 t = f3{total.x / 2000.0f, total.y / 2000.0f, total.z / 2000.0f};
        t = f3{gt_tonemap(t.x) * 2000.0f, gt_tonemap(t.y) * 2000.0f, gt_tonemap(t.z) * 2000.0f};
        float k = fc.paper_white_nit / 230.0f;
        f3 pq = pq_encode(f3{t.x * k, t.y * k, t.z * k});
        out[0] = pq.x; out[1] = pq.y; out[2] = pq.z; out[3] = 1.0f;
    } else {
        float k = fc.paper_white_nit / 40000.0f;
        out[0] = gt_tonemap(total.x * k);
        out[1] = gt_tonemap(total.y * k);
        out[2] = gt_tonemap(total.z * k);
        out[3] = 1.0f;
    }
}

// Edge-aware a-trous pass (no counterpart in the reference; the definition the GPU filter
// implements): 5 x 5 taps at step s with B3-spline weights (1/16, 1/4, 3/8, 1/4, 1/16)
// per axis, times max(0, n_p . n_q)^16, times exp(-|L_p - L_q| / sigma_L); taps outside the
// image or on another object id get weight 0. The last pass remodulates and tone maps.
float b3w(int k) { return k == 0 ? 0.375f : (k == 1 ? 0.25f : 0.0625f); }
float pow16(float v) { float a = v * v; a = a * a; a = a * a; return a * a; }
void atrous_pixel(const GkrtFrameConstants& fc, int W, int H, int x, int y, int step, const float* in, float* out,
                  bool last, void** im) {
    Img g{W, H};
    const size_t pix = (size_t)y * W + x;
    const float* NB = (const float*)im[GKRT_IMG_NORMAL];
    const uint32_t* ID = (const uint32_t*)im[GKRT_IMG_OBJECT_ID];
    const f3 lw{0.212671f, 0.715160f, 0.072169f};
    const f4 cp = ld4(in, g, x, y);
    const f3 np = xyz(ld4(NB, g, x, y));
    const uint32_t idp = ldu(ID, g, x, y);
    const float lp = dot3(xyz(cp), lw);
    const float inv_sl = 1.0f / fmax_(fc.bf_sigma_lum, 1e-4f);
    f3 sum{0.0f, 0.0f, 0.0f};
    float wsum = 0.0f;
    for (int dy = -2; dy <= 2; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
            const int qx = x + dx * step, qy = y + dy * step;
            if (!g.in(qx, qy)) continue;
            if (ldu(ID, g, qx, qy) != idp) continue;
            const f4 cq = ld4(in, g, qx, qy);
            const float wn = pow16(fmax_(dot3(np, xyz(ld4(NB, g, qx, qy))), 0.0f));
            const float wl = std::exp(-(std::fabs(lp - dot3(xyz(cq), lw)) * inv_sl));
            const float w = ((b3w(dx < 0 ? -dx : dx) * b3w(dy < 0 ? -dy : dy)) * wn) * wl;
            sum = add(sum, mul(xyz(cq), w));
            wsum = wsum + w;
        }
    const f3 f{sum.x / wsum, sum.y / wsum, sum.z / wsum};
    if (!last) {
        float* q = out + 4 * pix;
        q[0] = f.x; q[1] = f.y; q[2] = f.z; q[3] = cp.w;
        return;
    }
    const f3 al = xyz(ld4((const float*)im[GKRT_IMG_ACCUM_ALBEDO], g, x, y));
    const f3 sp = xyz(ld4((const float*)im[GKRT_IMG_ACCUM_SPECULAR], g, x, y));
    write_composed(fc, pix, f3{fma_(f.x, al.x, sp.x), fma_(f.y, al.y, sp.y), fma_(f.z, al.z, sp.z)}, im);
}

void denoise_pixel(const GkrtFrameConstants& fc, int W, int H, int x, int y, void** im) {
    Img g{W, H};
    const size_t pix = (size_t)y * W + x;
    const float* AD = (const float*)im[GKRT_IMG_ACCUM_DIFFUSE];
    const float* AS = (const float*)im[GKRT_IMG_ACCUM_SPECULAR];
    const float* AA = (const float*)im[GKRT_IMG_ACCUM_ALBEDO];
    f3 total{0, 0, 0};
    const f3 eps{0.001f, 0.001f, 0.001f};
    if (fc.bf_size > 0u) {
        f3 cc = add(xyz(ld4(AD, g, x, y)), eps);
        f3 cspec = add(xyz(ld4(AS, g, x, y)), eps);
        float clum = dot3(cc, kLumW);
        const float sigma = fc.bf_sigma, sigmaL = fc.bf_sigma_lum * 100.0f;
        const float den_s = (2.0f * sigma) * sigma, den_l = (2.0f * sigmaL) * sigmaL;
        float wsum = 0.0f;
        for (int i = -5; i <= 5; i += 2) {
            for (int j = -5; j <= 5; j += 2) {
                f3 ci = add(xyz(ld4(AD, g, x + j, y + i)), eps);
                float lumi = dot3(ci, kLumW);
                float dist = saturate((float)(i * i + j * j) / 25.0f);
                float dl = (clum - lumi) * (clum - lumi);
                float Fi = std::exp(-(dist * dist) / den_s);
                float Li = std::exp(-(dl * dl) / den_l);
                total = add(total, mul(mul(ci, Fi), Li));
                wsum = wsum + Fi * Li;
            }
        }
        total = f3{total.x / wsum, total.y / wsum, total.z / wsum};
        f3 a = xyz(ld4(AA, g, x, y));
        total = f3{fma_(total.x, a.x, cspec.x), fma_(total.y, a.y, cspec.y), fma_(total.z, a.z, cspec.z)};
    } else {
        f3 d = xyz(ld4(AD, g, x, y)), s = xyz(ld4(AS, g, x, y)), a = xyz(ld4(AA, g, x, y));
        total = f3{fma_(d.x, a.x, s.x), fma_(d.y, a.y, s.y), fma_(d.z, a.z, s.z)};
    }
    write_composed(fc, pix, total, im);
}

// Emissive-triangle table and alias table (Walker's method, Vose's construction): entries in
// the order instance, material slot 0..15, triangle; pick probability power / total with
// power = area x luminance of the emission; w = area / probability = total / luminance.
void build_emitters(OScene& S) {
    std::vector<float> power, lum;
    for (const GkrtInstance& in : S.inst) {
        if (!in.visible) continue;
        const GkrtMesh& m = S.meshes[in.mesh_id];
        for (int slot = 0; slot < 16; ++slot) {
            if (in.mat_id[slot] >= S.mats.size()) continue;
            const GkrtMaterial& mt = S.mats[in.mat_id[slot]];
            if (mt.material_model != GKRT_MAT_DIFFUSE_LIGHT) continue;
            const float l = (0.2126f * mt.diffuse[0] + 0.7152f * mt.diffuse[1]) + 0.0722f * mt.diffuse[2];
            if (!(l > 0.0f)) continue;
            for (uint32_t t = 0; t < m.index_count / 3; ++t) {
                if ((S.slot[S.idx[m.index_offset + 3 * t] + m.vertex_offset] & 15u) != (uint32_t)slot) continue;
                float w[3][3];
                for (int v = 0; v < 3; ++v) {
                    const f3 p = S.pos[S.idx[m.index_offset + 3 * t + v] + m.vertex_offset];
                    for (int r = 0; r < 3; ++r)
                        w[v][r] = ((in.world[4 * r] * p.x + in.world[4 * r + 1] * p.y) + in.world[4 * r + 2] * p.z) +
                                  in.world[4 * r + 3];
                }
                float e1[3], e2[3];
                for (int r = 0; r < 3; ++r) { e1[r] = w[1][r] - w[0][r]; e2[r] = w[2][r] - w[0][r]; }
                const float cx = e1[1] * e2[2] - e1[2] * e2[1], cy = e1[2] * e2[0] - e1[0] * e2[2],
                            cz = e1[0] * e2[1] - e1[1] * e2[0];
                const float len = std::sqrt((cx * cx + cy * cy) + cz * cz);
                const float area = 0.5f * len;
                if (!(area > 0.0f) || !std::isfinite(area)) continue;
                const float inv = 1.0f / len;
                const float e[20] = {w[0][0], w[0][1], w[0][2], 0.0f, e1[0], e1[1], e1[2], 0.0f,
                                     e2[0], e2[1], e2[2], 0.0f, cx * inv, cy * inv, cz * inv, 0.0f,
                                     mt.diffuse[0], mt.diffuse[1], mt.diffuse[2], mt.diffuse[3]};
                S.emit.insert(S.emit.end(), e, e + 20);
                power.push_back(area * l);
                lum.push_back(l);
            }
        }
    }
    const size_t n = power.size();
    if (n == 0) return;
    double total = 0.0;
    for (size_t j = 0; j < n; ++j) total += (double)power[j];
    for (size_t j = 0; j < n; ++j) S.emit[20 * j + 3] = (float)(total / (double)lum[j]);
    std::vector<double> q(n);
    std::vector<size_t> under, over;
    for (size_t j = 0; j < n; ++j) {
        q[j] = (double)power[j] * (double)n / total;
        if (q[j] < 1.0) under.push_back(j);
        else over.push_back(j);
    }
    S.emit_thr.assign(n, 1.0f);
    S.emit_alias.resize(n);
    for (size_t j = 0; j < n; ++j) S.emit_alias[j] = (uint32_t)j;
    while (!under.empty() && !over.empty()) {
        const size_t a = under.back(), b = over.back();
        under.pop_back();
        over.pop_back();
        S.emit_thr[a] = (float)q[a];
        S.emit_alias[a] = (uint32_t)b;
        q[b] = (q[b] + q[a]) - 1.0;
        if (q[b] < 1.0) under.push_back(b);
        else over.push_back(b);
    }
}


// ---- differentiable rendering (path replay): restatement of the GPU adjoint ----
// The paths are built with the same FP32 operations as the forward estimator; the derivative
// terms (products of the other factors, score terms) and their sums are FP64.
struct AdjFactor {
    f4 f;
    uint32_t mat;
};
struct AdjPath {
    std::vector<AdjFactor> fac;
    std::vector<std::pair<uint32_t, double>> ggx;   // (material, d log p / d a)
    f4 rest{1.0f, 1.0f, 1.0f, 1.0f};
};

float ggx_terms(float a, float c) {   // a^2 (1 + a^2) / (c^2 (a^2 - 1) + 1)^2
    const float a2 = a * a;
    const float q = fma_(c * c, a2 - 1.0f, 1.0f);
    return (a2 * (1.0f + a2)) / (q * q);
}
double ggx_score_d(double a, double c) {
    const double a2 = a * a, c2 = c * c;
    return 2.0 / a + 2.0 * a / (1.0 + a2) - 4.0 * a * c2 / (c2 * (a2 - 1.0) + 1.0);
}

bool adj_ray_color(const OScene& S, const GkrtFrameConstants& fc, const float* sample_rough, Vtx& v, f3& dir,
                   f4& color, uint32_t seed[4], bool first, bool& hitReflect, bool& hitMetal, AdjPath& R,
                   uint64_t* rays) {
    const GkrtMaterial& mat = get_mat(S, v.mat);
    const bool diel = mat.material_model == GKRT_MAT_DIELECTRIC;
    const float startPosOffset = diel ? 0.0f : 1.0f;
    const float dotValue = dot3(dir, v.N);
    const bool back = dotValue > 0.0f;
    const f3 outward = back ? neg(v.N) : v.N;
    const float niOverNt = back ? mat.refraction_index2 : (1.0f / mat.refraction_index2);
    const float cosine = dotValue > 0.0f ? mat.refraction_index * dotValue : -dotValue;
    const float reflectProb = schlick(cosine, mat.refraction_index);
    const bool chanceReflect = rand1(seed) < reflectProb;
    const bool chanceMetal = rand1(seed) < mat.metalness;
    const bool chanceGGX = chanceReflect || chanceMetal;
    f3 tdir;
    float c = 0.0f, a_s = 0.0f;
    if (chanceGGX) {
        const f3 axis = reflect3(dir, outward);
        const uint32_t nm = (uint32_t)S.mats.size();
        const float fs = sample_rough ? sample_rough[v.mat < nm ? v.mat : nm - 1] : mat.fuzziness;
        const float r = std::sqrt(fs);
        a_s = r * r;
        tdir = ggx_sampling(seed, r, axis);
        c = dot3(axis, tdir);
    } else {
        tdir = align_with_normal(hemi1(seed), outward);
    }
    if (first) { hitReflect = chanceGGX; hitMetal = chanceMetal; }
    const bool refracted = diel && !chanceReflect;
    if (refracted) tdir = refract3(dir, outward, niOverNt);
    if (chanceGGX && !refracted && a_s > 1e-6f) {
        const float re = std::sqrt(mat.fuzziness);
        const float a_e = re * re;
        if (a_e != a_s) {
            const float w = ggx_terms(a_e, c) / ggx_terms(a_s, c);
            color = f4{color.x * w, color.y * w, color.z * w, color.w * w};
            R.rest = f4{R.rest.x * w, R.rest.y * w, R.rest.z * w, R.rest.w * w};
        }
        R.ggx.push_back({v.mat, a_e > 1e-6f ? ggx_score_d((double)a_e, (double)c) : 0.0});
    }
    dir = tdir;
    const f3 org = fma3(v.N, 0.001f * startPosOffset, v.P);
    Vtx nv;
    if (trace_ray(S, org, tdir, kPT_MAX, nv, nullptr, rays)) {
        v = nv;
        const GkrtMaterial& hm = get_mat(S, v.mat);
        const f4 alb{hm.diffuse[0], hm.diffuse[1], hm.diffuse[2], hm.diffuse[3]};
        if (hm.material_model == GKRT_MAT_DIFFUSE_LIGHT || !chanceReflect) {
            color = mul4(color, alb);
            R.fac.push_back({alb, v.mat});
        }
        if (back && !diel) {
            color = f4{0.5f, 0.5f, 0.5f, 0.0f};
            R.fac.clear();
            R.ggx.clear();
            R.rest = color;
            return true;
        }
        return hm.material_model == GKRT_MAT_DIFFUSE_LIGHT;
    }
    const f4 sk = sky_color(fc);
    color = mul4(color, sk);
    R.rest = mul4(R.rest, sk);
    return true;
}

// One pixel: image (composed radiance) and, when dimg is given, the gradient sums.
void adjoint_pixel(const OScene& S, const GkrtFrameConstants& fc, int W, int H, int x, int y, uint32_t spp,
                   const float* sample_rough, float* img, const float* dimg, double* ga, double* gr, uint64_t* rays) {
    uint32_t seed[4] = {(uint32_t)x, (uint32_t)y, fc.total_frames, 0u};
    float uvx = fma_((float)x / (float)W, 2.0f, -1.0f);
    float uvy = fma_((float)y / (float)H, 2.0f, -1.0f);
    if (fc.taa) {
        const float* h = kHalton[fc.total_frames % 8];
        uvx = uvx + (h[0] - 0.5f) / (float)W;
        uvy = uvy + (h[1] - 0.5f) / (float)H;
    }
    f2 disk = unit_disk(seed);
    float ha = fc.aperture / 2.0f;
    f2 off{ha * disk.x, ha * disk.y};
    f4 origin = mat4_mul(fc.model_view_inverse, f4{off.x, off.y, 0.0f, 1.0f});
    f4 target = mat4_mul(fc.projection_inverse, f4{uvx, uvy, 1.0f, 1.0f});
    f3 tv = f3{fma_(target.x, fc.focus_distance, -off.x), fma_(target.y, fc.focus_distance, -off.y),
               target.z * fc.focus_distance};
    f3 tn = normalize3(tv);
    f4 direction = mat4_mul(fc.model_view_inverse, f4{tn.x, tn.y, tn.z, 0.0f});
    f3 o3 = xyz(origin), d3 = xyz(direction);
    Vtx pv;
    const size_t pix = (size_t)y * W + x;
    float* out = img ? img + 4 * pix : nullptr;
    if (!trace_ray(S, o3, d3, kPT_MAX, pv, nullptr, rays)) {
        const f4 sk = sky_color(fc);
        if (out) { out[0] = sk.x; out[1] = sk.y; out[2] = sk.z; out[3] = 1.0f; }
        return;
    }
    const GkrtMaterial& pm = get_mat(S, pv.mat);
    if (pm.material_model != GKRT_MAT_DIELECTRIC) pv.P = fma3(normalize3(d3), -0.03f, pv.P);
    if (pm.material_model == GKRT_MAT_DIFFUSE_LIGHT) {
        if (out) { out[0] = pm.diffuse[0]; out[1] = pm.diffuse[1]; out[2] = pm.diffuse[2]; out[3] = 1.0f; }
        return;
    }
    const bool pdiel = pm.material_model == GKRT_MAT_DIELECTRIC;
    const uint32_t maxB = pdiel ? fc.max_number_of_bounces : fc.number_of_bounces;
    const f4 eye = mat4_mul(fc.model_view_inverse, f4{0.0f, 0.0f, 0.0f, 1.0f});
    const f4 ap{pm.diffuse[0], pm.diffuse[1], pm.diffuse[2], pm.diffuse[3]};
    const double g[3] = {dimg ? dimg[4 * pix] : 0.0, dimg ? dimg[4 * pix + 1] : 0.0, dimg ? dimg[4 * pix + 2] : 0.0};
    const uint32_t nm = (uint32_t)S.mats.size();
    f4 fcol{0.0f, 0.0f, 0.0f, 0.0f}, frefl{0.0f, 0.0f, 0.0f, 0.0f};
    for (uint32_t i = 0; i < spp; ++i) {
        AdjPath R;
        f4 rc{1.0f, 1.0f, 1.0f, 1.0f};
        f3 dir = normalize3(sub(pv.P, xyz(eye)));
        Vtx vs = pv;
        bool hitReflect = false, hitMetal = false, dc = false;
        const bool exitFirst = adj_ray_color(S, fc, sample_rough, vs, dir, rc, seed, true, hitReflect, hitMetal, R, rays);
        if (!exitFirst) {
            if (fc.fast_gather && !pdiel) {
                const f4 pt = probe_term(S, vs.P, vs.N);
                rc = mul4(rc, pt);
                R.rest = mul4(R.rest, pt);
            } else {
                for (uint32_t b = 1; b < maxB; ++b) {
                    if (adj_ray_color(S, fc, sample_rough, vs, dir, rc, seed, false, dc, dc, R, rays)) break;
                    const bool early = !pdiel && rand1(seed) < 0.5f;
                    if (b == maxB - 1 || early) {
                        const f4 pt = probe_term(S, vs.P, vs.N);
                        rc = mul4(rc, pt);
                        R.rest = mul4(R.rest, pt);
                        break;
                    }
                }
            }
        }
        if (hitMetal) {
            rc = mul4(rc, ap);
            R.fac.push_back({ap, pv.mat});
        }
        if (hitReflect) frefl = add4(frefl, rc);
        else fcol = add4(fcol, rc);
        if (dimg) {
            const double sp = (double)spp;
            double u[3];
            const double apd[3] = {ap.x, ap.y, ap.z};
            const double rcd[3] = {rc.x, rc.y, rc.z};
            for (int k = 0; k < 3; ++k) u[k] = hitReflect ? g[k] / sp : g[k] * apd[k] / sp;
            const uint32_t mp = pv.mat < nm ? pv.mat : nm - 1;
            if (!hitReflect)
                for (int k = 0; k < 3; ++k) ga[3 * mp + k] += g[k] * rcd[k] / sp;
            const size_t nf = R.fac.size();
            for (size_t k = 0; k < nf; ++k) {
                double d[3] = {R.rest.x, R.rest.y, R.rest.z};
                for (size_t j = 0; j < nf; ++j) {
                    if (j == k) continue;
                    d[0] *= R.fac[j].f.x; d[1] *= R.fac[j].f.y; d[2] *= R.fac[j].f.z;
                }
                const uint32_t mk = R.fac[k].mat < nm ? R.fac[k].mat : nm - 1;
                for (int q = 0; q < 3; ++q) ga[3 * mk + q] += d[q] * u[q];
            }
            const double uc = u[0] * rcd[0] + u[1] * rcd[1] + u[2] * rcd[2];
            for (const auto& e : R.ggx) gr[e.first < nm ? e.first : nm - 1] += uc * e.second;
        }
    }
    if (out) {
        const float fs = (float)spp;
        fcol = f4{fcol.x / fs, fcol.y / fs, fcol.z / fs, fcol.w / fs};
        frefl = f4{frefl.x / fs, frefl.y / fs, frefl.z / fs, frefl.w / fs};
        out[0] = fma_(fcol.x, ap.x, frefl.x);
        out[1] = fma_(fcol.y, ap.y, frefl.y);
        out[2] = fma_(fcol.z, ap.z, frefl.z);
        out[3] = 1.0f;
    }
}
}  // namespace

// ---- ambient-cube probe grid: voxelization and bake (test restatement of k_probes.cu) ----
// VoxelizeCube (src/Assets/CPUAccelerationStructure.cpp:70-160) and FGpuProbeGenerator::
// RenderAmbientCubeOnly / FaceTask (assets/shaders/common/AmbientCube.slang:477-553, 656-690).

struct ProbeHitO {
    bool hit = false, back = false;
    float t = 0.0f;
    uint32_t mat = 0;
    Vtx v;   // P, N, mat, inst and uv (the texture coordinates at the hit)
};

f3 probe_origin(uint32_t g) {
    uint32_t y = g / (uint32_t)(kCubeXY * kCubeXY);
    uint32_t z = (g - y * (uint32_t)(kCubeXY * kCubeXY)) / (uint32_t)kCubeXY;
    uint32_t x = g - y * (uint32_t)(kCubeXY * kCubeXY) - z * (uint32_t)kCubeXY;
    return f3{(float)x * kCubeUnit + kCubeOff[0], (float)y * kCubeUnit + kCubeOff[1], (float)z * kCubeUnit + kCubeOff[2]};
}

f3 face_basis(int f) {   // +Y, -Y, +X, -X, +Z, -Z
    float s = (f & 1) ? -1.0f : 1.0f;
    return f < 2 ? f3{0.0f, s, 0.0f} : (f < 4 ? f3{s, 0.0f, 0.0f} : f3{0.0f, 0.0f, s});
}

// Closest hit over [EPS, tmax] with its float t, material, back-face flag (object-space face
// normal cross(v1 - v0, v2 - v1) against the object-space direction) and shading vertex.
ProbeHitO probe_hit(const OScene& S, f3 o, f3 d, float tmax) {
    ProbeHitO r;
    HitRec h = trace(S, o, d, kEPS, tmax, false, false, nullptr);
    if (!h.hit) return r;
    r.hit = true;
    const GkrtInstance& in = S.inst[h.inst];
    const GkrtMesh& m = S.meshes[in.mesh_id];
    LocalRay lr = to_object(in, o, d);
    f3 v0, v1, v2;
    uint32_t vi[3];
    tri_verts(S, m, h.prim, v0, v1, v2, vi);
    HybridHit hh = hybrid_eval(lr.o, lr.s, v0, v1, v2);
    r.t = hh.t;
    r.mat = in.mat_id[S.slot[vi[0]] & 15u];
    f3 a = sub(v1, v0), b = sub(v2, v1);
    f3 n{fma_(a.y, b.z, -(a.z * b.y)), fma_(a.z, b.x, -(a.x * b.z)), fma_(a.x, b.y, -(a.y * b.x))};
    r.back = fma_(n.z, lr.d.z, fma_(n.y, lr.d.y, n.x * lr.d.x)) > 0.0f;
    f3 n0 = S.nrm[vi[0]], n1 = S.nrm[vi[1]], n2 = S.nrm[vi[2]];
    f3 e1 = sub(n1, n0), e2 = sub(n2, n0);
    f3 nobj = f3{fma_(e2.x, hh.b2, fma_(e1.x, hh.b1, n0.x)), fma_(e2.y, hh.b2, fma_(e1.y, hh.b1, n0.y)),
                 fma_(e2.z, hh.b2, fma_(e1.z, hh.b1, n0.z))};
    r.v.N = normalize3(xform_normal(in.world_inv, nobj));
    r.v.P = fma3(d, hh.t, o);
    r.v.mat = r.mat;
    r.v.inst = h.inst;
    r.v.uv = f2{0.0f, 0.0f};
    if (!S.uv.empty()) {
        const f2 a = S.uv[vi[0]], b = S.uv[vi[1]], c = S.uv[vi[2]];
        r.v.uv = f2{fma_(c.x - a.x, hh.b2, fma_(b.x - a.x, hh.b1, a.x)), fma_(c.y - a.y, hh.b2, fma_(b.y - a.y, hh.b1, a.y))};
    }
    return r;
}

void voxelize_probe(const OScene& S, uint32_t g, uint32_t out[4]) {
    const f3 o = probe_origin(g);
    uint32_t mat = 0;
    float dist[6];
    for (int f = 0; f < 6; ++f) {   // InsideGeometry along +Y, -Y, +X, -X, +Z, -Z
        dist[f] = 255.0f;
        ProbeHitO h = probe_hit(S, o, face_basis(f), kCubeUnit * 64.0f);
        if (!h.hit) continue;
        dist[f] = h.t;
        if (h.t <= kCubeUnit) {
            mat = h.mat;
            if (h.back || get_mat(S, h.mat).material_model == GKRT_MAT_DIFFUSE_LIGHT) dist[f] = 0.0f;
        }
    }
    float md = fmin_(fmin_(fmin_(fmin_(fmin_(dist[0], dist[1]), dist[2]), dist[3]), dist[4]), dist[5]);
    if (md > 254.0f) {   // DetectDistance along the six distinct diagonals of the reference's list
        const float k = 0.577350269f;
        const int sgn[6][3] = {{1, 1, 1}, {-1, 1, 1}, {-1, -1, 1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}};
        for (int q = 0; q < 6; ++q) {
            f3 d{(float)sgn[q][0] * k, (float)sgn[q][1] * k, (float)sgn[q][2] * k};
            ProbeHitO h = probe_hit(S, o, d, kCubeUnit * 64.0f);
            md = fmin_(md, h.hit ? h.t : 255.0f);
        }
    }
    float c[6];
    for (int f = 0; f < 6; ++f) c[f] = fmin_(fmax_(dist[f] / kCubeUnit, 0.0f), 1.0f);
    float inside = ((((c[0] * c[1]) * c[2]) * c[3]) * c[4]) * c[5];
    out[0] = mat;
    out[1] = 0;
    out[2] = ((uint32_t)(md / kCubeUnit) & 0xFFu) | (((uint32_t)(inside * 255.0f) & 0xFFu) << 8) |
             (((uint32_t)(c[4] * 255.0f) & 0xFFu) << 16) | (((uint32_t)(c[5] * 255.0f) & 0xFFu) << 24);
    out[3] = ((uint32_t)(c[2] * 255.0f) & 0xFFu) | (((uint32_t)(c[3] * 255.0f) & 0xFFu) << 8) |
             (((uint32_t)(c[0] * 255.0f) & 0xFFu) << 16) | (((uint32_t)(c[1] * 255.0f) & 0xFFu) << 24);
}

uint32_t pack_rgb10a2(f4 c) {   // AmbientCube.slang:59-69
    float r = fmin_(fmax_(c.x * 0.001953125f, 0.0f), 1.0f), g = fmin_(fmax_(c.y * 0.001953125f, 0.0f), 1.0f);
    float b = fmin_(fmax_(c.z * 0.001953125f, 0.0f), 1.0f), a = fmin_(fmax_(c.w * 0.001953125f, 0.0f), 1.0f);
    return (uint32_t)(r * 1023.0f) | ((uint32_t)(g * 1023.0f) << 10) | ((uint32_t)(b * 1023.0f) << 20) |
           ((uint32_t)(a * 3.0f) << 30);
}

f4 sample_cube_di(const uint32_t* cube, f3 n) {   // sampleAmbientCubeHL2_DI, AmbientCube.slang:127-150
    float wx = fmax_(n.x, 0.0f), wnx = fmax_(-n.x, 0.0f), wy = fmax_(n.y, 0.0f), wny = fmax_(-n.y, 0.0f);
    float wz = fmax_(n.z, 0.0f), wnz = fmax_(-n.z, 0.0f);
    float sum = ((((wx + wnx) + wy) + wny) + wz) + wnz;
    f4 col{0.0f, 0.0f, 0.0f, 0.0f};
    col = add4(col, scale4(unpack_rgb10a2(cube[10]), wx));
    col = add4(col, scale4(unpack_rgb10a2(cube[11]), wnx));
    col = add4(col, scale4(unpack_rgb10a2(cube[8]), wy));
    col = add4(col, scale4(unpack_rgb10a2(cube[9]), wny));
    col = add4(col, scale4(unpack_rgb10a2(cube[6]), wz));
    col = add4(col, scale4(unpack_rgb10a2(cube[7]), wnz));
    return scale4(col, sum > 0.0f ? 1.0f / sum : 1.0f);
}

// interpolateAmbientCubesV2<DIAmbientCubeSampler> (AmbientCube.slang:290-382) over given arrays.
f4 probe_di(const uint32_t* cubes, const uint32_t* voxels, f3 p, f3 n) {
    float npx = (p.x - kCubeOff[0]) / kCubeUnit, npy = (p.y - kCubeOff[1]) / kCubeUnit,
          npz = (p.z - kCubeOff[2]) / kCubeUnit;
    if (!(npx >= 0.0f) || !(npy >= 0.0f) || !(npz >= 0.0f) || npx > (float)(kCubeXY - 2) || npy > (float)(kCubeZ - 2) ||
        npz > (float)(kCubeXY - 2))
        return f4{0.0f, 0.0f, 0.0f, 1.0f};
    float fx = std::floor(npx), fy = std::floor(npy), fz = std::floor(npz);
    int bx = (int)fx, by = (int)fy, bz = (int)fz;
    float frx = npx - fx, fry = npy - fy, frz = npz - fz;
    float tw = 0.0f;
    f4 res{0.0f, 0.0f, 0.0f, 0.0f};
    for (int i = 0; i < 8; ++i) {
        int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        size_t id = (size_t)(by + oy) * kCubeXY * kCubeXY + (size_t)(bz + oz) * kCubeXY + (size_t)(bx + ox);
        uint32_t u0 = voxels[id * 4 + 2], u1 = voxels[id * 4 + 3];
        float d0y = (float)((u0 >> 8) & 0xFFu) / 255.0f;
        if (d0y < 0.01f) continue;
        float d0z = (float)((u0 >> 16) & 0xFFu) / 255.0f, d0w = (float)((u0 >> 24) & 0xFFu) / 255.0f;
        float d1x = (float)(u1 & 0xFFu) / 255.0f, d1y = (float)((u1 >> 8) & 0xFFu) / 255.0f;
        float d1z = (float)((u1 >> 16) & 0xFFu) / 255.0f, d1w = (float)((u1 >> 24) & 0xFFu) / 255.0f;
        f3 pl{frx - (float)ox, fry - (float)oy, frz - (float)oz};
        float dist = length3(pl);
        f3 dir = normalize3(pl);
        float hl = std::sqrt(fmax_(dir.x, 0.0f)) * d1x;
        hl = hl + std::sqrt(fmax_(-dir.x, 0.0f)) * d1y;
        hl = hl + std::sqrt(fmax_(dir.y, 0.0f)) * d1z;
        hl = hl + std::sqrt(fmax_(-dir.y, 0.0f)) * d1w;
        hl = hl + std::sqrt(fmax_(dir.z, 0.0f)) * d0z;
        hl = hl + std::sqrt(fmax_(-dir.z, 0.0f)) * d0w;
        if (dist > hl + 0.05f) continue;
        float wx = ox == 0 ? 1.0f - frx : frx, wy = oy == 0 ? 1.0f - fry : fry, wz = oz == 0 ? 1.0f - frz : frz;
        float wgt = (wx * wy) * wz;
        res = add4(res, scale4(sample_cube_di(cubes + id * 14, n), wgt));
        tw = tw + wgt;
    }
    if (tw > 0.0f) return f4{res.x / tw, res.y / tw, res.z / tw, res.w / tw};
    return f4{0.0f, 0.0f, 0.0f, 0.0f};
}

inline float lerpf_(float a, float b, float t) { return fma_(t, b - a, a); }

// One bake step of probe g: new cube words (14) and age; cubes_prev / voxels are whole grids.
void bake_probe(const OScene& S, const GkrtFrameConstants& fc, uint32_t g, const uint32_t* cubes_prev,
                const uint32_t* voxels, uint32_t out[14], uint32_t* age) {
    static const float g44[32] = {-0.75f, -0.75f, -0.25f, -0.75f, 0.25f, -0.75f, 0.75f, -0.75f,
                                  -0.75f, -0.25f, -0.25f, -0.25f, 0.25f, -0.25f, 0.75f, -0.25f,
                                  -0.75f, 0.25f,  -0.25f, 0.25f,  0.25f, 0.25f,  0.75f, 0.25f,
                                  -0.75f, 0.75f,  -0.25f, 0.75f,  0.25f, 0.75f,  0.75f, 0.75f};
    static const float g33[18] = {-0.667f, -0.667f, 0.0f, -0.667f, 0.667f, -0.667f, -0.667f, 0.0f, 0.0f,
                                  0.0f,    0.667f,  0.0f, -0.667f, 0.667f, 0.0f,    0.667f, 0.667f, 0.667f};
    const uint32_t* prev = cubes_prev + (size_t)g * 14;
    const uint32_t* vox = voxels + (size_t)g * 4;
    for (int w = 0; w < 14; ++w) out[w] = prev[w];
    *age = vox[1];
    if ((vox[2] & 0xFFu) >= 8u) return;   // surface probes only
    *age = vox[1] + 1u;
    uint32_t sky[6];
    uint32_t sun = (prev[13] >> 16) & 0xFFu;
    const int dws[6] = {8, 9, 10, 11, 6, 7};
    const int sws[6] = {12, 12, 13, 13, 12, 12}, sbs[6] = {2, 3, 0, 1, 0, 1};
    // light 0: centre lerp(p1, p3, 0.5), power = its material's diffuse, area
    bool lvalid = !S.lights.empty();
    f3 lpos{0.0f, 0.0f, 0.0f};
    f4 lpow{0.0f, 0.0f, 0.0f, 0.0f};
    float larea = 0.0f;
    if (lvalid) {
        const GkrtLight& L = S.lights[0];
        lpos = f3{fma_(0.5f, L.p3[0] - L.p1[0], L.p1[0]), fma_(0.5f, L.p3[1] - L.p1[1], L.p1[1]),
                  fma_(0.5f, L.p3[2] - L.p1[2], L.p1[2])};
        const GkrtMaterial& lm = S.mats[L.light_mat_idx];
        lpow = f4{lm.diffuse[0], lm.diffuse[1], lm.diffuse[2], lm.diffuse[3]};
        larea = L.normal_area[3];
    }
    for (int f = 0; f < 6; ++f) {
        const f3 basis = face_basis(f);
        const f3 o = fma3(basis, kCubeUnit * 0.25f, probe_origin(g));
        f4 direct{0.0f, 0.0f, 0.0f, 0.0f}, bounce{0.0f, 0.0f, 0.0f, 0.0f};
        float skyv = 0.0f;
        const uint32_t j = vox[1] % 9u;
        const float jx = g33[2 * j] * 0.25f, jy = g33[2 * j + 1] * 0.25f;
        for (int i = 0; i < 16; ++i) {
            f3 hv = normalize3(f3{g44[2 * i] + jx, g44[2 * i + 1] + jy, 1.0f});
            f3 dir = align_with_normal(hv, basis);
            ProbeHitO h = probe_hit(S, o, dir, 20.0f);
            if (h.hit) {
                // the material's diffuse times its diffuse texture (AmbientCube.slang:504-510)
                const GkrtMaterial& hm = get_mat(S, h.v.mat);
                f4 alb{hm.diffuse[0], hm.diffuse[1], hm.diffuse[2], hm.diffuse[3]};
                if (hm.diffuse_texture_id >= 0) alb = mul4(alb, tex_sample(S, hm.diffuse_texture_id, h.v.uv.x, h.v.uv.y));
                bounce = add4(bounce, scale4(mul4(alb, probe_di(cubes_prev, voxels, h.v.P, h.v.N)), 1.25f));
            } else {
                // (AmbientCube.slang:512-516) the sky texture's projection, or the constant sky
                direct = add4(direct, (fc.flags & GKRT_FRAME_SKY_TEXTURE) ? sky_rough(S, fc, dir) : sky_color(fc));
                skyv = skyv + 1.0f;
            }
        }
        direct = scale4(direct, 0.0625f);
        bounce = scale4(bounce, 0.0625f);
        if (lvalid) {
            f3 dv = sub(lpos, o);
            float len = length3(dv);
            f3 dn{dv.x / len, dv.y / len, dv.z / len};
            bool hit = trace(S, fma3(dn, kCubeUnit * 0.5f, o), dn, kEPS, len - kCubeUnit, true, false, nullptr).hit;
            float atten = hit ? 0.0f : 1.0f;
            f3 ldir = normalize3(dv);
            float ndotl = fmin_(fmax_(dot3(basis, ldir), 0.0f), 1.0f);
            float att = (ndotl * larea) / ((len * len) * 3.14159f);
            direct = add4(direct, scale4(scale4(lpow, att), atten));
        }
        if (fc.has_sun) {
            f3 sd{fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]};
            bool hit = trace(S, o, sd, kEPS, kPT_MAX, true, false, nullptr).hit;
            float atten = hit ? 0.0f : 1.0f;
            float ndotl = fmin_(fmax_(dot3(basis, sd), 0.0f), 1.0f);
            if (f == 0) sun = atten > 0.0f ? 1u : 0u;
            f4 sc4{fc.sun_color[0], fc.sun_color[1], fc.sun_color[2], fc.sun_color[3]};
            direct = add4(direct, scale4(scale4(scale4(scale4(sc4, atten), ndotl), 1.0f), 0.25f));
        }
        float ov = (float)((prev[sws[f]] >> (8 * sbs[f])) & 0xFFu);
        sky[f] = (uint32_t)lerpf_(ov, (255.0f * skyv) / 16.0f, 0.125f) & 0xFFu;
        f4 od = unpack_rgb10a2(prev[dws[f]]), oi = unpack_rgb10a2(prev[dws[f] - 6]);
        out[dws[f]] = pack_rgb10a2(f4{lerpf_(od.x, direct.x, 0.125f), lerpf_(od.y, direct.y, 0.125f),
                                      lerpf_(od.z, direct.z, 0.125f), lerpf_(od.w, direct.w, 0.125f)});
        out[dws[f] - 6] = pack_rgb10a2(f4{lerpf_(oi.x, bounce.x, 0.125f), lerpf_(oi.y, bounce.y, 0.125f),
                                          lerpf_(oi.z, bounce.z, 0.125f), lerpf_(oi.w, bounce.w, 0.125f)});
    }
    out[12] = sky[4] | (sky[5] << 8) | (sky[0] << 16) | (sky[1] << 24);
    out[13] = sky[2] | (sky[3] << 8) | (sun << 16) | (prev[13] & 0xFF000000u);
}

// ================================ output stage ========================================
// The presentation image as 8-bit BGRA words (the reference's B8G8R8A8_UNORM swapchain image).
// A UNORM store clamps to [0, 1] (NaN to 0), scales by 255 and rounds to nearest even.

static uint32_t unorm8_o(float v) {
    v = std::fmin(std::fmax(v, 0.0f), 1.0f);
    return (uint32_t)std::nearbyint(v * 255.0f);
}
static uint32_t bgra_o(const float* c) {
    return unorm8_o(c[2]) | (unorm8_o(c[1]) << 8) | (unorm8_o(c[0]) << 16) | (unorm8_o(c[3]) << 24);
}

// Resolve pass: vkCmdBlitImage with VK_FILTER_LINEAR from the render extent onto the rectangle
// (ox, oy, ow, oh) (VulkanBaseRenderer.cpp:1036-1068). The Vulkan specification's scaled-blit
// rule: destination centre x + 0.5 -> u = (x - ox + 0.5) * W / ow, then a linear filter with
// clamp-to-edge: texels floor(u - 0.5) and the next, weights 1 - a and a, a = frac(u - 0.5).
static void output_resolve_o(const float* src, int W, int H, int P, uint32_t* out, int OW, int OH, int ox, int oy,
                             int ow, int oh) {
    const float su = (float)W / (float)ow, sv = (float)H / (float)oh;
    const long long xa = std::max<long long>(ox, 0), xb = std::min<long long>((long long)ox + ow, OW);
    const long long ya = std::max<long long>(oy, 0), yb = std::min<long long>((long long)oy + oh, OH);
    for (long long y = ya; y < yb; ++y)
        for (long long x = xa; x < xb; ++x) {
            const float u = ((float)(x - ox) + 0.5f) * su - 0.5f;
            const float v = ((float)(y - oy) + 0.5f) * sv - 0.5f;
            const float fu = std::floor(u), fv = std::floor(v);
            const float a = u - fu, b = v - fv;
            const int i0 = (int)fu, j0 = (int)fv;
            const int i[2] = {std::min(std::max(i0, 0), W - 1), std::min(std::max(i0 + 1, 0), W - 1)};
            const int j[2] = {std::min(std::max(j0, 0), H - 1), std::min(std::max(j0 + 1, 0), H - 1)};
            const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
            float c[4];
            for (int k = 0; k < 4; ++k) {
                const float t00 = src[4 * ((size_t)j[0] * P + i[0]) + k], t10 = src[4 * ((size_t)j[0] * P + i[1]) + k];
                const float t01 = src[4 * ((size_t)j[1] * P + i[0]) + k], t11 = src[4 * ((size_t)j[1] * P + i[1]) + k];
                c[k] = ((t00 * w00 + t10 * w10) + t01 * w01) + t11 * w11;
            }
            out[(size_t)y * OW + x] = bgra_o(c);
        }
}

// Process.UpScaleFSR.comp.slang: FsrEasuCF (:23-29), FsrEasuTapF (:74-101), FsrEasuSetF (:105-132),
// FsrEasuCon (:32-72), FsrEasuF (:135-248), main (:264-299). rsqrt as 1 / sqrt.
namespace easu_o {
struct V4 { float v[4]; };
struct Img { const float* p; int W, H, P; };
static V4 tex(const Img& s, int x, int y) {
    V4 r;
    for (int k = 0; k < 4; ++k) r.v[k] = s.p[4 * ((size_t)y * s.P + x) + k];
    return r;
}
static V4 cf(const Img& s, float px, float py) {   // FsrEasuCF: int(p * size), clamped
    int cx = (int)(px * (float)s.W), cy = (int)(py * (float)s.H);
    cx = std::min(std::max(cx, 0), s.W - 1);
    cy = std::min(std::max(cy, 0), s.H - 1);
    return tex(s, cx, cy);
}
static float luma(const V4& c) { return c.v[1] + 0.5f * (c.v[0] + c.v[2]); }
static float sat(float x) { return std::fmin(std::fmax(x, 0.0f), 1.0f); }
static void setf(float& dx, float& dy, float& len, float w, float lA, float lB, float lC, float lD, float lE) {
    float lenX = std::fmax(std::fabs(lD - lC), std::fabs(lC - lB));
    float dirX = lD - lB;
    dx += dirX * w;
    lenX = sat(std::fabs(dirX) / lenX);
    lenX *= lenX;
    len += lenX * w;
    float lenY = std::fmax(std::fabs(lE - lC), std::fabs(lC - lA));
    float dirY = lE - lA;
    dy += dirY * w;
    lenY = sat(std::fabs(dirY) / lenY);
    lenY *= lenY;
    len += lenY * w;
}
static void tapf(V4& aC, float& aW, float offx, float offy, float dx, float dy, float lx, float ly, float lob,
                 float clp, const V4& c) {
    float vx = offx * dx + offy * dy;
    float vy = offx * (-dy) + offy * dx;
    vx *= lx;
    vy *= ly;
    float d2 = std::fmin(vx * vx + vy * vy, clp);
    float wB = 0.4f * d2 - 1.0f;
    float wA = lob * d2 - 1.0f;
    wB *= wB;
    wA *= wA;
    wB = 1.5625f * wB - 0.5625f;
    float w = wB * wA;
    for (int k = 0; k < 4; ++k) aC.v[k] += c.v[k] * w;
    aW += w;
}
static V4 easu(const Img& s, float OWf, float OHf, float ipx, float ipy) {
    const float Wf = (float)s.W, Hf = (float)s.H;
    // FsrEasuCon(con0..3, viewport = input = W x H, output = OW x OH)
    const float con0[4] = {Wf / OWf, Hf / OHf, 0.5f * Wf / OWf - 0.5f, 0.5f * Hf / OHf - 0.5f};
    const float con1[4] = {1.0f / Wf, 1.0f / Hf, 1.0f / Wf, -1.0f / Hf};
    const float con2[4] = {-1.0f / Wf, 2.0f / Hf, 1.0f / Wf, 2.0f / Hf};
    const float con3[2] = {0.0f / Wf, 4.0f / Hf};
    float ppx = ipx * con0[0] + con0[2], ppy = ipy * con0[1] + con0[3];
    const float fpx = std::floor(ppx), fpy = std::floor(ppy);
    ppx -= fpx;
    ppy -= fpy;
    const float p0x = fpx * con1[0] + con1[2], p0y = fpy * con1[1] + con1[3];
    const float p1x = p0x + con2[0], p1y = p0y + con2[1];
    const float p2x = p0x + con2[2], p2y = p0y + con2[3];
    const float p3x = p0x + con3[0], p3y = p0y + con3[1];
    const float off[4] = {-0.5f * con1[0], 0.5f * con1[0], -0.5f * con1[1], 0.5f * con1[1]};   // x y z w
    const V4 bC = cf(s, p0x + off[0], p0y + off[3]), cC = cf(s, p0x + off[1], p0y + off[3]);
    const V4 iC = cf(s, p1x + off[0], p1y + off[3]), jC = cf(s, p1x + off[1], p1y + off[3]);
    const V4 fC = cf(s, p1x + off[1], p1y + off[2]), eC = cf(s, p1x + off[0], p1y + off[2]);
    const V4 kC = cf(s, p2x + off[0], p2y + off[3]), lC = cf(s, p2x + off[1], p2y + off[3]);
    const V4 hC = cf(s, p2x + off[1], p2y + off[2]), gC = cf(s, p2x + off[0], p2y + off[2]);
    const V4 oC = cf(s, p3x + off[1], p3y + off[2]), nC = cf(s, p3x + off[0], p3y + off[2]);
    const float bL = luma(bC), cL = luma(cC), iL = luma(iC), jL = luma(jC), fL = luma(fC), eL = luma(eC);
    const float kL = luma(kC), lL = luma(lC), hL = luma(hC), gL = luma(gC), oL = luma(oC), nL = luma(nC);
    float dx = 0.0f, dy = 0.0f, len = 0.0f;
    setf(dx, dy, len, (1.0f - ppx) * (1.0f - ppy), bL, eL, fL, gL, jL);
    setf(dx, dy, len, ppx * (1.0f - ppy), cL, fL, gL, hL, kL);
    setf(dx, dy, len, (1.0f - ppx) * ppy, fL, iL, jL, kL, nL);
    setf(dx, dy, len, ppx * ppy, gL, jL, kL, lL, oL);
    const float d2x = dx * dx, d2y = dy * dy;
    float dirR = d2x + d2y;
    const bool zro = dirR < (1.0f / 32768.0f);
    dirR = 1.0f / std::sqrt(dirR);
    dirR = zro ? 1.0f : dirR;
    dx = zro ? 1.0f : dx;
    dx *= dirR;
    dy *= dirR;
    len = len * 0.5f;
    len *= len;
    const float stretch = (dx * dx + dy * dy) / std::fmax(std::fabs(dx), std::fabs(dy));
    const float l2x = 1.0f + (stretch - 1.0f) * len, l2y = 1.0f - 0.5f * len;
    const float lob = 0.5f - 0.29f * len;
    const float clp = 1.0f / lob;
    V4 mn, mx;
    for (int k = 0; k < 4; ++k) {
        mn.v[k] = std::fmin(std::fmin(fC.v[k], gC.v[k]), std::fmin(jC.v[k], kC.v[k]));
        mx.v[k] = std::fmax(std::fmax(fC.v[k], gC.v[k]), std::fmax(jC.v[k], kC.v[k]));
    }
    V4 aC = {{0.0f, 0.0f, 0.0f, 0.0f}};
    float aW = 0.0f;
    tapf(aC, aW, 0.0f - ppx, -1.0f - ppy, dx, dy, l2x, l2y, lob, clp, bC);
    tapf(aC, aW, 1.0f - ppx, -1.0f - ppy, dx, dy, l2x, l2y, lob, clp, cC);
    tapf(aC, aW, -1.0f - ppx, 1.0f - ppy, dx, dy, l2x, l2y, lob, clp, iC);
    tapf(aC, aW, 0.0f - ppx, 1.0f - ppy, dx, dy, l2x, l2y, lob, clp, jC);
    tapf(aC, aW, 0.0f - ppx, 0.0f - ppy, dx, dy, l2x, l2y, lob, clp, fC);
    tapf(aC, aW, -1.0f - ppx, 0.0f - ppy, dx, dy, l2x, l2y, lob, clp, eC);
    tapf(aC, aW, 1.0f - ppx, 1.0f - ppy, dx, dy, l2x, l2y, lob, clp, kC);
    tapf(aC, aW, 2.0f - ppx, 1.0f - ppy, dx, dy, l2x, l2y, lob, clp, lC);
    tapf(aC, aW, 2.0f - ppx, 0.0f - ppy, dx, dy, l2x, l2y, lob, clp, hC);
    tapf(aC, aW, 1.0f - ppx, 0.0f - ppy, dx, dy, l2x, l2y, lob, clp, gC);
    tapf(aC, aW, 1.0f - ppx, 2.0f - ppy, dx, dy, l2x, l2y, lob, clp, oC);
    tapf(aC, aW, 0.0f - ppx, 2.0f - ppy, dx, dy, l2x, l2y, lob, clp, nC);
    V4 r;
    for (int k = 0; k < 4; ++k) r.v[k] = std::fmin(mx.v[k], std::fmax(mn.v[k], aC.v[k] / aW));
    return r;
}
}  // namespace easu_o

static void output_fsr_o(const float* src, int W, int H, int P, uint32_t* out, int OW, int OH, int offx, int offy,
                         int outw, int outh) {
    const easu_o::Img s{src, W, H, P};
    const int gw = (outw / 8) * 8, gh = (outh / 8) * 8;   // vkCmdDispatch(outw / 8, outh / 8) of 8 x 8 groups
    for (int y = 0; y < gh; ++y)
        for (int x = 0; x < gw; ++x) {
            easu_o::V4 c;
            if (OW != W || OH != H) {
                const float uvx = (float)x / (float)outw, uvy = (float)y / (float)outh;
                c = easu_o::easu(s, (float)OW, (float)OH, uvx * (float)OW, uvy * (float)OH);
            } else {
                int sx = (int)((float)x * (float)OW / (float)outw), sy = (int)((float)y * (float)OH / (float)outh);
                sx = std::min(std::max(sx, 0), W - 1);
                sy = std::min(std::max(sy, 0), H - 1);
                c = easu_o::tex(s, sx, sy);
            }
            const long long dx = (long long)x + offx, dy = (long long)y + offy;
            if (dx < 0 || dy < 0 || dx >= OW || dy >= OH) continue;
            out[(size_t)dy * OW + (size_t)dx] = bgra_o(c.v);
        }
}

// ===================================== C API ==========================================
extern "C" {

float gko_atan2(float y, float x) { return atan2_(y, x); }
float gko_acos(float x) { return acos_(x); }
// The oracle's texture lookup and sky radiance, for their tests.
void gko_tex_sample(void* h, int id, float u, float v, float* out) {
    const f4 c = tex_sample(*static_cast<OScene*>(h), id, u, v);
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
}
// The projection of texture id (27 floats: red, green, blue terms) and the bake's sky lookup.
int gko_texture_sh(void* h, uint32_t id, float* out) {
    const OScene* S = static_cast<OScene*>(h);
    if (id >= S->tex.size()) return -1;
    std::memcpy(out, S->tex[id].sh, 27 * sizeof(float));
    return 0;
}
void gko_sky_rough(void* h, const GkrtFrameConstants* fc, const float* dir, float* out) {
    const f4 c = sky_rough(*static_cast<OScene*>(h), *fc, f3{dir[0], dir[1], dir[2]});
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
}
void gko_sky_dir(void* h, const GkrtFrameConstants* fc, const float* dir, float* out) {
    const f4 c = sky_dir(*static_cast<OScene*>(h), *fc, f3{dir[0], dir[1], dir[2]});
    out[0] = c.x; out[1] = c.y; out[2] = c.z; out[3] = c.w;
}

// ProjectHdrToSh (Texture.cpp:180-254) of an equirectangular RGBA float image: per texel
// (x, y) the direction at theta = (y + 1/2) pi / h, phi = (x + 1/2) 2 pi / w, i.e.
// (sin theta cos phi, cos theta, sin theta sin phi), the nine real harmonics of bands 0-2 with
// the shader's constants, and the solid-angle weight sin theta (pi / h)(2 pi / w); the sums are
// not normalised. Summed in double, rows first to last and texels left to right, then rounded
// to float (the reference sums in float).
void project_sh(const f4* t, uint32_t w, uint32_t h, float out[27]) {
    const double pi = 3.14159265358979323846;
    const double k0 = 0.282095, k1 = 0.488603, k2 = 1.092548, k3 = 0.315392, k4 = 0.546274;
    double sum[27];
    for (int k = 0; k < 27; ++k) sum[k] = 0.0;
    for (uint32_t y = 0; y < h; ++y) {
        const double theta = ((double)y + 0.5) / (double)h * pi;
        const double sth = std::sin(theta), cth = std::cos(theta);
        const double wgt = sth * (pi / (double)h) * (2.0 * pi / (double)w);
        for (uint32_t x = 0; x < w; ++x) {
            const double phi = ((double)x + 0.5) / (double)w * (2.0 * pi);
            const double dx = sth * std::cos(phi), dy = cth, dz = sth * std::sin(phi);
            const double y9[9] = {k0, -k1 * dy, k1 * dz, -k1 * dx, k2 * dx * dy, -k2 * dy * dz,
                                  k3 * (3.0 * dy * dy - 1.0), -k2 * dx * dz, k4 * (dx * dx - dz * dz)};
            const f4 c = t[(size_t)y * w + x];
            for (int i = 0; i < 9; ++i) {
                sum[i] += (double)c.x * y9[i] * wgt;
                sum[9 + i] += (double)c.y * y9[i] * wgt;
                sum[18 + i] += (double)c.z * y9[i] * wgt;
            }
        }
    }
    for (int k = 0; k < 27; ++k) out[k] = (float)sum[k];
}

// Texture `id` of the oracle scene: texels as the sampler returns them (RGBA8 UNORM c / 255;
// sRGB through the sRGB transfer function in double; RGBA32F as given). 0 on success.
int gko_texture_upload(void* h, uint32_t id, uint32_t w, uint32_t ht, uint32_t format, const void* texels) {
    OScene* S = static_cast<OScene*>(h);
    if (id >= GKRT_MAX_TEXTURES || !w || !ht || format > GKRT_TEX_RGBA32F || !texels) return -1;
    if (S->tex.size() <= id) S->tex.resize(id + 1);
    OScene::Tex& t = S->tex[id];
    t.w = w;
    t.h = ht;
    const size_t n = (size_t)w * ht;
    t.t.resize(n);
    std::fill(t.sh, t.sh + 27, 0.0f);
    if (format == GKRT_TEX_RGBA32F) {
        std::memcpy(t.t.data(), texels, n * 16);
        project_sh(t.t.data(), w, ht, t.sh);
        return 0;
    }
    const uint8_t* b = static_cast<const uint8_t*>(texels);
    auto unorm = [](uint8_t c) { return (float)c / 255.0f; };
    auto srgb = [](uint8_t c) {
        const double v = (double)c / 255.0;
        return (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    };
    for (size_t i = 0; i < n; ++i) {
        const uint8_t* c = b + 4 * i;
        t.t[i] = format == GKRT_TEX_RGBA8_SRGB ? f4{srgb(c[0]), srgb(c[1]), srgb(c[2]), unorm(c[3])}
                                               : f4{unorm(c[0]), unorm(c[1]), unorm(c[2]), unorm(c[3])};
    }
    return 0;
}

void* gko_scene_create(const GkrtSceneDesc* d) {
    OScene* S = new OScene();
    S->pos.resize(d->vertex_count);
    S->nrm.resize(d->vertex_count);
    S->slot.assign(d->material_slots, d->material_slots + d->vertex_count);
    for (uint32_t i = 0; i < d->vertex_count; ++i) {
        S->pos[i] = f3{d->positions[4 * i], d->positions[4 * i + 1], d->positions[4 * i + 2]};
        S->nrm[i] = f3{d->normals[4 * i], d->normals[4 * i + 1], d->normals[4 * i + 2]};
    }
    if (d->texcoords) {
        S->uv.resize(d->vertex_count);
        for (uint32_t i = 0; i < d->vertex_count; ++i) S->uv[i] = f2{d->texcoords[2 * i], d->texcoords[2 * i + 1]};
    }
    if (d->tangents) {
        S->tan.resize(d->vertex_count);
        for (uint32_t i = 0; i < d->vertex_count; ++i)
            S->tan[i] = f4{d->tangents[4 * i], d->tangents[4 * i + 1], d->tangents[4 * i + 2], d->tangents[4 * i + 3]};
    }
    S->idx.assign(d->indices, d->indices + d->index_count);
    S->meshes.assign(d->meshes, d->meshes + d->mesh_count);
    S->mats.assign(d->materials, d->materials + d->material_count);
    S->inst.assign(d->instances, d->instances + d->instance_count);
    build_emitters(*S);
    if (d->lights && d->light_count) S->lights.assign(d->lights, d->lights + d->light_count);
    if (d->probe_cubes && d->probe_voxels) {
        size_t n = (size_t)kCubeXY * kCubeXY * kCubeZ;
        S->cubes.assign(d->probe_cubes, d->probe_cubes + n * 14);
        S->voxels.assign(d->probe_voxels, d->probe_voxels + n * 4);
        S->has_probes = true;
    }
    // BLAS per mesh over triangle boxes (float min/max of the vertices: exact).
    S->blas.resize(S->meshes.size());
    std::vector<Box> rootbox(S->meshes.size());
    for (size_t mi = 0; mi < S->meshes.size(); ++mi) {
        const GkrtMesh& m = S->meshes[mi];
        uint32_t nt = m.index_count / 3;
        std::vector<Box> boxes(nt);
        Box rb{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
        for (uint32_t t = 0; t < nt; ++t) {
            f3 v[3];
            tri_verts(*S, m, t, v[0], v[1], v[2]);
            for (int k = 0; k < 3; ++k) {
                float a = comp(v[0], k), b = comp(v[1], k), c = comp(v[2], k);
                boxes[t].lo[k] = std::min(a, std::min(b, c));
                boxes[t].hi[k] = std::max(a, std::max(b, c));
                rb.lo[k] = std::min(rb.lo[k], boxes[t].lo[k]);
                rb.hi[k] = std::max(rb.hi[k], boxes[t].hi[k]);
            }
        }
        build_bvh(S->blas[mi], boxes);
        rootbox[mi] = rb;
    }
    // TLAS over instance world boxes (corners transformed in double, padded).
    std::vector<Box> ib;
    std::vector<uint32_t> map;
    for (size_t ii = 0; ii < S->inst.size(); ++ii) {
        const GkrtInstance& in = S->inst[ii];
        if (!in.visible) continue;
        const Box& rb = rootbox[in.mesh_id];
        Box w{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};
        for (int c = 0; c < 8; ++c) {
            double p[3] = {(c & 1) ? rb.hi[0] : rb.lo[0], (c & 2) ? rb.hi[1] : rb.lo[1], (c & 4) ? rb.hi[2] : rb.lo[2]};
            for (int r = 0; r < 3; ++r) {
                double v = (double)in.world[4 * r] * p[0] + (double)in.world[4 * r + 1] * p[1] +
                           (double)in.world[4 * r + 2] * p[2] + (double)in.world[4 * r + 3];
                w.lo[r] = std::min(w.lo[r], (float)v);
                w.hi[r] = std::max(w.hi[r], (float)v);
            }
        }
        for (int r = 0; r < 3; ++r) {
            float pad = 1e-4f * (std::fabs(w.lo[r]) + std::fabs(w.hi[r]) + (w.hi[r] - w.lo[r])) + 1e-6f;
            w.lo[r] -= pad;
            w.hi[r] += pad;
        }
        ib.push_back(w);
        map.push_back((uint32_t)ii);
    }
    build_bvh(S->tlas, ib);
    for (auto& p : S->tlas.prims) p = map[p];
    return S;
}

void gko_scene_destroy(void* s) { delete (OScene*)s; }

// Closest (mode 0) or any (mode 1) hit of device-layout rays, FP64 definition.
// brute != 0 tests every triangle of every instance. Fills GkrtHit like the GPU.
void gko_trace_rays(void* s, const GkrtRay* rays, GkrtHit* hits, uint32_t n, uint32_t mode, int brute,
                    int threads) {
    const OScene& S = *(const OScene*)s;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 64)
#endif
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        const GkrtRay& r = rays[i];
        f3 o{r.origin[0], r.origin[1], r.origin[2]}, d{r.dir[0], r.dir[1], r.dir[2]};
        HitRec h = trace(S, o, d, r.tmin, r.tmax, mode == GKRT_TRACE_ANY, brute != 0, nullptr);
        GkrtHit& H = hits[i];
        std::memset(&H, 0, sizeof(H));
        if (!h.hit) {
            H.t = -1.0f; H.inst = 0xFFFFFFFFu; H.prim = 0xFFFFFFFFu;
            continue;
        }
        H.inst = h.inst;
        H.prim = h.prim;
        if (mode == GKRT_TRACE_ANY) { H.t = (float)h.td; continue; }
        const GkrtInstance& in = S.inst[h.inst];
        LocalRay lr = to_object(in, o, d);
        f3 v0, v1, v2;
        tri_verts(S, S.meshes[in.mesh_id], h.prim, v0, v1, v2);
        HybridHit hh = hybrid_eval(lr.o, lr.s, v0, v1, v2);
        H.t = hh.t; H.b1 = hh.b1; H.b2 = hh.b2;
    }
}

// The "rt pass" over rows [y0, y1) (or every pixel when y1 <= y0). images: GKRT_IMG_COUNT
// host pointers laid out like the product's images (NULL allowed for HIT_*).
// Returns the number of rays traced (camera + bounce + shadow).
uint64_t gko_trace_pass(void* s, const GkrtFrameConstants* fc, int W, int H, void** images, int y0, int y1,
                        int threads) {
    const OScene& S = *(const OScene*)s;
    if (y1 <= y0) { y0 = 0; y1 = H; }
    std::atomic<uint64_t> total{0};
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        uint64_t local = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 64) nowait
#endif
        for (int64_t p = (int64_t)y0 * W; p < (int64_t)y1 * W; ++p)
            shade_pixel(S, *fc, W, H, (int)(p % W), (int)(p / W), images, &local);
        total += local;
    }
    return total.load();
}

// Adjoint restatement over the pixel window [x0, x1) x [y0, y1): image (dense W x H float4,
// window written) and, when dimg is given, FP64 gradient sums (ga: 3 per material, gr: 1).
uint64_t gko_adjoint(void* s, const GkrtFrameConstants* fc, int W, int H, int x0, int y0, int x1, int y1,
                     uint32_t spp, const float* sample_rough, float* img, const float* dimg, double* ga, double* gr,
                     int threads) {
    const OScene& S = *(const OScene*)s;
    const size_t nm = S.mats.size();
    std::atomic<uint64_t> total{0};
    std::vector<std::vector<double>> parts;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel
#endif
    {
        std::vector<double> la(dimg ? 3 * nm : 0, 0.0), lr(dimg ? nm : 0, 0.0);
        uint64_t local = 0;
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16) nowait
#endif
        for (int64_t p = 0; p < (int64_t)(x1 - x0) * (y1 - y0); ++p) {
            const int x = x0 + (int)(p % (x1 - x0)), y = y0 + (int)(p / (x1 - x0));
            adjoint_pixel(S, *fc, W, H, x, y, spp, sample_rough, img, dimg, la.data(), lr.data(), &local);
        }
        total += local;
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            if (dimg) {
                for (size_t k = 0; k < 3 * nm; ++k) ga[k] += la[k];
                for (size_t k = 0; k < nm; ++k) gr[k] += lr[k];
            }
        }
    }
    return total.load();
}

void gko_reproject_pass(const GkrtFrameConstants* fc, int W, int H, void** images, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static)
#endif
    for (int64_t p = 0; p < (int64_t)W * H; ++p) reproject_pixel(*fc, W, H, (int)(p % W), (int)(p / W), images);
}

void gko_denoise_pass(const GkrtFrameConstants* fc, int W, int H, void** images, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    if (fc->denoiser == GKRT_DENOISE_ATROUS && fc->bf_size > 0u) {
        std::vector<float> t0((size_t)W * H * 4), t1((size_t)W * H * 4);
        const float* src = (const float*)images[GKRT_IMG_ACCUM_DIFFUSE];
        float* bufs[2] = {t0.data(), t1.data()};
        for (int pass = 0; pass < 3; ++pass) {
            float* dst = bufs[pass & 1];
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
            for (int64_t p = 0; p < (int64_t)W * H; ++p)
                atrous_pixel(*fc, W, H, (int)(p % W), (int)(p / W), 1 << pass, src, dst, pass == 2, images);
            src = dst;
        }
        return;
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int64_t p = 0; p < (int64_t)W * H; ++p) denoise_pixel(*fc, W, H, (int)(p % W), (int)(p / W), images);
}

void gko_set_fast(int on) { g_fast = on; }

// Output stage on a W x H RGBA32F image (pitch P pixels) into OW x OH BGRA8 words.
void gko_output_resolve(const float* src, int W, int H, int P, uint32_t* out, int OW, int OH, int ox, int oy, int ow,
                        int oh) {
    output_resolve_o(src, W, H, P, out, OW, OH, ox, oy, ow, oh);
}
void gko_output_fsr(const float* src, int W, int H, int P, uint32_t* out, int OW, int OH, int offx, int offy,
                    int outw, int outh) {
    output_fsr_o(src, W, H, P, out, OW, OH, offx, offy, outw, outh);
}
// ScreenShot::SaveSwapChainToFileFast (ScreenShot.cpp:18-79): bytes (bits 16, 8, 0) of each word.
void gko_screenshot(const uint32_t* img, int OW, int x0, int y0, int w, int h, uint8_t* rgb) {
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const uint32_t p = img[(size_t)(y0 + y) * OW + (x0 + x)];
            uint8_t* d = rgb + 3 * ((size_t)y * w + x);
            d[0] = (uint8_t)((p >> 16) & 0xFFu);
            d[1] = (uint8_t)((p >> 8) & 0xFFu);
            d[2] = (uint8_t)(p & 0xFFu);
        }
}

// Probe voxelization of probes [first, first + count): 4 words each into out.
void gko_probe_voxelize(void* s, uint32_t first, uint32_t count, uint32_t* out, int threads) {
    const OScene& S = *(const OScene*)s;
#pragma omp parallel for schedule(dynamic, 16) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int64_t k = 0; k < (int64_t)count; ++k) voxelize_probe(S, first + (uint32_t)k, out + 4 * k);
}

// One bake step of probes [first, first + count) from whole-grid cubes_prev / voxels: 14 cube
// words and the new age of each probe.
void gko_probe_bake(void* s, const GkrtFrameConstants* fc, uint32_t first, uint32_t count, const uint32_t* cubes_prev,
                    const uint32_t* voxels, uint32_t* cubes_out, uint32_t* ages_out, int threads) {
    const OScene& S = *(const OScene*)s;
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads > 0 ? threads : omp_get_max_threads())
    for (int64_t k = 0; k < (int64_t)count; ++k)
        bake_probe(S, *fc, first + (uint32_t)k, cubes_prev, voxels, cubes_out + 14 * k, ages_out + k);
}

// Small known-answer hooks for the unit tests.
void gko_pcg4d(uint32_t v[4]) { pcg4d(v); }
float gko_uint_to_float(uint32_t x) { return u2f(x); }
void gko_sincos_2pi(float u, float* s, float* c) { sincos_2pi(u, s, c); }
void gko_sample_hemi(uint32_t seed[4], float out[3]) { f3 v = hemi1(seed); out[0] = v.x; out[1] = v.y; out[2] = v.z; }
void gko_sample_ggx(uint32_t seed[4], float roughness, const float n[3], float out[3]) {
    f3 v = ggx_sampling(seed, roughness, f3{n[0], n[1], n[2]});
    out[0] = v.x; out[1] = v.y; out[2] = v.z;
}
float gko_schlick(float c, float ri) { return schlick(c, ri); }
float gko_gt_tonemap(float x) { return gt_tonemap(x); }
int gko_exact_tri(const float o[3], const float d[3], const float v[9], double out[3]) {
    RayShear sh = make_shear(f3{d[0], d[1], d[2]});
    ExactHit x = exact_test(f3{o[0], o[1], o[2]}, sh, f3{v[0], v[1], v[2]}, f3{v[3], v[4], v[5]}, f3{v[6], v[7], v[8]});
    out[0] = x.t; out[1] = x.b1; out[2] = x.b2;
    return x.hit ? 1 : 0;
}
// out: t, e (sheared bound), b1, b2, plane t, plane e, plane ok
int gko_fp32_tri(const float o[3], const float d[3], const float v[9], float out[7]) {
    RayShear sh = make_shear(f3{d[0], d[1], d[2]});
    f3 O{o[0], o[1], o[2]}, D{d[0], d[1], d[2]}, V0{v[0], v[1], v[2]}, V1{v[3], v[4], v[5]}, V2{v[6], v[7], v[8]};
    Fp32Result r = fp32_test(O, sh, V0, V1, V2);
    out[0] = r.t; out[1] = r.e; out[2] = r.b1; out[3] = r.b2;
    float tp = 0.0f, ep = 0.0f;
    bool ok = r.kind == 1 && plane_interval(O, D, V0, V1, V2, r.e, &tp, &ep);
    out[4] = tp; out[5] = ep; out[6] = ok ? 1.0f : 0.0f;
    return r.kind;
}

}  // extern "C"
