// gk_trace.cuh — two-level BVH traversal with an exact closest-hit contract (sm_103a).
//
// Replaces the RT-core RayQuery of FHardwareRayTracerV2 (assets/shaders/common/
// Shading.slang:737-826). GB300 has no RT cores, so traversal is software: 64-byte
// two-child nodes read as four 16-byte vector loads, 48-byte triangles in leaf order,
// a per-thread stack in shared memory (strided by the block size, conflict-free) and a
// marker entry for the hand-over from the instance level to the mesh level.
//
// Hit contract. The reported hit is the minimum of (t, instance index, primitive index)
// under an FP64 evaluation of the watertight ray/triangle test (Woop, Benthin, Wald,
// JCGT 2013) on the FP32 object-space ray. The kernel computes in FP32 with certified
// error bounds and uses FP64 only where the bounds do not decide:
//   * edge functions U, V, W within their error bound of zero -> FP64 test;
//   * t within its error bound of tmin/tmax -> FP64 t;
//   * two hits whose t-intervals overlap -> the ray is traced again with every candidate
//     decided in FP64 (exact mode).
// Box tests widen the slab interval by 1e-6 relative (> 2.5 gamma_3), so no box holding
// the FP64 winner is culled. The float t and barycentrics used for shading are those of
// the FP32 test when it is certain, else the rounded FP64 values.
#pragma once
#include "gk_device.cuh"

namespace gk {

struct __align__(16) BvhNode {
    float4 a;   // c0.lo.x c0.lo.y c0.lo.z c0.hi.x
    float4 b;   // c0.hi.y c0.hi.z c1.lo.x c1.lo.y
    float4 c;   // c1.lo.z c1.hi.x c1.hi.y c1.hi.z
    int4 d;     // ref0 ref1 - -   (ref >= 0: interior node; ref < 0: ~(payload << 3 | count-1))
};

struct __align__(16) DevInst {
    float winv[12];       // world -> object rows
    int blas_root;        // interior node index of the mesh BVH
    uint32_t index_offset;
    uint32_t vertex_offset;
    uint32_t instance_id;
};

constexpr int kStackSize = 64;
constexpr int kRefPop = 0x7FFFFFFE;
constexpr int kRefMarker = 0x7FFFFFFF;
constexpr int kIterCap = 1 << 22;
constexpr uint32_t kErrStack = 1u, kErrIter = 2u;

// Per-thread event counts, flushed once per warp at the end of a kernel.
struct Counters {
    uint32_t rays, fallbacks, retraces, nodes, tris;
};

struct SceneView {
    const BvhNode* nodes;
    const float4* tris;     // 3 float4 per triangle, v0.w = primitive index bits
    const DevInst* inst;
    int tlas_root;          // -1: empty scene
    uint32_t* error;
};

struct Shear {
    int kx, ky, kz;
    float Sx, Sy, Sz;
    double Sxd, Syd, Szd;
};

GK_D float pick(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

GK_D Shear make_shear(f3 d) {
    Shear s;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    float am = ax;
    if (ay > am) { kz = 1; am = ay; }
    if (az > am) { kz = 2; }
    int kx = kz == 2 ? 0 : kz + 1;
    int ky = kx == 2 ? 0 : kx + 1;
    float dz = pick(d, kz);
    if (dz < 0.0f) { int t = kx; kx = ky; ky = t; }
    float dx = pick(d, kx), dy = pick(d, ky);
    s.kx = kx; s.ky = ky; s.kz = kz;
    s.Sx = div_(dx, dz);
    s.Sy = div_(dy, dz);
    s.Sz = rcp_(dz);
    s.Sxd = (double)dx / (double)dz;
    s.Syd = (double)dy / (double)dz;
    s.Szd = 1.0 / (double)dz;
    return s;
}

struct ExactHit { bool hit; double t, b1, b2; };

// FP64 watertight test; products and sums rounded in double, nothing fused.
GK_D ExactHit exact_test(f3 o, const Shear& s, f3 v0, f3 v1, f3 v2) {
    ExactHit r; r.hit = false; r.t = 0.0; r.b1 = 0.0; r.b2 = 0.0;
    double Ak = (double)pick(v0, s.kz) - (double)pick(o, s.kz);
    double Bk = (double)pick(v1, s.kz) - (double)pick(o, s.kz);
    double Ck = (double)pick(v2, s.kz) - (double)pick(o, s.kz);
    double Ax = ((double)pick(v0, s.kx) - (double)pick(o, s.kx)) - s.Sxd * Ak;
    double Ay = ((double)pick(v0, s.ky) - (double)pick(o, s.ky)) - s.Syd * Ak;
    double Bx = ((double)pick(v1, s.kx) - (double)pick(o, s.kx)) - s.Sxd * Bk;
    double By = ((double)pick(v1, s.ky) - (double)pick(o, s.ky)) - s.Syd * Bk;
    double Cx = ((double)pick(v2, s.kx) - (double)pick(o, s.kx)) - s.Sxd * Ck;
    double Cy = ((double)pick(v2, s.ky) - (double)pick(o, s.ky)) - s.Syd * Ck;
    double U = Cx * By - Cy * Bx;
    double V = Ax * Cy - Ay * Cx;
    double W = Bx * Ay - By * Ax;
    bool in = (U >= 0.0 && V >= 0.0 && W >= 0.0) || (U <= 0.0 && V <= 0.0 && W <= 0.0);
    if (!in) return r;
    double det = U + V + W;
    if (det == 0.0) return r;
    double T = U * (s.Szd * Ak) + V * (s.Szd * Bk) + W * (s.Szd * Ck);
    r.hit = true;
    r.t = T / det;
    r.b1 = V / det;
    r.b2 = W / det;
    return r;
}

struct Fp32Hit { int kind; float t, e, b1, b2; };   // kind: 0 certain miss, 1 certain hit, 2 undecided

// FP32 test with certified bounds on U, V, W (first order: 3.02u x magnitude x lateral
// offset) and on t. Unit roundoff u = 2^-24.
GK_D Fp32Hit fp32_test(f3 o, const Shear& s, f3 v0, f3 v1, f3 v2) {
    const float kU = 5.9604645e-08f;
    Fp32Hit r; r.kind = 0; r.t = 0.0f; r.e = 0.0f; r.b1 = 0.0f; r.b2 = 0.0f;
    f3 a = v0 - o, b = v1 - o, c = v2 - o;
    float akx = pick(a, s.kx), aky = pick(a, s.ky), akz = pick(a, s.kz);
    float bkx = pick(b, s.kx), bky = pick(b, s.ky), bkz = pick(b, s.kz);
    float ckx = pick(c, s.kx), cky = pick(c, s.ky), ckz = pick(c, s.kz);
    float Ax = fmaf_(-s.Sx, akz, akx), Ay = fmaf_(-s.Sy, akz, aky);
    float Bx = fmaf_(-s.Sx, bkz, bkx), By = fmaf_(-s.Sy, bkz, bky);
    float Cx = fmaf_(-s.Sx, ckz, ckx), Cy = fmaf_(-s.Sy, ckz, cky);
    float U = fmaf_(Cx, By, -(Cy * Bx));
    float V = fmaf_(Ax, Cy, -(Ay * Cx));
    float W = fmaf_(Bx, Ay, -(By * Ax));
    float aSx = fabsf(s.Sx), aSy = fabsf(s.Sy);
    float mAx = fmaf_(aSx, fabsf(akz), fabsf(akx)), mAy = fmaf_(aSy, fabsf(akz), fabsf(aky));
    float mBx = fmaf_(aSx, fabsf(bkz), fabsf(bkx)), mBy = fmaf_(aSy, fabsf(bkz), fabsf(bky));
    float mCx = fmaf_(aSx, fabsf(ckz), fabsf(ckx)), mCy = fmaf_(aSy, fabsf(ckz), fabsf(cky));
    // first-order error: magnitude x lateral offset (3.02u), second order 9.2u^2 magnitude^2,
    // product/result rounding u|Cy Bx| + 1.01u|U|; constants rounded up to 4u, 16u^2, 2u
    const float kA = 4.0f * kU, kB = 2.0f * kU, kC = 16.0f * kU * kU;
    float eU = fmaf_(kA, fmaf_(mCx, fabsf(By), fmaf_(fabsf(Cx), mBy, fmaf_(mCy, fabsf(Bx), fabsf(Cy) * mBx))),
                     fmaf_(kC, fmaf_(mCx, mBy, mCy * mBx), kB * (fabsf(Cy * Bx) + fabsf(U))));
    float eV = fmaf_(kA, fmaf_(mAx, fabsf(Cy), fmaf_(fabsf(Ax), mCy, fmaf_(mAy, fabsf(Cx), fabsf(Ay) * mCx))),
                     fmaf_(kC, fmaf_(mAx, mCy, mAy * mCx), kB * (fabsf(Ay * Cx) + fabsf(V))));
    float eW = fmaf_(kA, fmaf_(mBx, fabsf(Ay), fmaf_(fabsf(Bx), mAy, fmaf_(mBy, fabsf(Ax), fabsf(By) * mAx))),
                     fmaf_(kC, fmaf_(mBx, mAy, mBy * mAx), kB * (fabsf(By * Ax) + fabsf(W))));
    bool pos = (U > eU) || (V > eV) || (W > eW);
    bool ng = (U < -eU) || (V < -eV) || (W < -eW);
    if (pos && ng) return r;
    bool allpos = (U > eU) && (V > eV) && (W > eW);
    bool allneg = (U < -eU) && (V < -eV) && (W < -eW);
    if (!(allpos || allneg)) { r.kind = 2; return r; }
    float det = (U + V) + W;
    float adet = fabsf(det);
    float ED = fmaf_(2.01f * kU, adet, (eU + eV) + eW);
    if (ED >= 0.5f * adet) { r.kind = 2; return r; }
    float Az = s.Sz * akz, Bz = s.Sz * bkz, Cz = s.Sz * ckz;
    float T = fmaf_(W, Cz, fmaf_(V, Bz, U * Az));
    float t = div_(T, det);
    float aAz = fabsf(Az), aBz = fabsf(Bz), aCz = fabsf(Cz);
    float sumUZ = fmaf_(fabsf(W), aCz, fmaf_(fabsf(V), aBz, fabsf(U) * aAz));
    float ET = fmaf_(6.1f * kU, sumUZ, fmaf_(eW, aCz, fmaf_(eV, aBz, eU * aAz)));
    float at = fabsf(t);
    float e = 1.25f * div_(fmaf_(at, ED, ET), adet - ED);
    e = fmaf_(4.0f * kU, at, e);
    r.kind = 1;
    r.t = t;
    r.e = e;
    r.b1 = div_(V, det);
    r.b2 = div_(W, det);
    return r;
}

GK_D f3 safe_inv(f3 d) {
    float x = fabsf(d.x) < 1e-20f ? copysignf(1e-20f, d.x) : d.x;
    float y = fabsf(d.y) < 1e-20f ? copysignf(1e-20f, d.y) : d.y;
    float z = fabsf(d.z) < 1e-20f ? copysignf(1e-20f, d.z) : d.z;
    return F3(rcp_(x), rcp_(y), rcp_(z));
}

// Slab test widened by 1e-6 relative; tcull already carries the same widening.
GK_D bool slab(float lx, float ly, float lz, float hx, float hy, float hz, f3 o, f3 inv, float tmin, float tcull,
               float& tnear) {
    float t0x = (lx - o.x) * inv.x, t1x = (hx - o.x) * inv.x;
    float t0y = (ly - o.y) * inv.y, t1y = (hy - o.y) * inv.y;
    float t0z = (lz - o.z) * inv.z, t1z = (hz - o.z) * inv.z;
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fmaxf(t0z, t1z)) * 1.000001f;
    tnear = tn;
    return tn <= fminf(tf, tcull);
}

struct TraceOut {
    bool hit;
    bool ambiguous;
    uint32_t inst, prim, tri;
};

enum { kClosest = 0, kAny = 1, kExact = 2 };

GK_D f3 tri_v(const float4* tris, uint32_t ti, int k, uint32_t* prim = nullptr) {
    float4 v = __ldg(&tris[3 * ti + k]);
    if (prim) *prim = __float_as_uint(v.w);
    return F3(v.x, v.y, v.z);
}

// MODE kClosest: interval bookkeeping, returns ambiguous on overlapping candidates.
// MODE kAny:     first valid hit.
// MODE kExact:   every candidate decided in FP64, key (t, inst, prim).
template <int MODE>
GK_D TraceOut traverse(const SceneView& S, f3 wo, f3 wd, float tmin, float tmax, uint32_t* stk, int stride,
                       Counters& cn) {
    TraceOut R;
    R.hit = false; R.ambiguous = false; R.inst = 0xFFFFFFFFu; R.prim = 0xFFFFFFFFu; R.tri = 0xFFFFFFFFu;
    if (S.tlas_root < 0) return R;
    float best_lo = 0.0f, best_hi = 0.0f;
    double best_td = 0.0;
    float tcull = tmax * 1.000001f;
    const double tmind = (double)tmin, tmaxd = (double)tmax;
    const f3 winv = safe_inv(wd);
    f3 o = wo, d = wd, inv = winv;
    Shear sh = make_shear(wd);
    int level = 0;
    uint32_t cur = 0;
    int sp = 0;
    int ref = S.tlas_root;
    int iter = 0;
    for (;;) {
        if (++iter > kIterCap) { atomicOr(S.error, kErrIter); break; }
        if (ref == kRefPop) {
            if (sp == 0) break;
            --sp;
            ref = (int)stk[sp * stride];
            continue;
        }
        if (ref == kRefMarker) {
            o = wo; d = wd; inv = winv; level = 0;
            ref = kRefPop;
            continue;
        }
        if (ref >= 0) {
            ++cn.nodes;
            const float4* np = reinterpret_cast<const float4*>(S.nodes + ref);
            float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
            int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
            float tn0, tn1;
            bool h0 = slab(na.x, na.y, na.z, na.w, nb.x, nb.y, o, inv, tmin, tcull, tn0);
            bool h1 = slab(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, o, inv, tmin, tcull, tn1);
            if (h0 && h1) {
                int nearr = nd.x, farr = nd.y;
                if (tn1 < tn0) { nearr = nd.y; farr = nd.x; }
                if (sp >= kStackSize) { atomicOr(S.error, kErrStack); break; }
                stk[sp * stride] = (uint32_t)farr;
                ++sp;
                ref = nearr;
            } else if (h0) {
                ref = nd.x;
            } else if (h1) {
                ref = nd.y;
            } else {
                ref = kRefPop;
            }
            continue;
        }
        const uint32_t payload = ~(uint32_t)ref;
        if (level == 0) {
            cur = payload >> 3;
            const DevInst* ip = S.inst + cur;
            float w[12];
#pragma unroll
            for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
            o = xpoint(w, wo);
            d = xvector(w, wd);
            inv = safe_inv(d);
            sh = make_shear(d);
            if (sp >= kStackSize) { atomicOr(S.error, kErrStack); break; }
            stk[sp * stride] = (uint32_t)kRefMarker;
            ++sp;
            level = 1;
            ref = __ldg(&ip->blas_root);
            continue;
        }
        const uint32_t first = payload >> 3, cnt = (payload & 7u) + 1u;
        ref = kRefPop;
        for (uint32_t k = 0; k < cnt; ++k) {
            const uint32_t ti = first + k;
            uint32_t prim;
            f3 v0 = tri_v(S.tris, ti, 0, &prim), v1 = tri_v(S.tris, ti, 1), v2 = tri_v(S.tris, ti, 2);
            ++cn.tris;
            Fp32Hit f = fp32_test(o, sh, v0, v1, v2);
            if (f.kind == 0) continue;
            if (MODE == kExact) {
                ExactHit x = exact_test(o, sh, v0, v1, v2);
                ++cn.fallbacks;
                if (!x.hit || !(x.t >= tmind && x.t <= tmaxd)) continue;
                bool better = !R.hit || x.t < best_td ||
                              (x.t == best_td && (cur < R.inst || (cur == R.inst && prim < R.prim)));
                if (better) {
                    R.hit = true; R.inst = cur; R.prim = prim; R.tri = ti;
                    best_td = x.t;
                    tcull = (float)x.t * 1.000001f;
                }
                continue;
            }
            float t, e;
            double td = 0.0;
            bool have_td = false;
            if (f.kind == 2) {
                ExactHit x = exact_test(o, sh, v0, v1, v2);
                ++cn.fallbacks;
                if (!x.hit) continue;
                td = x.t; have_td = true;
                t = (float)x.t;
                e = 2.384185791e-07f * fabsf(t);   // 4u |t|
            } else {
                t = f.t; e = f.e;
            }
            if (t + e < tmin || t - e > tmax) continue;
            if (t - e < tmin || t + e > tmax) {
                if (!have_td) {
                    ExactHit x = exact_test(o, sh, v0, v1, v2);
                    ++cn.fallbacks;
                    td = x.t;
                }
                if (!(td >= tmind && td <= tmaxd)) continue;
            }
            if (MODE == kAny) {
                R.hit = true; R.inst = cur; R.prim = prim; R.tri = ti;
                return R;
            }
            const float lo = t - e, hi = t + e;
            if (R.hit) {
                if (lo > best_hi) continue;
                if (!(hi < best_lo)) { R.ambiguous = true; return R; }
            }
            R.hit = true; R.inst = cur; R.prim = prim; R.tri = ti;
            best_lo = lo; best_hi = hi;
            tcull = hi * 1.000001f;
        }
    }
    return R;
}

// Float t and barycentrics of the winning triangle (the values shading uses).
struct HitShade { float t, b1, b2; };
GK_D HitShade hit_shade(const SceneView& S, f3 wo, f3 wd, uint32_t inst, uint32_t tri) {
    const DevInst* ip = S.inst + inst;
    float w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
    f3 o = xpoint(w, wo), d = xvector(w, wd);
    Shear sh = make_shear(d);
    f3 v0 = tri_v(S.tris, tri, 0), v1 = tri_v(S.tris, tri, 1), v2 = tri_v(S.tris, tri, 2);
    Fp32Hit f = fp32_test(o, sh, v0, v1, v2);
    HitShade h;
    if (f.kind == 1) { h.t = f.t; h.b1 = f.b1; h.b2 = f.b2; return h; }
    ExactHit x = exact_test(o, sh, v0, v1, v2);
    h.t = (float)x.t; h.b1 = (float)x.b1; h.b2 = (float)x.b2;
    return h;
}

// Closest hit under the contract: fast pass, exact re-trace when t-ambiguous.
GK_D TraceOut trace_closest(const SceneView& S, f3 wo, f3 wd, float tmin, float tmax, uint32_t* stk, int stride,
                            Counters& cn) {
    TraceOut r = traverse<kClosest>(S, wo, wd, tmin, tmax, stk, stride, cn);
    if (r.ambiguous) {
        ++cn.retraces;
        r = traverse<kExact>(S, wo, wd, tmin, tmax, stk, stride, cn);
    }
    return r;
}

}  // namespace gk
