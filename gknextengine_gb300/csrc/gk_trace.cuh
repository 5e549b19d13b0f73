// gk_trace.cuh — two-level BVH traversal with an exact closest-hit contract (sm_103a).
//
// Replaces the RT-core RayQuery of FHardwareRayTracerV2 (assets/shaders/common/
// Shading.slang:737-826). GB300 has no RT cores, so traversal is software, over either of
// the two node formats the builders produce from the same SAH trees:
//   * two-child nodes (64 bytes, four 16-byte loads per node, a stack of node refs): used by
//     the rt pass, whose per-pixel megakernel interleaves shading with traversal and runs
//     fastest with the short node step;
//   * compressed 8-wide nodes (96 bytes, six loads test eight 8-bit child boxes, a stack of
//     sorted node groups): used by the ray-query kernels, where traversal runs alone and the
//     wide nodes halve the node steps of incoherent rays.
// Both keep 48-byte triangles in leaf order, a per-thread stack in shared memory (strided
// by the block size, conflict-free) and a marker entry for the hand-over from the instance
// level to the mesh level.
//
// Hit contract. The reported hit is the minimum of (t, instance index, primitive index)
// under an FP64 evaluation of the watertight ray/triangle test (Woop, Benthin, Wald,
// JCGT 2013) on the FP32 object-space ray. The kernel computes in FP32 with certified
// error bounds and uses FP64 only where the bounds do not decide:
//   * edge functions U, V, W within their error bound of zero -> FP64 test;
//   * t within its error bound of tmin/tmax -> FP64 t;
//   * two hits whose t-intervals overlap -> both are decided in FP64 (the incumbent's
//     triangle is fetched again) and the key is compared exactly.
// Box tests widen the slab interval by 1e-6 relative (> 2.5 gamma_3), so no box holding
// the FP64 winner is culled. A ray component of exactly zero lying on a box face is the one
// case a t-interval widening cannot cover ((hi - o) * inv is 0 there), so the builders store
// every node box widened in space as well (widen_lo / widen_hi): a triangle edge on the
// face stays inside the box the ray is tested against. The 8-bit child boxes of the wide
// nodes decode EXACTLY to planes at or outside those widened boxes (WideNode below), so the
// compression adds boxes, never removes them. The float t and barycentrics used for shading
// are those of the FP32 test when it is certain, else the rounded FP64 values.
#pragma once
#include "gk_device.cuh"

namespace gk {

// Two-child node: the output of the SAH builders, collapsed into WideNode for traversal.
struct __align__(16) BvhNode {
    float4 a;   // c0.lo.x c0.lo.y c0.lo.z c0.hi.x
    float4 b;   // c0.hi.y c0.hi.z c1.lo.x c1.lo.y
    float4 c;   // c1.lo.z c1.hi.x c1.hi.y c1.hi.z
    int4 d;     // ref0 ref1 - -   (ref >= 0: interior node; ref < 0: ~(payload << 3 | count-1))
};

// Compressed 8-wide node. Per axis a scale s = 2^e (-100 <= e <= 38) and an integer origin k
// (|k| < 2^22, origin p = k s exact in float); child slot j's planes are (k + q) s for 8-bit
// q_lo = floor(lo / s) - 1 - k and q_hi = ceil(hi / s) + 1 - k of the child's stored (widened)
// box: every encoded box lies at least one step s outside the box it encodes.
// Traversal evaluates a plane's t as fma(2^23 + q, C, B') with C = s inv (exact) and
// B' = (p - o) inv - 2^23 C (three roundings), whose error is below 5.02u|t| + 0.5001 s|inv|:
// the step margin absorbs the absolute part and the 1e-6 slab widening the relative part, so
// no box holding the exact winner is culled.
struct __align__(16) WideNode {
    float4 h;       // origin p x y z; w bits: 0-7 / 8-15 / 16-23 = e + 127 per axis, 24-31 valid-slot mask
    uint4 q[3];     // per axis: q_lo slots 0-3, q_lo 4-7, q_hi 0-3, q_hi 4-7 (slot j in byte j & 3)
    int4 ref[2];    // slot refs, BvhNode encoding (interior refs index the WideNode array)
};

struct __align__(16) DevInst {
    float winv[12];       // world -> object rows
    int blas_root;        // root BvhNode index of the mesh BVH
    uint32_t index_offset;
    uint32_t vertex_offset;
    uint32_t instance_id;
    int blas_wide_root;   // root WideNode index of the mesh BVH
    uint32_t pad[3];
};

// Node boxes as stored: 1e-6 relative plus 1e-10 absolute beyond the primitives' bounds.
GK_HD float widen_lo(float v) { return v - (fabsf(v) * 1e-6f + 1e-10f); }
GK_HD float widen_hi(float v) { return v + (fabsf(v) * 1e-6f + 1e-10f); }

constexpr int kStackEntries = 24;                // wide node-group entries per thread (3 words each)
constexpr int kStackSize = 3 * kStackEntries;    // 32-bit words per thread; two-child refs: one word each
constexpr int kRefPop = 0x7FFFFFFE;
constexpr int kRefMarker = 0x7FFFFFFF;
constexpr int kIterCap = 1 << 22;
// Speculative traversal (keep taking node steps while a found leaf waits for the leaf phase)
// is measured slower here: a lane stops at its first leaf.
constexpr bool kSpeculative = false;   // measured: 4.01 ms without, 4.16 ms with (1080p bricks)
constexpr uint32_t kErrStack = 1u, kErrIter = 2u;
// (4u is the TMA wait timeout of the post passes, gk_tma.cuh)
constexpr uint32_t kErrRefit = 8u;   // a refit box that the 8-wide nodes cannot quantize
constexpr uint32_t kErrBounds = 16u;  // checked builds: an index outside its array (access skipped)

// Checked builds (GKRT_CHECKED) test every node, triangle and instance index against its array
// before the access; a bad index records kErrBounds, ends the ray and skips the access. The
// default build compiles the checks away.
#ifdef GKRT_CHECKED
#define GK_CHECK_OR_END(ok, S, T, ret)              \
    do {                                            \
        if (!(ok)) {                                \
            atomicOr((S).error, kErrBounds);        \
            (T).done = true;                        \
            (T).has_leaf = false;                   \
            return ret;                             \
        }                                           \
    } while (0)
#else
#define GK_CHECK_OR_END(ok, S, T, ret) \
    do {                               \
    } while (0)
#endif

// Per-thread event counts, flushed once per warp at the end of a kernel. Context counter
// slots: 0 rays, 1 FP64 fallbacks, 2 exact re-traces, 3 node visits, 4 triangle tests,
// 5 hit fetches (closest hits whose vertex, normal, material and instance data were read),
// all per pass; 6 rays since the context was created.
struct Counters {
    uint32_t rays, fallbacks, retraces, nodes, tris, hits;
};

struct SceneView {
    const BvhNode* nodes;   // two-child nodes
    const WideNode* wide;   // the same trees collapsed into 8-wide nodes
    const float4* tris;     // 3 float4 per triangle, v0.w = primitive index bits
    const DevInst* inst;
    int tlas_root;          // two-child root of the instance level, -1: empty scene
    int tlas_wide_root;     // wide root of the instance level
    uint32_t* error;
    uint32_t node_count, wide_count, tri_count, inst_count;   // array sizes (checked builds)
};

struct Shear {
    int kx, ky, kz;
    float Sx, Sy, Sz;
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
    return s;
}

// FP64 shear constants, computed only when an FP64 decision is needed.
struct ShearD { double Sxd, Syd, Szd; };
GK_D ShearD shear_d(f3 d, const Shear& s) {
    const double dz = (double)pick(d, s.kz);
    ShearD r;
    r.Sxd = (double)pick(d, s.kx) / dz;
    r.Syd = (double)pick(d, s.ky) / dz;
    r.Szd = 1.0 / dz;
    return r;
}

struct ExactHit { bool hit; double t, b1, b2; };

// FP64 watertight test; products and sums rounded in double, nothing fused.
// Out of line: taken rarely, and inlining it at every call site bloats the hot kernel.
static __device__ __noinline__ ExactHit exact_test(f3 o, f3 d, Shear s, f3 v0, f3 v1, f3 v2) {
    ExactHit r; r.hit = false; r.t = 0.0; r.b1 = 0.0; r.b2 = 0.0;
    const ShearD sd = shear_d(d, s);
    double Ak = (double)pick(v0, s.kz) - (double)pick(o, s.kz);
    double Bk = (double)pick(v1, s.kz) - (double)pick(o, s.kz);
    double Ck = (double)pick(v2, s.kz) - (double)pick(o, s.kz);
    double Ax = ((double)pick(v0, s.kx) - (double)pick(o, s.kx)) - sd.Sxd * Ak;
    double Ay = ((double)pick(v0, s.ky) - (double)pick(o, s.ky)) - sd.Syd * Ak;
    double Bx = ((double)pick(v1, s.kx) - (double)pick(o, s.kx)) - sd.Sxd * Bk;
    double By = ((double)pick(v1, s.ky) - (double)pick(o, s.ky)) - sd.Syd * Bk;
    double Cx = ((double)pick(v2, s.kx) - (double)pick(o, s.kx)) - sd.Sxd * Ck;
    double Cy = ((double)pick(v2, s.ky) - (double)pick(o, s.ky)) - sd.Syd * Ck;
    double U = Cx * By - Cy * Bx;
    double V = Ax * Cy - Ay * Cx;
    double W = Bx * Ay - By * Ax;
    bool in = (U >= 0.0 && V >= 0.0 && W >= 0.0) || (U <= 0.0 && V <= 0.0 && W <= 0.0);
    if (!in) return r;
    double det = U + V + W;
    if (det == 0.0) return r;
    double T = U * (sd.Szd * Ak) + V * (sd.Szd * Bk) + W * (sd.Szd * Ck);
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

// Certified interval for the exact hit distance, from the plane of the triangle:
// t = dot(n, v0 - o) / dot(n, d), n = (v1 - v0) x (v2 - v0). Its error grows like
// u |t| / cos(theta), while the bound carried by the sheared edge functions grows like
// u |t| * distance / size, far too wide for small distant triangles. Used only to order
// candidates and to check [tmin, tmax]; the shading t stays the sheared FP32 value.
// e_woop (the sheared bound) scaled by 2^-28 covers the FP64 evaluation's own error.
// Returns false when dot(n, d) is not bounded away from zero (grazing).
GK_D bool plane_interval(f3 o, f3 d, f3 v0, f3 v1, f3 v2, float e_woop, float& tp, float& ep) {
    const float kU = 5.9604645e-08f;
    const f3 e1 = v1 - v0, e2 = v2 - v0, w = v0 - o;
    const float nx = fmaf_(e1.y, e2.z, -(e1.z * e2.y));
    const float ny = fmaf_(e1.z, e2.x, -(e1.x * e2.z));
    const float nz = fmaf_(e1.x, e2.y, -(e1.y * e2.x));
    // |n_i - n_i*| <= 3u (|a b| + |c d|) + u |n_i|, rounded up to 4u and 2u
    const float enx = fmaf_(4.0f * kU, fabsf(e1.y * e2.z) + fabsf(e1.z * e2.y), (2.0f * kU) * fabsf(nx));
    const float eny = fmaf_(4.0f * kU, fabsf(e1.z * e2.x) + fabsf(e1.x * e2.z), (2.0f * kU) * fabsf(ny));
    const float enz = fmaf_(4.0f * kU, fabsf(e1.x * e2.y) + fabsf(e1.y * e2.x), (2.0f * kU) * fabsf(nz));
    const float num = fmaf_(nz, w.z, fmaf_(ny, w.y, nx * w.x));
    const float den = fmaf_(nz, d.z, fmaf_(ny, d.y, nx * d.x));
    const float anx = fabsf(nx), any_ = fabsf(ny), anz = fabsf(nz);
    const float awx = fabsf(w.x), awy = fabsf(w.y), awz = fabsf(w.z);
    const float adx = fabsf(d.x), ady = fabsf(d.y), adz = fabsf(d.z);
    const float enum_ = fmaf_(5.0f * kU, fmaf_(anz, awz, fmaf_(any_, awy, anx * awx)),
                              fmaf_(enz, awz, fmaf_(eny, awy, enx * awx)));
    const float eden = fmaf_(4.0f * kU, fmaf_(anz, adz, fmaf_(any_, ady, anx * adx)),
                             fmaf_(enz, adz, fmaf_(eny, ady, enx * adx)));
    const float aden = fabsf(den);
    if (!(aden > 2.0f * eden)) return false;
    tp = div_(num, den);
    const float atp = fabsf(tp);
    ep = fmaf_(1.25f, div_(fmaf_(atp, eden, enum_), aden - eden), fmaf_(4.0f * kU, atp, 3.7252903e-09f * e_woop));
    return true;
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

enum { kClosest = 0, kAny = 1 };

GK_D f3 tri_v(const float4* tris, uint32_t ti, int k, uint32_t* prim = nullptr) {
    float4 v = __ldg(&tris[3 * ti + k]);
    if (prim) *prim = __float_as_uint(v.w);
    return F3(v.x, v.y, v.z);
}

// Resumable traversal state of one ray. The stack lives in shared memory (caller-owned,
// strided); everything else is here, so a ray can be advanced one step at a time and a
// lane can leave the traversal loop and come back.
struct Trav {
    f3 wo, wd, winv;      // world ray and its safe reciprocal direction (restored on leaving an instance)
    f3 o, d, inv;         // ray in the current space (world or instance)
    float tmin;           // read by the ray-query kernels (kRayTmin); the rt pass uses kTmin
    float tmax, tcull, best_lo, best_hi;
    double best_td;
    uint32_t inst, prim, tri;   // current best
    uint32_t cur;               // instance being traversed
    int ref, sp, iter;
    int mode;                   // kClosest / kAny
    uint32_t leaf;              // postponed triangle leaf (payload), valid when has_leaf
    bool hit, best_exact, inblas, done, ambiguous, has_leaf;
};

constexpr float kTmin = 1e-3f;   // EPS, assets/shaders/common/PreProcessor.slang:13

// tmin: the ray's lower bound, honoured by the functions instantiated with kRayTmin (the ray
// queries); the rt pass and the bake kernels trace every ray from EPS and keep it a constant.
template <bool kWide = false>
GK_D void trav_init(Trav& T, const SceneView& S, f3 wo, f3 wd, float tmax, int mode, float tmin = kTmin) {
    T.wo = wo; T.wd = wd; T.o = wo; T.d = wd;
    T.inv = safe_inv(wd);
    T.winv = T.inv;
    T.tmin = tmin;
    T.tmax = tmax;
    T.tcull = tmax * 1.000001f;
    T.best_lo = 0.0f; T.best_hi = 0.0f; T.best_td = 0.0;
    T.inst = 0xFFFFFFFFu; T.prim = 0xFFFFFFFFu; T.tri = 0xFFFFFFFFu;
    T.cur = 0; T.sp = 0; T.iter = 0;
    T.mode = mode;
    T.hit = false; T.best_exact = false; T.inblas = false; T.ambiguous = false;
    T.has_leaf = false; T.leaf = 0u;
    T.ref = kWide ? S.tlas_wide_root : S.tlas_root;
    T.done = T.ref < 0;
}

// FP64 t of the current best candidate: its triangle against its instance's
// object-space ray (recomputed with the same FP32 operations as during traversal).
GK_D double exact_t_of(const Trav& T, const SceneView& S, Shear sh) {
    f3 o = T.o, d = T.d;
    if (!T.inblas || T.inst != T.cur) {
        const DevInst* ip = S.inst + T.inst;
        float w[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
        o = xpoint(w, T.wo);
        d = xvector(w, T.wd);
        sh = make_shear(d);
    }
    const f3 v0 = tri_v(S.tris, T.tri, 0), v1 = tri_v(S.tris, T.tri, 1), v2 = tri_v(S.tris, T.tri, 2);
    return exact_test(o, d, sh, v0, v1, v2).t;
}

// Test the triangles of one leaf against the current best. Returns true when the ray is
// finished early (any-hit found). kRayTmin: the ray's own tmin, else the constant EPS.
template <bool kRayTmin = false>
GK_D bool trav_leaf(Trav& T, const SceneView& S, uint32_t first, uint32_t cnt, Counters& cn) {
    const float tmin = kRayTmin ? T.tmin : kTmin;
    const double tmind = (double)tmin, tmaxd = (double)T.tmax;
    const Shear sh = make_shear(T.d);
    for (uint32_t k = 0; k < cnt; ++k) {
        const uint32_t ti = first + k;
        uint32_t prim;
        const f3 v0 = tri_v(S.tris, ti, 0, &prim), v1 = tri_v(S.tris, ti, 1), v2 = tri_v(S.tris, ti, 2);
        ++cn.tris;
        const Fp32Hit f = fp32_test(T.o, sh, v0, v1, v2);
        if (f.kind == 0) continue;
        float t, e;
        double td = 0.0;
        bool have_td = false;
        if (f.kind == 1 && plane_interval(T.o, T.d, v0, v1, v2, f.e, t, e)) {
            // certified interval from the plane equation
        } else {
            const ExactHit x = exact_test(T.o, T.d, sh, v0, v1, v2);
            ++cn.fallbacks;
            if (!x.hit) continue;
            td = x.t; have_td = true;
            t = (float)x.t;
            e = 2.384185791e-07f * fabsf(t);   // 4u |t|
        }
        if (t + e < tmin || t - e > T.tmax) continue;
        if (t - e < tmin || t + e > T.tmax) {
            if (!have_td) {
                const ExactHit x = exact_test(T.o, T.d, sh, v0, v1, v2);
                ++cn.fallbacks;
                td = x.t; have_td = true;
                t = (float)x.t;
                e = 2.384185791e-07f * fabsf(t);
            }
            if (!(td >= tmind && td <= tmaxd)) continue;
        }
        if (T.mode == kAny) {
            T.hit = true; T.inst = T.cur; T.prim = prim; T.tri = ti;
            return true;
        }
        const float lo = t - e, hi = t + e;
        if (T.hit) {
            if (have_td && T.best_exact) {
                // both FP64: compare the key (t, instance, primitive) exactly
                const bool closer = td < T.best_td ||
                                    (td == T.best_td && (T.cur < T.inst || (T.cur == T.inst && prim < T.prim)));
                if (!closer) continue;
            } else {
                if (lo > T.best_hi) continue;
                if (!(hi < T.best_lo)) {
                    // intervals overlap: decide both in FP64 and compare the key exactly
                    ++cn.retraces;
                    if (!have_td) {
                        const ExactHit x = exact_test(T.o, T.d, sh, v0, v1, v2);
                        ++cn.fallbacks;
                        td = x.t; have_td = true;
                        t = (float)x.t;
                        e = 2.384185791e-07f * fabsf(t);
                    }
                    if (!T.best_exact) {
                        T.best_td = exact_t_of(T, S, sh);
                        T.best_exact = true;
                        ++cn.fallbacks;
                    }
                    const bool closer = td < T.best_td ||
                                        (td == T.best_td && (T.cur < T.inst || (T.cur == T.inst && prim < T.prim)));
                    if (!closer) continue;
                }
            }
        }
        T.hit = true; T.inst = T.cur; T.prim = prim; T.tri = ti;
        T.best_lo = lo; T.best_hi = hi;
        T.best_exact = have_td;
        T.best_td = td;
        T.tcull = hi * 1.000001f;
    }
    return false;
}

// Node phase over two-child nodes ("while-while", Aila and Laine, HPG 2009). One step
// resolves the lane's next reference to a node and tests that node: a pop, the hand-back
// from an instance to the instance level (which pops again: the entries below a marker all
// belong to the instance level) and an instance entry (whose mesh root is then tested) take
// no step of their own, so every step of the warp's node loop is one box test per lane.
// The first triangle leaf found is postponed into T.leaf and the lane waits for the leaf
// phase; so does a lane about to leave the instance of its postponed leaf. Returns true
// while the lane can take another node step.
// cap: the stack's capacity in words (entries); the caller's stack holds at least cap * stride.
template <bool kRayTmin = false>
GK_D bool trav_node_step(Trav& T, const SceneView& S, uint32_t* stk, int stride, Counters& cn, int cap = kStackSize) {
    const float tmin = kRayTmin ? T.tmin : kTmin;
    if (++T.iter > kIterCap) { atomicOr(S.error, kErrIter); T.done = true; return false; }
    int ref = T.ref;
    if (ref == kRefPop) {
        if (T.sp == 0) { T.done = true; return false; }
        --T.sp;
        ref = (int)stk[T.sp * stride];
    }
    if (ref == kRefMarker) {
        if (T.has_leaf) { T.ref = kRefMarker; return false; }   // the postponed leaf needs this instance's ray
        T.o = T.wo; T.d = T.wd; T.inv = T.winv;
        T.inblas = false;
        if (T.sp == 0) { T.done = true; T.ref = kRefPop; return false; }
        --T.sp;
        ref = (int)stk[T.sp * stride];
    }
    if (ref < 0 && !T.inblas) {         // an instance: enter it
        T.cur = ~(uint32_t)ref >> 3;
        GK_CHECK_OR_END(T.cur < S.inst_count, S, T, false);
        const DevInst* ip = S.inst + T.cur;
        float w[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
        T.o = xpoint(w, T.wo);
        T.d = xvector(w, T.wd);
        T.inv = safe_inv(T.d);
        if (T.sp >= cap) { atomicOr(S.error, kErrStack); T.done = true; return false; }
        stk[T.sp * stride] = (uint32_t)kRefMarker;
        ++T.sp;
        T.inblas = true;
        ref = __ldg(&ip->blas_root);
    }
    if (ref < 0) {                      // a triangle leaf: postpone it
        if (T.has_leaf) { T.ref = ref; return false; }   // one postponed leaf at a time
        T.leaf = ~(uint32_t)ref;
        T.has_leaf = true;
        T.ref = kRefPop;
        return kSpeculative;
    }
    GK_CHECK_OR_END((uint32_t)ref < S.node_count, S, T, false);
    ++cn.nodes;
    const float4* np = reinterpret_cast<const float4*>(S.nodes + ref);
    const float4 na = __ldg(np), nb = __ldg(np + 1), nc = __ldg(np + 2);
    const int4 nd = __ldg(reinterpret_cast<const int4*>(np + 3));
    float tn0, tn1;
    const bool h0 = slab(na.x, na.y, na.z, na.w, nb.x, nb.y, T.o, T.inv, tmin, T.tcull, tn0);
    const bool h1 = slab(nb.z, nb.w, nc.x, nc.y, nc.z, nc.w, T.o, T.inv, tmin, T.tcull, tn1);
    if (h0 && h1) {
        int nearr = nd.x, farr = nd.y;
        if (tn1 < tn0) { nearr = nd.y; farr = nd.x; }
        if (T.sp >= cap) { atomicOr(S.error, kErrStack); T.done = true; return false; }
        stk[T.sp * stride] = (uint32_t)farr;
        ++T.sp;
        T.ref = nearr;
    } else if (h0) {
        T.ref = nd.x;
    } else if (h1) {
        T.ref = nd.y;
    } else {
        T.ref = kRefPop;
    }
    return true;
}

// t of byte `b` of `word` (a WideNode plane): fma(2^23 + q, C, B').
GK_D float wide_t(uint32_t word, int b, float C, float Bp) {
    return fmaf_(__uint_as_float(__byte_perm(word, 0x4B000000u, 0x7540u + (uint32_t)b)), C, Bp);
}

GK_D void wide_sort_cx(uint32_t& a, uint32_t& b) {
    const uint32_t lo = min(a, b);
    b = max(a, b);
    a = lo;
}

GK_D void trav_to_world(Trav& T) {
    T.o = T.wo; T.d = T.wd; T.inv = T.winv;
    T.inblas = false;
}

// Node phase of the traversal ("while-while", Aila and Laine, HPG 2009, over 8-wide nodes).
// The group stack holds one entry per wide node with more than one child left to visit:
// three words (node index or kRefMarker; pending slots; t lower bound). Pending word: bits
// 0-2 the count c of slots left, bits 3 + 3i the i-th slot to visit next, nearest first.
// A step pops (dropping groups whose nearest pending child lies beyond the current hit) and
// tests the popped node's eight children in the same call, so the lanes of a warp stay on
// the same instructions. A triangle leaf is postponed into T.leaf and the lane waits for the
// leaf phase; so does a lane about to leave the instance of its postponed leaf. Returns true
// while the lane can take another node step.
GK_D bool trav_node_step_wide(Trav& T, const SceneView& S, uint32_t* stk, int stride, Counters& cn) {
    if (++T.iter > kIterCap) { atomicOr(S.error, kErrIter); T.done = true; return false; }
    int ref = T.ref;
    if (ref == kRefMarker) {            // hand-back deferred until the postponed leaf was tested
        if (T.has_leaf) return false;
        trav_to_world(T);
        ref = kRefPop;
    }
    if (ref == kRefPop) {
        for (;;) {
            if (T.sp == 0) { T.done = true; T.ref = kRefPop; return false; }
            uint32_t* e = stk + 3 * (T.sp - 1) * stride;
            const uint32_t node = e[0];
            if (node == (uint32_t)kRefMarker) {
                --T.sp;
                if (T.has_leaf) { T.ref = kRefMarker; return false; }
                trav_to_world(T);
                continue;
            }
            const uint32_t w = e[stride];
            if (__uint_as_float(e[2 * stride]) > T.tcull) { --T.sp; continue; }
            GK_CHECK_OR_END(node < S.wide_count, S, T, false);
            const uint32_t c = w & 7u, slot = (w >> 3) & 7u;
            if (c <= 1u) --T.sp;
            else e[stride] = ((w >> 3) & ~7u) | (c - 1u);
            ref = __ldg(reinterpret_cast<const int*>(S.wide + node) + 16 + slot);
            break;
        }
    }
    if (ref >= 0) {
        GK_CHECK_OR_END((uint32_t)ref < S.wide_count, S, T, false);
        ++cn.nodes;
        const float4* np = reinterpret_cast<const float4*>(S.wide + ref);
        const float4 h = __ldg(np);
        const uint4 qx = __ldg(reinterpret_cast<const uint4*>(np + 1));
        const uint4 qy = __ldg(reinterpret_cast<const uint4*>(np + 2));
        const uint4 qz = __ldg(reinterpret_cast<const uint4*>(np + 3));
        const uint32_t meta = __float_as_uint(h.w);
        const float Cx = __uint_as_float((meta & 0xFFu) << 23) * T.inv.x;
        const float Cy = __uint_as_float(((meta >> 8) & 0xFFu) << 23) * T.inv.y;
        const float Cz = __uint_as_float(((meta >> 16) & 0xFFu) << 23) * T.inv.z;
        const float Bx = fmaf_(-8388608.0f, Cx, (h.x - T.o.x) * T.inv.x);
        const float By = fmaf_(-8388608.0f, Cy, (h.y - T.o.y) * T.inv.y);
        const float Bz = fmaf_(-8388608.0f, Cz, (h.z - T.o.z) * T.inv.z);
        // near / far plane words by the sign of the direction (the slab min / max)
        const bool nx = T.inv.x < 0.0f, ny = T.inv.y < 0.0f, nz = T.inv.z < 0.0f;
        const uint32_t nx0 = nx ? qx.z : qx.x, nx1 = nx ? qx.w : qx.y, fx0 = nx ? qx.x : qx.z, fx1 = nx ? qx.y : qx.w;
        const uint32_t ny0 = ny ? qy.z : qy.x, ny1 = ny ? qy.w : qy.y, fy0 = ny ? qy.x : qy.z, fy1 = ny ? qy.y : qy.w;
        const uint32_t nz0 = nz ? qz.z : qz.x, nz1 = nz ? qz.w : qz.y, fz0 = nz ? qz.x : qz.z, fz1 = nz ? qz.y : qz.w;
        uint32_t key[8];
        uint32_t nhit = 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            const int b = i & 3;
            const float tnx = wide_t(i < 4 ? nx0 : nx1, b, Cx, Bx), tfx = wide_t(i < 4 ? fx0 : fx1, b, Cx, Bx);
            const float tny = wide_t(i < 4 ? ny0 : ny1, b, Cy, By), tfy = wide_t(i < 4 ? fy0 : fy1, b, Cy, By);
            const float tnz = wide_t(i < 4 ? nz0 : nz1, b, Cz, Bz), tfz = wide_t(i < 4 ? fz0 : fz1, b, Cz, Bz);
            // slab interval widened by 1e-6 relative; T.tcull carries the same widening
            const float tn = fmaxf(fmaxf(tnx, tny), fmaxf(tnz, T.tmin));
            const float tf = fminf(fminf(tfx, tfy), tfz) * 1.000001f;
            const bool hit = ((meta >> (24 + i)) & 1u) && tn <= fminf(tf, T.tcull);
            key[i] = hit ? ((__float_as_uint(tn) & ~7u) | (uint32_t)i) : 0xFFFFFFFFu;
            nhit += hit ? 1u : 0u;
        }
        if (nhit == 0u) {
            T.ref = kRefPop;
            return true;
        }
        // Batcher's odd-even merge sort of the 8 keys (tnear bits, slot in the low bits)
        wide_sort_cx(key[0], key[1]); wide_sort_cx(key[2], key[3]); wide_sort_cx(key[4], key[5]);
        wide_sort_cx(key[6], key[7]); wide_sort_cx(key[0], key[2]); wide_sort_cx(key[1], key[3]);
        wide_sort_cx(key[4], key[6]); wide_sort_cx(key[5], key[7]); wide_sort_cx(key[1], key[2]);
        wide_sort_cx(key[5], key[6]); wide_sort_cx(key[0], key[4]); wide_sort_cx(key[1], key[5]);
        wide_sort_cx(key[2], key[6]); wide_sort_cx(key[3], key[7]); wide_sort_cx(key[2], key[4]);
        wide_sort_cx(key[3], key[5]); wide_sort_cx(key[1], key[2]); wide_sort_cx(key[3], key[4]);
        wide_sort_cx(key[5], key[6]);
        if (nhit > 1u) {
            if (T.sp >= kStackEntries) { atomicOr(S.error, kErrStack); T.done = true; return false; }
            uint32_t w = nhit - 1u;
#pragma unroll
            for (int j = 1; j < 8; ++j) w |= (key[j] & 7u) << (3 * j);
            uint32_t* e = stk + 3 * T.sp * stride;
            e[0] = (uint32_t)ref;
            e[stride] = w;
            e[2 * stride] = key[1] & ~7u;   // <= the nearest pending child's tnear
            ++T.sp;
        }
        const uint32_t s0 = key[0] & 7u;
        const int4 rr = __ldg(reinterpret_cast<const int4*>(np + 4 + (s0 >> 2)));
        ref = (s0 & 2u) ? ((s0 & 1u) ? rr.w : rr.z) : ((s0 & 1u) ? rr.y : rr.x);
        if (ref >= 0) {
            T.ref = ref;
            return true;
        }
        // nearest child is an instance or a triangle leaf: enter or postpone it here
    }
    const uint32_t payload = ~(uint32_t)ref;
    if (!T.inblas) {
        T.cur = payload >> 3;
        GK_CHECK_OR_END(T.cur < S.inst_count, S, T, false);
        const DevInst* ip = S.inst + T.cur;
        float w[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
        T.o = xpoint(w, T.wo);
        T.d = xvector(w, T.wd);
        T.inv = safe_inv(T.d);
        if (T.sp >= kStackEntries) { atomicOr(S.error, kErrStack); T.done = true; return false; }
        uint32_t* e = stk + 3 * T.sp * stride;
        e[0] = (uint32_t)kRefMarker;
        e[stride] = 0u;
        e[2 * stride] = 0u;
        ++T.sp;
        T.inblas = true;
        T.ref = __ldg(&ip->blas_wide_root);
        return true;
    }
    if (T.has_leaf) {                   // one postponed leaf at a time
        T.ref = ref;
        return false;
    }
    T.leaf = payload;
    T.has_leaf = true;
    T.ref = kRefPop;
    return kSpeculative;
}

// Leaf phase: test the postponed leaf's triangles.
template <bool kRayTmin = false>
GK_D void trav_leaf_step(Trav& T, const SceneView& S, Counters& cn) {
    if (!T.has_leaf) return;
    GK_CHECK_OR_END((T.leaf >> 3) + (T.leaf & 7u) + 1u <= S.tri_count, S, T, );
    T.has_leaf = false;
    if (trav_leaf<kRayTmin>(T, S, T.leaf >> 3, (T.leaf & 7u) + 1u, cn)) T.done = true;
}

GK_D bool trav_finished(const Trav& T) { return T.done && !T.has_leaf; }

// Whole-ray traversal on top of the two phases: hits with tmin <= t <= tmax.
template <int MODE, bool kWide = false>
GK_D TraceOut traverse(const SceneView& S, f3 wo, f3 wd, float tmin, float tmax, uint32_t* stk, int stride,
                       Counters& cn) {
    Trav T;
    trav_init<kWide>(T, S, wo, wd, tmax, MODE, tmin);
    while (!trav_finished(T)) {
        if (kWide) {
            while (!T.done && trav_node_step_wide(T, S, stk, stride, cn)) {
            }
        } else {
            while (!T.done && trav_node_step<true>(T, S, stk, stride, cn)) {
            }
        }
        trav_leaf_step<true>(T, S, cn);
    }
    TraceOut R;
    R.hit = T.hit; R.ambiguous = false; R.inst = T.inst; R.prim = T.prim; R.tri = T.tri;
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
    ExactHit x = exact_test(o, d, sh, v0, v1, v2);
    h.t = (float)x.t; h.b1 = (float)x.b1; h.b2 = (float)x.b2;
    return h;
}

// Closest hit under the contract.
GK_D TraceOut trace_closest(const SceneView& S, f3 wo, f3 wd, float tmin, float tmax, uint32_t* stk, int stride,
                            Counters& cn) {
    return traverse<kClosest>(S, wo, wd, tmin, tmax, stk, stride, cn);
}

}  // namespace gk
