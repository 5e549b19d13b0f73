// oracle_isect.h — the FP64 closest-hit definition used as ground truth, and the
// FP32 "hybrid" evaluation of the same triangle test whose float results (t, barycentrics)
// feed shading.
//
// TEST INFRASTRUCTURE ONLY (the checker of the GPU kernels; never part of the product).
//
// Ground truth (FP64): for a ray given in FP32 object-space coordinates, the watertight
// ray/triangle test of Woop, Benthin and Wald (JCGT 2013) evaluated entirely in double:
// shear constants from the dominant direction axis, edge functions U, V, W, a hit when all
// three are >= 0 or all <= 0 with det = U+V+W != 0, t = T/det, valid when tmin <= t <= tmax.
// The closest hit is the minimum of the key (t, instance index, primitive index).
// The reference traverses with RayQuery on RT cores (assets/shaders/common/Shading.slang:
// 784-826), whose tie rules are not specified; this definition replaces them.
//
// Hybrid (FP32, what shading uses): the same test in float with certified error bounds;
// where a sign or the t range is not certain the double result is used. hybrid_eval()
// returns the float t and barycentrics a GPU implementation of the same rules produces.
#pragma once
#include "oracle_math.h"
#include <cfloat>

namespace gko {

struct RayShear {
    int kx, ky, kz;
    float Sx, Sy, Sz;   // FP32 shear constants
    double Sxd, Syd, Szd;
};

static inline RayShear make_shear(f3 d) {
    RayShear s;
    float ad[3] = {std::fabs(d.x), std::fabs(d.y), std::fabs(d.z)};
    int kz = 0;
    if (ad[1] > ad[kz]) kz = 1;
    if (ad[2] > ad[kz]) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    const float dv[3] = {d.x, d.y, d.z};
    if (dv[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    s.kx = kx; s.ky = ky; s.kz = kz;
    s.Sx = dv[kx] / dv[kz];
    s.Sy = dv[ky] / dv[kz];
    s.Sz = 1.0f / dv[kz];
    s.Sxd = (double)dv[kx] / (double)dv[kz];
    s.Syd = (double)dv[ky] / (double)dv[kz];
    s.Szd = 1.0 / (double)dv[kz];
    return s;
}

static inline float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

struct ExactHit {
    bool hit;       // edge test passed and det != 0 (range not applied)
    double t, b1, b2;
};

// The pure FP64 test. No fused operations; products and sums rounded in double.
static inline ExactHit exact_test(f3 o, const RayShear& s, f3 v0, f3 v1, f3 v2) {
    ExactHit r{false, 0.0, 0.0, 0.0};
    double A[3] = {(double)v0.x - (double)o.x, (double)v0.y - (double)o.y, (double)v0.z - (double)o.z};
    double B[3] = {(double)v1.x - (double)o.x, (double)v1.y - (double)o.y, (double)v1.z - (double)o.z};
    double C[3] = {(double)v2.x - (double)o.x, (double)v2.y - (double)o.y, (double)v2.z - (double)o.z};
    double Ax = A[s.kx] - s.Sxd * A[s.kz], Ay = A[s.ky] - s.Syd * A[s.kz];
    double Bx = B[s.kx] - s.Sxd * B[s.kz], By = B[s.ky] - s.Syd * B[s.kz];
    double Cx = C[s.kx] - s.Sxd * C[s.kz], Cy = C[s.ky] - s.Syd * C[s.kz];
    double U = Cx * By - Cy * Bx;
    double V = Ax * Cy - Ay * Cx;
    double W = Bx * Ay - By * Ax;
    bool inside = (U >= 0.0 && V >= 0.0 && W >= 0.0) || (U <= 0.0 && V <= 0.0 && W <= 0.0);
    if (!inside) return r;
    double det = U + V + W;
    if (det == 0.0) return r;
    double Az = s.Szd * A[s.kz], Bz = s.Szd * B[s.kz], Cz = s.Szd * C[s.kz];
    double T = U * Az + V * Bz + W * Cz;
    r.hit = true;
    r.t = T / det;
    r.b1 = V / det;
    r.b2 = W / det;
    return r;
}

// FP32 evaluation with certified bounds (unit roundoff u = 2^-24).
// Result kinds: 0 certain miss, 1 certain hit (t, e valid), 2 uncertain (use FP64).
struct Fp32Result {
    int kind;
    float t, e, b1, b2;
};

static const float kU = 5.9604645e-08f;   // 2^-24

static inline Fp32Result fp32_test(f3 o, const RayShear& s, f3 v0, f3 v1, f3 v2) {
    Fp32Result r{0, 0.0f, 0.0f, 0.0f, 0.0f};
    f3 a = sub(v0, o), b = sub(v1, o), c = sub(v2, o);
    float akx = comp(a, s.kx), aky = comp(a, s.ky), akz = comp(a, s.kz);
    float bkx = comp(b, s.kx), bky = comp(b, s.ky), bkz = comp(b, s.kz);
    float ckx = comp(c, s.kx), cky = comp(c, s.ky), ckz = comp(c, s.kz);
    float Ax = fma_(-s.Sx, akz, akx), Ay = fma_(-s.Sy, akz, aky);
    float Bx = fma_(-s.Sx, bkz, bkx), By = fma_(-s.Sy, bkz, bky);
    float Cx = fma_(-s.Sx, ckz, ckx), Cy = fma_(-s.Sy, ckz, cky);
    float U = fma_(Cx, By, -(Cy * Bx));
    float V = fma_(Ax, Cy, -(Ay * Cx));
    float W = fma_(Bx, Ay, -(By * Ax));
    // magnitudes before cancellation: |p_kx| + |S| |p_kz|
    float aSx = std::fabs(s.Sx), aSy = std::fabs(s.Sy);
    float mAx = fma_(aSx, std::fabs(akz), std::fabs(akx)), mAy = fma_(aSy, std::fabs(akz), std::fabs(aky));
    float mBx = fma_(aSx, std::fabs(bkz), std::fabs(bkx)), mBy = fma_(aSy, std::fabs(bkz), std::fabs(bky));
    float mCx = fma_(aSx, std::fabs(ckz), std::fabs(ckx)), mCy = fma_(aSy, std::fabs(ckz), std::fabs(cky));
    // |U - U_exact| <= 3.02u (mCx|By| + |Cx|mBy + mCy|Bx| + |Cy|mBx)
    //                 + 9.2u^2 (mCx mBy + mCy mBx) + u |Cy Bx| + 1.01u |U|
    // (first-order terms scale with magnitude x lateral offset, not magnitude^2);
    // constants rounded up to 4u, 16u^2 and 2u.
    const float kA = 4.0f * kU, kB = 2.0f * kU, kC = 16.0f * kU * kU;
    float eU = fma_(kA, fma_(mCx, std::fabs(By), fma_(std::fabs(Cx), mBy, fma_(mCy, std::fabs(Bx), std::fabs(Cy) * mBx))),
                    fma_(kC, fma_(mCx, mBy, mCy * mBx), kB * (std::fabs(Cy * Bx) + std::fabs(U))));
    float eV = fma_(kA, fma_(mAx, std::fabs(Cy), fma_(std::fabs(Ax), mCy, fma_(mAy, std::fabs(Cx), std::fabs(Ay) * mCx))),
                    fma_(kC, fma_(mAx, mCy, mAy * mCx), kB * (std::fabs(Ay * Cx) + std::fabs(V))));
    float eW = fma_(kA, fma_(mBx, std::fabs(Ay), fma_(std::fabs(Bx), mAy, fma_(mBy, std::fabs(Ax), std::fabs(By) * mAx))),
                    fma_(kC, fma_(mBx, mAy, mBy * mAx), kB * (std::fabs(By * Ax) + std::fabs(W))));
    bool pos = (U > eU) || (V > eV) || (W > eW);
    bool negc = (U < -eU) || (V < -eV) || (W < -eW);
    if (pos && negc) { r.kind = 0; return r; }
    bool allpos = (U > eU) && (V > eV) && (W > eW);
    bool allneg = (U < -eU) && (V < -eV) && (W < -eW);
    if (!(allpos || allneg)) { r.kind = 2; return r; }
    float det = (U + V) + W;
    float adet = std::fabs(det);
    float ED = fma_(2.01f * kU, adet, (eU + eV) + eW);
    if (ED >= 0.5f * adet) { r.kind = 2; return r; }
    float Az = s.Sz * akz, Bz = s.Sz * bkz, Cz = s.Sz * ckz;
    float T = fma_(W, Cz, fma_(V, Bz, U * Az));
    float t = T / det;
    float aAz = std::fabs(Az), aBz = std::fabs(Bz), aCz = std::fabs(Cz);
    float sumUZ = fma_(std::fabs(W), aCz, fma_(std::fabs(V), aBz, std::fabs(U) * aAz));
    float ET = fma_(6.1f * kU, sumUZ, fma_(eW, aCz, fma_(eV, aBz, eU * aAz)));
    float at = std::fabs(t);
    float e = 1.25f * (fma_(at, ED, ET) / (adet - ED));
    e = fma_(4.0f * kU, at, e);
    r.kind = 1;
    r.t = t;
    r.e = e;
    r.b1 = V / det;
    r.b2 = W / det;
    return r;
}

// Certified interval for the exact hit distance from the plane equation
// t = dot(n, v0 - o) / dot(n, d), n = (v1 - v0) x (v2 - v0); false when dot(n, d) is not
// bounded away from zero. e_woop (the sheared FP32 bound) scaled by 2^-28 covers the
// FP64 evaluation's own rounding.
static inline bool plane_interval(f3 o, f3 d, f3 v0, f3 v1, f3 v2, float e_woop, float* tp, float* ep) {
    f3 e1 = sub(v1, v0), e2 = sub(v2, v0), w = sub(v0, o);
    float nx = fma_(e1.y, e2.z, -(e1.z * e2.y));
    float ny = fma_(e1.z, e2.x, -(e1.x * e2.z));
    float nz = fma_(e1.x, e2.y, -(e1.y * e2.x));
    float enx = fma_(4.0f * kU, std::fabs(e1.y * e2.z) + std::fabs(e1.z * e2.y), (2.0f * kU) * std::fabs(nx));
    float eny = fma_(4.0f * kU, std::fabs(e1.z * e2.x) + std::fabs(e1.x * e2.z), (2.0f * kU) * std::fabs(ny));
    float enz = fma_(4.0f * kU, std::fabs(e1.x * e2.y) + std::fabs(e1.y * e2.x), (2.0f * kU) * std::fabs(nz));
    float num = fma_(nz, w.z, fma_(ny, w.y, nx * w.x));
    float den = fma_(nz, d.z, fma_(ny, d.y, nx * d.x));
    float anx = std::fabs(nx), any_ = std::fabs(ny), anz = std::fabs(nz);
    float awx = std::fabs(w.x), awy = std::fabs(w.y), awz = std::fabs(w.z);
    float adx = std::fabs(d.x), ady = std::fabs(d.y), adz = std::fabs(d.z);
    float enum_ = fma_(5.0f * kU, fma_(anz, awz, fma_(any_, awy, anx * awx)), fma_(enz, awz, fma_(eny, awy, enx * awx)));
    float eden = fma_(4.0f * kU, fma_(anz, adz, fma_(any_, ady, anx * adx)), fma_(enz, adz, fma_(eny, ady, enx * adx)));
    float aden = std::fabs(den);
    if (!(aden > 2.0f * eden)) return false;
    *tp = num / den;
    float atp = std::fabs(*tp);
    *ep = fma_(1.25f, fma_(atp, eden, enum_) / (aden - eden), fma_(4.0f * kU, atp, 3.7252903e-09f * e_woop));
    return true;
}

// Shading values of a triangle known (by the FP64 definition) to be the closest hit:
// float t and barycentrics from the FP32 path when it is certain, else from FP64.
struct HybridHit { float t, b1, b2; bool used_fp64; };
static inline HybridHit hybrid_eval(f3 o, const RayShear& s, f3 v0, f3 v1, f3 v2) {
    Fp32Result f = fp32_test(o, s, v0, v1, v2);
    if (f.kind == 1) return HybridHit{f.t, f.b1, f.b2, false};
    ExactHit x = exact_test(o, s, v0, v1, v2);
    return HybridHit{(float)x.t, (float)x.b1, (float)x.b2, true};
}

}  // namespace gko
