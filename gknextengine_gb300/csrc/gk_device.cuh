// gk_device.cuh — device-side scalar math of the path-tracing pass (sm_103a).
//
// Translation units that include this file are compiled with -fmad=false: no multiply-add
// is fused unless it is written as __fmaf_rn here, and division/sqrt are the IEEE-rounded
// forms. The float results of shading are therefore a fixed function of the inputs,
// independent of the compiler's scheduling choices; the CPU oracle checks them
// bit-for-bit.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace gk {

#define GK_D __device__ __forceinline__
#define GK_HD __host__ __device__ __forceinline__

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

GK_D float fmaf_(float a, float b, float c) { return __fmaf_rn(a, b, c); }
GK_D float div_(float a, float b) { return __fdiv_rn(a, b); }
GK_D float rcp_(float a) { return __frcp_rn(a); }
GK_D float sqrt_(float a) { return __fsqrt_rn(a); }

GK_D f3 F3(float x, float y, float z) { f3 r; r.x = x; r.y = y; r.z = z; return r; }
GK_D f4 F4(float x, float y, float z, float w) { f4 r; r.x = x; r.y = y; r.z = z; r.w = w; return r; }
GK_D f3 xyz(f4 v) { return F3(v.x, v.y, v.z); }
GK_D f3 operator+(f3 a, f3 b) { return F3(a.x + b.x, a.y + b.y, a.z + b.z); }
GK_D f3 operator-(f3 a, f3 b) { return F3(a.x - b.x, a.y - b.y, a.z - b.z); }
GK_D f3 operator*(f3 a, float s) { return F3(a.x * s, a.y * s, a.z * s); }
GK_D f3 operator-(f3 a) { return F3(-a.x, -a.y, -a.z); }
GK_D f4 operator*(f4 a, f4 b) { return F4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
GK_D f4 operator+(f4 a, f4 b) { return F4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
GK_D f4 operator*(f4 a, float s) { return F4(a.x * s, a.y * s, a.z * s, a.w * s); }
GK_D f4 ldf4(const float4* p) { float4 v = __ldg(p); return F4(v.x, v.y, v.z, v.w); }

// dot: z*z' + (y*y' + x*x'), fused from the inside out
GK_D float dot3(f3 a, f3 b) { return fmaf_(a.z, b.z, fmaf_(a.y, b.y, a.x * b.x)); }
GK_D float len3(f3 a) { return sqrt_(dot3(a, a)); }
GK_D f3 normalize3(f3 a) { float k = div_(1.0f, sqrt_(dot3(a, a))); return a * k; }
GK_D f3 fma3(f3 v, float s, f3 o) { return F3(fmaf_(v.x, s, o.x), fmaf_(v.y, s, o.y), fmaf_(v.z, s, o.z)); }
// cross: each component a*b - c*d with the product fused into the difference
GK_D f3 cross3(f3 a, f3 b) {
    return F3(fmaf_(a.y, b.z, -(a.z * b.y)), fmaf_(a.z, b.x, -(a.x * b.z)), fmaf_(a.x, b.y, -(a.y * b.x)));
}
GK_D f3 reflect3(f3 d, f3 n) {
    float k = 2.0f * dot3(n, d);
    return F3(fmaf_(-k, n.x, d.x), fmaf_(-k, n.y, d.y), fmaf_(-k, n.z, d.z));
}
GK_D f3 refract3(f3 I, f3 N, float eta) {
    float dni = dot3(N, I);
    float t1 = fmaf_(-dni, dni, 1.0f);
    float k = fmaf_(-(eta * eta), t1, 1.0f);
    if (k < 0.0f) return F3(0.0f, 0.0f, 0.0f);
    float s = fmaf_(eta, dni, sqrt_(k));
    return F3(fmaf_(eta, I.x, -(s * N.x)), fmaf_(eta, I.y, -(s * N.y)), fmaf_(eta, I.z, -(s * N.z)));
}
GK_D float sat(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
GK_D float mx(float a, float b) { return a > b ? a : b; }
GK_D float mn(float a, float b) { return a < b ? a : b; }

// column-major 4x4 (glm memory order) times a 4-vector; row r accumulates x, y, z, w in that order
GK_D f4 mat4v(const float* m, f4 v) {
    float o[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = fmaf_(m[12 + r], v.w, fmaf_(m[8 + r], v.z, fmaf_(m[4 + r], v.y, m[r] * v.x)));
    return F4(o[0], o[1], o[2], o[3]);
}
// affine 3x4 row-major: point / direction / transpose-3x3 (normal with the inverse)
GK_D f3 xpoint(const float* m, f3 p) {
    return F3(fmaf_(m[0], p.x, fmaf_(m[1], p.y, fmaf_(m[2], p.z, m[3]))),
              fmaf_(m[4], p.x, fmaf_(m[5], p.y, fmaf_(m[6], p.z, m[7]))),
              fmaf_(m[8], p.x, fmaf_(m[9], p.y, fmaf_(m[10], p.z, m[11]))));
}
GK_D f3 xvector(const float* m, f3 v) {
    return F3(fmaf_(m[0], v.x, fmaf_(m[1], v.y, m[2] * v.z)),
              fmaf_(m[4], v.x, fmaf_(m[5], v.y, m[6] * v.z)),
              fmaf_(m[8], v.x, fmaf_(m[9], v.y, m[10] * v.z)));
}
GK_D f3 xnormal(const float* w, f3 n) {
    return F3(fmaf_(w[8], n.z, fmaf_(w[4], n.y, w[0] * n.x)),
              fmaf_(w[9], n.z, fmaf_(w[5], n.y, w[1] * n.x)),
              fmaf_(w[10], n.z, fmaf_(w[6], n.y, w[2] * n.x)));
}

// ---- PCG4D (Const_Func.slang:227-258) ----
struct Rng { uint32_t v[4]; };
GK_D void pcg4d(Rng& s) {
    uint32_t a = s.v[0] * 1664525u + 1013904223u, b = s.v[1] * 1664525u + 1013904223u;
    uint32_t c = s.v[2] * 1664525u + 1013904223u, d = s.v[3] * 1664525u + 1013904223u;
    a += b * d; b += c * a; c += a * b; d += b * c;
    a ^= a >> 16; b ^= b >> 16; c ^= c >> 16; d ^= d >> 16;
    a += b * d; b += c * a; c += a * b; d += b * c;
    s.v[0] = a; s.v[1] = b; s.v[2] = c; s.v[3] = d;
}
GK_D float u2f(uint32_t x) { return __uint_as_float(0x3f800000u | (x >> 9)) - 1.0f; }
GK_D float rnd1(Rng& s) { pcg4d(s); return u2f(s.v[0]); }
GK_D f2 rnd2(Rng& s) { pcg4d(s); f2 r; r.x = u2f(s.v[0]); r.y = u2f(s.v[1]); return r; }

// ---- sin/cos: Taylor series to x^9 / x^10 on |x| <= pi/4 (error below 2^-27 before
// rounding), Horner with fused steps; 2*pi*u through an exact quadrant split. Our own
// routine, so that CPU checks round the same way. ----
GK_D void sincos_poly(float x, float& s, float& c) {
    float x2 = x * x;
    float ps = fmaf_(x2, 2.75573192e-06f, -1.98412698e-04f);
    ps = fmaf_(x2, ps, 8.33333358e-03f);
    ps = fmaf_(x2, ps, -1.66666672e-01f);
    s = fmaf_(x * x2, ps, x);
    float pc = fmaf_(x2, -2.75573192e-07f, 2.48015876e-05f);
    pc = fmaf_(x2, pc, -1.38888892e-03f);
    pc = fmaf_(x2, pc, 4.16666679e-02f);
    pc = fmaf_(x2, pc, -0.5f);
    c = fmaf_(x2, pc, 1.0f);
}
GK_D void sincos2pi(float u, float& s, float& c) {
    float v = 4.0f * u;
    float q = rintf(v);
    float x = (v - q) * 1.57079637f;
    float sp, cp;
    sincos_poly(x, sp, cp);
    int qi = ((int)q) & 3;
    if (qi == 0) { s = sp; c = cp; }
    else if (qi == 1) { s = cp; c = -sp; }
    else if (qi == 2) { s = -sp; c = -cp; }
    else { s = -cp; c = sp; }
}

// ---- atan2 and acos for the sky's equirectangular lookup (SampleIBLV2). atan on [0, 1]:
// above tan(pi/12) the argument is reduced by atan(a) = pi/6 + atan((a sqrt3 - 1) / (a + sqrt3)),
// then the Taylor series x - x^3/3 + ... - x^15/15 on |x| <= tan(pi/12) (truncation below
// 2^-36), Horner with fused steps; octant fix-ups give atan2; acos(x) = atan2(sqrt((1 - x)
// (1 + x)), x). Our own routines, so that CPU checks round the same way. ----
GK_D float atan01(float a) {
    const bool red = a > 0.267949194f;
    const float x = red ? div_(fmaf_(a, 1.73205081f, -1.0f), a + 1.73205081f) : a;
    const float x2 = x * x;
    float p = fmaf_(x2, -6.66666701e-02f, 7.69230798e-02f);   // -1/15, 1/13
    p = fmaf_(x2, p, -9.09090936e-02f);                        // -1/11
    p = fmaf_(x2, p, 1.11111112e-01f);                         //  1/9
    p = fmaf_(x2, p, -1.42857149e-01f);                        // -1/7
    p = fmaf_(x2, p, 2.00000003e-01f);                         //  1/5
    p = fmaf_(x2, p, -3.33333343e-01f);                        // -1/3
    const float r = fmaf_(x * x2, p, x);
    return red ? r + 0.523598790f : r;                         // + pi/6
}
GK_D float atan2_(float y, float x) {
    const float ax = fabsf(x), ay = fabsf(y);
    if (!(ax > 0.0f) && !(ay > 0.0f)) return 0.0f;
    const bool swap = ay > ax;
    float r = atan01(swap ? div_(ax, ay) : div_(ay, ax));
    if (swap) r = 1.57079637f - r;                             // pi/2 - r
    if (x < 0.0f) r = 3.14159274f - r;                         // pi - r
    return y < 0.0f ? -r : r;
}
GK_D float acos_(float x) {
    const float s = sqrt_(mx((1.0f - x) * (1.0f + x), 0.0f));
    return atan2_(s, x);
}

// ---- samplers (Const_Func.slang:8-49, 260-340) ----
GK_D void onb(f3 n, f3& b1, f3& b2) {
    float sz = n.z < 0.0f ? -1.0f : 1.0f;
    float a = div_(-1.0f, sz + n.z);
    b2 = F3((n.x * n.y) * a, fmaf_(n.y * n.y, a, sz), -n.y);
    b1 = F3(fmaf_((sz * n.x) * n.x, a, 1.0f), sz * b2.x, -sz * n.x);
}
GK_D f3 to_world(f3 v, f3 T, f3 B, f3 N) {
    return F3(fmaf_(v.z, N.x, fmaf_(v.y, B.x, v.x * T.x)), fmaf_(v.z, N.y, fmaf_(v.y, B.y, v.x * T.y)),
              fmaf_(v.z, N.z, fmaf_(v.y, B.z, v.x * T.z)));
}
GK_D f3 align_normal(f3 v, f3 n) { f3 T, B; onb(n, T, B); return to_world(v, T, B, n); }
GK_D f3 hemisphere_cos(Rng& s) {
    f2 u = rnd2(s);
    float sn, cs;
    sincos2pi(u.x, sn, cs);
    float r = sqrt_(u.y);
    return F3(r * cs, r * sn, sqrt_(1.0f - u.y));
}
GK_D f3 cone(Rng& s, float cos_theta) {
    f2 u = rnd2(s);
    float sn, cs;
    sincos2pi(u.x, sn, cs);
    float ct = fmaf_(u.y, cos_theta - 1.0f, 1.0f);
    float r = sqrt_(fmaf_(-ct, ct, 1.0f));
    return F3(r * cs, r * sn, ct);
}
GK_D f2 unit_disk(Rng& s) {
    f2 u = rnd2(s);
    float ox = u.x + (u.x - 1.0f), oy = u.y + (u.y - 1.0f);
    f2 r;
    if ((ox > -1e-35f && ox < 1e-35f) && (oy > -1e-35f && oy < 1e-35f)) { r.x = 0.0f; r.y = 0.0f; return r; }
    const float pi4 = 0.785398163397448309616f;
    float sn, cs;
    if (fabsf(ox) > fabsf(oy)) {
        sincos_poly(div_(pi4 * oy, ox), sn, cs);
        r.x = ox * cs; r.y = ox * sn;
        return r;
    }
    sincos_poly(div_(pi4 * ox, oy), sn, cs);
    r.x = oy * sn;
    r.y = oy * sqrt_(fmaf_(-sn, sn, 1.0f));
    return r;
}
// Bounded VNDF sampling of GGX (Eto and Tokuyoshi 2023), Const_Func.slang:310-328
GK_D f3 ggx_vndf(float alpha, f3 wi_, f2 uv) {
    f3 wi = normalize3(F3(wi_.x * alpha, wi_.y * alpha, wi_.z));
    float b = wi.z;
    if (wi_.z > 0.0f) {
        float a = sat(alpha);
        float lxy = sqrt_(fmaf_(wi_.y, wi_.y, wi_.x * wi_.x));
        float aw = div_(a * wi_.z, 1.0f + lxy);
        b = b * div_(fmaf_(-a, a, 1.0f), fmaf_(aw, aw, 1.0f));
    }
    float z = fmaf_(1.0f - uv.y, 1.0f + b, -b);
    float sn, cs;
    sincos2pi(uv.x, sn, cs);
    float r = sqrt_(sat(fmaf_(-z, z, 1.0f)));
    f3 m = wi + F3(r * cs, r * sn, z);
    return normalize3(F3(m.x * alpha, m.y * alpha, m.z));
}
GK_D f3 ggx_sample(Rng& s, float roughness, f3 n) {
    f3 T, B;
    onb(n, T, B);
    f3 loc = F3(dot3(T, n), dot3(B, n), dot3(n, n));
    f2 uv = rnd2(s);
    return to_world(ggx_vndf(roughness * roughness, loc, uv), T, B, n);
}
GK_D float schlick(float cosine, float ri) {
    float r0 = div_(1.0f - ri, 1.0f + ri);
    r0 = r0 * r0;
    float x = 1.0f - cosine;
    float p5 = (((x * x) * x) * x) * x;
    return fmaf_(1.0f - r0, p5, r0);
}

}  // namespace gk
