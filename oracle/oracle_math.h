// oracle_math.h — scalar float/double helpers for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY. The oracle is the checker of the GB300 kernels and is never
// linked into, imported by or called from the product library.
//
// Arithmetic discipline (so that results are reproducible bit-for-bit on any IEEE host):
// the file is compiled with -ffp-contract=off, and every fused multiply-add is written
// out as std::fmaf; every other operation is a single IEEE-rounded float op in the order
// written. sqrt and division are IEEE (correctly rounded) on every host.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace gko {

struct f2 { float x, y; };
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };

static inline float fma_(float a, float b, float c) { return std::fmaf(a, b, c); }

static inline f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
static inline f4 mk4(float x, float y, float z, float w) { return f4{x, y, z, w}; }
static inline f3 xyz(const f4& v) { return f3{v.x, v.y, v.z}; }

static inline f3 add(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline f3 sub(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline f3 mul(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
static inline f3 neg(f3 a) { return f3{-a.x, -a.y, -a.z}; }
static inline f4 mul4(f4 a, f4 b) { return f4{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
static inline f4 add4(f4 a, f4 b) { return f4{a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
static inline f4 scale4(f4 a, float s) { return f4{a.x * s, a.y * s, a.z * s, a.w * s}; }

// dot(a, b) = fma(a.z, b.z, fma(a.y, b.y, a.x * b.x))
static inline float dot3(f3 a, f3 b) { return fma_(a.z, b.z, fma_(a.y, b.y, a.x * b.x)); }
static inline float length3(f3 a) { return std::sqrt(dot3(a, a)); }
// normalize(v) = v * (1 / sqrt(dot(v, v)))
static inline f3 normalize3(f3 a) {
    float inv = 1.0f / std::sqrt(dot3(a, a));
    return mul(a, inv);
}
// v * s + o, one fma per component
static inline f3 fma3(f3 v, float s, f3 o) { return f3{fma_(v.x, s, o.x), fma_(v.y, s, o.y), fma_(v.z, s, o.z)}; }
// cross(a, b): each component fma(p, q, -(r * s))
static inline f3 cross3(f3 a, f3 b) {
    return f3{fma_(a.y, b.z, -(a.z * b.y)), fma_(a.z, b.x, -(a.x * b.z)), fma_(a.x, b.y, -(a.y * b.x))};
}

// reflect(d, n) = d - 2 dot(n, d) n  ->  fma(-k, n, d), k = 2 dot(n, d)
static inline f3 reflect3(f3 d, f3 n) {
    float k = 2.0f * dot3(n, d);
    return f3{fma_(-k, n.x, d.x), fma_(-k, n.y, d.y), fma_(-k, n.z, d.z)};
}

// refract(I, N, eta), the HLSL/GLSL definition.
static inline f3 refract3(f3 I, f3 N, float eta) {
    float dni = dot3(N, I);
    float t1 = fma_(-dni, dni, 1.0f);
    float k = fma_(-(eta * eta), t1, 1.0f);
    if (k < 0.0f) return f3{0.0f, 0.0f, 0.0f};
    float s = fma_(eta, dni, std::sqrt(k));
    return f3{fma_(eta, I.x, -(s * N.x)), fma_(eta, I.y, -(s * N.y)), fma_(eta, I.z, -(s * N.z))};
}

static inline float saturate(float x) { return x < 0.0f ? 0.0f : (x > 1.0f ? 1.0f : x); }
static inline float fmin_(float a, float b) { return a < b ? a : b; }
static inline float fmax_(float a, float b) { return a > b ? a : b; }

// Column-major 4x4 matrix (glm layout) times a 4-vector:
// r = fma(m[12+r], w, fma(m[8+r], z, fma(m[4+r], y, m[r] * x)))
static inline f4 mat4_mul(const float* m, f4 v) {
    f4 o;
    float* po = &o.x;
    for (int r = 0; r < 4; ++r)
        po[r] = fma_(m[12 + r], v.w, fma_(m[8 + r], v.z, fma_(m[4 + r], v.y, m[r] * v.x)));
    return o;
}

// Row-major affine 3x4 (x' = m0 x + m1 y + m2 z + m3):
// point  : fma(m0, x, fma(m1, y, fma(m2, z, m3)))
// vector : fma(m0, x, fma(m1, y, m2 * z))
static inline f3 xform_point(const float* m, f3 p) {
    return f3{fma_(m[0], p.x, fma_(m[1], p.y, fma_(m[2], p.z, m[3]))),
              fma_(m[4], p.x, fma_(m[5], p.y, fma_(m[6], p.z, m[7]))),
              fma_(m[8], p.x, fma_(m[9], p.y, fma_(m[10], p.z, m[11])))};
}
static inline f3 xform_vector(const float* m, f3 v) {
    return f3{fma_(m[0], v.x, fma_(m[1], v.y, m[2] * v.z)),
              fma_(m[4], v.x, fma_(m[5], v.y, m[6] * v.z)),
              fma_(m[8], v.x, fma_(m[9], v.y, m[10] * v.z))};
}
// transpose of the 3x3 part applied to v (normal transform with the world->object matrix):
// fma(m[8], z, fma(m[4], y, m[0] * x)) per output
static inline f3 xform_normal(const float* winv, f3 n) {
    return f3{fma_(winv[8], n.z, fma_(winv[4], n.y, winv[0] * n.x)),
              fma_(winv[9], n.z, fma_(winv[5], n.y, winv[1] * n.x)),
              fma_(winv[10], n.z, fma_(winv[6], n.y, winv[2] * n.x))};
}

// ---------------------------------------------------------------------------------------
// PCG4D hash RNG (assets/shaders/common/Const_Func.slang:227-258).
static inline void pcg4d(uint32_t v[4]) {
    for (int i = 0; i < 4; ++i) v[i] = v[i] * 1664525u + 1013904223u;
    v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
    for (int i = 0; i < 4; ++i) v[i] = v[i] ^ (v[i] >> 16u);
    v[0] += v[1] * v[3]; v[1] += v[2] * v[0]; v[2] += v[0] * v[1]; v[3] += v[1] * v[2];
}
// uint_to_float: asfloat(0x3f800000 | (x >> 9)) - 1 (Const_Func.slang:235)
static inline float u2f(uint32_t x) {
    uint32_t b = 0x3f800000u | (x >> 9);
    float f;
    std::memcpy(&f, &b, 4);
    return f - 1.0f;
}
static inline float rand1(uint32_t s[4]) { pcg4d(s); return u2f(s[0]); }
static inline f2 rand2(uint32_t s[4]) { pcg4d(s); return f2{u2f(s[0]), u2f(s[1])}; }

// ---------------------------------------------------------------------------------------
// sin and cos from Taylor polynomials on |x| <= pi/4 (truncation below 2^-27), Horner with
// fma. This replaces the vendor sin/cos of the shaders so both sides of a parity check
// round identically. The GPU library carries its own copy of the same mathematics.
static inline void sincos_poly(float x, float* s, float* c) {
    float x2 = x * x;
    float ps = fma_(x2, 2.75573192e-06f, -1.98412698e-04f);   //  1/9!, -1/7!
    ps = fma_(x2, ps, 8.33333358e-03f);                       //  1/5!
    ps = fma_(x2, ps, -1.66666672e-01f);                      // -1/3!
    *s = fma_(x * x2, ps, x);
    float pc = fma_(x2, -2.75573192e-07f, 2.48015876e-05f);   // -1/10!, 1/8!
    pc = fma_(x2, pc, -1.38888892e-03f);                      // -1/6!
    pc = fma_(x2, pc, 4.16666679e-02f);                       //  1/4!
    pc = fma_(x2, pc, -0.5f);                                 // -1/2!
    *c = fma_(x2, pc, 1.0f);
}
// sin(2 pi u), cos(2 pi u) for u in [0, 1]: quadrant from rint(4u), exact remainder.
static inline void sincos_2pi(float u, float* s, float* c) {
    float v = 4.0f * u;
    float q = std::nearbyint(v);
    float r = v - q;
    float x = r * 1.57079637f;  // pi/2 in float
    float sp, cp;
    sincos_poly(x, &sp, &cp);
    int qi = ((int)q) & 3;
    if (qi == 0) { *s = sp; *c = cp; }
    else if (qi == 1) { *s = cp; *c = -sp; }
    else if (qi == 2) { *s = -sp; *c = -cp; }
    else { *s = -cp; *c = sp; }
}

// atan on [0, 1]: above tan(pi/12) reduced by atan(a) = pi/6 + atan((a sqrt3 - 1) / (a + sqrt3)),
// then the Taylor series x - x^3/3 + ... - x^15/15 (Horner with fma); atan2 by octant fix-ups;
// acos(x) = atan2(sqrt((1 - x)(1 + x)), x). The sky lookup of the shading (SampleIBLV2)
// uses these on both sides of the parity check.
static inline float atan01(float a) {
    const bool red = a > 0.267949194f;                                  // tan(pi/12)
    const float x = red ? fma_(a, 1.73205081f, -1.0f) / (a + 1.73205081f) : a;
    const float x2 = x * x;
    float p = fma_(x2, -6.66666701e-02f, 7.69230798e-02f);
    p = fma_(x2, p, -9.09090936e-02f);
    p = fma_(x2, p, 1.11111112e-01f);
    p = fma_(x2, p, -1.42857149e-01f);
    p = fma_(x2, p, 2.00000003e-01f);
    p = fma_(x2, p, -3.33333343e-01f);
    const float r = fma_(x * x2, p, x);
    return red ? r + 0.523598790f : r;
}
static inline float atan2_(float y, float x) {
    const float ax = std::fabs(x), ay = std::fabs(y);
    if (!(ax > 0.0f) && !(ay > 0.0f)) return 0.0f;
    const bool swap = ay > ax;
    float r = atan01(swap ? ax / ay : ay / ax);
    if (swap) r = 1.57079637f - r;
    if (x < 0.0f) r = 3.14159274f - r;
    return y < 0.0f ? -r : r;
}
static inline float acos_(float x) {
    const float s = std::sqrt(fmax_((1.0f - x) * (1.0f + x), 0.0f));
    return atan2_(s, x);
}

}  // namespace gko
