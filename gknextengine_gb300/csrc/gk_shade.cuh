// gk_shade.cuh — the per-pixel path-tracing logic of gkNextRenderer on the GPU.
//
// Follows FPathTracingRendererV2 (assets/shaders/common/Shading.slang:995-1261) with the
// traced camera ray of FHardwarePrimaryRayCaster (Shading.slang:283-334), sun-cone NEE of
// FHardwareDirectIlluminatorV2 (Shading.slang:886-908), probe termination
// interpolateAmbientCubesV2 (assets/shaders/common/AmbientCube.slang:290-382) and the
// sample multiplier of assets/shaders/Core.PathTracing.comp.slang:16-30.
#pragma once
#include "../../include/gkrt.h"
#include "gk_trace.cuh"

namespace gk {

// A texture of the pool: RGBA float texels, rows first to last; null texels: no texture.
struct DevTex {
    const float4* texels;
    uint32_t w, h;
};

struct ShadeScene {
    SceneView S;
    const float4* normals;       // per vertex
    const uint32_t* slots;       // per vertex material slot
    const uint32_t* indices;
    const uint32_t* inst_mat;    // 16 per instance
    const float* inst_prev;      // 24 per instance: combined_prev, then the world transform (3x4)
    const GkrtMaterial* mats;
    uint32_t nmat;
    const uint32_t* cubes;       // optional probe grid
    const uint32_t* voxels;
    const float4* emit;          // emissive triangles, 5 float4 each (see nee_sample)
    const float2* emit_alias;    // alias table: (threshold, alias index bits) per entry
    uint32_t nemit;              // 0: no emissive-triangle NEE
    const DevTex* tex;           // GKRT_MAX_TEXTURES entries (the texture pool)
    const float2* uv;            // per vertex texture coordinates, or null
    const float4* tangents;      // per vertex object-space tangent (w: handedness), or null
};

struct Vtx {
    f3 P, N;
    uint32_t mat;
    uint32_t inst;
};

struct MatV {
    f4 diffuse;
    float fuzz, ri, metal, ri2;
    uint32_t model;
    int dtex, mtex, ntex;   // diffuse, MRA and normal-map texture ids (-1: none)
};

GK_D MatV load_mat(const ShadeScene& sc, uint32_t i) {
    if (i >= sc.nmat) i = sc.nmat - 1;
    const float4* p = reinterpret_cast<const float4*>(sc.mats + i);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    MatV m;
    m.diffuse = F4(a.x, a.y, a.z, a.w);
    m.dtex = __float_as_int(b.x);
    m.mtex = __float_as_int(b.y);
    m.ntex = __float_as_int(b.z);
    m.fuzz = b.w;
    m.ri = c.x;
    m.model = __float_as_uint(c.y);
    m.metal = c.z;
    m.ri2 = c.w;
    return m;
}

// FHardwareRayTracerV2::TraceRay after the query (Shading.slang:801-823): position,
// interpolated shading normal through WorldToObject, and the material of vertex 0's slot.
static __device__ __noinline__ Vtx hit_vertex(const ShadeScene& sc, f3 o, f3 d, uint32_t inst, uint32_t prim, uint32_t tri) {
    const HitShade h = hit_shade(sc.S, o, d, inst, tri);
    const DevInst* ip = sc.S.inst + inst;
    const uint32_t ioff = __ldg(&ip->index_offset) + 3u * prim, voff = __ldg(&ip->vertex_offset);
    const uint32_t i0 = __ldg(&sc.indices[ioff]) + voff, i1 = __ldg(&sc.indices[ioff + 1]) + voff,
                   i2 = __ldg(&sc.indices[ioff + 2]) + voff;
    const float4 a = __ldg(&sc.normals[i0]), b = __ldg(&sc.normals[i1]), c = __ldg(&sc.normals[i2]);
    const f3 n0 = F3(a.x, a.y, a.z), e1 = F3(b.x, b.y, b.z) - n0, e2 = F3(c.x, c.y, c.z) - n0;
    const f3 nobj = F3(fmaf_(e2.x, h.b2, fmaf_(e1.x, h.b1, n0.x)), fmaf_(e2.y, h.b2, fmaf_(e1.y, h.b1, n0.y)),
                       fmaf_(e2.z, h.b2, fmaf_(e1.z, h.b1, n0.z)));
    float w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
    Vtx out;
    out.N = normalize3(xnormal(w, nobj));
    out.P = fma3(d, h.t, o);
    out.mat = __ldg(&sc.inst_mat[16u * inst + (__ldg(&sc.slots[i0]) & 15u)]);
    out.inst = inst;
    return out;
}

GK_D f4 sky(const GkrtFrameConstants& fc) {
    if (!fc.has_sky) return F4(0.0f, 0.0f, 0.0f, 0.0f);
    return F4(mn(10.0f, fc.sky_color[0]), mn(10.0f, fc.sky_color[1]), mn(10.0f, fc.sky_color[2]),
              mn(1.0f, fc.sky_color[3])) * fc.sky_intensity;
}

// ---- textures (the pool's sampler at level 0: Vulkan's linear filter, repeat addressing) ----
// Texel index of the integral float f modulo n (exact: fmodf is exact).
GK_D uint32_t wrap_repeat(float f, uint32_t n) {
    float m = fmodf(f, (float)n);
    if (m < 0.0f) m = m + (float)n;
    const uint32_t i = (uint32_t)m;
    return i < n ? i : 0u;
}
GK_D f4 texel(const DevTex& t, uint32_t x, uint32_t y) {
    const float4 v = __ldg(&t.texels[(size_t)y * t.w + x]);
    return F4(v.x, v.y, v.z, v.w);
}
// SampleLevel(uv, 0): x = u w - 1/2 and y = v h - 1/2 split into texel and fraction, the four
// texels weighted in one fixed order. An id without a texture samples as opaque white.
GK_D f4 tex_sample(const DevTex* pool, int id, float u, float v) {
    const f4 white = F4(1.0f, 1.0f, 1.0f, 1.0f);
    if (id < 0 || id >= (int)GKRT_MAX_TEXTURES) return white;
    DevTex t;
    t.texels = reinterpret_cast<const float4*>(__ldg(reinterpret_cast<const unsigned long long*>(&pool[id].texels)));
    t.w = __ldg(&pool[id].w);
    t.h = __ldg(&pool[id].h);
    if (!t.texels || !t.w || !t.h) return white;
    float x = fmaf_(u, (float)t.w, -0.5f), y = fmaf_(v, (float)t.h, -0.5f);
    if (!(fabsf(x) < 1e30f)) x = -0.5f;   // non-finite coordinates read texel 0's neighbourhood
    if (!(fabsf(y) < 1e30f)) y = -0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float a = x - fx, b = y - fy;
    const uint32_t x0 = wrap_repeat(fx, t.w), x1 = wrap_repeat(fx + 1.0f, t.w);
    const uint32_t y0 = wrap_repeat(fy, t.h), y1 = wrap_repeat(fy + 1.0f, t.h);
    const float ia = 1.0f - a, ib = 1.0f - b;
    const float w00 = ia * ib, w10 = a * ib, w01 = ia * b, w11 = a * b;
    const f4 t00 = texel(t, x0, y0), t10 = texel(t, x1, y0), t01 = texel(t, x0, y1), t11 = texel(t, x1, y1);
    return F4(fmaf_(t11.x, w11, fmaf_(t01.x, w01, fmaf_(t10.x, w10, t00.x * w00))),
              fmaf_(t11.y, w11, fmaf_(t01.y, w01, fmaf_(t10.y, w10, t00.y * w00))),
              fmaf_(t11.z, w11, fmaf_(t01.z, w01, fmaf_(t10.z, w10, t00.z * w00))),
              fmaf_(t11.w, w11, fmaf_(t01.w, w01, fmaf_(t10.w, w10, t00.w * w00))));
}

// Radiance of a sky miss in direction dir: SampleIBLV2 (Shading.slang:194-199) with the
// texture sky_index when the frame asks for it, else the constant colour.
GK_D f4 sky_dir(const ShadeScene& sc, const GkrtFrameConstants& fc, f3 dir) {
    if (!fc.has_sky || !(fc.flags & GKRT_FRAME_SKY_TEXTURE)) return sky(fc);
    const f3 d = normalize3(dir);
    const float u = (atan2_(d.x, d.z) + 3.14159274f * fc.sky_rotation) * 0.159154937f;   // M_1_OVER_TWO_PI
    const float v = acos_(d.y) * 0.318309873f;                                        // M_1_PI
    const f4 c = tex_sample(sc.tex, (int)fc.sky_index, u, v);
    return F4(mn(10.0f, c.x), mn(10.0f, c.y), mn(10.0f, c.z), mn(1.0f, c.w)) * fc.sky_intensity;
}

// Texture coordinates and the object-space normal and tangent at a hit: the barycentric mix
// a + (b - a) b1 + (c - a) b2 of TraceRay (Shading.slang:820) for each. The tangent's w is the
// reference's vertex packing of the handedness, 2 when positive and 0 otherwise
// (MakeVertex, Vertex.hpp:97; UnpackVertexV2, Const_Func.slang:356-364).
struct HitAttr {
    float u, v;
    f3 ln;
    f4 lt;
};
static __device__ __noinline__ HitAttr hit_attr(const ShadeScene& sc, f3 o, f3 d, uint32_t inst, uint32_t prim,
                                                uint32_t tri) {
    const HitShade h = hit_shade(sc.S, o, d, inst, tri);
    const DevInst* ip = sc.S.inst + inst;
    const uint32_t ioff = __ldg(&ip->index_offset) + 3u * prim, voff = __ldg(&ip->vertex_offset);
    const uint32_t i0 = __ldg(&sc.indices[ioff]) + voff, i1 = __ldg(&sc.indices[ioff + 1]) + voff,
                   i2 = __ldg(&sc.indices[ioff + 2]) + voff;
    HitAttr r;
    r.u = 0.0f; r.v = 0.0f;
    r.lt = F4(0.0f, 0.0f, 0.0f, 0.0f);
    if (sc.uv) {
        const float2 a = __ldg(&sc.uv[i0]), b = __ldg(&sc.uv[i1]), c = __ldg(&sc.uv[i2]);
        r.u = fmaf_(c.x - a.x, h.b2, fmaf_(b.x - a.x, h.b1, a.x));
        r.v = fmaf_(c.y - a.y, h.b2, fmaf_(b.y - a.y, h.b1, a.y));
    }
    {
        const float4 a = __ldg(&sc.normals[i0]), b = __ldg(&sc.normals[i1]), c = __ldg(&sc.normals[i2]);
        r.ln = F3(fmaf_(c.x - a.x, h.b2, fmaf_(b.x - a.x, h.b1, a.x)), fmaf_(c.y - a.y, h.b2, fmaf_(b.y - a.y, h.b1, a.y)),
                  fmaf_(c.z - a.z, h.b2, fmaf_(b.z - a.z, h.b1, a.z)));
    }
    if (sc.tangents) {
        float4 a = __ldg(&sc.tangents[i0]), b = __ldg(&sc.tangents[i1]), c = __ldg(&sc.tangents[i2]);
        a.w = a.w > 0.0f ? 2.0f : 0.0f;
        b.w = b.w > 0.0f ? 2.0f : 0.0f;
        c.w = c.w > 0.0f ? 2.0f : 0.0f;
        r.lt = F4(fmaf_(c.x - a.x, h.b2, fmaf_(b.x - a.x, h.b1, a.x)), fmaf_(c.y - a.y, h.b2, fmaf_(b.y - a.y, h.b1, a.y)),
                  fmaf_(c.z - a.z, h.b2, fmaf_(b.z - a.z, h.b1, a.z)), fmaf_(c.w - a.w, h.b2, fmaf_(b.w - a.w, h.b1, a.w)));
    }
    return r;
}

// The primary vertex's albedo, roughness and normal after FetchGBufferV2 (Shading.slang:82-112):
// diffuse x diffuse texture, fuzziness x the MRA texture's green channel, and the normal map in
// the mesh's tangent frame (mikkTSpace, :74-80) carried to world space by the instance's
// transform. The traced camera ray of the reference leaves the vertex's local normal and
// tangent unset; here they are the barycentric mixes of the vertex attributes, as the
// visibility-buffer caster computes them (GeneralFunc.slang:49-51).
struct GBufTex {
    f4 albedo;
    float rough;
    f3 n;
};
static __device__ __noinline__ GBufTex fetch_gbuffer(const ShadeScene& sc, const MatV& m, const HitAttr& a, f3 n,
                                                     uint32_t inst) {
    GBufTex g;
    g.albedo = m.diffuse;
    if (m.dtex >= 0) g.albedo = g.albedo * tex_sample(sc.tex, m.dtex, a.u, a.v);
    g.rough = m.fuzz;
    if (m.mtex >= 0) g.rough = g.rough * tex_sample(sc.tex, m.mtex, a.u, a.v).y;
    g.n = n;
    if (m.ntex >= 0) {
        const f4 t = tex_sample(sc.tex, m.ntex, a.u, a.v);
        const f3 vn = F3(fmaf_(t.x, 2.0f, -1.0f), fmaf_(t.y, 2.0f, -1.0f), fmaf_(t.z, 2.0f, -1.0f));
        const f3 T = F3(a.lt.x, a.lt.y, a.lt.z);
        const f3 B = cross3(a.ln, T) * a.lt.w;
        const f3 nl = normalize3(F3(fmaf_(vn.z, a.ln.x, fmaf_(vn.y, B.x, vn.x * T.x)),
                                    fmaf_(vn.z, a.ln.y, fmaf_(vn.y, B.y, vn.x * T.y)),
                                    fmaf_(vn.z, a.ln.z, fmaf_(vn.y, B.z, vn.x * T.z))));
        float w[12];
#pragma unroll
        for (int k = 0; k < 12; ++k) w[k] = __ldg(&sc.inst_prev[24u * inst + 12u + k]);
        g.n = normalize3(xvector(w, nl));
    }
    return g;
}

// ---- probes (AmbientCube.slang:71-78, 178-223, 290-382) ----
// Grid: CUBE_SIZE_XY x CUBE_SIZE_Z x CUBE_SIZE_XY probes, CUBE_UNIT apart from CUBE_OFFSET
// (AmbientCube.slang:12-15); index y * 192 * 192 + z * 192 + x.
constexpr int kProbeXY = 192, kProbeZ = 48;
constexpr float kProbeOffX = -24.0f, kProbeOffY = -0.34375f, kProbeOffZ = -24.0f;

// Light 0 of the scene as the probe bake uses it (FaceTask, AmbientCube.slang:528-537):
// the centre lerp(p1, p3, 0.5) of the quad, the power (its material's diffuse) and the area.
struct ProbeLight {
    f3 pos;
    f4 power;
    float area;
    int valid;
};

// The sky texture's nine-term spherical-harmonic projection per colour channel (ProjectHdrToSh,
// Texture.cpp:180-254; computed by the host at texture upload, zero for 8-bit textures as the
// reference projects HDR loads only), which the probe bake evaluates for its sky misses
// (SampleIBLRough, Shading.slang:188-192). on = 0: the frame has no sky texture and the bake
// sees the constant sky colour.
struct SkySH {
    float c[27];   // red terms 0..8, green 9..17, blue 18..26
    int on;
};
// EvaluateSH (Shading.slang:150-186) at direction n with SampleIBLRough's rotation
// 1 - SkyRotation about y, as (rgb, 1) times (HasSky ? SkyIntensity : 0).
GK_D f4 sky_sh(const SkySH& s, const GkrtFrameConstants& fc, f3 n) {
    float sn, cs;
    sincos2pi((1.0f - fc.sky_rotation) * 0.5f, sn, cs);   // angle (1 - rotate) pi
    const float rx = n.x * cs + n.z * sn, ry = n.y, rz = -n.x * sn + n.z * cs;
    float b[9];
    b[0] = 0.282095f;
    b[1] = -0.488603f * ry;
    b[2] = 0.488603f * rz;
    b[3] = -0.488603f * rx;
    b[4] = (1.092548f * rx) * ry;
    b[5] = (-1.092548f * ry) * rz;
    b[6] = 0.315392f * ((3.0f * ry) * ry - 1.0f);
    b[7] = (-1.092548f * rx) * rz;
    b[8] = 0.546274f * (rx * rx - rz * rz);
    float r = 0.0f, g = 0.0f, bl = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        r = r + s.c[i] * b[i];
        g = g + s.c[9 + i] * b[i];
        bl = bl + s.c[18 + i] * b[i];
    }
    return F4(r, g, bl, 1.0f) * (fc.has_sky ? fc.sky_intensity : 0.0f);
}
GK_D f4 unpack10(uint32_t p) {
    float r = div_((float)(p & 0x3FFu), 1023.0f), g = div_((float)((p >> 10) & 0x3FFu), 1023.0f),
          b = div_((float)((p >> 20) & 0x3FFu), 1023.0f);
    return F4(r * 512.0f, g * 512.0f, b * 512.0f, 0.0f * 512.0f);
}
GK_D f4 cube_sample(const uint32_t* cube, f3 n) {
    float wx = mx(n.x, 0.0f), wnx = mx(-n.x, 0.0f), wy = mx(n.y, 0.0f), wny = mx(-n.y, 0.0f);
    float wz = mx(n.z, 0.0f), wnz = mx(-n.z, 0.0f);
    float sum = ((((wx + wnx) + wy) + wny) + wz) + wnz;
    uint32_t s0 = __ldg(&cube[12]), s1 = __ldg(&cube[13]);
    float sk = 0.0f;
    sk = sk + (float)(s0 & 0xFFu) * wz;
    sk = sk + (float)((s0 >> 8) & 0xFFu) * wnz;
    sk = sk + (float)((s0 >> 16) & 0xFFu) * wy;
    sk = sk + (float)((s0 >> 24) & 0xFFu) * wny;
    sk = sk + (float)(s1 & 0xFFu) * wx;
    sk = sk + (float)((s1 >> 8) & 0xFFu) * wnx;
    const int ord[12] = {10, 11, 8, 9, 6, 7, 4, 5, 2, 3, 0, 1};
    const float w[12] = {wx, wnx, wy, wny, wz, wnz, wx, wnx, wy, wny, wz, wnz};
    f4 col = F4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int i = 0; i < 12; ++i) col = col + unpack10(__ldg(&cube[ord[i]])) * w[i];
    float k = sum > 0.0f ? div_(1.0f, sum) : 1.0f;
    col.x = col.x * k; col.y = col.y * k; col.z = col.z * k;
    sk = sk * k;
    col.w = div_(sk, 255.0f);
    return col;
}
static __device__ __noinline__ f4 probe_grid(const ShadeScene& sc, float npx, float npy, float npz, f3 n);
GK_D f4 probe_term(const ShadeScene& sc, f3 p, f3 n) {
    float npx = div_(p.x - -24.0f, 0.25f), npy = div_(p.y - -0.34375f, 0.25f), npz = div_(p.z - -24.0f, 0.25f);
    // written as !(>=) so that a NaN position takes the early out
    if (!(npx >= 0.0f) || !(npy >= 0.0f) || !(npz >= 0.0f) || npx > 190.0f || npy > 46.0f || npz > 190.0f)
        return F4(0.0f, 0.0f, 0.0f, 1.0f);
    if (!sc.cubes) return F4(0.0f, 0.0f, 0.0f, 0.0f);
    return probe_grid(sc, npx, npy, npz, n);
}
// The 8-probe interpolation itself (only reached when a probe grid was uploaded).
static __device__ __noinline__ f4 probe_grid(const ShadeScene& sc, float npx, float npy, float npz, f3 n) {
    float fx = floorf(npx), fy = floorf(npy), fz = floorf(npz);
    int bx = (int)fx, by = (int)fy, bz = (int)fz;
    float frx = npx - fx, fry = npy - fy, frz = npz - fz;
    float tw = 0.0f;
    f4 res = F4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 8; ++i) {
        int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        size_t id = (size_t)(by + oy) * 192 * 192 + (size_t)(bz + oz) * 192 + (size_t)(bx + ox);
        uint32_t u0 = __ldg(&sc.voxels[id * 4 + 2]), u1 = __ldg(&sc.voxels[id * 4 + 3]);
        float d0y = div_((float)((u0 >> 8) & 0xFFu), 255.0f);
        if (d0y < 0.01f) continue;
        float d0z = div_((float)((u0 >> 16) & 0xFFu), 255.0f), d0w = div_((float)((u0 >> 24) & 0xFFu), 255.0f);
        float d1x = div_((float)(u1 & 0xFFu), 255.0f), d1y = div_((float)((u1 >> 8) & 0xFFu), 255.0f);
        float d1z = div_((float)((u1 >> 16) & 0xFFu), 255.0f), d1w = div_((float)((u1 >> 24) & 0xFFu), 255.0f);
        f3 pl = F3(frx - (float)ox, fry - (float)oy, frz - (float)oz);
        float dist = len3(pl);
        f3 dir = normalize3(pl);
        float hl = sqrt_(mx(dir.x, 0.0f)) * d1x;
        hl = hl + sqrt_(mx(-dir.x, 0.0f)) * d1y;
        hl = hl + sqrt_(mx(dir.y, 0.0f)) * d1z;
        hl = hl + sqrt_(mx(-dir.y, 0.0f)) * d1w;
        hl = hl + sqrt_(mx(dir.z, 0.0f)) * d0z;
        hl = hl + sqrt_(mx(-dir.z, 0.0f)) * d0w;
        if (dist > hl + 0.05f) continue;
        float wx = ox == 0 ? 1.0f - frx : frx, wy = oy == 0 ? 1.0f - fry : fry, wz = oz == 0 ? 1.0f - frz : frz;
        float wgt = (wx * wy) * wz;
        res = res + cube_sample(sc.cubes + id * 14, n) * wgt;
        tw = tw + wgt;
    }
    if (tw > 0.0f) return F4(div_(res.x, tw), div_(res.y, tw), div_(res.z, tw), div_(res.w, tw));
    return F4(0.0f, 0.0f, 0.0f, 0.0f);
}

// Emissive-triangle NEE (GKRT_NEE_EMISSIVE; no counterpart in the built reference path, its
// math follows the legacy area-light branch of ScatterLambertian,
// assets/shaders/glsl_legacy/common/Scatter.glsl:55-76, with the light chosen by an alias
// table over power = area x luminance instead of uniformly). Entry j of sc.emit:
//   [p0.xyz, w_j = area_j / pick-probability_j], [p1 - p0, 0], [p2 - p0, 0], [unit normal, 0],
//   [emission rgba].
// One uniform number picks slot i and tests its threshold (the fraction of u * n), a second
// pair places a uniform point on the triangle. The sample is the throughput times
//   Le * cos_s * |cos_l| * w_j / (pi * d^2),
// tested for visibility over [EPS, d - EPS] from the bounce ray's origin (the segment of
// TraceSegment, Shading.slang:759-782). Emitters are two-sided, as hits on them are.
struct NeeSample {
    f3 o, dir;
    float tmax;
    f4 contrib;
};
GK_D bool nee_sample(const ShadeScene& sc, Rng& seed, f3 P, f3 N, f4 rc, NeeSample& s) {
    const uint32_t n = sc.nemit;
    const float x = rnd1(seed) * (float)n;
    uint32_t i = (uint32_t)x;
    if (i > n - 1u) i = n - 1u;
    const float frac = x - (float)i;
    const float2 pa = __ldg(&sc.emit_alias[i]);
    const uint32_t j = frac < pa.x ? i : __float_as_uint(pa.y);
    const f2 r = rnd2(seed);
    const float4* g = sc.emit + 5u * j;
    const float4 g0 = __ldg(g), g1 = __ldg(g + 1), g2 = __ldg(g + 2), g3 = __ldg(g + 3), g4 = __ldg(g + 4);
    const float su = sqrt_(r.x), bs = su * (1.0f - r.y), bt = su * r.y;
    const f3 q = F3((g0.x + g1.x * bs) + g2.x * bt, (g0.y + g1.y * bs) + g2.y * bt, (g0.z + g1.z * bs) + g2.z * bt);
    s.o = fma3(N, 0.001f, P);
    const f3 lv = q - s.o;
    const float d2 = dot3(lv, lv);
    const float dist = sqrt_(d2);
    if (!(dist > 2e-3f)) return false;
    s.dir = lv * div_(1.0f, dist);
    const float cs = dot3(N, s.dir);
    if (!(cs > 0.0f)) return false;
    const float cl = fabsf(dot3(F3(g3.x, g3.y, g3.z), s.dir));
    if (!(cl > 0.0f)) return false;
    const float gm = div_((cs * cl) * g0.w, d2 * 3.14159265358979323846f);
    s.contrib = (rc * F4(g4.x, g4.y, g4.z, g4.w)) * gm;
    s.tmax = dist - 1e-3f;
    return true;
}

struct PixelImages {
    float4* single_diffuse;
    float4* single_specular;
    float4* albedo;
    float4* normal;
    uint32_t* object_id;
    float2* motion;
    float* prev_depth;
    uint32_t* motion_moment;
    uint32_t* hit_inst;
    uint32_t* hit_prim;
};

__constant__ float c_halton[16] = {0.5f, 0.3333f, 0.25f, 0.6667f, 0.75f, 0.1111f, 0.125f, 0.4444f,
                                   0.625f, 0.7778f, 0.375f, 0.2222f, 0.875f, 0.5556f, 0.0625f, 0.8889f};

}  // namespace gk
