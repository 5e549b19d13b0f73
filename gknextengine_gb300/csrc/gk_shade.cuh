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

struct ShadeScene {
    SceneView S;
    const float4* normals;       // per vertex
    const uint32_t* slots;       // per vertex material slot
    const uint32_t* indices;
    const uint32_t* inst_mat;    // 16 per instance
    const float* inst_prev;      // 12 per instance: combined_prev
    const GkrtMaterial* mats;
    uint32_t nmat;
    const uint32_t* cubes;       // optional probe grid
    const uint32_t* voxels;
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
};

GK_D MatV load_mat(const ShadeScene& sc, uint32_t i) {
    if (i >= sc.nmat) i = sc.nmat - 1;
    const float4* p = reinterpret_cast<const float4*>(sc.mats + i);
    float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    MatV m;
    m.diffuse = F4(a.x, a.y, a.z, a.w);
    m.fuzz = b.w;
    m.ri = c.x;
    m.model = __float_as_uint(c.y);
    m.metal = c.z;
    m.ri2 = c.w;
    return m;
}

// FHardwareRayTracerV2::TraceRay: closest hit -> position, shading normal, material.
GK_D bool trace_ray(const ShadeScene& sc, f3 o, f3 d, float tmax, Vtx& out, uint32_t* prim_out, uint32_t* stk,
                    int stride, Counters& cn) {
    ++cn.rays;
    TraceOut r = trace_closest(sc.S, o, d, 1e-3f, tmax, stk, stride, cn);
    if (!r.hit) return false;
    HitShade h = hit_shade(sc.S, o, d, r.inst, r.tri);
    const DevInst* ip = sc.S.inst + r.inst;
    const uint32_t ioff = __ldg(&ip->index_offset) + 3u * r.prim, voff = __ldg(&ip->vertex_offset);
    const uint32_t i0 = __ldg(&sc.indices[ioff]) + voff, i1 = __ldg(&sc.indices[ioff + 1]) + voff,
                   i2 = __ldg(&sc.indices[ioff + 2]) + voff;
    float4 a = __ldg(&sc.normals[i0]), b = __ldg(&sc.normals[i1]), c = __ldg(&sc.normals[i2]);
    f3 n0 = F3(a.x, a.y, a.z), e1 = F3(b.x, b.y, b.z) - n0, e2 = F3(c.x, c.y, c.z) - n0;
    f3 nobj = F3(fmaf_(e2.x, h.b2, fmaf_(e1.x, h.b1, n0.x)), fmaf_(e2.y, h.b2, fmaf_(e1.y, h.b1, n0.y)),
                 fmaf_(e2.z, h.b2, fmaf_(e1.z, h.b1, n0.z)));
    float w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
    out.N = normalize3(xnormal(w, nobj));
    out.P = fma3(d, h.t, o);
    out.mat = __ldg(&sc.inst_mat[16u * r.inst + (__ldg(&sc.slots[i0]) & 15u)]);
    out.inst = r.inst;
    if (prim_out) *prim_out = r.prim;
    return true;
}

GK_D bool trace_occlusion(const ShadeScene& sc, f3 o, f3 d, uint32_t* stk, int stride, Counters& cn) {
    ++cn.rays;
    TraceOut r = traverse<kAny>(sc.S, o, d, 1e-3f, 1000.0f, stk, stride, cn);
    return r.hit;
}

GK_D f4 sky(const GkrtFrameConstants& fc) {
    if (!fc.has_sky) return F4(0.0f, 0.0f, 0.0f, 0.0f);
    return F4(mn(10.0f, fc.sky_color[0]), mn(10.0f, fc.sky_color[1]), mn(10.0f, fc.sky_color[2]),
              mn(1.0f, fc.sky_color[3])) * fc.sky_intensity;
}

// ---- probes (AmbientCube.slang:71-78, 178-223, 290-382) ----
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
GK_D f4 probe_term(const ShadeScene& sc, f3 p, f3 n) {
    float npx = div_(p.x - -24.0f, 0.25f), npy = div_(p.y - -0.34375f, 0.25f), npz = div_(p.z - -24.0f, 0.25f);
    // written as !(>=) so that a NaN position takes the early out
    if (!(npx >= 0.0f) || !(npy >= 0.0f) || !(npz >= 0.0f) || npx > 190.0f || npy > 46.0f || npz > 190.0f)
        return F4(0.0f, 0.0f, 0.0f, 1.0f);
    if (!sc.cubes) return F4(0.0f, 0.0f, 0.0f, 0.0f);
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

// GetRayColor (Shading.slang:1003-1082)
GK_D bool ray_color(const ShadeScene& sc, const GkrtFrameConstants& fc, Vtx& v, f3& dir, f4& color, Rng& seed,
                    bool& hitReflect, bool& hitMetal, uint32_t* stk, int stride, Counters& cn) {
    const MatV mat = load_mat(sc, v.mat);
    const bool diel = mat.model == GKRT_MAT_DIELECTRIC;
    const float startPosOffset = diel ? 0.0f : 1.0f;
    const float dotValue = dot3(dir, v.N);
    const bool back = dotValue > 0.0f;
    const f3 outward = back ? -v.N : v.N;
    const float niOverNt = back ? mat.ri2 : div_(1.0f, mat.ri2);
    const float cosine = dotValue > 0.0f ? mat.ri * dotValue : -dotValue;
    const float reflectProb = schlick(cosine, mat.ri);
    const bool chanceReflect = rnd1(seed) < reflectProb;
    const bool chanceMetal = rnd1(seed) < mat.metal;
    const bool chanceGGX = chanceReflect || chanceMetal;
    f3 tdir;
    if (chanceGGX) tdir = ggx_sample(seed, sqrt_(mat.fuzz), reflect3(dir, outward));
    else tdir = align_normal(hemisphere_cos(seed), outward);
    hitReflect = chanceGGX;
    hitMetal = chanceMetal;
    if (diel && !chanceReflect) tdir = refract3(dir, outward, niOverNt);
    dir = tdir;
    f3 org = fma3(v.N, 0.001f * startPosOffset, v.P);
    Vtx nv;
    if (trace_ray(sc, org, tdir, 1000.0f, nv, nullptr, stk, stride, cn)) {
        v = nv;
        const MatV hm = load_mat(sc, v.mat);
        if (hm.model == GKRT_MAT_DIFFUSE_LIGHT || !chanceReflect) color = color * hm.diffuse;
        if (back && !diel) { color = F4(0.5f, 0.5f, 0.5f, 0.0f); return true; }
        return hm.model == GKRT_MAT_DIFFUSE_LIGHT;
    }
    color = color * sky(fc);
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

// One pixel of Core.PathTracing (PrimaryHit + Render + DirectIlluminate).
GK_D void shade_pixel(const ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H, int x, int y,
                      const PixelImages& im, uint32_t* stk, int stride, Counters& cn) {
    const size_t pix = (size_t)y * W + x;
    Rng seed;
    seed.v[0] = (uint32_t)x; seed.v[1] = (uint32_t)y; seed.v[2] = fc.total_frames; seed.v[3] = 0u;
    const bool want_ids = (fc.flags & GKRT_FRAME_PRIMARY_IDS) != 0u;
    float uvx = fmaf_(div_((float)x, (float)W), 2.0f, -1.0f);
    float uvy = fmaf_(div_((float)y, (float)H), 2.0f, -1.0f);
    if (fc.taa) {
        const uint32_t hi = fc.total_frames % 8u;
        uvx = uvx + div_(c_halton[2 * hi] - 0.5f, (float)W);
        uvy = uvy + div_(c_halton[2 * hi + 1] - 0.5f, (float)H);
    }
    f2 disk = unit_disk(seed);
    const float ha = div_(fc.aperture, 2.0f);
    const float offx = ha * disk.x, offy = ha * disk.y;
    f4 origin = mat4v(fc.model_view_inverse, F4(offx, offy, 0.0f, 1.0f));
    f4 target = mat4v(fc.projection_inverse, F4(uvx, uvy, 1.0f, 1.0f));
    f3 tn = normalize3(F3(fmaf_(target.x, fc.focus_distance, -offx), fmaf_(target.y, fc.focus_distance, -offy),
                          target.z * fc.focus_distance));
    f4 direction = mat4v(fc.model_view_inverse, F4(tn.x, tn.y, tn.z, 0.0f));
    const f3 o3 = xyz(origin), d3 = xyz(direction);
    const f3 primDir = normalize3(d3);
    Vtx pv;
    uint32_t pprim = 0;
    const bool hit = trace_ray(sc, o3, d3, 1000.0f, pv, &pprim, stk, stride, cn);
    im.single_specular[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (!hit) {
        f4 s = sky(fc);
        im.single_diffuse[pix] = make_float4(s.x, s.y, s.z, s.w);
        im.motion[pix] = make_float2(0.0f, 0.0f);
        im.albedo[pix] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
        im.normal[pix] = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
        im.object_id[pix] = 65535u;
        im.prev_depth[pix] = 100000.0f;
        if (want_ids) { im.hit_inst[pix] = 0xFFFFFFFFu; im.hit_prim[pix] = 0xFFFFFFFFu; }
        return;
    }
    if (want_ids) { im.hit_inst[pix] = pv.inst; im.hit_prim[pix] = pprim; }
    const f4 P4 = F4(pv.P.x, pv.P.y, pv.P.z, 1.0f);
    const f4 clip = mat4v(fc.view_projection, P4);
    const f4 ch = mat4v(fc.view_projection_unjit, P4);
    const float cfx = div_(ch.x, ch.w) * 0.5f, cfy = div_(ch.y, ch.w) * 0.5f;
    float cp[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) cp[k] = __ldg(&sc.inst_prev[12u * pv.inst + k]);
    const f3 prevP = xpoint(cp, pv.P);
    const f4 ph = mat4v(fc.prev_view_projection_unjit, F4(prevP.x, prevP.y, prevP.z, 1.0f));
    const float pfx = div_(ph.x, ph.w) * 0.5f, pfy = div_(ph.y, ph.w) * 0.5f;
    uint32_t mom = im.motion_moment[pix];
    if (len3(pv.P - prevP) > 0.02f) mom = fc.temporal_frames;
    else mom = mom > 0u ? mom - 1u : 0u;
    im.motion_moment[pix] = mom;
    const MatV pm = load_mat(sc, pv.mat);
    im.albedo[pix] = make_float4(pm.diffuse.x, pm.diffuse.y, pm.diffuse.z, pm.diffuse.w);
    im.normal[pix] = make_float4(pv.N.x, pv.N.y, pv.N.z, pm.fuzz);
    im.object_id[pix] = __ldg(&sc.S.inst[pv.inst].instance_id);
    im.motion[pix] = make_float2((pfx - cfx) * (float)W, (pfy - cfy) * (float)H);
    im.prev_depth[pix] = div_(clip.z, clip.w);
    if (pm.model != GKRT_MAT_DIELECTRIC) pv.P = fma3(primDir, -0.03f, pv.P);
    if (pm.model == GKRT_MAT_DIFFUSE_LIGHT) {
        im.single_diffuse[pix] = make_float4(pm.diffuse.x, pm.diffuse.y, pm.diffuse.z, pm.diffuse.w);
        return;
    }
    const bool pdiel = pm.model == GKRT_MAT_DIELECTRIC;
    int samples = (int)fc.number_of_samples * (mom > 0u ? 4 : 1);
    if (samples < 1) samples = 1;
    const f4 eye = mat4v(fc.model_view_inverse, F4(0.0f, 0.0f, 0.0f, 1.0f));
    const uint32_t maxB = pdiel ? fc.max_number_of_bounces : fc.number_of_bounces;
    const f3 sunDir = F3(fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]);
    const f4 sunCol = F4(fc.sun_color[0], fc.sun_color[1], fc.sun_color[2], fc.sun_color[3]);
    const float kCosCone = 0.999990482f;
    f4 fcol = F4(0.0f, 0.0f, 0.0f, 0.0f), frefl = F4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < samples; ++i) {
        f4 rc = F4(1.0f, 1.0f, 1.0f, 1.0f);
        f3 dir = normalize3(pv.P - xyz(eye));
        Vtx vs = pv;
        bool hitReflect = false, hitMetal = false;
        const bool exitFirst = ray_color(sc, fc, vs, dir, rc, seed, hitReflect, hitMetal, stk, stride, cn);
        if (!exitFirst) {
            if (fc.fast_gather && !pdiel) {
                rc = rc * probe_term(sc, vs.P, vs.N);
            } else {
                for (uint32_t b = 1; b < maxB; ++b) {
                    bool dc = false, dc2 = false;
                    if (ray_color(sc, fc, vs, dir, rc, seed, dc, dc2, stk, stride, cn)) break;
                    if (fc.has_sun && rnd1(seed) < 0.5f) {
                        const f3 cd = align_normal(cone(seed, kCosCone), sunDir);
                        if (!trace_occlusion(sc, vs.P, cd, stk, stride, cn)) { rc = rc * sunCol; break; }
                    }
                    const bool early = !pdiel && rnd1(seed) < 0.5f;
                    if (b == maxB - 1u || early) { rc = rc * probe_term(sc, vs.P, vs.N); break; }
                }
            }
        }
        if (hitMetal) rc = rc * pm.diffuse;
        if (hitReflect) frefl = frefl + rc;
        else fcol = fcol + rc;
    }
    const float fs = (float)samples;
    fcol = F4(div_(fcol.x, fs), div_(fcol.y, fs), div_(fcol.z, fs), div_(fcol.w, fs));
    frefl = F4(div_(frefl.x, fs), div_(frefl.y, fs), div_(frefl.z, fs), div_(frefl.w, fs));
    const float dd = mx(dot3(sunDir, normalize3(pv.N)), 0.0f) * 0.318309886183790671538f;
    float shadow = 0.0f;
    if (fc.has_sun) {
        const f3 cd = align_normal(cone(seed, kCosCone), sunDir);
        shadow = trace_occlusion(sc, pv.P, cd, stk, stride, cn) ? 0.0f : 1.0f;
    }
    fcol = fcol + F4((sunCol.x * dd) * shadow, (sunCol.y * dd) * shadow, (sunCol.z * dd) * shadow,
                     (sunCol.w * dd) * shadow);
    im.single_diffuse[pix] = make_float4(fcol.x, fcol.y, fcol.z, fcol.w);
    im.single_specular[pix] = make_float4(frefl.x, frefl.y, frefl.z, frefl.w);
}

}  // namespace gk
