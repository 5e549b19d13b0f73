// k_pathtrace.cu — the "rt pass" (Core.PathTracing) and ray-query kernels for sm_103a.
//
// The rt pass is one persistent kernel: every lane runs the per-pixel logic of
// FPathTracingRendererV2 (assets/shaders/common/Shading.slang:1084-1241, with the traced
// camera ray of FHardwarePrimaryRayCaster, :283-334) as a state machine that stops
// whenever it needs a ray traced. The warp alternates two phases: all lanes advance their
// rays through the BVH until every ray of the warp is finished, then every lane runs its
// state machine to its next ray, or takes the next pixel from a global counter
// (warp-aggregated atomics, 8 x 4 pixel tiles) when its path has ended. A lane whose path
// ends early thus refills instead of idling until the longest path of its warp is done.
// (Refilling in the middle of the traversal phase was measured slower: shading is the
// divergent, expensive part, and is best run for all lanes at once.) Each path keeps its
// own RNG stream, so results do not depend on the schedule.
#include "gk_shade.cuh"
#include "gkrt_internal.h"

namespace gk {

constexpr int kPtThreads = 128;
// Resident blocks per SM, per instantiation: 4 (128 registers, few spills) without emissive
// NEE, 5 (96 registers, spills) with it, whose shadow rays add a second traversal per vertex
// that more warps hide better. Same box, current kernel: the 1080p brick trace pass (no NEE)
// 3 / 4 / 5 / 6 blocks 3.94 / 3.43 / 3.56 / 3.54 ms; the 4K city (alias-table NEE) 116.4 /
// 102.9 / 97.0 ms for 3 / 4 / 5 blocks.
template <bool kNee>
constexpr int pt_blocks() { return kNee ? 5 : 4; }
constexpr int kRefillBelow = 1;    // shade and refill once every lane of the warp has finished its ray
constexpr float kCosCone = 0.999990482f;   // cos(0.25 deg), Shading.slang:897

// Warp-aggregated flush: one atomic per counter per warp. Slots 0-5 are per pass
// (rays, FP64 fallbacks, exact re-traces, node visits, triangle tests, hit fetches); slot 6
// counts rays since the context was created.
__device__ __forceinline__ void flush_counters(const Counters& c, unsigned long long* out) {
    unsigned long long v[6] = {c.rays, c.fallbacks, c.retraces, c.nodes, c.tris, c.hits};
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 6; ++k) v[k] += __shfl_down_sync(0xFFFFFFFFu, v[k], o);
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (v[k]) atomicAdd(&out[k], v[k]);
        if (v[0]) atomicAdd(&out[6], v[0]);
    }
}

enum Stage : uint32_t {
    ST_PRIMARY = 0, ST_FIRST = 1, ST_BOUNCE = 2, ST_SUN = 3, ST_DIRECT = 4,
    ST_NEE_FIRST = 5, ST_NEE_BOUNCE = 6   // emissive-triangle shadow ray before the first / a later bounce
};

// Per-thread slots in shared memory (strided by the block size): the primary vertex,
// the per-pixel loop bounds, the two accumulators, the pending emissive-NEE sample and, in the
// textured instantiation, the primary albedo (material diffuse x diffuse texture).
enum Slot {
    SL_PX = 0, SL_PY, SL_PZ, SL_NX, SL_NY, SL_NZ, SL_MAT, SL_LOOP, SL_FC, SL_FR = SL_FC + 4, SL_NEE = SL_FR + 4,
    SL_COUNT = SL_NEE + 4, SL_ALB = SL_COUNT, SL_COUNT_TEX = SL_ALB + 4
};

struct Lane {
    int pix;          // pixel index, -1 when the lane holds no pixel
    Rng seed;
    uint32_t stage;
    uint32_t i, b;    // sample and bounce indices
    bool chanceReflect, back, diel, hitReflect, hitMetal;
    bool neeLobe;     // the bounce in flight was sampled from the diffuse lobe of an emissive-NEE vertex
    f4 rc;            // throughput of the current sample (RayColor)
    Vtx vs;           // current path vertex
    f3 dir;           // current path direction
};

struct Ctx {
    const ShadeScene& sc;
    const GkrtFrameConstants& fc;
    const PixelImages& im;
    int W, H, P;      // P: image row pitch in pixels
    float* ps;        // this thread's first shared slot
    int stride;
    Counters& cn;
    __device__ float& slot(int k) const { return ps[k * stride]; }
};

__device__ __forceinline__ void emit(Trav& T, const Ctx& c, f3 o, f3 d, int mode, float tmax = 1000.0f) {
    ++c.cn.rays;
    trav_init(T, c.sc.S, o, d, tmax, mode);
}

__device__ __forceinline__ f3 pv_pos(const Ctx& c) { return F3(c.slot(SL_PX), c.slot(SL_PY), c.slot(SL_PZ)); }
__device__ __forceinline__ f3 pv_nrm(const Ctx& c) { return F3(c.slot(SL_NX), c.slot(SL_NY), c.slot(SL_NZ)); }
// primaryAlbedo_ of the reference: the material's diffuse, times its diffuse texture (kTex)
template <bool kTex>
__device__ __forceinline__ f4 pv_albedo(const Ctx& c) {
    if (kTex) return F4(c.slot(SL_ALB), c.slot(SL_ALB + 1), c.slot(SL_ALB + 2), c.slot(SL_ALB + 3));
    return load_mat(c.sc, __float_as_uint(c.slot(SL_MAT))).diffuse;
}

// Run the lane's state machine on the ray that just finished, up to the next ray
// (returns true) or the end of the pixel (returns false). Follows FPathTracingRendererV2:
// PrimaryHit (Shading.slang:1186-1223), Render (:1084-1184) with GetRayColor
// (:1003-1082) split at its trace, the sun test of the bounce loop (:1135-1144), early exit
// and probe termination (:1146-1154), and DirectIlluminate (:886-908).
//
// The logic is laid out as guarded sections in one fixed order; every lane passes each
// section at most once per call, so lanes in different states re-converge after each
// section and the expensive ones (the sampling before a trace, the hit reconstruction
// after it) run once per warp for all the lanes that need them.
// kTex: textured materials and the textured sky compiled in (the scene has texture ids or the
// frame samples a sky texture).
template <bool kNee, bool kTex>
__device__ bool advance(Lane& L, Trav& T, const Ctx& c) {
    const GkrtFrameConstants& fc = c.fc;
    const f3 sunDir = F3(fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]);
    const uint32_t stage = L.stage;
    bool emitted = false, need_begin = false, need_pre = false, pre_first = false;
    bool need_end = false, need_after_sun = false, need_finish = false;
    float shadow = 0.0f;

    // 1. the camera ray's hit: G-buffer outputs, motion, sample set-up
    if (stage == ST_PRIMARY) {
        const int pix = L.pix;
        const bool want_ids = (fc.flags & GKRT_FRAME_PRIMARY_IDS) != 0u;
        c.im.single_specular[pix] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (!T.hit) {
            const f4 s = kTex ? sky_dir(c.sc, fc, normalize3(T.wd)) : sky(fc);
            c.im.single_diffuse[pix] = make_float4(s.x, s.y, s.z, s.w);
            c.im.motion[pix] = make_float2(0.0f, 0.0f);
            c.im.albedo[pix] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
            c.im.normal[pix] = make_float4(0.0f, 1.0f, 0.0f, 1.0f);
            c.im.object_id[pix] = 65535u;
            c.im.prev_depth[pix] = 100000.0f;
            if (want_ids) { c.im.hit_inst[pix] = 0xFFFFFFFFu; c.im.hit_prim[pix] = 0xFFFFFFFFu; }
            L.pix = -1;
        } else {
            ++c.cn.hits;
            Vtx pv = hit_vertex(c.sc, T.wo, T.wd, T.inst, T.prim, T.tri);
            if (want_ids) { c.im.hit_inst[pix] = T.inst; c.im.hit_prim[pix] = T.prim; }
            const f4 P4 = F4(pv.P.x, pv.P.y, pv.P.z, 1.0f);
            const f4 clip = mat4v(fc.view_projection, P4);
            const f4 ch = mat4v(fc.view_projection_unjit, P4);
            const float cfx = div_(ch.x, ch.w) * 0.5f, cfy = div_(ch.y, ch.w) * 0.5f;
            float cp[12];
#pragma unroll
            for (int q = 0; q < 12; ++q) cp[q] = __ldg(&c.sc.inst_prev[24u * pv.inst + q]);
            const f3 prevP = xpoint(cp, pv.P);
            const f4 ph = mat4v(fc.prev_view_projection_unjit, F4(prevP.x, prevP.y, prevP.z, 1.0f));
            const float pfx = div_(ph.x, ph.w) * 0.5f, pfy = div_(ph.y, ph.w) * 0.5f;
            uint32_t mom = c.im.motion_moment[pix];
            if (len3(pv.P - prevP) > 0.02f) mom = fc.temporal_frames;
            else mom = mom > 0u ? mom - 1u : 0u;
            c.im.motion_moment[pix] = mom;
            const MatV pm = load_mat(c.sc, pv.mat);
            f4 palb = pm.diffuse;
            float prough = pm.fuzz;
            if (kTex) {   // FetchGBufferV2 (Shading.slang:82-112)
                const HitAttr ha = hit_attr(c.sc, T.wo, T.wd, T.inst, T.prim, T.tri);
                const GBufTex g = fetch_gbuffer(c.sc, pm, ha, pv.N, pv.inst);
                palb = g.albedo;
                prough = g.rough;
                pv.N = g.n;
            }
            c.im.albedo[pix] = make_float4(palb.x, palb.y, palb.z, palb.w);
            c.im.normal[pix] = make_float4(pv.N.x, pv.N.y, pv.N.z, prough);
            c.im.object_id[pix] = __ldg(&c.sc.S.inst[pv.inst].instance_id);
            c.im.motion[pix] = make_float2((pfx - cfx) * (float)c.W, (pfy - cfy) * (float)c.H);
            c.im.prev_depth[pix] = div_(clip.z, clip.w);
            if (pm.model != GKRT_MAT_DIELECTRIC) pv.P = fma3(normalize3(T.wd), -0.03f, pv.P);
            if (pm.model == GKRT_MAT_DIFFUSE_LIGHT) {
                c.im.single_diffuse[pix] = make_float4(pm.diffuse.x, pm.diffuse.y, pm.diffuse.z, pm.diffuse.w);
                L.pix = -1;
            } else {
                const bool pdiel = pm.model == GKRT_MAT_DIELECTRIC;
                int samples = (int)fc.number_of_samples * (mom > 0u ? 4 : 1);
                if (samples < 1) samples = 1;
                if (samples > 0xFFFF) samples = 0xFFFF;
                uint32_t maxB = pdiel ? fc.max_number_of_bounces : fc.number_of_bounces;
                if (maxB > 0x7FFFu) maxB = 0x7FFFu;
                c.slot(SL_PX) = pv.P.x; c.slot(SL_PY) = pv.P.y; c.slot(SL_PZ) = pv.P.z;
                c.slot(SL_NX) = pv.N.x; c.slot(SL_NY) = pv.N.y; c.slot(SL_NZ) = pv.N.z;
                c.slot(SL_MAT) = __uint_as_float(pv.mat);
                c.slot(SL_LOOP) = __uint_as_float((uint32_t)samples | (maxB << 16) | (pdiel ? 0x80000000u : 0u));
#pragma unroll
                for (int q = 0; q < 4; ++q) { c.slot(SL_FC + q) = 0.0f; c.slot(SL_FR + q) = 0.0f; }
                if (kTex) {
                    c.slot(SL_ALB) = palb.x; c.slot(SL_ALB + 1) = palb.y;
                    c.slot(SL_ALB + 2) = palb.z; c.slot(SL_ALB + 3) = palb.w;
                }
                L.i = 0;
                need_begin = true;
            }
        }
    }

    // 2. GetRayColor after its trace (Shading.slang:1039-1081), then the bounce loop's sun test
    if (stage == ST_FIRST || stage == ST_BOUNCE) {
        bool term;
        if (T.hit) {
            ++c.cn.hits;
            L.vs = hit_vertex(c.sc, T.wo, T.wd, T.inst, T.prim, T.tri);
            const MatV hm = load_mat(c.sc, L.vs.mat);
            if (kNee && L.neeLobe && hm.model == GKRT_MAT_DIFFUSE_LIGHT) {
                // the emitter this diffuse bounce reached was sampled by the vertex's NEE
                L.rc = F4(0.0f, 0.0f, 0.0f, 0.0f);
                term = true;
            } else {
                f4 halb = hm.diffuse;
                if (kTex && hm.dtex >= 0) {   // the hit's diffuse texture (Shading.slang:1046-1050)
                    const HitAttr ha = hit_attr(c.sc, T.wo, T.wd, T.inst, T.prim, T.tri);
                    halb = halb * tex_sample(c.sc.tex, hm.dtex, ha.u, ha.v);
                }
                if (hm.model == GKRT_MAT_DIFFUSE_LIGHT || !L.chanceReflect) L.rc = L.rc * halb;
                if (L.back && !L.diel) { L.rc = F4(0.5f, 0.5f, 0.5f, 0.0f); term = true; }
                else term = hm.model == GKRT_MAT_DIFFUSE_LIGHT;
            }
        } else {
            L.rc = L.rc * (kTex ? sky_dir(c.sc, fc, T.wd) : sky(fc));
            term = true;
        }
        const uint32_t loop = __float_as_uint(c.slot(SL_LOOP));
        if (term) {
            need_end = true;
        } else if (stage == ST_FIRST) {
            const uint32_t maxB = (loop >> 16) & 0x7FFFu;
            const bool pdiel = (loop >> 31) != 0u;
            if (fc.fast_gather && !pdiel) {
                L.rc = L.rc * probe_term(c.sc, L.vs.P, L.vs.N);
                need_end = true;
            } else {
                L.b = 1;
                if (L.b < maxB) need_pre = true;
                else need_end = true;
            }
        } else if (fc.has_sun && rnd1(L.seed) < 0.5f) {
            const f3 cd = align_normal(cone(L.seed, kCosCone), sunDir);
            L.stage = ST_SUN;
            emit(T, c, L.vs.P, cd, kAny);
            emitted = true;
        } else {
            need_after_sun = true;
        }
    }

    // 3. the sun test's answer
    if (stage == ST_SUN) {
        if (!T.hit) {
            L.rc = L.rc * F4(fc.sun_color[0], fc.sun_color[1], fc.sun_color[2], fc.sun_color[3]);
            need_end = true;
        } else {
            need_after_sun = true;
        }
    }

    // 4. early exit or last bounce: probe termination, else the next bounce
    if (need_after_sun) {
        const uint32_t loop = __float_as_uint(c.slot(SL_LOOP));
        const uint32_t maxB = (loop >> 16) & 0x7FFFu;
        const bool pdiel = (loop >> 31) != 0u;
        const bool early = !pdiel && rnd1(L.seed) < 0.5f;
        if (L.b == maxB - 1u || early) {
            L.rc = L.rc * probe_term(c.sc, L.vs.P, L.vs.N);
            need_end = true;
        } else {
            ++L.b;
            need_pre = true;
        }
    }

    // 5. end of a sample (Shading.slang:1159-1176), then the next sample or DirectIlluminate
    if (need_end) {
        if (L.hitMetal) L.rc = L.rc * pv_albedo<kTex>(c);
        const int acc = L.hitReflect ? SL_FR : SL_FC;
        c.slot(acc) = c.slot(acc) + L.rc.x;
        c.slot(acc + 1) = c.slot(acc + 1) + L.rc.y;
        c.slot(acc + 2) = c.slot(acc + 2) + L.rc.z;
        c.slot(acc + 3) = c.slot(acc + 3) + L.rc.w;
        const uint32_t samples = __float_as_uint(c.slot(SL_LOOP)) & 0xFFFFu;
        if (++L.i < samples) {
            need_begin = true;
        } else {
            const float fs = (float)samples;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                c.slot(SL_FC + q) = div_(c.slot(SL_FC + q), fs);
                c.slot(SL_FR + q) = div_(c.slot(SL_FR + q), fs);
            }
            if (fc.has_sun) {
                const f3 cd = align_normal(cone(L.seed, kCosCone), sunDir);
                L.stage = ST_DIRECT;
                emit(T, c, pv_pos(c), cd, kAny);
                emitted = true;
            } else {
                shadow = 0.0f;
                need_finish = true;
            }
        }
    }

    // 6. DirectIlluminate's answer
    if (stage == ST_DIRECT) {
        shadow = T.hit ? 0.0f : 1.0f;
        need_finish = true;
    }

    // 6b. an emissive-NEE shadow ray's answer, then the bounce ray its vertex sampled
    if (kNee && (stage == ST_NEE_FIRST || stage == ST_NEE_BOUNCE)) {
        if (!T.hit) {
            const int acc = L.hitReflect ? SL_FR : SL_FC;
#pragma unroll
            for (int q = 0; q < 4; ++q) c.slot(acc + q) = c.slot(acc + q) + c.slot(SL_NEE + q);
        }
        L.stage = stage == ST_NEE_FIRST ? ST_FIRST : ST_BOUNCE;
        emit(T, c, fma3(L.vs.N, 0.001f, L.vs.P), L.dir, kClosest);
        emitted = true;
    }

    // 7. the pixel's outputs (Shading.slang:1175-1183)
    if (need_finish) {
        const float dd = mx(dot3(sunDir, normalize3(pv_nrm(c))), 0.0f) * 0.318309886183790671538f;
        f4 fcol = F4(c.slot(SL_FC), c.slot(SL_FC + 1), c.slot(SL_FC + 2), c.slot(SL_FC + 3));
        const f4 frefl = F4(c.slot(SL_FR), c.slot(SL_FR + 1), c.slot(SL_FR + 2), c.slot(SL_FR + 3));
        fcol = fcol + F4((fc.sun_color[0] * dd) * shadow, (fc.sun_color[1] * dd) * shadow,
                         (fc.sun_color[2] * dd) * shadow, (fc.sun_color[3] * dd) * shadow);
        c.im.single_diffuse[L.pix] = make_float4(fcol.x, fcol.y, fcol.z, fcol.w);
        c.im.single_specular[L.pix] = make_float4(frefl.x, frefl.y, frefl.z, frefl.w);
        L.pix = -1;
    }

    // 8. start of a sample (Shading.slang:1103-1117)
    if (need_begin) {
        const f4 eye = mat4v(fc.model_view_inverse, F4(0.0f, 0.0f, 0.0f, 1.0f));
        L.rc = F4(1.0f, 1.0f, 1.0f, 1.0f);
        L.vs.P = pv_pos(c);
        L.vs.N = pv_nrm(c);
        L.vs.mat = __float_as_uint(c.slot(SL_MAT));
        L.dir = normalize3(L.vs.P - xyz(eye));
        L.hitReflect = false;
        L.hitMetal = false;
        need_pre = true;
        pre_first = true;
    }

    // 9. GetRayColor up to its trace (Shading.slang:1007-1039)
    if (need_pre) {
        const MatV mat = load_mat(c.sc, L.vs.mat);
        const bool diel = mat.model == GKRT_MAT_DIELECTRIC;
        const float startPosOffset = diel ? 0.0f : 1.0f;
        const float dotValue = dot3(L.dir, L.vs.N);
        const bool back = dotValue > 0.0f;
        const f3 outward = back ? -L.vs.N : L.vs.N;
        const float niOverNt = back ? mat.ri2 : div_(1.0f, mat.ri2);
        const float cosine = dotValue > 0.0f ? mat.ri * dotValue : -dotValue;
        const float reflectProb = schlick(cosine, mat.ri);
        const bool chanceReflect = rnd1(L.seed) < reflectProb;
        const bool chanceMetal = rnd1(L.seed) < mat.metal;
        const bool chanceGGX = chanceReflect || chanceMetal;
        f3 tdir;
        if (chanceGGX) tdir = ggx_sample(L.seed, sqrt_(mat.fuzz), reflect3(L.dir, outward));
        else tdir = align_normal(hemisphere_cos(L.seed), outward);
        if (pre_first) { L.hitReflect = chanceGGX; L.hitMetal = chanceMetal; }
        if (diel && !chanceReflect) tdir = refract3(L.dir, outward, niOverNt);
        L.dir = tdir;
        L.chanceReflect = chanceReflect;
        L.back = back;
        L.diel = diel;
        L.neeLobe = kNee && !back && !diel && !chanceGGX;
        NeeSample ns;
        if (kNee && L.neeLobe && nee_sample(c.sc, L.seed, L.vs.P, L.vs.N, L.rc, ns)) {
            f4 contrib = ns.contrib;
            if (L.hitMetal) contrib = contrib * pv_albedo<kTex>(c);
            c.slot(SL_NEE) = contrib.x; c.slot(SL_NEE + 1) = contrib.y;
            c.slot(SL_NEE + 2) = contrib.z; c.slot(SL_NEE + 3) = contrib.w;
            L.stage = pre_first ? ST_NEE_FIRST : ST_NEE_BOUNCE;
            emit(T, c, ns.o, ns.dir, kAny, ns.tmax);
        } else {
            L.stage = pre_first ? ST_FIRST : ST_BOUNCE;
            emit(T, c, fma3(L.vs.N, 0.001f * startPosOffset, L.vs.P), tdir, kClosest);
        }
        emitted = true;
    }
    return emitted;
}

// Camera ray of FHardwarePrimaryRayCaster (Shading.slang:286-304) for pixel index pix.
__device__ void start_pixel(Lane& L, Trav& T, const Ctx& c, int x, int y) {
    const GkrtFrameConstants& fc = c.fc;
    L.pix = y * c.P + x;
    L.seed.v[0] = (uint32_t)x; L.seed.v[1] = (uint32_t)y; L.seed.v[2] = fc.total_frames; L.seed.v[3] = 0u;
    float uvx = fmaf_(div_((float)x, (float)c.W), 2.0f, -1.0f);
    float uvy = fmaf_(div_((float)y, (float)c.H), 2.0f, -1.0f);
    if (fc.taa) {
        const uint32_t hi = fc.total_frames % 8u;
        uvx = uvx + div_(c_halton[2 * hi] - 0.5f, (float)c.W);
        uvy = uvy + div_(c_halton[2 * hi + 1] - 0.5f, (float)c.H);
    }
    const f2 disk = unit_disk(L.seed);
    const float ha = div_(fc.aperture, 2.0f);
    const float offx = ha * disk.x, offy = ha * disk.y;
    const f4 origin = mat4v(fc.model_view_inverse, F4(offx, offy, 0.0f, 1.0f));
    const f4 target = mat4v(fc.projection_inverse, F4(uvx, uvy, 1.0f, 1.0f));
    const f3 tn = normalize3(F3(fmaf_(target.x, fc.focus_distance, -offx), fmaf_(target.y, fc.focus_distance, -offy),
                                target.z * fc.focus_distance));
    const f4 direction = mat4v(fc.model_view_inverse, F4(tn.x, tn.y, tn.z, 0.0f));
    L.stage = ST_PRIMARY;
    emit(T, c, xyz(origin), xyz(direction), kClosest);
}

// kNee: emissive-triangle NEE compiled in (GKRT_NEE_EMISSIVE with a non-empty table); the
// reference mode runs the instantiation without it.
//
// Shared memory (dynamic): per-thread traversal stacks of stack_words entries (the scene's
// two-child depth bound), then the per-pixel slots. A stack no larger than the scene needs
// leaves the rest of the SM's 256 KB to L1, which serves the node fetches (measured on 1080p
// bricks: 72-word stacks 4.15 ms, 36-word 4.01 ms).
template <bool kNee, bool kTex>
__global__ void __launch_bounds__(kPtThreads, pt_blocks<kNee>()) k_trace_pass(ShadeScene sc, GkrtFrameConstants fc, int W, int H,
                                                           int P, PixelImages im, unsigned long long* counters,
                                                           unsigned int* work, int stack_words) {
    extern __shared__ uint32_t dyn_smem[];
    uint32_t* stack = dyn_smem;
    float* pslots = reinterpret_cast<float*>(dyn_smem + stack_words * kPtThreads);
    const int tid = threadIdx.x;
    const unsigned lane = tid & 31u;
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    const Ctx c{sc, fc, im, W, H, P, pslots + tid, kPtThreads, cn};
    const int tiles_x = (W + 7) / 8, tiles_y = (H + 3) / 4;
    const unsigned total = (unsigned)tiles_x * (unsigned)tiles_y * 32u;
    Lane L;
    L.pix = -1;
    L.stage = ST_PRIMARY;
    L.neeLobe = false;
    Trav T;
    T.done = true;
    bool tracing = false, exhausted = false;
    for (;;) {
        if (!tracing) {
            if (L.pix >= 0) tracing = advance<kNee, kTex>(L, T, c);
            while (!tracing && !exhausted) {
                // next pixel: warp-aggregated fetch over 8 x 4 tiles
                const unsigned m = __activemask();
                const int leader = __ffs(m) - 1;
                const unsigned rank = __popc(m & ((1u << lane) - 1u));
                unsigned base = 0;
                if ((int)lane == leader) base = atomicAdd(work, (unsigned)__popc(m));
                base = __shfl_sync(m, base, leader);
                const unsigned k = base + rank;
                if (k >= total) { exhausted = true; break; }
                const unsigned tile = k >> 5, in = k & 31u;
                const int x = (int)((tile % (unsigned)tiles_x) * 8u + (in & 7u));
                const int y = (int)((tile / (unsigned)tiles_x) * 4u + (in >> 3));
                if (x >= W || y >= H) continue;
                start_pixel(L, T, c, x, y);
                tracing = true;
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, tracing) == 0u) break;
        // traversal phase: node steps while any lane can take one, then the postponed leaves
        // of all lanes together, until every ray of the warp is finished
        for (;;) {
            bool can = tracing && !T.done;
            while (__any_sync(0xFFFFFFFFu, can)) {
                if (can) can = trav_node_step(T, sc.S, stack + tid, kPtThreads, cn, stack_words);
            }
            if (tracing) {
                trav_leaf_step(T, sc.S, cn);
                if (trav_finished(T)) tracing = false;
            }
            if (__popc(__ballot_sync(0xFFFFFFFFu, tracing)) < kRefillBelow) break;
        }
    }
    flush_counters(cn, counters);
}

constexpr int kRqThreads = 128;

__global__ void __launch_bounds__(kRqThreads) k_trace_rays(SceneView S, const GkrtRay* rays, GkrtHit* hits,
                                                           uint32_t n, uint32_t mode,
                                                           unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kRqThreads];
    const uint32_t i = blockIdx.x * kRqThreads + threadIdx.x;
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    if (i < n) {
        GkrtRay r = rays[i];
        f3 o = F3(r.origin[0], r.origin[1], r.origin[2]), d = F3(r.dir[0], r.dir[1], r.dir[2]);
        GkrtHit h;
        h.t = -1.0f; h.b1 = 0.0f; h.b2 = 0.0f; h.inst = 0xFFFFFFFFu; h.prim = 0xFFFFFFFFu;
        h.pad[0] = h.pad[1] = h.pad[2] = 0u;
        cn.rays = 1;
        // hits with r.tmin <= t <= r.tmax (the reference's shaders pass EPS as TMin)
        const TraceOut t = mode == GKRT_TRACE_ANY
                               ? traverse<kAny, true>(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kRqThreads, cn)
                               : traverse<kClosest, true>(S, o, d, r.tmin, r.tmax, stack + threadIdx.x, kRqThreads, cn);
        if (t.hit) {
            ++cn.hits;
            const HitShade s = hit_shade(S, o, d, t.inst, t.tri);
            h.t = s.t; h.inst = t.inst; h.prim = t.prim;
            if (mode != GKRT_TRACE_ANY) { h.b1 = s.b1; h.b2 = s.b2; }
        }
        hits[i] = h;
    }
    flush_counters(cn, counters);
}

}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_trace_pass(const ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H, int P,
                                   const PixelImages& im, unsigned long long* counters, unsigned int* work,
                                   int num_sms, int stack_words, bool textured, cudaStream_t st) {
    if (stack_words < 1 || stack_words > kStackSize) return cudaErrorInvalidValue;
    const bool nee = fc.nee_mode == GKRT_NEE_EMISSIVE && sc.nemit > 0u;
    const bool tex = textured || (fc.has_sky && (fc.flags & GKRT_FRAME_SKY_TEXTURE));
    if (tex && !sc.tex) return cudaErrorInvalidValue;
    const size_t smem = (size_t)(stack_words + (tex ? SL_COUNT_TEX : SL_COUNT)) * kPtThreads * 4u;
    // resident blocks per SM of each instantiation and stack size, queried once per device
    static int occ[kMaxDevices][2][2][kStackSize + 1] = {};
    const int dev = current_device_slot();
    if (dev < 0) return cudaErrorInvalidDevice;
    int* o = &occ[dev][nee][tex][stack_words];
    cudaError_t e = cudaSuccess;
    if (!*o) {
        e = nee ? (tex ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, k_trace_pass<true, true>, kPtThreads, smem)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, k_trace_pass<true, false>, kPtThreads, smem))
                : (tex ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, k_trace_pass<false, true>, kPtThreads, smem)
                       : cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, k_trace_pass<false, false>, kPtThreads, smem));
        if (e != cudaSuccess) return e;
    }
    int per_sm = *o;
    if (per_sm < 1) per_sm = 1;
    const int pixels = W * H;
    int blocks = num_sms * per_sm;
    const int need = (pixels + kPtThreads - 1) / kPtThreads;
    if (blocks > need) blocks = need;
    e = cudaMemsetAsync(work, 0, sizeof(unsigned int), st);
    if (e != cudaSuccess) return e;
    if (nee && tex)
        k_trace_pass<true, true><<<blocks, kPtThreads, smem, st>>>(sc, fc, W, H, P, im, counters, work, stack_words);
    else if (nee)
        k_trace_pass<true, false><<<blocks, kPtThreads, smem, st>>>(sc, fc, W, H, P, im, counters, work, stack_words);
    else if (tex)
        k_trace_pass<false, true><<<blocks, kPtThreads, smem, st>>>(sc, fc, W, H, P, im, counters, work, stack_words);
    else
        k_trace_pass<false, false><<<blocks, kPtThreads, smem, st>>>(sc, fc, W, H, P, im, counters, work, stack_words);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_trace_rays(const SceneView& S, const GkrtRay* rays, GkrtHit* hits, uint32_t n,
                                   uint32_t mode, unsigned long long* counters, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    k_trace_rays<<<(n + kRqThreads - 1) / kRqThreads, kRqThreads, 0, st>>>(S, rays, hits, n, mode, counters);
    return cudaGetLastError();
}
