// k_adjoint.cu — differentiable rendering of the path-tracing estimator (path replay).
//
// No counterpart in the reference. The forward kernel evaluates the pass's estimator
// (FPathTracingRendererV2::Render / GetRayColor, assets/shaders/common/Shading.slang:1003-1184,
// reference NEE mode, no sun) for `spp` samples per pixel from the primary hit, and the
// composed linear radiance of the compose pass (diffuse x primary albedo + specular,
// Process.DenoiseJBF.comp.slang:147, without the filter). The backward kernel replays the
// same paths (same per-pixel RNG stream) and accumulates d loss / d material parameters:
//
//   albedo    every path is a product of albedo factors (the hit surface's albedo when the
//             bounce leaving the previous vertex was not a Schlick reflection, Shading.slang:
//             1053-1056; the primary albedo for metallic first bounces, :1159-1162; the
//             primary albedo of the remodulation) times the rest; d path / d factor k is the
//             product of the other factors and the rest (prefix x suffix, no division);
//   roughness the reference gives GGX-sampled bounces weight 1 and its roughness acts only
//             through the sampled direction. Sampling is detached here: the microfacet normal
//             m is drawn with roughness a_s and the bounce is weighted by p(m; a)/p(m; a_s),
//             where p is the density of the bounded VNDF sampler for a view along the
//             sampling axis (Eto and Tokuyoshi 2023; Const_Func.slang:310-340):
//                 p(m; a) = D(m; a) (axis . m) (1 + a^2),  D the GGX distribution.
//             At a = a_s the weight is exactly 1, so the value is the reference estimator's;
//             the gradient is the likelihood-ratio (score) term d log p / d a. The change of
//             the sampler's support with a is not differentiated.
//
// One thread per pixel, the samples in sequence; gradients are summed per block in shared
// memory (FP32) and added to FP64 global sums once per block.
#include "gk_shade.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kAdjThreads = 128;
constexpr int kMaxFactors = 24;    // albedo factors along one path (bounces + 2)
constexpr int kMaxGgx = 24;

struct Factor {
    f4 f;
    uint32_t mat;
};

struct PathRec {
    Factor fac[kMaxFactors];
    int nf;
    uint32_t ggx_mat[kMaxGgx];
    float ggx_score[kMaxGgx];
    int ng;
    f4 rest;           // product of every non-albedo multiplier (weights, sky, probes)
    bool overflow;
};

__device__ __forceinline__ void rec_factor(PathRec& R, f4 f, uint32_t mat) {
    if (R.nf < kMaxFactors) { R.fac[R.nf].f = f; R.fac[R.nf].mat = mat; ++R.nf; }
    else R.overflow = true;
}

__device__ __forceinline__ float ggx_density_ratio_terms(float a, float c) {
    // a^2 (1 + a^2) / (c^2 (a^2 - 1) + 1)^2, the a-dependent part of p(m; a)
    const float a2 = a * a;
    const float q = fmaf_(c * c, a2 - 1.0f, 1.0f);
    return div_(a2 * (1.0f + a2), q * q);
}

__device__ __forceinline__ float ggx_score(float a, float c) {
    // d/da log p(m; a) = 2/a + 2a/(1 + a^2) - 4 a c^2 / (c^2 (a^2 - 1) + 1)
    const float a2 = a * a, c2 = c * c;
    return (div_(2.0f, a) + div_(2.0f * a, 1.0f + a2)) - div_((4.0f * a) * c2, fmaf_(c2, a2 - 1.0f, 1.0f));
}

struct AdjCtx {
    const ShadeScene& sc;
    const GkrtFrameConstants& fc;
    const float* sample_rough;   // per material, or null: sample with the material's own
    uint32_t* stack;
    Counters& cn;
};

// GetRayColor (Shading.slang:1003-1082) with detached GGX sampling and path records.
// Returns true when the path ends.
__device__ bool adj_ray_color(const AdjCtx& a, Vtx& v, f3& dir, f4& color, Rng& seed, bool first,
                              bool& hitReflect, bool& hitMetal, PathRec& R) {
    const MatV mat = load_mat(a.sc, v.mat);
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
    float ggx_c = 0.0f, a_s = 0.0f;
    if (chanceGGX) {
        const f3 axis = reflect3(dir, outward);
        const uint32_t mi = v.mat < a.sc.nmat ? v.mat : a.sc.nmat - 1u;
        const float fs = a.sample_rough ? __ldg(&a.sample_rough[mi]) : mat.fuzz;
        const float r = sqrt_(fs);
        a_s = r * r;
        tdir = ggx_sample(seed, r, axis);
        ggx_c = dot3(axis, tdir);
    } else {
        tdir = align_normal(hemisphere_cos(seed), outward);
    }
    if (first) { hitReflect = chanceGGX; hitMetal = chanceMetal; }
    const bool refracted = diel && !chanceReflect;
    if (refracted) tdir = refract3(dir, outward, niOverNt);
    if (chanceGGX && !refracted && a_s > 1e-6f) {
        const float re = sqrt_(mat.fuzz);
        const float a_e = re * re;
        if (a_e != a_s) {
            const float w = div_(ggx_density_ratio_terms(a_e, ggx_c), ggx_density_ratio_terms(a_s, ggx_c));
            color = color * w;
            R.rest = R.rest * w;
        }
        if (R.ng < kMaxGgx) {
            R.ggx_mat[R.ng] = v.mat;
            R.ggx_score[R.ng] = a_e > 1e-6f ? ggx_score(a_e, ggx_c) : 0.0f;
            ++R.ng;
        } else {
            R.overflow = true;
        }
    }
    dir = tdir;
    ++a.cn.rays;
    const f3 org = fma3(v.N, 0.001f * startPosOffset, v.P);
    const TraceOut t = traverse<kClosest>(a.sc.S, org, tdir, kTmin, 1000.0f, a.stack, kAdjThreads, a.cn);
    if (t.hit) {
        v = hit_vertex(a.sc, org, tdir, t.inst, t.prim, t.tri);
        const MatV hm = load_mat(a.sc, v.mat);
        if (hm.model == GKRT_MAT_DIFFUSE_LIGHT || !chanceReflect) {
            color = color * hm.diffuse;
            rec_factor(R, hm.diffuse, v.mat);
        }
        if (back && !diel) {
            color = F4(0.5f, 0.5f, 0.5f, 0.0f);   // constant: no parameter reaches this path
            R.nf = 0;
            R.ng = 0;
            R.rest = color;
            return true;
        }
        return hm.model == GKRT_MAT_DIFFUSE_LIGHT;
    }
    const f4 s = sky(a.fc);
    color = color * s;
    R.rest = R.rest * s;
    return true;
}

// Camera ray of FHardwarePrimaryRayCaster (Shading.slang:286-304), as start_pixel.
__device__ void camera_ray(const GkrtFrameConstants& fc, int x, int y, int W, int H, Rng& seed, f3& o, f3& d) {
    float uvx = fmaf_(div_((float)x, (float)W), 2.0f, -1.0f);
    float uvy = fmaf_(div_((float)y, (float)H), 2.0f, -1.0f);
    if (fc.taa) {
        const uint32_t hi = fc.total_frames % 8u;
        uvx = uvx + div_(c_halton[2 * hi] - 0.5f, (float)W);
        uvy = uvy + div_(c_halton[2 * hi + 1] - 0.5f, (float)H);
    }
    const f2 disk = unit_disk(seed);
    const float ha = div_(fc.aperture, 2.0f);
    const float offx = ha * disk.x, offy = ha * disk.y;
    const f4 origin = mat4v(fc.model_view_inverse, F4(offx, offy, 0.0f, 1.0f));
    const f4 target = mat4v(fc.projection_inverse, F4(uvx, uvy, 1.0f, 1.0f));
    const f3 tn = normalize3(F3(fmaf_(target.x, fc.focus_distance, -offx), fmaf_(target.y, fc.focus_distance, -offy),
                                target.z * fc.focus_distance));
    const f4 direction = mat4v(fc.model_view_inverse, F4(tn.x, tn.y, tn.z, 0.0f));
    o = xyz(origin);
    d = xyz(direction);
}

template <bool kBackward>
__global__ void __launch_bounds__(kAdjThreads) k_adjoint(ShadeScene sc, GkrtFrameConstants fc, int W, int H,
                                                         uint32_t spp, const float* sample_rough, float4* image,
                                                         const float4* dimage, double* g_alb, double* g_rough,
                                                         unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kAdjThreads];
    extern __shared__ float sgrad[];   // backward: 4 per material (albedo rgb, roughness)
    const int tid = threadIdx.x;
    const uint32_t nm = sc.nmat;
    if (kBackward) {
        for (uint32_t i = tid; i < 4u * nm; i += kAdjThreads) sgrad[i] = 0.0f;
        __syncthreads();
    }
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    const AdjCtx a{sc, fc, sample_rough, stack + tid, cn};
    const int pix = blockIdx.x * kAdjThreads + tid;
    if (pix < W * H) {
        const int x = pix % W, y = pix / W;
        Rng seed;
        seed.v[0] = (uint32_t)x; seed.v[1] = (uint32_t)y; seed.v[2] = fc.total_frames; seed.v[3] = 0u;
        f3 o, d;
        camera_ray(fc, x, y, W, H, seed, o, d);
        ++cn.rays;
        const TraceOut t = traverse<kClosest>(sc.S, o, d, kTmin, 1000.0f, stack + tid, kAdjThreads, cn);
        f4 out = F4(0.0f, 0.0f, 0.0f, 1.0f);
        f4 g = F4(0.0f, 0.0f, 0.0f, 0.0f);
        if (kBackward) {
            const float4 gi = dimage[pix];
            g = F4(gi.x, gi.y, gi.z, 0.0f);
        }
        if (!t.hit) {
            const f4 s = sky(fc);
            out = F4(s.x, s.y, s.z, 1.0f);
        } else {
            Vtx pv = hit_vertex(sc, o, d, t.inst, t.prim, t.tri);
            const MatV pm = load_mat(sc, pv.mat);
            if (pm.model != GKRT_MAT_DIELECTRIC) pv.P = fma3(normalize3(d), -0.03f, pv.P);
            if (pm.model == GKRT_MAT_DIFFUSE_LIGHT) {
                out = F4(pm.diffuse.x, pm.diffuse.y, pm.diffuse.z, 1.0f);
            } else {
                const bool pdiel = pm.model == GKRT_MAT_DIELECTRIC;
                const uint32_t maxB = pdiel ? fc.max_number_of_bounces : fc.number_of_bounces;
                const f4 eye = mat4v(fc.model_view_inverse, F4(0.0f, 0.0f, 0.0f, 1.0f));
                const f4 ap = pm.diffuse;
                const float inv_spp = div_(1.0f, (float)spp);
                f4 fcol = F4(0.0f, 0.0f, 0.0f, 0.0f), frefl = F4(0.0f, 0.0f, 0.0f, 0.0f);
                for (uint32_t i = 0; i < spp; ++i) {
                    PathRec R;
                    R.nf = 0; R.ng = 0; R.rest = F4(1.0f, 1.0f, 1.0f, 1.0f); R.overflow = false;
                    f4 rc = F4(1.0f, 1.0f, 1.0f, 1.0f);
                    f3 dir = normalize3(pv.P - xyz(eye));
                    Vtx vs = pv;
                    bool hitReflect = false, hitMetal = false, dc = false;
                    const bool exitFirst = adj_ray_color(a, vs, dir, rc, seed, true, hitReflect, hitMetal, R);
                    if (!exitFirst) {
                        if (fc.fast_gather && !pdiel) {
                            const f4 pt = probe_term(sc, vs.P, vs.N);
                            rc = rc * pt;
                            R.rest = R.rest * pt;
                        } else {
                            for (uint32_t b = 1; b < maxB; ++b) {
                                if (adj_ray_color(a, vs, dir, rc, seed, false, dc, dc, R)) break;
                                const bool early = !pdiel && rnd1(seed) < 0.5f;
                                if (b == maxB - 1u || early) {
                                    const f4 pt = probe_term(sc, vs.P, vs.N);
                                    rc = rc * pt;
                                    R.rest = R.rest * pt;
                                    break;
                                }
                            }
                        }
                    }
                    if (hitMetal) {
                        rc = rc * ap;
                        rec_factor(R, ap, pv.mat);
                    }
                    if (hitReflect) frefl = frefl + rc;
                    else fcol = fcol + rc;
                    if (kBackward && !R.overflow) {
                        // upstream of this path's value: remodulated (diffuse) or not (specular)
                        const f4 u = hitReflect ? g * inv_spp : (g * ap) * inv_spp;
                        if (!hitReflect) {
                            const uint32_t mp = pv.mat < nm ? pv.mat : nm - 1u;
                            atomicAdd(&sgrad[4 * mp + 0], (g.x * rc.x) * inv_spp);
                            atomicAdd(&sgrad[4 * mp + 1], (g.y * rc.y) * inv_spp);
                            atomicAdd(&sgrad[4 * mp + 2], (g.z * rc.z) * inv_spp);
                        }
                        // d path / d factor k = prefix(k) * suffix(k) * rest
                        f4 pre = F4(1.0f, 1.0f, 1.0f, 1.0f);
                        for (int k = 0; k < R.nf; ++k) {
                            f4 suf = R.rest;
                            for (int j = k + 1; j < R.nf; ++j) suf = suf * R.fac[j].f;
                            const f4 dk = (pre * suf) * u;
                            const uint32_t mk = R.fac[k].mat < nm ? R.fac[k].mat : nm - 1u;
                            atomicAdd(&sgrad[4 * mk + 0], dk.x);
                            atomicAdd(&sgrad[4 * mk + 1], dk.y);
                            atomicAdd(&sgrad[4 * mk + 2], dk.z);
                            pre = pre * R.fac[k].f;
                        }
                        const float uc = fmaf_(u.z, rc.z, fmaf_(u.y, rc.y, u.x * rc.x));
                        for (int k = 0; k < R.ng; ++k) {
                            const uint32_t mk = R.ggx_mat[k] < nm ? R.ggx_mat[k] : nm - 1u;
                            atomicAdd(&sgrad[4 * mk + 3], uc * R.ggx_score[k]);
                        }
                    }
                }
                const float fs = (float)spp;
                fcol = F4(div_(fcol.x, fs), div_(fcol.y, fs), div_(fcol.z, fs), div_(fcol.w, fs));
                frefl = F4(div_(frefl.x, fs), div_(frefl.y, fs), div_(frefl.z, fs), div_(frefl.w, fs));
                out = F4(fmaf_(fcol.x, ap.x, frefl.x), fmaf_(fcol.y, ap.y, frefl.y), fmaf_(fcol.z, ap.z, frefl.z), 1.0f);
            }
        }
        if (!kBackward) image[pix] = make_float4(out.x, out.y, out.z, out.w);
    }
    if (kBackward) {
        __syncthreads();
        for (uint32_t i = tid; i < nm; i += kAdjThreads) {
            if (sgrad[4 * i] != 0.0f) atomicAdd(&g_alb[3 * i + 0], (double)sgrad[4 * i]);
            if (sgrad[4 * i + 1] != 0.0f) atomicAdd(&g_alb[3 * i + 1], (double)sgrad[4 * i + 1]);
            if (sgrad[4 * i + 2] != 0.0f) atomicAdd(&g_alb[3 * i + 2], (double)sgrad[4 * i + 2]);
            if (sgrad[4 * i + 3] != 0.0f) atomicAdd(&g_rough[i], (double)sgrad[4 * i + 3]);
        }
    }
    // ray counters: warp sums, one atomic per warp
    unsigned long long r = cn.rays;
    for (int o2 = 16; o2 > 0; o2 >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o2);
    if ((tid & 31) == 0 && r) atomicAdd(&counters[0], r);
}

// Material parameters from device arrays: diffuse rgb and fuzziness of materials
// [first, first + count).
__global__ void k_set_params(GkrtMaterial* mats, const float* alb, const float* rough, uint32_t first,
                             uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    GkrtMaterial& m = mats[first + i];
    if (alb) {
        m.diffuse[0] = alb[3 * i];
        m.diffuse[1] = alb[3 * i + 1];
        m.diffuse[2] = alb[3 * i + 2];
    }
    if (rough) m.fuzziness = rough[i];
}

}  // namespace

}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_adjoint(const ShadeScene& sc, const GkrtFrameConstants& fc, int W, int H, uint32_t spp,
                                const float* sample_rough, float4* image, const float4* dimage, double* g_alb,
                                double* g_rough, unsigned long long* counters, cudaStream_t st) {
    const int blocks = (W * H + kAdjThreads - 1) / kAdjThreads;
    if (dimage) {
        const size_t smem = 4u * sc.nmat * sizeof(float);
        cudaError_t e = cudaFuncSetAttribute(k_adjoint<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k_adjoint<true><<<blocks, kAdjThreads, smem, st>>>(sc, fc, W, H, spp, sample_rough, nullptr, dimage, g_alb,
                                                           g_rough, counters);
    } else {
        k_adjoint<false><<<blocks, kAdjThreads, 0, st>>>(sc, fc, W, H, spp, sample_rough, image, nullptr, nullptr,
                                                         nullptr, counters);
    }
    return cudaGetLastError();
}

cudaError_t gkrt_launch_set_params(GkrtMaterial* mats, const float* alb, const float* rough, uint32_t first,
                                   uint32_t count, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    k_set_params<<<(count + 127) / 128, 128, 0, st>>>(mats, alb, rough, first, count);
    return cudaGetLastError();
}
