// k_post.cu — "reproject pass" and "compose pass" kernels for sm_103a.
//
// Reprojection follows assets/shaders/Process.ReProject.comp.slang:19-223; the compose
// pass follows assets/shaders/Process.DenoiseJBF.comp.slang:4-184 with the tone mappers of
// assets/shaders/common/Const_Func.slang:51-126. Both are HBM-bound stencils. Images are
// dense FP32 arrays (pitch = width); a read outside the image returns zero.
#include "gk_device.cuh"
#include "gkrt_internal.h"

namespace gk {

struct ImgDims { int W, H; };

GK_D bool inb(const ImgDims& g, int x, int y) { return x >= 0 && y >= 0 && x < g.W && y < g.H; }
GK_D f4 ld4(const float4* p, const ImgDims& g, int x, int y) {
    if (!inb(g, x, y)) return F4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 v = __ldg(&p[(size_t)y * g.W + x]);
    return F4(v.x, v.y, v.z, v.w);
}
GK_D f2 ld2(const float2* p, const ImgDims& g, int x, int y) {
    f2 r; r.x = 0.0f; r.y = 0.0f;
    if (!inb(g, x, y)) return r;
    float2 v = __ldg(&p[(size_t)y * g.W + x]);
    r.x = v.x; r.y = v.y;
    return r;
}
GK_D uint32_t ldu(const uint32_t* p, const ImgDims& g, int x, int y) {
    if (!inb(g, x, y)) return 0u;
    return __ldg(&p[(size_t)y * g.W + x]);
}
GK_D float lerpf(float a, float b, float t) { return fmaf_(t, b - a, a); }
GK_D f3 lerp3(f3 a, f3 b, float t) { return F3(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t)); }
GK_D f4 lerp4(f4 a, f4 b, float t) {
    return F4(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t), lerpf(a.w, b.w, t));
}
GK_D float4 st4(f4 v) { return make_float4(v.x, v.y, v.z, v.w); }

// calculateWeight (Process.ReProject.comp.slang:32-47)
GK_D float reproj_weight(float cd, bool same, bool center, f3 n, f3 cn) {
    if (center) return 0.4f;
    if (!same) return 0.0f;
    float nd = sat(dot3(n, cn));
    if (nd < 0.98f) return 0.0f;
    float nw = div_(nd - 0.98f, 1.0f - 0.98f);
    return div_(nw * 2.0f, fmaf_(cd, 1.5f, 4.0f));
}

// FilterHistoryColor (Process.ReProject.comp.slang:49-68)
GK_D f3 history(const float4* prev, const ImgDims& g, f2 sub, int px, int py, uint32_t cur, uint32_t p0,
                uint32_t p1, uint32_t p2, uint32_t p3, f3 c) {
    f3 h0 = cur == p0 ? xyz(ld4(prev, g, px, py)) : c;
    f3 h1 = cur == p1 ? xyz(ld4(prev, g, px + 1, py)) : c;
    f3 h2 = cur == p2 ? xyz(ld4(prev, g, px, py + 1)) : c;
    f3 h3 = cur == p3 ? xyz(ld4(prev, g, px + 1, py + 1)) : c;
    f3 h = lerp3(lerp3(h0, h1, sub.x), lerp3(h2, h3, sub.x), sub.y);
    return F3(fminf(fmaxf(h.x, 0.0f), 1600.0f), fminf(fmaxf(h.y, 0.0f), 1600.0f), fminf(fmaxf(h.z, 0.0f), 1600.0f));
}

__global__ void __launch_bounds__(256) k_reproject(ReprojectArgs a) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    const ImgDims g{a.W, a.H};
    if (x >= a.W || y >= a.H) return;
    const size_t pix = (size_t)y * a.W + x;
    if (a.progressive) {
        const float k = 1.0f / 512.0f;
        a.acc_d[pix] = st4(lerp4(ld4(a.prev_d, g, x, y), ld4(a.src_d, g, x, y), k));
        a.acc_s[pix] = st4(lerp4(ld4(a.prev_s, g, x, y), ld4(a.src_s, g, x, y), k));
        a.acc_a[pix] = st4(lerp4(ld4(a.prev_a, g, x, y), ld4(a.src_a, g, x, y), k));
        return;
    }
    const f4 cd = ld4(a.src_d, g, x, y), cs = ld4(a.src_s, g, x, y), ca = ld4(a.src_a, g, x, y);
    const f2 mv = ld2(a.motion, g, x, y);
    const float fxm = (float)x + mv.x, fym = (float)y + mv.y;
    const float flx = floorf(fxm), fly = floorf(fym);
    const int px = (int)flx, py = (int)fly;
    const bool inside = px < a.W && py < a.H && px >= -1 && py >= -1;
    const uint32_t cur = ldu(a.id0, g, x, y);
    uint32_t p0 = ldu(a.id1, g, px, py);
    const bool miss = cur == 65535u;
    const uint32_t moment = ldu(a.moment, g, x, y);
    if (miss || !inside || moment > 0u) {
        a.acc_d[pix] = st4(cd);
        a.acc_s[pix] = st4(cs);
        a.acc_a[pix] = st4(ca);
        return;
    }
    const f3 cn = xyz(ld4(a.normal, g, x, y));
    f4 sd = F4(0.0f, 0.0f, 0.0f, 0.0f), ss = F4(0.0f, 0.0f, 0.0f, 0.0f);
    float tw = 0.0f, mir = 0.0f;
    for (int oy = -2; oy <= 2; ++oy) {
        for (int ox = -2; ox <= 2; ++ox) {
            const int sx = x + ox, sy = y + oy;
            const uint32_t pid = ldu(a.id0, g, sx, sy);
            const f3 wn = xyz(ld4(a.normal, g, sx, sy));
            const float fox = (float)ox, foy = (float)oy;
            const float w = reproj_weight(sqrt_(fmaf_(foy, foy, fox * fox)), pid == cur, ox == 0 && oy == 0, wn, cn);
            sd = sd + ld4(a.src_d, g, sx, sy) * w;
            ss = ss + ld4(a.src_s, g, sx, sy) * w;
            tw = tw + w;
            const f2 m2 = ld2(a.motion, g, x + 2 * ox, y + 2 * oy);
            mir = mir + sqrt_(fmaf_(m2.y, m2.y, m2.x * m2.x));
        }
    }
    sd = F4(div_(sd.x, tw), div_(sd.y, tw), div_(sd.z, tw), div_(sd.w, tw));
    ss = F4(div_(ss.x, tw), div_(ss.y, tw), div_(ss.z, tw), div_(ss.w, tw));
    uint32_t p1 = ldu(a.id1, g, px + 1, py), p2 = ldu(a.id1, g, px, py + 1), p3 = ldu(a.id1, g, px + 1, py + 1);
    if (fabsf(mir) < 0.1f) { p0 = cur; p1 = cur; p2 = cur; p3 = cur; }
    f2 sub; sub.x = fxm - flx; sub.y = fym - fly;
    const f3 hd = history(a.prev_d, g, sub, px, py, cur, p0, p1, p2, p3, xyz(sd));
    const f3 hs = history(a.prev_s, g, sub, px, py, cur, p0, p1, p2, p3, xyz(ss));
    const f3 ha = history(a.prev_a, g, sub, px, py, cur, p0, p1, p2, p3, xyz(ca));
    const float keep = sat(div_(1.0f, (float)(a.temporal_frames > 1u ? a.temporal_frames : 1u)));
    const f3 od = lerp3(hd, xyz(cd), keep), os = lerp3(hs, xyz(cs), keep), oa = lerp3(ha, xyz(ca), keep);
    a.acc_d[pix] = make_float4(od.x, od.y, od.z, ld4(a.prev_d, g, x, y).w);
    a.acc_s[pix] = make_float4(os.x, os.y, os.z, ld4(a.prev_s, g, x, y).w);
    a.acc_a[pix] = make_float4(oa.x, oa.y, oa.z, ld4(a.prev_a, g, x, y).w);
}

// GranTurismoTonemapper (Const_Func.slang:100-121)
GK_D float gt_tonemap(float x) {
    const float P = 1.0f, a = 0.7f, m = 0.22f, l = 0.4f, c = 1.33f, b = 0.0f, e = 2.71828f;
    const float l0 = div_((P - m) * l, a);
    const float L_x = m + a * (x - m);
    const float T_x = m * powf(div_(x, m), c) + b;
    const float S0 = m + l0, S1 = m + a * l0;
    const float C2 = div_(a * P, P - S1);
    const float S_x = P - (P - S1) * powf(e, -div_(C2 * (x - S0), P));
    float w0;
    if (x <= 0.0f) w0 = 1.0f;
    else if (x >= m) w0 = 0.0f;
    else { float q = div_(x, m); w0 = 1.0f - (q * q) * (3.0f - 2.0f * q); }
    const float w2 = x <= m + l0 ? 0.0f : 1.0f;
    const float w1 = (1.0f - w0) - w2;
    return (T_x * w0 + L_x * w1) + S_x * w2;
}
GK_D float pq_encode(float v) {
    const float m1 = 0.1593017578125f, m2 = 78.84375f, c1 = 0.8359375f, c2 = 18.8515625f, c3 = 18.6875f;
    float Lm = powf(div_(v, 10000.0f), m1);
    float N = (c1 + c2 * Lm) * div_(1.0f, 1.0f + c3 * Lm);
    return powf(N, m2);
}

__global__ void __launch_bounds__(256) k_compose(ComposeArgs a) {
    const int x = blockIdx.x * 16 + (threadIdx.x & 15), y = blockIdx.y * 16 + (threadIdx.x >> 4);
    if (x >= a.W || y >= a.H) return;
    const ImgDims g{a.W, a.H};
    const size_t pix = (size_t)y * a.W + x;
    f3 total;
    if (a.bf_size > 0u) {
        const f3 eps = F3(0.001f, 0.001f, 0.001f);
        const f3 lw = F3(0.212671f, 0.715160f, 0.072169f);
        const f3 cc = xyz(ld4(a.acc_d, g, x, y)) + eps;
        const f3 cspec = xyz(ld4(a.acc_s, g, x, y)) + eps;
        const float clum = dot3(cc, lw);
        const float sigmaL = a.bf_sigma_lum * 100.0f;
        const float den_s = (2.0f * a.bf_sigma) * a.bf_sigma, den_l = (2.0f * sigmaL) * sigmaL;
        total = F3(0.0f, 0.0f, 0.0f);
        float wsum = 0.0f;
        for (int i = -5; i <= 5; i += 2) {
            for (int j = -5; j <= 5; j += 2) {
                const f3 ci = xyz(ld4(a.acc_d, g, x + j, y + i)) + eps;
                const float lumi = dot3(ci, lw);
                const float dist = sat(div_((float)(i * i + j * j), 25.0f));
                const float dl = (clum - lumi) * (clum - lumi);
                const float Fi = expf(div_(-(dist * dist), den_s));
                const float Li = expf(div_(-(dl * dl), den_l));
                total = total + (ci * Fi) * Li;
                wsum = wsum + Fi * Li;
            }
        }
        total = F3(div_(total.x, wsum), div_(total.y, wsum), div_(total.z, wsum));
        const f3 al = xyz(ld4(a.acc_a, g, x, y));
        total = F3(fmaf_(total.x, al.x, cspec.x), fmaf_(total.y, al.y, cspec.y), fmaf_(total.z, al.z, cspec.z));
    } else {
        const f3 d = xyz(ld4(a.acc_d, g, x, y)), s = xyz(ld4(a.acc_s, g, x, y)), al = xyz(ld4(a.acc_a, g, x, y));
        total = F3(fmaf_(d.x, al.x, s.x), fmaf_(d.y, al.y, s.y), fmaf_(d.z, al.z, s.z));
    }
    a.out_linear[pix] = make_float4(total.x, total.y, total.z, 1.0f);
    if (a.hdr) {
        const float k = div_(a.paper_white_nit, 230.0f);
        float r = gt_tonemap(div_(total.x, 2000.0f)) * 2000.0f, gg = gt_tonemap(div_(total.y, 2000.0f)) * 2000.0f,
              bb = gt_tonemap(div_(total.z, 2000.0f)) * 2000.0f;
        a.out[pix] = make_float4(pq_encode(r * k), pq_encode(gg * k), pq_encode(bb * k), 1.0f);
    } else {
        const float k = div_(a.paper_white_nit, 40000.0f);
        a.out[pix] = make_float4(gt_tonemap(total.x * k), gt_tonemap(total.y * k), gt_tonemap(total.z * k), 1.0f);
    }
}

}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_reproject(const ReprojectArgs& a, cudaStream_t st) {
    dim3 grid((a.W + 15) / 16, (a.H + 15) / 16);
    k_reproject<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_compose(const ComposeArgs& a, cudaStream_t st) {
    dim3 grid((a.W + 15) / 16, (a.H + 15) / 16);
    k_compose<<<grid, 256, 0, st>>>(a);
    return cudaGetLastError();
}
