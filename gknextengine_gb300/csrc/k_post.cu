// k_post.cu — "reproject pass" and "compose pass" kernels for sm_103a.
//
// Reprojection follows assets/shaders/Process.ReProject.comp.slang:19-223; the compose
// pass follows assets/shaders/Process.DenoiseJBF.comp.slang:4-184 with the tone mappers of
// assets/shaders/common/Const_Func.slang:51-126. The edge-aware a-trous filter (5 x 5, three
// passes with steps 1, 2, 4) has no counterpart in the reference.
//
// All three are HBM-bound stencils over FP32 images (rows padded to a multiple of 4 pixels).
// Each 16 x 16 block stages the neighbourhoods it reads (image tile plus halo) into shared
// memory with 2D TMA loads (gk_tma.cuh), one mbarrier per block, then computes from shared
// memory; data-dependent reads (history at the reprojected position) go through L2. Reads
// outside the image are zero, as the TMA fill and the ld* helpers both give.
#include "gk_device.cuh"
#include "gk_tma.cuh"
#include "gkrt_internal.h"

namespace gk {

constexpr int kTile = 16;

struct ImgDims { int W, H, P; };   // width, height, pitch in pixels

GK_D bool inb(const ImgDims& g, int x, int y) { return x >= 0 && y >= 0 && x < g.W && y < g.H; }
GK_D f4 ld4(const float4* p, const ImgDims& g, int x, int y) {
    if (!inb(g, x, y)) return F4(0.0f, 0.0f, 0.0f, 0.0f);
    float4 v = __ldg(&p[(size_t)y * g.P + x]);
    return F4(v.x, v.y, v.z, v.w);
}
GK_D uint32_t ldu(const uint32_t* p, const ImgDims& g, int x, int y) {
    if (!inb(g, x, y)) return 0u;
    return __ldg(&p[(size_t)y * g.P + x]);
}
GK_D float lerpf(float a, float b, float t) { return fmaf_(t, b - a, a); }
GK_D f3 lerp3(f3 a, f3 b, float t) { return F3(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t)); }
GK_D f4 lerp4(f4 a, f4 b, float t) {
    return F4(lerpf(a.x, b.x, t), lerpf(a.y, b.y, t), lerpf(a.z, b.z, t), lerpf(a.w, b.w, t));
}
GK_D float4 st4(f4 v) { return make_float4(v.x, v.y, v.z, v.w); }
GK_D f4 tf4(const float4* t, int stride, int x, int y) {
    float4 v = t[y * stride + x];
    return F4(v.x, v.y, v.z, v.w);
}

// Arm the block's barrier (thread 0), then all threads wait. Returns false on a timeout.
struct TileLoad {
    uint64_t* bar;
    GK_D void begin() {
        if (threadIdx.x == 0) { mbar_init(bar, 1); mbar_fence_init(); }
        __syncthreads();
    }
    GK_D bool wait(uint32_t* err) { return mbar_wait_bounded(bar, 0u, err); }
};

// ---------------------------------------------------------------------------------------
// reprojection (Process.ReProject.comp.slang:71-223)

// calculateWeight (Process.ReProject.comp.slang:32-47) with the tap's distance term given as
// the reciprocal rd = 1 / (1.5 cd + 4) (a per-tap constant): the two divisions become
// multiplications, within a few ulps of the quotients.
GK_D float reproj_weight(float rd, bool same, bool center, f3 n, f3 cn) {
    if (center) return 0.4f;
    if (!same) return 0.0f;
    float nd = sat(dot3(n, cn));
    if (nd < 0.98f) return 0.0f;
    float nw = (nd - 0.98f) * 50.0f;   // 1 / (1 - 0.98)
    return (nw * 2.0f) * rd;
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

// staged neighbourhoods of one 16 x 16 block
constexpr int kRpHalo = 2;                          // 5 x 5 spatial fill
constexpr int kRpT = kTile + 2 * kRpHalo;           // 20 pixels
constexpr int kRpIdX = kTile + 8;                   // id tile starts 4 left (16-byte aligned x)
constexpr int kRpMv = kTile + 8;                    // motion read at 2x offsets: halo 4

__global__ void __launch_bounds__(256) k_reproject(ReprojectArgs a, const __grid_constant__ CUtensorMap m_sd,
                                                   const __grid_constant__ CUtensorMap m_ss,
                                                   const __grid_constant__ CUtensorMap m_nrm,
                                                   const __grid_constant__ CUtensorMap m_id,
                                                   const __grid_constant__ CUtensorMap m_mv) {
    __shared__ __align__(128) float4 t_sd[kRpT * kRpT];
    __shared__ __align__(128) float4 t_ss[kRpT * kRpT];
    __shared__ __align__(128) float4 t_nrm[kRpT * kRpT];
    __shared__ __align__(128) uint32_t t_id[kRpT * kRpIdX];
    __shared__ __align__(128) float2 t_mv[kRpMv * kRpMv];
    __shared__ float t_mvl[kRpMv * kRpMv];   // |motion| of each staged pixel (the taps' mir terms)
    __shared__ __align__(8) uint64_t bar;
    const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = x0 + tx, y = y0 + ty;
    const ImgDims g{a.W, a.H, a.P};
    if (a.progressive) {
        if (x < a.W && y < a.H) {
            const size_t pix = (size_t)y * a.P + x;
            const float k = 1.0f / 512.0f;
            a.acc_d[pix] = st4(lerp4(ld4(a.prev_d, g, x, y), ld4(a.src_d, g, x, y), k));
            a.acc_s[pix] = st4(lerp4(ld4(a.prev_s, g, x, y), ld4(a.src_s, g, x, y), k));
            a.acc_a[pix] = st4(lerp4(ld4(a.prev_a, g, x, y), ld4(a.src_a, g, x, y), k));
        }
        return;
    }
    TileLoad tl{&bar};
    tl.begin();
    if (threadIdx.x == 0) {
        const uint32_t bytes = 3u * kRpT * kRpT * 16u + kRpT * kRpIdX * 4u + kRpMv * kRpMv * 8u;
        mbar_expect_tx(&bar, bytes);
        tma_load_2d(t_sd, &m_sd, 4 * (x0 - kRpHalo), y0 - kRpHalo, &bar);
        tma_load_2d(t_ss, &m_ss, 4 * (x0 - kRpHalo), y0 - kRpHalo, &bar);
        tma_load_2d(t_nrm, &m_nrm, 4 * (x0 - kRpHalo), y0 - kRpHalo, &bar);
        tma_load_2d(t_id, &m_id, x0 - 4, y0 - kRpHalo, &bar);
        tma_load_2d(t_mv, &m_mv, 2 * (x0 - 4), y0 - 4, &bar);
    }
    // the block agrees on the load's outcome before the barrier below
    if (!__syncthreads_and(tl.wait(a.err) ? 1 : 0)) return;
    for (int i = threadIdx.x; i < kRpMv * kRpMv; i += 256) {
        const float2 m2 = t_mv[i];
        t_mvl[i] = sqrt_(fmaf_(m2.y, m2.y, m2.x * m2.x));
    }
    __syncthreads();
    if (x >= a.W || y >= a.H) return;
    const size_t pix = (size_t)y * a.P + x;
    // tile-local coordinates of (x, y)
    const int cx = tx + kRpHalo, cy = ty + kRpHalo;      // colour/normal tiles
    const int ix = tx + 4;                               // id tile (starts 4 left)
    const f4 cd = tf4(t_sd, kRpT, cx, cy), cs = tf4(t_ss, kRpT, cx, cy), ca = ld4(a.src_a, g, x, y);
    const float2 mv2 = t_mv[(ty + 4) * kRpMv + (tx + 4)];
    const float fxm = (float)x + mv2.x, fym = (float)y + mv2.y;
    const float flx = floorf(fxm), fly = floorf(fym);
    const int px = (int)flx, py = (int)fly;
    const bool inside = px < a.W && py < a.H && px >= -1 && py >= -1;
    const uint32_t cur = t_id[cy * kRpIdX + ix];
    uint32_t p0 = ldu(a.id1, g, px, py);
    const bool miss = cur == 65535u;
    const uint32_t moment = ldu(a.moment, g, x, y);
    if (miss || !inside || moment > 0u) {
        a.acc_d[pix] = st4(cd);
        a.acc_s[pix] = st4(cs);
        a.acc_a[pix] = st4(ca);
        return;
    }
    const f3 cn = xyz(tf4(t_nrm, kRpT, cx, cy));
    f4 sd = F4(0.0f, 0.0f, 0.0f, 0.0f), ss = F4(0.0f, 0.0f, 0.0f, 0.0f);
    float tw = 0.0f, mir = 0.0f;
    // 1 / (1.5 d + 4) of the tap distance d = sqrt(ox^2 + oy^2), six values (r^2 = 0, 1, 2, 4, 5, 8)
    float dtab[6];
#pragma unroll
    for (int q = 0; q < 6; ++q)
        dtab[q] = div_(1.0f, fmaf_(sqrt_((float)(q < 3 ? q : (q == 3 ? 4 : (q == 4 ? 5 : 8)))), 1.5f, 4.0f));
#pragma unroll
    for (int oy = -2; oy <= 2; ++oy) {
#pragma unroll
        for (int ox = -2; ox <= 2; ++ox) {
            const uint32_t pid = t_id[(cy + oy) * kRpIdX + (ix + ox)];
            const f3 wn = xyz(tf4(t_nrm, kRpT, cx + ox, cy + oy));
            const int r2 = ox * ox + oy * oy;
            const float rd = dtab[r2 < 3 ? r2 : (r2 == 4 ? 3 : (r2 == 5 ? 4 : 5))];
            const float w = reproj_weight(rd, pid == cur, ox == 0 && oy == 0, wn, cn);
            sd = sd + tf4(t_sd, kRpT, cx + ox, cy + oy) * w;
            ss = ss + tf4(t_ss, kRpT, cx + ox, cy + oy) * w;
            tw = tw + w;
            mir = mir + t_mvl[(ty + 4 + 2 * oy) * kRpMv + (tx + 4 + 2 * ox)];
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

// ---------------------------------------------------------------------------------------
// compose: remodulation and tone map (Process.DenoiseJBF.comp.slang:145-181)

// GranTurismoTonemapper (Const_Func.slang:100-121). The toe (T) and shoulder (S) curves are
// evaluated only where their weight is not zero; powf is the fast form (__powf, a few ulps).
GK_D float gt_tonemap(float x) {
    const float P = 1.0f, a = 0.7f, m = 0.22f, l = 0.4f, c = 1.33f, b = 0.0f, e = 2.71828f;
    const float l0 = div_((P - m) * l, a);
    const float L_x = m + a * (x - m);
    const float S0 = m + l0, S1 = m + a * l0;
    const float C2 = div_(a * P, P - S1);
    float w0;
    if (x <= 0.0f) w0 = 1.0f;
    else if (x >= m) w0 = 0.0f;
    else { float q = div_(x, m); w0 = 1.0f - (q * q) * (3.0f - 2.0f * q); }
    const float w2 = x <= m + l0 ? 0.0f : 1.0f;
    const float w1 = (1.0f - w0) - w2;
    const float T_x = w0 != 0.0f ? m * __powf(div_(x, m), c) + b : 0.0f;
    const float S_x = w2 != 0.0f ? P - (P - S1) * __powf(e, -div_(C2 * (x - S0), P)) : 0.0f;
    return (T_x * w0 + L_x * w1) + S_x * w2;
}
GK_D float pq_encode(float v) {
    const float m1 = 0.1593017578125f, m2 = 78.84375f, c1 = 0.8359375f, c2 = 18.8515625f, c3 = 18.6875f;
    float Lm = powf(div_(v, 10000.0f), m1);
    float N = (c1 + c2 * Lm) * div_(1.0f, 1.0f + c3 * Lm);
    return powf(N, m2);
}
GK_D void write_composed(const ComposeArgs& a, size_t pix, f3 total) {
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

// joint bilateral filter (Process.DenoiseJBF.comp.slang:49-148): 36 taps at stride 2 over
// 11 x 11; the 26 x 26 diffuse neighbourhood of the block is staged by TMA. The spatial weight
// takes four values (computed once per pixel); the range weight uses the fast exponential
// (__expf, relative error below 1e-6 where the weight matters).
constexpr int kJbfHalo = 5;
constexpr int kJbfT = kTile + 2 * kJbfHalo;   // 26

__global__ void __launch_bounds__(256) k_compose_jbf(ComposeArgs a, const __grid_constant__ CUtensorMap m_d) {
    __shared__ __align__(128) float4 t_d[kJbfT * kJbfT];
    __shared__ __align__(8) uint64_t bar;
    const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = x0 + tx, y = y0 + ty;
    const ImgDims g{a.W, a.H, a.P};
    if (a.bf_size > 0u) {
        TileLoad tl{&bar};
        tl.begin();
        if (threadIdx.x == 0) {
            mbar_expect_tx(&bar, kJbfT * kJbfT * 16u);
            tma_load_2d(t_d, &m_d, 4 * (x0 - kJbfHalo), y0 - kJbfHalo, &bar);
        }
        if (!tl.wait(a.err)) return;
    }
    if (x >= a.W || y >= a.H) return;
    const size_t pix = (size_t)y * a.P + x;
    f3 total;
    if (a.bf_size > 0u) {
        const f3 eps = F3(0.001f, 0.001f, 0.001f);
        const f3 lw = F3(0.212671f, 0.715160f, 0.072169f);
        const int cx = tx + kJbfHalo, cy = ty + kJbfHalo;
        const f3 cc = xyz(tf4(t_d, kJbfT, cx, cy)) + eps;
        const f3 cspec = xyz(ld4(a.acc_s, g, x, y)) + eps;
        const float clum = dot3(cc, lw);
        const float sigmaL = a.bf_sigma_lum * 100.0f;
        const float den_s = (2.0f * a.bf_sigma) * a.bf_sigma, den_l = (2.0f * sigmaL) * sigmaL;
        // spatial weights: i^2 + j^2 over the taps takes the values 2, 10, 18, 26, 34, 50, and
        // dist = sat((i^2 + j^2) / 25) is 1 from 26 on
        float fs[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const float dist = sat(div_((float)(q < 3 ? 2 + 8 * q : 26), 25.0f));
            fs[q] = expf(div_(-(dist * dist), den_s));
        }
        const float ninv_l = -div_(1.0f, den_l);
        total = F3(0.0f, 0.0f, 0.0f);
        float wsum = 0.0f;
#pragma unroll
        for (int i = -5; i <= 5; i += 2) {
#pragma unroll
            for (int j = -5; j <= 5; j += 2) {
                const int r2 = i * i + j * j;
                const float Fi = r2 == 2 ? fs[0] : (r2 == 10 ? fs[1] : (r2 == 18 ? fs[2] : fs[3]));
                const f3 ci = xyz(tf4(t_d, kJbfT, cx + j, cy + i)) + eps;
                const float lumi = dot3(ci, lw);
                const float dl = (clum - lumi) * (clum - lumi);
                const float Li = __expf((dl * dl) * ninv_l);
                const float w = Fi * Li;
                total = total + ci * w;
                wsum = wsum + w;
            }
        }
        total = F3(div_(total.x, wsum), div_(total.y, wsum), div_(total.z, wsum));
        const f3 al = xyz(ld4(a.acc_a, g, x, y));
        total = F3(fmaf_(total.x, al.x, cspec.x), fmaf_(total.y, al.y, cspec.y), fmaf_(total.z, al.z, cspec.z));
    } else {
        const f3 d = xyz(ld4(a.acc_d, g, x, y)), s = xyz(ld4(a.acc_s, g, x, y)), al = xyz(ld4(a.acc_a, g, x, y));
        total = F3(fmaf_(d.x, al.x, s.x), fmaf_(d.y, al.y, s.y), fmaf_(d.z, al.z, s.z));
    }
    write_composed(a, pix, total);
}

// ---------------------------------------------------------------------------------------
// edge-aware a-trous filter (no counterpart in the reference)
//
// Pass with step s over the demodulated diffuse: 5 x 5 taps at offsets s * (-2..2) with the
// B3-spline weights h = (1/16, 1/4, 3/8, 1/4, 1/16) per axis, multiplied by
//   normal weight  max(0, n_p . n_q)^16,
//   luminance weight  exp(-|L_p - L_q| / sigma_L)  (sigma_L = bf_sigma_lum),
//   0 when the object ids differ or q lies outside the image.
// Three passes with s = 1, 2, 4; the last one remodulates (x albedo + specular) and tone maps.

GK_D float b3(int k) { return k == 0 ? 0.375f : (k == 1 ? 0.25f : 0.0625f); }
GK_D float pow16(float v) { float a = v * v; a = a * a; a = a * a; return a * a; }

// One pass, templated on its step S so that every tap's shared-memory offset is an immediate.
// The taps read the luminance from the colour's fourth channel: the first pass (S = 1) writes
// it into its staged tile after the load (each thread its share), and every pass but the last
// stores its output with the output's luminance there, which only the next pass reads. The
// image bounds are tested once per tap row and column.
template <int S>
__global__ void __launch_bounds__(256) k_atrous(AtrousArgs a, const __grid_constant__ CUtensorMap m_in,
                                                const __grid_constant__ CUtensorMap m_nrm,
                                                const __grid_constant__ CUtensorMap m_id) {
    constexpr int halo = 2 * S, T = kTile + 2 * halo;
    constexpr int hid = (halo + 3) & ~3, Tid = kTile + 2 * hid;   // id tile starts on a 16-byte boundary
    __shared__ __align__(128) float4 t_c[T * T];
    __shared__ __align__(128) float4 t_n[T * T];
    __shared__ __align__(128) uint32_t t_id[T * Tid];
    __shared__ __align__(8) uint64_t bar;
    const int x0 = blockIdx.x * kTile, y0 = blockIdx.y * kTile;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const int x = x0 + tx, y = y0 + ty;
    TileLoad tl{&bar};
    tl.begin();
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (uint32_t)(T * T) * 32u + (uint32_t)(Tid * T) * 4u);
        tma_load_2d(t_c, &m_in, 4 * (x0 - halo), y0 - halo, &bar);
        tma_load_2d(t_n, &m_nrm, 4 * (x0 - halo), y0 - halo, &bar);
        tma_load_2d(t_id, &m_id, x0 - hid, y0 - halo, &bar);
    }
    // the block agrees on the load's outcome before the barriers below
    if (!__syncthreads_and(tl.wait(a.err) ? 1 : 0)) return;
    const int cx = tx + halo, cy = ty + halo;
    const f3 lw = F3(0.212671f, 0.715160f, 0.072169f);
    if (S == 1) {
        for (int i = threadIdx.x; i < T * T; i += 256) {
            float4 v = t_c[i];
            v.w = dot3(F3(v.x, v.y, v.z), lw);
            t_c[i] = v;
        }
        __syncthreads();
    }
    if (x >= a.W || y >= a.H) return;
    const size_t pix = (size_t)y * a.P + x;
    const float4* cbase = t_c + cy * T + cx;
    const float4* nbase = t_n + cy * T + cx;
    const uint32_t* ibase = t_id + cy * Tid + tx + hid;
    const float4 c4 = *cbase;
    const f3 np = xyz(tf4(t_n, T, cx, cy));
    const uint32_t idp = *ibase;
    const float lp = c4.w;
    const float inv_sl = div_(1.0f, fmaxf(a.sigma_lum, 1e-4f));
    bool vx[5], vy[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        const int qx = x + (k - 2) * S, qy = y + (k - 2) * S;
        vx[k] = qx >= 0 && qx < a.W;
        vy[k] = qy >= 0 && qy < a.H;
    }
    f3 sum = F3(0.0f, 0.0f, 0.0f);
    float wsum = 0.0f;
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            if (!(vx[dx + 2] && vy[dy + 2])) continue;
            if (ibase[dy * S * Tid + dx * S] != idp) continue;
            const float4 cq = cbase[dy * S * T + dx * S];
            const float4 nq = nbase[dy * S * T + dx * S];
            const float wn = pow16(fmaxf(fmaf_(np.z, nq.z, fmaf_(np.y, nq.y, np.x * nq.x)), 0.0f));
            // fast exponential (__expf): relative error below 1e-6 where the weight matters
            const float wl = __expf(-(fabsf(lp - cq.w) * inv_sl));
            const float w = ((b3(dx < 0 ? -dx : dx) * b3(dy < 0 ? -dy : dy)) * wn) * wl;
            sum = sum + F3(cq.x, cq.y, cq.z) * w;
            wsum = wsum + w;
        }
    }
    // the centre tap always passes (weight 0.140625 > 0)
    const f3 f = F3(div_(sum.x, wsum), div_(sum.y, wsum), div_(sum.z, wsum));
    if (!a.last) {
        a.out[pix] = make_float4(f.x, f.y, f.z, dot3(f, lw));
        return;
    }
    const ImgDims g{a.W, a.H, a.P};
    const f3 al = xyz(ld4(a.albedo, g, x, y)), sp = xyz(ld4(a.spec, g, x, y));
    ComposeArgs c;
    c.W = a.W; c.H = a.H; c.P = a.P; c.bf_size = 0u; c.hdr = a.hdr; c.paper_white_nit = a.paper_white_nit;
    c.out = a.final_out; c.out_linear = a.final_linear;
    write_composed(c, pix, F3(fmaf_(f.x, al.x, sp.x), fmaf_(f.y, al.y, sp.y), fmaf_(f.z, al.z, sp.z)));
}

}  // namespace gk

using namespace gk;

namespace {
// 2D maps over float4 / u32 / float2 images with the given box in pixels.
cudaError_t map_f4(CUtensorMap* m, const void* base, int W, int H, int P, int bw, int bh) {
    return gkrt_encode_tmap_2d(m, base, 4u * W, H, 16u * P, 4u * bw, bh, true);
}
cudaError_t map_u32(CUtensorMap* m, const void* base, int W, int H, int P, int bw, int bh) {
    return gkrt_encode_tmap_2d(m, base, W, H, 4u * P, bw, bh, false);
}
cudaError_t map_f2(CUtensorMap* m, const void* base, int W, int H, int P, int bw, int bh) {
    return gkrt_encode_tmap_2d(m, base, 2u * W, H, 8u * P, 2u * bw, bh, true);
}
}  // namespace

namespace gk {
namespace {
// the learned denoiser's output (dense W x H x 4, log(1 + radiance)) through the compose writer
__global__ void k_unet_compose(ComposeArgs a, const float* y) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, yy = blockIdx.y;
    if (x >= a.W || yy >= a.H) return;
    const float* v = y + ((size_t)yy * a.W + x) * 4;
    write_composed(a, (size_t)yy * a.P + x,
                   F3(fmaxf(expm1f(fminf(v[0], kUnetMaxLog)), 0.0f), fmaxf(expm1f(fminf(v[1], kUnetMaxLog)), 0.0f),
                      fmaxf(expm1f(fminf(v[2], kUnetMaxLog)), 0.0f)));
}
}  // namespace
}  // namespace gk

cudaError_t gkrt_launch_unet_compose(const ComposeArgs& a, const float* y, cudaStream_t st) {
    k_unet_compose<<<dim3((a.W + 127) / 128, a.H), 128, 0, st>>>(a, y);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_reproject(const ReprojectArgs& a, cudaStream_t st) {
    CUtensorMap m_sd, m_ss, m_nrm, m_id, m_mv;
    cudaError_t e;
    if ((e = map_f4(&m_sd, a.src_d, a.W, a.H, a.P, kRpT, kRpT)) != cudaSuccess) return e;
    if ((e = map_f4(&m_ss, a.src_s, a.W, a.H, a.P, kRpT, kRpT)) != cudaSuccess) return e;
    if ((e = map_f4(&m_nrm, a.normal, a.W, a.H, a.P, kRpT, kRpT)) != cudaSuccess) return e;
    if ((e = map_u32(&m_id, a.id0, a.W, a.H, a.P, kRpIdX, kRpT)) != cudaSuccess) return e;
    if ((e = map_f2(&m_mv, a.motion, a.W, a.H, a.P, kRpMv, kRpMv)) != cudaSuccess) return e;
    dim3 grid((a.W + kTile - 1) / kTile, (a.H + kTile - 1) / kTile);
    k_reproject<<<grid, 256, 0, st>>>(a, m_sd, m_ss, m_nrm, m_id, m_mv);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_compose(const ComposeArgs& a, cudaStream_t st) {
    CUtensorMap m_d;
    cudaError_t e;
    if ((e = map_f4(&m_d, a.acc_d, a.W, a.H, a.P, kJbfT, kJbfT)) != cudaSuccess) return e;
    dim3 grid((a.W + kTile - 1) / kTile, (a.H + kTile - 1) / kTile);
    k_compose_jbf<<<grid, 256, 0, st>>>(a, m_d);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_atrous(const AtrousArgs& base, const float4* in, float4* tmp0, float4* tmp1,
                               cudaStream_t st) {
    dim3 grid((base.W + kTile - 1) / kTile, (base.H + kTile - 1) / kTile);
    const float4* src = in;
    float4* bufs[2] = {tmp0, tmp1};
    for (int p = 0; p < 3; ++p) {
        AtrousArgs a = base;
        a.step = 1 << p;
        a.last = p == 2 ? 1u : 0u;
        a.out = bufs[p & 1];
        const int T = kTile + 4 * a.step, Tid = kTile + 2 * ((2 * a.step + 3) & ~3);
        CUtensorMap m_in, m_n, m_id;
        cudaError_t e;
        if ((e = map_f4(&m_in, src, a.W, a.H, a.P, T, T)) != cudaSuccess) return e;
        if ((e = map_f4(&m_n, a.normal, a.W, a.H, a.P, T, T)) != cudaSuccess) return e;
        if ((e = map_u32(&m_id, a.id0, a.W, a.H, a.P, Tid, T)) != cudaSuccess) return e;
        if (p == 0) k_atrous<1><<<grid, 256, 0, st>>>(a, m_in, m_n, m_id);
        else if (p == 1) k_atrous<2><<<grid, 256, 0, st>>>(a, m_in, m_n, m_id);
        else k_atrous<4><<<grid, 256, 0, st>>>(a, m_in, m_n, m_id);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
        src = a.out;
    }
    return cudaSuccess;
}
