// k_probes.cu — ambient-cube probe grid: voxelization and bake on the GPU (sm_103a).
//
// The probe grid (192 x 48 x 192 probes, 0.25 m apart, AmbientCube.slang:12-15) feeds the
// path termination of the rt pass (probe_term). Two kernels fill it:
//   k_probe_voxelize  the distance data of every probe: six axis rays and, in open space, six
//                     diagonal rays, as the reference's CPU voxelizer does with tinybvh
//                     (VoxelizeCube / InsideGeometry / DetectDistance,
//                     src/Assets/CPUAccelerationStructure.cpp:70-160);
//   k_probe_bake      one bake step of a slice of probes (Bake.HwAmbientCube.comp.slang:1-19,
//                     FGpuProbeGenerator::RenderAmbientCubeOnly and FaceTask,
//                     AmbientCube.slang:477-553, 656-690): per face 16 rays over a jittered
//                     4 x 4 grid, the bounce light of their hits from the probes around them,
//                     the sky, light 0 and the sun, blended into the packed colours with
//                     weight 1/8. Eight lanes serve one probe, six of them a face each.
// The bake reads the neighbour probes it interpolates from a snapshot of the grid taken
// before the step, so results do not depend on the order in which probes are updated (the
// reference reads and writes one buffer concurrently).
#include "gk_shade.cuh"
#include "gkrt_internal.h"

namespace gk {

namespace {

constexpr int kVoxThreads = 128;
constexpr int kBakeThreads = 128;
constexpr float kCubeUnit = 0.25f;
constexpr float kFastMaxTrace = 20.0f;          // FAST_MAX_TRACE_DISTANCE, Shading.slang:16
constexpr float kOcclusionMax = 1000.0f;        // PT_MAX_TRACE_DISTANCE of TraceOcclusion
constexpr float kInvSqrt3 = 0.577350269f;

__constant__ float c_grid4x4[32] = {-0.75f, -0.75f, -0.25f, -0.75f, 0.25f, -0.75f, 0.75f, -0.75f,
                                    -0.75f, -0.25f, -0.25f, -0.25f, 0.25f, -0.25f, 0.75f, -0.25f,
                                    -0.75f, 0.25f,  -0.25f, 0.25f,  0.25f, 0.25f,  0.75f, 0.25f,
                                    -0.75f, 0.75f,  -0.25f, 0.75f,  0.25f, 0.75f,  0.75f, 0.75f};
__constant__ float c_grid3x3[18] = {-0.667f, -0.667f, 0.0f, -0.667f, 0.667f, -0.667f, -0.667f, 0.0f, 0.0f,
                                    0.0f,    0.667f,  0.0f, -0.667f, 0.667f, 0.0f,    0.667f, 0.667f, 0.667f};

// Warp-aggregated flush of the ray counters (per-pass slots 0-5, total rays in slot 6).
__device__ __forceinline__ void flush_ray_counters(const Counters& c, unsigned long long* out) {
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

GK_D f3 probe_origin(uint32_t g) {
    const uint32_t y = g / (uint32_t)(kProbeXY * kProbeXY);
    const uint32_t z = (g - y * (uint32_t)(kProbeXY * kProbeXY)) / (uint32_t)kProbeXY;
    const uint32_t x = g - y * (uint32_t)(kProbeXY * kProbeXY) - z * (uint32_t)kProbeXY;
    return F3((float)x * kCubeUnit + kProbeOffX, (float)y * kCubeUnit + kProbeOffY, (float)z * kCubeUnit + kProbeOffZ);
}

GK_D f3 face_basis(int f) {   // +Y, -Y, +X, -X, +Z, -Z (the order of RenderAmbientCubeOnly)
    const float s = (f & 1) ? -1.0f : 1.0f;
    return f < 2 ? F3(0.0f, s, 0.0f) : (f < 4 ? F3(s, 0.0f, 0.0f) : F3(0.0f, 0.0f, s));
}

struct ProbeHit {
    bool hit, back;
    float t;
    uint32_t mat;
    Vtx v;
    float tu, tv;   // texture coordinates at the hit (0 without texcoords)
};

// Closest hit over [EPS, tmax]: its float t, material, whether the ray met the triangle's
// back (object-space face normal cross(v1 - v0, v2 - v1), CPUAccelerationStructure.cpp:193-196)
// and, if want_vertex, the shading vertex.
GK_D ProbeHit probe_trace(const ShadeScene& sc, f3 o, f3 d, float tmax, bool want_vertex, uint32_t* stk, int stride,
                          Counters& cn) {
    ProbeHit r;
    r.hit = false; r.back = false; r.t = 0.0f; r.mat = 0u; r.tu = 0.0f; r.tv = 0.0f;
    ++cn.rays;
    const TraceOut t = traverse<kClosest, true>(sc.S, o, d, kTmin, tmax, stk, stride, cn);
    if (!t.hit) return r;
    r.hit = true;
    const HitShade h = hit_shade(sc.S, o, d, t.inst, t.tri);
    r.t = h.t;
    const DevInst* ip = sc.S.inst + t.inst;
    const uint32_t ioff = __ldg(&ip->index_offset) + 3u * t.prim, voff = __ldg(&ip->vertex_offset);
    r.mat = __ldg(&sc.inst_mat[16u * t.inst + (__ldg(&sc.slots[__ldg(&sc.indices[ioff]) + voff]) & 15u)]);
    const f3 v0 = tri_v(sc.S.tris, t.tri, 0), v1 = tri_v(sc.S.tris, t.tri, 1), v2 = tri_v(sc.S.tris, t.tri, 2);
    const f3 a = v1 - v0, b = v2 - v1;
    const f3 n = F3(fmaf_(a.y, b.z, -(a.z * b.y)), fmaf_(a.z, b.x, -(a.x * b.z)), fmaf_(a.x, b.y, -(a.y * b.x)));
    float w[12];
#pragma unroll
    for (int k = 0; k < 12; ++k) w[k] = __ldg(&ip->winv[k]);
    const f3 dl = xvector(w, d);
    r.back = fmaf_(n.z, dl.z, fmaf_(n.y, dl.y, n.x * dl.x)) > 0.0f;
    if (want_vertex) {
        r.v = hit_vertex(sc, o, d, t.inst, t.prim, t.tri);
        if (sc.uv) {
            const HitAttr a = hit_attr(sc, o, d, t.inst, t.prim, t.tri);
            r.tu = a.u;
            r.tv = a.v;
        }
    }
    return r;
}

GK_D uint32_t pack10(f4 c) {   // packRGB10A2 (AmbientCube.slang:59-69), MAX_ILLUMINANCE 512
    const float r = mn(mx(c.x * 0.001953125f, 0.0f), 1.0f), g = mn(mx(c.y * 0.001953125f, 0.0f), 1.0f);
    const float b = mn(mx(c.z * 0.001953125f, 0.0f), 1.0f), a = mn(mx(c.w * 0.001953125f, 0.0f), 1.0f);
    return (uint32_t)(r * 1023.0f) | ((uint32_t)(g * 1023.0f) << 10) | ((uint32_t)(b * 1023.0f) << 20) |
           ((uint32_t)(a * 3.0f) << 30);
}

GK_D float lerpf_(float a, float b, float t) { return fmaf_(t, b - a, a); }

// sampleAmbientCubeHL2_DI (AmbientCube.slang:127-150): the direct colours only.
GK_D f4 cube_sample_di(const uint32_t* cube, f3 n) {
    const float wx = mx(n.x, 0.0f), wnx = mx(-n.x, 0.0f), wy = mx(n.y, 0.0f), wny = mx(-n.y, 0.0f);
    const float wz = mx(n.z, 0.0f), wnz = mx(-n.z, 0.0f);
    const float sum = ((((wx + wnx) + wy) + wny) + wz) + wnz;
    f4 col = F4(0.0f, 0.0f, 0.0f, 0.0f);
    col = col + unpack10(__ldg(&cube[10])) * wx;
    col = col + unpack10(__ldg(&cube[11])) * wnx;
    col = col + unpack10(__ldg(&cube[8])) * wy;
    col = col + unpack10(__ldg(&cube[9])) * wny;
    col = col + unpack10(__ldg(&cube[6])) * wz;
    col = col + unpack10(__ldg(&cube[7])) * wnz;
    return col * (sum > 0.0f ? div_(1.0f, sum) : 1.0f);
}

// interpolateAmbientCubesV2<DIAmbientCubeSampler> (AmbientCube.slang:290-382) over the snapshot.
GK_D f4 probe_di(const uint32_t* cubes, const uint32_t* voxels, f3 p, f3 n) {
    const float npx = div_(p.x - kProbeOffX, kCubeUnit), npy = div_(p.y - kProbeOffY, kCubeUnit),
                npz = div_(p.z - kProbeOffZ, kCubeUnit);
    if (!(npx >= 0.0f) || !(npy >= 0.0f) || !(npz >= 0.0f) || npx > (float)(kProbeXY - 2) ||
        npy > (float)(kProbeZ - 2) || npz > (float)(kProbeXY - 2))
        return F4(0.0f, 0.0f, 0.0f, 1.0f);
    const float fx = floorf(npx), fy = floorf(npy), fz = floorf(npz);
    const int bx = (int)fx, by = (int)fy, bz = (int)fz;
    const float frx = npx - fx, fry = npy - fy, frz = npz - fz;
    float tw = 0.0f;
    f4 res = F4(0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < 8; ++i) {
        const int ox = i & 1, oy = (i >> 1) & 1, oz = (i >> 2) & 1;
        const size_t id = (size_t)(by + oy) * kProbeXY * kProbeXY + (size_t)(bz + oz) * kProbeXY + (size_t)(bx + ox);
        const uint32_t u0 = __ldg(&voxels[id * 4 + 2]), u1 = __ldg(&voxels[id * 4 + 3]);
        const float d0y = div_((float)((u0 >> 8) & 0xFFu), 255.0f);
        if (d0y < 0.01f) continue;
        const float d0z = div_((float)((u0 >> 16) & 0xFFu), 255.0f), d0w = div_((float)((u0 >> 24) & 0xFFu), 255.0f);
        const float d1x = div_((float)(u1 & 0xFFu), 255.0f), d1y = div_((float)((u1 >> 8) & 0xFFu), 255.0f);
        const float d1z = div_((float)((u1 >> 16) & 0xFFu), 255.0f), d1w = div_((float)((u1 >> 24) & 0xFFu), 255.0f);
        const f3 pl = F3(frx - (float)ox, fry - (float)oy, frz - (float)oz);
        const float dist = len3(pl);
        const f3 dir = normalize3(pl);
        float hl = sqrt_(mx(dir.x, 0.0f)) * d1x;
        hl = hl + sqrt_(mx(-dir.x, 0.0f)) * d1y;
        hl = hl + sqrt_(mx(dir.y, 0.0f)) * d1z;
        hl = hl + sqrt_(mx(-dir.y, 0.0f)) * d1w;
        hl = hl + sqrt_(mx(dir.z, 0.0f)) * d0z;
        hl = hl + sqrt_(mx(-dir.z, 0.0f)) * d0w;
        if (dist > hl + 0.05f) continue;
        const float wx = ox == 0 ? 1.0f - frx : frx, wy = oy == 0 ? 1.0f - fry : fry, wz = oz == 0 ? 1.0f - frz : frz;
        const float wgt = (wx * wy) * wz;
        res = res + cube_sample_di(cubes + id * 14, n) * wgt;
        tw = tw + wgt;
    }
    if (tw > 0.0f) return F4(div_(res.x, tw), div_(res.y, tw), div_(res.z, tw), div_(res.w, tw));
    return F4(0.0f, 0.0f, 0.0f, 0.0f);
}

// VoxelizeCube (CPUAccelerationStructure.cpp:112-160) for probes [first, first + count).
// VoxelData words: matId, age (0), distances (minDist / unit, inside, +Z, -Z), (+X, -X, +Y, -Y).
__global__ void __launch_bounds__(kVoxThreads) k_probe_voxelize(ShadeScene sc, uint32_t first, uint32_t count,
                                                                uint4* voxels, unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kVoxThreads];
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    const uint32_t k = blockIdx.x * kVoxThreads + threadIdx.x;
    if (k < count) {
        const uint32_t g = first + k;
        const f3 o = probe_origin(g);
        uint32_t mat = 0u;
        float dist[6];
#pragma unroll 1
        for (int f = 0; f < 6; ++f) {   // InsideGeometry along +Y, -Y, +X, -X, +Z, -Z
            dist[f] = 255.0f;
            const ProbeHit h = probe_trace(sc, o, face_basis(f), kCubeUnit * 64.0f, false, stack + threadIdx.x,
                                           kVoxThreads, cn);
            if (!h.hit) continue;
            dist[f] = h.t;
            if (h.t <= kCubeUnit) {
                mat = h.mat;
                if (h.back || load_mat(sc, h.mat).model == GKRT_MAT_DIFFUSE_LIGHT) dist[f] = 0.0f;
            }
        }
        float md = mn(mn(mn(mn(mn(dist[0], dist[1]), dist[2]), dist[3]), dist[4]), dist[5]);
        if (md > 254.0f) {
            // DetectDistance along the diagonals (the reference's list repeats two of them)
#pragma unroll 1
            for (int q = 0; q < 6; ++q) {
                const int sx = (q == 0 || q == 3) ? 1 : -1;
                const int sy = (q == 2 || q == 5) ? -1 : 1;
                const int sz = q < 3 ? 1 : -1;
                const f3 d = F3((float)sx * kInvSqrt3, (float)sy * kInvSqrt3, (float)sz * kInvSqrt3);
                const ProbeHit h = probe_trace(sc, o, d, kCubeUnit * 64.0f, false, stack + threadIdx.x, kVoxThreads, cn);
                md = mn(md, h.hit ? h.t : 255.0f);
            }
        }
        float c[6];
#pragma unroll
        for (int f = 0; f < 6; ++f) c[f] = mn(mx(div_(dist[f], kCubeUnit), 0.0f), 1.0f);
        const float inside = ((((c[0] * c[1]) * c[2]) * c[3]) * c[4]) * c[5];
        const uint32_t w2 = ((uint32_t)div_(md, kCubeUnit) & 0xFFu) | (((uint32_t)(inside * 255.0f) & 0xFFu) << 8) |
                            (((uint32_t)(c[4] * 255.0f) & 0xFFu) << 16) | (((uint32_t)(c[5] * 255.0f) & 0xFFu) << 24);
        const uint32_t w3 = ((uint32_t)(c[2] * 255.0f) & 0xFFu) | (((uint32_t)(c[3] * 255.0f) & 0xFFu) << 8) |
                            (((uint32_t)(c[0] * 255.0f) & 0xFFu) << 16) | (((uint32_t)(c[1] * 255.0f) & 0xFFu) << 24);
        voxels[g] = make_uint4(mat, 0u, w2, w3);
    }
    flush_ray_counters(cn, counters);
}

// One bake step of probes [first, first + count): 8 lanes per probe, lane f < 6 bakes face f.
__global__ void __launch_bounds__(kBakeThreads) k_probe_bake(ShadeScene sc, GkrtFrameConstants fc, ProbeLight lt,
                                                             SkySH sh, uint32_t first, uint32_t count,
                                                             const uint32_t* cubes_prev, uint32_t* cubes,
                                                             uint4* voxels, unsigned long long* counters) {
    __shared__ uint32_t stack[kStackSize * kBakeThreads];
    Counters cn;
    cn.rays = 0; cn.fallbacks = 0; cn.retraces = 0; cn.nodes = 0; cn.tris = 0; cn.hits = 0;
    const uint32_t lane = threadIdx.x & 31u, sub = lane & 7u;
    const uint32_t k = (blockIdx.x * kBakeThreads + threadIdx.x) >> 3;
    const uint32_t g = first + k;
    const bool valid = k < count;
    uint4 vox = make_uint4(0u, 0u, 0u, 0u);
    if (valid) vox = voxels[g];
    const bool surface = valid && (vox.z & 0xFFu) < 8u;   // RenderAmbientCubeOnly bakes surface probes only
    const int f = (int)sub;
    const bool active = surface && f < 6;
    const uint32_t* prev = cubes_prev + (size_t)g * 14u;
    uint32_t s0 = 0u, s1 = 0u;
    if (surface) { s0 = __ldg(&prev[12]); s1 = __ldg(&prev[13]); }
    // per face: direct word, indirect word, sky-visibility byte (word 12 / 13, byte)
    const int dw = f == 0 ? 8 : f == 1 ? 9 : f == 2 ? 10 : f == 3 ? 11 : f == 4 ? 6 : 7;
    const int iw = dw - 6;
    const int sw = (f == 2 || f == 3) ? 13 : 12;
    const int sb = f == 0 ? 2 : f == 1 ? 3 : f == 2 ? 0 : f == 3 ? 1 : f == 4 ? 0 : 1;
    uint32_t nd = 0u, ni = 0u, nsky = 0u, nsun = (s1 >> 16) & 0xFFu;
    if (active) {
        const f3 basis = face_basis(f);
        const f3 o = fma3(basis, kCubeUnit * 0.25f, probe_origin(g));
        f4 direct = F4(0.0f, 0.0f, 0.0f, 0.0f), bounce = F4(0.0f, 0.0f, 0.0f, 0.0f);
        float skyv = 0.0f;
        const uint32_t j = vox.y % 9u;
        const float jx = c_grid3x3[2 * j] * 0.25f, jy = c_grid3x3[2 * j + 1] * 0.25f;
#pragma unroll 1
        for (int i = 0; i < 16; ++i) {
            const f3 hv = normalize3(F3(c_grid4x4[2 * i] + jx, c_grid4x4[2 * i + 1] + jy, 1.0f));
            const f3 dir = align_normal(hv, basis);
            const ProbeHit h = probe_trace(sc, o, dir, kFastMaxTrace, true, stack + threadIdx.x, kBakeThreads, cn);
            if (h.hit) {
                // the hit material's diffuse times its diffuse texture (AmbientCube.slang:504-510)
                const MatV m = load_mat(sc, h.v.mat);
                f4 alb = m.diffuse;
                if (m.dtex >= 0) alb = alb * tex_sample(sc.tex, m.dtex, h.tu, h.tv);
                bounce = bounce + (alb * probe_di(cubes_prev, sc.voxels, h.v.P, h.v.N)) * 1.25f;
            } else {
                direct = direct + (sh.on ? sky_sh(sh, fc, dir) : sky(fc));
                skyv = skyv + 1.0f;
            }
        }
        direct = direct * 0.0625f;
        bounce = bounce * 0.0625f;
        if (lt.valid) {
            // TraceSegment(origin, lightPos, 0.125): the segment [0.125, len - 0.125] as a ray
            // from origin + 0.125 dir over [EPS, len - 0.25]
            const f3 dv = lt.pos - o;
            const float len = len3(dv);
            const f3 dn = F3(div_(dv.x, len), div_(dv.y, len), div_(dv.z, len));
            ++cn.rays;
            const TraceOut s = traverse<kAny, true>(sc.S, fma3(dn, kCubeUnit * 0.5f, o), dn, kTmin,
                                                    len - kCubeUnit, stack + threadIdx.x, kBakeThreads, cn);
            const float atten = s.hit ? 0.0f : 1.0f;
            const f3 ldir = normalize3(dv);
            const float ndotl = mn(mx(dot3(basis, ldir), 0.0f), 1.0f);
            const float att = div_(ndotl * lt.area, (len * len) * 3.14159f);
            direct = direct + (lt.power * att) * atten;
        }
        if (fc.has_sun) {
            const f3 sd = F3(fc.sun_direction[0], fc.sun_direction[1], fc.sun_direction[2]);
            ++cn.rays;
            const TraceOut s = traverse<kAny, true>(sc.S, o, sd, kTmin, kOcclusionMax, stack + threadIdx.x,
                                                    kBakeThreads, cn);
            const float atten = s.hit ? 0.0f : 1.0f;
            const float ndotl = mn(mx(dot3(basis, sd), 0.0f), 1.0f);
            if (f == 0) nsun = atten > 0.0f ? 1u : 0u;
            const f4 sc4 = F4(fc.sun_color[0], fc.sun_color[1], fc.sun_color[2], fc.sun_color[3]);
            direct = direct + (((sc4 * atten) * ndotl) * 1.0f) * 0.25f;
        }
        const float ov = (float)((__ldg(&prev[sw]) >> (8 * sb)) & 0xFFu);
        nsky = (uint32_t)lerpf_(ov, div_(255.0f * skyv, 16.0f), 0.125f) & 0xFFu;
        const f4 od = unpack10(__ldg(&prev[dw])), oi = unpack10(__ldg(&prev[iw]));
        nd = pack10(F4(lerpf_(od.x, direct.x, 0.125f), lerpf_(od.y, direct.y, 0.125f), lerpf_(od.z, direct.z, 0.125f),
                       lerpf_(od.w, direct.w, 0.125f)));
        ni = pack10(F4(lerpf_(oi.x, bounce.x, 0.125f), lerpf_(oi.y, bounce.y, 0.125f), lerpf_(oi.z, bounce.z, 0.125f),
                       lerpf_(oi.w, bounce.w, 0.125f)));
        cubes[(size_t)g * 14u + dw] = nd;
        cubes[(size_t)g * 14u + iw] = ni;
    }
    // gather the six sky-visibility bytes (and the sun byte of face +Y) to lane 0 of the group
    const unsigned base = lane & ~7u;
    uint32_t by[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) by[q] = __shfl_sync(0xFFFFFFFFu, nsky, base + q);
    const uint32_t sun = __shfl_sync(0xFFFFFFFFu, nsun, base);
    if (surface && sub == 0u) {
        // word 12: +Z, -Z, +Y, -Y; word 13: +X, -X, sun, unchanged
        cubes[(size_t)g * 14u + 12] = by[4] | (by[5] << 8) | (by[0] << 16) | (by[1] << 24);
        cubes[(size_t)g * 14u + 13] = by[2] | (by[3] << 8) | ((fc.has_sun ? sun : (s1 >> 16) & 0xFFu) << 16) |
                                      (s1 & 0xFF000000u);
        voxels[g].y = vox.y + 1u;
    }
    flush_ray_counters(cn, counters);
}

}  // namespace

}  // namespace gk

using namespace gk;

cudaError_t gkrt_launch_probe_voxelize(const ShadeScene& sc, uint32_t first, uint32_t count, uint4* voxels,
                                       unsigned long long* counters, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    k_probe_voxelize<<<(count + kVoxThreads - 1) / kVoxThreads, kVoxThreads, 0, st>>>(sc, first, count, voxels,
                                                                                     counters);
    return cudaGetLastError();
}

cudaError_t gkrt_launch_probe_bake(const ShadeScene& sc, const GkrtFrameConstants& fc, const ProbeLight& lt,
                                   const SkySH& sh, uint32_t first, uint32_t count, const uint32_t* cubes_prev, uint32_t* cubes,
                                   uint4* voxels, unsigned long long* counters, cudaStream_t st) {
    if (count == 0) return cudaSuccess;
    const uint64_t threads = (uint64_t)count * 8u;
    k_probe_bake<<<(unsigned)((threads + kBakeThreads - 1) / kBakeThreads), kBakeThreads, 0, st>>>(
        sc, fc, lt, sh, first, count, cubes_prev, cubes, voxels, counters);
    return cudaGetLastError();
}
