"""The oracle's rt pass (the shading restatement) against a second, independent restatement in
pure Python (FP64) written from the shader text, on a small Cornell render:

* camera ray: FHardwarePrimaryRayCaster::TracePrimaryRay (Shading.slang:283-334), the unit-disk
  draw included (Const_Func.slang:262-282);
* hits: the closest (t, instance, primitive) by brute force over every instance's triangles in
  object space (Moller-Trumbore in FP64), hit vertex as FHardwareRayTracerV2::TraceRay
  (Shading.slang:784-826): interpolated normal through the inverse transpose, material through
  the instance's slot table of vertex 0;
* Render (:1084-1184) with GetRayColor (:1003-1082): Schlick reflect / metal choices, GGX VNDF
  or cosine hemisphere (Const_Func.slang:290-340), back faces, emitters, sky, the sun-cone NEE
  per bounce, the 0.5 early exit, the primary's direct sun light (:886-908); PCG4D seeds per
  pixel (Const_Func.slang:227-258);
* path ends on zero probes, or on a random ambient-cube grid through interpolateAmbientCubesV2
  with the full sampler (AmbientCube.slang:178-222, 290-382; layouts BasicTypes.slang:116-151);
  FastGather's exit after the first bounce (ExitAfterFirst, :1118-1121); four times the samples
  where a moving instance set the motion moment (Core.PathTracing.comp.slang:28);
* the primary G-buffer of PrimaryHit (:1187-1223): albedo, normal and roughness, object id,
  motion vector and moment of a moving instance under a moving camera, NDC depth; with and
  without the TAA jitter (the Halton (2, 3) table of Shading.slang:4-13, computed here).

Choices where the shader leaves room, as this build reads it: ?: evaluates one side; the sky is
the constant colour (capped at 10) times the intensity; the camera ray is traced (the
visibility-buffer raster needs a graphics API). FP32 (oracle) against FP64 (here): per-pixel
radiance within 1e-3 relative on nearly every pixel (paths through triangle edges may part;
through the glass box on about 94 %), image means within 0.5 %."""
import math

import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from oracle import oracle as O

EPS, TMAX = 1e-3, 1000.0
M_PI = 3.14159265358979323846
MASK = 0xFFFFFFFF


def pcg4d(v):
    v = [(x * 1664525 + 1013904223) & MASK for x in v]
    v[0] = (v[0] + v[1] * v[3]) & MASK; v[1] = (v[1] + v[2] * v[0]) & MASK
    v[2] = (v[2] + v[0] * v[1]) & MASK; v[3] = (v[3] + v[1] * v[2]) & MASK
    v = [x ^ (x >> 16) for x in v]
    v[0] = (v[0] + v[1] * v[3]) & MASK; v[1] = (v[1] + v[2] * v[0]) & MASK
    v[2] = (v[2] + v[0] * v[1]) & MASK; v[3] = (v[3] + v[1] * v[2]) & MASK
    return v


class Rng:
    def __init__(self, x, y, frame):
        self.v = [x, y, frame, 0]

    def f1(self):
        self.v = pcg4d(self.v)
        return (self.v[0] >> 9) / 8388608.0

    def f2(self):
        self.v = pcg4d(self.v)
        return (self.v[0] >> 9) / 8388608.0, (self.v[1] >> 9) / 8388608.0


def add(a, b): return (a[0] + b[0], a[1] + b[1], a[2] + b[2])
def sub(a, b): return (a[0] - b[0], a[1] - b[1], a[2] - b[2])
def mul(a, s): return (a[0] * s, a[1] * s, a[2] * s)
def dot(a, b): return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]
def cross(a, b): return (a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])
def norm(a):
    l = math.sqrt(dot(a, a))
    return (a[0] / l, a[1] / l, a[2] / l)
def had(a, b): return tuple(x * y for x, y in zip(a, b))


def onb(n):
    sz = -1.0 if n[2] < 0.0 else 1.0
    a = -1.0 / (sz + n[2])
    b2 = (n[0] * n[1] * a, sz + n[1] * n[1] * a, -n[1])
    b1 = (1.0 + sz * n[0] * n[0] * a, sz * b2[0], -sz * n[0])
    return b1, b2


def to_world(v, t, b, n): return add(add(mul(t, v[0]), mul(b, v[1])), mul(n, v[2]))
def align(v, n):
    t, b = onb(n)
    return to_world(v, t, b, n)


def hemi1(rng):
    u = rng.f2()
    phi = 2.0 * M_PI * u[0]
    r = math.sqrt(u[1])
    return (r * math.cos(phi), r * math.sin(phi), math.sqrt(1.0 - u[1]))


def in_cone(rng, cos_theta):
    u = rng.f2()
    phi = 2.0 * M_PI * u[0]
    c = 1.0 + u[1] * (cos_theta - 1.0)
    s = math.sqrt(1.0 - c * c)
    return (s * math.cos(phi), s * math.sin(phi), c)


def unit_disk(rng):
    ox, oy = rng.f2()
    ox, oy = ox + ox - 1.0, oy + oy - 1.0
    if ox == 0.0 and oy == 0.0:
        return (0.0, 0.0)
    if abs(ox) > abs(oy):
        th = M_PI / 4 * oy / ox
        return (ox * math.cos(th), ox * math.sin(th))
    c = math.sin(M_PI / 4 * ox / oy)
    return (oy * c, oy * math.sqrt(1.0 - c * c))


def ggx(rng, roughness, n):
    t, b = onb(n)
    wi_ = (dot(n, t), dot(n, b), dot(n, n))            # to_local(normal, ...)
    alpha = roughness * roughness
    uv = rng.f2()
    wi = norm((wi_[0] * alpha, wi_[1] * alpha, wi_[2]))
    bz = wi[2]
    if wi_[2] > 0.0:
        a = min(max(alpha, 0.0), 1.0)
        s = a * wi_[2] / (1.0 + math.sqrt(wi_[0] ** 2 + wi_[1] ** 2))
        bz *= (1.0 - a * a) / (1.0 + s * s)
    z = (1.0 - uv[1]) * (1.0 + bz) - bz
    phi = 2.0 * M_PI * uv[0]
    r = math.sqrt(min(max(1.0 - z * z, 0.0), 1.0))
    m = add(wi, (r * math.cos(phi), r * math.sin(phi), z))
    wm = norm((m[0] * alpha, m[1] * alpha, m[2]))
    return to_world(wm, t, b, n)


def reflect(d, n): return sub(d, mul(n, 2.0 * dot(n, d)))
def refract(d, n, eta):
    c = dot(d, n)
    k = 1.0 - eta * eta * (1.0 - c * c)
    if k < 0.0:
        return (0.0, 0.0, 0.0)
    return sub(mul(d, eta), mul(n, eta * c + math.sqrt(k)))


def schlick(c, ri):
    r0 = (1 - ri) / (1 + ri)
    r0 *= r0
    return r0 + (1 - r0) * (1 - c) ** 5


def mat4(m, v):
    return tuple(sum(m[4 * c + r] * v[c] for c in range(4)) for r in range(4))


class Scene:
    def __init__(self, sc):
        self.sc = sc
        self.probes = None if sc.probe_cubes is None else (sc.probe_cubes.reshape(-1, 14),
                                                           sc.probe_voxels.reshape(-1, 4))
        self.tris = []                                  # (inst, prim, v0, v1, v2, i0, i1, i2)
        for ii, inst in enumerate(sc.instances):
            if not inst["visible"]:
                continue
            m = sc.meshes[inst["mesh_id"]]
            for p in range(m["index_count"] // 3):
                idx = [int(sc.indices[m["index_offset"] + 3 * p + k]) + int(m["vertex_offset"]) for k in range(3)]
                vs = [tuple(float(c) for c in sc.positions[i][:3]) for i in idx]
                self.tris.append((ii, p, vs[0], vs[1], vs[2], idx))

    def winv(self, ii):
        return [float(x) for x in self.sc.instances[ii]["world_inv"]]

    def hit(self, o, d, any_hit=False, tmax=TMAX, tmin=EPS):
        best = None
        cache = {}
        for ii, p, v0, v1, v2, idx in self.tris:
            if ii not in cache:
                w = self.winv(ii)
                cache[ii] = (tuple(w[4 * r] * o[0] + w[4 * r + 1] * o[1] + w[4 * r + 2] * o[2] + w[4 * r + 3]
                                   for r in range(3)),
                             tuple(w[4 * r] * d[0] + w[4 * r + 1] * d[1] + w[4 * r + 2] * d[2] for r in range(3)))
            oo, dd = cache[ii]
            e1, e2 = sub(v1, v0), sub(v2, v0)
            pv = cross(dd, e2)
            det = dot(e1, pv)
            if det == 0.0:
                continue
            tv = sub(oo, v0)
            b1 = dot(tv, pv) / det
            if b1 < 0.0 or b1 > 1.0:
                continue
            qv = cross(tv, e1)
            b2 = dot(dd, qv) / det
            if b2 < 0.0 or b1 + b2 > 1.0:
                continue
            t = dot(e2, qv) / det
            if t < tmin or t > tmax:
                continue
            if any_hit:
                return True
            key = (t, ii, p)
            if best is None or key < best[0]:
                best = (key, b1, b2, idx)
        if any_hit:
            return False
        return best

    def vertex(self, o, d, h):
        (t, ii, p), b1, b2, idx = h
        sc = self.sc
        n = [tuple(float(c) for c in sc.normals[i][:3]) for i in idx]
        b0 = 1.0 - b1 - b2
        nl = add(add(mul(n[0], b0), mul(n[1], b1)), mul(n[2], b2))
        w = self.winv(ii)
        nw = norm(tuple(sum(w[4 * j + i] * nl[j] for j in range(3)) for i in range(3)))
        slot = int(sc.material_slots[idx[0]]) & 15
        mat = int(sc.instances[ii]["mat_id"][slot])
        return {"P": add(o, mul(d, t)), "N": nw, "mat": mat}


# Ambient-cube probe grid (AmbientCube.slang:12-15): 192 x 48 x 192 probes, 0.25 m apart.
CUBE_XY, CUBE_Z, CUBE_UNIT = 192, 48, 0.25
CUBE_OFFSET = (-CUBE_XY / 2 * CUBE_UNIT, -1.375 * CUBE_UNIT, -CUBE_XY / 2 * CUBE_UNIT)


def unpack_color(w):
    """unpackRGB10A2 (AmbientCube.slang:74-81): 10-bit channels scaled to MAX_ILLUMINANCE 512."""
    return ((w & 0x3FF) / 1023.0 * 512.0, ((w >> 10) & 0x3FF) / 1023.0 * 512.0,
            ((w >> 20) & 0x3FF) / 1023.0 * 512.0, 0.0)


def unpack_bytes(w):
    return (w & 0xFF, (w >> 8) & 0xFF, (w >> 16) & 0xFF, (w >> 24) & 0xFF)


def sample_cube_full(cube, n):
    """sampleAmbientCubeHL2_Full (AmbientCube.slang:178-222). cube: the 14 words of AmbientCube
    (BasicTypes.slang:116-137): PosZ NegZ PosY NegY PosX NegX, the same six _D, two sky words."""
    wx, wnx, wy, wny, wz, wnz = (max(n[0], 0.0), max(-n[0], 0.0), max(n[1], 0.0), max(-n[1], 0.0),
                                 max(n[2], 0.0), max(-n[2], 0.0))
    total = wx + wnx + wy + wny + wz + wnz
    s0, s1 = unpack_bytes(cube[12]), unpack_bytes(cube[13])
    sky = s0[0] * wz + s0[1] * wnz + s0[2] * wy + s0[3] * wny + s1[0] * wx + s1[1] * wnx
    face = {"PZ": 0, "NZ": 1, "PY": 2, "NY": 3, "PX": 4, "NX": 5}
    weights = {"PX": wx, "NX": wnx, "PY": wy, "NY": wny, "PZ": wz, "NZ": wnz}
    col = [0.0, 0.0, 0.0]
    for shift in (6, 0):                                  # the _D faces, then the plain ones
        for f, wgt in weights.items():
            c = unpack_color(cube[face[f] + shift])
            for k in range(3):
                col[k] += wgt * c[k]
    k = 1.0 / total if total > 0.0 else 1.0
    return (col[0] * k, col[1] * k, col[2] * k, sky * k / 255.0)


def probe_term(cubes, voxels, p, n, sampler=sample_cube_full):
    """interpolateAmbientCubesV2<FullAmbientCubeSampler> (AmbientCube.slang:290-382), or with
    another sampler: the eight surrounding probes, trilinear weights, probes with no space
    around them (distance byte below 0.01) or hidden behind the voxel distances skipped."""
    near = [(p[k] - CUBE_OFFSET[k]) / CUBE_UNIT for k in range(3)]
    if (min(near) < 0 or near[0] > CUBE_XY - 2 or near[1] > CUBE_Z - 2 or near[2] > CUBE_XY - 2):
        return (0.0, 0.0, 0.0, 1.0)
    base = [math.floor(c) for c in near]
    frac = [c - b for c, b in zip(near, base)]
    total, res = 0.0, [0.0] * 4
    for i in range(8):
        off = (i & 1, (i >> 1) & 1, (i >> 2) & 1)
        q = [b + o for b, o in zip(base, off)]
        idx = q[1] * CUBE_XY * CUBE_XY + q[2] * CUBE_XY + q[0]
        d0 = [b / 255.0 for b in unpack_bytes(int(voxels[idx, 2]))]     # distanceToSolid_gg_z01
        d1 = [b / 255.0 for b in unpack_bytes(int(voxels[idx, 3]))]     # distanceToSolid_x01_y01
        if d0[1] < 0.01:
            continue
        pl = [f - o for f, o in zip(frac, off)]
        dist = math.sqrt(dot(pl, pl))
        if dist > 0.0:
            dr = [c / dist for c in pl]
            hit_len = (math.sqrt(max(dr[0], 0.0)) * d1[0] + math.sqrt(max(-dr[0], 0.0)) * d1[1] +
                       math.sqrt(max(dr[1], 0.0)) * d1[2] + math.sqrt(max(-dr[1], 0.0)) * d1[3] +
                       math.sqrt(max(dr[2], 0.0)) * d0[2] + math.sqrt(max(-dr[2], 0.0)) * d0[3])
            if dist > hit_len + 0.05:
                continue
        wgt = 1.0
        for k in range(3):
            wgt *= (1.0 - frac[k]) if off[k] == 0 else frac[k]
        c = sampler([int(w) for w in cubes[idx]], n)
        for k in range(4):
            res[k] += c[k] * wgt
        total += wgt
    return tuple(r / total for r in res) if total > 0.0 else (0.0, 0.0, 0.0, 0.0)


def random_probe_grid(seed):
    """Random cubes and voxel distances over the probes around the unit Cornell room; a fifth
    of them with no space around them; zero (skipped) probes elsewhere."""
    rng = np.random.default_rng(seed)
    cubes = np.zeros((CUBE_Z, CUBE_XY, CUBE_XY, 14), np.uint32)
    voxels = np.zeros((CUBE_Z, CUBE_XY, CUBE_XY, 4), np.uint32)
    ys, xs = slice(0, 9), slice(90, 102)               # y rows, then z and x columns
    cubes[ys, xs, xs] = rng.integers(0, 2 ** 32, cubes[ys, xs, xs].shape, dtype=np.uint32)
    cubes[ys, xs, xs, :12] &= np.uint32(0x07F1FC7F)    # colours up to 64 per channel
    vox = rng.integers(0, 2 ** 32, voxels[ys, xs, xs].shape, dtype=np.uint32)
    empty = rng.random(vox.shape[:-1]) < 0.2
    vox[..., 2] = np.where(empty, vox[..., 2] & np.uint32(0xFFFF00FF), vox[..., 2] | np.uint32(0x00000800))
    voxels[ys, xs, xs] = vox
    return cubes.reshape(-1, 14), voxels.reshape(-1, 4)


def render_pixel(S, fc, W, H, x, y):
    sc = S.sc
    rng = Rng(x, y, fc.total_frames)
    uvx, uvy = x / W * 2.0 - 1.0, y / H * 2.0 - 1.0
    assert not fc.taa
    disk = unit_disk(rng)
    ha = fc.aperture / 2.0
    off = (ha * disk[0], ha * disk[1])
    mvi, pinv = list(fc.model_view_inverse), list(fc.projection_inverse)
    origin = mat4(mvi, (off[0], off[1], 0.0, 1.0))[:3]
    target = mat4(pinv, (uvx, uvy, 1.0, 1.0))
    tn = norm((target[0] * fc.focus_distance - off[0], target[1] * fc.focus_distance - off[1],
               target[2] * fc.focus_distance))
    direction = mat4(mvi, (tn[0], tn[1], tn[2], 0.0))[:3]
    prim_dir = norm(direction)
    sky = (tuple(min(10.0, fc.sky_color[k]) * fc.sky_intensity for k in range(4)) if fc.has_sky
           else (0.0, 0.0, 0.0, 0.0))
    h = S.hit(origin, direction)
    if h is None:
        return sky[:3], (0.0, 0.0, 0.0)
    pv = S.vertex(origin, direction, h)
    cp = [float(c) for c in sc.instances[h[0][1]]["combined_prev"]]
    prev_p = tuple(cp[4 * r] * pv["P"][0] + cp[4 * r + 1] * pv["P"][1] + cp[4 * r + 2] * pv["P"][2] + cp[4 * r + 3]
                   for r in range(3))
    moment = fc.temporal_frames if math.dist(pv["P"], prev_p) > 0.02 else 0      # zeroed moments before
    mat = sc.materials[pv["mat"]]
    if mat["material_model"] != abi.MAT_DIELECTRIC:
        pv["P"] = sub(pv["P"], mul(prim_dir, 0.03))
    if mat["material_model"] == abi.MAT_DIFFUSE_LIGHT:
        return tuple(float(c) for c in mat["diffuse"][:3]), (0.0, 0.0, 0.0)
    primary_albedo = tuple(float(c) for c in mat["diffuse"][:4])
    sun_color = tuple(float(c) for c in fc.sun_color)
    sun_dir = tuple(float(c) for c in fc.sun_direction[:3])
    cone = math.cos(0.25 / 180.0 * M_PI)

    def get_ray_color(v, d, color):
        m = sc.materials[v["mat"]]
        diel = m["material_model"] == abi.MAT_DIELECTRIC
        dv = dot(d, v["N"])
        back = dv > 0
        outward = mul(v["N"], -1.0) if back else v["N"]
        ri2 = float(m["refraction_index2"])
        eta = ri2 if back else (1.0 / ri2 if ri2 != 0.0 else math.inf)   # FP32: 1 / 0 = inf, unused
        cosine = float(m["refraction_index"]) * dv if dv > 0 else -dv
        c_refl = rng.f1() < schlick(cosine, float(m["refraction_index"]))
        c_metal = rng.f1() < float(m["metalness"])
        c_ggx = c_refl or c_metal
        nxt = reflect(d, outward) if c_ggx else outward
        tdir = ggx(rng, math.sqrt(float(m["fuzziness"])), nxt) if c_ggx else align(hemi1(rng), nxt)
        if diel and not c_refl:
            tdir = refract(d, outward, eta)
        org = add(v["P"], mul(v["N"], 0.001 * (0.0 if diel else 1.0)))
        hh = S.hit(org, tdir)
        if hh is not None:
            nv = S.vertex(org, tdir, hh)
            hm = sc.materials[nv["mat"]]
            if hm["material_model"] == abi.MAT_DIFFUSE_LIGHT or not c_refl:
                color = had(color, tuple(float(c) for c in hm["diffuse"][:4]))
            if back and not diel:
                return True, nv, tdir, (0.5, 0.5, 0.5, 0.0), c_ggx, c_metal
            if hm["material_model"] == abi.MAT_DIFFUSE_LIGHT:
                return True, nv, tdir, color, c_ggx, c_metal
            return False, nv, tdir, color, c_ggx, c_metal
        return True, v, tdir, had(color, sky), c_ggx, c_metal

    final_c, final_r = [0.0] * 4, [0.0] * 4
    eye = mat4(mvi, (0.0, 0.0, 0.0, 1.0))[:3]
    diel0 = mat["material_model"] == abi.MAT_DIELECTRIC
    max_b = fc.max_number_of_bounces if diel0 else fc.number_of_bounces
    samples = max(1, fc.number_of_samples) * (4 if moment > 0 else 1)   # Core.PathTracing.comp.slang:28
    for _ in range(samples):
        color = (1.0, 1.0, 1.0, 1.0)
        d = norm(sub(pv["P"], eye))
        done, v, d, color, hit_reflect, hit_metal = get_ray_color(pv, d, color)
        if not done and fc.fast_gather and not diel0:   # ExitAfterFirst: the probes end the path
            color = had(color, probe_term(*S.probes, v["P"], v["N"]) if S.probes else (0.0,) * 4)
        elif not done:
            for b in range(1, max_b):
                stop, v, d, color, _, _ = get_ray_color(v, d, color)
                if stop:
                    break
                if fc.has_sun and rng.f1() < 0.5:
                    lc = align(in_cone(rng, cone), sun_dir)
                    if not S.hit(v["P"], lc, any_hit=True):
                        color = had(color, sun_color)
                        break
                early = b > 0 and not diel0 and rng.f1() < 0.5
                if b == max_b - 1 or early:
                    if S.probes is None:
                        color = (0.0, 0.0, 0.0, 0.0)      # zero ambient probes
                    else:
                        color = had(color, probe_term(*S.probes, v["P"], v["N"]))
                    break
        if hit_metal:
            color = had(color, primary_albedo)
        acc = final_r if hit_reflect else final_c
        for k in range(4):
            acc[k] += color[k]
    final_c = [c / samples for c in final_c]
    final_r = [c / samples for c in final_r]
    dcos = max(dot(sun_dir, pv["N"]), 0.0) * (1.0 / M_PI)
    shadow = 0.0
    if fc.has_sun:
        lc = align(in_cone(rng, cone), sun_dir)
        shadow = 0.0 if S.hit(pv["P"], lc, any_hit=True) else 1.0
    for k in range(3):
        final_c[k] += sun_color[k] * dcos * shadow
    return tuple(final_c[:3]), tuple(final_r[:3])


@pytest.mark.parametrize("sky_sun,materials,probes,variant", [
    (False, False, False, ""), (True, False, False, ""), (True, True, False, ""), (False, False, True, ""),
    (False, False, True, "fast_gather"), (True, False, False, "moving")])
def test_rt_pass_matches_the_python_restatement(sky_sun, materials, probes, variant):
    sc, cam, st = scenes.cornell()
    st.taa = False
    st.samples = 16           # most pixels then carry light from some path (zero probes end the rest)
    st.fast_gather = variant == "fast_gather"
    if variant == "moving":   # the tall box moved: its pixels' motion moments call for 4x the samples
        cp = sc.instances["combined_prev"][2].reshape(3, 4).astype(np.float64)
        cp[0, 3] += 0.1
        sc.instances["combined_prev"][2] = cp.reshape(-1).astype(np.float32)
    if materials:             # the boxes as a rough metal and a glass: GGX VNDF, metal tint, refraction
        sc.materials[5]["metalness"] = 1.0
        sc.materials[5]["fuzziness"] = 0.2
        sc.materials[6]["material_model"] = abi.MAT_DIELECTRIC
        sc.materials[6]["refraction_index"] = 1.5
        sc.materials[6]["refraction_index2"] = 1.5
        sc.materials[6]["fuzziness"] = 0.0
    if sky_sun:
        st.has_sky, st.sky_color, st.sky_intensity = True, (0.6, 0.7, 0.9, 1.0), 1.5
        st.has_sun, st.sun_direction, st.sun_intensity = True, (0.3, 0.6, 1.0), 3.0
    if probes:                # path ends read a random ambient-cube grid instead of zero probes
        sc.probe_cubes, sc.probe_voxels = (a.reshape(-1) for a in random_probe_grid(7))
    W = H = 24
    fc = camera.FrameBuilder(W, H, st).build(cam, 5)
    im = O.new_images(W, H)
    O.OracleScene(sc).trace_pass(fc, W, H, im)
    S = Scene(sc)
    got_d = im[abi.IMG_SINGLE_DIFFUSE][..., :3].astype(np.float64)
    got_s = im[abi.IMG_SINGLE_SPECULAR][..., :3].astype(np.float64)
    ref_d = np.zeros_like(got_d)
    ref_s = np.zeros_like(got_s)
    for y in range(H):
        for x in range(W):
            ref_d[y, x], ref_s[y, x] = render_pixel(S, fc, W, H, x, y)
    close = (np.isclose(got_d, ref_d, rtol=1e-3, atol=1e-4).all(axis=-1) &
             np.isclose(got_s, ref_s, rtol=1e-3, atol=1e-4).all(axis=-1))
    # Refraction and internal reflection in the glass box carry FP32-vs-FP64 differences to the
    # box's edges, where a path's next hit can change (neighbouring pixels then trade values):
    # per pixel a lower bar there, and the image means, which such trades leave unchanged.
    assert close.mean() >= (0.90 if materials else 0.98), (close.mean(), np.argwhere(~close)[:5])
    if sky_sun:   # dense, smooth images (every pixel sees sky or sun); the C1 image is sparse and
        # random probe colours make single pixels weigh too much in the mean
        np.testing.assert_allclose(got_d.mean(), ref_d.mean(), rtol=5e-3)
        np.testing.assert_allclose(got_s.mean(), ref_s.mean(), rtol=5e-3, atol=1e-6)
    lit = ref_d.sum(axis=-1) > 0
    assert lit.mean() > (0.8 if probes else 0.15)                      # pixels that carry light
    assert close[lit].mean() >= (0.90 if materials else 0.97)          # and those agree too
    if sky_sun:
        assert (ref_d.max(axis=-1) > 0.0).mean() > 0.5


def radical_inverse(i, base):
    f, r = 1.0, 0.0
    while i:
        f /= base
        r += f * (i % base)
        i //= base
    return r


# The TAA jitter table (Shading.slang:4-13): Halton (2, 3) points 1..8, base 3 to four decimals.
HALTON = [(radical_inverse(i, 2), round(radical_inverse(i, 3), 4)) for i in range(1, 9)]


def primary_gbuffer(S, fc, W, H, x, y):
    """PrimaryHit (Shading.slang:1187-1223): albedo, normal and roughness (FetchGBufferV2,
    Shading.slang:82-112, untextured), object id, motion vector in pixels and its moment
    (CalculateMotionVectorV2, Shading.slang:50-72, on zeroed moments), NDC depth; the miss
    defaults otherwise."""
    sc = S.sc
    rng = Rng(x, y, fc.total_frames)
    uvx, uvy = x / W * 2.0 - 1.0, y / H * 2.0 - 1.0
    if fc.taa:
        hx, hy = HALTON[fc.total_frames % 8]
        uvx, uvy = uvx + (hx - 0.5) / W, uvy + (hy - 0.5) / H
    disk = unit_disk(rng)
    ha = fc.aperture / 2.0
    mvi, pinv = list(fc.model_view_inverse), list(fc.projection_inverse)
    origin = mat4(mvi, (ha * disk[0], ha * disk[1], 0.0, 1.0))[:3]
    target = mat4(pinv, (uvx, uvy, 1.0, 1.0))
    tn = norm((target[0] * fc.focus_distance - ha * disk[0], target[1] * fc.focus_distance - ha * disk[1],
               target[2] * fc.focus_distance))
    direction = mat4(mvi, (tn[0], tn[1], tn[2], 0.0))[:3]
    h = S.hit(origin, direction)
    if h is None:
        return {"albedo": (1.0, 1.0, 1.0, 1.0), "normal": (0.0, 1.0, 0.0, 1.0), "id": 65535,
                "motion": (0.0, 0.0), "depth": 100000.0, "moment": 0, "prim": 0xFFFFFFFF}
    pv = S.vertex(origin, direction, h)
    P = pv["P"]
    m = sc.materials[pv["mat"]]
    inst = sc.instances[h[0][1]]
    clip = mat4(list(fc.view_projection), (*P, 1.0))
    cur = mat4(list(fc.view_projection_unjit), (*P, 1.0))
    cp = [float(c) for c in inst["combined_prev"]]
    prevP = tuple(cp[4 * r] * P[0] + cp[4 * r + 1] * P[1] + cp[4 * r + 2] * P[2] + cp[4 * r + 3]
                  for r in range(3))
    prv = mat4(list(fc.prev_view_projection_unjit), (*prevP, 1.0))
    motion = ((prv[0] / prv[3] - cur[0] / cur[3]) * 0.5 * W, (prv[1] / prv[3] - cur[1] / cur[3]) * 0.5 * H)
    moment = fc.temporal_frames if math.dist(P, prevP) > 0.02 else 0
    return {"albedo": tuple(float(c) for c in m["diffuse"][:4]), "normal": (*pv["N"], float(m["fuzziness"])),
            "id": int(inst["instance_id"]), "motion": motion, "depth": clip[2] / clip[3], "moment": moment,
            "prim": h[0][2]}


@pytest.mark.parametrize("taa", [False, True])
def test_primary_gbuffer_matches_the_python_restatement(taa):
    sc, cam, st = scenes.cornell()
    st.taa = taa              # Halton jitter of the primary ray, frame 5 (and frame 4 before it)
    # the tall box moved 0.1 along x since last frame (its motion vectors and moments), the
    # camera orbited a little (everyone's motion vectors)
    cp = sc.instances["combined_prev"][2].reshape(3, 4).astype(np.float64)
    cp[0, 3] += 0.1
    sc.instances["combined_prev"][2] = cp.reshape(-1).astype(np.float32)
    W = H = 32
    fb = camera.FrameBuilder(W, H, st)
    fb.build(cam.orbit(0.02), 4)
    fc = fb.build(cam, 5)
    im = O.new_images(W, H)
    O.OracleScene(sc).trace_pass(fc, W, H, im)
    S = Scene(sc)
    ref = [[primary_gbuffer(S, fc, W, H, x, y) for x in range(W)] for y in range(H)]
    rid = np.array([[p["id"] for p in row] for row in ref], np.uint32)
    rprim = np.array([[p["prim"] for p in row] for row in ref], np.uint32)
    same = (im[abi.IMG_OBJECT_ID] == rid) & (im[abi.IMG_HIT_PRIM] == rprim)
    # which triangle a pixel sees may part only on an edge (the exact FP64 watertight test
    # against FP64 Moller-Trumbore); everything else is compared where both see the same one
    assert same.mean() >= 0.99, np.argwhere(~same)[:5]
    assert {0, 1, 2, 65535} <= set(np.unique(rid).tolist())
    def field(k):
        return np.array([[p[k] for p in row] for row in ref], np.float64)
    np.testing.assert_array_equal(im[abi.IMG_ALBEDO][same], field("albedo")[same].astype(np.float32))
    np.testing.assert_allclose(im[abi.IMG_NORMAL][same], field("normal")[same], atol=2e-6)
    np.testing.assert_allclose(im[abi.IMG_PREV_DEPTH][same], field("depth")[same], rtol=1e-6, atol=1e-6)
    mv = field("motion")
    np.testing.assert_allclose(im[abi.IMG_MOTION][same], mv[same], atol=1e-4)   # pixels
    moved = same & (rid == 2)
    assert moved.any() and np.all(np.abs(mv[moved][:, 0]) > 0.5)      # the box moved on screen
    np.testing.assert_array_equal(im[abi.IMG_MOTION_MOMENT][same], field("moment")[same].astype(np.uint32))
    assert np.all(im[abi.IMG_MOTION_MOMENT][moved] == fc.temporal_frames)
