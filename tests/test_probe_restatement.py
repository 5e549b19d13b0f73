"""The oracle's probe voxelization and bake against a second, independent restatement in pure
Python (FP64, brute-force hits) on the Cornell box scaled to 4 m: the voxelization from
VoxelizeCube (src/Assets/CPUAccelerationStructure.cpp:70-160, with InsideGeometry,
DetectDistance and PackBytes), one bake step from FGpuProbeGenerator::RenderAmbientCubeOnly and
FaceTask (assets/shaders/common/AmbientCube.slang:477-553, 656-690).

Readings shared with the product: voxelization rays start at EPS (1e-3) instead of tinybvh's 0;
the face normal is cross(v1 - v0, v2 - v1) of the hit triangle (CPUAccelerationStructure.cpp:
193-196) taken to world space by the instance matrix; the bake reads the grid as it was before
the step; the sky without an environment map is the constant colour (rgb capped at 10, alpha at
1) times the intensity. Probes are drawn at random from around and inside
the room, and far above and beside it (where all six axis rays miss and the diagonals decide)."""
import math

import numpy as np

from gknextengine_gb300 import abi, camera
from oracle import oracle as O
from test_gpu_probes import big_cornell
from test_shading_restatement import (CUBE_OFFSET, CUBE_UNIT, CUBE_XY, EPS, Scene, align, cross, dot, norm,
                                      probe_term, sub, unpack_color)

AXES = ((0, 1, 0), (0, -1, 0), (1, 0, 0), (-1, 0, 0), (0, 0, 1), (0, 0, -1))      # PY NY PX NX PZ NZ
# DetectDistance's list as written (two entries appear twice)
DIAGONALS = ((1, 1, 1), (-1, 1, 1), (-1, -1, 1), (-1, 1, 1), (1, 1, -1), (-1, 1, -1), (-1, -1, -1),
             (-1, 1, -1))


def pack_bytes(a, b, c, d):
    return (a & 0xFF) | ((b & 0xFF) << 8) | ((c & 0xFF) << 16) | ((d & 0xFF) << 24)


def trace(S, o, d):
    """TraceRay: the closest hit within CUBE_UNIT * 64 of a unit direction; its distance, the
    world face normal and the material."""
    h = S.hit(o, d, tmax=CUBE_UNIT * 64.0)
    if h is None:
        return None
    (t, ii, p), _, _, idx = h
    sc = S.sc
    v = [tuple(float(c) for c in sc.positions[i][:3]) for i in idx]
    n = norm(cross(sub(v[1], v[0]), sub(v[2], v[1])))
    w = [float(x) for x in sc.instances[ii]["world"]]
    nw = tuple(w[4 * r] * n[0] + w[4 * r + 1] * n[1] + w[4 * r + 2] * n[2] for r in range(3))
    mat = int(sc.instances[ii]["mat_id"][int(sc.material_slots[idx[0]]) & 15])
    return t, nw, mat


def voxelize(S, g):
    y, rest = divmod(g, CUBE_XY * CUBE_XY)
    z, x = divmod(rest, CUBE_XY)
    o = (x * CUBE_UNIT + CUBE_OFFSET[0], y * CUBE_UNIT + CUBE_OFFSET[1], z * CUBE_UNIT + CUBE_OFFSET[2])
    mat = 0
    dist = []
    for d in AXES:                                      # InsideGeometry
        dd = 255.0
        h = trace(S, o, d)
        if h is not None:
            dd = h[0]
            if dd <= CUBE_UNIT:
                mat = h[2]
                if dot(h[1], d) > 0.0 or S.sc.materials[h[2]]["material_model"] == abi.MAT_DIFFUSE_LIGHT:
                    dd = 0.0
        dist.append(dd)
    md = min(dist)
    if md > 254.0:                                      # DetectDistance
        for d in DIAGONALS:
            h = trace(S, o, norm(d))
            md = min(md, h[0] if h is not None else 255.0)
    c = [min(max(dd / CUBE_UNIT, 0.0), 1.0) for dd in dist]
    inside = c[0] * c[1] * c[2] * c[3] * c[4] * c[5]
    b = [int(v * 255.0) for v in c]
    return (mat, 0, pack_bytes(int(md / CUBE_UNIT), int(inside * 255.0), b[4], b[5]),
            pack_bytes(b[2], b[3], b[0], b[1]))


def probe_index(x, y, z):
    return (y * CUBE_XY + z) * CUBE_XY + x


def test_voxelize_matches_the_python_restatement():
    sc, cam, st = big_cornell()
    S = Scene(sc)
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(3)
    # around and inside the 4 m room (x, z from -2 to 2 m is probes 88..104; y up to 4 m is 0..17)
    near = [probe_index(int(x), int(y), int(z)) for x, y, z in
            zip(rng.integers(84, 109, 300), rng.integers(0, 20, 300), rng.integers(84, 109, 300))]
    # far above and beside it: every axis ray misses
    far = [probe_index(int(x), int(y), int(z)) for x, y, z in
           zip(rng.integers(60, 132, 60), rng.integers(20, 40, 60), rng.integers(60, 132, 60))]
    probes = sorted(set(near + far))
    got = np.array([osc.probe_voxelize(g, 1)[0] for g in probes], np.uint64)
    ref = np.array([voxelize(S, g) for g in probes], np.uint64)
    same = (got == ref).all(axis=1)
    # The boxes' bottoms lie on the floor: from a probe inside a box the -y ray meets both at one
    # distance, the box's (a back face, distance 0) computed through its rotated frame, so which
    # comes first rests on the last bits (2 of 356 probes). Probes can also sit on wall planes.
    assert same.mean() >= 0.98, [(probes[i], got[i], ref[i]) for i in np.nonzero(~same)[0][:4]]
    inside = (ref[:, 2] >> 8) & 0xFF
    assert (inside == 0).any() and (inside == 255).any() and ((inside > 0) & (inside < 255)).any()
    assert (ref[:, 0] > 0).any()                                         # materials next to walls
    md = ref[:, 2] & 0xFF
    axis_miss = np.array([all(trace(S, o, d) is None for d in AXES) for o in
                          [(g % CUBE_XY * CUBE_UNIT + CUBE_OFFSET[0], g // (CUBE_XY * CUBE_XY) * CUBE_UNIT +
                            CUBE_OFFSET[1], g // CUBE_XY % CUBE_XY * CUBE_UNIT + CUBE_OFFSET[2]) for g in probes]])
    assert (axis_miss & (md < 252)).any()            # a diagonal found the room
    assert (axis_miss & (md == 252)).any()           # and none did (1020 & 0xFF)


# FaceTask's ray patterns (AmbientCube.slang:38-50): the 4 x 4 grid, jittered by the 3 x 3 one
GRID4 = [(-0.75 + 0.5 * (i % 4), -0.75 + 0.5 * (i // 4)) for i in range(16)]
GRID3 = [(x, y) for y in (-0.667, 0.0, 0.667) for x in (-0.667, 0.0, 0.667)]
# FaceTask calls in order: basis, direct word (_D), indirect word, sky byte (word, byte)
FACES = (((0, 1, 0), 8, 2, (12, 2)), ((0, -1, 0), 9, 3, (12, 3)), ((1, 0, 0), 10, 4, (13, 0)),
         ((-1, 0, 0), 11, 5, (13, 1)), ((0, 0, 1), 6, 0, (12, 0)), ((0, 0, -1), 7, 1, (12, 1)))


def sample_cube_di(cube, n):
    """sampleAmbientCubeHL2_DI (AmbientCube.slang:127-150): the direct (_D) faces only."""
    wx, wnx, wy, wny, wz, wnz = (max(n[0], 0.0), max(-n[0], 0.0), max(n[1], 0.0), max(-n[1], 0.0),
                                 max(n[2], 0.0), max(-n[2], 0.0))
    total = wx + wnx + wy + wny + wz + wnz
    col = [0.0] * 4
    for w, word in ((wx, 10), (wnx, 11), (wy, 8), (wny, 9), (wz, 6), (wnz, 7)):
        c = unpack_color(cube[word])
        for k in range(4):
            col[k] += w * c[k]
    k = 1.0 / total if total > 0.0 else 1.0
    return tuple(c * k for c in col)


def pack_color(c):
    """packRGB10A2 (AmbientCube.slang:59-69)."""
    q = [min(max(v / 512.0, 0.0), 1.0) for v in c]
    return int(q[0] * 1023.0) | (int(q[1] * 1023.0) << 10) | (int(q[2] * 1023.0) << 20) | (int(q[3] * 3.0) << 30)


def lerp(a, b, t):
    return a + t * (b - a)


def bake(S, fc, g, cubes, voxels):
    """One RenderAmbientCubeOnly step of probe g: its 14 new cube words and age."""
    out = [int(w) for w in cubes[g]]
    vox = [int(w) for w in voxels[g]]
    if (vox[2] & 0xFF) >= 8:                            # surface probes only
        return out, vox[1]
    iterate = vox[1]
    sc = S.sc
    y, rest = divmod(g, CUBE_XY * CUBE_XY)
    z, x = divmod(rest, CUBE_XY)
    center = (x * CUBE_UNIT + CUBE_OFFSET[0], y * CUBE_UNIT + CUBE_OFFSET[1], z * CUBE_UNIT + CUBE_OFFSET[2])
    sky = ((tuple(min(10.0, float(fc.sky_color[k])) * fc.sky_intensity for k in range(3)) +
            (min(1.0, float(fc.sky_color[3])) * fc.sky_intensity,)) if fc.has_sky else (0.0,) * 4)
    sky_bytes = {w: list(unpack_bytes(out[w])) for w in (12, 13)}
    for basis, dw, iw, (sw, sb) in FACES:
        o = tuple(c + b * CUBE_UNIT * 0.25 for c, b in zip(center, basis))
        direct, bounce, skyvis = [0.0] * 4, [0.0] * 4, 0.0
        jit = (GRID3[iterate % 9][0] * 0.25, GRID3[iterate % 9][1] * 0.25)
        for gx, gy in GRID4:
            d = align(norm((gx + jit[0], gy + jit[1], 1.0)), basis)
            h = S.hit(o, d, tmax=20.0)                  # FAST_MAX_TRACE_DISTANCE
            if h is not None:
                v = S.vertex(o, d, h)
                alb = [float(c) for c in sc.materials[v["mat"]]["diffuse"]]
                di = probe_term(cubes, voxels, v["P"], v["N"], sample_cube_di)
                for k in range(4):
                    bounce[k] += alb[k] * di[k] * 1.25
            else:
                for k in range(4):
                    direct[k] += sky[k]
                skyvis += 1.0
        direct = [c / 16.0 for c in direct]
        bounce = [c / 16.0 for c in bounce]
        if len(sc.lights):                              # light 0 at its centre
            L = sc.lights[0]
            lp = tuple(lerp(float(L["p1"][k]), float(L["p3"][k]), 0.5) for k in range(3))
            power = [float(c) for c in sc.materials[L["light_mat_idx"]]["diffuse"]]
            dv = sub(lp, o)
            ln = math.sqrt(dot(dv, dv))
            seg = tuple(c / ln for c in dv)             # TraceSegment(origin, lightPos, CUBE_UNIT * 0.5)
            lit = 0.0 if S.hit(o, seg, any_hit=True, tmin=CUBE_UNIT * 0.5, tmax=ln - CUBE_UNIT * 0.5) else 1.0
            ndotl = min(max(dot(basis, seg), 0.0), 1.0)
            att = ndotl * float(L["normal_area"][3]) / (ln * ln * 3.14159)
            for k in range(4):
                direct[k] += power[k] * att * lit
        if fc.has_sun:
            sd = tuple(float(c) for c in fc.sun_direction[:3])
            lit = 0.0 if S.hit(o, sd, any_hit=True) else 1.0
            ndotl = min(max(dot(basis, sd), 0.0), 1.0)
            if basis == (0, 1, 0):
                sky_bytes[13][2] = 1 if lit > 0.0 else 0
            for k in range(4):
                direct[k] += float(fc.sun_color[k]) * lit * ndotl * 0.25
        sky_bytes[sw][sb] = int(lerp(float(sky_bytes[sw][sb]), 255.0 * skyvis / 16.0, 0.125))
        out[dw] = pack_color([lerp(a, b, 0.125) for a, b in zip(unpack_color(out[dw]), direct)])
        out[iw] = pack_color([lerp(a, b, 0.125) for a, b in zip(unpack_color(out[iw]), bounce)])
    for w in (12, 13):
        out[w] = pack_bytes(*sky_bytes[w])
    return out, iterate + 1


def unpack_bytes(w):
    return (w & 0xFF, (w >> 8) & 0xFF, (w >> 16) & 0xFF, (w >> 24) & 0xFF)


def test_bake_matches_the_python_restatement():
    sc, cam, st = big_cornell()
    S = Scene(sc)
    osc = O.OracleScene(sc)
    layer = CUBE_XY * CUBE_XY
    # voxelize the probes around the room: y rows 0..19, z rows 80..111, every x
    voxels = np.zeros((48 * layer, 4), np.uint32)
    for yy in range(20):
        first = yy * layer + 80 * CUBE_XY
        voxels[first:first + 32 * CUBE_XY] = osc.probe_voxelize(first, 32 * CUBE_XY)
    voxels[:, 1] = np.random.default_rng(5).integers(0, 20, len(voxels))       # ages: the jitter
    rng = np.random.default_rng(6)
    cubes = rng.integers(0, 2 ** 32, (48 * layer, 14), dtype=np.uint32)
    cubes[:, :12] &= np.uint32(0x0FF3FCFF)            # grid lit up to 128 per channel
    fc = camera.FrameBuilder(64, 64, st).build(cam, 0)
    surface = np.nonzero((voxels[:, 2] & 0xFF) < 8)[0]
    zrow, ylayer = (surface // CUBE_XY) % CUBE_XY, surface // layer
    surface = surface[(zrow >= 80) & (zrow < 112) & (ylayer < 20)]              # the voxelized rows
    picks = [int(g) for g in rng.choice(surface, 40, replace=False)] + [int(np.nonzero((voxels[:, 2] & 0xFF) >= 8)[0][7])]
    n_close = n_exact = 0
    for g in picks:
        o, age = osc.probe_bake(fc, g, 1, cubes, voxels)
        r, rage = bake(S, fc, g, cubes, voxels)
        assert age[0] == rage
        got = [int(w) for w in o[0]]
        # FP32 against FP64: a packed channel may land one step apart (10-bit colours truncate,
        # the sky bytes too); a hemisphere ray that grazes an edge can change a face more.
        close = all(abs(((a >> s) & 0x3FF) - ((b >> s) & 0x3FF)) <= 1 and (a >> 30) == (b >> 30)
                    for a, b in zip(got[:12], r[:12]) for s in (0, 10, 20))
        close &= all(abs(x - y) <= 1 for a, b in zip(got[12:], r[12:])
                     for x, y in zip(unpack_bytes(a), unpack_bytes(b)))
        close &= (got[13] >> 16) & 0xFF == (r[13] >> 16) & 0xFF                # sun visibility
        n_close += close
        n_exact += got == r
    assert n_close >= 0.9 * len(picks), n_close
    assert n_exact >= 0.6 * len(picks), n_exact                        # most probes word for word
