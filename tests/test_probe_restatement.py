"""The oracle's probe voxelization against a second, independent restatement in pure Python
(FP64, brute-force hits) written from VoxelizeCube (src/Assets/CPUAccelerationStructure.cpp:
70-160, with InsideGeometry, DetectDistance and PackBytes) on the Cornell box scaled to 4 m.

Readings shared with the product: rays start at EPS (1e-3) instead of tinybvh's 0; the face
normal is cross(v1 - v0, v2 - v1) of the hit triangle (CPUAccelerationStructure.cpp:193-196)
taken to world space by the instance matrix. Probes are drawn at random from around and inside
the room, and far above and beside it (where all six axis rays miss and the diagonals decide)."""
import math

import numpy as np

from gknextengine_gb300 import abi
from oracle import oracle as O
from test_gpu_probes import big_cornell
from test_shading_restatement import CUBE_OFFSET, CUBE_UNIT, CUBE_XY, Scene, cross, dot, norm, sub

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
