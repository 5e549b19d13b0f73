"""Seeded synthetic scenes for the path-tracing pass.

The reference ships procedural scene templates (FProcModel::CreateCornellBox / CreateBox,
src/Assets/FProcModel.cpp:16-176; SceneList::CornellBox, src/Runtime/SceneList.cpp:180-226).
The workloads here follow those templates with the sizes and value distributions of the
benchmark configurations:

* cornell():  5 axis-aligned wall quads + 2 boxes rotated about Y (34 tris) and one
  0.25 x 0.25 emissive quad (2 tris, radiance 15); Lambertian albedo U(0.2, 0.9)^3 per
  object; 256 x 256, 40 deg FOV, pinhole, 1 spp, 4 bounces.
* bricks():   one studded-brick mesh (252 tris) instanced 4096 times on a 64 x 64 grid with
  integer heights 1..8 (1.03 M tris); GGX materials with roughness U(0.05, 1),
  metallic Bernoulli(0.3), base colour U(0, 1)^3; 64 emissive bricks, radiance U(5, 20);
  1920 x 1080, 1 spp, 8 bounces, camera orbiting 0.5 deg per frame.

Every array is produced with numpy's seeded generators, so the oracle and the GPU see the
same floats. The scene data is synthetic: the reference's .glb scenes are not used.
"""
from __future__ import annotations

import math

import numpy as np

from . import abi
from .camera import Camera, Settings


def affine_inverse(m12: np.ndarray) -> np.ndarray:
    """world->object for a row-major 3x4 object->world transform, in float64."""
    m = np.eye(4)
    m[:3, :] = np.asarray(m12, np.float64).reshape(3, 4)
    return np.linalg.inv(m)[:3, :].reshape(-1).astype(np.float32)


def trs(translate=(0, 0, 0), rot_y_deg=0.0, scale=(1, 1, 1)) -> np.ndarray:
    a = math.radians(rot_y_deg)
    c, s = math.cos(a), math.sin(a)
    r = np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])
    m = np.zeros((3, 4))
    m[:, :3] = r @ np.diag(scale)
    m[:, 3] = translate
    return m.reshape(-1)


def make_instance(mesh_id, world12, mat_ids, instance_id, prev_world12=None, visible=1):
    inst = np.zeros((), abi.INSTANCE_DTYPE)
    inst["instance_id"] = instance_id
    inst["mesh_id"] = mesh_id
    inst["visible"] = visible
    inst["world"] = np.asarray(world12, np.float32)
    inst["world_inv"] = affine_inverse(world12)
    inst["combined_prev"] = combined_prev(world12, world12 if prev_world12 is None else prev_world12)
    mids = np.zeros(16, np.uint32)
    mids[: len(mat_ids)] = mat_ids
    inst["mat_id"] = mids
    return inst


def combined_prev(world12, prev_world12) -> np.ndarray:
    """prevTransform * inverse(transform) (Node::TickVelocity, src/Assets/Node.cpp:94):
    maps a world position on the instance this frame to where it was last frame."""
    w = np.eye(4)
    w[:3, :] = np.asarray(world12, np.float64).reshape(3, 4)
    p = np.eye(4)
    p[:3, :] = np.asarray(prev_world12, np.float64).reshape(3, 4)
    return (p @ np.linalg.inv(w))[:3, :].reshape(-1).astype(np.float32)


def material(diffuse, model, fuzziness=1.0, ri=1.0, metalness=0.0, ri2=0.0):
    m = np.zeros((), abi.MATERIAL_DTYPE)
    m["diffuse"] = list(diffuse) + [1.0] if len(diffuse) == 3 else list(diffuse)
    m["diffuse_texture_id"] = -1
    m["mra_texture_id"] = -1
    m["normal_texture_id"] = -1
    m["fuzziness"] = fuzziness
    m["refraction_index"] = ri
    m["material_model"] = model
    m["metalness"] = metalness
    m["refraction_index2"] = ri2
    return m


# Material factories of src/Assets/Material.hpp:10-38.
def lambertian(rgb):
    return material(rgb, abi.MAT_LAMBERTIAN, fuzziness=1.0, ri=1.0, metalness=0.0)


def metallic(rgb, fuzz):
    return material(rgb, abi.MAT_METALLIC, fuzziness=fuzz, ri=1.45, metalness=1.0)


def mixture(rgb, fuzz):
    return material(rgb, abi.MAT_MIXTURE, fuzziness=fuzz, ri=1.45, metalness=0.0)


def diffuse_light(rgb):
    return material(rgb, abi.MAT_DIFFUSE_LIGHT, fuzziness=0.0, ri=0.0, metalness=0.0)


def dielectric(ri, fuzz=0.0):
    return material((1.0, 1.0, 1.0), abi.MAT_DIELECTRIC, fuzziness=fuzz, ri=ri, metalness=0.0, ri2=ri)


class MeshBuilder:
    def __init__(self):
        self.pos, self.nrm, self.slot, self.idx = [], [], [], []

    def quad(self, p0, p1, p2, p3, n, slot):
        """Two triangles (p0,p1,p2), (p0,p2,p3) with a flat normal, like AddTriangle."""
        b = len(self.pos)
        for p in (p0, p1, p2, p3):
            self.pos.append(list(p) + [1.0])
            self.nrm.append(list(n) + [0.0])
            self.slot.append(slot)
        self.idx += [b, b + 1, b + 2, b, b + 2, b + 3]

    def tri(self, p0, p1, p2, n0, n1, n2, slot):
        b = len(self.pos)
        for p, n in ((p0, n0), (p1, n1), (p2, n2)):
            self.pos.append(list(p) + [1.0])
            self.nrm.append(list(n) + [0.0])
            self.slot.append(slot)
        self.idx += [b, b + 1, b + 2]

    def box(self, lo, hi, slot=0, bottom=True):
        """Axis-aligned box with outward normals (FProcModel::CreateBox winding)."""
        (x0, y0, z0), (x1, y1, z1) = lo, hi
        self.quad((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0), (-1, 0, 0), slot)
        self.quad((x1, y0, z1), (x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (1, 0, 0), slot)
        self.quad((x1, y0, z0), (x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (0, 0, -1), slot)
        self.quad((x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1), (0, 0, 1), slot)
        if bottom:
            self.quad((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, -1, 0), slot)
        self.quad((x1, y1, z0), (x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (0, 1, 0), slot)

    def arrays(self):
        return (np.asarray(self.pos, np.float32), np.asarray(self.nrm, np.float32),
                np.asarray(self.slot, np.uint32), np.asarray(self.idx, np.uint32))


def _concat_meshes(builders):
    pos, nrm, slot, idx, meshes = [], [], [], [], []
    voff = ioff = 0
    for b in builders:
        p, n, s, i = b.arrays()
        meshes.append((ioff, len(i), voff, len(p)))
        pos.append(p); nrm.append(n); slot.append(s); idx.append(i)
        voff += len(p)
        ioff += len(i)
    return (np.concatenate(pos), np.concatenate(nrm), np.concatenate(slot), np.concatenate(idx),
            np.array(meshes, dtype=abi.MESH_DTYPE))


# ---------------------------------------------------------------------------------------
def cornell(seed: int = 1, width: int = 256, height: int = 256):
    """Config C1. Returns (SceneArrays, Camera, Settings)."""
    rng = np.random.default_rng(seed)
    room = MeshBuilder()
    # unit room x in [-0.5, 0.5], y in [0, 1], z in [-0.5, 0.5]; front open (CreateCornellBox, scale 1)
    l0, l1, l2, l3 = (-0.5, 0, 0.5), (-0.5, 0, -0.5), (-0.5, 1, -0.5), (-0.5, 1, 0.5)
    r0, r1, r2, r3 = (0.5, 0, 0.5), (0.5, 0, -0.5), (0.5, 1, -0.5), (0.5, 1, 0.5)
    room.quad(l0, l1, l2, l3, (1, 0, 0), 0)          # left
    room.quad(r2, r1, r0, r3, (-1, 0, 0), 1)         # right (AddTriangle 2,1,0 / 3,2,0)
    room.quad(l1, r1, r2, l2, (0, 0, 1), 2)          # back
    room.quad(l0, r0, r1, l1, (0, 1, 0), 3)          # floor
    room.quad(l2, r2, r3, l3, (0, -1, 0), 4)         # ceiling
    y = 0.999
    room.quad((-0.125, y, 0.125), (0.125, y, 0.125), (0.125, y, -0.125), (-0.125, y, -0.125), (0, -1, 0), 5)
    box = MeshBuilder()
    box.box((-0.5, 0.0, -0.5), (0.5, 1.0, 0.5), slot=0)
    pos, nrm, slot, idx, meshes = _concat_meshes([room, box])
    albedo = rng.uniform(0.2, 0.9, size=(7, 3))
    mats = [lambertian(albedo[i]) for i in range(7)] + [diffuse_light((15.0, 15.0, 15.0))]
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE)
    insts = [
        make_instance(0, trs(), [0, 1, 2, 3, 4, 7], instance_id=0),
        make_instance(1, trs((-0.17, 0.0, -0.15), rot_y_deg=18.0, scale=(0.3, 0.6, 0.3)), [5], instance_id=1),
        make_instance(1, trs((0.18, 0.0, 0.17), rot_y_deg=-17.0, scale=(0.3, 0.3, 0.3)), [6], instance_id=2),
    ]
    instances = np.array(insts, dtype=abi.INSTANCE_DTYPE)
    light = np.zeros(1, abi.LIGHT_DTYPE)
    light["p0"] = [-0.125, y, 0.125, 1]
    light["p1"] = [-0.125, y, -0.125, 1]
    light["p3"] = [0.125, y, 0.125, 1]
    light["normal_area"] = [0, -1, 0, 0.0625]
    light["light_mat_idx"] = 7
    scene = abi.SceneArrays(pos, nrm, slot, idx, meshes, materials, instances, lights=light, name="cornell")
    cam = Camera(eye=(0.0, 0.5, 1.94), center=(0.0, 0.5, 0.0), fov_deg=40.0)
    settings = Settings(samples=1, bounces=4, max_bounces=4, taa=False)
    return scene, cam, settings


def brick_mesh(studs_x=4, studs_z=2, pitch=0.5, height=0.6, stud_r=0.15, stud_h=0.17, segments=10):
    """A studded brick: a box (12 tris) plus studs_x*studs_z capped cylinders of
    3*segments tris each (4 x 2 studs, 10 segments: 252 tris)."""
    b = MeshBuilder()
    sx, sz = studs_x * pitch, studs_z * pitch
    b.box((0.0, 0.0, 0.0), (sx, height, sz), slot=0)
    for i in range(studs_x):
        for j in range(studs_z):
            cx, cz = (i + 0.5) * pitch, (j + 0.5) * pitch
            y0, y1 = height, height + stud_h
            ang = [2 * math.pi * k / segments for k in range(segments + 1)]
            for k in range(segments):
                a0, a1 = ang[k], ang[k + 1]
                p00 = (cx + stud_r * math.cos(a0), y0, cz + stud_r * math.sin(a0))
                p01 = (cx + stud_r * math.cos(a1), y0, cz + stud_r * math.sin(a1))
                p10 = (cx + stud_r * math.cos(a0), y1, cz + stud_r * math.sin(a0))
                p11 = (cx + stud_r * math.cos(a1), y1, cz + stud_r * math.sin(a1))
                n0 = (math.cos(a0), 0.0, math.sin(a0))
                n1 = (math.cos(a1), 0.0, math.sin(a1))
                b.tri(p00, p11, p01, n0, n1, n1, 0)
                b.tri(p00, p10, p11, n0, n0, n1, 0)
                b.tri((cx, y1, cz), p11, p10, (0, 1, 0), (0, 1, 0), (0, 1, 0), 0)
    return b


def bricks(seed: int = 2, width: int = 1920, height: int = 1080, grid: int = 64, emissive: int = 64):
    """Config C2. Returns (SceneArrays, Camera, Settings)."""
    rng = np.random.default_rng(seed)
    brick = brick_mesh()
    ground = MeshBuilder()
    pitch_x, pitch_z = 2.2, 1.2
    ext_x, ext_z = grid * pitch_x, grid * pitch_z
    ground.quad((-2.0, 0.0, -2.0), (-2.0, 0.0, ext_z + 2.0), (ext_x + 2.0, 0.0, ext_z + 2.0),
                (ext_x + 2.0, 0.0, -2.0), (0, 1, 0), 0)
    pos, nrm, slot, idx, meshes = _concat_meshes([brick, ground])
    n = grid * grid
    heights = rng.integers(1, 9, size=n)
    rough = rng.uniform(0.05, 1.0, size=n)
    metal = rng.random(n) < 0.3
    base = rng.uniform(0.0, 1.0, size=(n, 3))
    emit_ids = rng.choice(n, size=emissive, replace=False)
    radiance = rng.uniform(5.0, 20.0, size=emissive)
    mats = []
    for i in range(n):
        mats.append(metallic(base[i], rough[i]) if metal[i] else mixture(base[i], rough[i]))
    for k, i in enumerate(emit_ids):
        mats[i] = diffuse_light((radiance[k], radiance[k], radiance[k]))
    mats.append(lambertian((0.5, 0.5, 0.5)))
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE)
    insts = np.zeros(n + 1, abi.INSTANCE_DTYPE)
    gi, gj = np.meshgrid(np.arange(grid), np.arange(grid), indexing="ij")
    gi, gj = gi.reshape(-1), gj.reshape(-1)
    worlds = np.zeros((n, 12))
    worlds[:, 0] = 1.0
    worlds[:, 5] = heights
    worlds[:, 10] = 1.0
    worlds[:, 3] = gi * pitch_x
    worlds[:, 11] = gj * pitch_z
    invs = np.zeros((n, 12))
    invs[:, 0] = 1.0
    invs[:, 5] = 1.0 / heights
    invs[:, 10] = 1.0
    invs[:, 3] = -worlds[:, 3]
    invs[:, 11] = -worlds[:, 11]
    ident = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    insts["instance_id"][:n] = np.arange(n)
    insts["mesh_id"][:n] = 0
    insts["visible"] = 1
    insts["world"][:n] = worlds.astype(np.float32)
    insts["world_inv"][:n] = invs.astype(np.float32)
    insts["combined_prev"][:] = ident
    insts["mat_id"][:n, 0] = np.arange(n)
    insts["instance_id"][n] = n
    insts["mesh_id"][n] = 1
    insts["world"][n] = ident
    insts["world_inv"][n] = ident
    insts["mat_id"][n, 0] = n
    lights = np.zeros(0, abi.LIGHT_DTYPE)
    scene = abi.SceneArrays(pos, nrm, slot, idx, meshes, materials, insts, lights=lights, name="bricks")
    center = np.array([ext_x * 0.5, 0.0, ext_z * 0.5])
    cam = Camera(eye=center + np.array([0.0, 40.0, 90.0]), center=center + np.array([0.0, 2.0, 0.0]), fov_deg=40.0)
    # the configuration's denoiser: bilateral 5 x 5, three a-trous passes
    settings = Settings(samples=1, bounces=8, max_bounces=8, temporal_frames=16, taa=True,
                        denoiser=abi.DENOISE_ATROUS)
    return scene, cam, settings


def octa_sphere(levels: int = 4) -> MeshBuilder:
    """Unit sphere: an octahedron subdivided `levels` times (8 * 4**levels tris; 2048 at 4),
    vertex normals = positions."""
    P = [np.array(v, np.float64) for v in ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))]
    faces = [(0, 2, 4), (2, 1, 4), (1, 3, 4), (3, 0, 4), (2, 0, 5), (1, 2, 5), (3, 1, 5), (0, 3, 5)]
    tris = [(P[a], P[b], P[c]) for a, b, c in faces]
    for _ in range(levels):
        nxt = []
        for a, b, c in tris:
            ab, bc, ca = a + b, b + c, c + a
            ab, bc, ca = ab / np.linalg.norm(ab), bc / np.linalg.norm(bc), ca / np.linalg.norm(ca)
            nxt += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        tris = nxt
    m = MeshBuilder()
    for a, b, c in tris:
        m.tri(tuple(a), tuple(b), tuple(c), tuple(a), tuple(b), tuple(c), 0)
    return m


class CityMotion:
    """Per-frame instance transforms of city(): the spheres circle about fixed centres."""

    def __init__(self, instances, first_sphere, centre, radius, orbit, phase, omega):
        self.base = instances
        self.first = first_sphere
        self.centre, self.radius, self.orbit, self.phase, self.omega = centre, radius, orbit, phase, omega

    def _worlds(self, frame):
        a = self.phase + self.omega * frame
        n = self.radius.shape[0]
        w = np.zeros((n, 12))
        w[:, 0] = w[:, 5] = w[:, 10] = self.radius
        w[:, 3] = self.centre[:, 0] + self.orbit * np.cos(a)
        w[:, 7] = self.centre[:, 1]
        w[:, 11] = self.centre[:, 2] + self.orbit * np.sin(a)
        return w

    def instances(self, frame: int) -> np.ndarray:
        """Instances of `frame`; combined_prev maps this frame's positions to last frame's."""
        inst = self.base.copy()
        w = self._worlds(frame)
        pw = self._worlds(frame - 1 if frame > 0 else 0)
        s = slice(self.first, self.first + w.shape[0])
        inst["world"][s] = w.astype(np.float32)
        inv = np.zeros_like(w)
        inv[:, 0] = inv[:, 5] = inv[:, 10] = 1.0 / self.radius
        inv[:, 3] = -w[:, 3] / self.radius
        inv[:, 7] = -w[:, 7] / self.radius
        inv[:, 11] = -w[:, 11] / self.radius
        inst["world_inv"][s] = inv.astype(np.float32)
        cp = np.zeros_like(w)   # translation only: prev = x + (t_prev - t)
        cp[:, 0] = cp[:, 5] = cp[:, 10] = 1.0
        cp[:, 3] = pw[:, 3] - w[:, 3]
        cp[:, 7] = pw[:, 7] - w[:, 7]
        cp[:, 11] = pw[:, 11] - w[:, 11]
        inst["combined_prev"][s] = cp.astype(np.float32)
        return inst


def city(seed: int = 3, width: int = 3840, height: int = 2160, boxes: int = 20000, spheres: int = 5000,
         emissive_spheres: int = 5, sphere_levels: int = 4):
    """Config C3: 20k extruded boxes (a unit box mesh of 12 tris, footprints U(2, 5) m,
    heights LogNormal(3, 0.6)) on a jittered grid, 5k spheres (one 2048-tri octahedral sphere
    mesh) circling above them, of which 5 are emissive (10,240 emissive tris, sampled through
    the alias table), GGX roughness U(0.02, 1); 3840 x 2160, 1 spp, 8 bounces, no sky.
    Returns (SceneArrays, Camera, Settings, CityMotion); the spheres move every frame, so the
    instance level is rebuilt every frame."""
    rng = np.random.default_rng(seed)
    box = MeshBuilder()
    box.box((-0.5, 0.0, -0.5), (0.5, 1.0, 0.5), slot=0)
    sph = octa_sphere(sphere_levels)
    grid = int(math.ceil(math.sqrt(boxes)))
    pitch = 6.0
    ext = grid * pitch
    ground = MeshBuilder()
    ground.quad((-10.0, 0.0, -10.0), (-10.0, 0.0, ext + 10.0), (ext + 10.0, 0.0, ext + 10.0), (ext + 10.0, 0.0, -10.0),
                (0, 1, 0), 0)
    pos, nrm, slot, idx, meshes = _concat_meshes([box, sph, ground])
    npal = 256
    rough = rng.uniform(0.02, 1.0, npal)
    metal = rng.random(npal) < 0.3
    base = rng.uniform(0.05, 0.95, (npal, 3))
    mats = [metallic(base[i], rough[i]) if metal[i] else mixture(base[i], rough[i]) for i in range(npal)]
    rad = rng.uniform(20.0, 60.0, emissive_spheres)
    tint = rng.uniform(0.6, 1.0, (emissive_spheres, 3))
    for k in range(emissive_spheres):
        mats.append(diffuse_light(tuple(rad[k] * tint[k])))
    mats.append(lambertian((0.4, 0.4, 0.4)))
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE)
    ground_mat = len(mats) - 1
    n = boxes + spheres + 1
    insts = np.zeros(n, abi.INSTANCE_DTYPE)
    ident = np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], np.float32)
    insts["instance_id"] = np.arange(n)
    insts["visible"] = 1
    insts["combined_prev"][:] = ident
    # buildings
    gi, gj = np.divmod(np.arange(boxes), grid)
    cx = (gi + 0.5) * pitch + rng.uniform(-0.5, 0.5, boxes)
    cz = (gj + 0.5) * pitch + rng.uniform(-0.5, 0.5, boxes)
    sx, sz = rng.uniform(2.0, 5.0, boxes), rng.uniform(2.0, 5.0, boxes)
    hy = np.clip(rng.lognormal(3.0, 0.6, boxes), 2.0, 200.0)
    w = np.zeros((boxes, 12))
    w[:, 0], w[:, 5], w[:, 10] = sx, hy, sz
    w[:, 3], w[:, 11] = cx, cz
    inv = np.zeros((boxes, 12))
    inv[:, 0], inv[:, 5], inv[:, 10] = 1.0 / sx, 1.0 / hy, 1.0 / sz
    inv[:, 3], inv[:, 11] = -cx / sx, -cz / sz
    insts["mesh_id"][:boxes] = 0
    insts["world"][:boxes] = w.astype(np.float32)
    insts["world_inv"][:boxes] = inv.astype(np.float32)
    insts["mat_id"][:boxes, 0] = rng.integers(0, npal, boxes)
    # spheres
    s0 = boxes
    centre = np.stack([rng.uniform(0.0, ext, spheres), rng.uniform(60.0, 160.0, spheres),
                       rng.uniform(0.0, ext, spheres)], 1)
    radius = rng.uniform(1.0, 3.0, spheres)
    orbit = rng.uniform(2.0, 12.0, spheres)
    phase = rng.uniform(0.0, 2 * math.pi, spheres)
    omega = rng.uniform(0.02, 0.08, spheres) * rng.choice([-1.0, 1.0], spheres)
    insts["mesh_id"][s0:s0 + spheres] = 1
    smat = rng.integers(0, npal, spheres)
    emit_ids = rng.choice(spheres, emissive_spheres, replace=False)
    smat[emit_ids] = npal + np.arange(emissive_spheres)
    radius[emit_ids] = 6.0
    insts["mat_id"][s0:s0 + spheres, 0] = smat
    # ground
    insts["mesh_id"][n - 1] = 2
    insts["world"][n - 1] = ident
    insts["world_inv"][n - 1] = ident
    insts["mat_id"][n - 1, 0] = ground_mat
    motion = CityMotion(insts, s0, centre, radius, orbit, phase, omega)
    insts = motion.instances(0)
    motion.base = insts
    scene = abi.SceneArrays(pos, nrm, slot, idx, meshes, materials, insts, lights=np.zeros(0, abi.LIGHT_DTYPE),
                            name="city")
    c = np.array([ext * 0.5, 0.0, ext * 0.5])
    cam = Camera(eye=c + np.array([0.0, 260.0, 520.0]), center=c + np.array([0.0, 20.0, 0.0]), fov_deg=40.0)
    settings = Settings(samples=1, bounces=8, max_bounces=8, temporal_frames=16, taa=True,
                        nee_mode=abi.NEE_EMISSIVE)
    return scene, cam, settings, motion


def cornell_materials(seed: int = 4, tiles: int = 16, width: int = 512, height: int = 512, spp: int = 16):
    """Config C4: the Cornell box with its walls and both boxes tiled tiles x tiles, tile
    (i, j) using material tiles * i + j (256 materials: albedo U(0.2, 0.9)^3, roughness
    U(0.05, 1), metalness 0.25, Schlick index 1.5, drawn from `seed`), plus the 0.25 x 0.25
    light (material 256, radiance 15). Instances address 16 material slots, so each surface
    group is split into `tiles` row meshes whose slot j is the tile column.
    Returns (SceneArrays, Camera, Settings) with settings.samples = spp."""
    rng = np.random.default_rng(seed)
    nmat = tiles * tiles

    def tiled_quad(rows, p0, p1, p3, n):
        # p0 + u (p1 - p0) + v (p3 - p0); row i along v, column j along u
        p0, p1, p3 = (np.asarray(p, np.float64) for p in (p0, p1, p3))
        eu, ev = (p1 - p0) / tiles, (p3 - p0) / tiles
        for i in range(tiles):
            for j in range(tiles):
                a = p0 + eu * j + ev * i
                rows[i].quad(tuple(a), tuple(a + eu), tuple(a + eu + ev), tuple(a + ev), n, j)

    room = [MeshBuilder() for _ in range(tiles)]
    # the five walls of cornell(), each with outward-facing (into the room) normals
    tiled_quad(room, (-0.5, 0, 0.5), (-0.5, 0, -0.5), (-0.5, 1, 0.5), (1, 0, 0))      # left
    tiled_quad(room, (0.5, 0, -0.5), (0.5, 0, 0.5), (0.5, 1, -0.5), (-1, 0, 0))       # right
    tiled_quad(room, (-0.5, 0, -0.5), (0.5, 0, -0.5), (-0.5, 1, -0.5), (0, 0, 1))     # back
    tiled_quad(room, (-0.5, 0, 0.5), (0.5, 0, 0.5), (-0.5, 0, -0.5), (0, 1, 0))       # floor
    tiled_quad(room, (-0.5, 1, -0.5), (0.5, 1, -0.5), (-0.5, 1, 0.5), (0, -1, 0))     # ceiling
    box = [MeshBuilder() for _ in range(tiles)]
    x0, y0, z0, x1, y1, z1 = -0.5, 0.0, -0.5, 0.5, 1.0, 0.5
    tiled_quad(box, (x0, y0, z1), (x0, y0, z0), (x0, y1, z1), (-1, 0, 0))
    tiled_quad(box, (x1, y0, z0), (x1, y0, z1), (x1, y1, z0), (1, 0, 0))
    tiled_quad(box, (x0, y0, z0), (x1, y0, z0), (x0, y1, z0), (0, 0, -1))
    tiled_quad(box, (x1, y0, z1), (x0, y0, z1), (x1, y1, z1), (0, 0, 1))
    tiled_quad(box, (x0, y0, z0), (x0, y0, z1), (x1, y0, z0), (0, -1, 0))
    tiled_quad(box, (x0, y1, z1), (x0, y1, z0), (x1, y1, z1), (0, 1, 0))
    light = MeshBuilder()
    y = 0.999
    light.quad((-0.125, y, 0.125), (0.125, y, 0.125), (0.125, y, -0.125), (-0.125, y, -0.125), (0, -1, 0), 0)
    pos, nrm, slot, idx, meshes = _concat_meshes(room + box + [light])
    albedo = rng.uniform(0.2, 0.9, (nmat, 3))
    rough = rng.uniform(0.05, 1.0, nmat)
    mats = [material(tuple(albedo[k]), abi.MAT_LAMBERTIAN, fuzziness=float(rough[k]), ri=1.5, metalness=0.25)
            for k in range(nmat)]
    mats.append(diffuse_light((15.0, 15.0, 15.0)))
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE)
    insts = []
    row_ids = list(range(tiles))
    for i in row_ids:
        insts.append(make_instance(i, trs(), [tiles * i + j for j in range(tiles)], instance_id=0))
    for k, w in enumerate((trs((-0.17, 0.0, -0.15), rot_y_deg=18.0, scale=(0.3, 0.6, 0.3)),
                           trs((0.18, 0.0, 0.17), rot_y_deg=-17.0, scale=(0.3, 0.3, 0.3)))):
        for i in row_ids:
            insts.append(make_instance(tiles + i, w, [tiles * i + j for j in range(tiles)], instance_id=1 + k))
    insts.append(make_instance(2 * tiles, trs(), [nmat], instance_id=3))
    instances = np.array(insts, dtype=abi.INSTANCE_DTYPE)
    scene = abi.SceneArrays(pos, nrm, slot, idx, meshes, materials, instances, name="cornell-256-materials")
    cam = Camera(eye=(0.0, 0.5, 1.94), center=(0.0, 0.5, 0.0), fov_deg=40.0)
    settings = Settings(samples=spp, bounces=4, max_bounces=4, taa=False)
    return scene, cam, settings


def planar_attributes(pos: np.ndarray, nrm: np.ndarray, tiles: float = 2.0):
    """Texture coordinates and tangents for axis-aligned geometry: each vertex projects onto the
    two axes across its normal's dominant axis (u along the first, scaled by `tiles`); the
    tangent runs along u, its w the sign of the normal's dominant component (so both
    handedness cases occur)."""
    p = np.asarray(pos, np.float64)[:, :3]
    n = np.asarray(nrm, np.float64)[:, :3]
    k = np.argmax(np.abs(n), axis=1)
    a = (k + 1) % 3
    b = (k + 2) % 3
    r = np.arange(p.shape[0])
    uv = np.stack([p[r, a] * tiles, p[r, b] * tiles], axis=1).astype(np.float32)
    tan = np.zeros((p.shape[0], 4), np.float32)
    tan[r, a] = 1.0
    tan[:, 3] = np.where(n[r, k] > 0, 1.0, -1.0)
    return uv, tan


def procedural_textures(seed: int = 3, size: int = 32):
    """Test textures: an sRGB checker with coloured noise (RGBA8), a linear RGBA32F gradient, an
    MRA map (RGBA8 UNORM, green = roughness), a tangent-space normal map of round bumps (RGBA8
    UNORM) and an equirectangular HDR sky (RGBA32F, 64 x 32) with a sun above the clamp of 10."""
    rng = np.random.default_rng(seed)
    s = size
    y, x = np.mgrid[0:s, 0:s]
    chk = ((x // 4 + y // 4) % 2).astype(np.float64)
    col = np.zeros((s, s, 4), np.uint8)
    col[..., :3] = np.clip(40 + 180 * chk[..., None] + rng.integers(0, 35, (s, s, 3)), 0, 255)
    col[..., 3] = 255
    grad = np.zeros((s, s, 4), np.float32)
    grad[..., 0] = x / (s - 1)
    grad[..., 1] = y / (s - 1)
    grad[..., 2] = 0.3 + 0.4 * np.sin(x * 0.7) ** 2
    grad[..., 3] = 1.0
    mra = np.zeros((s, s, 4), np.uint8)
    mra[..., 1] = np.clip(30 + 220 * ((x * 7 + y * 3) % s) / s, 0, 255)
    mra[..., 2] = 128
    mra[..., 3] = 255
    cx, cy = (x % 8) - 3.5, (y % 8) - 3.5
    h = np.exp(-(cx * cx + cy * cy) / 6.0)
    nx, ny = -cx * h * 0.4, -cy * h * 0.4
    nz = np.sqrt(np.maximum(1.0 - nx * nx - ny * ny, 0.0))
    nmap = np.zeros((s, s, 4), np.uint8)
    nmap[..., 0] = np.round((nx * 0.5 + 0.5) * 255)
    nmap[..., 1] = np.round((ny * 0.5 + 0.5) * 255)
    nmap[..., 2] = np.round((nz * 0.5 + 0.5) * 255)
    nmap[..., 3] = 255
    sy, sx = np.mgrid[0:32, 0:64]
    sky = np.zeros((32, 64, 4), np.float32)
    sky[..., 0] = 0.3 + 0.5 * (1 - sy / 31)
    sky[..., 1] = 0.4 + 0.4 * (1 - sy / 31)
    sky[..., 2] = 0.6 + 0.3 * np.cos(sx / 63 * 2 * np.pi) ** 2
    sun = np.exp(-(((sx - 20) ** 2) + ((sy - 9) ** 2)) / 3.0)
    sky[..., :3] += 40.0 * sun[..., None]
    sky[..., 3] = 1.0
    return {"checker": (abi.TEX_RGBA8_SRGB, col), "gradient": (abi.TEX_RGBA32F, grad),
            "mra": (abi.TEX_RGBA8_UNORM, mra), "normal": (abi.TEX_RGBA8_UNORM, nmap), "sky": (abi.TEX_RGBA32F, sky)}


def cornell_textured(seed: int = 1):
    """The C1 Cornell box with textured materials and an HDR sky: left wall an sRGB checker,
    back wall a float gradient, floor a GGX mixture with an MRA map and a normal map, the tall
    box the checker and the normal map, the short box a metal with the gradient (textured
    primary albedo on metallic paths), the ceiling an id with no texture (white). Texture ids:
    checker 5, gradient 6, MRA 7, normal 8, missing 9, sky 2. The sky texture is on with a
    rotation; the camera sits farther out so that camera rays and bounces reach the sky.
    Returns (SceneArrays, Camera, Settings)."""
    sc, cam, st = cornell(seed)
    uv, tan = planar_attributes(sc.positions, sc.normals)
    t = procedural_textures(seed + 2)
    mats = sc.materials.copy()
    mats[0]["diffuse_texture_id"] = 5
    mats[2]["diffuse_texture_id"] = 6
    mats[3] = mixture((0.8, 0.75, 0.7), 0.6)
    mats[3]["mra_texture_id"] = 7
    mats[3]["normal_texture_id"] = 8
    mats[4]["diffuse_texture_id"] = 9
    mats[5]["diffuse_texture_id"] = 5
    mats[5]["normal_texture_id"] = 8
    mats[6] = metallic((0.9, 0.8, 0.6), 0.3)
    mats[6]["diffuse_texture_id"] = 6
    textures = {5: t["checker"], 6: t["gradient"], 7: t["mra"], 8: t["normal"], 2: t["sky"]}
    sc = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, mats, sc.instances,
                         lights=sc.lights, name="cornell-textured", texcoords=uv, tangents=tan, textures=textures)
    cam = Camera(eye=(0.3, 0.6, 1.6), center=(0.0, 0.45, 0.0), fov_deg=42.0)
    st.has_sky = True
    st.sky_intensity = 0.7
    st.sky_texture = 2
    st.sky_rotation = 0.3
    return sc, cam, st
