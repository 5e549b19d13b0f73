"""GPU BVH builder (binned SAH on the device) against the host builder and the oracle.

Closest hits are defined independently of the tree (minimum of (t, instance, primitive)
under the FP64 watertight test), so every tree must give bit-identical hits. Tree quality is
checked through the node visits of the same rays on the GPU-built and host-built trees.
"""
import numpy as np
import pytest

from gknextengine_gb300 import abi, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_parity import assert_hits_equal, gpu_trace_rays, random_rays

pytestmark = pytest.mark.gpu

# mesh sizes covering: empty mesh, single-triangle root (wrapped leaf), roots finished by the
# small-range kernel (<= 32), the first big root (33), multi-chunk roots (> 1024 triangles)
SOUP_SIZES = (0, 1, 2, 5, 32, 33, 700, 5000, 60000)


def soup(seed=7, sizes=SOUP_SIZES, dup=64):
    """Meshes of random small triangles, one instance each (plus an invisible one), and one
    mesh of `dup` identical triangles (all centroids equal: the median-split path)."""
    rng = np.random.default_rng(seed)
    pos, nrm, slot, idx, meshes = [], [], [], [], []
    voff = ioff = 0
    for n in list(sizes) + [dup]:
        if n == dup and len(meshes) == len(sizes):
            c = np.repeat(rng.uniform(-1, 1, (1, 3)), n, axis=0)
            e = np.repeat(rng.normal(scale=0.05, size=(1, 2, 3)), n, axis=0)
        else:
            c = rng.uniform(-1, 1, (n, 3))
            e = rng.normal(scale=0.03 + 2.0 / max(n, 1) ** 0.5, size=(n, 2, 3))
        p = np.zeros((3 * n, 4), np.float32)
        p[0::3, :3] = c
        p[1::3, :3] = c + e[:, 0]
        p[2::3, :3] = c + e[:, 1]
        p[:, 3] = 1.0
        q = np.zeros_like(p)
        q[:, 1] = 1.0
        pos.append(p)
        nrm.append(q)
        slot.append(np.zeros(3 * n, np.uint32))
        idx.append(np.arange(3 * n, dtype=np.uint32))
        meshes.append((ioff, 3 * n, voff, 3 * n))
        voff += 3 * n
        ioff += 3 * n
    meshes = np.array(meshes, dtype=abi.MESH_DTYPE)
    mats = np.array([scenes.lambertian((0.5, 0.5, 0.5))], dtype=abi.MATERIAL_DTYPE)
    insts = []
    for m in range(len(meshes)):
        w = scenes.trs((rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-3, 3)),
                       rot_y_deg=float(rng.uniform(0, 360)), scale=tuple(rng.uniform(0.5, 2.0, 3)))
        insts.append(scenes.make_instance(m, w, [0], instance_id=m))
    insts.append(scenes.make_instance(len(meshes) - 2, scenes.trs((0.1, 0.2, 0.3)), [0], instance_id=99,
                                      visible=0))
    inst = np.array(insts, dtype=abi.INSTANCE_DTYPE)
    return abi.SceneArrays(np.concatenate(pos), np.concatenate(nrm), np.concatenate(slot), np.concatenate(idx),
                           meshes, mats, inst, name="soup")


@pytest.fixture(scope="module")
def soup_env():
    sc = soup()
    r = PathTracingRenderer(0)
    r.load_scene(sc)   # GPU builder (default)
    yield sc, r, O.OracleScene(sc)
    r.close()


def test_gpu_built_soup_exact(soup_env):
    sc, r, osc = soup_env
    rng = np.random.default_rng(11)
    rays = random_rays(rng, 60000, (-5, -5, -5), (5, 5, 5))
    g = gpu_trace_rays(r, rays)
    o = osc.trace_rays(rays)
    assert (o["inst"] != 0xFFFFFFFF).mean() > 0.2
    assert_hits_equal(g, o)
    s = r.stats()
    assert s.device_error == 0 and s.bvh_nodes > 0 and s.tlas_nodes > 0


def test_gpu_and_host_builds_agree(soup_env):
    sc, r, osc = soup_env
    rng = np.random.default_rng(12)
    rays = random_rays(rng, 60000, (-5, -5, -5), (5, 5, 5))
    g = gpu_trace_rays(r, rays)
    sg = r.stats()
    r.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
    try:
        h = gpu_trace_rays(r, rays)
        sh = r.stats()
    finally:
        r.build_bvh(abi.BUILD_ALL)
    assert_hits_equal(g, h)
    # same split rule: trees of comparable quality
    ratio = sg.node_visits / sh.node_visits
    assert 0.85 < ratio < 1.15, ratio
    assert abs(sg.bvh_nodes - sh.bvh_nodes) <= 0.1 * sh.bvh_nodes, (sg.bvh_nodes, sh.bvh_nodes)


def test_bricks_gpu_build_exact():
    sc, cam, st = scenes.bricks(width=64, height=36)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        osc = O.OracleScene(sc)
        rng = np.random.default_rng(13)
        rays = random_rays(rng, 40000, (-2.0, 0.2, -2.0), (140.0, 8.0, 76.0))
        g = gpu_trace_rays(r, rays)
        sg = r.stats()
        assert_hits_equal(g, osc.trace_rays(rays))
        r.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
        gpu_trace_rays(r, rays)
        sh = r.stats()
        ratio = sg.node_visits / sh.node_visits
        assert 0.85 < ratio < 1.15, ratio


def test_instance_rebuild_per_frame(soup_env):
    """gkrt_scene_update_instances rebuilds the instance level on the GPU every call."""
    sc, r, _ = soup_env
    rng = np.random.default_rng(14)
    inst = sc.instances.copy()
    try:
        for frame in range(4):
            for i in range(len(inst)):
                w = scenes.trs((rng.uniform(-3, 3), rng.uniform(-3, 3), rng.uniform(-3, 3)),
                               rot_y_deg=float(rng.uniform(0, 360)), scale=tuple(rng.uniform(0.5, 2.0, 3)))
                inst[i]["world"] = w
                inst[i]["world_inv"] = scenes.affine_inverse(w)
            inst["visible"] = 1
            inst["visible"][frame % len(inst)] = 0
            r.update_instances(inst)
            sc2 = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes,
                                  sc.materials, inst, name="soup-moved")
            rays = random_rays(rng, 20000, (-5, -5, -5), (5, 5, 5))
            assert_hits_equal(gpu_trace_rays(r, rays), O.OracleScene(sc2).trace_rays(rays))
    finally:
        r.update_instances(sc.instances)


@pytest.mark.parametrize("host", [False, True])
def test_rays_along_box_faces(host):
    """Rays with direction components of exactly zero that run along tile boundaries, i.e.
    exactly on the faces of the boxes around the tiles: hits on the shared edges must match
    the FP64 definition (the stored node boxes are widened so no such box is culled)."""
    sc, cam, st = scenes.cornell_materials(spp=1)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        if host:
            r.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
        osc = O.OracleScene(sc)
        rng = np.random.default_rng(15)
        n = 30000
        edges = (np.arange(17) / 16.0 - 0.5).astype(np.float32)
        rays = np.zeros(n, abi.RAY_DTYPE)
        rays["origin"][:, 0] = rng.choice(edges, n)
        rays["origin"][:, 1] = rng.choice((edges + 0.5).astype(np.float32), n)
        rays["origin"][:, 2] = rng.uniform(-0.45, 0.45, n).astype(np.float32)
        d = rng.normal(size=(n, 3))
        axis = rng.integers(0, 3, n)
        d[np.arange(n), axis] = 0.0          # one component exactly zero
        d[: n // 3, 1] = 0.0                 # and a third of the rays with two
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rays["dir"] = d
        rays["tmin"] = 1e-3
        rays["tmax"] = 1000.0
        assert_hits_equal(gpu_trace_rays(r, rays), osc.trace_rays(rays))


def instance_field(n, seed=21):
    """n instances of one 12-triangle box, scattered with random rotations and scales (about
    1 % overlap); a third of them share one position (all centroids equal within that group)."""
    rng = np.random.default_rng(seed)
    b = scenes.MeshBuilder()
    b.box((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), slot=0)
    pos, nrm, slot, idx, meshes = scenes._concat_meshes([b])
    mats = np.array([scenes.lambertian((0.5, 0.5, 0.5))], dtype=abi.MATERIAL_DTYPE)
    side = 2.0 * n ** (1.0 / 3.0)
    p = rng.uniform(-side, side, (n, 3))
    p[: n // 3] = p[0]
    insts = np.zeros(n, abi.INSTANCE_DTYPE)
    for i in range(n):
        insts[i] = scenes.make_instance(0, scenes.trs(tuple(p[i]), rot_y_deg=float(rng.uniform(0, 360)),
                                                      scale=tuple(rng.uniform(0.2, 1.0, 3))), [0], instance_id=i)
    return abi.SceneArrays(pos, nrm, slot, idx, meshes, mats, insts, name="instance-field"), side


@pytest.mark.parametrize("n", [1, 2, 33, 2049, 30000, 70000])
def test_instance_level_sizes(n):
    """The instance level built on the GPU for instance counts that take each path of the
    builder: one instance (a wrapped leaf), a root finished by the small-range kernel, a first
    big round, several rounds, and tens of thousands of instances (a third of them with equal
    centroids: the median split). Ray-query hits equal the oracle's; a rebuild after moving
    every instance equals the oracle again."""
    sc, side = instance_field(n)
    rng = np.random.default_rng(n)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        st = r.stats()
        assert st.device_error == 0
        rays = random_rays(rng, 20000, (-side, -side, -side), (side, side, side))
        assert_hits_equal(gpu_trace_rays(r, rays), O.OracleScene(sc).trace_rays(rays))
        inst = sc.instances.copy()
        w = inst["world"].reshape(-1, 3, 4).copy()
        w[:, :, 3] += rng.normal(0.0, 0.5, (n, 3))
        inst["world"] = w.reshape(-1, 12)
        inst["world_inv"] = np.stack([scenes.affine_inverse(x) for x in inst["world"]])
        r.update_instances(inst)
        sc2 = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials,
                              inst, name="instance-field-moved")
        assert_hits_equal(gpu_trace_rays(r, rays), O.OracleScene(sc2).trace_rays(rays))
        assert r.stats().tlas_nodes == max(n - 1, 1)   # one instance per leaf
