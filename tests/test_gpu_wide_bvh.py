"""Compressed 8-wide nodes: the collapse of the two-child SAH trees and their 8-bit child
boxes, checked through exact hits against the oracle where quantization is hardest
(geometry far from the origin, tiny geometry, both at once) and through the tree shape.

The decoded child planes must contain the stored boxes exactly (a plane that rounds inward
by one ulp would cull the FP64 winner on grazing rays), so these rays start on and run
along the faces of the triangles' own boxes as well as at random."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_bvh import soup
from test_gpu_parity import assert_hits_equal, gpu_trace_rays

pytestmark = pytest.mark.gpu


def placed(sc, offset, scale):
    """The soup with every instance moved by `offset` and scaled by `scale` (world space)."""
    inst = sc.instances.copy()
    for i in range(len(inst)):
        w = np.asarray(inst[i]["world"], np.float64).reshape(3, 4).copy()
        w[:, :3] *= scale
        w[:, 3] = w[:, 3] * scale + np.asarray(offset)
        inst[i]["world"] = w.astype(np.float32).reshape(inst[i]["world"].shape)
        inst[i]["world_inv"] = scenes.affine_inverse(inst[i]["world"])
    return abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials, inst,
                           name="soup-placed")


def face_rays(rng, sc, n, offset, scale):
    """Rays starting on planes through triangle vertices (world space), one or two direction
    components exactly zero, so they run along box faces of the leaves and of the nodes."""
    inst = sc.instances[sc.instances["visible"] == 1]
    pick = rng.integers(0, len(inst), n)
    v = sc.positions[rng.integers(0, len(sc.positions), n), :3].astype(np.float64)
    org = np.zeros((n, 3))
    for k in range(n):
        w = np.asarray(inst[pick[k]]["world"], np.float64).reshape(3, 4)
        org[k] = w[:, :3] @ v[k] + w[:, 3]
    d = rng.normal(size=(n, 3))
    axis = rng.integers(0, 3, n)
    d[np.arange(n), axis] = 0.0
    d[np.arange(n // 4), (axis[: n // 4] + 1) % 3] = 0.0     # a quarter run along an axis
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # start behind the vertex along the ray, beyond the fixed tmin (EPS = 1e-3) of ray queries
    back = rng.uniform(2.0, 8.0, n)[:, None] * max(scale, 1e-3)
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = (org - back * d).astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1e3
    return rays


def aimed_rays(rng, n, offset, scale):
    """Rays from 2..10 units (at least 2e-3) away, aimed at random points of the soup's region."""
    tgt = np.asarray(offset) + rng.uniform(-4.0, 4.0, (n, 3)) * scale
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dist = rng.uniform(2.0, 10.0, n)[:, None] * max(scale, 1e-3)
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = (tgt - dist * d).astype(np.float32)
    rays["dir"] = d.astype(np.float32)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1e3
    return rays


@pytest.mark.parametrize("offset,scale", [((0.0, 0.0, 0.0), 1.0), ((1.5e5, -7.0e4, 3.3e4), 1.0),
                                          ((0.0, 0.0, 0.0), 1e-4), ((2.0e3, 1.0e3, -4.0e3), 0.05)])
@pytest.mark.parametrize("host", [False, True])
def test_wide_nodes_exact_far_and_tiny(offset, scale, host):
    sc = placed(soup(seed=21, sizes=(1, 5, 33, 700, 5000)), offset, scale)
    osc = O.OracleScene(sc)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        if host:
            r.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
        rng = np.random.default_rng(22)
        rays = aimed_rays(rng, 20000, offset, scale)
        g = gpu_trace_rays(r, rays)
        o = osc.trace_rays(rays)
        assert (o["inst"] != 0xFFFFFFFF).mean() > 0.1
        assert_hits_equal(g, o)
        fr = face_rays(rng, sc, 20000, offset, scale)
        fo = osc.trace_rays(fr)
        assert (fo["inst"] != 0xFFFFFFFF).mean() > 0.2
        assert_hits_equal(gpu_trace_rays(r, fr), fo)
        assert r.stats().device_error == 0


def test_wide_tree_shape():
    """The collapse keeps at most one wide node per two-child interior node, packs the 1M
    triangle bricks mesh level about three binary levels per wide level, and stays within
    the traversal stack."""
    sc, cam, st = scenes.bricks(width=64, height=36)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        s = r.stats()
        assert s.wide_nodes > 0
        assert s.wide_nodes <= s.bvh_nodes + s.tlas_nodes
        assert s.wide_nodes < 0.5 * (s.bvh_nodes + s.tlas_nodes), (s.wide_nodes, s.bvh_nodes, s.tlas_nodes)
        assert 2 <= s.wide_depth <= 31, s.wide_depth
        r.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
        h = r.stats()
        assert abs(h.wide_nodes - s.wide_nodes) <= 0.1 * s.wide_nodes
