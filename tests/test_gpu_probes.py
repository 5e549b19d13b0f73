"""Ambient-cube probe grid on the GPU: voxelization (the reference's CPU VoxelizeCube) and the
bake (RenderAmbientCubeOnly), word for word against the oracle, then the rt pass with the
baked grid (path termination reads it) against the oracle rendering with the same grid.

The scene is the Cornell box scaled to 4 m (so it spans 16 probes a side) with its open front
to a bright sky and sun, and its ceiling light as light 0."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_parity import ATOL, RTOL, _compare_trace_images

pytestmark = pytest.mark.gpu

XY, ZL = 192, 48
LAYER = XY * XY
Y_LAYERS = 20          # probes up to y = 4.66 m: the 4 m room and above
ROWS = (80, 112)       # z rows 80..111 (z = -4 .. 3.75 m); every x of each row


def big_cornell(scale=4.0):
    sc, cam, st = scenes.cornell()
    inst = sc.instances.copy()
    for i in range(len(inst)):
        w = np.asarray(inst[i]["world"], np.float64).reshape(3, 4).copy()
        w *= scale
        inst[i]["world"] = w.astype(np.float32).reshape(12)
        inst[i]["world_inv"] = scenes.affine_inverse(inst[i]["world"])
    lights = sc.lights.copy()
    for k in ("p0", "p1", "p3"):
        lights[k][:, :3] *= scale
    lights["normal_area"][:, 3] *= scale * scale
    sc2 = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials, inst,
                          lights=lights, name="cornell-4m")
    cam = camera.Camera(eye=(0.0, 2.0, 7.76), center=(0.0, 2.0, 0.0), fov_deg=40.0)
    # bright enough for the packed colours (10 bits up to 512) to register a 1/8 blend step
    st.has_sky, st.sky_color, st.sky_intensity = True, (0.6, 0.7, 0.9, 1.0), 40.0
    st.has_sun, st.sun_direction, st.sun_intensity = True, (0.3, 0.6, 1.0), 200.0
    return sc2, cam, st


def ranges():
    """Contiguous probe index ranges covering the test region (whole x rows)."""
    return [(y * LAYER + ROWS[0] * XY, (ROWS[1] - ROWS[0]) * XY) for y in range(Y_LAYERS)]


@pytest.fixture(scope="module")
def env():
    sc, cam, st = big_cornell()
    r = PathTracingRenderer(0)
    r.load_scene(sc)
    r.probe_voxelize()
    r.synchronize()
    yield sc, cam, st, r, O.OracleScene(sc)
    r.close()


def test_voxelize_matches_oracle(env):
    sc, cam, st, r, osc = env
    _, vox = r.probe_download()
    for first, count in ranges():
        o = osc.probe_voxelize(first, count)
        g = vox[first:first + count]
        bad = np.nonzero((g != o).any(axis=1))[0]
        assert bad.size == 0, (first, bad[:5], g[bad[:3]], o[bad[:3]])
    reg = np.concatenate([vox[f:f + c] for f, c in ranges()])
    inside = (reg[:, 2] >> 8) & 0xFF
    near = (reg[:, 2] & 0xFF) < 8
    assert (inside == 0).any() and (inside == 255).any() and near.any()
    assert (reg[:, 0] > 0).any()          # material ids recorded next to surfaces
    assert (reg[:, 1] == 0).all()         # ages reset
    assert r.stats().device_error == 0


def test_bake_matches_oracle_two_steps(env):
    sc, cam, st, r, osc = env
    fc = camera.FrameBuilder(64, 64, st).build(cam, 0)
    first = ranges()[0][0]
    count = ranges()[-1][0] + ranges()[-1][1] - first
    for step in range(2):
        prev, vox = r.probe_download()
        r.probe_bake(fc, first, count)
        r.synchronize()
        cubes, vox2 = r.probe_download()
        o, ages = osc.probe_bake(fc, first, count, prev, vox)
        g = cubes[first:first + count]
        bad = np.nonzero((g != o).any(axis=1))[0]
        assert bad.size == 0, (step, bad[:5], g[bad[:2]], o[bad[:2]])
        assert np.array_equal(vox2[first:first + count, 1], ages)
        # probes outside the range are untouched
        assert np.array_equal(cubes[:first], prev[:first])
        surf = (vox[first:first + count, 2] & 0xFF) < 8
        assert surf.sum() > 1000
        lit = ((g[surf][:, 6:12] & 0x3FFFFFFF) != 0).any(axis=1)
        assert lit.mean() > 0.5, lit.mean()
        if step == 1:   # the second step sees the first step's light as bounce light
            assert ((g[surf][:, 0:6] & 0x3FFFFFFF) != 0).any(axis=1).mean() > 0.01
    assert r.stats().device_error == 0


def test_trace_pass_with_baked_probes(env):
    """Path termination reads the baked grid (fast gather): the rt pass against the oracle
    rendering with the downloaded grid."""
    sc, cam, st, r, osc = env
    cubes, vox = r.probe_download()
    assert (cubes != 0).any()
    st.fast_gather = True
    try:
        W = H = 96
        r.create_swap_chain(W, H)
        st.flags = abi.FRAME_PRIMARY_IDS
        fc = camera.FrameBuilder(W, H, st).build(cam, 3)
        r.trace_pass(fc)
        r.synchronize()
        gim = r.images()
        sc_p = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials,
                               sc.instances, lights=sc.lights, probe_cubes=cubes.reshape(-1),
                               probe_voxels=vox.reshape(-1), name="cornell-4m-probes")
        oim = O.new_images(W, H)
        O.OracleScene(sc_p).trace_pass(fc, W, H, oim)
        _compare_trace_images(gim, oim)
        assert gim[abi.IMG_SINGLE_DIFFUSE][..., :3].max() > 0.0
    finally:
        st.fast_gather = False
