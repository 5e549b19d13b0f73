"""Emissive-triangle NEE (GKRT_NEE_EMISSIVE) on the GPU against the oracle.

The alias table is built on the host by the library and by the oracle independently; the
kernel's light picks, points, shadow segments and contributions must reproduce the oracle's
(ids bit-exact, radiance within 1e-4 relative).
"""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_parity import _compare_trace_images, _moving_cornell

pytestmark = pytest.mark.gpu


def _pass(r, osc, fc, W, H):
    r.trace_pass(fc)
    r.synchronize()
    gim = r.images()
    oim = O.new_images(W, H)
    orays = osc.trace_pass(fc, W, H, oim)
    _compare_trace_images(gim, oim)
    assert r.stats().rays_traced == orays
    return gim


def test_cornell_nee_pass():
    sc, cam, st = scenes.cornell()
    W = H = 256
    st.nee_mode = abi.NEE_EMISSIVE
    st.flags = abi.FRAME_PRIMARY_IDS
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        assert r.stats().emitters == 2
        osc = O.OracleScene(sc)
        fb = camera.FrameBuilder(W, H, st)
        for f in range(2):
            _pass(r, osc, fb.build(cam, f), W, H)


def test_bricks_nee_pass():
    sc, cam, st = scenes.bricks()
    W, H = 320, 180
    st.nee_mode = abi.NEE_EMISSIVE
    st.flags = abi.FRAME_PRIMARY_IDS
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        assert r.stats().emitters == 64 * 252
        _pass(r, O.OracleScene(sc), camera.FrameBuilder(W, H, st).build(cam, 0), W, H)


def test_nee_table_follows_instance_updates():
    """Moving, hiding and re-materialising instances rebuilds the emitter table."""
    sc, cam, st = _moving_cornell()
    W, H = 96, 96
    st.nee_mode = abi.NEE_EMISSIVE
    st.flags = abi.FRAME_PRIMARY_IDS
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        fb = camera.FrameBuilder(W, H, st)
        inst = sc.instances.copy()
        # the tall box becomes an emitter (material 7 on its slot 0), then moves
        inst[1]["mat_id"][0] = 7
        for f, dx in enumerate((0.0, 0.05, -0.05)):
            w = scenes.trs((-0.17 + dx, 0.0, -0.15), rot_y_deg=18.0, scale=(0.3, 0.6, 0.3))
            inst[1]["world"] = w
            inst[1]["world_inv"] = scenes.affine_inverse(w)
            r.update_instances(inst)
            assert r.stats().emitters == 2 + 12
            sc2 = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes,
                                  sc.materials, inst, name="cornell-moved")
            _pass(r, O.OracleScene(sc2), fb.build(cam, f), W, H)
        inst[1]["visible"] = 0
        r.update_instances(inst)
        assert r.stats().emitters == 2
