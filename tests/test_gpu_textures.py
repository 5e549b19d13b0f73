"""Textured materials and the HDR sky on the GPU against the oracle: diffuse textures at every
hit (sRGB checker, float gradient, a metal with a textured primary albedo), the MRA texture's
roughness in the G-buffer, normal maps at the primary vertex (both tangent handednesses), an
id without a texture (white), and the equirectangular sky with a rotation and a sun above the
clamp of 10, over several frames with TAA, reprojection and the bilateral compose. Hit ids
are bit-exact and radiance within RTOL; a textured glTF file renders the same way."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, gltf, scenes
from gknextengine_gb300.native import GkrtError
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_parity import ATOL, RTOL, _compare_trace_images

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H", [(96, 64), (61, 47)])
def test_textured_cornell_matches_oracle(W, H):
    sc, cam, st = scenes.cornell_textured()
    st.taa = True
    st.flags = abi.FRAME_PRIMARY_IDS
    osc = O.OracleScene(sc)
    oim = O.new_images(W, H)
    fb = camera.FrameBuilder(W, H, st)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        for f in range(3):
            fc = fb.build(cam.orbit(2.0 * f), f)
            r.render(fc)
            r.synchronize()
            O.render_frame(osc, fc, W, H, oim)
            gim = r.images()
            _compare_trace_images(gim, oim)
            for k in (abi.IMG_PREV_DIFFUSE, abi.IMG_DENOISED_LINEAR):
                np.testing.assert_allclose(gim[k], oim[k], rtol=RTOL, atol=ATOL, err_msg=f"frame {f} image {k}")
        # the textures and the sky matter: varied albedo on textured walls, MRA roughness, sky misses
        hit = gim[abi.IMG_HIT_INST] != 0xFFFFFFFF
        assert (~hit).mean() > 0.05
        assert np.unique(np.round(gim[abi.IMG_ALBEDO][hit][:, 0], 4)).size > 50
        assert np.unique(np.round(gim[abi.IMG_NORMAL][hit][:, 3], 4)).size > 10


def test_textured_cornell_emissive_nee_matches_oracle():
    """The textured scene under emissive-triangle NEE (the instantiation with both the alias
    table and the texture fetches): three frames equal to the oracle's, ids exact."""
    sc, cam, st = scenes.cornell_textured()
    st.nee_mode = abi.NEE_EMISSIVE
    st.flags = abi.FRAME_PRIMARY_IDS
    W, H = 80, 56
    osc = O.OracleScene(sc)
    oim = O.new_images(W, H)
    fb = camera.FrameBuilder(W, H, st)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        assert r.stats().emitters > 0
        for f in range(3):
            fc = fb.build(cam.orbit(1.5 * f), f)
            r.render(fc)
            r.synchronize()
            O.render_frame(osc, fc, W, H, oim)
            _compare_trace_images(r.images(), oim)


def test_textured_render_differs_from_untextured():
    """The same frame with the textures, and with the materials' texture ids set to -1 and no
    sky texture, differ (both equal the oracle's own renderings)."""
    sc, cam, st = scenes.cornell_textured()
    W = H = 48
    fc_tex = camera.FrameBuilder(W, H, st).build(cam, 0)
    plain = sc.materials.copy()
    for k in ("diffuse_texture_id", "mra_texture_id", "normal_texture_id"):
        plain[k] = -1
    sc2 = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, plain, sc.instances,
                          lights=sc.lights)
    st.sky_texture = None
    fc_plain = camera.FrameBuilder(W, H, st).build(cam, 0)
    out = []
    for s, fc in ((sc, fc_tex), (sc2, fc_plain)):
        with PathTracingRenderer(0) as r:
            r.load_scene(s)
            r.create_swap_chain(W, H)
            r.trace_pass(fc)
            r.synchronize()
            g = r.read_image(abi.IMG_SINGLE_DIFFUSE)
        oim = O.new_images(W, H)
        O.OracleScene(s).trace_pass(fc, W, H, oim)
        np.testing.assert_allclose(g, oim[abi.IMG_SINGLE_DIFFUSE], rtol=RTOL, atol=ATOL)
        out.append(g)
    assert np.abs(out[0] - out[1]).mean() > 1e-3


def test_textured_glb_renders_like_the_oracle():
    from test_textures import textured_glb
    data, _ = textured_glb()
    sc, cam, st, info = gltf.load_glb(data)
    sky = scenes.procedural_textures()["sky"]
    sc.textures[st.sky_texture] = sky        # the file's SkyIdx, as the caller uploads a sky there
    st.sky_intensity = 0.5
    st.flags = abi.FRAME_PRIMARY_IDS
    W, H = 64, 48
    fc = camera.FrameBuilder(W, H, st).build(cam, 0)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        r.trace_pass(fc)
        r.synchronize()
        gim = r.images()
    oim = O.new_images(W, H)
    O.OracleScene(sc).trace_pass(fc, W, H, oim)
    _compare_trace_images(gim, oim)


def test_texture_upload_errors_and_replacement():
    sc, cam, st = scenes.cornell_textured()
    W = H = 32
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        bad = [(abi.MAX_TEXTURES, abi.TEX_RGBA32F, np.zeros((2, 2, 4), np.float32)),
               (3, 7, np.zeros((2, 2, 4), np.uint8))]
        for tid, fmt, t in bad:
            with pytest.raises(GkrtError) as e:
                r.upload_texture(tid, fmt, t)
            assert e.value.code == abi.GKRT_ERR_INVALID_ARG
        import ctypes as C
        t = np.zeros((2, 2, 4), np.uint8)
        rc = r._lib.gkrt_texture_upload(r._h, 3, 2, 2, abi.TEX_RGBA8_UNORM, t.ctypes.data, 15)
        assert rc == abi.GKRT_ERR_INVALID_ARG
        fc = camera.FrameBuilder(W, H, st).build(cam, 0)
        r.trace_pass(fc)
        r.synchronize()
        a = r.read_image(abi.IMG_ALBEDO)
        # replace the checker (id 5) by a flat red texture: the left wall's albedo follows
        red = np.zeros((4, 4, 4), np.uint8)
        red[..., 0] = 255
        red[..., 3] = 255
        r.upload_texture(5, abi.TEX_RGBA8_UNORM, red)
        sc.textures[5] = (abi.TEX_RGBA8_UNORM, red)
        r.trace_pass(fc)
        r.synchronize()
        b = r.read_image(abi.IMG_ALBEDO)
        oim = O.new_images(W, H)
        O.OracleScene(sc).trace_pass(fc, W, H, oim)
        np.testing.assert_allclose(b, oim[abi.IMG_ALBEDO], rtol=RTOL, atol=ATOL)
        assert not np.array_equal(a, b)


def _scaled(sc, scale):
    """The scene with every instance and light scaled by `scale` about the origin."""
    inst = sc.instances.copy()
    for i in range(len(inst)):
        w = np.asarray(inst[i]["world"], np.float64).reshape(3, 4) * scale
        inst[i]["world"] = w.astype(np.float32).reshape(12)
        inst[i]["world_inv"] = scenes.affine_inverse(inst[i]["world"])
    lights = sc.lights.copy()
    for k in ("p0", "p1", "p3"):
        lights[k][:, :3] *= scale
    lights["normal_area"][:, 3] *= scale * scale
    return abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials, inst,
                           lights=lights, name=sc.name + "-x4", texcoords=sc.texcoords, tangents=sc.tangents,
                           textures=sc.textures)


def test_textured_bake_matches_oracle():
    """Two bake steps of the textured Cornell box (4 m) under the HDR sky: hits take the diffuse
    texture (AmbientCube.slang:504-510), sky misses the sky texture's spherical-harmonic
    projection (SampleIBLRough); GPU words equal the oracle's, and both inputs change them."""
    from test_gpu_probes import ranges
    sc, cam, st = scenes.cornell_textured()
    sc = _scaled(sc, 4.0)
    # bright enough for the packed colours (10 bits up to 512) to register a 1/8 blend step,
    # the sun's light then as bounce light through the textured albedos
    st.sky_intensity = 40.0
    st.has_sun, st.sun_direction, st.sun_intensity = True, (0.3, 0.6, 1.0), 200.0
    fc = camera.FrameBuilder(64, 64, st).build(cam, 0)
    assert fc.flags & abi.FRAME_SKY_TEXTURE
    first = ranges()[0][0]
    count = ranges()[-1][0] + ranges()[-1][1] - first
    osc = O.OracleScene(sc)
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.probe_voxelize()
        r.synchronize()
        for step in range(2):
            prev, vox = r.probe_download()
            r.probe_bake(fc, first, count)
            r.synchronize()
            cubes, _ = r.probe_download()
            o, _ = osc.probe_bake(fc, first, count, prev, vox)
            g = cubes[first:first + count]
            bad = np.nonzero((g != o).any(axis=1))[0]
            assert bad.size == 0, (step, bad[:5], g[bad[:2]], o[bad[:2]])
        assert r.stats().device_error == 0
    # the same step without the sky texture (constant sky) and without textures differs
    surf = (vox[first:first + count, 2] & 0xFF) < 8
    assert surf.sum() > 1000
    st.sky_texture = None
    fc_const = camera.FrameBuilder(64, 64, st).build(cam, 0)
    o_const, _ = osc.probe_bake(fc_const, first, count, prev, vox)
    assert ((o_const != o)[surf][:, 6:12]).any(axis=1).mean() > 0.05
    mats = sc.materials.copy()
    mats["diffuse_texture_id"] = -1
    plain = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, mats, sc.instances,
                            lights=sc.lights, name="cornell-x4-untextured", texcoords=sc.texcoords,
                            tangents=sc.tangents, textures=sc.textures)
    o_plain, _ = O.OracleScene(plain).probe_bake(fc, first, count, prev, vox)
    assert ((o_plain != o)[surf][:, 0:6]).any(axis=1).mean() > 0.01   # bounce light through textured albedo


def test_adjoint_refuses_textures():
    sc, cam, st = scenes.cornell_textured()
    W = H = 32
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        st.has_sun = False
        fc = camera.FrameBuilder(W, H, st).build(cam, 0)
        import torch
        img = torch.zeros((H, W, 4), device="cuda")
        with pytest.raises(GkrtError) as e:
            r.adjoint_forward(fc, 1, img.data_ptr())
        assert e.value.code == abi.GKRT_ERR_UNSUPPORTED
