"""Textured materials and the HDR sky on the CPU side: the oracle's atan2/acos against float64,
its texture lookup against a float64 restatement of Vulkan's linear filter with repeat
addressing (SampleLevel(uv, 0) of the pool's sampler, Sampler.hpp:9-27), the RGBA8 decodes, the
equirectangular sky lookup (SampleIBLV2, Shading.slang:194-199), the PNG and Radiance RGBE
readers, and glTF textures and vertex attributes."""
import json
import os
import struct
import zlib

import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, gltf, imageio, scenes
from oracle import oracle as O
from oracle.oracle import REFERENCE_TREE


def _ulp(x):
    return np.spacing(np.abs(np.float32(x))).astype(np.float64)


def test_atan2_acos_accuracy():
    rng = np.random.default_rng(1)
    L = O.lib()
    ys = np.concatenate([rng.normal(size=4000), rng.uniform(-1e-3, 1e-3, 500), [0.0, -0.0, 1.0, -1.0, 0.0]])
    xs = np.concatenate([rng.normal(size=4000), rng.uniform(-1e-3, 1e-3, 500), [1.0, 1.0, 0.0, 0.0, -1.0]])
    for y, x in zip(ys.astype(np.float32), xs.astype(np.float32)):
        got = L.gko_atan2(float(y), float(x))
        ref = np.arctan2(np.float64(y), np.float64(x))
        if y == 0 and x == 0:
            assert got == 0.0
            continue
        assert abs(got - ref) <= 4 * _ulp(ref) + 1e-30, (y, x, got, ref)
    for x in np.concatenate([np.linspace(-1, 1, 2001), [-1.0, 1.0, 0.9999999, -0.9999999]]).astype(np.float32):
        got = L.gko_acos(float(x))
        ref = np.arccos(np.float64(x))
        assert abs(got - ref) <= 4 * _ulp(ref) + 2e-7, (x, got, ref)


def _vulkan_linear(tex, u, v):
    """Vulkan's linear filter at level 0 with repeat addressing, in float64: i0 = floor(u w -
    1/2), alpha its fraction, texels i0 and i0 + 1 wrapped modulo the size."""
    h, w = tex.shape[:2]
    x, y = u * w - 0.5, v * h - 0.5
    fx, fy = np.floor(x), np.floor(y)
    a, b = x - fx, y - fy
    x0, x1 = int(fx) % w, int(fx + 1) % w
    y0, y1 = int(fy) % h, int(fy + 1) % h
    t = tex.astype(np.float64)
    return (t[y0, x0] * (1 - a) * (1 - b) + t[y0, x1] * a * (1 - b) + t[y1, x0] * (1 - a) * b +
            t[y1, x1] * a * b)


def _scene_with(textures):
    sc, _, _ = scenes.cornell()
    return abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials,
                           sc.instances, textures=textures)


def test_texture_sampling_matches_the_vulkan_filter():
    rng = np.random.default_rng(2)
    a = rng.uniform(-2.0, 5.0, (5, 3, 4)).astype(np.float32)      # 3 wide, 5 high
    b = rng.uniform(0.0, 1.0, (16, 32, 4)).astype(np.float32)
    osc = O.OracleScene(_scene_with({11: (abi.TEX_RGBA32F, a), 12: (abi.TEX_RGBA32F, b)}))
    uvs = np.concatenate([rng.uniform(-3.0, 4.0, (400, 2)), rng.uniform(-1e4, 1e4, (50, 2)),
                          [[0.0, 0.0], [1.0, 1.0], [-0.0, 0.5], [0.999999, 0.000001]]]).astype(np.float32)
    for tid, tex in ((11, a), (12, b)):
        for u, v in uvs:
            got = osc.tex_sample(tid, float(u), float(v))
            ref = _vulkan_linear(tex, np.float64(u), np.float64(v))
            # the float32 position of a far coordinate moves the fraction by up to u w 2^-24
            tol = 1e-5 * (1.0 + abs(float(u)) * tex.shape[1] + abs(float(v)) * tex.shape[0]) * np.abs(tex).max()
            np.testing.assert_allclose(got, ref, atol=tol, rtol=0)
        # texel centres return the texel exactly (power-of-two sizes: the centres are exact floats)
        h, w = tex.shape[:2]
        if w & (w - 1) or h & (h - 1):
            continue
        for j in range(h):
            for i in range(w):
                assert np.array_equal(osc.tex_sample(tid, (i + 0.5) / w, (j + 0.5) / h), tex[j, i])


def test_rgba8_decodes_and_missing_textures():
    c = np.arange(256, dtype=np.uint8)
    t = np.stack([c, c[::-1], c, c[::-1]], axis=-1).reshape(16, 16, 4)
    osc = O.OracleScene(_scene_with({3: (abi.TEX_RGBA8_UNORM, t), 4: (abi.TEX_RGBA8_SRGB, t)}))

    def srgb(x):
        v = x / 255.0
        return np.where(v <= 0.04045, v / 12.92, ((v + 0.055) / 1.055) ** 2.4).astype(np.float32)

    for j in range(16):
        for i in range(16):
            px = t[j, i].astype(np.int64)
            u, v = (i + 0.5) / 16, (j + 0.5) / 16
            assert np.array_equal(osc.tex_sample(3, u, v), (px.astype(np.float32) / np.float32(255.0)))
            got = osc.tex_sample(4, u, v)
            assert np.array_equal(got[:3], srgb(px[:3]))
            assert got[3] == np.float32(px[3]) / np.float32(255.0)
    for tid in (0, 5, 4095, -1, 4096):
        assert np.array_equal(osc.tex_sample(tid, 0.3, 0.7), np.ones(4, np.float32))


def test_sky_lookup():
    t = scenes.procedural_textures()["sky"][1]
    osc = O.OracleScene(_scene_with({2: (abi.TEX_RGBA32F, t)}))
    st = camera.Settings(has_sky=True, sky_intensity=0.5, sky_texture=2, sky_rotation=0.3,
                         sky_color=(0.1, 0.2, 0.3, 1.0))
    fc = camera.FrameBuilder(8, 8, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0)), 0)
    assert fc.flags & abi.FRAME_SKY_TEXTURE and fc.sky_index == 2
    rng = np.random.default_rng(3)
    d = rng.normal(size=(500, 3))
    for v in d.astype(np.float32):
        got = osc.sky_dir(fc, v)
        n = v.astype(np.float64) / np.linalg.norm(v.astype(np.float64))
        u = (np.arctan2(n[0], n[2]) + np.pi * 0.3) / (2 * np.pi)
        w = np.arccos(np.clip(n[1], -1, 1)) / np.pi
        ref = np.minimum(_vulkan_linear(t, u, w), [10.0, 10.0, 10.0, 1.0]) * 0.5
        np.testing.assert_allclose(got, ref, atol=2e-3 * 0.5 * 40.0, rtol=0)
    # the sun (40 above the sky) is clamped at 10 before the intensity
    hi = max(osc.sky_dir(fc, dv)[0] for dv in d.astype(np.float32))
    assert hi <= 10.0 * 0.5 + 1e-6
    # without the flag the sky is the constant colour
    st.sky_texture = None
    fc2 = camera.FrameBuilder(8, 8, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0)), 0)
    np.testing.assert_allclose(osc.sky_dir(fc2, np.array([0, 1, 0], np.float32)), [0.05, 0.1, 0.15, 0.5],
                               rtol=1e-6)


def _sh_numpy(t):
    """ProjectHdrToSh (Texture.cpp:180-254) in float64, vectorised: texel (x, y) at theta =
    (y + 1/2) pi / h, phi = (x + 1/2) 2 pi / w, weight sin(theta) (pi / h)(2 pi / w)."""
    h, w = t.shape[:2]
    th = (np.arange(h) + 0.5) / h * np.pi
    ph = (np.arange(w) + 0.5) / w * 2 * np.pi
    st, ct = np.sin(th)[:, None], np.cos(th)[:, None]
    dx, dy, dz = st * np.cos(ph)[None], np.broadcast_to(ct, (h, w)), st * np.sin(ph)[None]
    basis = np.stack([np.full((h, w), 0.282095), -0.488603 * dy, 0.488603 * dz, -0.488603 * dx,
                      1.092548 * dx * dy, -1.092548 * dy * dz, 0.315392 * (3 * dy * dy - 1),
                      -1.092548 * dx * dz, 0.546274 * (dx * dx - dz * dz)])
    wt = np.broadcast_to(st * (np.pi / h) * (2 * np.pi / w), (h, w))
    return np.einsum("khw,hwc->ck", basis * wt, t[..., :3].astype(np.float64))


def test_sky_sh_projection_and_the_bake_sky():
    """The probe bake's sky (SampleIBLRough): the texture's projection against a float64
    restatement, a constant sky evaluating to itself, skies linear in the direction evaluating
    to the same linear function (band 1 holds them exactly), with the rotation 1 - SkyRotation
    about y, 8-bit textures projecting to zero, and the frame's HasSky gate."""
    rng = np.random.default_rng(8)
    h, w = 32, 64
    th = (np.arange(h) + 0.5) / h * np.pi
    ph = (np.arange(w) + 0.5) / w * 2 * np.pi
    dx = (np.sin(th)[:, None] * np.cos(ph)[None]).astype(np.float32)
    dy = np.broadcast_to(np.cos(th)[:, None], (h, w)).astype(np.float32)
    rnd = rng.uniform(0.0, 3.0, (h, w, 4)).astype(np.float32)
    const = np.full((h, w, 4), 1.0, np.float32)
    const[..., :3] = (0.5, 1.5, 2.5)
    lin = np.ones((h, w, 4), np.float32)
    lin[..., 0] = 2.0 + dy
    lin[..., 1] = 2.0 + dx
    lin[..., 2] = 1.0
    rgba8 = rng.integers(0, 256, (h, w, 4), dtype=np.uint8)
    osc = O.OracleScene(_scene_with({1: (abi.TEX_RGBA32F, rnd), 2: (abi.TEX_RGBA32F, const),
                                     3: (abi.TEX_RGBA32F, lin), 4: (abi.TEX_RGBA8_SRGB, rgba8)}))
    np.testing.assert_allclose(osc.texture_sh(1), _sh_numpy(rnd), rtol=1e-6, atol=1e-6)
    assert not osc.texture_sh(4).any()

    def frame(idx, rot, has_sky=True, intensity=1.0):
        st = camera.Settings(has_sky=has_sky, sky_intensity=intensity, sky_texture=idx, sky_rotation=rot)
        return camera.FrameBuilder(8, 8, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0)), 0)

    dirs = rng.normal(size=(64, 3))
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    for n in dirs:
        # a constant sky: c0^2 4 pi = 1; the midpoint sums over 32 rows leak a few 1e-3 into
        # band 0 and the zonal band-2 term
        np.testing.assert_allclose(osc.sky_rough(frame(2, 0.4, intensity=2.0), n), [1.0, 3.0, 5.0, 2.0], rtol=4e-3)
        # rotation angle (1 - SkyRotation) pi: SkyRotation 1 leaves directions alone, 0 turns x to -x
        got = osc.sky_rough(frame(3, 1.0), n)
        np.testing.assert_allclose(got[:3], [2.0 + n[1], 2.0 + n[0], 1.0], atol=1e-2)
        got = osc.sky_rough(frame(3, 0.0), n)
        np.testing.assert_allclose(got[:3], [2.0 + n[1], 2.0 - n[0], 1.0], atol=1e-2)
    assert not osc.sky_rough(frame(2, 0.0, has_sky=False), dirs[0]).any()
    np.testing.assert_array_equal(osc.sky_rough(frame(4, 0.0), dirs[0]), [0.0, 0.0, 0.0, 1.0])   # (rgb, 1)


def test_rgbe_reader():
    rng = np.random.default_rng(4)
    rgbe = rng.integers(0, 256, (7, 40, 4)).astype(np.uint8)
    rgbe[1, 5:30] = (10, 20, 30, 130)   # runs for the run-length encoder
    rgbe[2, :, 3] = 0                   # exponent 0: black
    ref = np.ones((7, 40, 4), np.float32)
    e = rgbe[..., 3].astype(np.int64)
    ref[..., :3] = np.where(e[..., None] > 0, rgbe[..., :3] * np.ldexp(1.0, e - 136)[..., None], 0.0)
    for rle in (False, True):
        got = imageio.decode_hdr(imageio.encode_hdr(rgbe, rle=rle))
        assert np.array_equal(got, ref)
    with pytest.raises(ValueError):
        imageio.decode_hdr(b"P6\n1 1\n255\n\0\0\0")


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE_TREE, "assets", "textures")),
                    reason="reference tree absent")
def test_reference_skies_load():
    for name in imageio.REFERENCE_SKIES:
        a = imageio.load_hdr(os.path.join(REFERENCE_TREE, "assets", "textures", name))
        assert a.ndim == 3 and a.shape[1] == 2 * a.shape[0] and a.shape[2] == 4
        assert np.isfinite(a).all() and (a >= 0).all() and (a[..., 3] == 1).all()
        assert a[..., :3].max() > 1.0


def _png(rows, ctype, w, plte=None, trns=None, filters=(0,)):
    """A PNG of 8-bit samples (rows: (h, w * c) uint8) with the given per-row filters."""
    h = rows.shape[0]
    c = rows.shape[1] // w
    raw = bytearray()
    prev = np.zeros(rows.shape[1], np.int64)
    for y in range(h):
        ft = filters[y % len(filters)]
        line = rows[y].astype(np.int64)
        out = np.zeros_like(line)
        for x in range(line.size):
            a = line[x - c] if x >= c else 0
            b = prev[x]
            cc = prev[x - c] if x >= c else 0
            if ft == 0:
                p = 0
            elif ft == 1:
                p = a
            elif ft == 2:
                p = b
            elif ft == 3:
                p = (a + b) >> 1
            else:
                pa, pb, pc = abs(b - cc), abs(a - cc), abs(a + b - 2 * cc)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else cc)
            out[x] = (line[x] - p) & 0xFF
        raw += bytes([ft]) + out.astype(np.uint8).tobytes()
        prev = line

    def chunk(tag, data):
        return struct.pack(">I", len(data)) + tag + data + struct.pack(">I", zlib.crc32(tag + data) & 0xFFFFFFFF)
    s = b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if plte is not None:
        s += chunk(b"PLTE", plte.astype(np.uint8).tobytes())
    if trns is not None:
        s += chunk(b"tRNS", trns.astype(np.uint8).tobytes())
    return s + chunk(b"IDAT", zlib.compress(bytes(raw))) + chunk(b"IEND", b"")


def test_png_reader_filters_and_colour_types():
    rng = np.random.default_rng(5)
    w, h = 9, 10
    rgba = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    got = imageio.decode_png(_png(rgba.reshape(h, -1), 6, w, filters=(0, 1, 2, 3, 4)))
    assert np.array_equal(got, rgba)
    rgb = rgba[..., :3].copy()
    assert np.array_equal(imageio.decode_png(_png(rgb.reshape(h, -1), 2, w, filters=(4, 3, 2, 1))), rgb)
    assert np.array_equal(imageio.decode_png(_png(rgb.reshape(h, -1), 2, w), rgba=True)[..., 3], np.full((h, w), 255))
    grey = rgba[..., :1]
    g = imageio.decode_png(_png(grey.reshape(h, -1), 0, w, filters=(1, 4)))
    assert np.array_equal(g[..., 0], grey[..., 0]) and np.array_equal(g[..., 2], grey[..., 0])
    ga = rgba[..., :2]
    g = imageio.decode_png(_png(ga.reshape(h, -1), 4, w, filters=(3,)))
    assert np.array_equal(g[..., 1], ga[..., 0]) and np.array_equal(g[..., 3], ga[..., 1])
    plte = rng.integers(0, 256, (7, 3))
    idx = rng.integers(0, 7, (h, w)).astype(np.uint8)
    trns = np.array([0, 50, 255])
    p = imageio.decode_png(_png(idx, 3, w, plte=plte, trns=trns, filters=(2,)))
    assert np.array_equal(p[..., :3], plte[idx])
    alpha = np.full(256, 255)
    alpha[:3] = trns
    assert np.array_equal(p[..., 3], alpha[idx])


def textured_glb(with_ktx=False):
    """A quad with a PNG base-colour texture, TEXCOORD_0 and TANGENT (and, optionally, a second
    material whose texture is a KTX2 image, which is not decoded)."""
    from test_gltf import Builder, quad_mesh, write_glb
    b = Builder()
    q = quad_mesh(b)
    q["attributes"]["TEXCOORD_0"] = b.add(np.array([[0, 0], [2, 0], [2, 2], [0, 2]], np.float32), 5126, "VEC2")
    q["attributes"]["TANGENT"] = b.add(np.array([[1, 0, 0, 1]] * 4, np.float32), 5126, "VEC4")
    q["material"] = 0
    tex = np.zeros((4, 4, 4), np.uint8)
    tex[..., 0] = np.arange(16).reshape(4, 4) * 16
    tex[..., 1] = 200
    tex[..., 3] = 255
    png = imageio.encode_png(tex)
    while len(b.bin) % 4:
        b.bin.append(0)
    off = len(b.bin)
    b.bin += png
    b.views.append({"buffer": 0, "byteOffset": off, "byteLength": len(png)})
    images = [{"bufferView": len(b.views) - 1, "mimeType": "image/png"}]
    mats = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "roughnessFactor": 0.5,
                                      "metallicFactor": 0.0}}]
    if with_ktx:
        images.append({"bufferView": len(b.views) - 1, "mimeType": "image/ktx2"})
        mats.append({"pbrMetallicRoughness": {"baseColorTexture": {"index": 1}}, "normalTexture": {"index": 0}})
    doc = {"asset": {"version": "2.0"}, "scene": 0,
           "scenes": [{"nodes": [0, 1], "extras": {"SkyIdx": 3, "SkyRotation": 0.25}}],
           "nodes": [{"mesh": 0, "scale": [2.0, 1.0, 2.0]},
                     {"camera": 0, "translation": [0.0, 2.0, 4.0], "rotation": [-0.2588, 0.0, 0.0, 0.9659]}],
           "cameras": [{"type": "perspective", "perspective": {"yfov": 0.7, "znear": 0.1}}],
           "materials": mats, "textures": [{"source": i} for i in range(len(images))], "images": images,
           "meshes": [{"primitives": [q]}], "accessors": b.accessors, "bufferViews": b.views,
           "buffers": [{"byteLength": len(b.bin) + (-len(b.bin) % 4)}]}
    return write_glb(doc, bytes(b.bin)), tex


def test_gltf_textures_and_vertex_attributes():
    data, tex = textured_glb(with_ktx=True)
    sc, cam, st, info = gltf.load_glb(data)
    m = sc.materials
    assert m["diffuse_texture_id"][0] == gltf.TEXTURE_BASE
    assert m["diffuse_texture_id"][1] == gltf.TEXTURE_BASE + 1 and m["normal_texture_id"][1] == gltf.TEXTURE_BASE
    fmt, texels = sc.textures[gltf.TEXTURE_BASE]
    assert fmt == abi.TEX_RGBA8_UNORM or fmt == abi.TEX_RGBA8_SRGB
    assert fmt == abi.TEX_RGBA8_SRGB                     # base colour images are sRGB
    assert np.array_equal(texels, tex)
    assert gltf.TEXTURE_BASE + 1 not in sc.textures
    assert info["textures_not_decoded"] == [{"image": 1, "mime": "image/ktx2"}]
    np.testing.assert_array_equal(sc.texcoords[:4], [[0, 0], [2, 0], [2, 2], [0, 2]])
    np.testing.assert_array_equal(sc.tangents[:4], [[1, 0, 0, 1]] * 4)
    assert st.sky_texture == 3 and st.sky_rotation == 0.25
    fc = camera.FrameBuilder(8, 8, st).build(cam, 0)
    assert fc.flags & abi.FRAME_SKY_TEXTURE and fc.sky_index == 3
    # the oracle renders it with the texture (the sky texture 3 is absent: white)
    osc = O.OracleScene(sc)
    im = O.new_images(32, 32)
    fc = camera.FrameBuilder(32, 32, st).build(cam, 0)
    osc.trace_pass(fc, 32, 32, im)
    alb = im[abi.IMG_ALBEDO]
    hit = im[abi.IMG_HIT_INST] != 0xFFFFFFFF
    assert hit.any() and np.unique(np.round(alb[hit][:, 0], 5)).size > 8   # the texture varies the albedo
