"""glTF (.glb) scene loading (FSceneLoader::LoadGLTFScene): material rules, node transforms,
cameras, area lights, scene extras and accessor layouts on files written here, and the
reference's own uncompressed scenes when the reference tree is present."""
import json
import math
import os
import struct

import numpy as np
import pytest

from gknextengine_gb300 import abi, gltf

from oracle.oracle import REFERENCE_TREE

REF_MODELS = os.path.join(REFERENCE_TREE, "assets", "models")


def write_glb(doc: dict, binchunk: bytes) -> bytes:
    """A .glb from a JSON document and the binary chunk (both padded to 4 bytes)."""
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    binchunk = binchunk + b"\0" * (-len(binchunk) % 4)
    total = 12 + 8 + len(js) + 8 + len(binchunk)
    return (struct.pack("<III", 0x46546C67, 2, total) + struct.pack("<II", len(js), 0x4E4F534A) + js +
            struct.pack("<II", len(binchunk), 0x004E4942) + binchunk)


class Builder:
    def __init__(self):
        self.bin = bytearray()
        self.views, self.accessors = [], []

    def add(self, arr: np.ndarray, ctype: int, typ: str, stride: int = 0) -> int:
        while len(self.bin) % 4:
            self.bin.append(0)
        view = {"buffer": 0, "byteOffset": len(self.bin), "byteLength": arr.nbytes}
        if stride:
            view["byteStride"] = stride
        self.bin += arr.tobytes()
        self.views.append(view)
        count = arr.shape[0] if not stride else arr.nbytes // stride
        self.accessors.append({"bufferView": len(self.views) - 1, "componentType": ctype, "type": typ,
                               "count": count})
        return len(self.accessors) - 1


def quad_mesh(b: Builder, with_normals=True, idx16=True):
    p = np.array([[-1, 0, -1], [1, 0, -1], [1, 0, 1], [-1, 0, 1]], np.float32)
    prim = {"attributes": {"POSITION": b.add(p, 5126, "VEC3")},
            "indices": b.add(np.array([0, 2, 1, 0, 3, 2], np.uint16 if idx16 else np.uint32), 5123 if idx16 else 5125,
                             "SCALAR")}
    if with_normals:
        prim["attributes"]["NORMAL"] = b.add(np.tile(np.array([[0, 1, 0]], np.float32), (4, 1)), 5126, "VEC3")
    return prim


def interleaved_box(b: Builder):
    """Position and normal interleaved in one view (byteStride 24), 32-bit indices."""
    lo, hi = -0.5, 0.5
    pts, nrm, idx = [], [], []
    for axis in range(3):
        for s in (-1.0, 1.0):
            n = np.zeros(3); n[axis] = s
            u, v = [(a) for a in range(3) if a != axis]
            base = len(pts)
            for cu, cv in ((lo, lo), (hi, lo), (hi, hi), (lo, hi)):
                q = np.zeros(3); q[axis] = s * 0.5; q[u] = cu; q[v] = cv
                pts.append(q); nrm.append(n)
            idx += [base, base + 1, base + 2, base, base + 2, base + 3]
    inter = np.concatenate([np.array(pts, np.float32), np.array(nrm, np.float32)], axis=1)
    while len(b.bin) % 4:
        b.bin.append(0)
    off = len(b.bin)
    b.bin += inter.tobytes()
    b.views.append({"buffer": 0, "byteOffset": off, "byteLength": inter.nbytes, "byteStride": 24})
    vi = len(b.views) - 1
    b.accessors.append({"bufferView": vi, "componentType": 5126, "type": "VEC3", "count": len(pts)})
    b.accessors.append({"bufferView": vi, "byteOffset": 12, "componentType": 5126, "type": "VEC3", "count": len(pts)})
    ia = b.add(np.array(idx, np.uint32), 5125, "SCALAR")
    return {"attributes": {"POSITION": len(b.accessors) - 3, "NORMAL": len(b.accessors) - 2}, "indices": ia}


def make_scene(**extras):
    b = Builder()
    q0 = quad_mesh(b)
    q0["material"] = 0
    q1 = quad_mesh(b, with_normals=False, idx16=False)
    q1["material"] = 2
    box = interleaved_box(b)
    box["material"] = 1
    lines = {"attributes": {"POSITION": q0["attributes"]["POSITION"]}, "indices": q0["indices"], "mode": 1}
    mats = [
        {"pbrMetallicRoughness": {"baseColorFactor": [0.25, 0.64, 1.0, 1.0], "roughnessFactor": 0.3,
                                  "metallicFactor": 0.0}},
        {"pbrMetallicRoughness": {"baseColorFactor": [0.81, 0.81, 0.81, 1.0], "roughnessFactor": 0.2,
                                  "metallicFactor": 0.99}},
        {"pbrMetallicRoughness": {"roughnessFactor": 1.0, "metallicFactor": 0.0}},
        {"pbrMetallicRoughness": {"roughnessFactor": 0.1, "metallicFactor": 0.0},
         "extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.9},
                        "KHR_materials_ior": {"ior": 1.33}}, "extras": {"ior2": 1.1}},
        {"emissiveFactor": [1.0, 0.5, 0.25], "extensions": {"KHR_materials_emissive_strength": {"emissiveStrength": 2.0}}},
    ]
    s = math.sqrt(0.5)
    nodes = [
        {"name": "floor", "mesh": 0, "scale": [4.0, 1.0, 4.0]},
        {"name": "group", "translation": [1.0, 2.0, 3.0], "rotation": [0.0, s, 0.0, s], "children": [2, 3]},
        {"name": "boxchild", "mesh": 1, "translation": [0.5, 0.0, 0.0], "scale": [2.0, 2.0, 2.0]},
        {"name": "cam", "camera": 0, "translation": [0.0, 1.0, 5.0]},
        {"name": "lamp", "mesh": 2, "translation": [0.0, 3.0, 0.0], "scale": [0.5, 1.0, 0.25],
         "extras": {"arealight": 1}},
    ]
    doc = {"asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0, 1, 4], "extras": extras}],
           "nodes": nodes, "materials": mats, "cameras": [{"type": "perspective",
                                                            "perspective": {"yfov": 0.7, "znear": 0.1}}],
           "meshes": [{"primitives": [q0]}, {"primitives": [lines, box]}, {"primitives": [q1]}],
           "accessors": b.accessors, "bufferViews": b.views,
           "buffers": [{"byteLength": len(b.bin) + (-len(b.bin) % 4)}]}
    return write_glb(doc, bytes(b.bin))


def test_material_rules():
    sc, cam, st, info = gltf.load_glb(make_scene())
    m = sc.materials
    assert m["material_model"][0] == abi.MAT_MIXTURE
    np.testing.assert_allclose(m["diffuse"][0], [0.5, 0.8, 1.0, 1.0], rtol=1e-6)
    assert m["fuzziness"][0] == np.float32(0.3) and m["refraction_index"][0] == np.float32(1.46)
    assert m["material_model"][1] == abi.MAT_METALLIC
    assert m["material_model"][2] == abi.MAT_LAMBERTIAN          # roughness 1, metalness 0
    assert m["material_model"][3] == abi.MAT_DIELECTRIC
    assert m["refraction_index"][3] == np.float32(1.33) and m["refraction_index2"][3] == np.float32(1.1)
    assert m["material_model"][4] == abi.MAT_DIFFUSE_LIGHT
    np.testing.assert_allclose(m["diffuse"][4][:3], [200.0, 100.0, 50.0])
    assert (m["diffuse_texture_id"] == -1).all()


def test_nodes_transforms_and_sections():
    sc, cam, st, info = gltf.load_glb(make_scene())
    assert info["instance_names"] == ["floor", "boxchild", "lamp"]
    assert list(sc.instances["instance_id"]) == [0, 2, 4]        # ids count every node depth first
    assert list(sc.instances["mesh_id"]) == [0, 1, 2]
    # box child: world = group (T(1,2,3) R_y(90)) x child (T(0.5,0,0) S(2))
    w = sc.instances["world"][1].reshape(3, 4)
    np.testing.assert_allclose(w[:, 3], [1.0, 2.0, 2.5], atol=1e-6)
    np.testing.assert_allclose(w[:, :3], [[0, 0, 2], [0, 2, 0], [-2, 0, 0]], atol=1e-6)
    wi = sc.instances["world_inv"][1].reshape(3, 4)
    full = np.vstack([w, [0, 0, 0, 1]]) @ np.vstack([wi, [0, 0, 0, 1]])
    np.testing.assert_allclose(full, np.eye(4), atol=1e-6)
    # the lines primitive is skipped: the box is section 0 of mesh 1, material slots keep the
    # raw primitive order (slot 0 -> primitive 0's material index 0, slot 1 -> material 1)
    m1 = sc.meshes[1]
    assert (sc.material_slots[m1["vertex_offset"]:m1["vertex_offset"] + m1["vertex_count"]] == 0).all()
    assert list(sc.instances["mat_id"][1][:2]) == [0, 1]
    # computed normals for the primitive without NORMAL point up (+y) for the (0, 2, 1) winding
    m2 = sc.meshes[2]
    n = sc.normals[m2["vertex_offset"]:m2["vertex_offset"] + m2["vertex_count"], :3]
    np.testing.assert_allclose(n, np.tile([0.0, 1.0, 0.0], (4, 1)), atol=1e-6)
    assert sc.indices.size == 6 + 36 + 6


def test_camera_light_and_extras():
    sc, cam, st, info = gltf.load_glb(make_scene(SunIntensity=50.0, SunRotation=0.25, NoSky=1))
    # the camera node's own transform (the reference ignores the parent here)
    np.testing.assert_allclose(cam.eye, [0.0, 1.0, 5.0])
    np.testing.assert_allclose(cam.center, [0.0, 1.0, 4.0])
    assert info["lights"] == 1
    L = sc.lights[0]
    np.testing.assert_allclose(L["p0"][:3], [-0.5, 3.0, -0.25])
    np.testing.assert_allclose(L["p1"][:3], [-0.5, 3.0, 0.25])
    np.testing.assert_allclose(L["p3"][:3], [0.5, 3.0, -0.25])
    np.testing.assert_allclose(L["normal_area"], [0.0, 1.0, 0.0, 0.25], atol=1e-6)
    assert L["light_mat_idx"] == 2
    assert st.has_sun and st.sun_intensity == 50.0 and not st.has_sky
    d = np.array([math.sin(0.25 * math.pi), 0.75, math.cos(0.25 * math.pi)])
    np.testing.assert_allclose(st.sun_direction, d / np.linalg.norm(d), rtol=1e-6)
    sc2, cam2, st2, _ = gltf.load_glb(make_scene())
    assert st2.has_sky and st2.sky_intensity == 100.0 and not st2.has_sun   # EnvironmentSetting::Reset


def test_auto_camera_and_errors():
    raw = bytearray(make_scene())
    gl, binchunk = gltf.read_glb(bytes(raw))
    gl["nodes"][3].pop("camera")
    sc, cam, st, info = gltf.load_glb(write_glb(gl, binchunk))
    # union of the meshes' local boxes: [-1, 1] x [-0.5, 0.5] x [-1, 1]
    np.testing.assert_allclose(cam.center, [0.0, 0.0, 0.0])
    np.testing.assert_allclose(cam.eye, [0.0, 0.0, math.sqrt(4 + 1 + 4)], rtol=1e-6)
    gl["meshes"][0]["primitives"][0]["extensions"] = {"KHR_draco_mesh_compression": {}}
    with pytest.raises(gltf.GlbError):
        gltf.load_glb(write_glb(gl, binchunk))
    with pytest.raises(gltf.GlbError):
        gltf.load_glb(b"not a glb file at all")
    gl2, _ = gltf.read_glb(bytes(raw))
    gl2["accessors"][gl2["meshes"][0]["primitives"][0]["indices"]]["count"] = 1 << 20
    with pytest.raises(gltf.GlbError):
        gltf.load_glb(write_glb(gl2, binchunk))


@pytest.mark.skipif(not os.path.isdir(REF_MODELS), reason="reference tree absent")
@pytest.mark.parametrize("name,tris,meshes,insts,mats", [("rigid", 136, 2, 2, 2), ("pbr", 8764, 10, 10, 10),
                                                         ("simple", 1120, 5, 1118, 5)])
def test_reference_scenes(name, tris, meshes, insts, mats):
    sc, cam, st, info = gltf.load_glb(os.path.join(REF_MODELS, name + ".glb"))
    assert (sc.indices.size // 3, len(sc.meshes), len(sc.instances), len(sc.materials)) == (tris, meshes, insts, mats)
    assert np.isfinite(sc.positions).all() and np.isfinite(sc.instances["world"]).all()
    for m in sc.meshes:
        i = sc.indices[m["index_offset"]:m["index_offset"] + m["index_count"]]
        assert i.size == 0 or i.max() < m["vertex_count"]


@pytest.mark.gpu
def test_loaded_scene_renders_like_the_oracle():
    """A loaded file (mixture, metal, Lambertian, dielectric and emissive materials, a node
    hierarchy, a quad light) through the rt pass against the oracle."""
    from gknextengine_gb300 import camera
    from gknextengine_gb300.renderer import PathTracingRenderer
    from oracle import oracle as O
    from test_gpu_parity import _compare_trace_images
    sc, cam, st, info = gltf.load_glb(make_scene(SunIntensity=3.0))
    st.sky_intensity = 0.5
    st.flags = abi.FRAME_PRIMARY_IDS
    W = H = 64
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        fc = camera.FrameBuilder(W, H, st).build(cam, 0)
        r.trace_pass(fc)
        r.synchronize()
        gim = r.images()
        oim = O.new_images(W, H)
        O.OracleScene(sc).trace_pass(fc, W, H, oim)
        _compare_trace_images(gim, oim)
        assert (gim[abi.IMG_HIT_INST] != 0xFFFFFFFF).mean() > 0.2
