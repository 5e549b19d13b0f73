"""glTF 2.0 binary (.glb) scenes as the library's scene arrays.

Follows the reference's loader, FSceneLoader::LoadGLTFScene and ParseGltfNode
(src/Assets/FSceneLoader.cpp:103-187, 218-565), and its environment defaults
(EnvironmentSetting::Reset, src/Assets/Model.hpp:27-43):

* materials (:300-372): "mixture" with fuzziness = roughnessFactor, metalness =
  metallicFactor, refraction indices 1.46, diffuse = sqrt(baseColorFactor.rgb) with alpha 1;
  metallic when metalness > 0.95, Lambertian when fuzziness > 0.95 and metalness < 0.01;
  KHR_materials_ior sets both indices, extras.ior2 the second; KHR_materials_transmission
  above 0.8 makes a dielectric; KHR_materials_emissive_strength makes a diffuse light of
  emissive x strength x 100;
* meshes (:374-505): triangle primitives with indices; each becomes a section whose index
  is the vertices' material slot; indices are relative to the mesh's vertices;
* nodes (:103-187): depth first from the scene's roots; translation, rotation (normalised
  quaternion) and scale compose T R S and the world transform is parent x local (Node::
  RecalcTransform, src/Assets/Node.cpp:35-55); node ids count every node in that order; a
  node with a mesh is an instance whose material slots are max(0, primitive material); a
  node with a camera and no mesh adds a camera from its own T R S (40 degrees field of
  view); extras.arealight adds a quad light from the node's own transform (the reference
  reads it before the parent is attached) over the 2 x 2 quad of Blender's light object,
  with the material of the node's last primitive;
* scene extras (:516-553): SkyIdx, SkyIntensity, SkyRotation (sky on), SunIntensity (sun
  on), WithSun, SunRotation (sun direction normalize(sin pi r, 0.75, cos pi r)), NoSky;
* without a camera, AutoFocusCamera (:755-783): from the union of the meshes' local boxes,
  looking at its centre from +z at the box diagonal's length.

* textures (:259-309, 328-331): base colour (sRGB), metallic-roughness and normal textures;
  image i of the file becomes texture id TEXTURE_BASE + i (the pool's ids below that hold the
  skies, Engine.cpp:853-870); PNG images embedded in the binary chunk are decoded (8-bit, any
  colour type); TEXCOORD_0 and TANGENT become the scene's vertex attributes. The sky samples
  texture SkyIdx (default 0), rotated by SkyRotation, as the reference's pool does; the caller
  uploads the reference's sky there (imageio.load_hdr, imageio.REFERENCE_SKIES).

Not taken over: images in other formats (JPEG and KTX2/BasisU need third-party decoders; their
ids stay on the materials and sample as white, and info["textures_not_decoded"] lists them),
animations, KHR_draco_mesh_compression (a third-party decoder; such files raise GlbError), node
matrices (the reference reads TRS only), sparse accessors. A primitive without normals gets
area-weighted vertex normals (the reference would read an invalid accessor).
"""
from __future__ import annotations

import json
import math
import struct

import numpy as np

from . import abi, camera, imageio, scenes

TEXTURE_BASE = 100   # texture id of the file's image 0


class GlbError(ValueError):
    pass


_DTYPE = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5124: np.int32, 5125: np.uint32,
          5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}


def read_glb(source):
    """(json dict, binary chunk bytes) of a .glb file path or bytes."""
    data = source if isinstance(source, (bytes, bytearray)) else open(source, "rb").read()
    if len(data) < 20:
        raise GlbError("file too short for a glb header")
    magic, version, length = struct.unpack_from("<III", data, 0)
    if magic != 0x46546C67 or version != 2:
        raise GlbError("not a glTF 2.0 binary file")
    off, gl, binchunk = 12, None, b""
    while off + 8 <= min(length, len(data)):
        clen, ctype = struct.unpack_from("<II", data, off)
        chunk = bytes(data[off + 8:off + 8 + clen])
        if ctype == 0x4E4F534A:
            gl = json.loads(chunk.decode("utf-8"))
        elif ctype == 0x004E4942:
            binchunk = chunk
        off += 8 + clen
    if gl is None:
        raise GlbError("no JSON chunk")
    return gl, binchunk


def accessor(gl: dict, binchunk: bytes, idx: int) -> np.ndarray:
    """Accessor idx as an array (count, components)."""
    a = gl["accessors"][idx]
    if "sparse" in a:
        raise GlbError("sparse accessors are not supported")
    if "bufferView" not in a:
        raise GlbError("accessor without a buffer view")
    v = gl["bufferViews"][a["bufferView"]]
    if v.get("buffer", 0) != 0 or "uri" in gl["buffers"][v.get("buffer", 0)]:
        raise GlbError("only the binary chunk's buffer is supported")
    dt = np.dtype(_DTYPE[a["componentType"]]).newbyteorder("<")
    nc = _NCOMP[a["type"]]
    count = a["count"]
    esize = dt.itemsize * nc
    stride = v.get("byteStride", esize) or esize
    base = v.get("byteOffset", 0) + a.get("byteOffset", 0)
    if count and base + (count - 1) * stride + esize > len(binchunk):
        raise GlbError("accessor outside the binary chunk")
    raw = np.frombuffer(binchunk, np.uint8)
    rows = np.lib.stride_tricks.as_strided(raw[base:], shape=(count, esize), strides=(stride, 1)) if count else \
        np.zeros((0, esize), np.uint8)
    return np.ascontiguousarray(rows).view(dt).reshape(count, nc)


def quat_matrix(x, y, z, w) -> np.ndarray:
    n = math.sqrt(x * x + y * y + z * z + w * w) or 1.0
    x, y, z, w = x / n, y / n, z / n, w / n
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def local_transform(node: dict) -> np.ndarray:
    m = np.eye(4)
    t = node.get("translation", [0.0, 0.0, 0.0])
    r = node.get("rotation", [0.0, 0.0, 0.0, 1.0])
    s = node.get("scale", [1.0, 1.0, 1.0])
    m[:3, :3] = quat_matrix(*r) @ np.diag(s)
    m[:3, 3] = t
    return m


def _texture_id(gl: dict, ref) -> int:
    """Texture id of a glTF texture reference ({"index": t}): TEXTURE_BASE + its image index."""
    if not ref or "index" not in ref:
        return -1
    t = gl.get("textures", [])[ref["index"]]
    src = t.get("source", ref["index"])
    return TEXTURE_BASE + int(src)


def _material(mat: dict, gl: dict) -> np.ndarray:
    pbr = mat.get("pbrMetallicRoughness", {})
    base = pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0])
    rough = float(pbr.get("roughnessFactor", 1.0))
    metal = float(pbr.get("metallicFactor", 1.0))
    has_mra = "metallicRoughnessTexture" in pbr
    if has_mra:
        rough = 1.0
    model = abi.MAT_MIXTURE
    if metal > 0.95 and not has_mra:
        model = abi.MAT_METALLIC
    if rough > 0.95 and not has_mra and metal < 0.01:
        model = abi.MAT_LAMBERTIAN
    ri = ri2 = 1.46
    ext = mat.get("extensions", {})
    if "KHR_materials_ior" in ext:
        ri = ri2 = float(ext["KHR_materials_ior"].get("ior", 1.5))
    if "KHR_materials_transmission" in ext and float(ext["KHR_materials_transmission"].get("transmissionFactor",
                                                                                                0.0)) > 0.8:
        model = abi.MAT_DIELECTRIC
    if "ior2" in mat.get("extras", {}):
        ri2 = float(mat["extras"]["ior2"])
    if "KHR_materials_emissive_strength" in ext:
        em = mat.get("emissiveFactor", [0.0, 0.0, 0.0])
        p = float(ext["KHR_materials_emissive_strength"].get("emissiveStrength", 1.0)) * 100.0
        return scenes.diffuse_light((em[0] * p, em[1] * p, em[2] * p))
    m = scenes.material([math.sqrt(base[0]), math.sqrt(base[1]), math.sqrt(base[2]), 1.0], model,
                        fuzziness=rough, ri=ri, metalness=metal, ri2=ri2)
    m["normal_texture_scale"] = float(mat.get("normalTexture", {}).get("scale", 1.0))
    m["diffuse_texture_id"] = _texture_id(gl, pbr.get("baseColorTexture"))
    m["mra_texture_id"] = _texture_id(gl, pbr.get("metallicRoughnessTexture"))
    m["normal_texture_id"] = _texture_id(gl, mat.get("normalTexture"))
    return m


def _textures(gl: dict, binchunk: bytes):
    """{texture id: (format, texels)} of the images the materials use, and the images that
    are not decoded here. Base colour images are sRGB, the others linear."""
    srgb, used = set(), set()
    for mat in gl.get("materials", []):
        pbr = mat.get("pbrMetallicRoughness", {})
        for key, is_srgb in ((pbr.get("baseColorTexture"), True), (pbr.get("metallicRoughnessTexture"), False),
                             (mat.get("normalTexture"), False)):
            tid = _texture_id(gl, key)
            if tid >= 0:
                used.add(tid)
                if is_srgb:
                    srgb.add(tid)
    out, skipped = {}, []
    for tid in sorted(used):
        img = gl.get("images", [])[tid - TEXTURE_BASE]
        mime = img.get("mimeType", "")
        if "bufferView" not in img or mime != "image/png":
            skipped.append({"image": tid - TEXTURE_BASE, "mime": mime or img.get("uri", "")})
            continue
        v = gl["bufferViews"][img["bufferView"]]
        data = binchunk[v.get("byteOffset", 0):v.get("byteOffset", 0) + v["byteLength"]]
        out[tid] = (abi.TEX_RGBA8_SRGB if tid in srgb else abi.TEX_RGBA8_UNORM, imageio.decode_png(data, rgba=True))
    return out, skipped


def _float_attr(gl: dict, binchunk: bytes, idx: int) -> np.ndarray:
    """An accessor as float32, normalized integer types mapped to [0, 1] / [-1, 1]."""
    a = gl["accessors"][idx]
    v = accessor(gl, binchunk, idx)
    ct = a["componentType"]
    if ct == 5126 or not a.get("normalized", False):
        return v.astype(np.float32)
    scale = {5121: 255.0, 5123: 65535.0, 5120: 127.0, 5122: 32767.0}[ct]
    return np.maximum(v.astype(np.float32) / np.float32(scale), np.float32(-1.0))


def _vertex_normals(pos: np.ndarray, idx: np.ndarray) -> np.ndarray:
    n = np.zeros_like(pos, dtype=np.float64)
    t = idx.reshape(-1, 3)
    fn = np.cross(pos[t[:, 1]] - pos[t[:, 0]], pos[t[:, 2]] - pos[t[:, 0]])
    for k in range(3):
        np.add.at(n, t[:, k], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return (n / ln).astype(np.float32)


def load_glb(source, width: int = 1920, height: int = 1080):
    """(SceneArrays, Camera, camera.Settings, info) of a .glb file path or bytes; info holds
    the node names of the instances, all cameras and the light count."""
    gl, binchunk = read_glb(source)
    # materials and their textures
    mats = [_material(m, gl) for m in gl.get("materials", [])]
    textures, tex_skipped = _textures(gl, binchunk)
    if not mats:
        mats = [scenes.mixture((1.0, 1.0, 1.0), 1.0)]
    # meshes
    pos_l, nrm_l, slot_l, idx_l, mesh_rows, local_boxes, uv_l, tan_l = [], [], [], [], [], [], [], []
    any_uv = any_tan = False
    voff = ioff = 0
    for mesh in gl.get("meshes", []):
        mp, mn_, ms, mi, mu, mt = [], [], [], [], [], []
        section = 0
        vbase = 0
        for prim in mesh.get("primitives", []):
            if "KHR_draco_mesh_compression" in prim.get("extensions", {}):
                raise GlbError("Draco-compressed meshes are not supported")
            if prim.get("mode", 4) != 4 or "indices" not in prim:
                continue
            ind = accessor(gl, binchunk, prim["indices"])
            if gl["accessors"][prim["indices"]]["componentType"] not in (5123, 5124, 5125):
                raise GlbError("index type other than 16/32-bit")
            if ind.shape[0] == 0:
                continue
            attrs = prim.get("attributes", {})
            p = accessor(gl, binchunk, attrs["POSITION"]).astype(np.float32)[:, :3]
            ind = ind.reshape(-1).astype(np.int64)
            if ind.size % 3:
                raise GlbError("triangle list with a partial triangle")
            if ind.size and (ind.min() < 0 or ind.max() >= p.shape[0]):
                raise GlbError("index outside the primitive's vertices")
            n = (accessor(gl, binchunk, attrs["NORMAL"]).astype(np.float32)[:, :3] if "NORMAL" in attrs
                 else _vertex_normals(p, ind))
            uv = (_float_attr(gl, binchunk, attrs["TEXCOORD_0"])[:, :2] if "TEXCOORD_0" in attrs
                  else np.zeros((p.shape[0], 2), np.float32))
            tg = (_float_attr(gl, binchunk, attrs["TANGENT"])[:, :4] if "TANGENT" in attrs
                  else np.zeros((p.shape[0], 4), np.float32))
            any_uv = any_uv or "TEXCOORD_0" in attrs
            any_tan = any_tan or "TANGENT" in attrs
            mp.append(p); mn_.append(n); mu.append(uv); mt.append(tg)
            ms.append(np.full(p.shape[0], section, np.uint32))
            mi.append((ind + vbase).astype(np.uint32))
            vbase += p.shape[0]
            section += 1
        p = np.concatenate(mp) if mp else np.zeros((0, 3), np.float32)
        n = np.concatenate(mn_) if mn_ else np.zeros((0, 3), np.float32)
        uv_l.append(np.concatenate(mu) if mu else np.zeros((0, 2), np.float32))
        tan_l.append(np.concatenate(mt) if mt else np.zeros((0, 4), np.float32))
        i = np.concatenate(mi) if mi else np.zeros(0, np.uint32)
        pos_l.append(np.concatenate([p, np.ones((p.shape[0], 1), np.float32)], axis=1))
        nrm_l.append(np.concatenate([n, np.zeros((n.shape[0], 1), np.float32)], axis=1))
        slot_l.append(np.concatenate(ms) if ms else np.zeros(0, np.uint32))
        idx_l.append(i)
        mesh_rows.append((ioff, i.size, voff, p.shape[0]))
        local_boxes.append((p.min(axis=0), p.max(axis=0)) if p.shape[0] else None)
        voff += p.shape[0]
        ioff += i.size
    if not mesh_rows:
        raise GlbError("no triangle meshes")
    # environment (EnvironmentSetting::Reset and the scene's extras)
    st = camera.Settings(has_sky=True, sky_intensity=100.0, has_sun=False, sun_intensity=500.0)
    sky_rotation, sun_rotation, sky_idx = 0.0, 0.5, 0
    scene_idx = gl.get("scene", 0)
    root = gl["scenes"][scene_idx] if gl.get("scenes") else {"nodes": list(range(len(gl.get("nodes", []))))}
    ex = root.get("extras", {})
    if "SkyIdx" in ex or "SkyIntensity" in ex or "SkyRotation" in ex:
        st.has_sky = True
    if "SkyIntensity" in ex:
        st.sky_intensity = float(ex["SkyIntensity"])
    if "SkyRotation" in ex:
        sky_rotation = float(ex["SkyRotation"])
    if "SkyIdx" in ex:
        sky_idx = int(ex["SkyIdx"])
    if "SunIntensity" in ex:
        st.has_sun = True
        st.sun_intensity = float(ex["SunIntensity"])
    if "WithSun" in ex:
        st.has_sun = int(ex["WithSun"]) != 0
    if "SunRotation" in ex:
        sun_rotation = float(ex["SunRotation"])
    if "NoSky" in ex:
        st.has_sky = False
    sd = np.array([math.sin(sun_rotation * math.pi), 0.75, math.cos(sun_rotation * math.pi)], np.float32)
    st.sun_direction = tuple((sd / np.linalg.norm(sd)).tolist())
    # nodes, depth first from the scene's roots
    nodes = gl.get("nodes", [])
    insts, names, cams, lights = [], [], [], []
    counter = [0]

    def visit(ni, parent_world, depth):
        if depth > 256:
            raise GlbError("node hierarchy deeper than 256 (or cyclic)")
        node = nodes[ni]
        local = local_transform(node)
        world = parent_world @ local
        node_id = counter[0]
        counter[0] += 1
        primary = 0
        if "mesh" in node:
            prims = gl["meshes"][node["mesh"]].get("primitives", [])
            if len(prims) > 16:
                raise GlbError("a mesh with more than 16 primitives")
            mids = [max(0, int(p.get("material", -1))) for p in prims]
            if prims:
                primary = int(prims[-1].get("material", -1))
            mids = [m if m < len(mats) else 0 for m in mids]
            w12 = world[:3, :].reshape(-1)
            insts.append(scenes.make_instance(node["mesh"], w12, mids, instance_id=node_id))
            names.append(node.get("name", ""))
        elif "camera" in node:
            eye = local @ np.array([0.0, 0.0, 0.0, 1.0])
            fwd = local @ np.array([0.0, 0.0, -1.0, 0.0])
            cams.append(camera.Camera(eye=eye[:3], center=eye[:3] + fwd[:3], fov_deg=40.0))
        if "arealight" in node.get("extras", {}):
            p0 = (local @ np.array([-1.0, 0.0, -1.0, 1.0]))[:3]
            p1 = (local @ np.array([-1.0, 0.0, 1.0, 1.0]))[:3]
            p3 = (local @ np.array([1.0, 0.0, -1.0, 1.0]))[:3]
            d = local[:3, :3] @ np.array([0.0, 1.0, 0.0])
            lt = np.zeros((), abi.LIGHT_DTYPE)
            lt["p0"] = list(p0) + [1.0]
            lt["p1"] = list(p1) + [1.0]
            lt["p3"] = list(p3) + [1.0]
            lt["normal_area"] = list(d / (np.linalg.norm(d) or 1.0)) + [
                float(np.linalg.norm(np.cross(p1 - p0, p3 - p0)) / 2.0)]
            lt["light_mat_idx"] = max(0, primary)
            lights.append(lt)
        for c in node.get("children", []):
            visit(c, world, depth + 1)

    for ni in root.get("nodes", []):
        visit(ni, np.eye(4), 0)
    if not insts:
        raise GlbError("no mesh nodes")
    if not cams:
        boxes = [b for b in local_boxes if b is not None]
        lo = np.min([b[0] for b in boxes], axis=0).astype(np.float64)
        hi = np.max([b[1] for b in boxes], axis=0).astype(np.float64)
        c = (hi - lo) * 0.5 + lo
        cams.append(camera.Camera(eye=(c[0], c[1], c[2] + np.linalg.norm(hi - lo)), center=c, fov_deg=40.0))
    st.sky_color = (1.0, 1.0, 1.0, 1.0)
    st.sky_texture = sky_idx
    st.sky_rotation = sky_rotation
    sc = abi.SceneArrays(np.concatenate(pos_l), np.concatenate(nrm_l), np.concatenate(slot_l),
                         np.concatenate(idx_l), np.array(mesh_rows, dtype=abi.MESH_DTYPE),
                         np.array(mats, dtype=abi.MATERIAL_DTYPE), np.array(insts, dtype=abi.INSTANCE_DTYPE),
                         lights=np.array(lights, dtype=abi.LIGHT_DTYPE) if lights else None, name="glb",
                         texcoords=np.concatenate(uv_l) if any_uv else None,
                         tangents=np.concatenate(tan_l) if any_tan else None, textures=textures)
    info = {"instance_names": names, "cameras": cams, "lights": len(lights), "sky_rotation": sky_rotation,
            "sky_index": sky_idx, "nodes": counter[0], "textures": sorted(textures),
            "textures_not_decoded": tex_skipped}
    return sc, cams[0], st, info
