"""ctypes mirror of include/gkrt.h.

The structs and constants here are the Python view of the C ABI that a host engine binds
(the reference's renderer-pass inputs: GPUScene buffers, UniformBufferObject, bindless
images; see include/gkrt.h for the file:line citations). numpy structured dtypes with the
same byte layout are provided for the array-shaped inputs (instances, materials, lights)
so scenes can be built vectorised and passed without copies.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

GKRT_OK = 0
GKRT_ERR_INVALID_ARG = 1
GKRT_ERR_OOM = 2
GKRT_ERR_CUDA = 3
GKRT_ERR_TIMEOUT = 4
GKRT_ERR_DEVICE_LIMIT = 5
GKRT_ERR_UNSUPPORTED = 6
GKRT_ERR_STATE = 7
GKRT_ERR_NO_DEVICE = 8

STATUS_NAMES = {
    0: "GKRT_OK", 1: "GKRT_ERR_INVALID_ARG", 2: "GKRT_ERR_OOM", 3: "GKRT_ERR_CUDA",
    4: "GKRT_ERR_TIMEOUT", 5: "GKRT_ERR_DEVICE_LIMIT", 6: "GKRT_ERR_UNSUPPORTED",
    7: "GKRT_ERR_STATE", 8: "GKRT_ERR_NO_DEVICE",
}

MAT_LAMBERTIAN, MAT_METALLIC, MAT_DIELECTRIC, MAT_ISOTROPIC, MAT_DIFFUSE_LIGHT, MAT_MIXTURE = range(6)

DENOISE_JBF = 0
DENOISE_ATROUS = 1
DENOISE_UNET = 2
NEE_REFERENCE = 0
NEE_EMISSIVE = 1
FRAME_PRIMARY_IDS = 1

IMG_SINGLE_DIFFUSE = 0
IMG_SINGLE_SPECULAR = 1
IMG_ALBEDO = 2
IMG_NORMAL = 3
IMG_OBJECT_ID = 4
IMG_OBJECT_ID_PREV = 5
IMG_MOTION = 6
IMG_PREV_DEPTH = 7
IMG_MOTION_MOMENT = 8
IMG_ACCUM_DIFFUSE = 9
IMG_ACCUM_SPECULAR = 10
IMG_ACCUM_ALBEDO = 11
IMG_PREV_DIFFUSE = 12
IMG_PREV_SPECULAR = 13
IMG_PREV_ALBEDO = 14
IMG_DENOISED = 15
IMG_DENOISED_LINEAR = 16
IMG_HIT_INST = 17
IMG_HIT_PRIM = 18
IMG_COUNT = 19

FMT_F32X4, FMT_F32X2, FMT_F32, FMT_U32, FMT_BGRA8 = range(5)
OUTPUT_RESOLVE, OUTPUT_FSR = 0, 1

# (numpy dtype, channels) of each image, as the library allocates them
IMAGE_FORMATS = {
    IMG_SINGLE_DIFFUSE: (np.float32, 4), IMG_SINGLE_SPECULAR: (np.float32, 4),
    IMG_ALBEDO: (np.float32, 4), IMG_NORMAL: (np.float32, 4),
    IMG_OBJECT_ID: (np.uint32, 1), IMG_OBJECT_ID_PREV: (np.uint32, 1),
    IMG_MOTION: (np.float32, 2), IMG_PREV_DEPTH: (np.float32, 1),
    IMG_MOTION_MOMENT: (np.uint32, 1),
    IMG_ACCUM_DIFFUSE: (np.float32, 4), IMG_ACCUM_SPECULAR: (np.float32, 4),
    IMG_ACCUM_ALBEDO: (np.float32, 4), IMG_PREV_DIFFUSE: (np.float32, 4),
    IMG_PREV_SPECULAR: (np.float32, 4), IMG_PREV_ALBEDO: (np.float32, 4),
    IMG_DENOISED: (np.float32, 4), IMG_DENOISED_LINEAR: (np.float32, 4),
    IMG_HIT_INST: (np.uint32, 1), IMG_HIT_PRIM: (np.uint32, 1),
}

TRACE_CLOSEST = 0
TRACE_ANY = 1
BUILD_BLAS, BUILD_TLAS, BUILD_ALL = 1, 2, 3
BUILD_ON_HOST = 4

MATERIAL_DTYPE = np.dtype([
    ("diffuse", np.float32, 4), ("diffuse_texture_id", np.int32), ("mra_texture_id", np.int32),
    ("normal_texture_id", np.int32), ("fuzziness", np.float32), ("refraction_index", np.float32),
    ("material_model", np.uint32), ("metalness", np.float32), ("refraction_index2", np.float32),
    ("normal_texture_scale", np.float32), ("reserved", np.float32, 3),
])
assert MATERIAL_DTYPE.itemsize == 64

LIGHT_DTYPE = np.dtype([
    ("p0", np.float32, 4), ("p1", np.float32, 4), ("p3", np.float32, 4),
    ("normal_area", np.float32, 4), ("light_mat_idx", np.uint32), ("reserved", np.uint32, 3),
])
assert LIGHT_DTYPE.itemsize == 80

MESH_DTYPE = np.dtype([("index_offset", np.uint32), ("index_count", np.uint32),
                       ("vertex_offset", np.uint32), ("vertex_count", np.uint32)])

INSTANCE_DTYPE = np.dtype([
    ("instance_id", np.uint32), ("mesh_id", np.uint32), ("visible", np.uint32), ("reserved", np.uint32),
    ("world", np.float32, 12), ("world_inv", np.float32, 12), ("combined_prev", np.float32, 12),
    ("mat_id", np.uint32, 16),
])
assert INSTANCE_DTYPE.itemsize == 224

RAY_DTYPE = np.dtype([("origin", np.float32, 3), ("tmin", np.float32), ("dir", np.float32, 3),
                      ("tmax", np.float32)])
HIT_DTYPE = np.dtype([("t", np.float32), ("b1", np.float32), ("b2", np.float32), ("inst", np.uint32),
                      ("prim", np.uint32), ("pad", np.uint32, 3)])
assert RAY_DTYPE.itemsize == 32 and HIT_DTYPE.itemsize == 32


def _p(t):
    return C.POINTER(t)


class GkrtSceneDesc(C.Structure):
    _fields_ = [
        ("positions", _p(C.c_float)), ("normals", _p(C.c_float)), ("material_slots", _p(C.c_uint32)),
        ("vertex_count", C.c_uint32), ("indices", _p(C.c_uint32)), ("index_count", C.c_uint32),
        ("meshes", C.c_void_p), ("mesh_count", C.c_uint32), ("materials", C.c_void_p),
        ("material_count", C.c_uint32), ("instances", C.c_void_p), ("instance_count", C.c_uint32),
        ("lights", C.c_void_p), ("light_count", C.c_uint32), ("probe_cubes", _p(C.c_uint32)),
        ("probe_voxels", _p(C.c_uint32)), ("texcoords", _p(C.c_float)), ("tangents", _p(C.c_float)),
    ]


class GkrtFrameConstants(C.Structure):
    _fields_ = [
        ("model_view", C.c_float * 16), ("projection", C.c_float * 16),
        ("model_view_inverse", C.c_float * 16), ("projection_inverse", C.c_float * 16),
        ("view_projection", C.c_float * 16), ("prev_view_projection", C.c_float * 16),
        ("view_projection_unjit", C.c_float * 16), ("prev_view_projection_unjit", C.c_float * 16),
        ("sun_direction", C.c_float * 4), ("sun_color", C.c_float * 4), ("sky_color", C.c_float * 4),
        ("aperture", C.c_float), ("focus_distance", C.c_float), ("paper_white_nit", C.c_float),
        ("sky_intensity", C.c_float),
        ("total_frames", C.c_uint32), ("number_of_samples", C.c_uint32), ("number_of_bounces", C.c_uint32),
        ("max_number_of_bounces", C.c_uint32), ("temporal_frames", C.c_uint32), ("has_sky", C.c_uint32),
        ("has_sun", C.c_uint32), ("taa", C.c_uint32), ("fast_gather", C.c_uint32),
        ("progressive_render", C.c_uint32), ("bf_size", C.c_uint32), ("hdr", C.c_uint32),
        ("bf_sigma", C.c_float), ("bf_sigma_lum", C.c_float), ("bf_sigma_normal", C.c_float),
        ("denoiser", C.c_uint32), ("nee_mode", C.c_uint32), ("flags", C.c_uint32),
        ("sky_index", C.c_uint32), ("sky_rotation", C.c_float),
    ]


class GkrtImageView(C.Structure):
    _fields_ = [("device_ptr", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32),
                ("pitch_bytes", C.c_uint32), ("format", C.c_uint32)]


DEVICE_PASS_TIMERS = 1


class GkrtPassTimes(C.Structure):
    _fields_ = [("rt_pass_ms", C.c_float), ("reproject_pass_ms", C.c_float), ("compose_pass_ms", C.c_float),
                ("copy_pass_ms", C.c_float), ("tlas_update_ms", C.c_float), ("reserved", C.c_float * 3)]


class GkrtOutputDesc(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("offset_x", C.c_int32), ("offset_y", C.c_int32), ("width", C.c_uint32),
                ("height", C.c_uint32), ("source_image", C.c_uint32)]


class GkrtDeviceDesc(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32), ("watchdog_ms", C.c_uint32),
                ("reserved", C.c_uint32)]


class GkrtStats(C.Structure):
    _fields_ = [("rays_traced", C.c_uint64), ("exact_fallbacks", C.c_uint64), ("exact_retraces", C.c_uint64),
                ("node_visits", C.c_uint64), ("triangle_tests", C.c_uint64), ("rays_total", C.c_uint64),
                ("device_error", C.c_uint32), ("bvh_nodes", C.c_uint32), ("bvh_leaf_tris", C.c_uint32),
                ("tlas_nodes", C.c_uint32), ("emitters", C.c_uint32), ("build_launches", C.c_uint32),
                ("wide_nodes", C.c_uint32), ("wide_depth", C.c_uint32), ("tlas_refits", C.c_uint32),
                ("hit_fetches", C.c_uint32), ("tlas_rebuilds", C.c_uint32), ("pad", C.c_uint32)]


def fptr(a: np.ndarray, ctype=C.c_float):
    return a.ctypes.data_as(_p(ctype)) if a is not None else None


class SceneArrays:
    """Host-side scene arrays in the exact layouts GkrtSceneDesc points at, plus the scene's
    textures: {texture id: (format TEX_*, texels (h, w, 4) uint8 or float32)}."""

    def __init__(self, positions, normals, material_slots, indices, meshes, materials, instances,
                 lights=None, probe_cubes=None, probe_voxels=None, name="scene", texcoords=None, tangents=None,
                 textures=None):
        self.positions = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 4)
        self.normals = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 4)
        self.material_slots = np.ascontiguousarray(material_slots, dtype=np.uint32).reshape(-1)
        self.indices = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1)
        self.meshes = np.ascontiguousarray(meshes, dtype=MESH_DTYPE)
        self.materials = np.ascontiguousarray(materials, dtype=MATERIAL_DTYPE)
        self.instances = np.ascontiguousarray(instances, dtype=INSTANCE_DTYPE)
        self.lights = np.ascontiguousarray(lights if lights is not None else np.zeros(0, LIGHT_DTYPE),
                                           dtype=LIGHT_DTYPE)
        self.probe_cubes = None if probe_cubes is None else np.ascontiguousarray(probe_cubes, dtype=np.uint32)
        self.probe_voxels = None if probe_voxels is None else np.ascontiguousarray(probe_voxels, dtype=np.uint32)
        self.texcoords = None if texcoords is None else np.ascontiguousarray(texcoords, dtype=np.float32).reshape(-1, 2)
        self.tangents = None if tangents is None else np.ascontiguousarray(tangents, dtype=np.float32).reshape(-1, 4)
        self.textures = dict(textures or {})
        self.name = name

    @property
    def triangle_count(self) -> int:
        tris = self.meshes["index_count"].astype(np.int64) // 3
        vis = self.instances["visible"] != 0
        return int(tris[self.instances["mesh_id"][vis]].sum())

    def desc(self) -> GkrtSceneDesc:
        d = GkrtSceneDesc()
        d.positions = fptr(self.positions)
        d.normals = fptr(self.normals)
        d.material_slots = fptr(self.material_slots, C.c_uint32)
        d.vertex_count = self.positions.shape[0]
        d.indices = fptr(self.indices, C.c_uint32)
        d.index_count = self.indices.shape[0]
        d.meshes = self.meshes.ctypes.data
        d.mesh_count = self.meshes.shape[0]
        d.materials = self.materials.ctypes.data
        d.material_count = self.materials.shape[0]
        d.instances = self.instances.ctypes.data
        d.instance_count = self.instances.shape[0]
        d.lights = self.lights.ctypes.data if self.lights.shape[0] else None
        d.light_count = self.lights.shape[0]
        d.probe_cubes = fptr(self.probe_cubes, C.c_uint32) if self.probe_cubes is not None else None
        d.probe_voxels = fptr(self.probe_voxels, C.c_uint32) if self.probe_voxels is not None else None
        d.texcoords = fptr(self.texcoords) if self.texcoords is not None else None
        d.tangents = fptr(self.tangents) if self.tangents is not None else None
        return d


TEX_RGBA8_UNORM, TEX_RGBA8_SRGB, TEX_RGBA32F = 0, 1, 2
MAX_TEXTURES = 4096
FRAME_SKY_TEXTURE = 2


def texel_buffer(fmt: int, texels: np.ndarray) -> np.ndarray:
    """Texels (h, w, 4) as the contiguous buffer gkrt_texture_upload takes for `fmt`."""
    dt = np.float32 if fmt == TEX_RGBA32F else np.uint8
    t = np.ascontiguousarray(texels, dtype=dt)
    if t.ndim != 3 or t.shape[2] != 4:
        raise ValueError("texels must be (height, width, 4)")
    return t
