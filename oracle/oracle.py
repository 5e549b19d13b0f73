"""Python front end of the CPU oracle (test infrastructure only).

The oracle is the checker of the GB300 kernels: a C++ restatement of the reference's
path-tracing pass (gk_oracle.cpp, with its file:line citations) and the FP64 closest-hit
definition (oracle_isect.h). Only the tests, __graft_entry__.smoke() and the CPU-baseline
leg of bench.py use it; the product package never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

from gknextengine_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libgkoracle.so")
SOURCES = ["gk_oracle.cpp", "oracle_math.h", "oracle_isect.h", os.path.join("..", "include", "gkrt.h")]


def build(force: bool = False) -> str:
    """Compile the oracle with contraction off (see oracle_math.h)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(s) for s in srcs)):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           os.path.join(HERE, "gk_oracle.cpp"), "-o", LIB_PATH + ".tmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd.insert(1, "-mfma")
    subprocess.check_call(cmd)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.gko_scene_create.restype = C.c_void_p
        L.gko_scene_create.argtypes = [C.POINTER(abi.GkrtSceneDesc)]
        L.gko_scene_destroy.argtypes = [C.c_void_p]
        L.gko_trace_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_int, C.c_int]
        L.gko_adjoint.restype = C.c_uint64
        L.gko_adjoint.argtypes = [C.c_void_p, C.POINTER(abi.GkrtFrameConstants), C.c_int, C.c_int, C.c_int, C.c_int,
                                  C.c_int, C.c_int, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_int]
        L.gko_trace_pass.restype = C.c_uint64
        L.gko_trace_pass.argtypes = [C.c_void_p, C.POINTER(abi.GkrtFrameConstants), C.c_int, C.c_int,
                                     C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int]
        L.gko_reproject_pass.argtypes = [C.POINTER(abi.GkrtFrameConstants), C.c_int, C.c_int,
                                         C.POINTER(C.c_void_p), C.c_int]
        L.gko_denoise_pass.argtypes = [C.POINTER(abi.GkrtFrameConstants), C.c_int, C.c_int,
                                       C.POINTER(C.c_void_p), C.c_int]
        L.gko_uint_to_float.restype = C.c_float
        L.gko_uint_to_float.argtypes = [C.c_uint32]
        L.gko_sincos_2pi.argtypes = [C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]
        L.gko_schlick.restype = C.c_float
        L.gko_schlick.argtypes = [C.c_float, C.c_float]
        L.gko_gt_tonemap.restype = C.c_float
        L.gko_gt_tonemap.argtypes = [C.c_float]
        L.gko_set_fast.argtypes = [C.c_int]
        for n in ("gko_output_resolve", "gko_output_fsr"):
            getattr(L, n).argtypes = [C.c_void_p] + [C.c_int] * 3 + [C.c_void_p] + [C.c_int] * 6
        L.gko_screenshot.argtypes = [C.c_void_p] + [C.c_int] * 5 + [C.c_void_p]
        L.gko_probe_voxelize.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_int]
        L.gko_probe_bake.argtypes = [C.c_void_p, C.POINTER(abi.GkrtFrameConstants), C.c_uint32, C.c_uint32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.gko_texture_upload.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p]
        L.gko_atan2.argtypes = [C.c_float, C.c_float]
        L.gko_atan2.restype = C.c_float
        L.gko_acos.argtypes = [C.c_float]
        L.gko_acos.restype = C.c_float
        L.gko_tex_sample.argtypes = [C.c_void_p, C.c_int, C.c_float, C.c_float, C.c_void_p]
        L.gko_sky_dir.argtypes = [C.c_void_p, C.POINTER(abi.GkrtFrameConstants), C.c_void_p, C.c_void_p]
        L.gko_sky_rough.argtypes = [C.c_void_p, C.POINTER(abi.GkrtFrameConstants), C.c_void_p, C.c_void_p]
        L.gko_texture_sh.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p]
        L.gko_texture_sh.restype = C.c_int
        L.gko_exact_tri.restype = C.c_int
        L.gko_fp32_tri.restype = C.c_int
        _lib = L
    return _lib


def new_images(width: int, height: int) -> dict:
    """Host images in the product's layouts (abi.IMAGE_FORMATS), zero-initialised."""
    out = {}
    for k, (dt, ch) in abi.IMAGE_FORMATS.items():
        shape = (height, width) if ch == 1 else (height, width, ch)
        out[k] = np.zeros(shape, dt)
    return out


def _ptrs(images: dict):
    arr = (C.c_void_p * abi.IMG_COUNT)()
    for k in range(abi.IMG_COUNT):
        a = images.get(k)
        arr[k] = a.ctypes.data if a is not None else None
    return arr


class OracleScene:
    def __init__(self, scene: abi.SceneArrays):
        self.scene = scene
        self._desc = scene.desc()
        self.h = lib().gko_scene_create(C.byref(self._desc))
        for tid, (fmt, texels) in sorted(getattr(scene, "textures", {}).items()):
            t = abi.texel_buffer(fmt, texels)
            if lib().gko_texture_upload(self.h, tid, t.shape[1], t.shape[0], fmt, t.ctypes.data) != 0:
                raise ValueError(f"texture {tid} rejected by the oracle")

    def close(self):
        if self.h:
            lib().gko_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tex_sample(self, texture_id: int, u: float, v: float) -> np.ndarray:
        out = np.zeros(4, np.float32)
        lib().gko_tex_sample(self.h, texture_id, C.c_float(u), C.c_float(v), out.ctypes.data)
        return out

    def sky_dir(self, fc, d) -> np.ndarray:
        dd = np.ascontiguousarray(d, np.float32)
        out = np.zeros(4, np.float32)
        lib().gko_sky_dir(self.h, C.byref(fc), dd.ctypes.data, out.ctypes.data)
        return out

    def sky_rough(self, fc, d) -> np.ndarray:
        """The probe bake's sky radiance in direction d (SampleIBLRough)."""
        dd = np.ascontiguousarray(d, np.float32)
        out = np.zeros(4, np.float32)
        lib().gko_sky_rough(self.h, C.byref(fc), dd.ctypes.data, out.ctypes.data)
        return out

    def texture_sh(self, texture_id: int) -> np.ndarray:
        """The spherical-harmonic projection of a texture, (3, 9): red, green, blue terms."""
        out = np.zeros(27, np.float32)
        if lib().gko_texture_sh(self.h, texture_id, out.ctypes.data) != 0:
            raise ValueError(f"no texture {texture_id}")
        return out.reshape(3, 9)

    def trace_rays(self, rays: np.ndarray, mode: int = abi.TRACE_CLOSEST, brute: bool = False,
                   threads: int = 0) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=abi.RAY_DTYPE)
        hits = np.zeros(rays.shape[0], abi.HIT_DTYPE)
        lib().gko_trace_rays(self.h, rays.ctypes.data, hits.ctypes.data, rays.shape[0], mode, int(brute), threads)
        return hits

    def probe_voxelize(self, first: int, count: int, threads: int = 0) -> np.ndarray:
        """VoxelData words (count, 4) of probes [first, first + count)."""
        out = np.zeros((count, 4), np.uint32)
        lib().gko_probe_voxelize(self.h, first, count, out.ctypes.data, threads)
        return out

    def probe_bake(self, fc, first: int, count: int, cubes_prev: np.ndarray, voxels: np.ndarray, threads: int = 0):
        """One bake step of probes [first, first + count) from whole-grid arrays; returns
        (cube words (count, 14), ages (count,))."""
        cubes_prev = np.ascontiguousarray(cubes_prev, np.uint32)
        voxels = np.ascontiguousarray(voxels, np.uint32)
        out = np.zeros((count, 14), np.uint32)
        ages = np.zeros(count, np.uint32)
        lib().gko_probe_bake(self.h, C.byref(fc), first, count, cubes_prev.ctypes.data, voxels.ctypes.data,
                             out.ctypes.data, ages.ctypes.data, threads)
        return out, ages

    def trace_pass(self, fc, width, height, images, y0=0, y1=0, threads=0) -> int:
        return int(lib().gko_trace_pass(self.h, C.byref(fc), width, height, _ptrs(images), y0, y1, threads))

    def adjoint(self, fc, width, height, spp, sample_rough=None, dimage=None, window=None, threads=0):
        """The differentiable estimator over a pixel window (x0, y0, x1, y1): the composed image
        (dense H x W x 4, zero outside the window) and, when dimage (H x W x 4) is given, the
        FP64 gradient sums (albedo (n, 3), roughness (n,))."""
        x0, y0, x1, y1 = window or (0, 0, width, height)
        nm = self.scene.materials.shape[0]
        img = np.zeros((height, width, 4), np.float32)
        ga = np.zeros((nm, 3), np.float64)
        gr = np.zeros(nm, np.float64)
        sr = None if sample_rough is None else np.ascontiguousarray(sample_rough, np.float32)
        di = None if dimage is None else np.ascontiguousarray(dimage, np.float32)
        lib().gko_adjoint(self.h, C.byref(fc), width, height, x0, y0, x1, y1, spp,
                          sr.ctypes.data if sr is not None else None, img.ctypes.data,
                          di.ctypes.data if di is not None else None, ga.ctypes.data, gr.ctypes.data, threads)
        return img, ga, gr


def reproject_pass(fc, width, height, images, threads=0):
    lib().gko_reproject_pass(C.byref(fc), width, height, _ptrs(images), threads)


def denoise_pass(fc, width, height, images, threads=0):
    lib().gko_denoise_pass(C.byref(fc), width, height, _ptrs(images), threads)


def _output(fn, src, out_w, out_h, a, b, c, d, out=None):
    src = np.ascontiguousarray(src, np.float32)
    H, W = src.shape[:2]
    if out is None:
        out = np.zeros((out_h, out_w), np.uint32)
    assert out.dtype == np.uint32 and out.shape == (out_h, out_w) and out.flags["C_CONTIGUOUS"]
    fn(src.ctypes.data, W, H, W, out.ctypes.data, out_w, out_h, a, b, c, d)
    return out


def output_resolve(src, out_w, out_h, offset=(0, 0), size=None, out=None):
    """The resolve pass (linear blit) of an (H, W, 4) float image onto the rectangle offset +
    size of an out_w x out_h presentation image of BGRA8 words (uint32 (out_h, out_w))."""
    w, h = size if size is not None else (out_w, out_h)
    return _output(lib().gko_output_resolve, src, out_w, out_h, offset[0], offset[1], w, h, out)


def output_fsr(src, out_w, out_h, offset=(0, 0), size=None, out=None):
    """Process.UpScaleFSR.comp.slang with push constants offset and size (output_w, output_h)."""
    w, h = size if size is not None else (out_w, out_h)
    return _output(lib().gko_output_fsr, src, out_w, out_h, offset[0], offset[1], w, h, out)


def screenshot(img, x, y, w, h):
    """ScreenShot.cpp's crop of a BGRA8 presentation image as (h, w, 3) bytes R, G, B."""
    img = np.ascontiguousarray(img, np.uint32)
    out = np.empty((h, w, 3), np.uint8)
    lib().gko_screenshot(img.ctypes.data, img.shape[1], x, y, w, h, out.ctypes.data)
    return out


def end_frame(images):
    """History hand-over of the copy pass (PathTracingRenderer.cpp:159-182 and the
    object-id copy, VulkanBaseRenderer.cpp:1136-1152) as the buffer swap the library does."""
    for a, b in ((abi.IMG_ACCUM_DIFFUSE, abi.IMG_PREV_DIFFUSE), (abi.IMG_ACCUM_SPECULAR, abi.IMG_PREV_SPECULAR),
                 (abi.IMG_ACCUM_ALBEDO, abi.IMG_PREV_ALBEDO), (abi.IMG_OBJECT_ID, abi.IMG_OBJECT_ID_PREV)):
        images[a], images[b] = images[b], images[a]


def render_frame(oscene: OracleScene, fc, width, height, images, threads=0) -> int:
    rays = oscene.trace_pass(fc, width, height, images, threads=threads)
    reproject_pass(fc, width, height, images, threads)
    denoise_pass(fc, width, height, images, threads)
    end_frame(images)
    return rays


def pcg4d(v):
    a = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in v])
    lib().gko_pcg4d(a)
    return [int(x) for x in a]


def sincos_2pi(u: float):
    s, c = C.c_float(), C.c_float()
    lib().gko_sincos_2pi(C.c_float(u), C.byref(s), C.byref(c))
    return s.value, c.value


# ---- the reference's own CPU BVH (tinybvh, vendored in gkNextEngine), test use only ----
REF_DIR = os.path.join(HERE, "_ref")
REF_LIB = os.path.join(REF_DIR, "libtinybvh_ref.so")
# The reference tree, read where it lies (present where this library is developed, absent on
# GPU hosts); the environment variable GKNE_REFERENCE_TREE points elsewhere. Pins that need
# it are skipped when it is absent.
REFERENCE_TREE = os.environ.get("GKNE_REFERENCE_TREE", "/root/reference")
REFERENCE_TINYBVH = os.path.join(REFERENCE_TREE, "src", "ThirdParty", "tinybvh")


def build_ref(force: bool = False):
    """Compile ref_tinybvh.cpp against tiny_bvh.h where it lies in the reference tree.
    Returns the library path, or None when the reference tree is not present (the GPU machine)
    or the header does not build on this host."""
    src = os.path.join(HERE, "ref_tinybvh.cpp")
    if not force and os.path.exists(REF_LIB) and os.path.getmtime(REF_LIB) >= os.path.getmtime(src):
        return REF_LIB
    if not os.path.isdir(REFERENCE_TINYBVH):
        return None
    os.makedirs(REF_DIR, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++20", "-fopenmp", "-fPIC", "-shared", "-w", "-I" + REFERENCE_TINYBVH, src,
           "-o", REF_LIB + ".tmp"]
    if platform.machine() in ("x86_64", "AMD64"):
        cmd[1:1] = ["-mavx2", "-mfma"]   # tiny_bvh.h uses SSE4/AVX intrinsics unconditionally on x86
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        return None
    os.replace(REF_LIB + ".tmp", REF_LIB)
    return REF_LIB


_ref = None


def ref_lib():
    """ctypes handle of the tinybvh shim, or None when it is unavailable."""
    global _ref
    if _ref is None:
        p = REF_LIB if os.path.exists(REF_LIB) else build_ref()
        if not p:
            return None
        L = C.CDLL(p)
        L.gkref_closest_double.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.gkref_closest_float.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
        L.gkref_closest_float.restype = C.c_int64
        _ref = L
    return _ref


def ref_closest_double(tri_verts: np.ndarray, origins: np.ndarray, dirs: np.ndarray):
    """tinybvh BVH_Double closest hits: tri_verts (n,3,3) float64; returns (t, prim)."""
    L = ref_lib()
    v = np.ascontiguousarray(tri_verts, np.float64).reshape(-1, 9)
    r = np.ascontiguousarray(np.concatenate([origins, dirs], axis=1), np.float64)
    t = np.zeros(r.shape[0], np.float64)
    p = np.zeros(r.shape[0], np.int64)
    L.gkref_closest_double(v.ctypes.data, v.shape[0], r.ctypes.data, r.shape[0], t.ctypes.data, p.ctypes.data)
    return t, p
