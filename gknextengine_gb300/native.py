"""ctypes binding of libgkrt.so (the C ABI of include/gkrt.h).

The product path is this library and nothing else: if the shared object is missing or
fails to load, every call raises. There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libgkrt.so")

_lib = None


class GkrtError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{abi.STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str | None = None):
    """Load libgkrt.so (or the library the environment variable GKRT_LIBRARY names, e.g. the
    bounds-checked libgkrt_checked.so); raises if it is absent (build it with
    gknextengine_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or os.environ.get("GKRT_LIBRARY") or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"libgkrt.so not found at {p}: run __graft_entry__.build() first")
    L = C.CDLL(p)
    vp = C.c_void_p
    L.gkrt_abi_version.restype = C.c_int
    L.gkrt_context_create.argtypes = [C.POINTER(abi.GkrtDeviceDesc), C.POINTER(vp)]
    L.gkrt_context_destroy.argtypes = [vp]
    L.gkrt_last_error_message.restype = C.c_char_p
    L.gkrt_last_error_message.argtypes = [vp]
    L.gkrt_resize.argtypes = [vp, C.c_uint32, C.c_uint32]
    L.gkrt_scene_upload.argtypes = [vp, C.POINTER(abi.GkrtSceneDesc)]
    L.gkrt_scene_update_instances.argtypes = [vp, vp, C.c_uint32, vp]
    L.gkrt_scene_refit_instances.argtypes = [vp, vp, C.c_uint32, vp]
    L.gkrt_scene_update_instances_auto.argtypes = [vp, vp, C.c_uint32, C.c_float, vp]
    L.gkrt_build_bvh.argtypes = [vp, C.c_uint32, vp]
    for n in ("gkrt_trace_pass", "gkrt_reproject_pass", "gkrt_denoise_pass", "gkrt_render_frame"):
        getattr(L, n).argtypes = [vp, C.POINTER(abi.GkrtFrameConstants), vp]
    L.gkrt_end_frame.argtypes = [vp, vp]
    L.gkrt_get_image.argtypes = [vp, C.c_int, C.POINTER(abi.GkrtImageView)]
    L.gkrt_copy_image_to_host.argtypes = [vp, C.c_int, vp, C.c_size_t, vp]
    L.gkrt_copy_image_to_host_async.argtypes = [vp, C.c_int, vp, C.c_size_t, vp]
    L.gkrt_upload_image.argtypes = [vp, C.c_int, vp, C.c_size_t, vp]
    L.gkrt_trace_rays.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, vp]
    L.gkrt_texture_upload.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.c_size_t]
    L.gkrt_trace_rays_noalloc.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, vp]
    L.gkrt_get_stats.argtypes = [vp, C.POINTER(abi.GkrtStats)]
    L.gkrt_get_pass_times.argtypes = [vp, C.POINTER(abi.GkrtPassTimes)]
    L.gkrt_output_resize.argtypes = [vp, C.c_uint32, C.c_uint32]
    L.gkrt_output_pass.argtypes = [vp, C.POINTER(abi.GkrtOutputDesc), vp]
    L.gkrt_get_output.argtypes = [vp, C.POINTER(abi.GkrtImageView)]
    L.gkrt_copy_output_to_host.argtypes = [vp, vp, C.c_size_t, vp]
    L.gkrt_screenshot.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.c_size_t, vp]
    L.gkrt_probe_voxelize.argtypes = [vp, vp]
    L.gkrt_probe_bake.argtypes = [vp, C.POINTER(abi.GkrtFrameConstants), C.c_uint32, C.c_uint32, vp]
    L.gkrt_probe_download.argtypes = [vp, vp, vp]
    L.gkrt_synchronize.argtypes = [vp, vp]
    L.gkrt_affine_inverse.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float)]
    L.gkrt_conv3x3_bf16.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp, C.c_uint32, vp,
                                    C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp]
    L.gkrt_conv3x3_bf16_fused.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp, C.c_uint32,
                                          vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, C.c_uint32, C.c_uint32, vp,
                                          C.c_uint32, C.c_uint32, vp]
    L.gkrt_conv3x3_wgrad_bf16.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp]
    L.gkrt_unet_init.argtypes = [vp, C.c_uint64]
    L.gkrt_unet_param_count.argtypes = [vp, C.POINTER(C.c_uint32)]
    L.gkrt_unet_get_params.argtypes = [vp, vp, vp]
    L.gkrt_unet_set_params.argtypes = [vp, vp]
    L.gkrt_unet_get_state.argtypes = [vp, vp, vp, C.POINTER(C.c_uint64)]
    L.gkrt_unet_set_state.argtypes = [vp, vp, vp, C.c_uint64]
    L.gkrt_unet_forward.argtypes = [vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, vp, vp, vp]
    L.gkrt_unet_backward.argtypes = [vp, vp, vp]
    L.gkrt_unet_zero_grad.argtypes = [vp, vp]
    L.gkrt_unet_train_step.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, C.c_uint32, C.c_float,
                                       C.POINTER(C.c_double), vp]
    L.gkrt_set_material_params.argtypes = [vp, vp, vp, C.c_uint32, C.c_uint32, vp]
    L.gkrt_adjoint_forward.argtypes = [vp, C.POINTER(abi.GkrtFrameConstants), C.c_uint32, vp, vp, vp]
    L.gkrt_adjoint_backward.argtypes = [vp, C.POINTER(abi.GkrtFrameConstants), C.c_uint32, vp, vp, vp, vp, vp]
    if L.gkrt_abi_version() != 2:
        raise RuntimeError("libgkrt ABI version mismatch")
    _lib = L
    return L


# every function include/gkrt.h declares (checked by the CPU test suite)
EXPORTED = [
    "gkrt_context_create", "gkrt_context_destroy", "gkrt_last_error_message", "gkrt_abi_version",
    "gkrt_resize", "gkrt_scene_upload", "gkrt_scene_update_instances", "gkrt_scene_refit_instances",
    "gkrt_scene_update_instances_auto",
    "gkrt_build_bvh",
    "gkrt_trace_pass", "gkrt_reproject_pass", "gkrt_denoise_pass", "gkrt_end_frame", "gkrt_render_frame",
    "gkrt_output_resize", "gkrt_output_pass", "gkrt_get_output", "gkrt_copy_output_to_host",
    "gkrt_screenshot",
    "gkrt_get_image", "gkrt_copy_image_to_host", "gkrt_copy_image_to_host_async", "gkrt_upload_image", "gkrt_trace_rays", "gkrt_trace_rays_noalloc",
    "gkrt_texture_upload",
    "gkrt_get_stats", "gkrt_get_pass_times", "gkrt_probe_voxelize", "gkrt_probe_bake", "gkrt_probe_download",
    "gkrt_synchronize", "gkrt_affine_inverse",
    "gkrt_set_material_params", "gkrt_adjoint_forward", "gkrt_adjoint_backward", "gkrt_conv3x3_bf16", "gkrt_conv3x3_bf16_fused",
    "gkrt_conv3x3_wgrad_bf16",
    "gkrt_unet_init", "gkrt_unet_param_count", "gkrt_unet_get_params", "gkrt_unet_set_params", "gkrt_unet_get_state", "gkrt_unet_set_state", "gkrt_unet_forward",
    "gkrt_unet_backward", "gkrt_unet_zero_grad", "gkrt_unet_train_step",
]
