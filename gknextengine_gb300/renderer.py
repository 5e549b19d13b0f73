"""PathTracingRenderer: the host-side mirror of the reference's logic renderer.

The reference drives its path tracer through LogicRendererBase
(src/Rendering/VulkanBaseRenderer.hpp:213-243): OnDeviceSet, CreateSwapChain(extent),
DeleteSwapChain, Render(commandBuffer, imageIndex), BeforeNextFrame; the path-tracing
implementation records "rt pass", "reproject pass", "compose pass" and "copy pass"
(src/Rendering/PathTracing/PathTracingRenderer.cpp:104-218). This class keeps those names
and that order over the C ABI, with CUDA streams in place of command buffers. Errors are
raised as GkrtError, carrying the library's status code and message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi, native


class PathTracingRenderer:
    def __init__(self, device: int = 0, watchdog_ms: int = 0, pass_timers: bool = False):
        self._lib = native.load()
        d = abi.GkrtDeviceDesc()
        d.device = device
        d.watchdog_ms = watchdog_ms
        d.flags = abi.DEVICE_PASS_TIMERS if pass_timers else 0
        h = C.c_void_p()
        rc = self._lib.gkrt_context_create(C.byref(d), C.byref(h))
        if rc != abi.GKRT_OK:
            raise native.GkrtError(rc, "gkrt_context_create failed")
        self._h = h
        self.width = self.height = 0
        self.output_width = self.output_height = 0   # presentation image (output_resize)
        self._scene = None

    # -- helpers ---------------------------------------------------------------------------
    def _check(self, rc: int):
        if rc != abi.GKRT_OK:
            msg = self._lib.gkrt_last_error_message(self._h)
            raise native.GkrtError(rc, msg.decode() if msg else "")

    @staticmethod
    def _stream(stream):
        if stream is None:
            return None
        if isinstance(stream, int):
            return C.c_void_p(stream)
        return C.c_void_p(int(stream.cuda_stream))   # torch.cuda.Stream

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gkrt_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- LogicRendererBase ---------------------------------------------------------------
    def create_swap_chain(self, width: int, height: int):
        """CreateSwapChain(extent): (re)allocates the image set."""
        self._check(self._lib.gkrt_resize(self._h, width, height))
        self.width, self.height = int(width), int(height)

    resize = create_swap_chain

    def load_scene(self, scene: abi.SceneArrays):
        """Scene::RebuildMeshBuffer + RayTraceBaseRenderer::CreateAccelerationStructures."""
        self._scene = scene
        desc = scene.desc()
        self._check(self._lib.gkrt_scene_upload(self._h, C.byref(desc)))
        for tid, (fmt, texels) in sorted(getattr(scene, "textures", {}).items()):
            self.upload_texture(tid, fmt, texels)

    def upload_texture(self, texture_id: int, fmt: int, texels: np.ndarray):
        """Texture `texture_id` of the pool (GlobalTexturePool): texels (h, w, 4) uint8 for the
        RGBA8 formats, float32 for TEX_RGBA32F."""
        t = abi.texel_buffer(fmt, texels)
        self._check(self._lib.gkrt_texture_upload(self._h, texture_id, t.shape[1], t.shape[0], fmt,
                                                  t.ctypes.data, t.nbytes))

    @property
    def material_count(self) -> int:
        return 0 if getattr(self, "_scene", None) is None else int(self._scene.materials.shape[0])

    def update_instances(self, instances: np.ndarray, stream=None):
        """Per-frame NodeProxy upload + TLAS rebuild (Scene::UpdateNodesGpuDriven, AfterUpdateScene)."""
        inst = np.ascontiguousarray(instances, dtype=abi.INSTANCE_DTYPE)
        self._check(self._lib.gkrt_scene_update_instances(self._h, inst.ctypes.data, inst.shape[0],
                                                          self._stream(stream)))

    def refit_instances(self, instances: np.ndarray, stream=None):
        """The same update with the instance level refit in place (topology kept, no host
        synchronisation); rebuilds instead when the set of instances in the tree changes."""
        inst = np.ascontiguousarray(instances, dtype=abi.INSTANCE_DTYPE)
        self._check(self._lib.gkrt_scene_refit_instances(self._h, inst.ctypes.data, inst.shape[0],
                                                         self._stream(stream)))

    def update_instances_auto(self, instances: np.ndarray, growth_limit: float = 1.25, stream=None):
        """The same update, refit while the node visits per ray of the newest finished trace pass
        stay below growth_limit times those right after the last rebuild, else rebuilt."""
        inst = np.ascontiguousarray(instances, dtype=abi.INSTANCE_DTYPE)
        self._check(self._lib.gkrt_scene_update_instances_auto(self._h, inst.ctypes.data, inst.shape[0],
                                                               C.c_float(growth_limit), self._stream(stream)))

    def build_bvh(self, flags: int = abi.BUILD_ALL, stream=None):
        self._check(self._lib.gkrt_build_bvh(self._h, flags, self._stream(stream)))

    def trace_pass(self, fc, stream=None):
        self._check(self._lib.gkrt_trace_pass(self._h, C.byref(fc), self._stream(stream)))

    def reproject_pass(self, fc, stream=None):
        self._check(self._lib.gkrt_reproject_pass(self._h, C.byref(fc), self._stream(stream)))

    def denoise_pass(self, fc, stream=None):
        self._check(self._lib.gkrt_denoise_pass(self._h, C.byref(fc), self._stream(stream)))

    def end_frame(self, stream=None):
        self._check(self._lib.gkrt_end_frame(self._h, self._stream(stream)))

    def render(self, fc, stream=None):
        """Render(): rt pass -> reproject pass -> compose pass -> copy pass."""
        self._check(self._lib.gkrt_render_frame(self._h, C.byref(fc), self._stream(stream)))

    def synchronize(self, stream=None):
        self._check(self._lib.gkrt_synchronize(self._h, self._stream(stream)))

    # -- outputs ---------------------------------------------------------------------------
    def image_view(self, image_id: int) -> abi.GkrtImageView:
        v = abi.GkrtImageView()
        self._check(self._lib.gkrt_get_image(self._h, image_id, C.byref(v)))
        return v

    def read_image(self, image_id: int, stream=None, out: np.ndarray | None = None) -> np.ndarray:
        dt, ch = abi.IMAGE_FORMATS[image_id]
        shape = (self.height, self.width) if ch == 1 else (self.height, self.width, ch)
        if out is None:
            out = np.empty(shape, dt)
        self._check(self._lib.gkrt_copy_image_to_host(self._h, image_id, out.ctypes.data, out.nbytes,
                                                      self._stream(stream)))
        return out

    # ---- output stage: the presentation image (headless swapchain image, 8-bit BGRA) ----
    def output_resize(self, width: int, height: int):
        """SwapChain extent: (re)allocates the presentation image, black."""
        self._check(self._lib.gkrt_output_resize(self._h, width, height))
        self.output_width, self.output_height = int(width), int(height)

    def output_pass(self, mode=abi.OUTPUT_RESOLVE, offset=(0, 0), size=None, source=abi.IMG_DENOISED, stream=None):
        """Resolve (linear blit onto the rectangle offset + size, default the whole presentation
        image) or FSR compose (Process.UpScaleFSR: offset and size are its push constants)."""
        w, h = size if size is not None else (self.output_width, self.output_height)
        d = abi.GkrtOutputDesc(mode, int(offset[0]), int(offset[1]), int(w), int(h), int(source))
        self._check(self._lib.gkrt_output_pass(self._h, C.byref(d), self._stream(stream)))

    def read_output(self, stream=None) -> np.ndarray:
        """The presentation image as (height, width, 4) bytes B, G, R, A."""
        out = np.empty((self.output_height, self.output_width, 4), np.uint8)
        self._check(self._lib.gkrt_copy_output_to_host(self._h, out.ctypes.data, out.nbytes, self._stream(stream)))
        return out

    def save_screenshot(self, path: str, x=0, y=0, width=None, height=None, stream=None) -> np.ndarray:
        """ScreenShot::SaveSwapChainToFileFast: the crop written as an 8-bit RGB PNG."""
        from . import imageio
        rgb = self.screenshot(x, y, width, height, stream)
        imageio.write_png(path, rgb)
        return rgb

    def save_hdr(self, path: str, image_id=abi.IMG_DENOISED_LINEAR, stream=None) -> np.ndarray:
        """A linear float image written as PFM (the HDR dump in place of ScreenShot.cpp's AVIF)."""
        from . import imageio
        img = self.read_image(image_id, stream)
        imageio.write_pfm(path, img)
        return img

    def screenshot(self, x=0, y=0, width=None, height=None, stream=None) -> np.ndarray:
        """ScreenShot::SaveSwapChainToFileFast's crop: (height, width, 3) bytes R, G, B."""
        w = self.output_width - x if width is None else width
        h = self.output_height - y if height is None else height
        out = np.empty((h, w, 3), np.uint8)
        self._check(self._lib.gkrt_screenshot(self._h, x, y, w, h, out.ctypes.data, out.nbytes, self._stream(stream)))
        return out

    def read_image_async(self, image_id: int, out: np.ndarray, stream=None) -> np.ndarray:
        """The copy of read_image ordered on stream without waiting (out: page-locked memory for
        the copy to overlap other work; synchronize before reading it)."""
        dt, ch = abi.IMAGE_FORMATS[image_id]
        shape = (self.height, self.width) if ch == 1 else (self.height, self.width, ch)
        if out.dtype != np.dtype(dt) or out.shape != shape or not out.flags["C_CONTIGUOUS"]:
            raise ValueError(f"out must be a contiguous {dt} array of shape {shape}")
        self._check(self._lib.gkrt_copy_image_to_host_async(self._h, image_id, out.ctypes.data, out.nbytes,
                                                            self._stream(stream)))
        return out

    def write_image(self, image_id: int, data: np.ndarray, stream=None):
        dt, ch = abi.IMAGE_FORMATS[image_id]
        a = np.ascontiguousarray(data, dtype=dt)
        self._check(self._lib.gkrt_upload_image(self._h, image_id, a.ctypes.data, a.nbytes, self._stream(stream)))

    def images(self, ids=None) -> dict:
        ids = range(abi.IMG_COUNT) if ids is None else ids
        return {i: self.read_image(i) for i in ids}

    def trace_rays_device(self, rays_ptr: int, hits_ptr: int, count: int, mode=abi.TRACE_CLOSEST, stream=None):
        """Ray queries on device buffers (GkrtRay / GkrtHit layouts)."""
        self._check(self._lib.gkrt_trace_rays(self._h, C.c_void_p(rays_ptr), C.c_void_p(hits_ptr), count, mode,
                                              self._stream(stream)))

    # ---- ambient-cube probe grid (AmbientCube.slang; see gkrt.h) ----
    PROBE_COUNT = 192 * 192 * 48

    def probe_voxelize(self, stream=None):
        """Distance data of every probe (the reference's CPU voxelizer, on the GPU)."""
        self._check(self._lib.gkrt_probe_voxelize(self._h, self._stream(stream)))

    def probe_bake(self, fc, first: int = 0, count: int | None = None, stream=None):
        """One bake step of probes [first, first + count)."""
        if count is None:
            count = self.PROBE_COUNT - first
        self._check(self._lib.gkrt_probe_bake(self._h, C.byref(fc), first, count, self._stream(stream)))

    def probe_bake_slice(self, fc, frame: int, temporal_frames: int = 120, stream=None):
        """The reference's per-frame schedule (RayTraceBaseRenderer::PostRender): slice
        frame % F of (27648 // F) groups of 64 probes."""
        per = (self.PROBE_COUNT // 64) // temporal_frames
        self.probe_bake(fc, (frame % temporal_frames) * per * 64, per * 64, stream)

    def probe_download(self):
        """(cubes (N, 14) uint32, voxels (N, 4) uint32) of the whole grid."""
        cubes = np.zeros((self.PROBE_COUNT, 14), np.uint32)
        vox = np.zeros((self.PROBE_COUNT, 4), np.uint32)
        self._check(self._lib.gkrt_probe_download(self._h, cubes.ctypes.data, vox.ctypes.data))
        return cubes, vox

    def trace_rays_noalloc_device(self, rays_ptr: int, hits_ptr: int, count: int, mode=abi.TRACE_CLOSEST,
                                  stream=None):
        """Ray queries that allocate no device memory (static scratch; see gkrt.h)."""
        self._check(self._lib.gkrt_trace_rays_noalloc(self._h, C.c_void_p(rays_ptr), C.c_void_p(hits_ptr), count,
                                                      mode, self._stream(stream)))

    # ---- differentiable rendering (path-replay adjoint; device pointers) ----
    def set_material_params(self, albedo_ptr: int | None, rough_ptr: int | None, first: int, count: int,
                            stream=None):
        """Overwrite diffuse rgb (3 floats each) and fuzziness of materials [first, first+count)."""
        self._check(self._lib.gkrt_set_material_params(self._h, C.c_void_p(albedo_ptr or 0),
                                                       C.c_void_p(rough_ptr or 0), first, count,
                                                       self._stream(stream)))

    def adjoint_forward(self, fc, spp: int, image_ptr: int, sample_rough_ptr: int | None = None, stream=None):
        """The estimator's composed radiance (dense width x height float4) with spp samples."""
        self._check(self._lib.gkrt_adjoint_forward(self._h, C.byref(fc), spp, C.c_void_p(sample_rough_ptr or 0),
                                                   C.c_void_p(image_ptr), self._stream(stream)))

    def adjoint_backward(self, fc, spp: int, dimage_ptr: int, grad_albedo_ptr: int, grad_rough_ptr: int,
                         sample_rough_ptr: int | None = None, stream=None):
        """Adds d loss / d (albedo rgb, roughness) per material (doubles) for d loss / d image."""
        self._check(self._lib.gkrt_adjoint_backward(self._h, C.byref(fc), spp, C.c_void_p(sample_rough_ptr or 0),
                                                    C.c_void_p(dimage_ptr), C.c_void_p(grad_albedo_ptr),
                                                    C.c_void_p(grad_rough_ptr), self._stream(stream)))

    def pass_times(self) -> dict:
        """GPU ms of each pass's last run (contexts made with pass_timers=True): the reference's
        "rt pass", "reproject pass", "compose pass", "copy pass" and "TLAS Update" timers."""
        t = abi.GkrtPassTimes()
        self._check(self._lib.gkrt_get_pass_times(self._h, C.byref(t)))
        return {"rt pass": t.rt_pass_ms, "reproject pass": t.reproject_pass_ms, "compose pass": t.compose_pass_ms,
                "copy pass": t.copy_pass_ms, "TLAS Update": t.tlas_update_ms}

    def stats(self) -> abi.GkrtStats:
        s = abi.GkrtStats()
        self._check(self._lib.gkrt_get_stats(self._h, C.byref(s)))
        return s
