"""Training data and training loop of the learned denoiser (GKRT_DENOISE_UNET).

The path tracer makes its own training pairs: for a set of Cornell-box variants (camera
orbit angle and albedos drawn from a seeded generator) it renders a high-spp reference by
averaging independent 1-spp trace passes, and each training step renders a fresh 1-spp
frame of a random variant as the network input (radiance composed as the compose pass does,
albedo, normal, depth). The network itself runs in libgkrt (gkrt_unet_*); torch only holds
device memory. The images of the pass are pitched by width rounded up to 4, so widths here
are multiples of 8 and the image views are dense.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import abi, camera, scenes
from .renderer import PathTracingRenderer


def _torch():
    import torch
    return torch


def device_view(view, channels: int):
    """A dense torch view (H, W, channels) of one of the pass's float images (no copy)."""
    torch = _torch()
    n = view.height * (view.pitch_bytes // 4)

    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (view.device_ptr, False), "version": 3}

    t = torch.as_tensor(_A(), device="cuda").view(view.height, view.pitch_bytes // (4 * channels), channels)
    return t[:, :view.width]


class CornellVariants:
    """Cornell-box variants on one renderer: camera orbit angle U(-35, 35) degrees and
    per-object albedo U(0.15, 0.9)^3 from `seed`."""

    def __init__(self, renderer: PathTracingRenderer, width: int, height: int, count: int, seed: int = 5):
        self.r = renderer
        self.W, self.H = width, height
        self.scene, self.cam, self.settings = scenes.cornell()
        self.settings.taa = False
        self.settings.flags = 0
        rng = np.random.default_rng(seed)
        self.angles = rng.uniform(-35.0, 35.0, count)
        self.albedo = rng.uniform(0.15, 0.9, (count, 7, 3)).astype(np.float32)
        self.fb = camera.FrameBuilder(width, height, self.settings)
        torch = _torch()
        self._alb = torch.zeros((7, 3), device="cuda")
        self._rough = torch.as_tensor(self.scene.materials["fuzziness"][:7].copy(), device="cuda")
        renderer.load_scene(self.scene)
        renderer.create_swap_chain(width, height)

    def select(self, v: int):
        torch = _torch()
        self._alb.copy_(torch.as_tensor(self.albedo[v], device="cuda"))
        self.r.set_material_params(self._alb.data_ptr(), self._rough.data_ptr(), 0, 7)

    def frame(self, v: int, seed: int):
        return self.fb.build(self.cam.orbit(float(self.angles[v])), int(seed))

    def render_input(self, v: int, seed: int, out):
        """One 1-spp pass of variant v into out (H, W, 10): radiance, albedo, normal, depth."""
        self.select(v)
        self.r.trace_pass(self.frame(v, seed))
        d = device_view(self.r.image_view(abi.IMG_SINGLE_DIFFUSE), 4)
        s = device_view(self.r.image_view(abi.IMG_SINGLE_SPECULAR), 4)
        a = device_view(self.r.image_view(abi.IMG_ALBEDO), 4)
        n = device_view(self.r.image_view(abi.IMG_NORMAL), 4)
        z = device_view(self.r.image_view(abi.IMG_PREV_DEPTH), 1)
        out[..., 0:3] = d[..., :3] * a[..., :3] + s[..., :3]
        out[..., 3:6] = a[..., :3]
        out[..., 6:9] = n[..., :3]
        out[..., 9:10] = z
        return out

    def render_reference(self, v: int, spp: int, seed0: int = 1 << 20):
        """Mean of spp independent 1-spp passes (composed radiance), (H, W, 3)."""
        torch = _torch()
        self.select(v)
        acc = torch.zeros((self.H, self.W, 3), dtype=torch.float64, device="cuda")
        d = device_view(self.r.image_view(abi.IMG_SINGLE_DIFFUSE), 4)
        s = device_view(self.r.image_view(abi.IMG_SINGLE_SPECULAR), 4)
        a = device_view(self.r.image_view(abi.IMG_ALBEDO), 4)
        for k in range(spp):
            self.r.trace_pass(self.frame(v, seed0 + k))
            acc += (d[..., :3] * a[..., :3] + s[..., :3]).double()
        return (acc / spp).float()


def relmse(x, y) -> float:
    """mean over pixels and RGB of (x - y)^2 / (y^2 + 1e-2)."""
    d = (x[..., :3].double() - y[..., :3].double())
    return float((d * d / (y[..., :3].double() ** 2 + 1e-2)).mean())


class Unet:
    """The library's denoiser network on a renderer's context."""

    def __init__(self, renderer: PathTracingRenderer, seed: int = 7):
        self.r = renderer
        self.L = renderer._lib
        self.h = renderer._h
        self._check(self.L.gkrt_unet_init(self.h, seed))
        n = C.c_uint32()
        self._check(self.L.gkrt_unet_param_count(self.h, C.byref(n)))
        self.nparams = n.value

    def _check(self, rc):
        self.r._check(rc)

    def train_step(self, inp, target, lr: float) -> float:
        B, H, W = inp.shape[0], inp.shape[1], inp.shape[2]
        loss = C.c_double()
        self._check(self.L.gkrt_unet_train_step(self.h, C.c_void_p(inp.data_ptr()), C.c_void_p(target.data_ptr()),
                                                B, H, W, C.c_float(lr), C.byref(loss), None))
        return loss.value

    def forward(self, inp, out_linear=None, out_raw=None):
        B, H, W = inp.shape[0], inp.shape[1], inp.shape[2]
        self._check(self.L.gkrt_unet_forward(self.h, C.c_void_p(inp.data_ptr()), B, H, W,
                                             C.c_void_p(out_linear.data_ptr() if out_linear is not None else 0),
                                             C.c_void_p(out_raw.data_ptr() if out_raw is not None else 0), None))

    def backward(self, d_raw):
        self._check(self.L.gkrt_unet_backward(self.h, C.c_void_p(d_raw.data_ptr()), None))

    def zero_grad(self):
        self._check(self.L.gkrt_unet_zero_grad(self.h, None))

    def params(self, with_grads: bool = False):
        p = np.zeros(self.nparams, np.float32)
        g = np.zeros(self.nparams, np.float32) if with_grads else None
        self._check(self.L.gkrt_unet_get_params(self.h, p.ctypes.data, g.ctypes.data if g is not None else None))
        return (p, g) if with_grads else p

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        self._check(self.L.gkrt_unet_set_params(self.h, p.ctypes.data))

    def optimizer_state(self):
        """(first moments, second moments, step) of Adam."""
        m = np.zeros(self.nparams, np.float32)
        v = np.zeros(self.nparams, np.float32)
        step = C.c_uint64()
        self._check(self.L.gkrt_unet_get_state(self.h, m.ctypes.data, v.ctypes.data, C.byref(step)))
        return m, v, step.value

    def set_optimizer_state(self, m, v, step: int):
        m = np.ascontiguousarray(m, np.float32)
        v = np.ascontiguousarray(v, np.float32)
        self._check(self.L.gkrt_unet_set_state(self.h, m.ctypes.data, v.ctypes.data, int(step)))

    def save(self, path: str):
        """Parameters and Adam's state to a checkpoint file (checkpoint.py)."""
        from . import checkpoint
        m, v, step = self.optimizer_state()
        checkpoint.save(path, self.params(), m, v, step)

    def load(self, path: str):
        """Restore a checkpoint written by save(); training continues from its step."""
        from . import checkpoint
        p, m, v, step = checkpoint.load(path, self.nparams)
        self.set_params(p)
        self.set_optimizer_state(m, v, step)


def train(net: Unet, data: CornellVariants, refs, steps: int, batch: int = 2, lr: float = 5e-4, seed: int = 9,
          lr_decay_from: float = 0.6, warmup: int = 40):
    """Adam steps on fresh 1-spp inputs of random variants against their references: linear
    warm-up over `warmup` steps, constant, then a decay to lr/10 over the last 40%.
    Returns the per-step losses (mean squared log error)."""
    torch = _torch()
    rng = np.random.default_rng(seed)
    H, W = data.H, data.W
    inp = torch.zeros((batch, H, W, 10), device="cuda")
    tgt = torch.zeros((batch, H, W, 3), device="cuda")
    losses = []
    for step in range(steps):
        for b in range(batch):
            v = int(rng.integers(0, len(refs)))
            data.render_input(v, 1000 + step * batch + b, inp[b])
            tgt[b] = refs[v]
        frac = step / max(steps - 1, 1)
        cur = lr if frac < lr_decay_from else lr * (0.1 ** ((frac - lr_decay_from) / (1.0 - lr_decay_from)))
        cur *= min(1.0, (step + 1) / warmup)
        losses.append(net.train_step(inp, tgt, cur))
    return losses


def evaluate(r: PathTracingRenderer, net: Unet, width: int = 1920, height: int = 1080, variant: int = 16,
             count: int = 17, seed: int = 5, ref_spp: int = 4096, reps: int = 10):
    """RelMSE against a ref_spp reference of one held-out Cornell variant: the raw 1-spp frame,
    the bilateral filter (the reference's JBF) and the a-trous filter on that frame (history
    weight 0), the learned denoiser on it, and the temporal steady state of the two filters
    (8 x 16 frames of reprojection at 1/16). Times are per 1080p frame, CUDA events."""
    torch = _torch()
    data = CornellVariants(r, width, height, count=count, seed=seed)
    t0 = time.perf_counter()
    ref = data.render_reference(variant, ref_spp)
    out = {"scene": f"cornell variant {variant} {width}x{height}", "reference_spp": ref_spp,
           "metric": "mean (x-y)^2/(y^2+1e-2) over px, RGB, linear radiance",
           "reference_seconds": time.perf_counter() - t0}
    st = data.settings
    fseed = 424242
    fc = data.frame(variant, fseed)
    inp = torch.zeros((1, height, width, 10), device="cuda")
    data.render_input(variant, fseed, inp[0])
    out["raw_1spp"] = relmse(inp[0, ..., :3], ref)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    den = torch.zeros((1, height, width, 4), device="cuda")
    out["learned_ms"] = timed(lambda: net.forward(inp, out_linear=den))
    out["learned_1spp"] = relmse(den[0], ref)
    out["trace_ms"] = timed(lambda: r.trace_pass(fc))
    for name, mode in (("bilateral", abi.DENOISE_JBF), ("atrous", abi.DENOISE_ATROUS)):
        st.denoiser, st.bf_size, st.temporal_frames = mode, 5, 1
        fb = camera.FrameBuilder(width, height, st)
        f1 = fb.build(data.cam.orbit(float(data.angles[variant])), fseed)
        r.create_swap_chain(width, height)
        r.trace_pass(f1)
        r.reproject_pass(f1)
        out[f"{name}_ms"] = timed(lambda: r.denoise_pass(f1))
        out[f"{name}_1spp"] = relmse(device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4), ref)
        st.temporal_frames = 16
        fb = camera.FrameBuilder(width, height, st)
        r.create_swap_chain(width, height)
        for f in range(128):
            r.render(fb.build(data.cam.orbit(float(data.angles[variant])), 500000 + f))
        out[f"{name}_temporal"] = relmse(device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4), ref)
        out["reproject_ms"] = timed(lambda: r.reproject_pass(f1))
    out["learned_over_bilateral"] = out["learned_1spp"] / out["bilateral_1spp"]
    out["frame_ms_bilateral"] = out["trace_ms"] + out["reproject_ms"] + out["bilateral_ms"]
    out["frame_ms_learned"] = out["trace_ms"] + out["learned_ms"]
    return out


def train_default(r: PathTracingRenderer, steps: int = 600, variants: int = 16, ref_spp: int = 256,
                  width: int = 512, height: int = 512, seed: int = 5):
    """The training run the tests and the benchmark use; returns (net, losses, seconds)."""
    data = CornellVariants(r, width, height, count=variants + 1, seed=seed)
    t0 = time.perf_counter()
    refs = [data.render_reference(v, ref_spp) for v in range(variants)]
    t_data = time.perf_counter() - t0
    net = Unet(r, seed=7)
    t0 = time.perf_counter()
    losses = train(net, data, refs, steps=steps, batch=2, lr=5e-4)
    _torch().cuda.synchronize()
    return net, losses, {"data_s": t_data, "train_s": time.perf_counter() - t0, "steps": steps,
                         "ms_per_step": (time.perf_counter() - t0) / steps * 1e3}
