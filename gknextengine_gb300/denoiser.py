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
import json
import os
import sys
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


def compose_input(r: PathTracingRenderer, out):
    """The pass's images after a trace pass as the network's input, out (H, W, 10): radiance
    composed as the compose pass does (diffuse x albedo + specular), albedo, normal, depth."""
    d = device_view(r.image_view(abi.IMG_SINGLE_DIFFUSE), 4)
    s = device_view(r.image_view(abi.IMG_SINGLE_SPECULAR), 4)
    a = device_view(r.image_view(abi.IMG_ALBEDO), 4)
    n = device_view(r.image_view(abi.IMG_NORMAL), 4)
    z = device_view(r.image_view(abi.IMG_PREV_DEPTH), 1)
    out[..., 0:3] = d[..., :3] * a[..., :3] + s[..., :3]
    out[..., 3:6] = a[..., :3]
    out[..., 6:9] = n[..., :3]
    out[..., 9:10] = z
    return out


def render_reference_frames(r: PathTracingRenderer, fb: camera.FrameBuilder, cam: camera.Camera, spp: int,
                            spp_per_pass: int = 64, seed0: int = 1 << 20):
    """Composed radiance (H, W, 3) averaged over spp samples per pixel: spp / spp_per_pass
    trace passes of the static view, each with spp_per_pass samples per pixel (the pass's own
    multi-sample loop) and its own RNG stream (TotalFrames seed0 + pass index)."""
    torch = _torch()
    passes = max(1, spp // spp_per_pass)
    keep = fb.s.samples
    fb.s.samples = spp_per_pass
    try:
        acc = torch.zeros((r.height, r.width, 3), dtype=torch.float64, device="cuda")
        d = device_view(r.image_view(abi.IMG_SINGLE_DIFFUSE), 4)
        s = device_view(r.image_view(abi.IMG_SINGLE_SPECULAR), 4)
        a = device_view(r.image_view(abi.IMG_ALBEDO), 4)
        for k in range(passes):
            r.trace_pass(fb.build(cam, seed0 + k))
            acc += (d[..., :3] * a[..., :3] + s[..., :3]).double()
    finally:
        fb.s.samples = keep
    return (acc / passes).float()


# ---- the C5 training set: renderer-generated 1-spp / 4096-spp crop pairs ----

def cornell_family_view(seed: int, index: int):
    """View `index` of the training family: the C1 Cornell box (scenes.cornell) with seeded
    variations, so that the network meets other materials, lighting regimes and framings while
    staying on config-1 frames. Per view:
      * albedos U(0.15, 0.9)^3; each wall Lambertian (70 %), a GGX mixture (20 %) or a rough
        metal (10 %); each box Lambertian (30 %), mixture (30 %), metal with roughness
        U(0.02, 1) (25 %) or glass (15 %);
      * lighting: the ceiling light at radiance U(5, 25) (55 %), dimmed to U(0.5, 5) (15 %), or
        off with a box as the only emitter, radiance U(5, 20) (30 %); otherwise a box emits
        with probability 0.1;
      * the boxes moved, turned and scaled inside the room;
      * the camera orbited U(-50, 50) degrees, moved 0.6 to 3 times as far, raised or lowered,
        with a field of view U(25, 60) degrees;
      * in half of the views the whole scene and the camera scaled by a factor log-uniform in
        [1, 80]: the image stays the same while the depth channel (NDC depth, near 0.2, far
        2000) moves towards 1 as in large scenes.
    Returns (SceneArrays, Camera, Settings) with C1's 4 bounces and no TAA."""
    rng = np.random.default_rng([seed, index])
    sc, cam, st = scenes.cornell(seed=int(rng.integers(1 << 30)))
    mats = []
    for i in range(5):
        alb = rng.uniform(0.15, 0.9, 3)
        u = rng.random()
        mats.append(scenes.lambertian(alb) if u < 0.7 else
                    scenes.mixture(alb, rng.uniform(0.05, 1.0)) if u < 0.9 else
                    scenes.metallic(alb, rng.uniform(0.2, 1.0)))
    u = rng.random()
    mode = "ceiling" if u < 0.55 else "dim" if u < 0.7 else "box"
    emitting_box = int(rng.integers(0, 2)) if mode == "box" else (int(rng.integers(0, 2)) if rng.random() < 0.1 else -1)
    for b in range(2):
        alb = rng.uniform(0.15, 0.9, 3)
        u = rng.random()
        if b == emitting_box:
            mats.append(scenes.diffuse_light(np.full(3, rng.uniform(5.0, 20.0))))
        else:
            mats.append(scenes.lambertian(alb) if u < 0.3 else
                        scenes.mixture(alb, rng.uniform(0.05, 1.0)) if u < 0.6 else
                        scenes.metallic(alb, rng.uniform(0.02, 1.0)) if u < 0.85 else scenes.dielectric(1.5))
    light = {"ceiling": rng.uniform(5.0, 25.0), "dim": rng.uniform(0.5, 5.0), "box": 0.0}[mode]
    mats.append(scenes.diffuse_light(np.full(3, light)))
    materials = np.array(mats, dtype=abi.MATERIAL_DTYPE)
    inst = sc.instances.copy()
    scale = float(np.exp(rng.uniform(0.0, np.log(80.0)))) if rng.random() < 0.5 else 1.0
    inst[0] = scenes.make_instance(0, scenes.trs(scale=(scale, scale, scale)), [0, 1, 2, 3, 4, 7], 0)
    for k, (mat, iid) in enumerate(((5, 1), (6, 2))):
        sxz = rng.uniform(0.15, 0.35)
        world = scenes.trs((rng.uniform(-0.3, 0.3), 0.0, rng.uniform(-0.3, 0.3)), rot_y_deg=rng.uniform(-45, 45),
                           scale=(sxz, rng.uniform(0.15, 0.7), sxz * rng.uniform(0.7, 1.4)))
        inst[1 + k] = scenes.make_instance(1, world * scale, [mat], iid)
    lights = sc.lights.copy()
    for f in ("p0", "p1", "p3"):
        lights[f][:, :3] *= scale
    lights["normal_area"][:, 3] *= scale * scale
    sc = abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, materials, inst,
                         lights=lights, name=f"cornell-family-{seed}-{index}")
    c = cam.orbit(float(rng.uniform(-50.0, 50.0)))
    eye = c.center + (c.eye - c.center) * rng.uniform(0.6, 3.0)
    eye[1] = c.center[1] + rng.uniform(-0.35, 0.45)
    cam = camera.Camera(eye=eye * scale, center=c.center * scale, fov_deg=float(rng.uniform(25.0, 60.0)))
    st.taa = False
    st.flags = 0
    return sc, cam, st


def build_crop_set(r: PathTracingRenderer, views: int = 128, view_size: int = 1024, crop: int = 256,
                   ref_spp: int = 4096, inputs_per_crop: int = 4, seed: int = 11, spp_per_pass: int = 64,
                   log=None):
    """The C5 training set on the GPU: `views` family views rendered at view_size^2, each cut
    into (view_size / crop)^2 crops (128 views x 16 = 2048 crops of 256 x 256). Per crop: the
    ref_spp-sample composed radiance (the target) and inputs_per_crop independent 1-spp inputs
    (10 channels each). Returns (inputs (N, R, crop, crop, 10), targets (N, crop, crop, 3),
    info), device float32."""
    torch = _torch()
    g = view_size // crop
    n = views * g * g
    inputs = torch.zeros((n, inputs_per_crop, crop, crop, 10), device="cuda")
    targets = torch.zeros((n, crop, crop, 3), device="cuda")
    full = torch.zeros((view_size, view_size, 10), device="cuda")
    t0 = time.perf_counter()
    for v in range(views):
        sc, cam, st = cornell_family_view(seed, v)
        r.load_scene(sc)
        if (r.width, r.height) != (view_size, view_size):
            r.create_swap_chain(view_size, view_size)
        fb = camera.FrameBuilder(view_size, view_size, st)
        ref = render_reference_frames(r, fb, cam, ref_spp, spp_per_pass)
        base = v * g * g
        targets[base:base + g * g] = ref.view(g, crop, g, crop, 3).permute(0, 2, 1, 3, 4).reshape(g * g, crop, crop, 3)
        for k in range(inputs_per_crop):
            r.trace_pass(fb.build(cam, 1000 + k))
            compose_input(r, full)
            inputs[base:base + g * g, k] = full.view(g, crop, g, crop, 10).permute(0, 2, 1, 3, 4).reshape(
                g * g, crop, crop, 10)
        if log and (v + 1) % 16 == 0:
            torch.cuda.synchronize()
            log(f"crop set: {v + 1}/{views} views, {time.perf_counter() - t0:.1f} s")
    torch.cuda.synchronize()
    return inputs, targets, {"views": views, "view_size": view_size, "crop": crop, "crops": n,
                             "reference_spp": ref_spp, "inputs_per_crop": inputs_per_crop, "seed": seed,
                             "seconds": time.perf_counter() - t0}


def lr_at(step: int, steps: int, lr: float, lr_decay_from: float = 0.6, warmup: int = 40) -> float:
    """Linear warm-up over `warmup` steps, constant, then a decay to lr / 10 over the steps
    after lr_decay_from."""
    frac = step / max(steps - 1, 1)
    cur = lr if frac < lr_decay_from else lr * (0.1 ** ((frac - lr_decay_from) / (1.0 - lr_decay_from)))
    return cur * min(1.0, (step + 1) / warmup)


def train_crops(net: "Unet", inputs, targets, steps: int, batch: int = 8, lr: float = 5e-4, seed: int = 9,
                log=None):
    """Adam steps on random crops of the set, each with one of its 1-spp inputs picked at
    random. Returns the per-step losses (mean squared log error)."""
    torch = _torch()
    gen = torch.Generator(device="cuda").manual_seed(seed)
    n, R = inputs.shape[0], inputs.shape[1]
    losses = []
    t0 = time.perf_counter()
    for step in range(steps):
        idx = torch.randint(0, n, (batch,), device="cuda", generator=gen)
        rep = torch.randint(0, R, (batch,), device="cuda", generator=gen)
        inp = inputs[idx, rep].contiguous()
        tgt = targets[idx].contiguous()
        losses.append(net.train_step(inp, tgt, lr_at(step, steps, lr)))
        if log and (step + 1) % 1000 == 0:
            log(f"train: step {step + 1}/{steps}, loss {np.mean(losses[-200:]):.5f}, "
                f"{time.perf_counter() - t0:.1f} s")
    return losses


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


def evaluate_view(r: PathTracingRenderer, net: "Unet", scene, cam: camera.Camera, settings: camera.Settings,
                  name: str, width: int = 1920, height: int = 1080, ref_spp: int = 4096, reps: int = 10,
                  load: bool = True):
    """RelMSE against a ref_spp reference of one static view, for the raw 1-spp frame, the
    reference's joint bilateral filter (JBF, 5 x 5) and the a-trous filter on that frame
    (history weight 1), the learned denoiser through the library's own denoise pass
    (GKRT_DENOISE_UNET) on the same frame, and the temporal steady state of the two filters
    (128 frames of reprojection at 1/16). Frame times in ms, CUDA events: a bilateral frame is
    trace + reproject + JBF, a learned frame is trace + the learned denoise pass. TAA is off, so
    every frame sees the camera the reference was rendered with."""
    torch = _torch()
    st = settings
    st.taa = False
    st.flags = 0
    if load:
        r.load_scene(scene)
    r.create_swap_chain(width, height)
    fb = camera.FrameBuilder(width, height, st)
    t0 = time.perf_counter()
    ref = render_reference_frames(r, fb, cam, ref_spp)
    torch.cuda.synchronize()
    out = {"scene": f"{name} {width}x{height}", "reference_spp": ref_spp,
           "metric": "mean (x-y)^2/(y^2+1e-2) over px, RGB, linear radiance",
           "reference_seconds": time.perf_counter() - t0}
    fseed = 424242

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

    linear = device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4)
    keep = (st.denoiser, st.bf_size, st.temporal_frames)
    try:
        st.denoiser, st.temporal_frames = abi.DENOISE_UNET, 1
        fb = camera.FrameBuilder(width, height, st)
        f1 = fb.build(cam, fseed)
        r.trace_pass(f1)
        inp = torch.zeros((height, width, 10), device="cuda")
        out["raw_1spp"] = relmse(compose_input(r, inp)[..., :3], ref)
        out["trace_ms"] = timed(lambda: r.trace_pass(f1))
        out["learned_ms"] = timed(lambda: r.denoise_pass(f1))
        out["learned_1spp"] = relmse(linear, ref)
        for fname, mode in (("bilateral", abi.DENOISE_JBF), ("atrous", abi.DENOISE_ATROUS)):
            st.denoiser, st.bf_size, st.temporal_frames = mode, 5, 1
            fb = camera.FrameBuilder(width, height, st)
            f1 = fb.build(cam, fseed)
            r.create_swap_chain(width, height)
            r.trace_pass(f1)
            r.reproject_pass(f1)
            out[f"{fname}_ms"] = timed(lambda: r.denoise_pass(f1))
            linear = device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4)
            out[f"{fname}_1spp"] = relmse(linear, ref)
            out["reproject_ms"] = timed(lambda: r.reproject_pass(f1))
            st.temporal_frames = 16
            fb = camera.FrameBuilder(width, height, st)
            r.create_swap_chain(width, height)
            for f in range(128):
                r.render(fb.build(cam, 500000 + f))
            linear = device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4)
            out[f"{fname}_temporal"] = relmse(linear, ref)
    finally:
        st.denoiser, st.bf_size, st.temporal_frames = keep
    out["learned_over_bilateral"] = out["learned_1spp"] / out["bilateral_1spp"]
    out["learned_over_bilateral_temporal"] = out["learned_1spp"] / out["bilateral_temporal"]
    out["frame_ms_bilateral"] = out["trace_ms"] + out["reproject_ms"] + out["bilateral_ms"]
    out["frame_ms_learned"] = out["trace_ms"] + out["learned_ms"]
    out["frame_time_ratio"] = out["frame_ms_learned"] / out["frame_ms_bilateral"]
    return out


# The network trained on the C5 crop set (train_c5 below), shipped with the library.
C5_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "unet_c5.ckpt")


def load_c5(r: PathTracingRenderer, path: str = C5_WEIGHTS) -> "Unet":
    """The shipped C5 network on a renderer's context (the context's denoise pass uses it)."""
    net = Unet(r, seed=7)
    net.load(path)
    return net


def evaluate_c5(r: PathTracingRenderer, net: "Unet", width: int = 1920, height: int = 1080,
                ref_spp: int = 4096) -> dict:
    """The learned denoiser against the filters on two views, neither in the training set: the
    config-1 Cornell box itself (scenes.cornell, its own albedos) and a frame of the C2 brick
    scene (1.03 M triangles, GGX metals and mixtures, 64 emissive bricks, 8 bounces), a scene
    family the network has never seen."""
    sc, cam, st = scenes.cornell()
    cornell = evaluate_view(r, net, sc, cam, st, "config-1 cornell (held out)", width, height, ref_spp)
    sc, cam, st = scenes.bricks()
    bricks = evaluate_view(r, net, sc, cam, st, "c2 bricks (unseen scene family)", width, height, ref_spp)
    return {"cornell": cornell, "bricks": bricks}


def train_c5(r: PathTracingRenderer, steps: int = 8000, batch: int = 8, lr: float = 5e-4, views: int = 128,
             ref_spp: int = 4096, inputs_per_crop: int = 4, seed: int = 11, log=None):
    """The C5 training run: the crop set (build_crop_set: 2048 crops of 256 x 256 with 4096-spp
    targets) rendered by the path tracer, then `steps` Adam steps of the library's own training
    kernels on batches of crops. Returns (net, losses, info)."""
    inputs, targets, info = build_crop_set(r, views=views, ref_spp=ref_spp, inputs_per_crop=inputs_per_crop,
                                           seed=seed, log=log)
    net = Unet(r, seed=7)
    t0 = time.perf_counter()
    losses = train_crops(net, inputs, targets, steps, batch=batch, lr=lr, log=log)
    _torch().cuda.synchronize()
    info.update({"steps": steps, "batch": batch, "lr": lr, "train_s": time.perf_counter() - t0,
                 "loss_first": float(np.mean(losses[:50])), "loss_last": float(np.mean(losses[-200:]))})
    del inputs, targets
    return net, losses, info


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


def main(argv=None):
    """python -m gknextengine_gb300.denoiser --train-c5 OUT.ckpt [--steps N] [--views V]:
    renders the C5 crop set, trains, writes the checkpoint and prints the evaluation."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-c5", required=True, help="checkpoint file to write")
    ap.add_argument("--steps", type=int, default=8000)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--views", type=int, default=128)
    ap.add_argument("--ref-spp", type=int, default=4096)
    ap.add_argument("--eval-spp", type=int, default=4096)
    ap.add_argument("--info", default=None, help="JSON file for the training and evaluation record")
    a = ap.parse_args(argv)

    def log(msg):
        print(msg, flush=True)

    with PathTracingRenderer(0) as r:
        net, losses, info = train_c5(r, steps=a.steps, batch=a.batch, views=a.views, ref_spp=a.ref_spp, log=log)
        net.save(a.train_c5)
        info["losses_every_100"] = [float(np.mean(losses[i:i + 100])) for i in range(0, len(losses), 100)]
        log(json.dumps({k: v for k, v in info.items() if k != "losses_every_100"}))
        ev = evaluate_c5(r, net, ref_spp=a.eval_spp)
        log(json.dumps(ev))
        if a.info:
            with open(a.info, "w") as f:
                json.dump({"training": info, "evaluation": ev}, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
