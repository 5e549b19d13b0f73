"""The learned denoiser on the GPU: forward output and every parameter gradient against the
numpy restatement (bf16 storage at the same points, FP64 arithmetic), training on the path
tracer's own 1-spp / high-spp pairs, and its gain over the bilateral filter against a
4096-spp reference at 1920 x 1080."""
import time

import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.denoiser import CornellVariants, Unet, device_view, relmse, train
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import unet_ref

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    assert torch.cuda.is_available()
    return torch


def test_unet_matches_cpu_oracle():
    torch = _torch()
    with PathTracingRenderer(0) as r:
        net = Unet(r, seed=3)
        assert net.nparams == unet_ref.param_count()
        rng = np.random.default_rng(4)
        B, H, W = 2, 64, 48
        inp = np.zeros((B, H, W, 10), np.float32)
        inp[..., :3] = rng.exponential(0.5, (B, H, W, 3))
        inp[..., 3:6] = rng.uniform(0.1, 0.9, (B, H, W, 3))
        n = rng.normal(size=(B, H, W, 3))
        inp[..., 6:9] = n / np.linalg.norm(n, axis=-1, keepdims=True)
        inp[..., 9] = rng.uniform(0.9, 1.0, (B, H, W))
        p = net.params().astype(np.float64)
        # larger output weights than the initialisation's, so the gradients reach every layer
        p += rng.normal(0.0, 0.02, p.shape)
        net.set_params(p)
        p = net.params().astype(np.float64)
        x = torch.as_tensor(inp, device="cuda")
        raw = torch.zeros((B, H, W, 4), device="cuda")
        net.forward(x, out_raw=raw)
        torch.cuda.synchronize()
        y_ref, cache = unet_ref.forward(p, inp.astype(np.float64))
        y = raw.cpu().numpy()[..., :3]
        assert np.linalg.norm(y - y_ref) < 2e-2 * np.linalg.norm(y_ref)
        d = rng.normal(size=(B, H, W, 3)) / (B * H * W)
        d4 = np.zeros((B, H, W, 4), np.float32)
        d4[..., :3] = d
        net.zero_grad()
        net.backward(torch.as_tensor(d4, device="cuda"))
        _, g = net.params(with_grads=True)
        g_ref = unet_ref.backward(cache, d)
        off = 0
        rels, coss = [], []
        for l, (ci, co, _) in enumerate(unet_ref.LAYERS):
            n_ = 9 * ci * co + co
            a, b = g[off:off + n_].astype(np.float64), g_ref[off:off + n_]
            rels.append(np.linalg.norm(a - b) / (np.linalg.norm(b) + 1e-30))
            coss.append(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
            off += n_
        print("per-layer relative gradient error", np.round(rels, 4), "cosine", np.round(coss, 5))
        # The output layer's gradient depends on stored activations only and matches closely.
        # Deeper layers see gradients re-rounded to bf16 at every layer; the oracle itself moves
        # by 3-10% per layer between FP32 and FP64 accumulation, so the bar there is direction
        # (cosine) and a bounded relative error. The kernels themselves are pinned in
        # isolation by test_gpu_conv.py (weight and input gradients against torch).
        assert rels[-1] < 2e-2, rels
        assert min(coss) > 0.98 and max(rels) < 0.25, (rels, coss)


def test_unet_overfits_a_batch():
    torch = _torch()
    with PathTracingRenderer(0) as r:
        net = Unet(r, seed=5)
        g = torch.Generator(device="cuda").manual_seed(1)
        inp = torch.rand((2, 64, 64, 10), device="cuda", generator=g)
        # a target the network can represent: a smooth function of the albedo channels
        tgt = 0.8 * inp[..., 3:6] * inp[..., 4:5] + 0.1
        losses = [net.train_step(inp, tgt, 1e-3) for _ in range(200)]
        assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])


def test_denoiser_beats_bilateral():
    """Train on 512 x 512 Cornell variants (256-spp targets), then on a held-out 1080p variant
    compare RelMSE against 4096 spp: the network must reach <= 0.8 x the bilateral filter's
    (the reference's joint bilateral filter on the same 1-spp frame)."""
    torch = _torch()
    with PathTracingRenderer(0) as r:
        data = CornellVariants(r, 512, 512, count=17, seed=5)
        t0 = time.perf_counter()
        refs = [data.render_reference(v, 256) for v in range(16)]
        t_data = time.perf_counter() - t0
        net = Unet(r, seed=7)
        t0 = time.perf_counter()
        losses = train(net, data, refs, steps=600, batch=2, lr=5e-4)
        torch.cuda.synchronize()
        t_train = time.perf_counter() - t0
        # held-out variant 16 at 1080p
        Wt, Ht = 1920, 1080
        test = CornellVariants(r, Wt, Ht, count=17, seed=5)
        ref = test.render_reference(16, 4096)
        inp = torch.zeros((1, Ht, Wt, 10), device="cuda")
        test.render_input(16, 424242, inp[0])
        out = torch.zeros((1, Ht, Wt, 4), device="cuda")
        net.forward(inp, out_linear=out)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            net.forward(inp, out_linear=out)
        torch.cuda.synchronize()
        t_net = (time.perf_counter() - t0) / 5
        e_net = relmse(out[0], ref)
        # the same 1-spp frame through the reference's bilateral filter (history weight 0)
        st = test.settings
        st.denoiser, st.bf_size, st.temporal_frames = abi.DENOISE_JBF, 5, 1
        fb = camera.FrameBuilder(Wt, Ht, st)
        fc = fb.build(test.cam.orbit(float(test.angles[16])), 424242)
        r.create_swap_chain(Wt, Ht)
        r.trace_pass(fc)
        r.reproject_pass(fc)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            r.denoise_pass(fc)
        torch.cuda.synchronize()
        t_jbf = (time.perf_counter() - t0) / 5
        e_jbf = relmse(device_view(r.image_view(abi.IMG_DENOISED_LINEAR), 4), ref)
        e_raw = relmse(inp[0, ..., :3], ref)
        print(f"denoiser: data {t_data:.1f} s, train {t_train:.1f} s ({t_train / 600 * 1e3:.1f} ms/step), "
              f"loss {np.mean(losses[:20]):.4f} -> {np.mean(losses[-20:]):.4f}; 1080p RelMSE raw {e_raw:.4f}, "
              f"bilateral {e_jbf:.4f}, learned {e_net:.4f} (ratio {e_net / e_jbf:.3f}); "
              f"ms: bilateral {t_jbf * 1e3:.3f}, learned {t_net * 1e3:.3f}")
        assert e_net <= 0.8 * e_jbf
