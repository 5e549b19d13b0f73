"""The learned denoiser on the GPU: forward output and every parameter gradient against the
numpy restatement (bf16 storage at the same points, FP64 arithmetic), training on the path
tracer's own 1-spp / high-spp pairs, and its gain over the bilateral filter against a
4096-spp reference at 1920 x 1080."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.denoiser import Unet
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
        # gkrt_unet_forward is the inference forward (sub-pixel dec0a); its oracle, and the
        # training forward's, which the backward below runs again
        y_inf, _ = unet_ref.forward(p, inp.astype(np.float64), inference=True)
        y = raw.cpu().numpy()[..., :3]
        e_inf = np.linalg.norm(y - y_inf) / np.linalg.norm(y_inf)
        e_train = np.linalg.norm(y - y_ref) / np.linalg.norm(y_ref)
        print("forward relative error: inference oracle", e_inf, "training oracle", e_train)
        assert e_inf < 2e-2 and e_train < 2e-2
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
        # (cosine) and a bounded relative error (measured with these seeds: at most 0.134, the
        # cosine at least 0.992; a convolution kernel that sums the taps in another order gave
        # a cosine of 0.988). The kernels themselves are pinned in isolation by
        # test_gpu_conv.py (weight and input gradients against torch).
        assert rels[-1] < 2e-2, rels
        assert min(coss) > 0.98 and max(rels) < 0.18, (rels, coss)


def test_backward_needs_a_forward_and_follows_inference():
    """gkrt_unet_backward without a forward is a state error. After the inference forward it
    re-runs the training forward on the same input, so a second backward (now on the training
    forward's activations) gives the same gradients (up to the order of the weight-gradient
    partial sums)."""
    torch = _torch()
    from gknextengine_gb300.native import GkrtError
    with PathTracingRenderer(0) as r:
        net = Unet(r, seed=9)
        d = torch.zeros((1, 32, 32, 4), device="cuda")
        with pytest.raises(GkrtError) as e:
            net.backward(d)
        assert e.value.code == abi.GKRT_ERR_STATE
        g = torch.Generator(device="cuda").manual_seed(2)
        inp = torch.rand((1, 32, 32, 10), device="cuda", generator=g)
        raw = torch.zeros((1, 32, 32, 4), device="cuda")
        net.forward(inp, out_raw=raw)
        d = torch.randn((1, 32, 32, 4), device="cuda", generator=g) * 1e-3
        net.zero_grad()
        net.backward(d)
        _, g1 = net.params(with_grads=True)
        net.zero_grad()
        net.backward(d)   # the activations are the training forward's now: the same gradients
        _, g2 = net.params(with_grads=True)
        assert np.isfinite(g1).all() and np.abs(g1).max() > 0
        assert np.linalg.norm(g2 - g1) <= 1e-5 * np.linalg.norm(g1)


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


def test_checkpoint_resume(tmp_path):
    """Save after a few steps, load into a freshly initialised network on another context:
    parameters and Adam's state come back bit for bit, and both networks then take the same
    steps (equal up to the float-atomic order of the gradient sums)."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(2)
    inp = torch.rand((2, 32, 32, 10), device="cuda", generator=g)
    tgt = 0.8 * inp[..., 3:6] * inp[..., 4:5] + 0.1
    path = str(tmp_path / "unet.ckpt")
    with PathTracingRenderer(0) as r1, PathTracingRenderer(0) as r2:
        a = Unet(r1, seed=5)
        for _ in range(5):
            a.train_step(inp, tgt, 1e-3)
        a.save(path)
        pa, (ma, va, sa) = a.params(), a.optimizer_state()
        assert sa == 5
        b = Unet(r2, seed=11)
        assert not np.array_equal(b.params(), pa)
        b.load(path)
        mb, vb, sb = b.optimizer_state()
        assert np.array_equal(b.params().view(np.uint32), pa.view(np.uint32))
        assert np.array_equal(mb.view(np.uint32), ma.view(np.uint32)) and np.array_equal(vb.view(np.uint32),
                                                                                          va.view(np.uint32))
        assert sb == sa
        la = [a.train_step(inp, tgt, 1e-3) for _ in range(3)]
        lb = [b.train_step(inp, tgt, 1e-3) for _ in range(3)]
        np.testing.assert_allclose(la, lb, rtol=1e-3)
        np.testing.assert_allclose(b.params(), a.params(), rtol=1e-3, atol=1e-5)
        assert b.optimizer_state()[2] == 8


def test_training_on_crops_lowers_the_loss():
    """The C5 training path at a small size: a crop set rendered by the path tracer (4 family
    views at 512^2 cut into 16 crops of 128^2, 256-spp targets, two 1-spp inputs each), then
    300 Adam steps of the library's training kernels on random crops."""
    torch = _torch()
    from gknextengine_gb300.denoiser import Unet, build_crop_set, train_crops
    with PathTracingRenderer(0) as r:
        inputs, targets, info = build_crop_set(r, views=4, view_size=512, crop=128, ref_spp=256, inputs_per_crop=2)
        assert inputs.shape == (64, 2, 128, 128, 10) and targets.shape == (64, 128, 128, 3)
        assert torch.isfinite(targets).all() and float(targets.mean()) > 0.0
        # two 1-spp inputs of a crop are independent samples of its target
        assert not torch.equal(inputs[:, 0, ..., :3], inputs[:, 1, ..., :3])
        net = Unet(r, seed=7)
        losses = train_crops(net, inputs, targets, 300, batch=4)
        assert np.mean(losses[-30:]) < 0.5 * np.mean(losses[:10]), (np.mean(losses[:10]), np.mean(losses[-30:]))


def test_denoiser_beats_bilateral():
    """The shipped network (trained by train_c5 on 2048 crops of 256^2 with 4096-spp targets,
    Cornell-family views only) on a 1920 x 1080 frame of the C2 brick scene, a scene family it
    has never seen (1.03 M triangles, GGX metals and mixtures, 64 emissive bricks, 8 bounces):
    RelMSE against 4096 spp at most 0.8 x the reference's joint bilateral filter on the same
    1-spp frame, in at most 1.5 x its frame time (trace + reproject + JBF against trace + the
    learned denoise pass, CUDA events)."""
    from gknextengine_gb300.denoiser import evaluate_view, load_c5
    with PathTracingRenderer(0) as r:
        net = load_c5(r)
        sc, cam, st = scenes.bricks()
        ev = evaluate_view(r, net, sc, cam, st, "c2 bricks", 1920, 1080, ref_spp=4096)
        print(ev)
        assert ev["learned_1spp"] <= 0.8 * ev["bilateral_1spp"], ev
        assert ev["learned_1spp"] < ev["raw_1spp"]
        assert ev["frame_time_ratio"] <= 1.5, ev
