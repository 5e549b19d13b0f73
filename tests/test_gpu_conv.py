"""The tensor-core 3x3 convolution (gkrt_conv3x3_bf16) against torch's fp32 convolution of the
same bf16 values: odd image sizes (partial tiles, zero padding from out-of-range TMA boxes),
channel counts of the denoiser's layers, ReLU, bias, channel offsets into a wider tensor,
fp32 output."""
import ctypes as C

import numpy as np
import pytest

from gknextengine_gb300 import abi, native

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    assert torch.cuda.is_available()
    return torch


def conv(x, w, bias, cout, out, out_c, out_off, n_store=0, flags=0):
    L = native.load()
    B, H, W, cin = x.shape
    rc = L.gkrt_conv3x3_bf16(C.c_void_p(x.data_ptr()), B, H, W, cin, C.c_void_p(w.data_ptr()),
                             C.c_void_p(bias.data_ptr() if bias is not None else 0), cout,
                             C.c_void_p(out.data_ptr()), out_c, out_off, n_store, flags, None)
    assert rc == abi.GKRT_OK, rc


@pytest.mark.parametrize("B,H,W,cin,cout,relu", [(2, 37, 45, 64, 96, True), (1, 64, 64, 32, 32, False),
                                                  (1, 24, 40, 224, 96, True), (1, 17, 33, 160, 64, True),
                                                  (3, 8, 16, 96, 128, False), (1, 20, 20, 128, 256, True),
                                                  # halo tiles (Cout <= 64, weights <= 96 KB): partial
                                                  # 8 x 16 tiles, several chunks, images
                                                  (2, 37, 45, 96, 32, True), (1, 19, 23, 32, 64, False),
                                                  (1, 40, 24, 64, 64, True), (2, 9, 7, 32, 48, False)])
def test_conv_matches_torch(B, H, W, cin, cout, relu):
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(B * 1000 + cin + cout)
    x = torch.randn((B, H, W, cin), device="cuda", generator=g).bfloat16()
    w = (torch.randn((cout, 3, 3, cin), device="cuda", generator=g) / (3 * cin ** 0.5)).bfloat16()
    bias = torch.randn(cout, device="cuda", generator=g) * 0.1
    out_c, off = cout + 32, 16
    out = torch.full((B, H, W, out_c), 7.0, device="cuda").bfloat16()
    conv(x, w, bias, cout, out, out_c, off, flags=1 if relu else 0)
    torch.cuda.synchronize()
    ref = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), w.float().permute(0, 3, 1, 2), bias, padding=1)
    if relu:
        ref = torch.relu(ref)
    ref = ref.permute(0, 2, 3, 1)
    got = out[..., off:off + cout].float()
    torch.testing.assert_close(got, ref.bfloat16().float(), rtol=2e-2, atol=2e-2)
    # channels outside the written range are untouched
    assert bool((out[..., :off].float() == 7.0).all()) and bool((out[..., off + cout:].float() == 7.0).all())


@pytest.mark.parametrize("B,H,W,cin,cout", [(2, 37, 45, 32, 32), (1, 19, 23, 96, 32), (1, 24, 40, 64, 64),
                                            (2, 17, 33, 32, 48)])
def test_conv_fused_pool_and_upsample(B, H, W, cin, cout):
    """The epilogue's extra outputs (the denoiser's skip tensors) equal the same values computed
    from the convolution's own bf16 output: the 2x2 average ((a + b) + c) + d times 1/4 rounded to
    bf16, bit for bit, and the nearest upsampling; neighbouring channels stay untouched."""
    torch = _torch()
    L = native.load()
    g = torch.Generator(device="cuda").manual_seed(B * 7 + cin + cout + H)
    x = torch.randn((B, H, W, cin), device="cuda", generator=g).bfloat16()
    w = (torch.randn((cout, 3, 3, cin), device="cuda", generator=g) / (3 * cin ** 0.5)).bfloat16()
    bias = torch.randn(cout, device="cuda", generator=g) * 0.1
    out_c, off, pc, po, uc, uo = cout + 32, 16, cout + 24, 16, cout + 8, 8
    out = torch.full((B, H, W, out_c), 3.0, device="cuda").bfloat16()
    pool = torch.full((B, H // 2, W // 2, pc), 5.0, device="cuda").bfloat16()
    up = torch.full((B, 2 * H, 2 * W, uc), 6.0, device="cuda").bfloat16()
    rc = L.gkrt_conv3x3_bf16_fused(C.c_void_p(x.data_ptr()), B, H, W, cin, C.c_void_p(w.data_ptr()),
                                   C.c_void_p(bias.data_ptr()), cout, C.c_void_p(out.data_ptr()), out_c, off, 1,
                                   C.c_void_p(pool.data_ptr()), pc, po, C.c_void_p(up.data_ptr()), uc, uo, None)
    assert rc == abi.GKRT_OK, rc
    torch.cuda.synchronize()
    y = out[..., off:off + cout]
    ref = torch.relu(torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), w.float().permute(0, 3, 1, 2), bias,
                                                padding=1)).permute(0, 2, 3, 1)
    torch.testing.assert_close(y.float(), ref.bfloat16().float(), rtol=2e-2, atol=2e-2)
    yf = y.float()[:, :2 * (H // 2), :2 * (W // 2)]
    avg = ((((yf[:, 0::2, 0::2] + yf[:, 0::2, 1::2]) + yf[:, 1::2, 0::2]) + yf[:, 1::2, 1::2]) * 0.25).bfloat16()
    assert torch.equal(pool[..., po:po + cout], avg)
    rep = y.repeat_interleave(2, dim=1).repeat_interleave(2, dim=2)
    assert torch.equal(up[..., uo:uo + cout], rep)
    assert bool((pool[..., :po].float() == 5.0).all()) and bool((pool[..., po + cout:].float() == 5.0).all())
    assert bool((up[..., :uo].float() == 6.0).all()) and bool((up[..., uo + cout:].float() == 6.0).all())
    assert bool((out[..., :off].float() == 3.0).all()) and bool((out[..., off + cout:].float() == 3.0).all())


def test_conv_f32_output_subset():
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(3)
    B, H, W, cin, cout = 2, 19, 29, 32, 16
    x = torch.randn((B, H, W, cin), device="cuda", generator=g).bfloat16()
    w = (torch.randn((cout, 3, 3, cin), device="cuda", generator=g) / 17.0).bfloat16()
    out = torch.full((B, H, W, 4), -5.0, device="cuda")
    conv(x, w, None, cout, out, 4, 0, n_store=3, flags=2)
    torch.cuda.synchronize()
    ref = torch.nn.functional.conv2d(x.float().permute(0, 3, 1, 2), w.float().permute(0, 3, 1, 2), padding=1)
    ref = ref.permute(0, 2, 3, 1)[..., :3]
    torch.testing.assert_close(out[..., :3], ref, rtol=1e-4, atol=1e-4)
    assert bool((out[..., 3] == -5.0).all())


def test_conv_rejects_bad_shapes():
    torch = _torch()
    x = torch.zeros((1, 8, 16, 48), device="cuda").bfloat16()   # cin not a multiple of 32
    w = torch.zeros((16, 3, 3, 48), device="cuda").bfloat16()
    out = torch.zeros((1, 8, 16, 16), device="cuda").bfloat16()
    L = native.load()
    rc = L.gkrt_conv3x3_bf16(C.c_void_p(x.data_ptr()), 1, 8, 16, 48, C.c_void_p(w.data_ptr()), None, 16,
                             C.c_void_p(out.data_ptr()), 16, 0, 0, 0, None)
    assert rc == abi.GKRT_ERR_INVALID_ARG


@pytest.mark.parametrize("B,H,W,cin,cout", [(2, 37, 45, 64, 96), (1, 64, 64, 32, 32), (1, 24, 40, 224, 96),
                                             (3, 16, 16, 160, 64), (1, 33, 17, 96, 128)])
def test_wgrad_matches_torch(B, H, W, cin, cout):
    """gkrt_conv3x3_wgrad_bf16 against torch's weight gradient of the same bf16 values."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(B * 7 + cin + cout)
    x = torch.randn((B, H, W, cin), device="cuda", generator=g).bfloat16()
    dy = torch.randn((B, H, W, cout), device="cuda", generator=g).bfloat16()
    dw = torch.zeros((cout, 3, 3, cin), device="cuda")
    L = native.load()
    rc = L.gkrt_conv3x3_wgrad_bf16(C.c_void_p(dy.data_ptr()), C.c_void_p(x.data_ptr()), B, H, W, cin, cout,
                                   C.c_void_p(dw.data_ptr()), None)
    assert rc == abi.GKRT_OK
    torch.cuda.synchronize()
    ref = torch.nn.grad.conv2d_weight(x.float().permute(0, 3, 1, 2), (cout, cin, 3, 3),
                                      dy.float().permute(0, 3, 1, 2), padding=1).permute(0, 2, 3, 1)
    torch.testing.assert_close(dw, ref, rtol=1e-3, atol=1e-3 * float(ref.abs().max()))


def test_input_gradient_is_a_mirrored_convolution():
    """The denoiser's input gradient: the forward kernel with weights [cin][8 - tap][cout]."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(11)
    B, H, W, cin, cout = 2, 24, 40, 96, 64
    w = (torch.randn((cout, 3, 3, cin), device="cuda", generator=g) / 30).bfloat16()
    dy = torch.randn((B, H, W, cout), device="cuda", generator=g).bfloat16()
    wf = w.flip(1, 2).permute(3, 1, 2, 0).contiguous()   # [cin][3][3][cout], taps mirrored
    dx = torch.zeros((B, H, W, cin), device="cuda").bfloat16()
    conv(dy, wf, None, cin, dx, cin, 0)
    torch.cuda.synchronize()
    ref = torch.nn.grad.conv2d_input((B, cin, H, W), w.float().permute(0, 3, 1, 2), dy.float().permute(0, 3, 1, 2),
                                     padding=1).permute(0, 2, 3, 1)
    torch.testing.assert_close(dx.float(), ref.bfloat16().float(), rtol=2e-2, atol=2e-2)
