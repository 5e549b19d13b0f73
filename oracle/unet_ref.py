"""CPU oracle of the learned denoiser (test infrastructure only).

A numpy restatement of the library's U-Net (gknextengine_gb300/csrc/unet.cu): the same
layers, the same NHWC layouts, bf16 rounding at every point where the GPU stores bf16
(inputs, weights, activations, gradients), and FP64 arithmetic elsewhere, so that the GPU's
forward output and parameter gradients can be compared with tolerances set by FP32-vs-FP64
accumulation only. The reference has no learned denoiser of its own to pin this against
(its OIDN library is closed), so parity here is against this restatement.
"""
from __future__ import annotations

import numpy as np

# (cin, cout, relu) per layer: enc0a enc0b enc1a enc1b enc2a enc2b enc3a enc3b dec2a dec2b
# dec1a dec1b dec0a dec0b out
LAYERS = [(32, 32, 1), (32, 32, 1), (32, 64, 1), (64, 64, 1), (64, 96, 1), (96, 96, 1), (96, 128, 1),
          (128, 128, 1), (224, 96, 1), (96, 96, 1), (160, 64, 1), (64, 64, 1), (96, 32, 1), (32, 32, 1),
          (32, 32, 0)]


def bf16(x):
    """Round to bfloat16 (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(np.asarray(x, np.float32)).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    """Per layer (W [cout][3][3][cin], b [cout]) from the flat parameter vector."""
    out, off = [], 0
    for cin, cout, _ in LAYERS:
        n = 9 * cin * cout
        W = params[off:off + n].reshape(cout, 3, 3, cin)
        off += n
        out.append((W, params[off:off + cout]))
        off += cout
    return out


def conv(x, W):
    """3x3 same convolution, NHWC x (B, H, W, cin), W (cout, 3, 3, cin) -> (B, H, W, cout)."""
    B, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    out = np.zeros((B, H, Wd, W.shape[0]))
    for dy in range(3):
        for dx in range(3):
            out += xp[:, dy:dy + H, dx:dx + Wd, :] @ W[:, dy, dx, :].T
    return out


def conv_wgrad(dp, x):
    """dW (cout, 3, 3, cin) of conv(x, W) for output gradient dp."""
    B, H, Wd, _ = x.shape
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (0, 0)))
    dW = np.zeros((dp.shape[-1], 3, 3, x.shape[-1]))
    d2 = dp.reshape(-1, dp.shape[-1])
    for dy in range(3):
        for dx in range(3):
            dW[:, dy, dx, :] = d2.T @ xp[:, dy:dy + H, dx:dx + Wd, :].reshape(-1, x.shape[-1])
    return dW


def conv_dgrad(dp, W):
    """d input of conv(x, W): a convolution with the transposed, mirrored kernel."""
    Wf = W[:, ::-1, ::-1, :].transpose(3, 1, 2, 0)   # (cin, 3, 3, cout)
    return conv(dp, Wf)


def pool(x):
    B, H, W, C = x.shape
    return x.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4)) * 0.25


def pool_bwd(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_bwd(g):
    B, H, W, C = g.shape
    return g.reshape(B, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def pack_input(inp):
    """(B, H, W, 10) radiance, albedo, normal, depth -> the 32-channel bf16 network input."""
    x = np.zeros(inp.shape[:3] + (32,))
    x[..., :10] = inp
    x[..., :3] = np.log1p(np.maximum(inp[..., :3], 0.0))
    x[..., 9] = np.clip(inp[..., 9], 0.0, 1.0)
    return bf16(x)


def subpixel_weights(W):
    """dec0a's weights over its upsampled input channels (W (32, 3, 3, 96), channels 0-63) as a
    half-resolution convolution with 128 outputs, one group of 32 per output parity (a, b): the
    taps (dy, dx) of output pixel (2i + a, 2j + b) read the upsampled input at half-resolution
    offset (floor((a + dy) / 2), floor((b + dx) / 2)), so each half-resolution tap's weight is
    the sum of the full-resolution taps that read it (unet.cu, k_weights_subpixel)."""
    Wup = np.zeros((128, 3, 3, 64))
    for a in range(2):
        for b in range(2):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    dyl, dxl = (a + dy) // 2, (b + dx) // 2
                    Wup[(2 * a + b) * 32:(2 * a + b + 1) * 32, dyl + 1, dxl + 1, :] += W[:, dy + 1, dx + 1, :64]
    return Wup


def subpixel_conv(x_half, Wup, cout=32):
    """The full-resolution output of the parity convolution: pixel (2i + a, 2j + b) takes
    channels (2a + b) cout .. of conv(x_half, Wup) at (i, j)."""
    U = conv(x_half, Wup)
    B, h, w, _ = U.shape
    out = np.zeros((B, 2 * h, 2 * w, cout))
    for a in range(2):
        for b in range(2):
            out[:, a::2, b::2, :] = U[..., (2 * a + b) * cout:(2 * a + b + 1) * cout]
    return out, U


def forward(params, inp, inference=False):
    """Returns (y raw log-space output (B, H, W, 3), cache). inference: dec0a as the library's
    inference forward computes it (unet.cu, Unet::forward without train): the parity
    convolution of dec1b with bf16 sums of the weights, its output stored in bf16, added to the
    convolution over enc0b before the bias and ReLU."""
    P = [(bf16(W), b.astype(np.float64)) for W, b in unpack(params)]

    def layer(l, x, store=True):
        W, b = P[l]
        o = conv(x, W) + b
        if LAYERS[l][2]:
            o = np.maximum(o, 0.0)
        return bf16(o) if store else o

    c = {}
    c["x0"] = pack_input(inp)
    c["e0a"] = layer(0, c["x0"])
    c["e0b"] = layer(1, c["e0a"])
    c["p0"] = bf16(pool(c["e0b"]))
    c["e1a"] = layer(2, c["p0"])
    c["e1b"] = layer(3, c["e1a"])
    c["p1"] = bf16(pool(c["e1b"]))
    c["e2a"] = layer(4, c["p1"])
    c["e2b"] = layer(5, c["e2a"])
    c["p2"] = bf16(pool(c["e2b"]))
    c["e3a"] = layer(6, c["p2"])
    c["e3b"] = layer(7, c["e3a"])
    c["cat2"] = np.concatenate([up(c["e3b"]), c["e2b"]], -1)
    c["d2a"] = layer(8, c["cat2"])
    c["d2b"] = layer(9, c["d2a"])
    c["cat1"] = np.concatenate([up(c["d2b"]), c["e1b"]], -1)
    c["d1a"] = layer(10, c["cat1"])
    c["d1b"] = layer(11, c["d1a"])
    c["cat0"] = np.concatenate([up(c["d1b"]), c["e0b"]], -1)
    if inference:
        W32 = unpack(params)[12][0].astype(np.float32).astype(np.float64)
        u_full, _ = subpixel_conv(c["d1b"], bf16(subpixel_weights(W32)))
        # the parity outputs are stored in bf16: take the rounding per half-resolution value
        u_full = bf16(u_full)
        o = conv(c["e0b"], bf16(W32[..., 64:])) + P[12][1] + u_full
        c["d0a"] = bf16(np.maximum(o, 0.0))
    else:
        c["d0a"] = layer(12, c["cat0"])
    c["d0b"] = layer(13, c["d0a"])
    y = layer(14, c["d0b"], store=False)
    c["P"] = P
    return y[..., :3], c


def backward(c, d_raw):
    """Parameter gradients (flat, the layout of the parameter vector) for d loss / d y."""
    P = c["P"]
    grads = [None] * len(LAYERS)

    def lb(l, dy, y_act, x, want_dx=True):
        dp = dy * (y_act > 0) if LAYERS[l][2] else dy
        grads[l] = (conv_wgrad(dp, x), dp.sum(axis=(0, 1, 2)))
        return bf16(conv_dgrad(dp, P[l][0])) if want_dx else None

    gy = np.zeros(d_raw.shape[:3] + (32,))
    gy[..., :3] = bf16(d_raw)
    g = lb(14, gy, None, c["d0b"])
    g = lb(13, g, c["d0b"], c["d0a"])
    gc0 = lb(12, g, c["d0a"], c["cat0"])
    g = bf16(up_bwd(gc0[..., :64]))
    g = lb(11, g, c["d1b"], c["d1a"])
    gc1 = lb(10, g, c["d1a"], c["cat1"])
    g = bf16(up_bwd(gc1[..., :96]))
    g = lb(9, g, c["d2b"], c["d2a"])
    gc2 = lb(8, g, c["d2a"], c["cat2"])
    g = bf16(up_bwd(gc2[..., :128]))
    g = lb(7, g, c["e3b"], c["e3a"])
    g = lb(6, g, c["e3a"], c["p2"])
    g = bf16(gc2[..., 128:] + pool_bwd(g))
    g = lb(5, g, c["e2b"], c["e2a"])
    g = lb(4, g, c["e2a"], c["p1"])
    g = bf16(gc1[..., 96:] + pool_bwd(g))
    g = lb(3, g, c["e1b"], c["e1a"])
    g = lb(2, g, c["e1a"], c["p0"])
    g = bf16(gc0[..., 64:] + pool_bwd(g))
    g = lb(1, g, c["e0b"], c["e0a"])
    lb(0, g, c["e0a"], c["x0"], want_dx=False)
    return np.concatenate([np.concatenate([dW.reshape(-1), db]) for dW, db in grads])


def param_count():
    return sum(9 * ci * co + co for ci, co, _ in LAYERS)
