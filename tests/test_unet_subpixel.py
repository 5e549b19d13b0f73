"""The sub-pixel form of the denoiser's first decoder convolution, which the inference forward
runs (unet.cu): a 3x3 convolution over a nearest-upsampled input equals, per output parity, a
half-resolution 3x3 convolution whose tap weights are sums of the full-resolution taps. Exact
in FP64 with the oracle's weight-combination rule (the rule of the CUDA kernel), including the
zero padding at every border; with bf16 storage the inference output stays within bf16
rounding of the training forward."""
import numpy as np

from oracle import unet_ref as U


def test_subpixel_convolution_is_exact():
    rng = np.random.default_rng(7)
    for B, h, w in ((1, 5, 7), (2, 4, 4), (1, 1, 3)):
        x = rng.normal(size=(B, h, w, 64))
        W = rng.normal(size=(32, 3, 3, 96))
        ref = U.conv(U.up(x), W[..., :64])
        got, _ = U.subpixel_conv(x, U.subpixel_weights(W))
        assert got.shape == ref.shape
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)


def test_subpixel_weights_sum_every_tap_once_per_parity():
    W = np.ones((32, 3, 3, 96))
    Wup = U.subpixel_weights(W)
    for par in range(4):
        assert Wup[par * 32:(par + 1) * 32].sum(axis=(1, 2)).min() == 9.0   # 9 taps per output
    # parity (0, 0) reads offsets -1 and 0 along each axis (weights 1 and 2), never +1
    w00 = Wup[0, :, :, 0]
    np.testing.assert_array_equal(w00, [[1, 2, 0], [2, 4, 0], [0, 0, 0]])


def test_inference_forward_within_bf16_rounding_of_training_forward():
    rng = np.random.default_rng(11)
    B, H, W = 1, 16, 24
    inp = np.zeros((B, H, W, 10))
    inp[..., :3] = rng.exponential(0.5, (B, H, W, 3))
    inp[..., 3:6] = rng.uniform(0.1, 0.9, (B, H, W, 3))
    n = rng.normal(size=(B, H, W, 3))
    inp[..., 6:9] = n / np.linalg.norm(n, axis=-1, keepdims=True)
    inp[..., 9] = rng.uniform(0.9, 1.0, (B, H, W))
    params = rng.normal(0.0, 0.05, U.param_count()).astype(np.float32)
    y_train, c_train = U.forward(params.astype(np.float64), inp)
    y_inf, c_inf = U.forward(params.astype(np.float64), inp, inference=True)
    # dec0a differs by bf16 rounding of the summed weights and of the parity outputs
    d = c_inf["d0a"] - c_train["d0a"]
    assert np.abs(d).max() <= 2 ** -6 * np.abs(c_train["d0a"]).max()
    assert np.linalg.norm(y_inf - y_train) < 1e-2 * np.linalg.norm(y_train)
