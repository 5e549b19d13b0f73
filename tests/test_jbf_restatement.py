"""The oracle's joint bilateral compose (Process.DenoiseJBF.comp.slang) against a second,
independent restatement in numpy written from the shader: 36 taps at stride 2 over the 11 x 11
window (WINDOW_R = 5, :5), +0.001 on every fetched diffuse and specular texel (FetchDiffuse /
FetchSpec, :14-22), spatial weight exp(-d^2 / 2 sigma^2) with d = clamp((i^2 + j^2) / 25, 0, 1)
and luminance weight exp(-dl^2 / 2 (100 sigma_L)^2) with dl = (L_c - L_i)^2 (JBF, :49-73), the
sum divided by the weight and remodulated by the accumulated albedo plus the centre specular
(:145-150). Reads outside the image are zero. Compared before the tone map (exp differs by
ulps between libms: relative 1e-5)."""
import numpy as np

from gknextengine_gb300 import abi, camera
from oracle import oracle as O

LUM = np.array([0.212671, 0.715160, 0.072169], np.float32)


def dot3(a, w):
    return (a[..., 0] * w[0] + a[..., 1] * w[1]) + a[..., 2] * w[2]


def jbf_numpy(diffuse, spec, albedo, sigma, sigma_lum):
    f = np.float32
    H, W = diffuse.shape[:2]
    R = 5
    D = np.pad(diffuse[..., :3], ((R, R), (R, R), (0, 0))) + f(0.001)
    S = spec[..., :3] + f(0.001)
    centre = D[R:R + H, R:R + W]
    cl = dot3(centre, LUM)
    sl = f(sigma_lum) * f(100.0)
    two_s2, two_sl2 = f(2.0) * f(sigma) * f(sigma), f(2.0) * sl * sl
    total = np.zeros((H, W, 3), f)
    weight = np.zeros((H, W), f)
    for i in range(-R, R + 1, 2):          # row offset (localCoord.x)
        for j in range(-R, R + 1, 2):      # column offset (localCoord.y)
            ci = D[R + i:R + i + H, R + j:R + j + W]
            li = dot3(ci, LUM)
            d = f(min(max(float(i * i + j * j) / 25.0, 0.0), 1.0))
            dl = (cl - li) * (cl - li)
            fi = np.exp(-d * d / two_s2).astype(f)
            wl = np.exp(-dl * dl / two_sl2).astype(f)
            total = total + (ci * fi) * wl[..., None]
            weight = weight + fi * wl
    total = total / weight[..., None]
    return total * albedo[..., :3] + S


def test_jbf_compose_matches_the_numpy_restatement():
    rng = np.random.default_rng(21)
    W, H = 53, 37
    im = O.new_images(W, H)
    im[abi.IMG_ACCUM_DIFFUSE][...] = rng.uniform(0.0, 2.0, (H, W, 4)).astype(np.float32)
    # fireflies: with sigma_L = 300 the luminance weight only bites on luminance gaps of tens
    fly = rng.random((H, W)) < 0.05
    im[abi.IMG_ACCUM_DIFFUSE][fly, :3] = rng.uniform(20.0, 60.0, (int(fly.sum()), 3)).astype(np.float32)
    im[abi.IMG_ACCUM_SPECULAR][...] = rng.uniform(0.0, 0.5, (H, W, 4)).astype(np.float32)
    im[abi.IMG_ACCUM_ALBEDO][...] = rng.uniform(0.1, 1.0, (H, W, 4)).astype(np.float32)
    n = rng.normal(size=(H, W, 3))
    im[abi.IMG_NORMAL][..., :3] = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    im[abi.IMG_OBJECT_ID][...] = rng.integers(0, 4, (H, W)).astype(np.uint32)
    st = camera.Settings(bf_size=5, bf_sigma=2.0, bf_sigma_lum=3.0)
    fc = camera.FrameBuilder(W, H, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0), fov_deg=40.0), 0)
    O.denoise_pass(fc, W, H, im)
    got = im[abi.IMG_DENOISED_LINEAR][..., :3]
    ref = jbf_numpy(im[abi.IMG_ACCUM_DIFFUSE], im[abi.IMG_ACCUM_SPECULAR], im[abi.IMG_ACCUM_ALBEDO], 2.0, 3.0)
    np.testing.assert_allclose(got, ref, rtol=1e-5, atol=1e-6)
    # the comparison is sensitive: without the luminance weight, or without the +0.001 fetch
    # offset, the restatement would not match
    flat = jbf_numpy(im[abi.IMG_ACCUM_DIFFUSE], im[abi.IMG_ACCUM_SPECULAR], im[abi.IMG_ACCUM_ALBEDO], 2.0, 1e9)
    assert np.abs(flat - got).max() > 1e-3
    assert np.abs((ref - np.float32(0.001)) - got).max() > 1e-4
