"""Output stage on the CPU: the oracle's resolve blit, FSR compose and screenshot crop on
properties that pin them (identity scale, constant images, clipping, UNORM rounding), the
resolve blit against an independent numpy restatement, and the PNG / PFM writers."""
import numpy as np
import pytest

from gknextengine_gb300 import imageio
from oracle import oracle as O


def quantize(img):
    """UNORM8 of an (h, w, 4) float image as BGRA words (clamp, NaN to 0, x 255, ties to even)."""
    v = np.nan_to_num(np.asarray(img, np.float32), nan=0.0, posinf=1.0, neginf=0.0)
    q = np.rint(np.clip(v, 0.0, 1.0) * np.float32(255.0)).astype(np.uint32)
    return q[..., 2] | (q[..., 1] << 8) | (q[..., 0] << 16) | (q[..., 3] << 24)


def blit_numpy(src, out_w, out_h, ox, oy, ow, oh):
    """The scaled linear blit restated with numpy float32 arithmetic, same operation order."""
    H, W = src.shape[:2]
    out = np.zeros((out_h, out_w), np.uint32)
    f = np.float32
    su, sv = f(W) / f(ow), f(H) / f(oh)
    xs = np.arange(max(ox, 0), min(ox + ow, out_w))
    ys = np.arange(max(oy, 0), min(oy + oh, out_h))
    if xs.size == 0 or ys.size == 0:
        return out
    u = ((xs - ox).astype(np.float32) + f(0.5)) * su - f(0.5)
    v = ((ys - oy).astype(np.float32) + f(0.5)) * sv - f(0.5)
    fu, fv = np.floor(u), np.floor(v)
    a, b = (u - fu)[None, :, None], (v - fv)[:, None, None]
    i0, j0 = fu.astype(np.int64), fv.astype(np.int64)
    ia, ib = np.clip(i0, 0, W - 1), np.clip(i0 + 1, 0, W - 1)
    ja, jb = np.clip(j0, 0, H - 1), np.clip(j0 + 1, 0, H - 1)
    one = f(1.0)
    w00, w10, w01, w11 = (one - a) * (one - b), a * (one - b), (one - a) * b, a * b
    t = lambda jj, ii: src[jj][:, ii]
    c = ((t(ja, ia) * w00 + t(ja, ib) * w10) + t(jb, ia) * w01) + t(jb, ib) * w11
    out[np.ix_(ys, xs)] = quantize(c.astype(np.float32))
    return out


@pytest.fixture(scope="module")
def img():
    rng = np.random.default_rng(11)
    a = rng.uniform(-0.2, 1.2, (45, 64, 4)).astype(np.float32)
    a[3, 5, 1] = np.nan
    a[7, 9, 0] = np.inf
    return a


def test_unorm_rounding_ties_to_even():
    # (an infinite texel meets a zero filter weight, inf * 0 = NaN, and stores 0: not listed)
    vals = [0.5 / 255, 1.5 / 255, 2.5 / 255, 254.5 / 255, -1.0, 2.0, np.nan, 1.0]
    got = []
    for v in vals:   # one texel per blit: every filter tap is that texel
        a = np.array([[[v, 0.0, 0.0, 1.0]]], np.float32)
        w = O.output_resolve(a, 1, 1)
        assert w[0, 0] == quantize(a)[0, 0]
        got.append(int(w[0, 0] >> 16) & 0xFF)
    assert got == [0, 2, 2, 254, 0, 255, 0, 255]


def test_resolve_identity_is_the_quantized_image(img):
    clean = np.nan_to_num(img, nan=0.5, posinf=0.5)
    assert np.array_equal(O.output_resolve(clean, 64, 45), quantize(clean))
    # zero-weight taps still multiply: a NaN texel reaches its right and lower neighbours
    w = O.output_resolve(img, 64, 45)
    assert ((w[3, 5] >> 8) & 0xFF) == 0


@pytest.mark.parametrize("out_w,out_h,off,size", [
    (128, 90, (0, 0), None),              # 2x up
    (200, 120, (20, 7), (160, 106)),      # letterboxed, non-integer scale
    (40, 30, (0, 0), None),               # down
    (100, 80, (-30, -11), (120, 70)),     # partly off the image (clipped)
    (64, 45, (90, 3), (10, 10)),          # wholly off the image
])
def test_resolve_matches_numpy(img, out_w, out_h, off, size):
    w, h = size if size is not None else (out_w, out_h)
    o = O.output_resolve(img, out_w, out_h, off, (w, h))
    assert np.array_equal(o, blit_numpy(img, out_w, out_h, off[0], off[1], w, h))


def test_fsr_constant_image_stays_constant():
    c = np.empty((30, 40, 4), np.float32)
    c[...] = (0.25, 0.5, 0.75, 1.0)
    o = O.output_fsr(c, 72, 54)
    covered = o[:48, :72]                 # 54 / 8 * 8 rows, 72 / 8 * 8 columns
    assert np.all(covered == quantize(c)[0, 0])
    assert np.all(o[48:] == 0)


def test_fsr_same_size_is_a_copy_of_the_dispatch(img):
    o = O.output_fsr(img, 64, 45)
    q = quantize(img)
    assert np.array_equal(o[:40, :64], q[:40, :64]) and np.all(o[40:] == 0)
    # with offsets: pixels land shifted, those pushed past the edge are dropped
    o2 = O.output_fsr(img, 64, 45, offset=(5, -3), size=(64, 45))
    assert np.array_equal(o2[0:37, 5:64], q[3:40, 0:59])


def test_fsr_upscale_is_bounded_by_its_neighbourhood():
    rng = np.random.default_rng(3)
    a = rng.uniform(0.0, 1.0, (24, 32, 4)).astype(np.float32)
    o = O.output_fsr(a, 80, 60)[:56, :80]
    lo, hi = quantize(np.full((1, 1, 4), 0.0, np.float32)), quantize(np.full((1, 1, 4), 1.0, np.float32))
    for sh in (16, 8, 0):
        ch = (o >> sh) & 0xFF
        assert ch.min() >= ((lo >> sh) & 0xFF).min() and ch.max() <= ((hi >> sh) & 0xFF).max()
    # deringing: every output lies within min/max of the source (0..255 after quantization)
    src_q = quantize(a)
    for sh in (16, 8, 0):
        assert ((o >> sh) & 0xFF).max() <= ((src_q >> sh) & 0xFF).max()
        assert ((o >> sh) & 0xFF).min() >= ((src_q >> sh) & 0xFF).min()


def test_screenshot_crop_byte_order(img):
    w = O.output_resolve(img, 64, 45)
    s = O.screenshot(w, 10, 4, 20, 9)
    crop = w[4:13, 10:30]
    assert np.array_equal(s[..., 0], (crop >> 16) & 0xFF)
    assert np.array_equal(s[..., 1], (crop >> 8) & 0xFF)
    assert np.array_equal(s[..., 2], crop & 0xFF)


def test_png_round_trip(tmp_path):
    rng = np.random.default_rng(5)
    for c in (3, 4):
        a = rng.integers(0, 256, (17, 23, c), dtype=np.uint8)
        p = tmp_path / f"x{c}.png"
        imageio.write_png(str(p), a)
        assert np.array_equal(imageio.decode_png(p.read_bytes()), a)


def test_pfm_round_trip(tmp_path):
    rng = np.random.default_rng(6)
    a = rng.normal(size=(9, 13, 4)).astype(np.float32)
    p = tmp_path / "x.pfm"
    imageio.write_pfm(str(p), a)
    assert np.array_equal(imageio.read_pfm(str(p)), a[..., :3])
