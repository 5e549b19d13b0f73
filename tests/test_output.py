"""Output stage on the CPU: the oracle's resolve blit, FSR compose and screenshot crop on
properties that pin them (identity scale, constant images, clipping, UNORM rounding), the
resolve blit and the FSR EASU against independent numpy restatements (vectorised float32 in
the same operation order), and the PNG / PFM writers."""
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


def easu_numpy(src, out_w, out_h, outw, outh, offx=0, offy=0):
    """Process.UpScaleFSR.comp.slang (EASU, different sizes) restated with numpy float32 in the
    shader's operation order; fmin/fmax ignore NaN as the GPU's min/max do."""
    f = np.float32
    H, W = src.shape[:2]
    Wf, Hf, OWf, OHf = f(W), f(H), f(out_w), f(out_h)
    gw, gh = (outw // 8) * 8, (outh // 8) * 8
    ys, xs = np.meshgrid(np.arange(gh), np.arange(gw), indexing="ij")
    ipx = (xs.astype(f) / f(outw)) * OWf
    ipy = (ys.astype(f) / f(outh)) * OHf
    c0 = (Wf / OWf, Hf / OHf, f(0.5) * Wf / OWf - f(0.5), f(0.5) * Hf / OHf - f(0.5))
    c1 = (f(1) / Wf, f(1) / Hf, f(1) / Wf, f(-1) / Hf)
    c2 = (f(-1) / Wf, f(2) / Hf, f(1) / Wf, f(2) / Hf)
    c3 = (f(0) / Wf, f(4) / Hf)
    ppx, ppy = ipx * c0[0] + c0[2], ipy * c0[1] + c0[3]
    fpx, fpy = np.floor(ppx), np.floor(ppy)
    ppx, ppy = ppx - fpx, ppy - fpy
    p0x, p0y = fpx * c1[0] + c1[2], fpy * c1[1] + c1[3]
    p1x, p1y = p0x + c2[0], p0y + c2[1]
    p2x, p2y = p0x + c2[2], p0y + c2[3]
    p3x, p3y = p0x + c3[0], p0y + c3[1]
    ox, oy, oz, ow = f(-0.5) * c1[0], f(0.5) * c1[0], f(-0.5) * c1[1], f(0.5) * c1[1]

    def cf(px, py):
        cx = np.clip((px * Wf).astype(np.int64), 0, W - 1)
        cy = np.clip((py * Hf).astype(np.int64), 0, H - 1)
        return src[cy, cx]                       # (gh, gw, 4)

    bC, cC = cf(p0x + ox, p0y + ow), cf(p0x + oy, p0y + ow)
    iC, jC = cf(p1x + ox, p1y + ow), cf(p1x + oy, p1y + ow)
    fC, eC = cf(p1x + oy, p1y + oz), cf(p1x + ox, p1y + oz)
    kC, lC = cf(p2x + ox, p2y + ow), cf(p2x + oy, p2y + ow)
    hC, gC = cf(p2x + oy, p2y + oz), cf(p2x + ox, p2y + oz)
    oC, nC = cf(p3x + oy, p3y + oz), cf(p3x + ox, p3y + oz)
    L = lambda c: c[..., 1] + f(0.5) * (c[..., 0] + c[..., 2])
    bL, cL, iL, jL, fL, eL, kL, lL, hL, gL, oL, nL = (L(c) for c in (bC, cC, iC, jC, fC, eC, kC, lC, hC, gC, oC, nC))
    sat = lambda v: np.fmin(np.fmax(v, f(0)), f(1))
    dx = np.zeros_like(ppx); dy = np.zeros_like(ppx); ln = np.zeros_like(ppx)

    def setf(w, lA, lB, lC_, lD, lE):
        nonlocal dx, dy, ln
        with np.errstate(divide="ignore", invalid="ignore"):
            lenX = np.fmax(np.abs(lD - lC_), np.abs(lC_ - lB))
            dirX = lD - lB
            dx = dx + dirX * w
            lenX = sat(np.abs(dirX) / lenX)
            lenX = lenX * lenX
            ln = ln + lenX * w
            lenY = np.fmax(np.abs(lE - lC_), np.abs(lC_ - lA))
            dirY = lE - lA
            dy = dy + dirY * w
            lenY = sat(np.abs(dirY) / lenY)
            lenY = lenY * lenY
            ln = ln + lenY * w

    one = f(1)
    setf((one - ppx) * (one - ppy), bL, eL, fL, gL, jL)
    setf(ppx * (one - ppy), cL, fL, gL, hL, kL)
    setf((one - ppx) * ppy, fL, iL, jL, kL, nL)
    setf(ppx * ppy, gL, jL, kL, lL, oL)
    dirR = dx * dx + dy * dy
    zro = dirR < f(1.0 / 32768.0)
    with np.errstate(divide="ignore", invalid="ignore"):
        dirR = f(1) / np.sqrt(dirR)
    dirR = np.where(zro, f(1), dirR).astype(f)
    dx = np.where(zro, f(1), dx).astype(f)
    dx, dy = dx * dirR, dy * dirR
    ln = ln * f(0.5)
    ln = ln * ln
    stretch = (dx * dx + dy * dy) / np.fmax(np.abs(dx), np.abs(dy))
    l2x, l2y = one + (stretch - one) * ln, one - f(0.5) * ln
    lob = f(0.5) - f(0.29) * ln
    clp = one / lob
    mn = np.fmin(np.fmin(fC, gC), np.fmin(jC, kC))
    mx = np.fmax(np.fmax(fC, gC), np.fmax(jC, kC))
    aC = np.zeros(ppx.shape + (4,), f)
    aW = np.zeros_like(ppx)
    for (tx, ty), c in (((0, -1), bC), ((1, -1), cC), ((-1, 1), iC), ((0, 1), jC), ((0, 0), fC), ((-1, 0), eC),
                        ((1, 1), kC), ((2, 1), lC), ((2, 0), hC), ((1, 0), gC), ((1, 2), oC), ((0, 2), nC)):
        offx_, offy_ = f(tx) - ppx, f(ty) - ppy
        vx = offx_ * dx + offy_ * dy
        vy = offx_ * (-dy) + offy_ * dx
        vx, vy = vx * l2x, vy * l2y
        d2 = np.fmin(vx * vx + vy * vy, clp)
        wB = f(0.4) * d2 - one
        wA = lob * d2 - one
        wB, wA = wB * wB, wA * wA
        wB = f(1.5625) * wB - f(0.5625)
        w = wB * wA
        aC = aC + c * w[..., None]
        aW = aW + w
    with np.errstate(divide="ignore", invalid="ignore"):
        q = aC / aW[..., None]
    pix = np.fmin(mx, np.fmax(mn, q)).astype(f)
    out = np.zeros((out_h, out_w), np.uint32)
    X, Y = xs + offx, ys + offy
    ok = (X >= 0) & (Y >= 0) & (X < out_w) & (Y < out_h)
    out[Y[ok], X[ok]] = quantize(pix)[ok]
    return out


@pytest.mark.filterwarnings("ignore::RuntimeWarning")   # the fixture's NaN and inf texels
@pytest.mark.parametrize("out_w,out_h,outw,outh,off", [(80, 60, 80, 60, (0, 0)), (123, 77, 123, 77, (0, 0)),
                                                        (200, 150, 64, 45, (30, 20)), (50, 40, 50, 40, (-9, 5))])
def test_fsr_matches_numpy(img, out_w, out_h, outw, outh, off):
    o = O.output_fsr(img, out_w, out_h, off, (outw, outh))
    assert np.array_equal(o, easu_numpy(img, out_w, out_h, outw, outh, *off))
