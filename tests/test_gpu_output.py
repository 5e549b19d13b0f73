"""Output stage on the GPU against the oracle, word for word: the resolve blit and the FSR
compose of arbitrary images (values outside [0, 1] and a NaN included) and of a rendered,
denoised Cornell frame, over scales up and down, letterboxed and clipped rectangles; and the
screenshot crop."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, imageio, native, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O

pytestmark = pytest.mark.gpu

W, H = 200, 120


@pytest.fixture(scope="module")
def r():
    sc, cam, st = scenes.cornell()
    r = PathTracingRenderer(0)
    r.load_scene(sc)
    r.create_swap_chain(W, H)
    yield r, cam, st
    r.close()


def words(bgra):
    return bgra.view(np.uint32).reshape(bgra.shape[:2])


CASES = [
    # (mode, presentation w x h, offset, size)
    (abi.OUTPUT_RESOLVE, (W, H), (0, 0), None),
    (abi.OUTPUT_RESOLVE, (480, 300), (0, 0), None),
    (abi.OUTPUT_RESOLVE, (480, 300), (40, 15), (400, 240)),
    (abi.OUTPUT_RESOLVE, (90, 70), (0, 0), None),
    (abi.OUTPUT_RESOLVE, (256, 160), (-37, -20), (300, 190)),
    (abi.OUTPUT_FSR, (W, H), (0, 0), None),
    (abi.OUTPUT_FSR, (W, H), (13, -5), (W, H)),
    (abi.OUTPUT_FSR, (480, 300), (0, 0), (W, H)),
    (abi.OUTPUT_FSR, (517, 283), (240, 150), (W, H)),
    (abi.OUTPUT_FSR, (150, 90), (0, 0), (W, H)),
]


@pytest.mark.parametrize("mode,osize,off,size", CASES)
def test_output_random_image(r, mode, osize, off, size):
    r, cam, st = r
    rng = np.random.default_rng(hash((mode, osize, off)) & 0xFFFF)
    img = rng.uniform(-0.1, 1.1, (H, W, 4)).astype(np.float32)
    img[rng.integers(0, H), rng.integers(0, W), 1] = np.nan
    r.write_image(abi.IMG_DENOISED, img)
    r.output_resize(*osize)
    r.output_pass(mode, off, size)
    g = words(r.read_output())
    o = (O.output_resolve if mode == abi.OUTPUT_RESOLVE else O.output_fsr)(img, osize[0], osize[1], off, size)
    bad = np.argwhere(g != o)
    assert bad.size == 0, (len(bad), bad[:4], g[tuple(bad[0])] if len(bad) else None)


def test_output_of_a_rendered_frame(r, tmp_path):
    r, cam, st = r
    st.flags = 0
    fb = camera.FrameBuilder(W, H, st)
    for k in range(3):
        r.render(fb.build(cam, k))
    r.synchronize()
    den = r.read_image(abi.IMG_DENOISED)
    assert np.isfinite(den).all() and den[..., :3].max() > 0.01
    r.output_resize(640, 400)
    r.output_pass(abi.OUTPUT_RESOLVE, (0, 8), (640, 384))
    g = words(r.read_output())
    assert np.array_equal(g, O.output_resolve(den, 640, 400, (0, 8), (640, 384)))
    assert np.all(g[:8] == 0) and np.all(g[392:] == 0)   # letterbox bars stay black
    r.output_pass(abi.OUTPUT_FSR, (0, 0), (W, H))
    g2 = words(r.read_output())
    o2 = O.output_fsr(den, 640, 400, (0, 0), (W, H), out=O.output_resolve(den, 640, 400, (0, 8), (640, 384)))
    assert np.array_equal(g2, o2)
    # screenshot: a crop as R, G, B bytes, and the PNG written from it
    s = r.save_screenshot(str(tmp_path / "shot.png"), 100, 50, 300, 200)
    assert np.array_equal(s, O.screenshot(g2, 100, 50, 300, 200))
    assert np.array_equal(imageio.decode_png((tmp_path / "shot.png").read_bytes()), s)
    full = r.screenshot()
    assert full.shape == (400, 640, 3) and np.array_equal(full, O.screenshot(g2, 0, 0, 640, 400))
    hdr = r.save_hdr(str(tmp_path / "linear.pfm"))
    assert np.array_equal(imageio.read_pfm(str(tmp_path / "linear.pfm")), hdr[..., :3])


def test_output_errors_are_status_codes(r):
    r, cam, st = r
    r.output_resize(64, 64)
    with pytest.raises(native.GkrtError):
        r.screenshot(60, 0, 8, 8)                       # crop leaves the image
    with pytest.raises(native.GkrtError):
        r.output_pass(abi.OUTPUT_RESOLVE, source=abi.IMG_MOTION)   # not an RGBA32F image
    with pytest.raises(native.GkrtError):
        r.output_pass(7)                                 # unknown mode
    r.output_resize(0, 0)
    with pytest.raises(native.GkrtError):
        r.output_pass(abi.OUTPUT_RESOLVE, size=(8, 8))   # no presentation image
    assert r.stats().device_error == 0
