"""Frame constants (NextEngine::GetUniformBufferObject, src/Runtime/Engine.cpp:736-849) as
FrameBuilder builds them, checked by the properties the reference's matrices have:

* glm::perspective with GLM_FORCE_DEPTH_ZERO_TO_ONE (src/Utilities/Glm.hpp:3): depth 0 at the
  near plane (0.2) and 1 at the far plane (2000), Y flipped (Projection[1][1] *= -1);
* the camera ray of a pixel centre (ProjectionInverse, ModelViewInverse) lands on that pixel
  under ViewProjection, and the inverses are inverses;
* the TAA jitter: Halton (2, 3) point (TotalFrames % TemporalFrames) + 1 (Engine.cpp:654-662,
  772-778), placed in Projection[2][0..1], moves NDC by -2 * jitter / size; the unjittered
  matrices ignore it; for eight temporal frames the points are the shader's table
  (Shading.slang:4-13) to its four decimals;
* last frame's view-projection is kept only when last frame's TotalFrames was not zero
  (Engine.cpp:786-787, prevUBO_ zeroed before the first frame);
* the settings rules: SunColor = intensity * (1, 1, 1, 0), HasSun needs an intensity, a
  progressive render reports 256 temporal frames."""
import math

import numpy as np
import pytest

from gknextengine_gb300 import camera

W, H = 320, 180


def m4(a):
    """A column-major float[16] as a float64 math matrix."""
    return np.asarray(list(a), np.float64).reshape(4, 4).T


def cam0():
    return camera.Camera(eye=(1.0, 2.0, 6.0), center=(0.2, 0.8, 0.0), fov_deg=45.0)


def test_projection_depth_range_and_flip():
    fc = camera.FrameBuilder(W, H, camera.Settings()).build(cam0(), 3)
    P = m4(fc.projection)
    for z, depth in ((-0.2, 0.0), (-2000.0, 1.0)):
        c = P @ np.array([0.0, 0.0, z, 1.0])
        assert c[2] / c[3] == pytest.approx(depth, abs=1e-6)
    c = P @ np.array([0.0, 1.0, -5.0, 1.0])            # up in view space is -y in clip space
    assert c[1] / c[3] < 0.0
    f = 1.0 / math.tan(math.radians(45.0) / 2.0)
    assert P[1, 1] == pytest.approx(-f, rel=1e-6) and P[0, 0] == pytest.approx(f * H / W, rel=1e-6)


@pytest.mark.parametrize("taa", [False, True])
def test_pixel_rays_land_on_their_pixels(taa):
    st = camera.Settings(taa=taa, temporal_frames=8)
    fc = camera.FrameBuilder(W, H, st).build(cam0(), 5)
    MVI, PI, VP = m4(fc.model_view_inverse), m4(fc.projection_inverse), m4(fc.view_projection)
    np.testing.assert_allclose(MVI @ m4(fc.model_view), np.eye(4), atol=1e-5)
    np.testing.assert_allclose(PI @ m4(fc.projection), np.eye(4), atol=1e-5)
    eye = (MVI @ np.array([0.0, 0.0, 0.0, 1.0]))[:3]
    np.testing.assert_allclose(eye, cam0().eye, atol=1e-5)
    for x, y in ((0, 0), (W - 1, H - 1), (W // 2, 17), (111, H - 40)):
        # TracePrimaryRay without the jitter term: the jitter lives in the projection here
        u, v = x / W * 2.0 - 1.0, y / H * 2.0 - 1.0
        t = PI @ np.array([u, v, 1.0, 1.0])
        d = (MVI @ np.array([*(t[:3] / np.linalg.norm(t[:3])), 0.0]))[:3]
        p = VP @ np.array([*(eye + 7.0 * d), 1.0])
        np.testing.assert_allclose(p[:2] / p[3], (u, v), atol=1e-5)


def test_taa_jitter_follows_the_halton_table():
    st = camera.Settings(taa=True, temporal_frames=8)
    fb = camera.FrameBuilder(W, H, st)
    table = [(0.5, 0.3333), (0.25, 0.6667), (0.75, 0.1111), (0.125, 0.4444), (0.625, 0.7778),
             (0.375, 0.2222), (0.875, 0.5556), (0.0625, 0.8889)]
    for k in range(12):
        fc = fb.build(cam0(), k)
        P, Pu = m4(fc.projection), m4(fc.view_projection_unjit) @ np.linalg.inv(m4(fc.model_view))
        hx, hy = table[k % 8]
        assert P[0, 2] == pytest.approx((hx - 0.5) / W * 2.0, abs=1e-4 / W)
        assert P[1, 2] == pytest.approx((hy - 0.5) / H * 2.0, abs=1e-4 / H)
        assert abs(Pu[0, 2]) < 1e-6 and abs(Pu[1, 2]) < 1e-6      # float32 rounding only
        q = np.array([0.3, -0.2, -9.0, 1.0])
        a, b = P @ q, Pu @ q
        # the entries multiply view z, negative in front of the camera (w = -z): NDC moves by -entry
        np.testing.assert_allclose(a[:2] / a[3] - b[:2] / b[3], (-P[0, 2], -P[1, 2]), rtol=1e-4, atol=1e-6)


def test_previous_view_projection_rule():
    fb = camera.FrameBuilder(W, H, camera.Settings())
    cams = [cam0().orbit(3.0 * k) for k in range(5)]
    fcs = [fb.build(c, k) for k, c in enumerate(cams)]
    for k, fc in enumerate(fcs):
        keep = k >= 2                    # frames 0 and 1: last TotalFrames was zero
        want = fcs[k - 1].view_projection_unjit if keep else fc.view_projection_unjit
        np.testing.assert_array_equal(list(fc.prev_view_projection_unjit), list(want))
        want = fcs[k - 1].view_projection if keep else fc.view_projection
        np.testing.assert_array_equal(list(fc.prev_view_projection), list(want))
    # a reset (scene load: TotalFrames back to 0) keeps the history on its own frame (last
    # frame's TotalFrames was 4) and drops it on the next
    a = fb.build(cams[0], 0)
    np.testing.assert_array_equal(list(a.prev_view_projection), list(fcs[4].view_projection))
    b = fb.build(cams[1], 1)
    np.testing.assert_array_equal(list(b.prev_view_projection), list(b.view_projection))
    c = fb.build(cams[2], 2)
    np.testing.assert_array_equal(list(c.prev_view_projection), list(b.view_projection))


def test_settings_rules():
    fb = camera.FrameBuilder(W, H, camera.Settings(has_sun=True, sun_intensity=0.0, progressive=True,
                                                   sun_direction=(0.0, 2.0, 0.0)))
    fc = fb.build(cam0(), 0)
    assert fc.has_sun == 0 and fc.temporal_frames == 256
    fc = camera.FrameBuilder(W, H, camera.Settings(has_sun=True, sun_intensity=3.5,
                                                   sun_direction=(1.0, 1.0, 0.0))).build(cam0(), 0)
    assert fc.has_sun == 1 and list(fc.sun_color) == [3.5, 3.5, 3.5, 0.0]
    np.testing.assert_allclose(list(fc.sun_direction), [math.sqrt(0.5), math.sqrt(0.5), 0.0, 0.0], atol=1e-7)


def test_reference_defaults():
    s = camera.Settings.reference_defaults()
    assert (s.samples, s.bounces, s.max_bounces, s.temporal_frames, s.taa) == (8, 5, 10, 16, True)
    assert (s.bf_size, s.bf_sigma, s.bf_sigma_lum, s.bf_sigma_normal, s.paper_white_nit) == (5, 2.0, 3.0, 0.005, 600.0)
    assert not s.fast_gather
