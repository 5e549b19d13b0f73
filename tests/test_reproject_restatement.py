"""The oracle's reprojection (Process.ReProject.comp.slang) against a second, independent
restatement in numpy written from the shader: history rejected on a miss, outside the image or
while the motion moment lasts (:110-121); otherwise a 5 x 5 spatial fill of the current frame
weighted 0.4 at the centre and by normal agreement (>= 0.98) on the same object elsewhere
(calculateWeight :32-47, :123-152); the object-id-gated bilinear history clamped to [0, 1600]
(FilterHistoryColor :49-68), with the gates opened when the motion in range is below 0.1
(:154-163); the blend 1 / TemporalFrames (:211-215). Reads outside the image are zero. Compared
on rgb (the product keeps the previous alpha) within 1e-5 relative: the product and the oracle
evaluate lerp as one fma and the distance weight with reciprocals. With ProgressiveRender set
(:95-101, the engine's progressive mode, TemporalFrames 256, Engine.cpp:826) every pixel blends
the whole float4 of the history image towards the current sample by 1/512, with no rejection."""
import numpy as np

from gknextengine_gb300 import abi, camera
from oracle import oracle as O


def _at(img, y, x):
    """img[y, x] with zero outside the image (y, x integer arrays)."""
    H, W = img.shape[:2]
    ok = (y >= 0) & (y < H) & (x >= 0) & (x < W)
    out = np.zeros(y.shape + img.shape[2:], img.dtype)
    out[ok] = img[y[ok], x[ok]]
    return out


def lerp(a, b, t):
    return a + t * (b - a)


def reproject_numpy(im, temporal_frames, progressive=False):
    f = np.float32
    SD, SS, SA = im[abi.IMG_SINGLE_DIFFUSE], im[abi.IMG_SINGLE_SPECULAR], im[abi.IMG_ALBEDO]
    PD, PS, PA = im[abi.IMG_PREV_DIFFUSE], im[abi.IMG_PREV_SPECULAR], im[abi.IMG_PREV_ALBEDO]
    if progressive:   # the whole float4, history towards the sample by 1/512 (:95-101)
        k = f(min(max(1.0 / 512.0, 0.0), 1.0))
        return [lerp(P, S, k).astype(f) for P, S in ((PD, SD), (PS, SS), (PA, SA))], None
    O0, O1 = im[abi.IMG_OBJECT_ID], im[abi.IMG_OBJECT_ID_PREV]
    MV, N, MM = im[abi.IMG_MOTION], im[abi.IMG_NORMAL], im[abi.IMG_MOTION_MOMENT]
    H, W = O0.shape
    y, x = np.meshgrid(np.arange(H), np.arange(W), indexing="ij")
    mx, my = MV[..., 0], MV[..., 1]
    px, py = np.floor(x.astype(f) + mx).astype(np.int64), np.floor(y.astype(f) + my).astype(np.int64)
    inside = (px < W) & (py < H) & (px >= -1) & (py >= -1)
    cur = O0
    prev0 = _at(O1, py, px)
    use = ~((cur == 65535) | ~inside | (MM > 0))
    CN = N[..., :3]
    sd = np.zeros((H, W, 4), f); ss = np.zeros((H, W, 4), f)
    tw = np.zeros((H, W), f); mir = np.zeros((H, W), f)
    for oy in range(-2, 3):
        for ox in range(-2, 3):
            sy, sx = y + oy, x + ox
            prim = _at(O0, sy, sx)
            wn = _at(N, sy, sx)[..., :3]
            dist = f(np.sqrt(f(ox * ox + oy * oy)))
            if ox == 0 and oy == 0:
                w = np.full((H, W), f(0.4))
            else:
                nd = np.clip((wn[..., 0] * CN[..., 0] + wn[..., 1] * CN[..., 1]) + wn[..., 2] * CN[..., 2], f(0), f(1))
                w = np.where((prim == cur) & (nd >= f(0.98)),
                             ((nd - f(0.98)) / (f(1) - f(0.98))) * f(2) / (dist * f(1.5) + f(4)), f(0)).astype(f)
            sd = sd + _at(SD, sy, sx) * w[..., None]
            ss = ss + _at(SS, sy, sx) * w[..., None]
            tw = tw + w
            m2 = _at(MV, y + 2 * oy, x + 2 * ox)
            mir = mir + np.sqrt(m2[..., 0] * m2[..., 0] + m2[..., 1] * m2[..., 1])
    with np.errstate(divide="ignore", invalid="ignore"):
        sd = sd / tw[..., None]
        ss = ss / tw[..., None]
    prev1, prev2, prev3 = _at(O1, py, px + 1), _at(O1, py + 1, px), _at(O1, py + 1, px + 1)
    still = np.abs(mir) < f(0.1)
    prev = [np.where(still, cur, p) for p in (prev0, prev1, prev2, prev3)]
    subx, suby = (x.astype(f) + mx) - np.floor(x.astype(f) + mx), (y.astype(f) + my) - np.floor(y.astype(f) + my)

    def history(P, fallback):
        taps = [_at(P, py, px), _at(P, py, px + 1), _at(P, py + 1, px), _at(P, py + 1, px + 1)]
        h = [np.where((cur == p)[..., None], t[..., :3], fallback[..., :3]) for t, p in zip(taps, prev)]
        v = lerp(lerp(h[0], h[1], subx[..., None]), lerp(h[2], h[3], subx[..., None]), suby[..., None])
        return np.clip(v, f(0), f(1600))

    keep = f(min(max(1.0 / max(1, temporal_frames), 0.0), 1.0))
    out = []
    for cur_img, hist in ((SD, history(PD, sd)), (SS, history(PS, ss)), (SA, history(PA, SA))):
        acc = np.where(use[..., None], lerp(hist, cur_img[..., :3], keep), cur_img[..., :3])
        out.append(acc.astype(f))
    return out, use


def _random_inputs(rng, W, H):
    im = O.new_images(W, H)
    for k in (abi.IMG_SINGLE_DIFFUSE, abi.IMG_SINGLE_SPECULAR, abi.IMG_ALBEDO, abi.IMG_PREV_DIFFUSE,
              abi.IMG_PREV_SPECULAR, abi.IMG_PREV_ALBEDO):
        im[k][...] = rng.uniform(0.0, 3.0, (H, W, 4)).astype(np.float32)
    im[abi.IMG_PREV_DIFFUSE][3, 4, :3] = -5.0              # clamped history
    im[abi.IMG_PREV_DIFFUSE][10, 11, :3] = 5000.0
    ids = rng.integers(1, 4, (H, W)).astype(np.uint32)
    ids[rng.random((H, W)) < 0.05] = 65535                 # misses
    im[abi.IMG_OBJECT_ID][...] = ids
    prev_ids = ids.copy()
    prev_ids[rng.random((H, W)) < 0.2] = 2                 # disocclusions gate history taps
    im[abi.IMG_OBJECT_ID_PREV][...] = prev_ids
    base = np.array([0.3, 0.8, 0.52])
    n = base / np.linalg.norm(base) + rng.normal(scale=0.08, size=(H, W, 3))
    im[abi.IMG_NORMAL][..., :3] = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
    mv = rng.uniform(-3.0, 3.0, (H, W, 2)).astype(np.float32)
    mv[5:25, 5:25] = 0.0                                   # a still region: gates opened
    mv[0:3, 0:8, 0] = -6.0                                  # leaves the image on the left
    im[abi.IMG_MOTION][...] = mv
    mm = np.zeros((H, W), np.uint32)
    mm[rng.random((H, W)) < 0.1] = 7                        # moving pixels: no history
    im[abi.IMG_MOTION_MOMENT][...] = mm
    return im


def test_reproject_matches_the_numpy_restatement():
    rng = np.random.default_rng(33)
    W, H = 47, 39
    im = _random_inputs(rng, W, H)
    st = camera.Settings(temporal_frames=16)
    fc = camera.FrameBuilder(W, H, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0), fov_deg=40.0), 0)
    assert fc.progressive_render == 0 and fc.temporal_frames == 16
    (d, s, a), use = reproject_numpy(im, 16)
    O.reproject_pass(fc, W, H, im)
    for k, ref in ((abi.IMG_ACCUM_DIFFUSE, d), (abi.IMG_ACCUM_SPECULAR, s), (abi.IMG_ACCUM_ALBEDO, a)):
        np.testing.assert_allclose(im[k][..., :3], ref, rtol=1e-5, atol=1e-5, err_msg=str(k))
    assert 0.2 < use.mean() < 0.9                            # both branches exercised


def test_progressive_reproject_matches_the_numpy_restatement():
    """ProgressiveRender: a 1/512 blend of the whole float4 at every pixel, moving, missed and
    disoccluded pixels included (the oracle keeps no alpha of its own here)."""
    rng = np.random.default_rng(34)
    W, H = 45, 37
    im = _random_inputs(rng, W, H)
    st = camera.Settings(progressive=True)
    fc = camera.FrameBuilder(W, H, st).build(camera.Camera(eye=(0, 0, 3), center=(0, 0, 0), fov_deg=40.0), 0)
    assert fc.progressive_render == 1 and fc.temporal_frames == 256
    (d, s, a), _ = reproject_numpy(im, fc.temporal_frames, progressive=True)
    O.reproject_pass(fc, W, H, im)
    for k, ref in ((abi.IMG_ACCUM_DIFFUSE, d), (abi.IMG_ACCUM_SPECULAR, s), (abi.IMG_ACCUM_ALBEDO, a)):
        np.testing.assert_allclose(im[k], ref, rtol=1e-6, atol=1e-6, err_msg=str(k))
    # the history dominates: 511/512 of it survives
    np.testing.assert_allclose(im[abi.IMG_ACCUM_DIFFUSE], im[abi.IMG_PREV_DIFFUSE], rtol=0.02, atol=0.02)
