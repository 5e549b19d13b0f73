"""CPU tests of the oracle: known answers, the FP64 hit definition, and its pins."""
import json
import math
import os

import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_pcg4d_known_answers():
    kat = json.load(open(os.path.join(GOLDEN, "rng_kat.json")))
    for case in kat:
        v = list(case["seed"])
        for step in case["sequence"]:
            v = O.pcg4d(v)
            assert v == step["state"]
            assert O.lib().gko_uint_to_float(v[0]) == np.float32(step["float"])


def test_uint_to_float_range():
    L = O.lib()
    assert L.gko_uint_to_float(0) == 0.0
    top = L.gko_uint_to_float(0xFFFFFFFF)
    assert top < 1.0 and top == np.float32(1.0) - np.float32(2.0 ** -23)


def test_sincos_2pi_accuracy():
    us = np.concatenate([np.linspace(0.0, 1.0, 20001, dtype=np.float32),
                         np.array([0.125, 0.25, 0.375, 0.5, 0.625, 0.75, 0.875, 0.9999999], np.float32)])
    worst = 0.0
    for u in us:
        s, c = O.sincos_2pi(float(u))
        a = 2.0 * math.pi * float(u)
        worst = max(worst, abs(s - math.sin(a)), abs(c - math.cos(a)))
    assert worst < 3e-7


def _rand_tris(rng, n):
    c = rng.uniform(-1, 1, (n, 1, 3))
    return (c + rng.normal(0, 0.3, (n, 3, 3))).astype(np.float32)


def test_fp32_bounds_are_conservative():
    """Whenever the FP32 test claims certainty it agrees with FP64, and the FP64 t lies in
    the FP32 interval."""
    rng = np.random.default_rng(7)
    L = O.lib()
    import ctypes as C
    tris = _rand_tris(rng, 4000)
    certain = undecided = 0
    for i in range(tris.shape[0]):
        v = np.ascontiguousarray(tris[i].reshape(-1))
        o = rng.uniform(-2, 2, 3).astype(np.float32)
        target = tris[i].mean(0) + rng.normal(0, 0.2, 3)
        d = (target - o).astype(np.float32)
        if i % 3 == 0:   # rays through vertices and edges
            d = (tris[i][i % 3] + (tris[i][(i + 1) % 3] - tris[i][i % 3]) * rng.random() - o).astype(np.float32)
        ex = np.zeros(3)
        f = np.zeros(7, np.float32)
        hit = L.gko_exact_tri(o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                              v.ctypes.data_as(C.c_void_p), ex.ctypes.data_as(C.c_void_p))
        kind = L.gko_fp32_tri(o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                              v.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p))
        if kind == 0:
            assert hit == 0
            certain += 1
        elif kind == 1:
            assert hit == 1
            assert abs(ex[0] - f[0]) <= f[1]
            if f[6]:
                assert abs(ex[0] - f[4]) <= f[5]
            certain += 1
        else:
            undecided += 1
    assert certain > 2500   # a third of the rays are aimed exactly at edges


def test_bvh_equals_brute_force_cornell():
    sc, cam, st = scenes.cornell()
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(3)
    n = 20000
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = rng.uniform(-0.45, 0.45, (n, 3)) + np.array([0, 0.5, 0])
    d = rng.normal(size=(n, 3))
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1000.0
    a = osc.trace_rays(rays)
    b = osc.trace_rays(rays, brute=True)
    assert np.array_equal(a["inst"], b["inst"]) and np.array_equal(a["prim"], b["prim"])
    assert np.array_equal(a["t"], b["t"])
    assert (a["inst"] != 0xFFFFFFFF).mean() > 0.5


def test_bvh_equals_brute_force_with_ray_tmin():
    """The oracle's ray queries honour each ray's tmin, through its BVH as by brute force."""
    sc, cam, st = scenes.cornell()
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(31)
    n = 20000
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = rng.uniform(-0.45, 0.45, (n, 3)) + np.array([0, 0.5, 0])
    d = rng.normal(size=(n, 3))
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = rng.uniform(0.0, 0.8, n)
    rays["tmax"] = 1000.0
    a = osc.trace_rays(rays)
    b = osc.trace_rays(rays, brute=True)
    assert np.array_equal(a["inst"], b["inst"]) and np.array_equal(a["prim"], b["prim"])
    hit = a["inst"] != 0xFFFFFFFF
    assert (a["t"][hit] >= rays["tmin"][hit]).all()
    base = rays.copy()
    base["tmin"] = 1e-3
    assert (osc.trace_rays(base)["t"][hit] < a["t"][hit]).sum() > n // 10


def test_bvh_equals_brute_force_bricks_subset():
    sc, cam, st = scenes.bricks()
    # keep a 6 x 6 patch of the grid so brute force stays cheap
    keep = np.zeros(sc.instances.shape[0], bool)
    gi = np.arange(4096) // 64
    gj = np.arange(4096) % 64
    keep[:4096] = (gi < 6) & (gj < 6)
    sc.instances["visible"][~keep] = 0
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(5)
    n = 4000
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = np.array([6.0, 12.0, 20.0]) + rng.normal(0, 1.0, (n, 3))
    tgt = np.stack([rng.uniform(0, 13, n), rng.uniform(0, 5, n), rng.uniform(0, 7, n)], 1)
    d = tgt - rays["origin"]
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1000.0
    a = osc.trace_rays(rays)
    b = osc.trace_rays(rays, brute=True)
    assert np.array_equal(a["inst"], b["inst"]) and np.array_equal(a["prim"], b["prim"])
    assert (a["inst"] != 0xFFFFFFFF).mean() > 0.3


def test_fp64_hits_match_reference_tinybvh():
    """The oracle's FP64 closest hit agrees with the reference's own CPU BVH library
    (tinybvh BVH_Double, vendored in gkNextEngine) away from numerical ties."""
    if O.ref_lib() is None:
        pytest.skip("reference tree (tinybvh header) not available on this host")
    rng = np.random.default_rng(11)
    tris = _rand_tris(rng, 3000)
    n = 20000
    org = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    # one mesh, one identity instance
    pos = np.concatenate([tris.reshape(-1, 3), np.ones((tris.shape[0] * 3, 1), np.float32)], 1)
    nrm = np.tile(np.array([[0, 1, 0, 0]], np.float32), (pos.shape[0], 1))
    idx = np.arange(pos.shape[0], dtype=np.uint32)
    meshes = np.array([(0, idx.shape[0], 0, pos.shape[0])], abi.MESH_DTYPE)
    mats = np.array([scenes.lambertian((0.5, 0.5, 0.5))], abi.MATERIAL_DTYPE)
    inst = np.array([scenes.make_instance(0, scenes.trs(), [0], 0)], abi.INSTANCE_DTYPE)
    sc = abi.SceneArrays(pos, nrm, np.zeros(pos.shape[0], np.uint32), idx, meshes, mats, inst)
    osc = O.OracleScene(sc)
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = org
    rays["dir"] = d
    rays["tmin"] = 0.0
    rays["tmax"] = 1e30
    ours = osc.trace_rays(rays)
    t_ref, p_ref = O.ref_closest_double(tris.astype(np.float64), org.astype(np.float64), d.astype(np.float64))
    ours_hit = ours["inst"] != 0xFFFFFFFF
    ref_hit = p_ref >= 0
    # compare where both decisions are far from ties: barycentrics away from edges
    b1, b2 = ours["b1"].astype(np.float64), ours["b2"].astype(np.float64)
    clear = ours_hit & (b1 > 1e-4) & (b2 > 1e-4) & (1 - b1 - b2 > 1e-4)
    agree = clear & ref_hit & (p_ref == ours["prim"].astype(np.int64))
    assert clear.sum() > 2000
    assert agree.sum() >= clear.sum() - 2, (clear.sum(), agree.sum())
    # misses agree too (rays that hit nothing in either)
    assert ((~ours_hit) == (~ref_hit)).mean() > 0.999


def test_oracle_cornell_golden():
    g = np.load(os.path.join(GOLDEN, "cornell_32.npz"))
    sc, cam, st = scenes.cornell()
    W = H = 32
    fc = camera.FrameBuilder(W, H, st).build(cam, 0)
    im = O.new_images(W, H)
    rays = O.OracleScene(sc).trace_pass(fc, W, H, im)
    assert rays == int(g["rays"][0])
    assert np.array_equal(im[abi.IMG_SINGLE_DIFFUSE], g["diffuse"])
    assert np.array_equal(im[abi.IMG_HIT_PRIM], g["hit_prim"])
    assert np.array_equal(im[abi.IMG_OBJECT_ID], g["object_id"])


def test_reproject_static_history_blend():
    """Static camera, same object ids, no motion: accumulation is lerp(prev, cur, 1/T)."""
    W, H = 24, 16
    im = O.new_images(W, H)
    rng = np.random.default_rng(0)
    im[abi.IMG_SINGLE_DIFFUSE][:] = rng.random((H, W, 4), np.float32)
    im[abi.IMG_PREV_DIFFUSE][:] = rng.random((H, W, 4), np.float32)
    im[abi.IMG_NORMAL][..., 1] = 1.0
    im[abi.IMG_OBJECT_ID][:] = 7
    im[abi.IMG_OBJECT_ID_PREV][:] = 7
    fc = abi.GkrtFrameConstants()
    fc.temporal_frames = 8
    O.reproject_pass(fc, W, H, im)
    acc = im[abi.IMG_ACCUM_DIFFUSE][4:-4, 4:-4, :3]
    prev = im[abi.IMG_PREV_DIFFUSE][4:-4, 4:-4, :3]
    cur = im[abi.IMG_SINGLE_DIFFUSE][4:-4, 4:-4, :3]
    np.testing.assert_allclose(acc, prev + (cur - prev) / 8.0, rtol=1e-6, atol=1e-6)


def test_compose_without_filter_is_remodulation():
    W, H = 8, 8
    im = O.new_images(W, H)
    rng = np.random.default_rng(1)
    for k in (abi.IMG_ACCUM_DIFFUSE, abi.IMG_ACCUM_SPECULAR, abi.IMG_ACCUM_ALBEDO):
        im[k][:] = rng.random((H, W, 4), np.float32)
    fc = abi.GkrtFrameConstants()
    fc.bf_size = 0
    fc.paper_white_nit = 600.0
    O.denoise_pass(fc, W, H, im)
    d, s, a = (im[k][..., :3].astype(np.float64) for k in (abi.IMG_ACCUM_DIFFUSE, abi.IMG_ACCUM_SPECULAR,
                                                             abi.IMG_ACCUM_ALBEDO))
    np.testing.assert_allclose(im[abi.IMG_DENOISED_LINEAR][..., :3], d * a + s, rtol=1e-6)


def test_fp32_bounds_far_small_triangles():
    """Small triangles far from the ray origin (size/distance ~ 1/1000): the bounds stay
    conservative and most decisions are still certain."""
    import ctypes as C
    rng = np.random.default_rng(17)
    L = O.lib()
    certain = 0
    n = 6000
    for i in range(n):
        c = rng.normal(size=3)
        c = c / np.linalg.norm(c) * rng.uniform(50, 150)
        tri = (c + rng.normal(0, 0.08, (3, 3))).astype(np.float32)
        o = rng.normal(0, 0.5, 3).astype(np.float32)
        tgt = tri[0] + (tri[1] - tri[0]) * rng.random() + (tri[2] - tri[0]) * rng.random() * 0.5
        d = (tgt - o).astype(np.float32)
        v = np.ascontiguousarray(tri.reshape(-1))
        ex = np.zeros(3)
        f = np.zeros(7, np.float32)
        hit = L.gko_exact_tri(o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                              v.ctypes.data_as(C.c_void_p), ex.ctypes.data_as(C.c_void_p))
        kind = L.gko_fp32_tri(o.ctypes.data_as(C.c_void_p), d.ctypes.data_as(C.c_void_p),
                              v.ctypes.data_as(C.c_void_p), f.ctypes.data_as(C.c_void_p))
        if kind == 0:
            assert hit == 0
        elif kind == 1:
            assert hit == 1 and abs(ex[0] - f[0]) <= f[1]
            assert f[6] and abs(ex[0] - f[4]) <= f[5]
            # the plane interval is far tighter than the sheared one
            assert f[5] <= f[1]
        certain += kind != 2
    assert certain > 0.95 * n


def _cornell_mean(mode, frames, W=24, H=24):
    """Mean and per-sample variance of the 1-spp radiance (diffuse + specular) over frames."""
    sc, cam, st = scenes.cornell()
    osc = O.OracleScene(sc)
    st.nee_mode = mode
    fb = camera.FrameBuilder(W, H, st)
    acc = np.zeros((H, W, 3))
    acc2 = np.zeros((H, W, 3))
    for f in range(frames):
        im = O.new_images(W, H)
        osc.trace_pass(fb.build(cam, f), W, H, im)
        v = (im[abi.IMG_SINGLE_DIFFUSE] + im[abi.IMG_SINGLE_SPECULAR])[..., :3].astype(np.float64)
        acc += v
        acc2 += v * v
    m = acc / frames
    return m.mean(), (acc2 / frames - m * m).mean(), W * H * 3


def test_emissive_nee_matches_bsdf_sampling_in_expectation():
    """GKRT_NEE_EMISSIVE replaces the emission that diffuse bounces reach by light samples at
    the vertices they leave: the same expectation, far lower variance."""
    frames = 1500
    m0, v0, n = _cornell_mean(abi.NEE_REFERENCE, frames)
    m1, v1, _ = _cornell_mean(abi.NEE_EMISSIVE, frames)
    se = math.sqrt((v0 + v1) / (frames * n))
    assert abs(m0 - m1) < 4.0 * se, (m0, m1, se)
    assert v1 < 0.1 * v0, (v0, v1)


def test_adjoint_oracle_matches_finite_differences():
    """The FP64 path-replay gradients of the oracle against central differences (h = 1e-3)
    of its own estimator, sampled with fixed (detached) roughness: 24 albedo and 8
    roughness parameters within 1%."""
    sc, cam, st = scenes.cornell_materials(spp=4)
    W = H = 40
    fc = camera.FrameBuilder(W, H, st).build(cam, 0)
    tgt = np.random.default_rng(0).uniform(0, 0.5, (H, W, 3))
    a0 = sc.materials["diffuse"][:, :3].copy()
    r0 = sc.materials["fuzziness"].copy()

    def loss(a, r):
        m = sc.materials.copy()
        m["diffuse"][:, :3] = a
        m["fuzziness"] = r
        o = O.OracleScene(abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, m,
                                          sc.instances))
        img = o.adjoint(fc, W, H, 4, sample_rough=r0)[0][..., :3].astype(np.float64)
        return ((img - tgt) ** 2).mean(), img

    L0, img = loss(a0, r0)
    dimg = np.zeros((H, W, 4), np.float32)
    dimg[..., :3] = 2.0 * (img - tgt) / img.size
    _, ga, gr = O.OracleScene(sc).adjoint(fc, W, H, 4, sample_rough=r0, dimage=dimg)
    h = 1e-3
    for m in np.argsort(-np.abs(ga[:256]).max(1))[:8]:
        for c in range(3):
            a1, a2 = a0.copy(), a0.copy()
            a1[m, c] += h
            a2[m, c] -= h
            fd = (loss(a1, r0)[0] - loss(a2, r0)[0]) / (2 * h)
            assert abs(ga[m, c] - fd) <= 0.01 * abs(fd), (m, c, ga[m, c], fd)
    for m in np.argsort(-np.abs(gr[:256]))[:8]:
        r1, r2 = r0.copy(), r0.copy()
        r1[m] += h
        r2[m] -= h
        fd = (loss(a0, r1)[0] - loss(a0, r2)[0]) / (2 * h)
        assert abs(gr[m] - fd) <= 0.01 * abs(fd), (m, gr[m], fd)


def test_unet_oracle_backward_matches_finite_differences(monkeypatch):
    """The numpy restatement of the denoiser, with bf16 rounding switched off: its backward pass
    against central differences of its forward pass, 3 parameters of every layer."""
    from oracle import unet_ref as U
    monkeypatch.setattr(U, "bf16", lambda x: np.asarray(x, np.float64))
    rng = np.random.default_rng(0)
    p = rng.normal(0, 0.05, U.param_count())
    inp = rng.uniform(0, 1, (1, 16, 16, 10))
    d = rng.normal(size=(1, 16, 16, 3))
    _, cache = U.forward(p, inp)
    g = U.backward(cache, d)
    off = 0
    for ci, co, _ in U.LAYERS:
        n = 9 * ci * co + co
        # weights on the first 10 input channels / first 3 outputs, where gradients are non-zero
        for i in off + rng.integers(0, n, 3):
            q1, q2 = p.copy(), p.copy()
            q1[i] += 1e-5
            q2[i] -= 1e-5
            fd = ((U.forward(q1, inp)[0] * d).sum() - (U.forward(q2, inp)[0] * d).sum()) / 2e-5
            assert abs(g[i] - fd) <= 1e-6 + 1e-5 * abs(fd), (i - off, g[i], fd)
        off += n
