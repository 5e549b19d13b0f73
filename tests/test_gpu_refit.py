"""Instance-level refit (gkrt_scene_refit_instances) against rebuilds and the oracle.

A small city (buildings, orbiting spheres, ground) is animated over several frames, with the
spheres moved far from where the tree was built and some buildings turned and shifted. The hit
rule (minimum (t, instance, primitive) under the FP64 test) does not depend on the tree, so a
refit tree must give the rebuilt tree's hits and images bit for bit, and the oracle's hits."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.renderer import PathTracingRenderer
from oracle import oracle as O
from test_gpu_parity import _compare_trace_images, assert_hits_equal, gpu_trace_rays, random_rays

pytestmark = pytest.mark.gpu

W, H = 192, 108


def small_city():
    return scenes.city(width=W, height=H, boxes=400, spheres=150, emissive_spheres=2, sphere_levels=2)


def frame_instances(motion, base, k):
    """Frame k: the spheres' orbit at 25x the city's speed, every seventh building turned and
    shifted a little more each frame, and from frame 3 on the spheres lifted 300 m."""
    inst = motion.instances(25 * k)
    rng = np.random.default_rng(100 + k)
    for i in range(0, motion.first, 7):
        w = np.asarray(base[i]["world"], np.float64).reshape(3, 4)
        t = w[:, 3] + np.array([0.5 * k, 0.0, -0.3 * k])
        m = scenes.trs(tuple(t), rot_y_deg=7.0 * k + rng.uniform(-2, 2),
                       scale=(w[0, 0], w[1, 1], w[2, 2]))
        inst["world"][i] = m
        inst["world_inv"][i] = scenes.affine_inverse(m)
    if k >= 3:
        s = slice(motion.first, motion.first + motion.radius.shape[0])
        w = inst["world"][s].astype(np.float64)
        w[:, 7] += 300.0
        inst["world"][s] = w.astype(np.float32)
        inst["world_inv"][s] = np.stack([scenes.affine_inverse(x) for x in inst["world"][s]])
    return inst


def with_instances(sc, inst):
    return abi.SceneArrays(sc.positions, sc.normals, sc.material_slots, sc.indices, sc.meshes, sc.materials, inst,
                           lights=sc.lights, name=sc.name)


@pytest.fixture(scope="module")
def env():
    sc, cam, st, motion = small_city()
    a, b = PathTracingRenderer(0), PathTracingRenderer(0)
    for r in (a, b):
        r.load_scene(sc)
        r.create_swap_chain(W, H)
    yield sc, cam, st, motion, a, b
    a.close()
    b.close()


def render(r, fc):
    r.trace_pass(fc)
    r.synchronize()
    return r.images()


def test_refit_equals_rebuild_over_frames(env):
    """Each frame: renderer a refits, renderer b rebuilds; every image is identical."""
    sc, cam, st, motion, a, b = env
    st.flags = abi.FRAME_PRIMARY_IDS
    fb = camera.FrameBuilder(W, H, st)
    r0 = a.stats().tlas_refits
    nodes0 = a.stats().tlas_nodes
    for k in range(1, 6):
        inst = frame_instances(motion, sc.instances, k)
        a.refit_instances(inst)
        b.update_instances(inst)
        fc = fb.build(cam, k)
        ga, gb = render(a, fc), render(b, fc)
        for i in ga:
            assert np.array_equal(ga[i].view(np.uint32), gb[i].view(np.uint32)), (k, i)
        sa, sb = a.stats(), b.stats()
        assert sa.tlas_refits == r0 + k
        assert sa.tlas_nodes == nodes0           # topology kept
        assert sa.rays_traced == sb.rays_traced
        assert sa.device_error == 0 and sb.device_error == 0


def test_refit_ray_queries_exact(env):
    """Closest hits through the 8-wide nodes of the refit tree against the oracle."""
    sc, cam, st, motion, a, b = env
    inst = frame_instances(motion, sc.instances, 6)
    a.refit_instances(inst)
    osc = O.OracleScene(with_instances(sc, inst))
    rng = np.random.default_rng(7)
    ext = np.sqrt(400) * 6.0
    rays = random_rays(rng, 40000, (0.0, 1.0, 0.0), (ext, 470.0, ext), tmax=2000.0)
    # rays aimed at sphere and building instances' origins
    tgt = inst["world"][rng.integers(0, inst.shape[0], 20000)][:, [3, 7, 11]].astype(np.float64)
    e = random_rays(rng, 20000, (0.0, 1.0, 0.0), (ext, 470.0, ext), tmax=2000.0)
    d = tgt + rng.normal(scale=1.0, size=tgt.shape) - e["origin"]
    e["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([rays, e])
    g = gpu_trace_rays(a, rays)
    o = osc.trace_rays(rays)
    assert_hits_equal(g, o)
    assert (o["inst"] != 0xFFFFFFFF).mean() > 0.3
    assert a.stats().device_error == 0


def test_refit_trace_pass_matches_oracle(env):
    sc, cam, st, motion, a, b = env
    inst = frame_instances(motion, sc.instances, 7)
    a.refit_instances(inst)
    st.flags = abi.FRAME_PRIMARY_IDS
    w, h = 96, 64
    a.create_swap_chain(w, h)
    try:
        fc = camera.FrameBuilder(w, h, st).build(cam, 7)
        gim = render(a, fc)
        oim = O.new_images(w, h)
        orays = O.OracleScene(with_instances(sc, inst)).trace_pass(fc, w, h, oim)
        _compare_trace_images(gim, oim)
        assert a.stats().rays_traced == orays
    finally:
        a.create_swap_chain(W, H)


def test_refit_rebuilds_when_members_change(env):
    """Hiding an instance changes the tree's members: the call rebuilds (no refit counted) and
    the result equals a plain rebuild's; later refits work on the new tree."""
    sc, cam, st, motion, a, b = env
    for r in (a, b):
        r.create_swap_chain(W, H)   # the same fresh image sets
    st.flags = abi.FRAME_PRIMARY_IDS
    fb = camera.FrameBuilder(W, H, st)
    inst = frame_instances(motion, sc.instances, 8)
    inst["visible"][motion.first:motion.first + 40] = 0
    n0 = a.stats().tlas_refits
    a.refit_instances(inst)
    b.update_instances(inst)
    assert a.stats().tlas_refits == n0
    fc = fb.build(cam, 8)
    ga, gb = render(a, fc), render(b, fc)
    for i in ga:
        assert np.array_equal(ga[i].view(np.uint32), gb[i].view(np.uint32)), i
    inst2 = frame_instances(motion, sc.instances, 9)
    inst2["visible"][motion.first:motion.first + 40] = 0
    a.refit_instances(inst2)
    b.update_instances(inst2)
    assert a.stats().tlas_refits == n0 + 1
    fc = fb.build(cam, 9)
    ga, gb = render(a, fc), render(b, fc)
    for i in ga:
        assert np.array_equal(ga[i].view(np.uint32), gb[i].view(np.uint32)), i
    assert a.stats().device_error == 0


def test_refit_of_a_host_built_tree_and_mesh_changes(env):
    """The instance level built by the host builder (links recorded by the same GPU collapse),
    then refit on the GPU; and instances that change mesh between frames (the refit computes
    their boxes from the new mesh). Both equal a rebuild image for image."""
    sc, cam, st, motion, a, b = env
    for r in (a, b):
        r.create_swap_chain(W, H)
    st.flags = abi.FRAME_PRIMARY_IDS
    fb = camera.FrameBuilder(W, H, st)
    try:
        inst10 = frame_instances(motion, sc.instances, 10)   # all visible again (the last test hid 40)
        for r in (a, b):
            r.update_instances(inst10)
        a.build_bvh(abi.BUILD_ALL | abi.BUILD_ON_HOST)
        b.build_bvh(abi.BUILD_ALL)
        n0 = a.stats().tlas_refits
        for k, swap in ((11, False), (12, True)):
            inst = frame_instances(motion, sc.instances, k)
            if swap:   # every fifth building becomes a sphere of the same transform, and back
                inst["mesh_id"][0:motion.first:5] = 1
            a.refit_instances(inst)
            b.update_instances(inst)
            fc = fb.build(cam, k)
            ga, gb = render(a, fc), render(b, fc)
            for i in ga:
                assert np.array_equal(ga[i].view(np.uint32), gb[i].view(np.uint32)), (k, i)
        assert a.stats().tlas_refits == n0 + 2
        assert a.stats().device_error == 0
    finally:
        a.build_bvh(abi.BUILD_ALL)


def test_auto_policy_refits_then_rebuilds():
    """gkrt_scene_update_instances_auto: small motions keep the tree (refits, no rebuild); once
    the spheres are scattered across the city the node visits per ray grow past the limit and
    the call rebuilds, after which visits fall back. Every frame's hits equal the oracle's."""
    sc, cam, st, motion = small_city()
    st.flags = abi.FRAME_PRIMARY_IDS
    fb = camera.FrameBuilder(W, H, st)
    rng = np.random.default_rng(7)
    rays = random_rays(rng, 4000, (-20.0, 0.0, -20.0), (140.0, 60.0, 140.0))
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        s0 = r.stats()
        visits = []

        def frame(k, inst, limit):
            r.update_instances_auto(inst, limit)
            r.trace_pass(fb.build(cam, k))
            r.synchronize()
            visits.append(r.stats().node_visits / max(r.stats().rays_traced, 1))

        for k in range(1, 5):   # small motions: refit
            frame(k, motion.instances(k), 1.25)
        s1 = r.stats()
        assert s1.tlas_refits - s0.tlas_refits == 4 and s1.tlas_rebuilds == s0.tlas_rebuilds
        # scatter the spheres across the whole city: the refit tree's boxes balloon
        inst = motion.instances(5)
        sph = slice(motion.first, motion.first + motion.radius.shape[0])
        w = inst["world"][sph].astype(np.float64)
        w[:, 3] = rng.uniform(0.0, 120.0, w.shape[0])
        w[:, 11] = rng.uniform(0.0, 120.0, w.shape[0])
        inst["world"][sph] = w.astype(np.float32)
        inst["world_inv"][sph] = np.stack([scenes.affine_inverse(x) for x in inst["world"][sph]])
        for k in range(5, 9):
            frame(k, inst, 1.25)
            assert_hits_equal(gpu_trace_rays(r, rays), O.OracleScene(with_instances(sc, inst)).trace_rays(rays))
        s2 = r.stats()
        assert s2.tlas_rebuilds > s1.tlas_rebuilds, visits   # the growth triggered a rebuild
        assert visits[-1] < max(visits[4:6]), visits          # and the rebuilt tree is cheaper
        assert s2.device_error == 0
        # growth_limit below 1 is refused
        from gknextengine_gb300.native import GkrtError
        with pytest.raises(GkrtError):
            r.update_instances_auto(inst, 0.5)
