"""The ray-query entry point for callers that cannot allocate device memory.

Some hosts cannot call cudaMalloc when they issue work: an engine whose device memory is
owned by its own pool allocator, or a process at its memory budget that must not grow.
gkrt_trace_rays_noalloc answers the same queries as gkrt_trace_rays
with its scratch in a fixed static device array. This test calls both through the C ABI on
the same rays, twice in a row, and requires bit-identical hits (the tolerance the ray
query parity tests use), and checks that an over-limit batch is refused with a clear
error. It sits in its own file so that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from gknextengine_gb300 import abi, native, scenes
from gknextengine_gb300.renderer import PathTracingRenderer

pytestmark = pytest.mark.gpu


def _rays(rng, n):
    rays = np.zeros(n, abi.RAY_DTYPE)
    rays["origin"] = np.stack([rng.uniform(-5, 145, n), rng.uniform(0.5, 30, n), rng.uniform(-5, 80, n)], 1)
    d = rng.normal(size=(n, 3))
    d[:, 1] = -np.abs(d[:, 1])
    rays["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmin"] = 1e-3
    rays["tmax"] = 1000.0
    rays["tmin"][::3] = rng.uniform(0.0, 20.0, rays["tmin"][::3].shape[0])   # per-ray lower bounds
    return rays


def test_noalloc_ray_queries_match_allocating_entry_point():
    import torch
    assert torch.cuda.is_available()
    sc, _, _ = scenes.bricks()
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        rng = np.random.default_rng(12)
        for call in range(2):
            rays = _rays(rng, 300_000 + call * 1000)
            n = rays.shape[0]
            rb = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
            h_ref = torch.zeros(n * abi.HIT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
            h_na = torch.full((n * abi.HIT_DTYPE.itemsize,), 0xAB, dtype=torch.uint8, device="cuda")
            for mode in (abi.TRACE_CLOSEST, abi.TRACE_ANY):
                r.trace_rays_device(rb.data_ptr(), h_ref.data_ptr(), n, mode)
                r.synchronize()
                s_ref = r.stats()
                free0 = torch.cuda.mem_get_info()[0]
                r.trace_rays_noalloc_device(rb.data_ptr(), h_na.data_ptr(), n, mode)
                r.synchronize()
                s_na = r.stats()
                if call > 0:   # the device's free memory does not move across the call
                    assert torch.cuda.mem_get_info()[0] == free0
                a = h_ref.cpu().numpy().view(abi.HIT_DTYPE)
                b = h_na.cpu().numpy().view(abi.HIT_DTYPE)
                assert np.array_equal(a["inst"], b["inst"]) and np.array_equal(a["prim"], b["prim"])
                assert np.array_equal(a["t"], b["t"])
                if mode == abi.TRACE_CLOSEST:
                    assert np.array_equal(a["b1"], b["b1"]) and np.array_equal(a["b2"], b["b2"])
                assert (a["inst"] != 0xFFFFFFFF).sum() > n // 4
                # per-call statistics come out the same from the static scratch
                assert s_na.rays_traced == s_ref.rays_traced == n
                assert s_na.node_visits == s_ref.node_visits
                assert s_na.triangle_tests == s_ref.triangle_tests
        # an empty batch resets the per-call statistics as gkrt_trace_rays does
        r.trace_rays_noalloc_device(rb.data_ptr(), h_na.data_ptr(), 0, abi.TRACE_CLOSEST)
        r.synchronize()
        s0 = r.stats()
        assert s0.rays_traced == 0 and s0.node_visits == 0 and s0.triangle_tests == 0


def test_noalloc_rejects_batches_above_the_scratch_limit():
    import torch
    sc, _, _ = scenes.cornell()
    with PathTracingRenderer(0) as r:
        L = native.load()
        rb = torch.zeros(64, dtype=torch.uint8, device="cuda")
        hb = torch.zeros(64, dtype=torch.uint8, device="cuda")
        # before a scene exists the call refuses instead of building anything
        rc = L.gkrt_trace_rays_noalloc(r._h, C.c_void_p(rb.data_ptr()), C.c_void_p(hb.data_ptr()), 1,
                                       abi.TRACE_CLOSEST, None)
        assert rc == abi.GKRT_ERR_STATE
        r.load_scene(sc)
        rc = L.gkrt_trace_rays_noalloc(r._h, C.c_void_p(rb.data_ptr()), C.c_void_p(hb.data_ptr()),
                                       4_194_305, abi.TRACE_CLOSEST, None)
        assert rc == abi.GKRT_ERR_INVALID_ARG
        assert b"4194304" in L.gkrt_last_error_message(r._h)
