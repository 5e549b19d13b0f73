"""Asynchronous image readback (gkrt_copy_image_to_host_async) against the synchronous copy,
with two frames in flight on separate streams as the benchmark runs them."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, scenes
from gknextengine_gb300.renderer import PathTracingRenderer

pytestmark = pytest.mark.gpu


def test_async_readback_two_frames_in_flight():
    import torch
    sc, cam, st = scenes.cornell()
    W, H = 96, 64
    with PathTracingRenderer(0) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        fb = camera.FrameBuilder(W, H, st)
        stream, copy_stream = torch.cuda.Stream(), torch.cuda.Stream()
        outs = [torch.empty((H, W, 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
        rendered = [torch.cuda.Event() for _ in range(2)]
        copied = [torch.cuda.Event() for _ in range(2)]
        frames = [fb.build(cam.orbit(2.0 * k), k) for k in range(4)]
        got = []
        for k, fc in enumerate(frames):
            j = k % 2
            r.trace_pass(fc, stream)
            r.reproject_pass(fc, stream)
            if k > 0:
                stream.wait_event(copied[1 - j])
            r.denoise_pass(fc, stream)
            r.end_frame(stream)
            rendered[j].record(stream)
            copy_stream.wait_event(rendered[j])
            if k > 1:
                copied[j].synchronize()
                got.append(outs[j].copy())
            r.read_image_async(abi.IMG_DENOISED, outs[j], copy_stream)
            copied[j].record(copy_stream)
        copy_stream.synchronize()
        got += [outs[0].copy(), outs[1].copy()]
        # the same frames, each read back synchronously
        r.create_swap_chain(W, H)
        ref = []
        for fc in frames:
            r.render(fc)
            ref.append(r.read_image(abi.IMG_DENOISED))
        for k in range(4):
            assert np.array_equal(got[k], ref[k]), k
        assert ref[3][..., :3].max() > 0.0
        with pytest.raises(ValueError):
            r.read_image_async(abi.IMG_DENOISED, np.zeros((H, W, 3), np.float32))
