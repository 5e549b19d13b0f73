"""Failure detection on the host: the stream watchdog of gkrt_synchronize. A context with a
1 ms watchdog and ~25 ms of queued frames reports GKRT_ERR_TIMEOUT instead of blocking; the
work itself completes normally and the context stays usable (no GPU fault is involved)."""
import time

import pytest

from gknextengine_gb300 import abi, camera, native, scenes
from gknextengine_gb300.renderer import PathTracingRenderer

pytestmark = pytest.mark.gpu


def test_watchdog_times_out_then_recovers():
    sc, cam, st = scenes.cornell()
    with PathTracingRenderer(0, watchdog_ms=1) as r:
        r.load_scene(sc)
        r.create_swap_chain(1920, 1080)
        fb = camera.FrameBuilder(1920, 1080, st)
        for k in range(8):
            r.render(fb.build(cam, k))
        with pytest.raises(native.GkrtError) as e:
            r.synchronize()
        assert e.value.code == abi.GKRT_ERR_TIMEOUT
        import torch
        torch.cuda.synchronize()          # the frames finish on their own
        time.sleep(0.05)
        r.synchronize()                   # drained: the same context answers normally
        s = r.stats()
        assert s.device_error == 0 and s.rays_traced > 0
