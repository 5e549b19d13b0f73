"""Per-pass GPU timers (GKRT_DEVICE_PASS_TIMERS), the reference's SCOPED_GPU_TIMER scopes: each
pass reports its last run's GPU time; a context without the flag refuses with a status code."""
import numpy as np
import pytest

from gknextengine_gb300 import abi, camera, native, scenes
from gknextengine_gb300.renderer import PathTracingRenderer

pytestmark = pytest.mark.gpu


def test_pass_times():
    sc, cam, st = scenes.cornell()
    st.denoiser = abi.DENOISE_ATROUS
    with PathTracingRenderer(0, pass_timers=True) as r:
        r.load_scene(sc)
        r.create_swap_chain(320, 240)
        t0 = r.pass_times()
        assert all(v == -1.0 for v in t0.values())          # nothing has run yet
        fb = camera.FrameBuilder(320, 240, st)
        inst = sc.instances.copy()
        r.update_instances(inst)
        for k in range(3):
            r.render(fb.build(cam, k))
        t = r.pass_times()
        assert t["rt pass"] > 0.0 and t["reproject pass"] > 0.0 and t["compose pass"] > 0.0
        assert t["copy pass"] >= 0.0 and t["TLAS Update"] >= 0.0
        assert t["rt pass"] > t["copy pass"]
        r.refit_instances(inst)
        assert r.pass_times()["TLAS Update"] >= 0.0
        assert r.stats().device_error == 0


def test_pass_times_need_the_flag():
    with PathTracingRenderer(0) as r:
        with pytest.raises(native.GkrtError):
            r.pass_times()
