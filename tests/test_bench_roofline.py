"""The rt pass's roofline as the benchmark line reports it: achieved issue rate = the warp
instructions per ray of the profiled 1080p launch (profiles/k_trace_pass_bricks1080p_dram.md)
times the frame's rays over the event-timed trace pass, against SMs x 4 issue slots x the
sampled SM clock; a reader re-derives every number from those counters."""
import os
import sys
from types import SimpleNamespace

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _stats(rays):
    return SimpleNamespace(rays_traced=rays, hit_fetches=0, node_visits=0, triangle_tests=0, exact_fallbacks=0,
                           exact_retraces=0)


def test_issue_roofline_follows_from_the_counters():
    n = bench.TRACE_NCU_1080P
    rays, trace_ms, sm_mhz, sms = 4_500_000, 3.44, 2070.0, 152
    out = bench.trace_roofline(_stats(rays), trace_ms, 7.6e9, 7.6e9 / (trace_ms * 1e-3) / 1e9, 6774.9, "measured",
                               sms, {"sm_mhz": sm_mhz})
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    achieved = n["inst"] / n["rays"] * rays / (trace_ms * 1e-3) / 1e9
    assert out["bound"] == "issue"
    assert abs(out["peak"] - peak) < 1e-9 and abs(peak - 1258.56) < 1e-6
    assert abs(out["achieved"] - achieved) < 1e-9
    assert abs(out["frac"] - achieved / peak) < 1e-12
    assert 400 < out["warp_instructions_per_ray"] < 440
    assert abs(out["threads_per_instruction"] - n["thread_inst"] / n["inst"]) < 1e-12
    # DRAM traffic of the profiled launch over the trace pass, against the measured HBM peak
    assert out["traffic"] == n["dram_bytes"]
    assert abs(out["hbm"]["dram_gbs"] - n["dram_bytes"] / (trace_ms * 1e-3) / 1e9) < 1e-9
    assert out["hbm"]["dram_frac"] < 0.01   # cache-resident BVH: DRAM is not the bound


def test_roofline_without_a_profile_for_the_size():
    saved = (bench.W_, bench.H_)
    try:
        bench.W_, bench.H_ = 640, 360
        out = bench.trace_roofline(_stats(500_000), 0.5, 1e9, 2000.0, 6774.9, "measured", 152, {"sm_mhz": 2070.0})
        assert out["achieved"] is None and out["frac"] is None and out["traffic"] is None
    finally:
        bench.W_, bench.H_ = saved
