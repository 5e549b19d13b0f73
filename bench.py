"""Benchmark of the ray-tracing pass: Mrays/s and ms/frame at 1080p, 1 spp.

Workload (one step = one frame of the reference's PathTracingRenderer::Render: rt pass,
reproject pass, compose pass, history hand-over): the studded-brick scene, 4096 instanced
bricks of 252 triangles (1.03 M triangles) on a 64 x 64 grid, GGX materials, 64 emissive
bricks, 1920 x 1080, 1 spp, 8 bounces, the camera orbiting 0.5 degrees per frame, temporal
reprojection and the joint bilateral filter. The scene is synthetic (seeded numpy).

* value   : rays (camera + bounce + shadow, counted on the device) per second over the K
            timed frames, inputs resident on the GPU, CUDA events on the launch stream.
* e2e     : the same frames through the C ABI with host buffers: frame constants from
            host memory and the denoised image read back to pinned host memory each frame.
* roofline: the trace kernel's algorithmic bytes per launch (node visits x 64 B + triangle
            tests x 48 B + rays x 32 B in + per-hit fetches) over its event-timed duration,
            against the measured HBM copy bandwidth.
* cpu_baseline: the CPU oracle (C++ restatement of the reference's shading logic) on the
            host cores over a bounded sample of the same frames.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gkrt|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mrays/s and ms/frame 1080p 1spp; denoised RelMSE vs 4096 spp vs bilateral"
UNIT = "Mrays/s"
W_, H_ = 1920, 1080
HIT_FETCH_BYTES = 3 * 4 + 3 * 16 + 64 + 64 + 48   # indices, normals, material, instance, triangle
NODE_BYTES, TRI_BYTES, RAY_BYTES = 64, 48, 32


WORKLOAD = "bricks"


def workload_config():
    if WORKLOAD == "city":
        return {"workload": f"city-10.48M-tris {W_}x{H_} 1spp depth8 alias-table-NEE moving-spheres "
                            "per-frame-instance-rebuild reproject+JBF",
                "triangles": 10480002, "instances": 25001, "emissive_triangles": 10240, "width": W_, "height": H_,
                "spp": 1, "max_depth": 8,
                "l2": "per-frame image working set 2 GB > L2 (129 MB)",
                "per_frame": "gkrt_scene_update_instances (instance-level BVH rebuild on the GPU + emitter "
                             "alias table) inside the timed frame",
                "data": "synthetic seeded scene (numpy default_rng seed 3)"}
    return {"workload": f"bricks-1.03M-tris {W_}x{H_} 1spp depth8 orbit0.5deg/frame reproject+JBF",
            "triangles": 1032194, "instances": 4097, "width": W_, "height": H_, "spp": 1, "max_depth": 8,
            "l2": "per-frame image working set 0.5 GB > L2 (129 MB); the 0.6 MB BVH stays L2-resident as "
                  "in steady-state rendering",
            "data": "synthetic seeded scene (numpy default_rng seed 2)"}


def load_workload():
    """(scene, camera, settings, per-frame instance function or None)."""
    from gknextengine_gb300 import scenes
    if WORKLOAD == "city":
        sc, cam, st, motion = scenes.city(width=W_, height=H_)
        return sc, cam, st, motion.instances
    sc, cam, st = scenes.bricks()
    return sc, cam, st, None


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._p = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                        "--format=csv,noheader,nounits", "-lms", "200"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._p = None
        return self

    def _read(self):
        for line in self._p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._p:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._p.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def cpu_baseline_measure(budget_s: float = 12.0):
    """The oracle on the host cores over whole 1080p frames of the workload (trace, reproject,
    compose), as many frames as fit in the time budget (at least one)."""
    from gknextengine_gb300 import camera, scenes
    from oracle import oracle as O
    O.lib().gko_set_fast(1)
    sc, cam, st = scenes.bricks()
    osc = O.OracleScene(sc)
    fb = camera.FrameBuilder(W_, H_, st)
    im = O.new_images(W_, H_)
    cores = os.cpu_count() or 1
    # one untimed band to warm caches and page in the scene
    fc = fb.build(cam, 0)
    osc.trace_pass(fc, W_, H_, im, y0=0, y1=8, threads=cores)
    rays = 0
    frames = 0
    t0 = time.perf_counter()
    while True:
        fc = fb.build(cam.orbit(0.5 * (frames + 1)), frames + 1)
        rays += O.render_frame(osc, fc, W_, H_, im, threads=cores)
        frames += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{frames} full 1080p frames of the workload (trace+reproject+compose), "
                      f"{rays} rays in {dt:.1f} s", "ms_per_frame": dt / frames * 1e3}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from gknextengine_gb300 import camera, scenes
    from oracle import oracle as O
    O.lib().gko_set_fast(1)
    sc, cam, st = scenes.bricks()
    osc = O.OracleScene(sc)
    fb = camera.FrameBuilder(W_, H_, st)
    im = O.new_images(W_, H_)
    cores = os.cpu_count() or 1
    band = 64   # rows per step: a bounded sample of each frame
    def step(i):
        fc = fb.build(cam.orbit(0.5 * i), i)
        y0 = (i * band) % (H_ - band)
        return osc.trace_pass(fc, W_, H_, im, y0=y0, y1=y0 + band, threads=cores)
    for i in range(args.warmup):
        step(i)
    rays = 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        rays += step(args.warmup + i)
    dt = time.perf_counter() - t0
    v = rays / dt / 1e6
    ms_frame = dt / args.steps * (H_ / band) * 1e3
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "ms_per_frame_extrapolated": ms_frame, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{band} rows of a 1080p frame per step (trace pass), {args.steps} steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def relmse(x, y):
    """mean over pixels and RGB of (x - y)^2 / (y^2 + 1e-2), linear radiance."""
    import numpy as np
    d = x[..., :3].astype(np.float64) - y[..., :3]
    return float(np.mean(d * d / (y[..., :3].astype(np.float64) ** 2 + 1e-2)))


def relmse_measure(device: int, W: int = 960, H: int = 540, ref_spp: int = 4096, temporal: int = 16):
    """Denoised RelMSE against a 4096-spp reference on the Cornell scene (static camera,
    no TAA jitter). The reference is the mean of 4096 independent 1-spp trace passes,
    remodulated like the compose pass (diffuse x albedo + specular). Compared: the raw
    1-spp image, the reference's JBF and the a-trous filter on one frame, and the same after
    `temporal` frames of reprojection."""
    import numpy as np
    import torch
    from gknextengine_gb300 import abi, camera, scenes
    from gknextengine_gb300.renderer import PathTracingRenderer
    sc, cam, st = scenes.cornell()
    st.taa = False
    out = {"scene": f"cornell {W}x{H}", "reference_spp": ref_spp, "metric": "mean (x-y)^2/(y^2+1e-2) over px, RGB"}
    with PathTracingRenderer(device) as r:
        r.load_scene(sc)
        r.create_swap_chain(W, H)
        fb = camera.FrameBuilder(W, H, st)
        t0 = time.perf_counter()
        acc_d = torch.zeros((H, r.image_view(abi.IMG_SINGLE_DIFFUSE).pitch_bytes // 16, 4), device="cuda")
        acc_s = torch.zeros_like(acc_d)
        vd = r.image_view(abi.IMG_SINGLE_DIFFUSE)
        vs = r.image_view(abi.IMG_SINGLE_SPECULAR)
        n = H * (vd.pitch_bytes // 16) * 4
        for f in range(ref_spp):
            fc = fb.build(cam, 100000 + f)
            r.trace_pass(fc)
            d = torch.as_tensor(_device_f32(vd.device_ptr, n)).view(H, -1, 4)
            s_ = torch.as_tensor(_device_f32(vs.device_ptr, n)).view(H, -1, 4)
            acc_d += d
            acc_s += s_
        torch.cuda.synchronize()
        out["reference_seconds"] = time.perf_counter() - t0
        alb = r.read_image(abi.IMG_ALBEDO)
        ref = (acc_d[:, :W].cpu().numpy() / ref_spp) * alb + acc_s[:, :W].cpu().numpy() / ref_spp
        for name, den, bf in (("raw", abi.DENOISE_JBF, 0), ("jbf", abi.DENOISE_JBF, 5),
                              ("atrous", abi.DENOISE_ATROUS, 5)):
            st.denoiser, st.bf_size = den, bf
            # one frame on its own (history weight 0), then the steady state of the temporal
            # blend (1/16 per frame) after 8 x 16 frames, when the zeroed start no longer counts
            for tf, frames, key in ((1, 1, f"{name}_1spp"), (temporal, 8 * temporal, f"{name}_temporal")):
                st.temporal_frames = tf
                fbn = camera.FrameBuilder(W, H, st)
                r.create_swap_chain(W, H)
                for f in range(frames):
                    r.render(fbn.build(cam, f))
                out[key] = relmse(r.read_image(abi.IMG_DENOISED_LINEAR), ref)
    return out


def _device_f32(ptr, n):
    """A float32 view of n floats of device memory (no copy)."""
    import torch
    class _A:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f4", "data": (ptr, False), "version": 3}
    return torch.as_tensor(_A(), device="cuda")


def run_gkrt(args):
    import numpy as np
    import torch

    from gknextengine_gb300 import abi, camera, scenes
    from gknextengine_gb300.renderer import PathTracingRenderer

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    sc, cam, st, frame_instances = load_workload()
    r = PathTracingRenderer(local)
    t0 = time.perf_counter()
    r.load_scene(sc)
    load_s = time.perf_counter() - t0
    r.create_swap_chain(W_, H_)
    stream = torch.cuda.Stream()
    # BVH build times (GPU builder, host clock around the synchronous calls)
    r.build_bvh(abi.BUILD_ALL, stream)
    t0 = time.perf_counter()
    r.build_bvh(abi.BUILD_ALL, stream)
    build_all_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    r.update_instances(sc.instances if frame_instances is None else frame_instances(0), stream)
    build_inst_ms = (time.perf_counter() - t0) * 1e3
    orbit = 0.5 if frame_instances is None else 0.25
    fb = camera.FrameBuilder(W_, H_, st)
    K, Wm = args.steps, args.warmup
    fcs = [fb.build(cam.orbit(orbit * i), i) for i in range(Wm + K)]
    insts = [frame_instances(i) for i in range(Wm + K)] if frame_instances is not None else None

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    # ---- warm-up, then K timed frames (device-resident inputs) ----
    for i in range(Wm):
        if insts is not None:
            r.update_instances(insts[i], stream)
        r.render(fcs[i], stream)
    r.synchronize(stream)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0 = r.stats()
    rays0, bl0 = s0.rays_total, s0.build_launches
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk, torch.cuda.stream(stream):
        start.record(stream)
        for k in range(K):
            fc = fcs[Wm + k]
            if insts is not None:
                r.update_instances(insts[Wm + k], stream)
            ev[k][0].record(stream)
            r.trace_pass(fc, stream)
            ev[k][1].record(stream)
            r.reproject_pass(fc, stream)
            r.denoise_pass(fc, stream)
            r.end_frame(stream)
        end.record(stream)
        torch.cuda.synchronize()
    barrier()
    st_last = r.stats()
    rays = st_last.rays_total - rays0
    build_launches = st_last.build_launches - bl0
    ms_total = start.elapsed_time(end)
    trace_ms = [a.elapsed_time(b) for a, b in ev]
    if world > 1:
        t = torch.tensor([ms_total], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_total = float(t.item())
        n = torch.tensor([float(rays)], device="cuda")
        torch.distributed.all_reduce(n)
        rays = int(n.item())
    value = rays / (ms_total * 1e-3) / 1e6

    # ---- algorithmic bytes of the trace kernel (counters of the last timed frame) ----
    hits_est = st_last.rays_traced   # upper bound on hits: every ray fetches hit data at most once
    alg_bytes = (st_last.node_visits * NODE_BYTES + st_last.triangle_tests * TRI_BYTES +
                 st_last.rays_traced * RAY_BYTES + hits_est * HIT_FETCH_BYTES + W_ * H_ * 7 * 16)
    trace_avg_ms = sum(trace_ms) / len(trace_ms)
    achieved = alg_bytes / (trace_avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()

    # ---- e2e through the C ABI with host buffers ----
    pinned = torch.empty((H_, W_, 4), dtype=torch.float32, pin_memory=True)
    out = pinned.numpy()
    for i in range(min(Wm, 3)):
        r.render(fcs[i], stream)
        r.read_image(abi.IMG_DENOISED, stream, out=out)
    r.synchronize(stream)
    barrier()
    t0 = time.perf_counter()
    e2e_rays0 = r.stats().rays_total
    for k in range(K):
        fc_host = fb.build(cam.orbit(orbit * (Wm + k)), Wm + k)   # frame constants built in host memory
        if insts is not None:
            r.update_instances(insts[Wm + k], stream)              # host instance records
        r.render(fc_host, stream)
        r.read_image(abi.IMG_DENOISED, stream, out=out)          # D2H into pinned memory, waits
    e2e_s = time.perf_counter() - t0
    e2e_rays = r.stats().rays_total - e2e_rays0
    barrier()
    e2e_value = e2e_rays / e2e_s / 1e6

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": Wm,
                "ms_per_step": ms_total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": workload_config(),
                "ms_per_frame": ms_total / K, "trace_ms": trace_avg_ms, "rays_per_frame": rays / max(K, 1) / world,
                "gpu_launches": 3 * K + 2 * K * (fcs[0].denoiser == abi.DENOISE_ATROUS) + build_launches,
                "bvh_build_ms": {"all_levels": build_all_ms, "instance_level": build_inst_ms,
                                 "scene_load_s": load_s, "triangles": int(sc.triangle_count),
                                 "instances": int(sc.instances.shape[0])},
                "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": ctypes.sizeof(abi.GkrtFrameConstants),
                        "d2h_bytes_per_step": W_ * H_ * 16, "ms_per_frame": e2e_s / K * 1e3},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": None, "kernel": "k_trace_pass",
                             "peak_kind": peak_kind,
                             "algorithmic_bytes_per_launch": alg_bytes,
                             "node_visits": st_last.node_visits, "triangle_tests": st_last.triangle_tests,
                             "exact_fallbacks": st_last.exact_fallbacks, "exact_retraces": st_last.exact_retraces},
                "clocks": clk.summary()}
        if world == 1 and WORKLOAD == "bricks" and not args.no_relmse:
            line["relmse"] = relmse_measure(local)
        if world == 1 and not args.no_cpu_baseline and WORKLOAD == "bricks":
            line["cpu_baseline"] = cpu_baseline_measure(args.cpu_budget)
        print(json.dumps(line))
    r.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gkrt", choices=["gkrt", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-relmse", action="store_true")
    ap.add_argument("--size", default=None, help="WxH override for profiling small cases (default 1920x1080)")
    ap.add_argument("--workload", default="bricks", choices=["bricks", "city"],
                    help="bricks: the 1080p headline workload; city: 10.5M tris at 4K with per-frame rebuild")
    args = ap.parse_args()
    global WORKLOAD, W_, H_
    WORKLOAD = args.workload
    if WORKLOAD == "city":
        W_, H_ = 3840, 2160
    if args.warmup < 3:
        args.warmup = 3
    if args.size:
        W_, H_ = (int(v) for v in args.size.lower().split("x"))
    if args.impl == "reference":
        return run_reference(args)
    return run_gkrt(args)


if __name__ == "__main__":
    sys.exit(main())
