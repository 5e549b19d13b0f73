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
* roofline: the trace kernel against its binding resource, instruction issue: warp
            instructions per ray (ncu) x the frame's rays over the event-timed duration,
            against SMs x 4 issue slots x the sampled SM clock. Beside it (roofline.hbm) the
            algorithmic bytes (node visits x 64 B + triangle tests x 48 B + rays x 32 B +
            hit fetches x 236 B + outputs, all device-counted) and the DRAM traffic (ncu)
            against the measured HBM copy bandwidth.
* city    : 3 timed 4K frames of the 10.5 M-triangle city with the per-frame instance rebuild.
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
# ncu counters of one 1080p k_trace_pass launch of the default workload (one capture of
# `python bench.py --steps 3 --warmup 3 --no-cpu-baseline --no-relmse --no-city`, fifth launch):
# warp instructions issued (sm__inst_executed.sum), thread instructions
# (smsp__thread_inst_executed.sum), DRAM bytes read + written, and the rays of that launch.
# The node and triangle reads of the algorithmic bytes are served by L1/L2.
TRACE_NCU_1080P = {"inst": 1876796969, "thread_inst": 23252036915, "dram_bytes": 7515904 + 116706048,
                   "rays": 4483043}
ISSUE_PER_SM_PER_CLOCK = 4   # four schedulers per SM, one warp instruction each per cycle


def trace_roofline(st, trace_ms, alg_bytes, alg_gbs, hbm_peak, peak_kind, num_sms, clocks):
    """Roofline of the rt-pass kernel against the bound that holds: issue slots. The BVH is
    cache-resident, so DRAM carries little more than the output images (dram_frac), and the
    kernel is bound by instruction issue and SIMT efficiency (divergent traversal and shading).
    achieved: warp instructions per ray (ncu, one 1080p launch) x the rays of the timed frame over
    its event-timed duration; peak: SMs x 4 issue slots x the SM clock sampled during the run."""
    n = TRACE_NCU_1080P
    full = WORKLOAD == "bricks" and (W_, H_) == (1920, 1080)
    sm_mhz = clocks.get("sm_mhz") or clocks.get("sm_max_mhz") or 2070.0
    issue_peak = num_sms * ISSUE_PER_SM_PER_CLOCK * sm_mhz * 1e6 / 1e9
    out = {"bound": "issue", "unit": "G warp-instructions/s", "kernel": "k_trace_pass",
           "peak": issue_peak, "peak_kind": f"{num_sms} SMs x {ISSUE_PER_SM_PER_CLOCK} issue slots x {sm_mhz:.0f} MHz",
           "achieved": None, "frac": None,
           "traffic": n["dram_bytes"] if full else None,
           "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 1080p k_trace_pass launch"}
    if full and n["inst"] and n["rays"]:
        achieved = n["inst"] / n["rays"] * st.rays_traced / (trace_ms * 1e-3) / 1e9
        out.update({"achieved": achieved, "frac": achieved / issue_peak,
                    "warp_instructions_per_ray": n["inst"] / n["rays"],
                    "threads_per_instruction": n["thread_inst"] / n["inst"]})
    dram_gbs = n["dram_bytes"] / (trace_ms * 1e-3) / 1e9 if full else None
    out["hbm"] = {"peak": hbm_peak, "peak_kind": peak_kind, "unit": "GB/s",
                  "algorithmic_bytes_per_launch": alg_bytes, "algorithmic_gbs": alg_gbs,
                  "algorithmic_frac": alg_gbs / hbm_peak,
                  "dram_gbs": dram_gbs, "dram_frac": dram_gbs / hbm_peak if dram_gbs else None}
    out.update({"rays": st.rays_traced, "hit_fetches": st.hit_fetches, "node_visits": st.node_visits,
                "triangle_tests": st.triangle_tests, "exact_fallbacks": st.exact_fallbacks,
                "exact_retraces": st.exact_retraces})
    return out


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
    return {"workload": f"bricks-1.03M-tris {W_}x{H_} 1spp depth8 orbit0.5deg/frame reproject+atrous5x5x3",
            "triangles": 1032194, "instances": 4097, "width": W_, "height": H_, "spp": 1, "max_depth": 8,
            "l2": "per-frame image working set 0.5 GB > L2 (129 MB); the 0.6 MB BVH stays L2-resident as "
                  "in steady-state rendering",
            "data": "synthetic seeded scene (numpy default_rng seed 2)"}


def measured_peak_bf16():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["bf16_tflops"]), "measured"
    except Exception:
        return 1900.0, "fallback"


UNET_LAYERS = [(32, 32, 0), (32, 32, 0), (32, 64, 1), (64, 64, 1), (64, 96, 2), (96, 96, 2), (96, 128, 3),
               (128, 128, 3), (224, 96, 2), (96, 96, 2), (160, 64, 1), (64, 64, 1), (96, 32, 0), (32, 32, 0),
               (32, 32, 0)]   # (cin, cout as computed, level)


def run_denoiser(args):
    """The learned denoiser at 1920 x 1080: forward (inference) ms/frame through the C ABI with
    device inputs, and one Adam training step at 2 x 512 x 512; tensor-core roofline of the
    forward (algorithmic FLOPs of the 15 convolutions over the measured time)."""
    import torch
    from gknextengine_gb300.denoiser import Unet
    from gknextengine_gb300.renderer import PathTracingRenderer
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    W, H = 1920, 1080
    flops = sum(2 * 9 * ci * co * (W >> lv) * (H >> lv) for ci, co, lv in UNET_LAYERS)
    with PathTracingRenderer(local) as r:
        net = Unet(r, seed=7)
        g = torch.Generator(device="cuda").manual_seed(0)
        inp = torch.rand((1, H, W, 10), device="cuda", generator=g)
        out = torch.zeros((1, H, W, 4), device="cuda")
        for _ in range(args.warmup):
            net.forward(inp, out_linear=out)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            e0.record()
            for _ in range(args.steps):
                net.forward(inp, out_linear=out)
            e1.record()
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        # end to end: input from pinned host memory, denoised frame back to pinned host memory
        hin = torch.rand((1, H, W, 10), generator=torch.Generator().manual_seed(1)).pin_memory()
        hout = torch.empty((1, H, W, 4), pin_memory=True)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            inp.copy_(hin, non_blocking=True)
            net.forward(inp, out_linear=out)
            hout.copy_(out, non_blocking=True)
            torch.cuda.synchronize()
        e2e_ms = (time.perf_counter() - t0) / args.steps * 1e3
        tin = torch.rand((2, 512, 512, 10), device="cuda", generator=g)
        tgt = torch.rand((2, 512, 512, 3), device="cuda", generator=g)
        for _ in range(3):
            net.train_step(tin, tgt, 1e-4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(10):
            net.train_step(tin, tgt, 1e-4)
        torch.cuda.synchronize()
        train_ms = (time.perf_counter() - t0) / 10 * 1e3
    peak, kind = measured_peak_bf16()
    achieved = flops / (ms * 1e-3) / 1e12
    line = {"metric": "learned denoiser ms/frame 1080p (bf16 U-Net forward)", "value": ms, "unit": "ms/frame",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": "U-Net 32/64/96/128, 15 3x3 convs, 1920x1080, batch 1",
                       "l2": "activations 0.4-0.8 GB per level-0 tensor > L2"},
            "gpu_launches": 0, "e2e": {"value": e2e_ms, "unit": "ms/frame", "h2d_bytes_per_step": H * W * 40,
                                       "d2h_bytes_per_step": H * W * 16},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None,
                         "kernel": "k_conv3x3, k_conv3x3_halo (16 launches: dec0a as its half-resolution sub-pixel "
                                   "part and its enc0b part, the same FLOPs)",
                         "peak_kind": kind, "algorithmic_flops_per_frame": flops},
            "train_step_ms_2x512x512": train_ms, "clocks": clk.summary()}
    # 16 convolutions (pools and upsamplings in their epilogues; dec0a in two), input packing and output
    line["gpu_launches"] = 16 + 2
    print(json.dumps(line))
    return 0


def load_workload():
    """(scene, camera, settings, per-frame instance function or None)."""
    from gknextengine_gb300 import scenes
    if WORKLOAD == "city":
        sc, cam, st, motion = scenes.city(width=W_, height=H_)
        return sc, cam, st, motion.instances
    sc, cam, st = scenes.bricks()
    return sc, cam, st, None


def job_totals(ms, units, world, device):
    """Whole-job figures over `world` ranks: the slowest rank's time (max over ranks) and the
    units all ranks processed (sum), by one all-reduce each when world > 1. The job's rate is
    units / ms."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        n = torch.tensor([float(units)], dtype=torch.float64, device=device)
        dist.all_reduce(n)
        ms, units = float(t.item()), float(n.item())
    return ms, units


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
    """The reference arm: the oracle (the C++ restatement of the reference's shading logic; the
    reference's Slang has no CPU build here) on all host cores, one whole frame of the workload
    per step (rt pass, reproject pass, compose pass: the work the GPU arm times)."""
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

    def step(i):
        fc = fb.build(cam.orbit(0.5 * i), i)
        return O.render_frame(osc, fc, W_, H_, im, threads=cores)

    for i in range(args.warmup):
        step(i)
    rays = 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        rays += step(args.warmup + i)
    dt = time.perf_counter() - t0
    v = rays / dt / 1e6
    line = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "ms_per_frame": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": workload_config(),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} whole {W_}x{H_} frames of the workload "
                                       f"(trace+reproject+compose), {rays} rays in {dt:.1f} s"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def relmse_measure(device: int):
    """Denoised RelMSE against 4096-spp references at 1920 x 1080 for the raw 1-spp frame, the
    reference's bilateral filter (JBF), the a-trous filter, the learned denoiser (the shipped
    network, trained by the library's own kernels on 2048 renderer-generated 256 x 256 crops of
    Cornell-family views with 4096-spp targets) and the filters' temporal steady state, on two
    views outside the training set: the config-1 Cornell box and a C2 brick-scene frame."""
    from gknextengine_gb300.denoiser import C5_WEIGHTS, evaluate_c5, load_c5
    from gknextengine_gb300.renderer import PathTracingRenderer
    with PathTracingRenderer(device) as r:
        net = load_c5(r)
        out = evaluate_c5(r, net)
    rec = os.path.splitext(C5_WEIGHTS)[0] + ".json"
    if os.path.exists(rec):
        with open(rec) as f:
            out["training"] = {k: v for k, v in json.load(f)["training"].items() if k != "losses_every_100"}
    return out


def city_measure(device: int, frames: int = 4, warmup: int = 3):
    """The 10.5 M-triangle city at 3840 x 2160 (alias-table NEE over 10,240 emissive
    triangles, 5 k moving spheres): `frames` timed frames after `warmup`, each with the
    per-frame instance update (GPU instance-level rebuild and emitter table) inside the frame,
    then the rt, reproject and compose passes. Device-resident inputs, CUDA events."""
    import numpy as np
    import torch
    from gknextengine_gb300 import camera, scenes
    from gknextengine_gb300.renderer import PathTracingRenderer
    W, H = 3840, 2160
    sc, cam, st, motion = scenes.city(width=W, height=H)
    with PathTracingRenderer(device) as r:
        t0 = time.perf_counter()
        r.load_scene(sc)
        load_s = time.perf_counter() - t0
        r.create_swap_chain(W, H)
        stream = torch.cuda.Stream()
        fb = camera.FrameBuilder(W, H, st)
        n = warmup + frames
        fcs = [fb.build(cam.orbit(0.25 * i), i) for i in range(n)]
        insts = [motion.instances(i) for i in range(n)]
        for i in range(warmup):
            r.update_instances(insts[i], stream)
            r.render(fcs[i], stream)
        r.synchronize(stream)
        rays0 = r.stats().rays_total
        ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(frames)]
        start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            start.record(stream)
            for k in range(frames):
                fc = fcs[warmup + k]
                ev[k][0].record(stream)
                r.update_instances(insts[warmup + k], stream)
                ev[k][1].record(stream)
                r.trace_pass(fc, stream)
                ev[k][2].record(stream)
                r.reproject_pass(fc, stream)
                r.denoise_pass(fc, stream)
                r.end_frame(stream)
            end.record(stream)
            torch.cuda.synchronize()
        rays = r.stats().rays_total - rays0
        ms = start.elapsed_time(end)
    return {"workload": "city-10.48M-tris 3840x2160 1spp depth8 alias-table-NEE moving-spheres "
                        "per-frame-instance-rebuild reproject+JBF",
            "mrays_s": rays / (ms * 1e-3) / 1e6, "ms_per_frame": ms / frames, "frames": frames,
            "rays_per_frame": rays / frames,
            "trace_ms": sum(a.elapsed_time(b) for _, a, b in ev) / frames,
            # median: the first timed frame follows a synchronize, so the update's host work
            # (tables, emitter alias table) runs on an idle GPU there; in the frames after it the
            # host prepares the update while the previous frame traces
            "update_span_ms": float(np.median([a.elapsed_time(b) for a, b, _ in ev])),
            "update_span_first_frame_ms": ev[0][0].elapsed_time(ev[0][1]),
            "scene_load_s": load_s, "triangles": int(sc.triangle_count)}


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
    ui0, ui1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    # one untimed update first: each page-locked staging table has two buffers, allocated on
    # first use, so the timed update is the steady-state per-frame one
    r.update_instances(sc.instances if frame_instances is None else frame_instances(0), stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ui0.record(stream)
    r.update_instances(sc.instances if frame_instances is None else frame_instances(0), stream)
    ui1.record(stream)
    build_inst_ms = (time.perf_counter() - t0) * 1e3
    ui1.synchronize()
    build_inst_device_ms = ui0.elapsed_time(ui1)
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
    ev_u = [torch.cuda.Event(enable_timing=True) for _ in range(K)]   # before each instance update
    with ClockSampler(local) as clk, torch.cuda.stream(stream):
        start.record(stream)
        for k in range(K):
            fc = fcs[Wm + k]
            ev_u[k].record(stream)
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
    update_span_ms = sum(u.elapsed_time(a) for u, (a, _) in zip(ev_u, ev)) / K
    ms_total, rays = job_totals(ms_total, rays, world, "cuda")
    value = rays / (ms_total * 1e-3) / 1e6

    # ---- algorithmic bytes of the trace kernel (device counters of the last timed frame) ----
    alg_bytes = (st_last.node_visits * NODE_BYTES + st_last.triangle_tests * TRI_BYTES +
                 st_last.rays_traced * RAY_BYTES + st_last.hit_fetches * HIT_FETCH_BYTES + W_ * H_ * 7 * 16)
    trace_avg_ms = sum(trace_ms) / len(trace_ms)
    achieved = alg_bytes / (trace_avg_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    num_sms = torch.cuda.get_device_properties(local).multi_processor_count

    # ---- e2e through the C ABI with host buffers ----
    # Two frames in flight, as the reference keeps frames in flight behind fences
    # (VulkanBaseRenderer.cpp:727-869): frame k's image streams back to page-locked memory on a
    # copy stream while frame k+1 renders; the compose pass of k+1 waits until k's copy is out.
    copy_stream = torch.cuda.Stream()
    outs = [torch.empty((H_, W_, 4), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    rendered = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]

    def e2e_frame(k, fc_host):
        j = k % 2
        r.trace_pass(fc_host, stream)
        r.reproject_pass(fc_host, stream)
        if k > 0:
            stream.wait_event(copied[1 - j])
        r.denoise_pass(fc_host, stream)
        r.end_frame(stream)
        rendered[j].record(stream)
        copy_stream.wait_event(rendered[j])
        if k > 1:
            copied[j].synchronize()          # frame k-2's buffer is back on the host before its reuse
        r.read_image_async(abi.IMG_DENOISED, outs[j], copy_stream)
        copied[j].record(copy_stream)

    for i in range(min(Wm, 3)):
        e2e_frame(i, fcs[i])
    copy_stream.synchronize()
    r.synchronize(stream)
    barrier()
    e2e_rays0 = r.stats().rays_total
    t0 = time.perf_counter()
    for k in range(K):
        fc_host = fb.build(cam.orbit(orbit * (Wm + k)), Wm + k)   # frame constants built in host memory
        if insts is not None:
            r.update_instances(insts[Wm + k], stream)              # host instance records
        e2e_frame(k, fc_host)
    copy_stream.synchronize()                                      # the last frame's image is on the host
    e2e_s = time.perf_counter() - t0
    e2e_rays = r.stats().rays_total - e2e_rays0
    barrier()
    e2e_ms, e2e_rays = job_totals(e2e_s * 1e3, e2e_rays, world, "cuda")
    e2e_s = e2e_ms * 1e-3
    e2e_value = e2e_rays / e2e_s / 1e6

    # ---- the same frames with the instance level refit instead of rebuilt (animated scenes) ----
    # Frame rays differ between runs of the same frames (moving pixels get 4x samples while
    # their motion moment lasts), so the comparison is Mrays/s and the update's own time.
    refit = None
    if insts is not None:
        def call_host_ms(fn, frames):   # host time of an update call with the GPU idle
            t = []
            for i in frames:
                r.synchronize(stream)
                t0 = time.perf_counter()
                fn(insts[i], stream)
                t.append(time.perf_counter() - t0)
            r.synchronize(stream)
            return sum(t) / len(t) * 1e3
        rebuild_host = call_host_ms(r.update_instances, [Wm + i % K for i in range(3)])
        r.update_instances(insts[0], stream)        # the tree of frame 0's layout; refits from here on
        refit_host = call_host_ms(r.refit_instances, range(1, Wm))
        for i in range(1, Wm):
            r.refit_instances(insts[i], stream)
            r.render(fcs[i], stream)
        r.synchronize(stream)
        s0r = r.stats()
        fe = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
        rs, re_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        barrier()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            rs.record(stream)
            for k in range(K):
                fc = fcs[Wm + k]
                fe[k][0].record(stream)
                r.refit_instances(insts[Wm + k], stream)
                fe[k][1].record(stream)
                r.trace_pass(fc, stream)
                fe[k][2].record(stream)
                r.reproject_pass(fc, stream)
                r.denoise_pass(fc, stream)
                r.end_frame(stream)
            re_.record(stream)
            torch.cuda.synchronize()
        s1r = r.stats()
        ms_r = rs.elapsed_time(re_)
        # every level rebuilt every frame (mesh trees too, although the moving spheres are
        # rigid instances of one mesh): the instances set by a refit, then a full GPU build
        fa = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
        ra0, ra1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0a = r.stats()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            ra0.record(stream)
            for k in range(K):
                fc = fcs[Wm + k]
                fa[k][0].record(stream)
                r.refit_instances(insts[Wm + k], stream)
                r.build_bvh(abi.BUILD_ALL, stream)
                fa[k][1].record(stream)
                r.trace_pass(fc, stream)
                r.reproject_pass(fc, stream)
                r.denoise_pass(fc, stream)
                r.end_frame(stream)
            ra1.record(stream)
            torch.cuda.synchronize()
        s1a = r.stats()
        ms_a = ra0.elapsed_time(ra1)
        all_levels = {"mrays_s": (s1a.rays_total - s0a.rays_total) / (ms_a * 1e-3) / 1e6, "ms_per_frame": ms_a / K,
                      "update_span_ms": sum(a.elapsed_time(b) for a, b in fa) / K}
        # the refit-or-rebuild policy over the same frames (growth limit 1.25)
        fp = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(K)]
        rp0, rp1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r.update_instances(insts[Wm], stream)
        r.synchronize(stream)
        s0p = r.stats()
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            rp0.record(stream)
            for k in range(K):
                fc = fcs[Wm + k]
                fp[k][0].record(stream)
                r.update_instances_auto(insts[Wm + k], 1.25, stream)
                fp[k][1].record(stream)
                r.trace_pass(fc, stream)
                r.reproject_pass(fc, stream)
                r.denoise_pass(fc, stream)
                r.end_frame(stream)
            rp1.record(stream)
            torch.cuda.synchronize()
        s1p = r.stats()
        ms_p = rp0.elapsed_time(rp1)
        auto = {"mrays_s": (s1p.rays_total - s0p.rays_total) / (ms_p * 1e-3) / 1e6, "ms_per_frame": ms_p / K,
                "update_span_ms": float(np.median([a.elapsed_time(b) for a, b in fp])),
                "refits": s1p.tlas_refits - s0p.tlas_refits, "rebuilds": s1p.tlas_rebuilds - s0p.tlas_rebuilds}
        refit = {"mrays_s": (s1r.rays_total - s0r.rays_total) / (ms_r * 1e-3) / 1e6,
                 "ms_per_frame": ms_r / K,
                 "trace_ms": sum(a.elapsed_time(b) for _, a, b in fe) / K,
                 "update_span_ms": sum(a.elapsed_time(b) for a, b, _ in fe) / K,
                 "rebuild_update_span_ms": update_span_ms,
                 "call_host_ms": refit_host, "rebuild_call_host_ms": rebuild_host,
                 "refits": s1r.tlas_refits - s0r.tlas_refits,
                 "node_visits_last_frame": s1r.node_visits,
                 "node_visits_last_frame_rebuilt": st_last.node_visits,
                 "all_levels_rebuilt_each_frame": all_levels, "auto_policy": auto}

    # ---- probe grid (after the timed frames: a baked grid changes path termination) ----
    probe_ms = None
    if WORKLOAD == "bricks" and rank == 0:
        e0, e1, e2, e3 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
        r.probe_voxelize(stream)
        r.probe_bake(fcs[0], 0, None, stream)
        r.synchronize(stream)
        per = (r.PROBE_COUNT // 64) // 120
        with torch.cuda.stream(stream):
            e0.record()
            r.probe_voxelize(stream)
            e1.record()
            r.probe_bake_slice(fcs[0], 7, 120, stream)
            e2.record()
            r.probe_bake(fcs[0], 0, None, stream)
            e3.record()
        r.synchronize(stream)
        probe_ms = {"voxelize_grid": e0.elapsed_time(e1), "bake_slice_f120": e1.elapsed_time(e2),
                    "bake_grid": e2.elapsed_time(e3), "slice_probes": per * 64, "grid_probes": r.PROBE_COUNT}

    # ---- the instance-level update inside a frame: enqueued while the GPU traces a frame, so the
    # host work (tables, emitter alias table) overlaps it and the span is the update's device time ----
    inst_inframe_ms = None
    if WORKLOAD == "bricks" and rank == 0:
        spans = []
        for k in range(4):
            u0, u1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                r.trace_pass(fcs[k % len(fcs)], stream)
                u0.record(stream)
                r.update_instances(sc.instances, stream)
                u1.record(stream)
            r.synchronize(stream)
            spans.append(u0.elapsed_time(u1))
        inst_inframe_ms = float(np.median(spans))

    # ---- output stage: the denoised frame onto a 4K presentation image (mean of 20 launches) ----
    output_ms = None
    if WORKLOAD == "bricks" and rank == 0:
        r.output_resize(3840, 2160)
        res = {}
        for name, mode, size in (("resolve_to_3840x2160", abi.OUTPUT_RESOLVE, (3840, 2160)),
                                 ("fsr_to_3840x2160", abi.OUTPUT_FSR, (3840, 2160))):
            r.output_pass(mode, (0, 0), size, stream=stream)
            r.synchronize(stream)
            o0, o1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                o0.record()
                for _ in range(20):
                    r.output_pass(mode, (0, 0), size, stream=stream)
                o1.record()
            r.synchronize(stream)
            res[name] = o0.elapsed_time(o1) / 20
        res["store_gbs_resolve"] = 3840 * 2160 * 4 / (res["resolve_to_3840x2160"] * 1e-3) / 1e9
        output_ms = res
        r.output_resize(0, 0)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": Wm,
                "ms_per_step": ms_total / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": workload_config(),
                "ms_per_frame": ms_total / K, "trace_ms": trace_avg_ms, "rays_per_frame": rays / max(K, 1) / world,
                "trace_pass_mrays_s": rays / max(K, 1) / world / (trace_avg_ms * 1e-3) / 1e6,
                "gpu_launches": 3 * K + 2 * K * (fcs[0].denoiser == abi.DENOISE_ATROUS) + build_launches,
                "probe_ms": probe_ms,
                "output_ms": output_ms,
                "tlas_refit": refit,
                "bvh_build_ms": {"all_levels": build_all_ms, "instance_level": build_inst_ms,
                                 "instance_level_device_span": build_inst_device_ms,
                                 "instance_level_in_frame_device_ms": inst_inframe_ms,
                                 "scene_load_s": load_s, "triangles": int(sc.triangle_count),
                                 "instances": int(sc.instances.shape[0])},
                "e2e": {"value": e2e_value, "unit": UNIT, "frames_in_flight": 2,
                        "h2d_bytes_per_step": ctypes.sizeof(abi.GkrtFrameConstants),
                        "d2h_bytes_per_step": W_ * H_ * 16, "ms_per_frame": e2e_s / K * 1e3},
                "roofline": trace_roofline(st_last, trace_avg_ms, alg_bytes, achieved, peak, peak_kind, num_sms,
                                           clk.summary()),
                "clocks": clk.summary()}
        if world == 1 and WORKLOAD == "bricks" and not args.no_city:
            line["city"] = city_measure(local)
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
    ap.add_argument("--no-city", action="store_true", help="skip the 4K city frames of the default line")
    ap.add_argument("--size", default=None, help="WxH override for profiling small cases (default 1920x1080)")
    ap.add_argument("--workload", default="bricks", choices=["bricks", "city", "denoiser"],
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
    if WORKLOAD == "denoiser":
        return run_denoiser(args)
    return run_gkrt(args)


if __name__ == "__main__":
    sys.exit(main())
