#!/usr/bin/env python
"""Throughput benchmark of the GB300 path tracer.

Workload (default): the Cornell room filled with a homogeneous isotropic
medium (sigma_a 0.05, sigma_s 0.2) plus 998,560 triangles as eight seeded
Perlin-displaced geodesic spheres with metallic/roughness materials,
1920 x 1080, 256 samples per pixel, depth 12, batch size 4: 530,841,600 paths
per step. A step is one full render through the C ABI (vvpt_render).

Our arm prints one JSON line: value = paths/s with the scene resident and the
outputs in device memory, timed with CUDA events on the stream the kernels run
on, a 512 MB L2 flush before every step; e2e = the same render with host
(pinned) output buffers, so the three RGBA32F images come back every step;
roofline = the dominant wavefront kernel's algorithmic bytes per launch over
its CUDA-event launch time (from a profiled render of the same workload);
cpu_baseline = the CPU oracle on a bounded pixel sample of the same workload.

--impl reference times the reference's path on the host cores. The reference
implements this path only as GLSL ray-tracing shaders that need a Vulkan RT
device, so the CPU restatement of those shaders (the oracle) stands in for it.

N > 1 GPUs (torchrun): every rank renders the full workload as an
independent replica (the path needs no exchange; replicas only), value is the
aggregate paths/s over the max per-rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "paths/sec"
UNIT = "paths/s"


def workload(name: str):
    from vviewer_gb300 import scenes
    if name == "cornell_medium":
        engine, info = scenes.cornell_medium(seed=1)
        desc = {"workload": "cornell_medium_1080p", "width": info.width, "height": info.height,
                "spp": info.samples, "depth": info.depth, "batch_size": info.batch_size,
                "triangles": 998596, "medium": {"sigma_a": 0.05, "sigma_s": 0.2, "g": 0.0},
                "materials": "Lambert walls, metallic/roughness spheres", "seed": 1}
    elif name == "instanced_sky":
        engine, info = scenes.instanced_sky_scene(seed=1)
        desc = {"workload": "instanced_sky_4k", "width": info.width, "height": info.height, "spp": info.samples,
                "depth": info.depth, "batch_size": info.batch_size, "instances": 512,
                "instanced_triangles": 20736000, "unique_triangles": 324000, "mesh_lights": 32,
                "sky": "4096x2048 procedural equirect, Gaussian sun peak 5e4", "lens_radius": 0.02,
                "env_is": True, "seed": 1}
    elif name == "cornell":
        engine, info = scenes.cornell_box(seed=1)
        desc = {"workload": "cornell_256", "width": info.width, "height": info.height, "spp": info.samples,
                "depth": info.depth, "batch_size": info.batch_size, "triangles": 36, "seed": 1}
    else:
        raise SystemExit(f"unknown workload {name}")
    return engine, info, desc


def apply_overrides(engine, info, desc, args):
    """Smaller cases of the same scene (profiling captures); the default is the full workload."""
    if args.width or args.height or args.spp:
        info.width = args.width or info.width
        info.height = args.height or info.height
        info.samples = args.spp or info.samples
        desc = {**desc, "workload": f"{desc['workload']}_{info.width}x{info.height}_{info.samples}spp",
                "width": info.width, "height": info.height, "spp": info.samples}
    return engine, info, desc


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernel: str, units_per_launch: float):
    """DRAM bytes per launch of `kernel`: the committed ncu summary's DRAM
    bytes per work unit (a capture of a smaller case of the same scene)
    times this run's work units per launch."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        text = f.read_text()
        m = re.search(rf"traffic_per_unit\[{re.escape(kernel)}\]\s*=\s*([0-9.eE+]+)", text)
        if m:
            return float(m.group(1)) * units_per_launch, f.name
    return None, None


def profiled_limiter(kernel: str):
    """The committed ncu summary's issue figures of `kernel` (lines
    `issue_active[k] = f` and `threads_per_warp_instruction[k] = n`): what
    bounds a kernel whose HBM roofline fraction is small by construction."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        text = f.read_text()
        a = re.search(rf"issue_active\[{re.escape(kernel)}\]\s*=\s*([0-9.eE+]+)", text)
        t = re.search(rf"threads_per_warp_instruction\[{re.escape(kernel)}\]\s*=\s*([0-9.eE+]+)", text)
        if a and t:
            return {"kind": "instruction issue under SIMT divergence, then memory latency",
                    "issue_active": float(a.group(1)), "threads_per_warp_instruction": float(t.group(1)),
                    "source": f.name}
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if self.file is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(engine, info, target_s: float = 15.0) -> dict:
    """The CPU oracle on a bounded, evenly spread pixel sample at full spp."""
    from oracle import oracle
    flat = engine.scene.build()
    sd = engine.scene.scene_data(info.width, info.height)
    npix = info.width * info.height
    cores = os.cpu_count() or 1

    def run(k):
        pix = np.linspace(0, npix - 1, k).astype(np.uint32)
        t = time.perf_counter()
        oracle.render(flat, sd, info, pixels=pix, threads=cores)
        return time.perf_counter() - t

    k = 4 * cores
    dt = run(k)
    while dt < 1.0 and k < npix:
        k = min(npix, k * 4)
        dt = run(k)
    k = int(min(npix, max(k, k * target_s / max(dt, 1e-6))))
    dt = run(k)
    paths = k * (info.samples // info.batch_size) * info.batch_size
    return {"value": paths / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{k} of {npix} pixels evenly spread, all {info.samples} spp, depth {info.depth}: "
                      f"{paths} paths in {dt:.1f} s"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import oracle
    engine, info, desc = apply_overrides(*workload(args.workload), args)
    flat = engine.scene.build()
    sd = engine.scene.scene_data(info.width, info.height)
    npix = info.width * info.height
    cores = os.cpu_count() or 1
    spp = (info.samples // info.batch_size) * info.batch_size
    # size one step at about 6 s of CPU work
    def timed(k):
        t = time.perf_counter()
        oracle.render(flat, sd, info, pixels=np.linspace(0, npix - 1, k).astype(np.uint32), threads=cores)
        return time.perf_counter() - t

    k = 8 * cores
    dt = timed(k)
    while dt < 1.0 and k < npix:
        k = min(npix, k * 4)
        dt = timed(k)
    k = int(min(npix, max(k, k * 6.0 / max(dt, 1e-6))))
    pix = np.linspace(0, npix - 1, k).astype(np.uint32)
    for _ in range(args.warmup):
        oracle.render(flat, sd, info, pixels=pix, threads=cores)
    times = []
    for _ in range(args.steps):
        t = time.perf_counter()
        oracle.render(flat, sd, info, pixels=pix, threads=cores)
        times.append(time.perf_counter() - t)
    total = sum(times)
    value = k * spp * args.steps / total
    sample = f"{k} of {npix} pixels evenly spread per step, all {info.samples} spp, depth {info.depth}"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": desc, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "the reference implements this path only as Vulkan ray-tracing shaders; its CPU "
                    "restatement (oracle/) runs on all host cores"}
    print(json.dumps(line), flush=True)


def replica_throughput(local_ms: float, units_per_rank: float, world: int, device=None) -> tuple[float, float]:
    """Whole-job throughput of N independent replicas: the slowest rank's time
    (max over ranks) and world * units / that time. Collective over the
    default process group when world > 1 (NCCL on GPUs, gloo in the tests)."""
    total_ms = local_ms
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([local_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, world * units_per_rank / (total_ms / 1e3)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    from vviewer_gb300 import Context

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    engine, info, desc = apply_overrides(*workload(args.workload), args)
    t0 = time.perf_counter()
    flat = engine.scene.build()
    sd = engine.scene.scene_data(info.width, info.height)
    scene_prep_s = time.perf_counter() - t0
    ctx = Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    gpu = ctx.upload(flat)
    upload_s = time.perf_counter() - t0
    H, W = info.height, info.width
    dev = {k: torch.zeros((H, W, 4), dtype=torch.float32, device="cuda") for k in ("radiance", "albedo", "normal")}
    dev_ptrs = {k: v.data_ptr() for k, v in dev.items()}
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    paths_per_step = W * H * (info.samples // info.batch_size) * info.batch_size

    env_is = bool(desc.get("env_is", False))
    tuning = None
    if args.tuning:
        slots, blocks = (int(x) for x in args.tuning.split(","))
        ctx.set_tuning(slots=slots, blocks_per_sm=blocks)
        tuning = {"slots": slots, "blocks_per_sm": blocks, "threads_per_block": 0, "iterations_per_graph": 0}
    elif not args.no_autotune:
        tuning = gpu.autotune(sd, info, budget_ms=4000.0, env_is=env_is)
    for _ in range(args.warmup):
        gpu.render(sd, info, outputs=dev_ptrs, env_is=env_is)
    torch.cuda.synchronize()

    step_ms = []
    launches = 0
    with ClockSampler(local) as clocks:
        for _ in range(args.steps):
            flush.fill_(1.0)  # evict L2 between steps
            barrier()
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            gpu.render(sd, info, outputs=dev_ptrs, env_is=env_is)
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
            step_ms.append(e0.elapsed_time(e1))
            launches += int(ctx.stats().kernel_launches)
    clock = clocks.summary()
    total_ms, value = replica_throughput(sum(step_ms), paths_per_step * args.steps, world, "cuda")
    stats = ctx.stats()

    # e2e: host (pinned) output buffers, SceneData/RenderInfo from the host every step
    pinned = {k: torch.zeros((H, W, 4), dtype=torch.float32).pin_memory() for k in ("radiance", "albedo", "normal")}
    host_ptrs = {k: v.data_ptr() for k, v in pinned.items()}
    e2e_s = []
    for i in range(args.warmup + args.steps):
        sd_step = engine.scene.scene_data(W, H)
        flush.fill_(1.0)
        torch.cuda.synchronize()
        barrier()
        t = time.perf_counter()
        gpu.render(sd_step, info, host_outputs=host_ptrs, env_is=env_is)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            e2e_s.append(dt)
    e2e_ms, _ = replica_throughput(1e3 * sum(e2e_s), paths_per_step * args.steps, world, "cuda")
    e2e_total = e2e_ms / 1e3
    import ctypes as C

    from vviewer_gb300 import _native as N
    e2e = {"value": world * paths_per_step * args.steps / e2e_total, "unit": UNIT,
           "h2d_bytes_per_step": C.sizeof(N.SceneData) + C.sizeof(N.RenderInfo),
           "d2h_bytes_per_step": 3 * H * W * 16}

    # roofline of the dominant kernel from one profiled render of the same workload
    gpu.render(sd, info, outputs=dev_ptrs, profile=True, env_is=env_is)
    prof = [k for k in ctx.kernel_profile() if k["name"] != "k_begin"]
    total_prof = sum(k["total_ms"] for k in ctx.kernel_profile())
    dom = max(prof, key=lambda k: k["total_ms"])
    avg_ms = dom["total_ms"] / max(dom["launches"], 1)
    bytes_per_launch = dom["units"] * dom["bytes_per_unit"] / max(dom["launches"], 1)
    achieved = bytes_per_launch / (avg_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic, traffic_src = profiled_traffic(dom["name"], dom["units"] / max(dom["launches"], 1))
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": dom["name"], "peak_source": f"{peak_kind} hbm_gbs (copy)",
                "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_ms,
                "traffic_source": traffic_src, "limiter": profiled_limiter(dom["name"]),
                "kernels": [{**k, "share": k["total_ms"] / total_prof} for k in ctx.kernel_profile()]}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {**desc, "parallelism": f"replicas x{world}", "tuning": tuning,
                       "l2": "512 MB L2 flush before every step; working set (path state + per-batch sums) > L2"},
            "e2e": e2e, "roofline": roofline, "gpu_launches": launches, "clocks": clock,
            "segments_per_step": int(stats.segments), "shadow_rays_per_step": int(stats.shadow_rays),
            "emitter_rays_per_step": int(stats.emitter_rays), "scene_prep_s": scene_prep_s,
            "scene_upload_bvh_s": upload_s}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(engine, info)
    gpu.release()
    ctx.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


N_SCENES = 64


def _job_scenes(ctx, n_scenes: int):
    """The seeded scene pool of the batched and serving workloads, resident."""
    from vviewer_gb300 import scenes
    engines = [scenes.random_scene(100 + k) for k in range(n_scenes)]
    gpus = [ctx.upload(e.scene.build()) for e in engines]
    tris = [sum(int(np.prod(m.indices.shape)) // 3 for m in e.scene.build().meshes) for e in engines]
    return engines, gpus, tris


def run_batched(args) -> None:
    """64 jobs from the seeded job mix, each with its own scene (10k-2M
    triangles, 256^2 to 1920x1080, 16/64/256 spp) rendered together through the job engine: one
    step submits all 64 and waits for the last. value = total paths / wall
    time with device outputs; e2e = the same with host outputs; the same jobs
    one after another through vvpt_render give sequential_paths_per_s."""
    import torch

    from vviewer_gb300 import Context, scenes
    ctx = Context(0)
    engines, gpus, tris = _job_scenes(ctx, N_SCENES)
    mix = scenes.job_mix(1, 64, N_SCENES, distinct=True)
    sds = [engines[k].scene.scene_data(i.width, i.height) for k, i in mix]
    paths = sum(i.width * i.height * (i.samples // i.batch_size) * i.batch_size for _, i in mix)
    dev = [{k: torch.zeros((i.height, i.width, 4), dtype=torch.float32, device="cuda")
            for k in ("radiance", "albedo", "normal")} for _, i in mix]
    ptrs = [{k: v.data_ptr() for k, v in d.items()} for d in dev]

    def step(host: bool):
        jobs = []
        for (k, info), sd, p in zip(mix, sds, ptrs):
            jobs.append(gpus[k].submit(sd, info, outputs=None if host else p))
        for j in jobs:
            j.wait()
        lat = []
        for j in jobs:
            ji = j.poll()
            lat.append(ji.end_ms - ji.submit_ms)
            j.release()
        return lat

    # queue sizes and persistent-block counts for the engine (it starts with
    # the context's tuning at the first submit)
    tuning = None
    if not args.no_autotune:
        rep = type(mix[0][1])(samples=64, depth=8, batch_size=4, width=1024, height=1024, write_files=False)
        tuning = gpus[0].autotune(engines[0].scene.scene_data(1024, 1024), rep, budget_ms=4000.0)
    warm = scenes.job_mix(2, 4, N_SCENES)
    for _ in range(max(args.warmup, 1)):
        js = [gpus[k].submit(engines[k].scene.scene_data(64, 64),
                             type(i)(samples=16, depth=8, batch_size=4, width=64, height=64, write_files=False))
              for k, i in warm]
        for j in js:
            j.wait()
            j.release()
    torch.cuda.synchronize()
    times, lats = [], []
    with ClockSampler(0) as clocks:
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            lats += step(False)
            torch.cuda.synchronize()
            times.append(time.perf_counter() - t)
    clock = clocks.summary()
    e2e_t = []
    for _ in range(args.steps):
        t = time.perf_counter()
        step(True)
        e2e_t.append(time.perf_counter() - t)
    line = {"metric": METRIC, "value": paths * args.steps / sum(times), "unit": UNIT, "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scenes)",
            "config": {"workload": "batched_64_jobs", "jobs": 64, "scenes": N_SCENES, "scene_triangles": tris,
                       "resolutions": "256^2 / 512^2 / 1024^2 / 1920x1080", "spp": "16 / 64 / 256",
                       "depth": 8, "batch_size": 4, "paths_per_step": paths, "seed": 1, "tuning": tuning,
                       "l2": "per-job batch sums and path state far above L2"},
            "e2e": {"value": paths * args.steps / sum(e2e_t), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": sum(3 * i.width * i.height * 16 for _, i in mix)},
            "job_latency_ms": {"p50": float(np.percentile(lats, 50)), "max": float(np.max(lats))},
            "clocks": clock}
    if args.sequential:
        t = time.perf_counter()
        for (k, info), sd, p in zip(mix, sds, ptrs):
            gpus[k].render(sd, info, outputs=p)
        torch.cuda.synchronize()
        line["sequential_paths_per_s"] = paths / (time.perf_counter() - t)
    for g in gpus:
        g.release()
    ctx.close()
    print(json.dumps(line), flush=True)


def run_serving(args) -> None:
    """512 requests with Poisson arrivals (mean gap 50 ms, seeded) against the
    resident pool of the batched workload's 64 scenes, sizes and spp drawn as
    in the batched workload, admitted against a 150 GB device-memory budget
    (--preview: 256^2 / 512^2 at 8 / 16 / 32 spp instead). A submitter
    thread issues each request at its arrival time; latency = submit to the
    finished image in host memory. value = aggregate paths/s from the first
    arrival to the last completion."""
    import threading

    import torch

    from vviewer_gb300 import Context, scenes
    ctx = Context(0)
    ctx.set_budget(150 * (1 << 30))
    engines, gpus, tris = _job_scenes(ctx, N_SCENES)
    reqs = scenes.serving_requests(1, args.requests, N_SCENES, preview=args.preview)
    sds = [engines[k].scene.scene_data(i.width, i.height) for _, k, i in reqs]
    paths = sum(i.width * i.height * (i.samples // i.batch_size) * i.batch_size for _, _, i in reqs)
    tuning = None
    if not args.no_autotune:
        rep = type(reqs[0][2])(samples=16, depth=8, batch_size=4, width=512, height=512, write_files=False)
        tuning = gpus[0].autotune(engines[0].scene.scene_data(512, 512), rep, budget_ms=3000.0)
    for _ in range(max(args.warmup, 1)):
        j = gpus[0].submit(sds[0], reqs[0][2])
        j.wait()
        j.release()
    torch.cuda.synchronize()
    jobs = [None] * len(reqs)

    def submitter():
        t0 = time.perf_counter()
        for n, ((at, k, info), sd) in enumerate(zip(reqs, sds)):
            delay = at / 1e3 - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            jobs[n] = gpus[k].submit(sd, info)

    with ClockSampler(0) as clocks:
        th = threading.Thread(target=submitter)
        t = time.perf_counter()
        th.start()
        th.join()
        for j in jobs:
            j.wait()
        wall = time.perf_counter() - t
    clock = clocks.summary()
    infos = [j.poll() for j in jobs]
    lat = np.array([ji.end_ms - ji.submit_ms for ji in infos])
    span_ms = max(ji.end_ms for ji in infos) - min(ji.submit_ms for ji in infos)
    for j in jobs:
        j.release()
    line = {"metric": METRIC, "value": paths / (span_ms / 1e3), "unit": UNIT, "n_gpus": 1, "steps": 1,
            "warmup": args.warmup, "ms_per_step": span_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes, Poisson arrivals)",
            "config": {"workload": "serving_512_requests", "requests": len(reqs), "mean_gap_ms": 50.0,
                       "scenes": N_SCENES, "scene_triangles": tris,
                       "resolutions": "256^2 / 512^2" if args.preview else "256^2 / 512^2 / 1024^2 / 1920x1080",
                       "spp": "8 / 16 / 32" if args.preview else "16 / 64 / 256", "depth": 8, "batch_size": 4,
                       "paths": paths, "seed": 1, "latency": "submit to the finished image on the host",
                       "budget_bytes": 150 * (1 << 30), "outputs": "host", "tuning": tuning},
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p90": float(np.percentile(lat, 90)),
                           "p99": float(np.percentile(lat, 99)), "max": float(lat.max()),
                           "mean": float(lat.mean())},
            "offered_paths_per_s": paths / (reqs[-1][0] / 1e3), "wall_s": wall,
            "e2e": {"value": paths / (span_ms / 1e3), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": sum(3 * i.width * i.height * 16 for _, _, i in reqs)},
            "clocks": clock}
    for g in gpus:
        g.release()
    ctx.close()
    print(json.dumps(line), flush=True)


def denoiser_flops(h: int, w: int, n: int = 1) -> float:
    """Multiply-add FLOPs of one U-Net forward pass (2 per MAC, 3x3 taps)."""
    from oracle import denoiser_oracle as D
    lv_of = []
    for l in range(D.LEVELS):
        lv_of += [l, l]
    for l in range(D.LEVELS - 2, -1, -1):
        lv_of += [l, l]
    lv_of.append(0)
    total = 0.0
    for (cin, cout, _), l in zip(D.layers(), lv_of):
        total += 2.0 * 9 * cin * cout * n * (h >> l) * (w >> l)
    return total


def denoiser_layer_bounds(h: int, w: int, hbm_gbs: float, tflops: float) -> list[dict]:
    """Per convolution layer of one forward pass: FLOPs, compulsory bytes
    (BF16 input and output activations once, BF16 weights once) and the
    roofline time max(bytes / HBM, FLOP / tensor peak). The 32-channel
    full-resolution layers sit below the ridge (about 144 FLOP/B against
    peak/HBM of about 285), so HBM bounds them."""
    from oracle import denoiser_oracle as D
    lv_of = []
    for l in range(D.LEVELS):
        lv_of += [l, l]
    for l in range(D.LEVELS - 2, -1, -1):
        lv_of += [l, l]
    lv_of.append(0)
    out = []
    for k, ((cin, cout, _), l) in enumerate(zip(D.layers(), lv_of)):
        px = (h >> l) * (w >> l)
        fl = 2.0 * 9 * cin * cout * px
        by = 2.0 * px * (cin + cout) + 2.0 * 9 * cin * cout
        t_hbm = by / (hbm_gbs * 1e9) * 1e3
        t_tc = fl / (tflops * 1e12) * 1e3
        out.append({"layer": k, "level": l, "cin": cin, "cout": cout, "flops": fl, "bytes": by,
                    "flop_per_byte": fl / by, "bound": "hbm" if t_hbm > t_tc else "tensor",
                    "bound_ms": max(t_hbm, t_tc)})
    return out


def run_denoise(args) -> None:
    """Denoiser inference at 3840 x 2160 (one frame; --width/--height for
    another size, multiples of 16) and one training step on 8 crops of 256^2,
    CUDA events on the library stream; roofline against the measured dense
    BF16 peak."""
    import torch

    from vviewer_gb300 import Context
    from vviewer_gb300.denoiser import Denoiser
    ctx = Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    dn = Denoiser(ctx, seed=1)
    H, W = (args.height or 2160), (args.width or 3840)
    if H % 16 or W % 16:
        raise SystemExit("denoise: width and height must be multiples of 16")
    g = torch.Generator(device="cuda").manual_seed(1)
    rad = torch.rand((H, W, 4), device="cuda", generator=g) * 4
    alb = torch.rand((H, W, 4), device="cuda", generator=g)
    nrm = torch.rand((H, W, 4), device="cuda", generator=g)
    out = torch.empty((H, W, 4), device="cuda")
    for _ in range(max(args.warmup, 1)):
        dn.apply(rad, alb, nrm, out)
    torch.cuda.synchronize()
    ms = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        dn.apply(rad, alb, nrm, out)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    infer_ms = sum(ms) / len(ms)
    flops = denoiser_flops(H, W)
    # training step, 8 x 256^2
    train_ms = None
    if not args.no_train:
        tb = [torch.rand((8, 256, 256, 4), device="cuda", generator=g) for _ in range(4)]
        for _ in range(3):
            dn.train_step(*tb, lr=1e-4)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(5):
            dn.train_step(*tb, lr=1e-4)
        torch.cuda.synchronize()
        train_ms = (time.perf_counter() - t0) / 5 * 1e3
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    achieved = flops / (infer_ms / 1e3) / 1e12
    layers = denoiser_layer_bounds(H, W, hbm, peak)
    bound_ms = sum(l["bound_ms"] for l in layers)
    line = {"metric": "denoised frames/s", "value": 1e3 / infer_ms, "unit": "frames/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": infer_ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (fp32 accumulate)", "data": "synthetic inputs",
            "config": {"workload": f"denoise_{W}x{H}", "network": "U-Net 5 levels 32/48/64/96/128, 3x3",
                       "train_batch": "8 x 256^2",
                       "l2": "inputs (3 RGBA32F images, 133 MB each at 3840x2160) and every activation larger "
                             "than L2"},
            "roofline": {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": None, "flops_per_frame": flops},
            "layer_roofline": {"bound_ms": bound_ms, "frac_of_bound": bound_ms / infer_ms,
                               "hbm_gbs": hbm, "tensor_tflops": peak, "layers": layers},
            "train_step_ms": train_ms,
            "train_tflops": 3 * denoiser_flops(256, 256, 8) / (train_ms / 1e3) / 1e12 if train_ms else None}
    dn.close()
    ctx.close()
    print(json.dumps(line), flush=True)


def pick_operating_point(sweep: list, target: float) -> tuple[dict, str]:
    """The served input spp of the converged workload: the fewest spp whose
    denoised error meets the target; when none does, the spp where the
    denoiser gains most over the plain tracer at equal error. Entries are in
    increasing spp order."""
    met = [r for r in sweep if r["rel_rmse_denoised"] <= target]
    if met:
        return met[0], "fewest spp meeting the target"
    return (max(sweep, key=lambda r: r["gain_at_equal_error"] or 0.0),
            "target not met at any spp: largest gain at equal error")


def _rel_rmse(img, ref) -> float:
    """Relative RMSE of an image against a reference: the root of
    sum((img - ref)^2) / sum(ref^2) over the pixels and the three radiance
    channels."""
    d = img[..., :3].double() - ref[..., :3].double()
    return float((d.pow(2).sum() / ref[..., :3].double().pow(2).sum()).sqrt())


def run_converged(args) -> None:
    """Converged images per hour at relative RMSE <= 1e-2 against an
    FP64-accumulated 4096-spp render of the same view, on the C5 scene (512
    instances of seeded displaced meshes, 32 mesh lights, thin lens, a
    4096 x 2048 sky with a 5e4 sun, environment importance sampled) at
    960 x 544 (multiples of 16 for the denoiser).

    Plain single-job tracer: vvpt_render at 64 / 256 / 1024 spp; the error is
    fitted as e^2 = a / spp + b and the spp for the target read off the fit.
    Batched, served and denoised: M requests of the view submitted together
    to the job engine at a low spp, each denoised as it completes; images per
    hour = M / wall time, latency = submit to denoised image (p50 / p99).
    The denoiser is first trained on crops of other seeds of the same scene
    generator: 512^2 inputs at 4 / 8 / 16 spp stored as FP16 (radiance,
    albedo, normal) and 4096-spp FP64-accumulated targets."""
    import torch

    from vviewer_gb300 import Context, scenes
    from vviewer_gb300.denoiser import Denoiser
    ctx = Context(0)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    W, H = 960, 544
    target = 1e-2
    ref_spp = 4096
    keys = ("radiance", "albedo", "normal")

    def bufs(w, h, m2=False):
        return {k: torch.zeros((h, w, 4), device="cuda") for k in keys + (("radiance_m2",) if m2 else ())}

    def render(g, sd, info, spp, w, h, fp64=False, m2=False, sampler="rtgems"):
        info.samples = spp
        b = bufs(w, h, m2)
        torch.cuda.synchronize()
        t = time.perf_counter()
        g.render(sd, info, outputs={k: v.data_ptr() for k, v in b.items()}, env_is=True, reduce_fp64=fp64,
                 want_m2=m2, sampler=sampler)
        torch.cuda.synchronize()
        return b, time.perf_counter() - t

    # ---- training set: crops of other seeds
    t_set = time.perf_counter()
    crops = {k: [] for k in keys + ("target",)}
    in_spps = (4, 8, 16)
    for seed in range(2, 2 + args.train_crops):
        e, info = scenes.instanced_sky_scene(seed, 512, 512, 4, 8, 4, sky_w=2048, sky_h=1024)
        g = ctx.upload(e.scene.build())
        sd = e.scene.scene_data(512, 512)
        ref, _ = render(g, sd, info, ref_spp, 512, 512, fp64=True)
        for spp in in_spps:
            noisy, _ = render(g, sd, info, spp, 512, 512)
            for k in keys:
                crops[k].append(noisy[k].half())
            crops["target"].append(ref["radiance"].half())
        g.release()
    tset = {k: torch.stack(v).contiguous() for k, v in crops.items()}
    t_set = time.perf_counter() - t_set
    dn = Denoiser(ctx, seed=1)
    losses = []
    gen = torch.Generator().manual_seed(1)
    t_train = time.perf_counter()
    for step in range(args.train_steps):
        idx = torch.randint(0, tset["radiance"].shape[0], (4,), generator=gen).cuda()
        ys = int(torch.randint(0, 512 - 256 + 1, (1,), generator=gen)) // 16 * 16
        xs = int(torch.randint(0, 512 - 256 + 1, (1,), generator=gen)) // 16 * 16
        sub = [tset[k][idx, ys:ys + 256, xs:xs + 256].float().contiguous() for k in keys + ("target",)]
        lr = 2e-3 if step < args.train_steps * 3 // 4 else 5e-4
        losses.append(dn.train_step(*sub, lr=lr))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t_train

    # ---- the view the served images are measured on
    e, info = scenes.instanced_sky_scene(1, W, H, 16, 8, 4, sky_w=4096, sky_h=2048)
    g = ctx.upload(e.scene.build())
    sd = e.scene.scene_data(W, H)
    # The reference image takes the low-discrepancy sampler: the same
    # estimator (same expected image) on sample streams independent of the
    # RTGEMS streams of the images measured against it, whose first batches
    # it would otherwise share (one seed per batch index).
    ref, t_ref = render(g, sd, info, ref_spp, W, H, fp64=True, m2=True, sampler="pmj")
    nb = ref_spp // info.batch_size
    x = ref["radiance"][..., :3].double()
    var = (nb * ref["radiance_m2"][..., :3].double() - x * x).clamp(min=0) / (nb - 1)
    ref_noise = float((var.sum() / x.pow(2).sum()).sqrt())  # the reference's own relative RMSE

    # plain single-job tracer
    plain = {}
    for spp in (64, 256, 1024):
        img, t = render(g, sd, info, spp, W, H)
        plain[spp] = (_rel_rmse(img["radiance"], ref["radiance"]), t)
    paths_per_s = W * H * 1024 / plain[1024][1]
    e64, e1024 = plain[64][0] ** 2, plain[1024][0] ** 2
    a = max((e64 - e1024) / (1 / 64 - 1 / 1024), 1e-30)
    b = max(e1024 - a / 1024, 0.0)

    def plain_spp_for(err):
        return a / (err ** 2 - b) if err ** 2 > b else float("inf")

    spp_plain = plain_spp_for(target)
    t_plain = W * H * spp_plain / paths_per_s

    # denoised error by input spp (the engine's images are vvpt_render's, bit for bit)
    den = torch.zeros((H, W, 4), device="cuda")
    sweep = []
    for spp in (4, 8, 16, 32, 64):
        img, t_r = render(g, sd, info, spp, W, H)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dn.apply(img["radiance"], img["albedo"], img["normal"], den)
        torch.cuda.synchronize()
        t_d = time.perf_counter() - t0
        err = _rel_rmse(den, ref["radiance"])
        spp_eq = plain_spp_for(err)
        finite = spp_eq != float("inf")
        sweep.append({"spp": spp, "rel_rmse_noisy": _rel_rmse(img["radiance"], ref["radiance"]),
                      "rel_rmse_denoised": err, "render_s": t_r, "denoise_s": t_d,
                      "plain_spp_same_error": spp_eq if finite else None,
                      # the plain tracer's time for the same error over this render + denoise
                      "gain_at_equal_error": (W * H * spp_eq / paths_per_s) / (t_r + t_d) if finite else None})
    pick, pick_rule = pick_operating_point(sweep, target)

    # batched + served + denoised: M requests together through the job engine
    M = args.requests_converged
    outs = [bufs(W, H) for _ in range(M)]
    dens = [torch.zeros((H, W, 4), device="cuda") for _ in range(M)]
    info.samples = pick["spp"]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    jobs, t_sub = [], []
    for o in outs:
        t_sub.append(time.perf_counter())
        jobs.append(g.submit(sd, info, outputs={k: v.data_ptr() for k, v in o.items()}, env_is=True))
    lat = []
    for j, o, dd, ts in zip(jobs, outs, dens, t_sub):
        j.wait()
        dn.apply(o["radiance"], o["albedo"], o["normal"], dd)
        torch.cuda.synchronize()
        lat.append(1e3 * (time.perf_counter() - ts))
        j.release()
    wall = time.perf_counter() - t0
    served_err = _rel_rmse(dens[-1], ref["radiance"])
    served_iph = 3600.0 * M / wall
    # the plain tracer at the error the served images reach (the target when met)
    err_eq = max(served_err, target)
    t_plain_eq = W * H * plain_spp_for(err_eq) / paths_per_s
    plain_iph = 3600.0 / t_plain_eq  # 0 when the fit says the plain tracer cannot reach that error
    g.release()
    line = {"metric": "converged images/hour at relative RMSE <= 1e-2 vs the plain single-job tracer",
            "unit": "images/h", "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 tracer, bf16 denoiser",
            "data": "synthetic (seeded procedural scene)", "value": served_iph,
            "config": {"workload": "converged_instanced_sky_960x544", "target_rel_rmse": target,
                       "metric": "sqrt(sum((x - ref)^2) / sum(ref^2)) over RGB",
                       "reference": f"{ref_spp} spp, FP64-accumulated batch sums (VVPT_RENDER_REDUCE_FP64), "
                                    "environment importance sampled, PMJ sampler (streams independent of the "
                                    "measured RTGEMS images)",
                       "requests": M, "request_spp": pick["spp"], "request_spp_rule": pick_rule,
                       "train": f"{args.train_steps} steps of 4 x 256^2 crops from {args.train_crops} seeds x "
                                f"{len(in_spps)} input spp (4/8/16, FP16), {ref_spp}-spp FP64 targets"},
            "target_met": served_err <= target, "served_rel_rmse": served_err,
            "reference_rel_noise": ref_noise,
            "reference_rel_noise_from_fit": float(np.sqrt(b)),
            "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                           "max": float(np.max(lat))},
            "plain": {"images_per_hour": plain_iph,
                      "spp": plain_spp_for(err_eq) if plain_iph > 0 else None,
                      "seconds_per_image": t_plain_eq if plain_iph > 0 else None,
                      "at_rel_rmse": err_eq, "spp_for_target": spp_plain if spp_plain != float("inf") else None,
                      "seconds_for_target": t_plain if t_plain != float("inf") else None,
                      "fit": {"a": a, "b": b, "rel_rmse": {str(k): v[0] for k, v in plain.items()},
                              "paths_per_s": paths_per_s}},
            "gain_vs_plain": served_iph / plain_iph if plain_iph > 0 else None,
            "denoised_sweep": sweep, "train_set_s": t_set, "train_s": t_train,
            "final_train_loss": float(np.mean(losses[-20:])), "reference_s": t_ref}
    dn.close()
    ctx.close()
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["cornell_medium", "cornell", "instanced_sky", "batched64", "serving512",
                                           "denoise", "converged"],
                    default="cornell_medium")
    ap.add_argument("--sequential", action="store_true", help="batched64: also time the jobs one by one")
    ap.add_argument("--requests", type=int, default=512, help="serving512: number of requests")
    ap.add_argument("--preview", action="store_true", help="serving512: preview sizes and spp")
    ap.add_argument("--train-steps", type=int, default=1500, help="converged: denoiser training steps")
    ap.add_argument("--train-crops", type=int, default=16, help="converged: training scenes (512^2 crops)")
    ap.add_argument("--requests-converged", type=int, default=16, help="converged: requests served together")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-train", action="store_true", help="denoise: inference only (no training steps)")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default tuning (no vvpt_autotune pass)")
    ap.add_argument("--tuning", default="", help="SLOTS,BLOCKS_PER_SM: a fixed tuning instead of the autotune pass")
    ap.add_argument("--width", type=int, default=0)
    ap.add_argument("--height", type=int, default=0)
    ap.add_argument("--spp", type=int, default=0)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched64":
        run_batched(args)
    elif args.workload == "serving512":
        run_serving(args)
    elif args.workload == "denoise":
        run_denoise(args)
    elif args.workload == "converged":
        run_converged(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
