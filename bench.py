"""Benchmark of the path-tracing hot path on one GB300.

Workload (one step = one frame): the Cornell box with mixture-pdf light
sampling - 555-unit room, 130x105 light at emission 15, 165x330x165 box
rotated +15 deg, glass sphere r=90 - rendered at 600x600, 1024 samples per
pixel, max depth 50, reference semantics (black background), FP32 radiance.
Metric: Msamples/s = 600*600*1024 camera samples / frame time.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

value:  frames rendered from the scene already resident in HBM, image left in
        HBM, timed with CUDA events on the library's stream; L2 (129 MB) is
        flushed by writing a 256 MB buffer between timed steps.
e2e:    the same frame through the C ABI with host buffers: scene-arena upload
        (H2D), render, image download (D2H) inside the timed region.
cpu_baseline / --impl reference: the reference algorithm on the host cores
        (oracle/_ref linked from the reference sources when it was built here,
        else the CPU oracle port), on a bounded band of image rows.
learned_equal_time: the second half of the metric - relMSE against an FP64
        high-spp render of the learned renderers (path guiding and the
        radiance cache on the small-light Cornell box, the radiance cache on
        the next-week scene) next to
        the plain tracer: at equal spp, at equal wall time, and the wall time
        each needs to reach the plain tracer's relMSE (skip with
        --no-learned).
other_configs: the other throughput workloads of the benchmark definition,
        each with its own CPU baseline - one weekend (400x400, 16 spp), the
        64-scene batch (one persistent launch, the reference's BVH topology)
        and the next-week scene (800x800, 256 spp, reference semantics)
        (skip with --no-configs).
roofline.flops: useful work - the arithmetic the reference's algorithm does
        per ray segment, counted by the CPU oracle on a band of the same
        frame - at the measured segment rate, against the FP32 peak.
Multi-GPU (torchrun, N ranks): one frame split by sample ranges, rank r
        rendering samples [r*spp/N, (r+1)*spp/N) of every pixel, the float4
        accumulators summed across ranks (NCCL all-reduce) and resolved;
        scaling "strong" (the frame's work is fixed).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "tiny-path-tracer_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for _p in (PKG, ORACLE):
    if _p not in sys.path:
        sys.path.insert(0, _p)

W, H, SPP, DEPTH = 600, 600, 1024, 50
# the metric as the benchmark configuration names it: throughput (value) and
# the learned renderers' equal-time relMSE (learned_equal_time)
METRIC = "Msamples/s on 1 GB300; equal-time relMSE vs FP64 oracle, guided vs plain"
WORKLOAD = "cornell_box_600x600_1024spp_depth50"
# wavefront traffic floor per ray segment: ray 32 B written + read, hit 16 B
# written + read, path state 48 B read + written (the dominant kernel pair)
BYTES_PER_SEGMENT = 192
TRAVERSE_BYTES_PER_SEGMENT = 64 + 16  # traverse reads the path record, writes the hit
# k_persistent DRAM read+write bytes and warp instructions per ray segment,
# from the ncu capture (--set full) of this script's 16 spp case in the tuned
# launch (--spp 16 --engine 2 --block 64 --wave 5): 9.367 MB and 3.412 G warp
# instructions over 30.42 M segments.  NCU_SOURCE is the fingerprint of the
# kernel sources that capture ran (kernel_source_fingerprint()); the bench
# line says whether the sources it runs still match it.
NCU_DRAM_BYTES_PER_SEGMENT = (8.197632e6 + 1.169152e6) / 30416883
NCU_WARP_INST_PER_SEGMENT = 3412038270 / 30416883
NCU_SOURCE = "2dddc7c1aa56f67c"


def kernel_source_fingerprint() -> str:
    """First 16 hex digits of the SHA-256 of csrc/device.cuh + csrc/kernels.cu."""
    import hashlib

    h = hashlib.sha256()
    for f in ("device.cuh", "kernels.cu"):
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tiny-path-tracer_gb300", "csrc", f),
                  "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]
# instruction issue peak: 152 SMs x 4 schedulers x 1 warp instruction per
# cycle at the maximum SM clock (MEASURED_PEAKS.json sm_max_mhz)
SMS, SCHEDULERS_PER_SM = 152, 4
FP32_LANES_PER_SM = 128  # FP32 peak = 152 SMs x 128 lanes x 2 flops (FMA) x clock
# Useful FLOPs per counted operation (the survey's work conventions): slab
# test 12 (3 axes x 2 FMA), sphere 20, rect 10, instance transform 40,
# lambertian / metal scatter 30, dielectric 60, light-pdf evaluation 40
FLOPS_PER = {"aabb_tests": 12, "sphere_tests": 20, "rect_tests": 10, "instance_xforms": 40, "lambertian": 30,
             "metal": 30, "dielectric": 60, "light_pdf_evals": 40}


def _peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "sm_mhz": float(d.get("sm_max_mhz", 2070.0)), "source": "measured"}
    return {"hbm_gbs": 6800.0, "sm_mhz": 2070.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def host_cores() -> int:
    """Cores this process may run on (affinity, then cgroup quota)."""
    n = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else (os.cpu_count() or 1)
    try:
        with open("/sys/fs/cgroup/cpu.max") as f:
            quota, period = f.read().split()[:2]
        if quota != "max":
            n = max(1, min(n, int(int(quota) / int(period))))
    except (OSError, ValueError):
        pass
    return n


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.strip().startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith(("model name", "cpu model")):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def host_info() -> dict:
    return {"cpu_model": cpu_model(), "hardware_concurrency": os.cpu_count() or 1, "cores_used": host_cores()}


def useful_flops_per_segment(text: str, width: int, height: int, rows: tuple[int, int], spp: int,
                             semantics: int = 0, background: int = 0) -> dict:
    """The CPU oracle's operation counts over a band of the frame (the
    reference's traversal: both children of every bvh_node whose box the
    ray enters), weighted by FLOPS_PER, per ray segment."""
    import pyoracle

    _, cnt = pyoracle.Scene(text).render(width, height, spp, DEPTH, semantics=semantics, background=background,
                                          seed=3, nthreads=host_cores(), rows=rows)
    segs = max(1, cnt["segments"])
    flops = sum(FLOPS_PER[k] * cnt[k] for k in FLOPS_PER)
    return {"flops_per_segment": flops / segs, "counts_per_segment": {k: cnt[k] / segs for k in FLOPS_PER},
            "oracle_segments_per_sample": segs / ((rows[1] - rows[0]) * width * spp),
            "sample": f"rows {rows[0]}..{rows[1]} of {width}x{height} at {spp} spp"}


def cpu_leg(text: str, rows: tuple[int, int], spp: int, prefer_ref: bool = True, repeats: int = 2, width: int = W,
            height: int = H, background: int = 0) -> dict:
    """The reference algorithm on host cores over image rows [rows); the best
    of `repeats` runs (the host is shared, single runs vary)."""
    best = None
    for _ in range(repeats):
        r = _cpu_leg_once(text, rows, spp, prefer_ref, width, height, background)
        if best is None or r["value"] > best["value"]:
            best = r
    return best


def _cpu_leg_once(text: str, rows: tuple[int, int], spp: int, prefer_ref: bool, width: int = W, height: int = H,
                  background: int = 0) -> dict:
    import pyoracle

    n_samples = (rows[1] - rows[0]) * width * spp
    cores = host_cores()
    if prefer_ref and pyoracle.ref_available() and background == 0:
        rs = pyoracle.RefScene(text)
        t0 = time.perf_counter()
        _, secs = rs.render(width, height, spp, DEPTH, lean=1, rows=rows)
        el = time.perf_counter() - t0
        kind, threads = "reference", pyoracle.ref_lib().ref_hardware_concurrency()
        note = "reference sources (oracle/_ref), one std::async task per row as main.cpp:157-159"
    else:
        os_ = pyoracle.Scene(text)
        t0 = time.perf_counter()
        os_.render(width, height, spp, DEPTH, semantics=0, background=background, seed=9, nthreads=cores, rows=rows)
        el = time.perf_counter() - t0
        kind, threads = "port", cores
        note = "CPU oracle port of the reference algorithm, all host cores"
    return {"value": n_samples / el / 1e6, "unit": "Msamples/s", "cores": threads, "kind": kind,
            "sample": f"rows {rows[0]}..{rows[1]} of {width}x{height} at {spp} spp ({n_samples} samples), {note}",
            "seconds": el}


def reference_arm(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from tpt import scenes

    text = scenes.cornell().text()
    vals = []
    leg = None
    for _ in range(args.warmup):
        cpu_leg(text, (280, 320), 8)
    for _ in range(args.steps):
        leg = cpu_leg(text, (0, 600), 32)
        vals.append(leg["value"])
    v = float(np.mean(vals))
    out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Msamples/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "config": {"workload": WORKLOAD},
           "cpu_baseline": {"value": v, "unit": "Msamples/s", "cores": leg["cores"], "kind": leg["kind"],
                            "sample": leg["sample"], **host_info()},
           "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def batch_leg(ctx, stream, steps: int, warmup: int, bvh: str = "reference", block: int = 0, wave: int = 0,
              with_cpu: bool = True) -> dict:
    """64 seeded random-sphere scenes (50..5000 spheres, 256^2..1024^2, 8..64
    spp) rendered in one persistent launch replayed from a CUDA graph; CPU
    baseline: the reference algorithm scene by scene on a band of rows of
    four of the scenes (smallest to largest sphere count)."""
    import torch
    import tpt
    from tpt import scenes

    sds = scenes.batch_scenes(seed=2, count=64)
    texts = [sd.text() for sd in sds]
    t0 = time.perf_counter()
    compiled = [tpt.Scene(t, bvh=bvh) for t in texts]  # host: parse, reference or SAH tree, flatten
    t1 = time.perf_counter()
    slots = [ctx.upload(sc) for sc in compiled]  # device copy (+ the GPU build of an LBVH scene)
    t2 = time.perf_counter()
    jobs = [(slot, sd.meta["width"], sd.meta["height"], sd.meta["spp"]) for slot, sd in zip(slots, sds)]
    outs = [torch.empty((h, w, 3), dtype=torch.float32, device="cuda") for _, w, h, _ in jobs]
    ptrs = [o.data_ptr() for o in outs]
    kw = dict(max_depth=50, background=tpt.BACKGROUND_SKY, seed=1, block=block, variant=wave)
    tuned = None
    if block == 0 and wave == 0:  # block, register variant, walk threshold by the autotuner (untimed)
        tuned = tpt.autotune_batch(ctx, jobs, ptrs, 8, max_depth=50, background=tpt.BACKGROUND_SKY, seed=1)
        kw.update(block=tuned[0], variant=tuned[1], flat_nodes=tuned[2], refill=tuned[3])
    for _ in range(warmup):
        tpt.render_batch(ctx, jobs, outs=ptrs, **kw)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    times, st = [], None
    for k in range(steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st = tpt.render_batch(ctx, jobs, outs=ptrs, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    for sl in slots:
        ctx.release(sl)
    samples = st["samples"]
    ms = float(np.mean(times))
    value = samples / (ms / 1e3) / 1e6
    cpu = None
    if with_cpu:
        order = sorted(range(len(sds)), key=lambda k: sds[k].meta["n_spheres"])
        picks = [order[0], order[len(order) // 3], order[2 * len(order) // 3], order[-1]]
        tot_s, tot_n, kinds = 0.0, 0, set()
        for k in picks:
            sd = sds[k]
            w, h, spp = sd.meta["width"], sd.meta["height"], sd.meta["spp"]
            r = _cpu_leg_once(texts[k], (h // 2 - 4, h // 2 + 4), spp, False, w, h, 1)
            tot_s += r["seconds"]
            tot_n += 8 * w * spp
            kinds.add(r["kind"])
        cpu = {"value": tot_n / tot_s / 1e6, "unit": "Msamples/s", "cores": host_cores(), "kind": "port",
               "sample": "8 rows through the middle of 4 of the 64 scenes (%s spheres) at their spp, scene by "
                         "scene, CPU oracle port of the reference algorithm, all host cores" %
                         "/".join(str(sds[k].meta["n_spheres"]) for k in picks)}
    return {"workload": "batch_64_random_sphere_scenes", "value": value, "unit": "Msamples/s", "ms_per_step": ms,
            "steps": steps, "scenes": len(jobs), "samples_per_step": samples, "bvh": bvh,
            "launch": {"block": kw["block"], "variant": kw["variant"], "flat_nodes": kw.get("flat_nodes", 0),
                       "refill": kw.get("refill", 1), "kernel": ("stepped walk" if kw["variant"] >= 14 else
                                                                 "whole-segment walk"),
                       "autotuned": tuned is not None},
            "segments_per_step": st["segments"], "scene_compile_s": t1 - t0, "scene_upload_s": t2 - t1,
            "gpu_launches": st["kernel_launches"] * steps, "clocks": clk, "cpu_baseline": cpu,
            "vs_cpu": value / cpu["value"] if cpu else None}


def batch_bench(args) -> None:
    """The batch workload alone (--workload batch)."""
    import torch
    import tpt

    torch.cuda.set_device(0)
    ctx = tpt.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    r = batch_leg(ctx, stream, args.steps, args.warmup, args.bvh, args.block, args.wave, not args.no_cpu)
    out = {"metric": "Msamples/s (64-scene random-sphere batch, one persistent launch, 1 GPU)",
           "value": r["value"], "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {k: r[k] for k in ("workload", "scenes", "samples_per_step", "bvh", "launch",
                                         "segments_per_step", "scene_compile_s", "scene_upload_s")},
           "gpu_launches": r["gpu_launches"], "clocks": r["clocks"], "cpu_baseline": r["cpu_baseline"]}
    print(json.dumps(out))
    ctx.close()


def plain_leg(ctx, stream, name: str, text: str, width: int, height: int, spp: int, background: int, steps: int,
              cpu_rows: tuple[int, int], cpu_spp: int, with_cpu: bool = True) -> dict:
    """One plain-tracer workload: autotuned launch, `steps` frames timed with
    CUDA events on the library's stream (L2 flushed between frames), image
    left in HBM; CPU baseline on a band of rows of the same frame."""
    import torch
    import tpt

    slot = ctx.upload(tpt.Scene(text))
    tuned = tpt.autotune(ctx, slot, width, height, 4, max_depth=DEPTH, background=background)
    kw = dict(max_depth=DEPTH, background=background, engine=tuned[0], block=tuned[1], wave=tuned[2],
              flat_nodes=tuned[3])
    img = torch.empty((height, width, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ctx.render(slot, width, height, spp, out=img.data_ptr(), seed=1, **kw)
    times, segs = [], 0
    for k in range(steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st = ctx.render(slot, width, height, spp, out=img.data_ptr(), seed=10 + k, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
        segs += st["segments"]
    ctx.release(slot)
    ms = float(np.mean(times))
    value = width * height * spp / (ms / 1e3) / 1e6
    cpu = None
    if with_cpu:
        cpu = cpu_leg(text, cpu_rows, cpu_spp, prefer_ref=True, width=width, height=height, background=background)
        cpu.pop("seconds", None)
    return {"workload": name, "value": value, "unit": "Msamples/s", "ms_per_step": ms, "steps": steps,
            "width": width, "height": height, "spp": spp, "semantics": "reference",
            "background": ["black", "sky"][background], "segments_per_sample": segs / steps / (width * height * spp),
            "engine": "%s (autotuned: block %d, %s %d)" % (["auto", "wavefront", "persistent"][tuned[0]], tuned[1],
                                                          "variant" if tuned[0] == 2 else "queue", tuned[2]),
            "cpu_baseline": cpu, "vs_cpu": value / cpu["value"] if cpu else None}


def other_configs(ctx, stream, with_cpu: bool) -> dict:
    """The benchmark definition's other throughput workloads."""
    from tpt import scenes

    out = {}
    for key, fn in (("one_weekend_400x400_16spp", lambda: plain_leg(
                        ctx, stream, "one_weekend_400x400_16spp_depth50", scenes.one_weekend().text(), 400, 400, 16,
                        1, 10, (0, 400), 16, with_cpu)),
                    ("batch_64_scenes_reference_bvh", lambda: batch_leg(ctx, stream, 2, 1, "reference",
                                                                        with_cpu=with_cpu)),
                    ("next_week_800x800_256spp", lambda: plain_leg(
                        ctx, stream, "next_week_800x800_256spp_depth50", scenes.next_week().text(), 800, 800, 256, 0,
                        3, (368, 432), 16, with_cpu))):
        try:
            out[key] = fn()
        except Exception as e:  # reported, never fatal to the headline line
            out[key] = {"error": str(e)}
    return out


def max_over_ranks(ms: float, dist, device: str) -> float:
    """The job's time: the slowest rank (all-reduce MAX; identity on one rank)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def frame_msamples(samples: int, t_max_ms: float) -> float:
    """Whole-job throughput of a split frame: the frame's samples (all ranks'
    shares together) over the slowest rank's time."""
    return samples / (t_max_ms / 1e3) / 1e6


def _relmse(x, ref, eps=1e-2) -> float:
    """mean over pixels and channels of (x - ref)^2 / (ref^2 + eps), eps 1e-2"""
    return float(np.mean((x.astype(np.float64) - ref) ** 2 / (ref.astype(np.float64) ** 2 + eps)))


def fit_to_target(pts, e_target, near=3):
    """Points (spp, ms, relMSE) -> (spp, ms, reached) where the relMSE equals
    e_target.  log relMSE is fitted by least squares as a line in log spp
    over the `near` points closest (in log spp) to a first fit's crossing,
    its slope held in [-1.5, -0.2] (a Monte Carlo error falls as 1/spp, a
    biased estimator's more slowly, never faster); one noisy point then
    moves the answer less than a two-point bracket would.  The time is a
    least-squares line in spp over the same points.  reached: some point is
    at or below the target."""
    pts = sorted(pts)

    def fit(sel):
        n = np.array([p[0] for p in sel], float)
        t = np.array([p[1] for p in sel], float)
        x, y = np.log(n), np.log(np.array([p[2] for p in sel], float))
        slope = np.polyfit(x, y, 1)[0] if len(sel) >= 2 and np.ptp(x) > 0 else -1.0
        slope = float(min(max(slope, -1.5), -0.2))
        icpt = float(np.mean(y - slope * x))
        n_star = float(np.exp((np.log(e_target) - icpt) / slope))
        if len(sel) >= 2 and np.ptp(n) > 0:
            b, a = np.polyfit(n, t, 1)
        else:
            b, a = t[0] / n[0], 0.0
        return n_star, float(a + b * n_star)

    n0, _ = fit(pts)
    sel = sorted(pts, key=lambda p: abs(np.log(p[0] / n0)))[:max(2, near)]
    n_star, t_star = fit(sel)
    return n_star, t_star, any(p[2] <= e_target for p in pts)


def learned_equal_time(ctx, which: str) -> dict:
    """Equal-time comparison of a learned renderer against the plain tracer,
    both scored by relMSE against an FP64-accumulated high-spp plain render
    (physical semantics).  Times are wall-clock milliseconds of the whole
    call (training, table refresh / cache inference included), images left
    on the device; both sides run on the engine the autotuner picks for the
    scene, so the plain baseline is the tracer's best configuration.

    guided: Cornell box with the 40x40 light and the second box, 600x600,
            plain at 1024 spp against guided at the spp that takes the same
            time (alpha 0.5, the 50/50 MIS of the configuration); FP64
            reference 16384 spp.  Also reported: the same comparison with
            the guide's share lowered to alpha 0.25 (the rest is the plain
            light/cosine mixture), which measured best on this scene.
    nrc:    the seeded next-week scene, 800x800, plain at 256 spp against the
            cached renderer at its default settings (an uncached 8-spp first
            pass, then paths end into the cache by the path-spread rule,
            c = 0.01, at the third bounce at the latest; 512 Adam steps after
            each of the first 2 of 3 passes) at the spp that takes the same
            time; FP64 reference 4096 spp.
    nrc_cornell: the cached renderer on the guided configuration's Cornell
            box (40x40 light, second box), 600x600, plain at 1024 spp; FP64
            reference 16384 spp.
    The cached renders run on the engine tpt_autotune_nrc picks for the
    scene (timed before, like the plain tracer's autotune).
    Every point (plain, learned at equal spp, at equal time, and the points
    of the time-to-plain-relMSE search) is the mean over five seeds (each
    learned run trains its own network online; per-seed values are reported
    too).  time_to_plain_relmse_ratio = the learned renderer's wall time at
    the spp where its relMSE equals the plain tracer's, over the plain
    tracer's wall time.  The reference's own noise adds ~spp/ref_spp of the
    plain relMSE to both."""
    import torch
    import tpt
    from tpt import scenes

    if which == "guided":
        sd, w, h, spp, ref_spp = scenes.cornell_guiding(), 600, 600, 1024, 16384
        run = lambda n, out, sd_: tpt.render_guided(ctx, slot, w, h, n, seed=sd_, out=out)
    else:
        if which == "nrc_cornell":
            sd, w, h, spp, ref_spp = scenes.cornell_guiding(), 600, 600, 1024, 16384
        else:
            sd, w, h, spp, ref_spp = scenes.next_week(), 800, 800, 256, 4096
        run = lambda n, out, sd_: tpt.render_nrc(ctx, slot, w, h, n, seed=sd_, out=out)
    slot = ctx.upload(tpt.Scene(sd.text()))
    # both sides use the engine the autotuner picks for this scene (physical
    # semantics): the plain baseline is the tracer's best configuration
    tuned = tpt.autotune(ctx, slot, w, h, 4, semantics=tpt.SEMANTICS_PHYSICAL)
    cache_engine = tpt.autotune_nrc(ctx, slot, w, h) if which != "guided" else None
    dev = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, r

    ref, _ = ctx.render(slot, w, h, ref_spp, semantics=tpt.SEMANTICS_PHYSICAL, seed=999, fp64=True)
    passes = 8
    seeds = (5, 6, 7, 8, 9)  # both sides: the mean over five seeds (each learned run trains its own network)
    plain = lambda n, sd_: ctx.render(slot, w, h, n, semantics=tpt.SEMANTICS_PHYSICAL, seed=sd_,
                                      out=dev.data_ptr())
    plain(spp, seeds[0])  # warm-up
    t_p, e_p = [], []
    for sd_ in seeds:
        t, _ = timed(lambda: plain(spp, sd_))
        t_p.append(t)
        e_p.append(_relmse(dev.cpu().numpy(), ref))
    t_plain, e_plain = float(np.mean(t_p)), float(np.mean(e_p))

    def at(run, n):
        """mean wall time and relMSE over the seeds at n spp"""
        ts, es, last = [], [], None
        for sd_ in seeds:
            t, last = timed(lambda: run(n, dev.data_ptr(), sd_))
            ts.append(t)
            es.append(_relmse(dev.cpu().numpy(), ref))
        return float(np.mean(ts)), float(np.mean(es)), es, last

    def time_to_plain(run, pts):
        """Wall time the learned renderer needs to reach the plain tracer's
        relMSE (points (spp, ms, relMSE), five seeds each): fit_to_target
        predicts the spp from the points measured so far, and a new point is
        measured there while no measured point lies within 15 % of the
        prediction (at most three); the answer is the fit over the final
        points."""
        for _ in range(3):
            n_pred, _, _ = fit_to_target(pts, e_plain)
            if min(abs(p[0] - n_pred) for p in pts) <= 0.15 * n_pred:
                break
            n = int(round(n_pred / passes)) * passes
            n = int(min(max(n, passes), 8 * spp))
            if any(p[0] == n for p in pts):
                break
            t, e, _, _ = at(run, n)
            pts.append((n, t, e))
        pts.sort()
        n_star, t_star, reached = fit_to_target(pts, e_plain)
        return {"spp": n_star, "ms": t_star, "ratio": t_star / t_plain, "reached": reached,
                "points": [{"spp": p[0], "ms": p[1], "relmse": p[2]} for p in pts]}

    def compare(run):
        run(spp, dev.data_ptr(), seeds[0])  # warm-up
        t_eq, e_eq, _, r = at(run, spp)
        spp_et = max(passes, int(round(spp * t_plain / t_eq / passes)) * passes)
        t_et, e_et, e_et_seeds, _ = at(run, spp_et)
        ttp = time_to_plain(run, [(spp, t_eq, e_eq), (spp_et, t_et, e_et)])
        return ({"spp": spp, "ms": t_eq, "relmse": e_eq, "stats": r[2], "seeds": list(seeds)},
                {"spp": spp_et, "ms": t_et, "relmse": e_et, "seeds": list(seeds)},
                {"equal_spp_relmse_ratio": e_eq / e_plain, "equal_time_relmse_ratio": e_et / e_plain,
                 "equal_time_relmse_ratio_per_seed": [e / e_plain for e in e_et_seeds],
                 "time_ratio_at_equal_spp": t_eq / t_plain,
                 "time_to_plain_relmse": ttp, "time_to_plain_relmse_ratio": ttp["ratio"]})

    eq, et, ratios = compare(run)
    extra = {}
    if which == "guided":
        _, et2, ratios2 = compare(lambda n, out, sd_: tpt.render_guided(ctx, slot, w, h, n, seed=sd_, out=out,
                                                                        alpha=0.25))
        extra = {"guided_alpha_0.25": dict(alpha=0.25, equal_time_spp=et2["spp"], equal_time_ms=et2["ms"],
                                           equal_time_relmse=et2["relmse"], **ratios2)}
    plain_rec = {"spp": spp, "ms": t_plain, "relmse": e_plain, "seeds": list(seeds),
                 "ms_per_seed": t_p, "relmse_per_seed": e_p}
    ctx.release(slot)
    name = "next_week_final_seeded" if which == "nrc" else "cornell_40x40_light_two_boxes"
    engines = ["auto", "wavefront", "persistent"]
    rec = {"scene": name, "width": w, "height": h, "ref_spp_fp64": ref_spp, "engine": engines[tuned[0]]}
    if cache_engine is not None:
        rec["cache_engine"] = engines[cache_engine]
    return {**rec, "plain": plain_rec, which: eq, which + "_equal_time": et, **ratios, **extra}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--engine", type=int, default=0)
    ap.add_argument("--wave", type=int, default=0)
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--bvh", default="reference", choices=["reference", "sah", "lbvh"],
                    help="batch workload: the reference's BVH topology, the SAH rebuild (host) or the "
                         "linear BVH (built on the GPU at upload)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the equal-time guided / cached comparisons of the default line")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other throughput workloads (one weekend, batch, next week) of the default line")
    ap.add_argument("--spp", type=int, default=SPP, help="smaller cases for profiling only")
    ap.add_argument("--workload", default="cornell", choices=["cornell", "batch"],
                    help="cornell: the headline workload; batch: 64 seeded random-sphere scenes in one launch")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
        return
    if args.workload == "batch":
        batch_bench(args)
        return

    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import tpt
    from tpt import frame_split, scenes

    text = scenes.cornell().text()
    ctx = tpt.Context(local)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)  # library work and the timing events share this stream
    scene = tpt.Scene(text)
    slot = ctx.upload(scene)
    arena_bytes = scene.info()["arena_bytes"]
    tuned = None
    if args.engine == 0:  # engine choice, block, register variant by the autotuner (untimed)
        tuned = tpt.autotune(ctx, slot, W, H, 16, max_depth=DEPTH)
    img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    kw = dict(max_depth=DEPTH, engine=args.engine, wave=args.wave, block=args.block, seed=1)
    if tuned:  # the e2e frames (fresh uploads) render with the same configuration
        kw.update(engine=tuned[0], block=tuned[1], wave=tuned[2], flat_nodes=tuned[3])

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_leg(text, (0, 600), 32)
        cpu.pop("seconds", None)
        cpu.update(host_info())
    # one frame per step; with N ranks each renders its share of the samples
    # and the float4 accumulators are summed across ranks (NCCL) and resolved
    accum = torch.empty(W * H * 4, dtype=torch.float32, device="cuda") if world > 1 else None
    rkw = {x: y for x, y in kw.items() if x != "seed"}

    def frame(seed, profile=False):
        if world == 1:
            return ctx.render(slot, W, H, args.spp, out=img.data_ptr(), profile=profile, seed=seed, **rkw)[1]
        return frame_split.render_split_frame(ctx, slot, W, H, args.spp, accum, rank, world, dist,
                                              out=img.data_ptr(), seed=seed, profile=profile, **rkw)[1]

    for w in range(args.warmup):
        frame(1)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    times, launches, tr_ms, tr_n, segs = [], 0, 0.0, 0, 0
    for k in range(args.steps):
        flush.fill_(k & 0xff)  # evict L2 between timed steps (outside the events)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st = frame(100 + k, profile=True)
        e1.record(stream)
        barrier()
        times.append(e0.elapsed_time(e1))
        launches += st["kernel_launches"]
        tr_ms += st["traverse_ms"]
        tr_n += st["traverse_launches"]
        segs += st["segments"]
    clk = clocks.stop()
    ms = float(np.sum(times))
    t_max = max_over_ranks(ms, dist, "cuda")
    value = frame_msamples(W * H * args.spp * args.steps, t_max)

    # e2e through the C ABI with host buffers: compile + upload, render (this
    # rank's share, the sum across ranks), resolve, image to the host
    e2e_times = []
    for k in range(max(1, min(args.steps, 3))):
        barrier()
        t0 = time.perf_counter()
        sc = tpt.Scene(text)
        s2 = ctx.upload(sc)
        if world == 1:
            host_img, _ = ctx.render(s2, W, H, args.spp, seed=200 + k, **rkw)
        else:
            host_img, _ = frame_split.render_split_frame(ctx, s2, W, H, args.spp, accum, rank, world, dist,
                                                         seed=200 + k, **rkw)
        ctx.release(s2)
        e2e_times.append(time.perf_counter() - t0)
    e2e_ms = max_over_ranks(1e3 * float(np.mean(e2e_times)), dist, "cuda")
    e2e_value = frame_msamples(W * H * args.spp, e2e_ms)

    learned = None
    if rank == 0 and not args.no_learned and args.spp == SPP:
        learned = {}
        for which in ("guided", "nrc", "nrc_cornell"):
            try:
                learned[which] = learned_equal_time(ctx, which)
            except Exception as e:  # reported, never fatal to the throughput line
                learned[which] = {"error": str(e)}
    configs = None
    if rank == 0 and not args.no_configs and args.spp == SPP:
        configs = other_configs(ctx, stream, not args.no_cpu)

    peaks = _peaks()
    roof = None
    if tr_n > 0 and tr_ms > 0:
        seg_per_launch = segs / tr_n
        wavefront = kw["engine"] == 1
        per_seg = TRAVERSE_BYTES_PER_SEGMENT if wavefront else BYTES_PER_SEGMENT
        algo_bytes = seg_per_launch * per_seg
        launch_s = tr_ms / tr_n / 1e3
        achieved = algo_bytes / launch_s / 1e9
        # DRAM bytes per segment from the ncu capture of the same kernel on the
        # 16 spp case (NCU_DRAM_BYTES_PER_SEGMENT), scaled to this launch's segments
        traffic = None if wavefront else seg_per_launch * NCU_DRAM_BYTES_PER_SEGMENT
        roof = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "kernel": "k_wf_traverse" if wavefront else "k_persistent",
                "peak_source": peaks["source"], "launch_ms": tr_ms / tr_n,
                "segments_per_launch": seg_per_launch, "algorithmic_bytes_per_segment": per_seg,
                "kernel_share": tr_ms / ms,
                "note": ("algorithmic bytes = the wavefront traffic floor per ray segment (ray, hit and path "
                         "state written and read); the kernel keeps that state in registers and the scene in "
                         "L1/L2, so it is issue-bound, not HBM-bound: see issue_roofline and flops")}
        if rank == 0 and args.spp == SPP:
            # useful work: the reference algorithm's arithmetic per segment (oracle counts
            # over a band of the frame) at the kernel's measured segment rate, against the
            # FP32 peak (derived: 152 SMs x 128 lanes x 2 flops per FMA x maximum SM clock)
            u = useful_flops_per_segment(text, W, H, (280, 320), 4)
            peak_fp32 = SMS * FP32_LANES_PER_SM * 2 * peaks["sm_mhz"] / 1e6  # TFLOP/s
            ach_fp32 = u["flops_per_segment"] * seg_per_launch / launch_s / 1e12
            roof["flops"] = {"bound": "fp32", "achieved": ach_fp32, "peak": peak_fp32, "unit": "TFLOP/s",
                             "frac": ach_fp32 / peak_fp32, "peak_source": "derived (152 x 128 x 2 x sm_max_mhz)",
                             "useful_flops_per_segment": u["flops_per_segment"],
                             "counts_per_segment": u["counts_per_segment"],
                             "oracle_sample": u["sample"],
                             "note": ("oracle-counted work of the reference's traversal (every child of every "
                                      "bvh_node whose box the ray enters) and shading, weighted 12 per slab "
                                      "test, 20 per sphere, 10 per rect, 40 per instance transform, 30 per "
                                      "lambertian or metal scatter, 60 per dielectric, 40 per light pdf")}
        if not wavefront:
            peak_issue = SMS * SCHEDULERS_PER_SM * peaks["sm_mhz"] / 1e3  # G warp instructions / s
            ach_issue = seg_per_launch * NCU_WARP_INST_PER_SEGMENT / launch_s / 1e9
            roof["issue_roofline"] = {
                "bound": "issue", "achieved": ach_issue, "peak": peak_issue, "unit": "G warp-inst/s",
                "frac": ach_issue / peak_issue, "warp_inst_per_segment": NCU_WARP_INST_PER_SEGMENT,
                "counts_source": NCU_SOURCE, "counts_match_kernel_source": kernel_source_fingerprint() == NCU_SOURCE,
                "note": ("instructions per segment from the ncu capture of the same kernel (16 spp case, "
                         "NCU_WARP_INST_PER_SEGMENT) x segments per second measured here; peak = 152 SMs x 4 "
                         "schedulers x 1 instruction per cycle at the maximum SM clock; "
                         "counts_match_kernel_source: whether the kernel sources running now are the ones "
                         "the capture ran")}
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
               "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f32",
               "data": "synthetic",
               "config": {"workload": WORKLOAD if args.spp == SPP else f"{WORKLOAD} (profiling case: {args.spp} spp)",
                          "width": W, "height": H, "spp": args.spp, "max_depth": DEPTH,
                          "semantics": "reference",
                          "engine": (["auto", "wavefront", "persistent"][tuned[0]] + " (autotuned: block %d, %s %d)" % (
                              tuned[1], "variant" if tuned[0] == 2 else "queue", tuned[2]) if tuned else
                              ["auto", "wavefront", "persistent"][args.engine]),
                          "split": ("one frame, samples split across %d ranks, float4 accumulators "
                                    "summed (NCCL all-reduce)" % world) if world > 1 else "one GPU",
                          "l2": "flushed between timed steps (256 MB write)",
                          "segments_per_step": segs / args.steps},
               "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": int(arena_bytes),
                       "d2h_bytes_per_step": int(W * H * 3 * 4)},
               "gpu_launches": int(launches), "clocks": clk, "roofline": roof, "cpu_baseline": cpu,
               "learned_equal_time": learned, "other_configs": configs}
        print(json.dumps(out))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
