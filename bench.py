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
        high-spp render of the learned renderers (path guiding on the small-
        light Cornell box, the radiance cache on the next-week scene) next to
        the plain tracer at equal spp and at equal wall time (skip with
        --no-learned).
Multi-GPU: N independent replicas (one frame each per step), scaling "weak".
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
# launch (--spp 16 --engine 2 --block 64 --wave 5): 9.174 MB and 3.412 G warp
# instructions over 30.42 M segments
NCU_DRAM_BYTES_PER_SEGMENT = (8.19712e6 + 0.976896e6) / 30416883
NCU_WARP_INST_PER_SEGMENT = 3411932611 / 30416883
# instruction issue peak: 152 SMs x 4 schedulers x 1 warp instruction per
# cycle at the maximum SM clock (MEASURED_PEAKS.json sm_max_mhz)
SMS, SCHEDULERS_PER_SM = 152, 4


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


def cpu_leg(text: str, rows: tuple[int, int], spp: int, prefer_ref: bool = True, repeats: int = 2) -> dict:
    """The reference algorithm on host cores over image rows [rows); the best
    of `repeats` runs (the host is shared, single runs vary)."""
    best = None
    for _ in range(repeats):
        r = _cpu_leg_once(text, rows, spp, prefer_ref)
        if best is None or r["value"] > best["value"]:
            best = r
    return best


def _cpu_leg_once(text: str, rows: tuple[int, int], spp: int, prefer_ref: bool) -> dict:
    import pyoracle

    n_samples = (rows[1] - rows[0]) * W * spp
    cores = host_cores()
    if prefer_ref and pyoracle.ref_available():
        rs = pyoracle.RefScene(text)
        t0 = time.perf_counter()
        _, secs = rs.render(W, H, spp, DEPTH, lean=1, rows=rows)
        el = time.perf_counter() - t0
        kind, threads = "reference", pyoracle.ref_lib().ref_hardware_concurrency()
        note = "reference sources (oracle/_ref), one std::async task per row as main.cpp:157-159"
    else:
        os_ = pyoracle.Scene(text)
        t0 = time.perf_counter()
        os_.render(W, H, spp, DEPTH, semantics=0, background=0, seed=9, nthreads=cores, rows=rows)
        el = time.perf_counter() - t0
        kind, threads = "port", cores
        note = "CPU oracle port of the reference algorithm, all host cores"
    return {"value": n_samples / el / 1e6, "unit": "Msamples/s", "cores": threads, "kind": kind,
            "sample": f"rows {rows[0]}..{rows[1]} of 600x600 at {spp} spp ({n_samples} samples), {note}",
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
                            "sample": leg["sample"]},
           "e2e": {"value": v, "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def batch_bench(args) -> None:
    """64 seeded random-sphere scenes (50..5000 spheres, 256^2..1024^2, 8..64
    spp) rendered in one persistent launch replayed from a CUDA graph."""
    import torch
    import tpt
    from tpt import scenes

    torch.cuda.set_device(0)
    ctx = tpt.Context(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    sds = scenes.batch_scenes(seed=2, count=64)
    texts = [sd.text() for sd in sds]
    t0 = time.perf_counter()
    compiled = [tpt.Scene(t, bvh=args.bvh) for t in texts]  # host: parse, reference or SAH tree, flatten
    t1 = time.perf_counter()
    slots = [ctx.upload(sc) for sc in compiled]  # device copy (+ the GPU build of an LBVH scene)
    t2 = time.perf_counter()
    jobs = [(slot, sd.meta["width"], sd.meta["height"], sd.meta["spp"]) for slot, sd in zip(slots, sds)]
    outs = [torch.empty((h, w, 3), dtype=torch.float32, device="cuda") for _, w, h, _ in jobs]
    ptrs = [o.data_ptr() for o in outs]
    kw = dict(max_depth=50, background=tpt.BACKGROUND_SKY, seed=1, block=args.block, variant=args.wave)
    tuned = None
    if args.block == 0 and args.wave == 0:  # block, register variant, walk threshold by the autotuner (untimed)
        tuned = tpt.autotune_batch(ctx, jobs, ptrs, 8, max_depth=50, background=tpt.BACKGROUND_SKY, seed=1)
        kw.update(block=tuned[0], variant=tuned[1], flat_nodes=tuned[2])
    for _ in range(args.warmup):
        tpt.render_batch(ctx, jobs, outs=ptrs, **kw)
    torch.cuda.synchronize()
    clocks = ClockSampler(0)
    clocks.start()
    times, st = [], None
    for k in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st = tpt.render_batch(ctx, jobs, outs=ptrs, **kw)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    clk = clocks.stop()
    samples = st["samples"]
    ms = float(np.mean(times))
    out = {"metric": "Msamples/s (64-scene random-sphere batch, one persistent launch, 1 GPU)",
           "value": samples / (ms / 1e3) / 1e6, "unit": "Msamples/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": "batch_64_random_sphere_scenes", "scenes": len(jobs), "samples_per_step": samples,
                      "bvh": args.bvh,
                      "launch": {"block": kw["block"], "variant": kw["variant"], "flat_nodes": kw.get("flat_nodes", 0),
                                 "autotuned": tuned is not None},
                      "spheres": [sd.meta["n_spheres"] for sd in sds][:8] + ["..."],
                      "segments_per_step": st["segments"], "scene_compile_s": t1 - t0, "scene_upload_s": t2 - t1},
           "gpu_launches": st["kernel_launches"] * args.steps, "clocks": clk}
    print(json.dumps(out))
    ctx.close()


def replica_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s replica: independent sample streams per GPU."""
    return base + 1_000_003 * rank


def max_over_ranks(ms: float, dist, device: str) -> float:
    """The job's time: the slowest rank (all-reduce MAX; identity on one rank)."""
    if dist is None:
        return ms
    import torch

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_msamples(samples_per_rank: int, world: int, t_max_ms: float) -> float:
    """Whole-job throughput: every rank's samples over the slowest rank's time."""
    return samples_per_rank * world / (t_max_ms / 1e3) / 1e6


def _relmse(x, ref, eps=1e-2) -> float:
    """mean over pixels and channels of (x - ref)^2 / (ref^2 + eps), eps 1e-2"""
    return float(np.mean((x.astype(np.float64) - ref) ** 2 / (ref.astype(np.float64) ** 2 + eps)))


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
            cached renderer (paths terminated into the cache after 2 bounces)
            at the spp that takes the same time; FP64 reference 4096 spp.
    The equal-time side is the mean over three seeds (each run trains its own
    network online; the per-seed ratios are reported too).  The reference's
    own noise adds ~spp/ref_spp of the plain relMSE to both."""
    import torch
    import tpt
    from tpt import scenes

    if which == "guided":
        sd, w, h, spp, ref_spp = scenes.cornell_guiding(), 600, 600, 1024, 16384
        run = lambda n, out, sd_: tpt.render_guided(ctx, slot, w, h, n, seed=sd_, out=out)
    else:
        sd, w, h, spp, ref_spp = scenes.next_week(), 800, 800, 256, 4096
        run = lambda n, out, sd_: tpt.render_nrc(ctx, slot, w, h, n, seed=sd_, out=out)
    slot = ctx.upload(tpt.Scene(sd.text()))
    # both sides use the engine the autotuner picks for this scene (physical
    # semantics): the plain baseline is the tracer's best configuration
    tuned = tpt.autotune(ctx, slot, w, h, 4, semantics=tpt.SEMANTICS_PHYSICAL)
    dev = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, r

    ref, _ = ctx.render(slot, w, h, ref_spp, semantics=tpt.SEMANTICS_PHYSICAL, seed=999, fp64=True)
    plain = lambda n: ctx.render(slot, w, h, n, semantics=tpt.SEMANTICS_PHYSICAL, seed=5, out=dev.data_ptr())
    plain(spp)  # warm-up
    t_plain, _ = timed(lambda: plain(spp))
    e_plain = _relmse(dev.cpu().numpy(), ref)
    passes = 8
    seeds = (5, 6, 7)  # equal-time runs: the mean over three seeds (each run trains its own network)

    def compare(run):
        run(spp, dev.data_ptr(), seeds[0])  # warm-up
        t_eq, r = timed(lambda: run(spp, dev.data_ptr(), seeds[0]))
        e_eq = _relmse(dev.cpu().numpy(), ref)
        spp_et = max(passes, int(round(spp * t_plain / t_eq / passes)) * passes)
        t_et, e_et = [], []
        for sd_ in seeds:
            t, _ = timed(lambda: run(spp_et, dev.data_ptr(), sd_))
            t_et.append(t)
            e_et.append(_relmse(dev.cpu().numpy(), ref))
        return ({"spp": spp, "ms": t_eq, "relmse": e_eq, "stats": r[2]},
                {"spp": spp_et, "ms": float(np.mean(t_et)), "relmse": float(np.mean(e_et)), "seeds": list(seeds)},
                {"equal_spp_relmse_ratio": e_eq / e_plain, "equal_time_relmse_ratio": float(np.mean(e_et)) / e_plain,
                 "equal_time_relmse_ratio_per_seed": [e / e_plain for e in e_et],
                 "time_ratio_at_equal_spp": t_eq / t_plain})

    eq, et, ratios = compare(run)
    extra = {}
    if which == "guided":
        _, et2, ratios2 = compare(lambda n, out, sd_: tpt.render_guided(ctx, slot, w, h, n, seed=sd_, out=out,
                                                                        alpha=0.25))
        extra = {"guided_alpha_0.25": dict(alpha=0.25, equal_time_spp=et2["spp"], equal_time_ms=et2["ms"],
                                           equal_time_relmse=et2["relmse"], **ratios2)}
    ctx.release(slot)
    name = "cornell_40x40_light_two_boxes" if which == "guided" else "next_week_final_seeded"
    return {"scene": name, "width": w, "height": h, "ref_spp_fp64": ref_spp,
            "engine": ["auto", "wavefront", "persistent"][tuned[0]],
            "plain": {"spp": spp, "ms": t_plain, "relmse": e_plain},
            which: eq, which + "_equal_time": et, **ratios, **extra}


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
    from tpt import scenes

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
    for w in range(args.warmup):
        ctx.render(slot, W, H, args.spp, out=img.data_ptr(), **kw)
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    times, launches, tr_ms, tr_n, segs = [], 0, 0.0, 0, 0
    for k in range(args.steps):
        flush.fill_(k & 0xff)  # evict L2 between timed steps (outside the events)
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _, st = ctx.render(slot, W, H, args.spp, out=img.data_ptr(), profile=True,
                           seed=replica_seed(100 + k, rank), **{x: y for x, y in kw.items() if x != "seed"})
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
    value = job_msamples(W * H * args.spp * args.steps, world, t_max)

    # e2e through the C ABI with host buffers
    host_img = np.zeros((H, W, 3), np.float32)
    e2e_times = []
    for k in range(max(1, min(args.steps, 3))):
        barrier()
        t0 = time.perf_counter()
        sc = tpt.Scene(text)
        s2 = ctx.upload(sc)
        host_img, _ = ctx.render(s2, W, H, args.spp, seed=200 + k, **{x: y for x, y in kw.items() if x != "seed"})
        ctx.release(s2)
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = W * H * args.spp / float(np.mean(e2e_times)) / 1e6

    learned = None
    if rank == 0 and not args.no_learned and args.spp == SPP:
        learned = {}
        for which in ("guided", "nrc"):
            try:
                learned[which] = learned_equal_time(ctx, which)
            except Exception as e:  # reported, never fatal to the throughput line
                learned[which] = {"error": str(e)}

    peaks = _peaks()
    roof = None
    if tr_n > 0 and tr_ms > 0:
        seg_per_launch = segs / tr_n
        wavefront = kw["engine"] == 1
        per_seg = TRAVERSE_BYTES_PER_SEGMENT if wavefront else BYTES_PER_SEGMENT
        algo_bytes = seg_per_launch * per_seg
        achieved = algo_bytes / (tr_ms / tr_n / 1e3) / 1e9
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
                         "L1/L2, so it is issue-bound, not HBM-bound: see issue_roofline")}
        if not wavefront:
            peak_issue = SMS * SCHEDULERS_PER_SM * peaks["sm_mhz"] / 1e3  # G warp instructions / s
            ach_issue = seg_per_launch * NCU_WARP_INST_PER_SEGMENT / (tr_ms / tr_n / 1e3) / 1e9
            roof["issue_roofline"] = {
                "bound": "issue", "achieved": ach_issue, "peak": peak_issue, "unit": "G warp-inst/s",
                "frac": ach_issue / peak_issue, "warp_inst_per_segment": NCU_WARP_INST_PER_SEGMENT,
                "note": ("the binding roof: instructions per segment from the ncu capture of the same kernel "
                         "(16 spp case) x segments per second measured here; peak = 152 SMs x 4 schedulers x "
                         "1 instruction per cycle at the maximum SM clock")}
    if rank == 0:
        out = {"metric": METRIC, "value": value, "unit": "Msamples/s", "n_gpus": world, "steps": args.steps,
               "warmup": args.warmup, "ms_per_step": t_max / args.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
               "config": {"workload": WORKLOAD if args.spp == SPP else f"{WORKLOAD} (profiling case: {args.spp} spp)",
                          "width": W, "height": H, "spp": args.spp, "max_depth": DEPTH,
                          "semantics": "reference",
                          "engine": (["auto", "wavefront", "persistent"][tuned[0]] + " (autotuned: block %d, %s %d)" % (
                              tuned[1], "variant" if tuned[0] == 2 else "queue", tuned[2]) if tuned else
                              ["auto", "wavefront", "persistent"][args.engine]),
                          "l2": "flushed between timed steps (256 MB write)",
                          "segments_per_step": segs / args.steps},
               "e2e": {"value": e2e_value, "unit": "Msamples/s", "h2d_bytes_per_step": int(arena_bytes),
                       "d2h_bytes_per_step": int(W * H * 3 * 4)},
               "gpu_launches": int(launches), "clocks": clk, "roofline": roof, "cpu_baseline": cpu,
               "learned_equal_time": learned}
        print(json.dumps(out))
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
