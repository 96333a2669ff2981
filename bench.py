#!/usr/bin/env python
"""Benchmark: Mpaths/s of the wavefront path tracer on the large-mesh Disney workload
(1920x1080, 64 spp, depth 16; 1024^2-vertex fBm terrain + 200 instanced level-4
icospheres, Disney materials, gradient sky + 8 quad lights; synthetic, seeded).

One step = one full frame (132.7 M camera paths). Prints one JSON line (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference renderer (the reference
itself cannot be built anywhere: its eDSL submodule and the OptiX SDK are absent) on the
host cores, on a bounded sample of the same frame.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpaths/s @1080p"
WORKLOAD = "terrain-1080p-64spp-depth16"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp", type=int, default=64)
    ap.add_argument("--grid", type=int, default=1024)
    ap.add_argument("--instances", type=int, default=200)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    # path-queue length (the renderer's state_count): 32 M states, 11.5 GB of queues, so
    # each bounce launch keeps every SM busy for milliseconds and launch tails are few
    ap.add_argument("--state-count", type=int, default=32 * 1024 * 1024)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-nrc", action="store_true", help="skip the radiance-cache equal-time study")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched uneven-scenes measurement")
    ap.add_argument("--nrc-frames", type=int, default=1000, help="frames of the radiance-cache study")
    ap.add_argument("--ref-spp", type=int, default=4096, help="spp of the converged reference image")
    ap.add_argument("--probe", choices=["nrc", "nrc-frames", "medium", "generate", "trace", "trace-two-level",
                                        "build-device"],
                    help="run one small profiling case and exit: nrc (cache inference on 2^20 queries and "
                         "training steps of 16,384 samples), medium (volume workload at 256x256, 4 spp), "
                         "generate / trace (terrain at 1920x1080, 1 spp, 2 M-state queue), trace-two-level "
                         "(the same through the two-level acceleration structure), build-device (the "
                         "terrain's BVH built on the device), nrc-frames (25 radiance-cache frames of the "
                         "Cornell box at 512x512)")
    ap.add_argument("--trace-probe", action="store_true",
                    help="trace the workload's camera rays, then one diffuse bounce ray per camera hit, "
                         "through btrc_trace_closest (two launches, for DRAM-traffic captures) and exit")
    return ap.parse_args()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(world, v: float) -> float:
    if world <= 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def bench_config(args, triangles: int) -> dict:
    """The workload description both arms print (same keys and values)."""
    return {"workload": WORKLOAD, "width": args.width, "height": args.height, "spp": args.spp, "max_depth": 16,
            "triangles": int(triangles), "state_count": args.state_count, "sampler": "independent",
            "filter": "gaussian r1.5",
            "l2": "inputs larger than L2: BVH + shading records of the 3.1 M-triangle scene > 129 MB",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


def scene_path(args):
    from btrc_gb300 import scenes
    return scenes.terrain(seed=1001, width=args.width, height=args.height, spp=args.spp, grid=args.grid,
                          instances=args.instances, state_count=args.state_count)


class ClockSampler:
    """nvidia-smi sampled every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

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
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, flag in zip(names, parts[4:8]):
                if flag.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(path: str, target_s: float, threads: int = 0) -> dict:
    """Oracle (CPU restatement of the reference renderer) on a bounded sample of the frame:
    the whole 1080p film at as many samples per pixel as fit in about target_s seconds."""
    from oracle import scene as OS
    S = OS.Scene(path)
    S.prepare()
    pixels = S.width * S.height
    threads = threads or os.cpu_count() or 1
    t0 = time.perf_counter()
    S.render(spp=1, threads=threads)
    dt = time.perf_counter() - t0
    spp = int(max(1, min(64, target_s / max(dt, 1e-3))))
    t0 = time.perf_counter()
    S.render(spp=spp, sample_begin=1, threads=threads)
    dt = time.perf_counter() - t0
    return {"value": spp * pixels / dt / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": "port",
            "sample": f"{spp} spp over the full 1920x1080 film ({spp * pixels} paths, {dt:.1f} s)",
            "label": "CPU restatement of Btrc's wavefront integrator (the reference itself cannot be built)"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    path = scene_path(args)
    from oracle import scene as OS
    S = OS.Scene(path)
    S.prepare()
    threads = os.cpu_count() or 1
    pixels = S.width * S.height
    # each step: the whole film at k spp, k sized to a bounded share of a few minutes
    t0 = time.perf_counter()
    S.render(spp=1, threads=threads)
    dt = time.perf_counter() - t0
    per_step = max(4.0, min(30.0, 60.0 / max(1, args.steps + args.warmup)))
    k_spp = int(max(1, min(args.spp, per_step / max(dt, 1e-3))))
    for w in range(args.warmup):
        S.render(spp=k_spp, sample_begin=(w * k_spp) % args.spp, threads=threads)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        S.render(spp=k_spp, sample_begin=((args.warmup + k) * k_spp) % args.spp, threads=threads)
        times.append(time.perf_counter() - t0)
    total = sum(times)
    n_step = k_spp * pixels
    value = n_step * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, len(S.tris)),
        "cpu_baseline": {"value": value, "unit": "Mpaths/s", "cores": threads, "kind": "port",
                         "sample": f"each step: {k_spp} spp over the full 1920x1080 film ({n_step} paths)"},
        "e2e": {"value": value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference renderer; Btrc itself cannot be built (eDSL submodule and "
                "OptiX SDK absent)",
    }
    print(json.dumps(line), flush=True)


def l2_figures():
    """L2 traffic of k_trace from the committed ncu capture of two launches of the 1080p
    terrain (lts__t_bytes and ncu's L2 throughput as a fraction of its peak)."""
    path = ROOT / "profiles" / "trace_traffic.json"
    try:
        tj = json.loads(path.read_text())
        return {k: tj[k] for k in ("lts_bytes_camera_launch", "lts_bytes_first_bounce_launch",
                                   "lts_frac_of_peak_camera", "lts_frac_of_peak_first_bounce",
                                   "l2_gbs_camera", "l2_gbs_first_bounce", "issue_frac_camera",
                                   "issue_frac_first_bounce") if k in tj} | {
            "source": "profiles/k_trace_l2_terrain-1080p.md (ncu, one pass, two launches); issue_frac = warp "
                      "instructions / (152 SMs x 4 per cycle x 2070 MHz x duration)"}
    except (OSError, ValueError):
        return None


def _time_to(curve, target):
    """First time at which a (time_ms, relMSE) curve reaches target, interpolated in
    log-log between the bracketing points; None if it never does."""
    prev = None
    for t, e in curve:
        if e <= target:
            if prev is None:
                return t
            (t0, e0), (t1, e1) = prev, (t, e)
            if e0 <= 0 or e1 <= 0 or e0 == e1:
                return t1
            a = (np.log(target) - np.log(e0)) / (np.log(e1) - np.log(e0))
            return float(np.exp(np.log(t0) + a * (np.log(t1) - np.log(t0))))
        prev = (t, e)
    return None


def nrc_study(B, ctx, sc, info, args, spread: float = 0.0):
    """Equal-time comparison of the radiance cache against the plain tracer on a built
    scene: relMSE against a converged plain render (args.ref_spp spp) as a
    function of wall time, for plain renders of 1..128 spp and for the cache (one path per
    pixel per frame, paths ending in the cache after one bounce, 1/16 of the pixels
    tracing training paths, 4 Adam steps of 16384 samples per frame, trained from scratch
    inside the timed region)."""
    import torch
    W, H = info.width, info.height
    img = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    t = time.perf_counter()
    ctx.render(sc, spp=args.ref_spp, out=img)
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t
    ref = img.clone().double()
    den = ref * ref + 1e-2

    def relmse(x):
        return float(((x.double() - ref) ** 2 / den).mean())
    target = 1e-2
    plain = []
    for spp in (1, 2, 4, 8, 16, 32, 64, 128):
        torch.cuda.synchronize()
        t = time.perf_counter()
        ctx.render(sc, spp=spp, out=img)
        torch.cuda.synchronize()
        plain.append(((time.perf_counter() - t) * 1000, relmse(img)))
    cache = B.RadianceCache(ctx, info.world_min, info.world_max, seed=1)
    acc = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
    curve, elapsed, st = [], 0.0, {}
    checkpoints = {1, 2, 4, 8, 16, 24, 32, 48, 64, 96, 128, 192, 256, 384, 512, 768, 1000}
    losses, queries, samples = [], 0, 0
    # a frame's image is complete when render_frame returns; its training runs on the
    # cache's own stream beside the next frame's path tracing, so each frame waits only for
    # torch's stream (the accumulation), not for the whole device
    cur = torch.cuda.current_stream()
    torch.cuda.synchronize()
    for f in range(args.nrc_frames):
        t = time.perf_counter()
        cache.render_frame(sc, f, out=img, terminate_vertex=1, train_stride=16, train_steps=4, train_batch=16384,
                           stats=st)
        acc += img
        cur.synchronize()
        elapsed += (time.perf_counter() - t) * 1000
        losses.append(st["loss"])
        queries, samples = st["queries"], st["train_samples"]
        if f + 1 in checkpoints or f + 1 == args.nrc_frames:
            curve.append((elapsed, relmse(acc / (f + 1))))
    # MLP throughput on the tensor cores: inference of 2^21 queries and training steps of
    # 2^14 samples, CUDA events on the context stream around the calls
    mlp = None
    try:
        nq = 1 << 21
        g = torch.Generator(device="cuda").manual_seed(0)
        q = torch.rand((nq, 13), device="cuda", generator=g)
        lo = torch.tensor(info.world_min, device="cuda")
        hi = torch.tensor(info.world_max, device="cuda")
        q[:, 0:3] = lo + (hi - lo) * q[:, 0:3]
        q[:, 3:9] = q[:, 3:9] * 2 - 1
        pred = torch.empty((nq, 4), device="cuda")
        # a stream of our own: handle 0 would select the library context's stream, which
        # events recorded on torch's default stream do not order against
        ts = torch.cuda.Stream()
        sid = ts.cuda_stream
        torch.cuda.synchronize()
        for _ in range(3):
            cache.infer(q, nq, pred, stream=sid)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ts)
        reps = 10
        for _ in range(reps):
            cache.infer(q, nq, pred, stream=sid)
        e1.record(ts)
        torch.cuda.synchronize()
        infer_ms = e0.elapsed_time(e1) / reps
        flops_fwd = 2 * (80 * 64 + 4 * 64 * 64 + 64 * 16)
        train_batch = torch.cat([q[:16384], torch.rand((16384, 3), device="cuda", generator=g)], 1).contiguous()
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            cache.train(train_batch, 16384)
        train_ms = (time.perf_counter() - t) * 1000 / reps
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        bf16_peak = peaks.get("bf16_tflops", 1900.0)
        infer_tflops = nq * flops_fwd / (infer_ms / 1000) / 1e12
        mlp = {"infer_queries": nq, "infer_ms": infer_ms, "infer_mqueries_s": nq / infer_ms / 1e3,
               "flops_per_query_fwd": flops_fwd, "infer_tflops": infer_tflops, "bf16_peak_tflops": bf16_peak,
               "infer_frac_of_bf16_peak": infer_tflops / bf16_peak,
               "hash_bytes_per_query": 16 * 8 * 2 * 2,
               "train_step_ms_16384": train_ms,
               "note": "inference: tcgen05.mma kind::f16 (BF16, FP32 accumulators in TMEM), hash-grid and SH "
                       "encoding in the same kernel, uniformly random queries; training step (mma.sync m16n8k16) "
                       "= fused forward/backward + weight-gradient GEMMs + Adam over all 16.8M hash and 22.5K MLP "
                       "parameters (wall time, synchronised)"}
    except Exception as ex:
        mlp = {"error": str(ex)}
    cache.close()
    # the same study with the path-spread termination rule (c = 0.01)
    spread_rule = None
    if spread > 0:
        cache = B.RadianceCache(ctx, info.world_min, info.world_max, seed=1)
        acc.zero_()
        scurve, selapsed, sst = [], 0.0, {}
        torch.cuda.synchronize()
        for f in range(args.nrc_frames):
            t = time.perf_counter()
            cache.render_frame(sc, f, out=img, terminate_vertex=1, train_stride=16, train_steps=4,
                               train_batch=16384, stats=sst, spread_threshold=spread)
            acc += img
            cur.synchronize()
            selapsed += (time.perf_counter() - t) * 1000
            if f + 1 in checkpoints or f + 1 == args.nrc_frames:
                scurve.append((selapsed, relmse(acc / (f + 1))))
        cache.close()
        tsp = _time_to(scurve, target)
        tpp = _time_to(plain, target)
        spread_rule = {"spread_c": spread, "nrc_ms_to_target": tsp,
                       "time_ratio_nrc_over_plain": (tsp / tpp) if (tsp and tpp) else None,
                       "nrc_ms_per_frame": selapsed / args.nrc_frames, "nrc_queries_per_frame": sst.get("queries"),
                       "nrc_curve_ms_relmse": [[round(t, 3), e] for t, e in scurve]}
    tp, tn = _time_to(plain, target), _time_to(curve, target)
    # the cache's relMSE at the plain tracer's time to reach the target, and vice versa
    at_plain = None
    if tp is not None:
        below = [e for t, e in curve if t <= tp]
        at_plain = below[-1] if below else None
    return {
        "target_relmse": target, "reference_spp": args.ref_spp, "reference_s": ref_s,
        "plain_curve_ms_relmse": [[round(t, 3), e] for t, e in plain],
        "nrc_curve_ms_relmse": [[round(t, 3), e] for t, e in curve],
        "plain_ms_to_target": tp, "nrc_ms_to_target": tn,
        "time_ratio_nrc_over_plain": (tn / tp) if (tp and tn) else None,
        "nrc_relmse_at_plain_time": at_plain,
        # the bound: one cache frame against one plain path per pixel. A cache that removed no
        # per-sample error could not reach the target sooner than the plain tracer at any
        # frame cost; a 2x shorter time needs the cache frame's error (cost x relMSE) halved
        "per_sample_relmse_ratio_nrc_over_plain": (curve[0][1] / plain[0][1]) if (curve and plain) else None,
        "nrc_frames": args.nrc_frames, "nrc_ms_per_frame": elapsed / args.nrc_frames,
        "nrc_queries_per_frame": queries, "nrc_train_samples_per_frame": samples,
        "nrc_loss_first_last": [float(np.mean(losses[:4])), float(np.mean(losses[-4:]))],
        "mlp": mlp,
        "spread_rule": spread_rule,
        "setup": "paths end in the cache at the first non-delta vertex after one bounce; 1/16 of the pixels "
                 "trace training paths each frame; 4 Adam steps x 16384 samples per frame, on the cache's own "
                 "stream beside the next frame's path tracing (the next frame's inference waits for them); "
                 "cache trained from scratch inside the timed frames",
    }


def batch_study(B, ctx):
    """Batched uneven scenes (64 seeded terrain scenes, 1e4..5e5 triangles, 128^2..512^2,
    16..64 spp, depth 12): aggregate Mpaths/s rendering them one after another with the
    default settings, and through 4 concurrent lanes with the autotuner's queue capacity
    and grid size (autotuning probes run before the timed batch)."""
    import torch
    from btrc_gb300 import scenes
    paths = scenes.batch(count=64, seed=1004)
    t = time.perf_counter()
    scs = ctx.load_build_scenes(paths)  # all 64 loads and builds on one pool of host threads
    build_s = time.perf_counter() - t
    infos = [s.info() for s in scs]
    outs = [torch.empty((i.height, i.width, 3), dtype=torch.float32, device="cuda") for i in infos]
    total_paths = sum(i.width * i.height * i.spp for i in infos)
    for s, o in zip(scs, outs):  # warm
        ctx.render(s, out=o)
    torch.cuda.synchronize()
    t = time.perf_counter()
    per = []
    for s, o in zip(scs, outs):
        t1 = time.perf_counter()
        ctx.render(s, out=o)
        per.append((time.perf_counter() - t1) * 1000)
    torch.cuda.synchronize()
    seq_ms = (time.perf_counter() - t) * 1000
    ctx.render_batch(scs, outs, lanes=4, autotune=True)  # tunes and warms
    runs = []
    for _ in range(3):
        stats, total_ms = ctx.render_batch(scs, outs, lanes=4, autotune=True)
        runs.append(total_ms)
    batch_ms = float(np.median(runs))
    caps = sorted({(st["capacity"], st["grid_pct"]) for st in stats})
    # one merged pass: every scene's paths in one queue through one set of stage kernels
    merged = None
    try:
        ctx.render_batch(scs, outs, autotune=True, merged=True)  # concatenates, tunes and warms
        mruns, mstats = [], None
        for _ in range(3):
            mstats, mtotal = ctx.render_batch(scs, outs, autotune=True, merged=True)
            mruns.append(mtotal)
        mms = float(np.median(mruns))
        done = [st["done_ms"] for st in mstats]
        merged = {"merged_mpaths_s": total_paths / (mms / 1000) / 1e6, "merged_ms": mms,
                  "autotuned_capacity_block_grid_pct": [mstats[0]["capacity"], mstats[0]["block"],
                                                        mstats[0]["grid_pct"]],
                  "per_scene_done_ms": {"min": min(done), "median": float(np.median(done)), "max": max(done)},
                  "note": "all scenes in one path queue through one set of persistent stage kernels under one "
                          "captured two-bounce graph; per-scene time is the device time to the end of the launch "
                          "after the first one that left none of the scene's paths in the queue (a census of the "
                          "queue after every launch; scenes with fewer paths are queued first)"}
    except Exception as ex:  # the merged pass must not sink the lanes figures
        merged = {"error": str(ex)}
    # the same batch with BVHs built on the device: load + build time, and the merged pass
    # through those trees (PLOC trees trace a little slower than the host's binned SAH)
    device = None
    try:
        t = time.perf_counter()
        dscs = ctx.load_build_scenes(paths, builder="device")
        torch.cuda.synchronize()
        dbuild_s = time.perf_counter() - t
        ctx.render_batch(dscs, outs, autotune=True, merged=True)
        druns = []
        for _ in range(3):
            _, dtotal = ctx.render_batch(dscs, outs, autotune=True, merged=True)
            druns.append(dtotal)
        dms = float(np.median(druns))
        device = {"scene_build_s": dbuild_s, "bvh_ms_max": max(x.info().bvh_ms for x in dscs),
                  "merged_mpaths_s": total_paths / (dms / 1000) / 1e6, "merged_ms": dms,
                  "build_plus_merged_s": dbuild_s + dms / 1000,
                  "host_build_plus_merged_s": build_s + (merged or {}).get("merged_ms", float("nan")) / 1000}
        for x in dscs:
            x.close()
    except Exception as ex:
        device = {"error": str(ex)}
    for s in scs:
        s.close()
    return {
        "scenes": len(scs), "total_paths": total_paths, "triangles_range": [min(i.triangles for i in infos),
                                                                             max(i.triangles for i in infos)],
        "sequential_mpaths_s": total_paths / (seq_ms / 1000) / 1e6, "sequential_ms": seq_ms,
        "batched_mpaths_s": total_paths / (batch_ms / 1000) / 1e6, "batched_ms": batch_ms, "lanes": 4,
        "per_scene_ms_sequential": {"min": min(per), "median": float(np.median(per)), "max": max(per)},
        "per_scene_ms_batched": {"min": min(st["ms"] for st in stats),
                                 "median": float(np.median([st["ms"] for st in stats])),
                                 "max": max(st["ms"] for st in stats)},
        "per_scene_done_ms_batched": {"min": min(st["done_ms"] for st in stats),
                                      "median": float(np.median([st["done_ms"] for st in stats])),
                                      "max": max(st["done_ms"] for st in stats),
                                      "note": "time from the start of the batch until the scene's image was complete"},
        "per_scene_done_ms_sequential": {"min": float(np.cumsum(per).min()),
                                         "median": float(np.median(np.cumsum(per))),
                                         "max": float(np.cumsum(per).max())},
        "autotuned_capacity_grid_pct": caps, "scene_build_s": build_s,
        "merged": merged, "device_bvh": device,
    }


def run_ours(args, world, rank, local):
    import torch

    import btrc_gb300 as B
    torch.cuda.set_device(local)
    path = scene_path(args)
    ctx = B.Context(local)
    t0 = time.perf_counter()
    sc = ctx.load_scene(path)
    load_s = time.perf_counter() - t0
    sc.build()
    info = sc.info()
    # the same scene with its BVH built on the device (PLOC + the same 8-wide collapse)
    build_cmp = {"host": {"build_ms": info.build_ms, "bvh_ms": info.bvh_ms, "bvh_nodes": info.bvh_nodes}}
    try:
        dsc = ctx.load_scene(path).build(builder="device")
        di = dsc.info()
        build_cmp["device"] = {"build_ms": di.build_ms, "bvh_ms": di.bvh_ms, "bvh_nodes": di.bvh_nodes,
                               "builder": di.bvh_builder}
        dsc.close()
    except Exception as ex:
        build_cmp["device"] = {"error": str(ex)}
    W, H, spp = info.width, info.height, args.spp
    paths = W * H * spp
    out_dev = torch.empty((H, W, 3), dtype=torch.float32, device="cuda")
    out_host = torch.empty((H, W, 3), dtype=torch.float32).pin_memory()

    for _ in range(args.warmup):
        ctx.render(sc, spp=spp, out=out_dev)

    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    clocks.start()
    dev_ms = []
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        st = {}
        ctx.render(sc, spp=spp, out=out_dev, stats=st)
        dev_ms.append(st["device_ms"])
    torch.cuda.synchronize()
    wall_dev = time.perf_counter() - wall0
    barrier(world)
    launches = st["kernel_launches"]

    # end to end: the C-ABI call with a host output buffer (image download inside)
    barrier(world)
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(max(2, args.steps // 2)):
        st2 = {}
        t = time.perf_counter()
        ctx.render(sc, spp=spp, out=out_host, stats=st2)  # host (pinned) output buffer
        e2e_ms.append((time.perf_counter() - t) * 1000)
    torch.cuda.synchronize()
    barrier(world)
    clk = clocks.stop()

    step_ms = all_max(world, float(np.mean(dev_ms)))
    value = world * paths / (step_ms / 1000) / 1e6
    e2e_step = all_max(world, float(np.mean(e2e_ms)))
    e2e_value = world * paths / (e2e_step / 1000) / 1e6

    # the same frame through the two-level form (one tree per geometry under a top level
    # over the instances): throughput and acceleration-structure bytes beside the
    # flattened form's
    try:
        tsc = ctx.load_scene(path).build(two_level=True)
        ti = tsc.info()
        ctx.render(tsc, spp=spp, out=out_dev)
        tms = []
        for _ in range(2):
            tst = {}
            ctx.render(tsc, spp=spp, out=out_dev, stats=tst)
            tms.append(tst["device_ms"])
        build_cmp["two_level"] = {"mpaths_s": paths / (float(np.mean(tms)) / 1000) / 1e6,
                                  "bvh_bytes": ti.bvh_bytes, "flattened_bvh_bytes": info.bvh_bytes,
                                  "build_ms": ti.build_ms}
        tsc.close()
    except Exception as ex:
        build_cmp["two_level"] = {"error": str(ex)}

    # roofline of the dominant stage: stage times by CUDA events (profile 1), traversal
    # work from counters (profile 2), both on the same frame
    prof = {}
    ctx.render(sc, spp=spp, out=out_dev, stats=prof, profile=1)
    cnt = {}
    ctx.render(sc, spp=spp, out=out_dev, stats=cnt, profile=2)
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    stage_ms = prof["stage_ms"]
    total_stage = sum(stage_ms.values())
    dom = max(stage_ms, key=stage_ms.get)
    trace_ms = stage_ms["trace"]
    trace_launches = prof["stage_launches"]["trace"]
    ext_rays = cnt["extension_rays"]
    node_b, tri_b = 80, 48
    # algorithmic bytes: node visits and triangle tests per ray from the oracle's traversal
    # of the same BVH on camera and bounce rays of this workload, weighted by this frame's
    # camera rays (one per path) and secondary rays; the kernel's own counters beside them
    cam_rays = min(cnt["paths"], ext_rays)
    sec_rays = ext_rays - cam_rays
    try:
        tc = traversal_counts(args, ctx, sc)
        c, b = tc["camera"], tc["bounce"]
        oracle_nodes = cam_rays * c["oracle_nodes"] + sec_rays * b["oracle_nodes"]
        oracle_tris = cam_rays * c["oracle_tris"] + sec_rays * b["oracle_tris"]
        counts_source = ("oracle: sequential exact-box traversal of the exported BVH on 1/8 of the camera rays "
                         "and one diffuse bounce ray per camera hit, weighted by this frame's camera and "
                         "secondary rays")
    except Exception as ex:  # fall back to the kernel's counters, and say so
        tc = {"error": str(ex)}
        oracle_nodes, oracle_tris = cnt["node_visits"], cnt["tri_tests"]
        counts_source = "kernel counters (profile 2): the oracle count failed"
    trace_bytes = ext_rays * (32 + 20) + oracle_nodes * node_b + oracle_tris * tri_b
    achieved = trace_bytes / (trace_ms / 1000) / 1e9 if trace_ms > 0 else None
    # DRAM bytes per camera / secondary ray from the committed ncu capture, scaled to this
    # run's average launch
    traffic_path = ROOT / "profiles" / "trace_traffic.json"
    traffic = None
    if traffic_path.exists():
        try:
            tj = json.loads(traffic_path.read_text())
            # camera rays (one per path) and secondary rays measured separately
            cam_rays = min(cnt["paths"], ext_rays)
            traffic = (tj["camera_dram_bytes_per_ray"] * cam_rays +
                       tj["secondary_dram_bytes_per_ray"] * (ext_rays - cam_rays)) / max(trace_launches, 1)
        except (ValueError, KeyError):
            traffic = None

    batch = None
    if rank == 0 and not args.no_batch:
        try:
            batch = batch_study(B, ctx)
        except Exception as ex:  # the study must not sink the throughput number
            batch = {"error": str(ex)}

    nrc = None
    nrc_interior = None
    if rank == 0 and not args.no_nrc:
        try:
            nrc = nrc_study(B, ctx, sc, info, args, spread=0.01)
        except Exception as ex:  # the study must not sink the throughput number
            nrc = {"error": str(ex)}
        # the same study in a closed interior, where most light arrives after several bounces
        try:
            from btrc_gb300 import scenes
            csc = ctx.load_scene(scenes.cornell(width=512, height=512, spp=16)).build()
            nrc_interior = nrc_study(B, ctx, csc, csc.info(), args, spread=0.01)
            nrc_interior = {"scene": "config 0's Cornell box (two icospheres, quad light) at 512x512",
                            **{k: nrc_interior[k] for k in ("target_relmse", "reference_spp", "plain_ms_to_target",
                                                            "nrc_ms_to_target", "time_ratio_nrc_over_plain",
                                                            "nrc_relmse_at_plain_time",
                                                            "per_sample_relmse_ratio_nrc_over_plain",
                                                            "nrc_ms_per_frame",
                                                            "nrc_queries_per_frame", "plain_curve_ms_relmse",
                                                            "nrc_curve_ms_relmse", "spread_rule")}}
            csc.close()
        except Exception as ex:
            nrc_interior = {"error": str(ex)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(path, args.cpu_seconds)
        except Exception as ex:  # the baseline must not sink the GPU number
            cpu = {"value": None, "unit": "Mpaths/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"failed: {ex}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": bench_config(args, info.triangles),
            "bvh_bytes": int(info.bvh_bytes), "shading_record_bytes": int(info.triangles) * 96,
            "e2e": {"value": e2e_value, "unit": "Mpaths/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": W * H * 3 * 4,
                    "note": "btrc_render through the C ABI into a pinned host buffer (image download "
                            "inside the timed call); the scene is resident, the per-frame input is the "
                            "kernel-parameter camera"},
            "gpu_launches": int(launches) * args.steps,
            "roofline": {"bound": "hbm", "kernel": "k_trace (closest hit)", "achieved": achieved,
                         "peak": hbm_peak, "unit": "GB/s",
                         "frac": (achieved / hbm_peak) if achieved else None, "traffic": traffic,
                         "bytes_per_ray": trace_bytes / max(ext_rays, 1),
                         "nodes_per_ray": oracle_nodes / max(ext_rays, 1),
                         "tris_per_ray": oracle_tris / max(ext_rays, 1),
                         "counts_source": counts_source,
                         "kernel_nodes_per_ray": cnt["node_visits"] / max(ext_rays, 1),
                         "kernel_tris_per_ray": cnt["tri_tests"] / max(ext_rays, 1),
                         "probe_counts": tc,
                         "l2": l2_figures(),
                         "launches": trace_launches, "avg_launch_ms": trace_ms / max(trace_launches, 1),
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback 6800",
                         "traffic_source": "ncu dram__bytes per camera ray and per secondary ray "
                                           "(profiles/trace_traffic.json) x this frame's rays / launches",
                         "stage_share": {k: v / total_stage for k, v in stage_ms.items() if total_stage > 0},
                         "dominant_stage": dom},
            "cpu_baseline": cpu,
            "clocks": clk,
            "radiance_cache": nrc,
            "radiance_cache_interior": nrc_interior,
            "batch": batch,
            "mrays_per_s": world * (st["extension_rays"] + st["shadow_rays"]) / (step_ms / 1000) / 1e6,
            "scene_load_s": load_s, "bvh_build_ms": info.build_ms,
            "scene_build": build_cmp,
        }
        print(json.dumps(line), flush=True)
    sc.close()
    ctx.close()


def probe_rays(args, ctx, sc, stride: int = 1):
    """Camera rays through pixel centres of the workload's camera (every stride-th pixel)
    and one ray per camera hit in a uniform direction of the upper hemisphere (the
    terrain's surfaces face up), traced through btrc_trace_closest."""
    import math
    import torch
    p = scene_path(args)
    js = json.loads(Path(p).read_text())
    W, H, cam = js["width"], js["height"], js["camera"]
    eye, dst, up = (np.array(cam[k], np.float64) for k in ("eye", "dst", "up"))
    fwd = (dst - eye) / np.linalg.norm(dst - eye)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    th = math.tan(math.radians(cam["fov_y"]["deg"]) / 2)
    X, Y = np.meshgrid((2 * (np.arange(W) + 0.5) / W - 1) * th * W / H, (1 - 2 * (np.arange(H) + 0.5) / H) * th)
    d = (fwd[None, None] + X[..., None] * right + Y[..., None] * upv).reshape(-1, 3)[::stride]
    d /= np.linalg.norm(d, axis=1, keepdims=True)

    def pack(o, dirs):
        r = np.zeros((len(o), 8), np.float32)
        r[:, 0:3], r[:, 4:7], r[:, 7] = o, dirs, 3.0e38
        return r

    def trace(rays):
        m = len(rays)
        dr = torch.from_numpy(rays).cuda()
        f = torch.zeros(m, dtype=torch.int32, device="cuda")
        h = torch.zeros((m, 4), dtype=torch.float32, device="cuda")
        ctx.trace_closest(sc, dr, m, f, h)
        torch.cuda.synchronize()
        return f.cpu().numpy().view(np.uint32), h.cpu().numpy()

    cam_rays = pack(np.broadcast_to(eye, d.shape), d)
    f, h = trace(cam_rays)
    hit = f != 0
    org = eye + d[hit] * (h[hit, 0:1].astype(np.float64) - 1e-4)
    nd = np.random.default_rng(3).normal(size=org.shape)
    nd /= np.linalg.norm(nd, axis=1, keepdims=True)
    nd[:, 1] = np.abs(nd[:, 1])
    return cam_rays, pack(org, nd), trace


def traversal_counts(args, ctx, sc):
    """Node visits and triangle tests per camera ray and per bounce ray: the oracle's
    sequential exact-box traversal of the same exported BVH on the same rays, and the
    kernel's own per-ray counters (btrc_trace_stats) beside it."""
    import torch
    import btrc_gb300 as B
    import oracle
    hctx = B.Context(-1)
    hsc = hctx.load_scene(scene_path(args)).build()
    nodes, tris = hsc.export_bvh()
    hsc.close()
    hctx.close()
    cam, sec, _ = probe_rays(args, ctx, sc, stride=8)
    out = {}
    for name, rays in (("camera", cam), ("bounce", sec)):
        nv, tt = oracle.wide_bvh_counts(nodes, tris, rays)
        dr = torch.from_numpy(rays).cuda()
        gn = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
        gt = torch.zeros(len(rays), dtype=torch.int32, device="cuda")
        ctx.trace_stats(sc, dr, len(rays), gn, gt)
        torch.cuda.synchronize()
        out[name] = {"rays": len(rays), "oracle_nodes": float(nv.mean()), "oracle_tris": float(tt.mean()),
                     "kernel_nodes": float(gn.cpu().numpy().mean()), "kernel_tris": float(gt.cpu().numpy().mean())}
    return out


def trace_probe(args):
    """Two closest-hit launches over the benchmark scene: the 1-spp pinhole camera rays
    through pixel centres, then one ray per camera hit in a uniform direction of the upper
    hemisphere (the terrain's surfaces face up), so that an ncu capture can measure DRAM
    bytes per camera ray and per secondary ray separately."""
    import math
    import torch
    import btrc_gb300 as B
    from btrc_gb300 import scenes
    p = scenes.terrain(seed=1001, width=args.width, height=args.height, spp=1, grid=args.grid,
                       instances=args.instances)
    js = json.loads(Path(p).read_text())
    W, H, cam = js["width"], js["height"], js["camera"]
    eye, dst, up = (np.array(cam[k], np.float64) for k in ("eye", "dst", "up"))
    fwd = (dst - eye) / np.linalg.norm(dst - eye)
    right = np.cross(fwd, up)
    right /= np.linalg.norm(right)
    upv = np.cross(right, fwd)
    th = math.tan(math.radians(cam["fov_y"]["deg"]) / 2)
    X, Y = np.meshgrid((2 * (np.arange(W) + 0.5) / W - 1) * th * W / H, (1 - 2 * (np.arange(H) + 0.5) / H) * th)
    d = (fwd[None, None] + X[..., None] * right + Y[..., None] * upv).reshape(-1, 3)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    ctx = B.Context(0)
    sc = ctx.load_scene(p).build()

    def trace(o, dirs):
        m = len(o)
        r = np.zeros((m, 8), np.float32)
        r[:, 0:3], r[:, 4:7], r[:, 7] = o, dirs, 3.0e38
        dr = torch.from_numpy(r).cuda()
        f = torch.zeros(m, dtype=torch.int32, device="cuda")
        h = torch.zeros((m, 4), dtype=torch.float32, device="cuda")
        ctx.trace_closest(sc, dr, m, f, h)
        torch.cuda.synchronize()
        return f.cpu().numpy().view(np.uint32), h.cpu().numpy()

    f, h = trace(np.broadcast_to(eye, d.shape), d)
    hit = f != 0
    org = eye + d[hit] * (h[hit, 0:1].astype(np.float64) - 1e-4)
    nd = np.random.default_rng(3).normal(size=org.shape)
    nd /= np.linalg.norm(nd, axis=1, keepdims=True)
    nd[:, 1] = np.abs(nd[:, 1])
    f2, _ = trace(org, nd)
    print(json.dumps({"camera_rays": len(d), "camera_hit_rate": float(hit.mean()), "secondary_rays": int(hit.sum()),
                      "secondary_hit_rate": float((f2 != 0).mean())}), flush=True)
    sc.close()
    ctx.close()


def probe(args):
    """Small cases for ncu captures (a few GB on the device at most, few launches)."""
    import torch
    import btrc_gb300 as B
    from btrc_gb300 import scenes
    ctx = B.Context(0)
    if args.probe == "nrc-frames":
        p = scenes.cornell(width=512, height=512, spp=16)
        sc = ctx.load_scene(p).build()
        info = sc.info()
        img = torch.empty((info.height, info.width, 3), dtype=torch.float32, device="cuda")
        cache = B.RadianceCache(ctx, info.world_min, info.world_max, seed=1)
        cur = torch.cuda.current_stream()
        walls, st = [], {}
        for f in range(25):
            t = time.perf_counter()
            cache.render_frame(sc, f, out=img, terminate_vertex=1, train_stride=16, train_steps=4,
                               train_batch=16384, stats=st)
            cur.synchronize()
            walls.append((time.perf_counter() - t) * 1000)
        torch.cuda.synchronize()
        print(json.dumps({"wall_ms": walls[5:], "render_ms": st["render_ms"], "queries": st["queries"]}), flush=True)
        cache.close()
        ctx.close()
        return
    if args.probe == "build-device":
        p = scenes.terrain(width=1920, height=1080, spp=1, state_count=1 << 21)
        sc = ctx.load_scene(p).build(builder="device")
        info = sc.info()
        print(json.dumps({"bvh_ms": info.bvh_ms, "build_ms": info.build_ms, "bvh_nodes": info.bvh_nodes,
                          "builder": info.bvh_builder}), flush=True)
        ctx.close()
        return
    if args.probe == "nrc":
        p = scenes.terrain(width=480, height=270, spp=1, grid=256, instances=20)
        sc = ctx.load_scene(p).build()
        info = sc.info()
        cache = B.RadianceCache(ctx, info.world_min, info.world_max, seed=1)
        nq = 1 << 20
        g = torch.Generator(device="cuda").manual_seed(0)
        q = torch.rand((nq, 13), device="cuda", generator=g)
        lo, hi = torch.tensor(info.world_min, device="cuda"), torch.tensor(info.world_max, device="cuda")
        q[:, 0:3] = lo + (hi - lo) * q[:, 0:3]
        q[:, 3:9] = q[:, 3:9] * 2 - 1
        pred = torch.empty((nq, 4), device="cuda")
        tb = torch.cat([q[:16384], torch.rand((16384, 3), device="cuda", generator=g)], 1).contiguous()
        for _ in range(3):
            cache.infer(q, nq, pred)
            cache.train(tb, 16384)
        torch.cuda.synchronize()
        cache.close()
    else:
        if args.probe == "medium":
            p = scenes.volume(width=256, height=256, spp=4, state_count=1 << 20)
        else:
            p = scenes.terrain(width=1920, height=1080, spp=1, state_count=1 << 21)
        sc = ctx.load_scene(p).build(two_level=args.probe == "trace-two-level")
        info = sc.info()
        img = torch.empty((info.height, info.width, 3), device="cuda")
        st = {}
        ctx.render(sc, out=img, stats=st)
        torch.cuda.synchronize()
        print(json.dumps({k: v for k, v in st.items() if k not in ("stage_ms", "stage_launches")}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.probe:
        probe(args)
        return
    if args.trace_probe:
        trace_probe(args)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
