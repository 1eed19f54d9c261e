#!/usr/bin/env python
"""Throughput of the 64-tree DDA traversal (primary G-buffer + 1 GI ray per hit pixel) on GB300.

Workload (the 1024^3 config): seeded heightfield + 3D value-noise caves, 4x4x4 chunks of 256^3 (a
5-level 64-tree world), 1920x1080 pinhole primary rays (FOV 70, 30 degrees down) plus one cosine-
weighted GI ray per hit pixel (Pass-2A sampling), up to 512 DDA steps per ray, LOD pushed out of
reach. A step is one frame. Prints one JSON line.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value     Mrays/s with pools and outputs resident in HBM, frame kernel timed with CUDA events on the
          library's stream, L2 flushed (256 MiB write) before every timed frame.
e2e       the same metric through the C ABI with host buffers (arc_set_camera + arc_trace_frame: launch
          + D2H of the G-buffer and both hit arrays every frame), wall-clock; the camera records
          themselves are built before the timed region.
reference the reference's CPU ray query (WorldMap::raycast_meters -> raycast_chunk_tree, restated in
          C in oracle/) on all host cores, full frames.
Multi-GPU: replicas only (each rank traces its own frame); value = all ranks' rays / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Mrays/s on 1 GB300 (primary+GI)"
UNIT = "Mrays/s"
SCENE = "c2_1024_caves"
WIDTH, HEIGHT = 1920, 1080
WORKLOAD = ("1024^3 caves world (4^3 chunks, 5-level 64-tree), 1920x1080 primary + 1 cosine GI ray per hit "
            "pixel, <=512 DDA steps per ray")


def _args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU baseline sample budget")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--variant", type=int, default=None, help="0 plain kernel, 1 persistent kernel (default: tuned)")
    p.add_argument("--reg-blocks", type=int, default=None, help="register budget (CTAs/SM the kernel is built for)")
    p.add_argument("--block-threads", type=int, default=None)
    p.add_argument("--order", type=int, default=None, help="block order of the plain kernel: 0 row-major, 1 Morton")
    p.add_argument("--features", type=int, default=None, help="traversal variant bits (ARC_FEAT_*)")
    p.add_argument("--refill-threshold", type=int, default=None,
                   help="variant 1: idle lanes before a refill; ARC_FEAT_GI_REPACK: DDA steps between repacks")
    p.add_argument("--flush-l2", action="store_true", help="with --frame-only, still flush L2 before every timed frame")
    p.add_argument("--frame-bands", type=int, default=None,
                   help="device frames in this many concurrent row bands (library default: 4; 1 = one launch)")
    p.add_argument("--width", type=int, default=WIDTH)
    p.add_argument("--height", type=int, default=HEIGHT)
    p.add_argument("--frame-only", action="store_true", help="time only the frame kernel (profiling runs)")
    p.add_argument("--no-autotune", action="store_true", help="keep the library's default launch configuration")
    p.add_argument("--no-batched", action="store_true", help="skip the multi-view batch section")
    p.add_argument("--no-nrc", action="store_true", help="skip the radiance-cache comparison section")
    p.add_argument("--nrc-frames", type=int, default=300)
    p.add_argument("--no-restir", action="store_true", help="skip the ReSTIR GI temporal pass section")
    p.add_argument("--restir-only", action="store_true", help="run only the ReSTIR GI temporal pass section (profiling runs)")
    p.add_argument("--no-c5", action="store_true", help="skip the 4096^3 edit + trace + NRC pipeline section")
    p.add_argument("--c5-frames", type=int, default=300)
    p.add_argument("--c5-width", type=int, default=3840)
    p.add_argument("--c5-height", type=int, default=2160)
    return p.parse_args()


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _camera(scene, frame, width=None, height=None):
    from arcadia_gb300 import layout as L

    return L.default_camera_for(scene, width or WIDTH, height or HEIGHT, quality=L.quality_parity(512),
                                frame_index=frame)


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while the GPU works.

    The sampler process is always reaped (stop() or interpreter exit), so no nvidia-smi child
    outlives the bench (a profiler waiting on children would otherwise never return)."""

    live = []

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        if self.p is not None:
            ClockSampler.live.append(self.p)
            import atexit

            atexit.register(ClockSampler._reap)

    @staticmethod
    def _reap():
        for p in ClockSampler.live:
            if p.poll() is None:
                p.kill()

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip() == "Active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)["hbm_gbs"], "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def _peaks_all():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}


def _l2_copy_gbs(dev, mib=32, iters=50):
    """Copy bandwidth of a working set resident in L2 (two buffers of `mib` MiB, read + write bytes):
    `iters` copies replayed from one CUDA graph (no launch gaps), best of 5 replays, CUDA events. The
    L2 ceiling of a traversal whose node fetches are mostly cache hits."""
    import torch

    a = torch.empty(mib << 20, dtype=torch.uint8, device=dev)
    b = torch.empty_like(a)
    a.fill_(1)
    side = torch.cuda.Stream(device=dev)
    with torch.cuda.stream(side):
        for _ in range(3):
            b.copy_(a)
    torch.cuda.synchronize(dev)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(iters):
            b.copy_(a)
    best = 0.0
    for _ in range(5):
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        g.replay()
        s1.record()
        s1.synchronize()
        best = max(best, 2.0 * a.numel() * iters / (s0.elapsed_time(s1) * 1e-3) / 1e9)
    del g, a, b
    return best


def _profile_traffic(kernel: str):
    """DRAM bytes of `kernel`'s frame (its launch, or its launches: the primary kernel and the GI pass)
    from a committed ncu summary (profiles/*.txt), if any."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".txt"):
            continue
        txt = open(os.path.join(d, fn)).read()
        if f"kernel={kernel}" in txt and f"workload={SCENE}" in txt:
            for line in txt.splitlines():
                if line.startswith("dram_bytes_per_frame=") or line.startswith("dram_bytes_per_launch="):
                    return float(line.split("=", 1)[1])
    return None


def _graph_ms(tracer):
    """Device time between the context's start/end events around the last launch."""
    return float(tracer.stats().last_kernel_ms)


def restir_section(t, scene, w, h, dev, bufs, frames=12):
    """ReSTIR GI temporal pass after each frame of the same world (frame kernel, SHARC update +
    resolve, then the pass on the frame's G-buffer and GI hit records), reference quality preset,
    static camera: the pass alone is timed with CUDA events on the library's stream."""
    import torch

    from arcadia_gb300 import layout as L

    gdm, gnm, gaa, hits, gi = bufs
    npx = w * h
    res = [torch.from_numpy(L.empty_reservoirs(npx).view(np.uint8)).to(dev) for _ in range(2)]
    stream = torch.cuda.ExternalStream(t.stream(), device=dev)
    t.sharc_reset()
    ms = []
    for i in range(frames):
        t.set_camera(L.default_camera_for(scene, w, h, quality=L.quality_high(), frame_index=i + 1))
        t.trace_frame_dev(w, h, gdm.data_ptr(), gnm.data_ptr(), gaa.data_ptr(), hits.data_ptr(), gi.data_ptr())
        t.sharc_update_dev(w, h, gdm.data_ptr(), gnm.data_ptr())
        t.sharc_resolve()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        t.restir_gi_temporal_dev(w, h, gdm.data_ptr(), gnm.data_ptr(), gi.data_ptr(), res[i % 2].data_ptr(),
                                 res[(i + 1) % 2].data_ptr())
        b.record(stream)
        t.synchronize()
        ms.append(a.elapsed_time(b))
    last = res[frames % 2].cpu().numpy().view(L.RESERVOIR_DTYPE)
    hit = last["primary_depth"] < 1e4
    m = (last["norm_m_flags"] >> 16) & 0xFF
    steady = statistics.mean(ms[2:])
    return {"workload": f"{w}x{h} frames of the 1024^3 caves world, high_quality preset, static camera",
            "ms_per_frame": round(steady, 4), "mpixels_per_s": round(npx / (steady * 1e-3) / 1e6, 1),
            "history_valid_fraction": round(float((m[hit] > 1).mean()), 4), "frames": frames,
            "per_pixel_bytes": 100, "rays_per_pixel": "1 sun shadow ray (+1 at secondary hits the cache misses)",
            "secondary_ray": "reused from the frame kernel's GI hit record (not traced again)",
            "l2": "not flushed; the pass reads 207 MB per 1080p frame (G-buffer, GI records, reservoirs)"}


def cpu_leg(scene_name, seconds, threads, reference_query=True, frame=0):
    """Times the CPU restatement on whole frames (pixel stride 1) until `seconds` of work are done."""
    from arcadia_gb300 import layout as L
    from oracle import pyorc

    scene = L.SCENES[scene_name]
    world = pyorc.build_world(scene)
    cam = _camera(scene, frame)
    pyorc.frame_sample(world, cam, 64, threads, cpu_query=reference_query)  # warm-up
    rays = frames = 0
    t0 = time.perf_counter()
    while True:
        r = pyorc.frame_sample(world, cam, 1, threads, cpu_query=reference_query)
        rays += r[0]
        frames += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return rays / dt / 1e6, frames, dt, world, cam


def bytes_per_pixel(world, cam, threads):
    """Algorithmic bytes per pixel path (primary + GI) from the instrumented oracle (every 16th pixel)."""
    from oracle import pyorc

    r = pyorc.frame_sample(world, cam, 16, threads, cpu_query=False)
    return r[4] / r[1]


def aggregate_ranks(total_ms: float, rays: float, device):
    """Whole-job figures of a replicas run: the slowest rank's time and the rays of all ranks (no-op
    without an initialised process group of more than one rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return total_ms, rays
    tt = torch.tensor([total_ms, float(rays)], dtype=torch.float64, device=device)
    mx = tt.clone()
    dist.all_reduce(mx, op=dist.ReduceOp.MAX)
    dist.all_reduce(tt, op=dist.ReduceOp.SUM)
    return float(mx[0]), float(tt[1])


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    from arcadia_gb300 import layout as L
    from oracle import pyorc

    scene = L.SCENES[SCENE]
    world = pyorc.build_world(scene)
    for i in range(args.warmup):
        pyorc.frame_sample(world, _camera(scene, i), 1, threads, cpu_query=True)
    rays = 0
    t0 = time.perf_counter()
    for i in range(args.steps):
        rays += pyorc.frame_sample(world, _camera(scene, args.warmup + i), 1, threads, cpu_query=True)[0]
    dt = time.perf_counter() - t0
    v = rays / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": round(v, 3), "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dt / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "scene": SCENE, "width": WIDTH, "height": HEIGHT, "parallelism": "host cores"},
        "cpu_baseline": {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} full frames ({WIDTH}x{HEIGHT} primary + GI) through the C restatement "
                                   "of WorldMap::raycast_meters -> raycast_chunk_tree"},
        "e2e": {"value": round(v, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch

    from arcadia_gb300 import build as nbuild
    from arcadia_gb300 import layout as L
    from arcadia_gb300 import native

    ws, rank, local = _dist()
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    nbuild.build()
    scene = L.SCENES[SCENE]
    roots, nodes, bricks, _ = native.build_world(scene)
    pal = native.default_palette()
    t = native.Tracer(local)
    t.upload_world(scene.grid, roots, nodes, bricks, pal)
    knobs = {k: v for k, v in (("variant", args.variant), ("reg_blocks", args.reg_blocks),
                               ("block_threads", args.block_threads), ("order", args.order),
                               ("features", args.features), ("refill_threshold", args.refill_threshold)) if v is not None}
    if knobs:
        t.set_launch_config(**knobs)
    if args.frame_bands is not None:
        rc = native.lib().arc_set_frame_bands(t.ctx, args.frame_bands)
        if rc:
            raise native.ArcError(rc, t.last_error())
    W_, H_ = args.width, args.height
    stream = torch.cuda.ExternalStream(t.stream(), device=torch.device("cuda", local))
    npx = W_ * H_
    dev = torch.device("cuda", local)
    gdm = torch.empty(npx * 2, dtype=torch.int32, device=dev)
    gnm = torch.empty(npx * 2, dtype=torch.int32, device=dev)
    gaa = torch.empty(npx, dtype=torch.int32, device=dev)
    hits = torch.empty(npx * 5, dtype=torch.int32, device=dev)
    gi = torch.empty(npx * 5, dtype=torch.int32, device=dev)
    n_gi = torch.zeros(max(args.steps, 1), dtype=torch.int64, device=dev)
    # L2 flush buffer (2x the 126 MB L2); profiling runs skip it so ncu has less memory to save/restore
    flush = torch.empty(16 if args.frame_only and not args.flush_l2 else 256 << 20, dtype=torch.uint8, device=dev)

    def frame(i, slot):
        t.set_camera(_camera(scene, i, W_, H_))
        t.trace_frame_dev(W_, H_, gdm.data_ptr(), gnm.data_ptr(), gaa.data_ptr(), hits.data_ptr(), gi.data_ptr(),
                          n_gi.data_ptr() + 8 * slot)

    if args.restir_only:
        r = restir_section(t, scene, W_, H_, dev, (gdm, gnm, gaa, hits, gi), frames=max(args.steps, 3))
        t.close()
        if rank == 0:
            print(json.dumps({"restir_gi_temporal": r}), flush=True)
        return

    tuned_ms = None
    if not knobs and not args.no_autotune:  # untimed setup: pick the launch configuration on this frame
        t.set_camera(_camera(scene, 0, W_, H_))
        _, tuned_ms = t.autotune_frame_dev(W_, H_, gdm.data_ptr(), gnm.data_ptr(), gaa.data_ptr(), hits.data_ptr(),
                                           gi.data_ptr(), frames=5)
    clocks = None if args.frame_only else ClockSampler(local)
    for i in range(args.warmup):
        frame(i, 0)
    t.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            starts[i].record(stream)
            frame(args.warmup + i, i)
            ends[i].record(stream)
    t.synchronize()
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = sum(ms)
    rays = args.steps * npx + int(n_gi.sum().item())
    total_ms, rays = aggregate_ranks(total_ms, rays, dev)
    value = rays / (total_ms * 1e-3) / 1e6
    cfg = t.launch_config()
    if args.frame_only:
        t.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 3), "unit": UNIT, "frame_only": True,
                              "width": W_, "height": H_, "ms_per_step": round(statistics.mean(ms), 4),
                              "variant": cfg.variant, "reg_blocks": cfg.reg_blocks}), flush=True)
        return

    # the library's default launch configuration (arc_create's: plain kernel + GI pass, 128 threads,
    # register budget 3, Morton block order, 4 row bands), same frames, against the tuned one above
    tuned_cfg = t.launch_config()
    t.set_launch_config(variant=0, block_threads=128, blocks_per_sm=0, tile_w=8, tile_h=4, refill_threshold=24,
                        reg_blocks=3, order=1, features=0)
    for i in range(args.warmup):  # untimed, as before the main loop
        frame(i, 0)
    t.synchronize()
    np_frames = min(args.steps, 20)
    with torch.cuda.stream(stream):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(np_frames)]
        for i in range(np_frames):
            flush.fill_(i & 0xFF)
            ev[i][0].record(stream)
            frame(args.warmup + i, i)
            ev[i][1].record(stream)
    t.synchronize()
    plain_ms = [a.elapsed_time(b) for a, b in ev]
    plain_rays = np_frames * npx + int(n_gi[:np_frames].sum().item())
    plain_value = plain_rays / (sum(plain_ms) * 1e-3) / 1e6
    t.set_launch_config(**{k: getattr(tuned_cfg, k) for k, _ in type(tuned_cfg)._fields_})

    # end to end through the C ABI with host (pinned) buffers
    pin = {k: torch.empty(n, dtype=torch.int32).pin_memory().numpy() for k, n in
           (("gdm", npx * 2), ("gnm", npx * 2), ("gaa", npx), ("hits", npx * 5), ("gi", npx * 5))}
    from arcadia_gb300.native import _p, lib
    import ctypes

    e2e_frames = min(args.steps, 20)
    cnt = ctypes.c_uint64()
    e2e_rays = 0
    for i in range(2):
        t.set_camera(_camera(scene, i))
        lib().arc_trace_frame(t.ctx, WIDTH, HEIGHT, _p(pin["gdm"]), _p(pin["gnm"]), _p(pin["gaa"]), _p(pin["hits"]),
                              _p(pin["gi"]), ctypes.byref(cnt))
    # the application's per-frame camera records are built beforehand (numpy takes ~0.1 ms each);
    # handing each to the library (arc_set_camera) is timed with its frame
    cams = [_camera(scene, args.warmup + i) for i in range(e2e_frames)]
    t0 = time.perf_counter()
    for i in range(e2e_frames):
        t.set_camera(cams[i])
        rc = lib().arc_trace_frame(t.ctx, WIDTH, HEIGHT, _p(pin["gdm"]), _p(pin["gnm"]), _p(pin["gaa"]), _p(pin["hits"]),
                                   _p(pin["gi"]), ctypes.byref(cnt))
        if rc:
            raise native.ArcError(rc, t.last_error())
        e2e_rays += npx + cnt.value
    e2e_dt = time.perf_counter() - t0
    e2e_value = e2e_rays / e2e_dt / 1e6

    # radiance caches at secondary hits on this world (NRC vs SHARC, same light transport)
    nrc = None
    if not args.no_nrc:
        from arcadia_gb300 import gi_cache

        t.set_launch_config(variant=cfg.variant)
        # operating point: 32,768 training samples and 4 Adam steps per frame, queries beside the updates
        nrc = gi_cache.run_comparison(t, SCENE, W_, H_, frames=args.nrc_frames, steps_per_frame=4, overlap=True,
                                      train_samples=32768, curve=(10, 20, 30, 60, 120))
        below = [c["frame"] for c in nrc["convergence"] if c["rel_mse_nrc"] < c["rel_mse_sharc"]]
        nrc["first_curve_frame_nrc_below_sharc"] = below[0] if below else None
        nrc["unit"] = "ms/frame"
        nrc["network"] = ("216-64x5-3, FP16 weights and activations, FP32 accumulation; tcgen05.mma with TMEM "
                          "accumulators for inference and training")
        nrc["pareto"] = []
        lr0 = gi_cache.LEARNING_RATE
        # the last two rows: the Adam rate the workload names (1e-3), at the operating point and at 65,536 samples
        for samples, steps, lr in ((16384, 4, lr0), (32768, 2, lr0), (65536, 2, lr0), (65536, 4, lr0), (65536, 8, lr0),
                                   (65536, 16, lr0), (32768, 4, 1e-3), (65536, 4, 1e-3)):
            r = gi_cache.run_comparison(t, SCENE, W_, H_, frames=args.nrc_frames, steps_per_frame=steps, curve=(),
                                        overlap=True, train_samples=samples, lr=lr)
            nrc["pareto"].append({"train_samples": samples, "train_steps_per_frame": steps, "lr": lr,
                                  "nrc_ms_per_frame": r["nrc_ms_per_frame"], "sharc_ms_per_frame": r["sharc_ms_per_frame"],
                                  "rel_mse_nrc": round(r["rel_mse_nrc"], 4), "rel_mse_sharc": round(r["rel_mse_sharc"], 4)})
        # the operating point with each query after its cache's update (no overlap)
        r = gi_cache.run_comparison(t, SCENE, W_, H_, frames=args.nrc_frames, steps_per_frame=4, curve=(),
                                    train_samples=32768)
        nrc["serial"] = {"train_samples": 32768, "train_steps_per_frame": 4, "nrc_ms_per_frame": r["nrc_ms_per_frame"],
                         "sharc_ms_per_frame": r["sharc_ms_per_frame"], "rel_mse_nrc": round(r["rel_mse_nrc"], 4),
                         "rel_mse_sharc": round(r["rel_mse_sharc"], 4)}
        kt = gi_cache.kernel_timing(t, SCENE, W_, H_)
        bf16_peak = _peaks_all().get("bf16_tflops")
        # the default form of a query on its own (four tile groups per CTA)
        q_tf = kt["tcgen05_four_groups"]["query_tflops"]
        kt["roofline_query"] = {"bound": "tensor", "achieved": q_tf, "peak": bf16_peak, "kernel": "infer_tc_kernel<4>",
                                "unit": "TFLOP/s", "peak_kind": "measured cuBLAS bf16 burst",
                                "frac": round(q_tf / bf16_peak, 4) if bf16_peak else None}
        nrc["kernels"] = kt

    # ReSTIR GI temporal pass on this world's frames (before the batch replaces world slot 0)
    restir = None
    if not args.no_restir:
        t.set_launch_config(variant=cfg.variant)
        restir = restir_section(t, scene, W_, H_, dev, (gdm, gnm, gaa, hits, gi))

    # many views over several worlds in one call replayed from a CUDA graph (autotuned kernel form)
    batched = None
    if not args.no_batched:
        from arcadia_gb300.batch import BENCH_SCENES, Batch

        b = Batch(t, BENCH_SCENES, 16)
        best, _ = t.autotune_views_dev(b.table, frames=2)
        n_gi_b = torch.zeros(1, dtype=torch.int64, device=dev)
        b.trace(n_gi_b.data_ptr(), use_graph=True)  # capture + first replay
        t.synchronize()
        b_ms = []
        for i in range(5):
            b.set_frame(1 + i)
            b.trace(n_gi_b.data_ptr(), use_graph=True)
            t.synchronize()
            b_ms.append(_graph_ms(t))
        n_gi_last = int(n_gi_b.item())
        batched = {"value": round((b.pixels + n_gi_last) / (statistics.mean(b_ms) * 1e-3) / 1e6, 3), "unit": UNIT,
                   "views": len(b.views), "scenes": BENCH_SCENES, "pixels_per_frame": b.pixels,
                   "gi_rays_last_frame": n_gi_last, "ms_per_frame": round(statistics.mean(b_ms), 3),
                   "cuda_graph": True, "launches_per_frame": 1,
                   "launch": {"kernel": "persistent" if best.variant == 1 else "plain",
                              "block_threads": best.block_threads, "reg_blocks": best.reg_blocks,
                              "refill_threshold": best.refill_threshold, "tile": [best.tile_w, best.tile_h]}}
    t.close()

    # full pipeline on the 4096^3 sparse world: in-place edits (1 % of the leaf bricks per frame), 4K
    # primary + GI, NRC training + query at the secondary hits, along a 300-frame camera path
    c5 = None
    if not args.no_c5:
        from arcadia_gb300.pipeline import FullPipeline

        sc5 = L.SCENES["c5_4096"]
        r5, n5, b5, _ = native.build_world(sc5)
        t5 = native.Tracer(local)
        t5.upload_world(sc5.grid, r5, n5, b5, pal, node_headroom=1 << 25, brick_headroom=1 << 22)
        p5 = FullPipeline(t5, sc5, args.c5_width, args.c5_height, n_bricks=len(b5), n_frames=args.c5_frames,
                          compare_every=30)
        c5 = p5.run(warmup=3)
        c5.update({"workload": "4096^3 sparse world (16^3 chunks: heightfield at 20-35 % of the height, caves in a "
                               "48-voxel band), edits + primary + GI + NRC per frame, camera path",
                   "scene": "c5_4096", "world_nodes": len(n5), "world_bricks": len(b5),
                   "quality": "high_quality preset (LOD on)", "unit_trace": "Mrays/s"})
        t5.close()
        del r5, n5, b5
    clk = clocks.stop() if clocks else None
    l2_gbs = _l2_copy_gbs(dev) if not args.frame_only else None  # untimed, after every timed section

    if rank != 0:
        return
    threads = os.cpu_count() or 1
    cpu = None
    bpp = None
    if not args.no_cpu_baseline:
        v, frames, dt, world, cam = cpu_leg(SCENE, args.cpu_seconds, threads, reference_query=True, frame=args.warmup)
        cpu = {"value": round(v, 3), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{frames} full frame(s) ({WIDTH}x{HEIGHT} primary + GI) in {dt:.1f} s through the C "
                         "restatement of WorldMap::raycast_meters -> raycast_chunk_tree",
               "build": "gcc -O3 -ffp-contract=off -fopenmp (portable flags: the same build on x86-64 and aarch64)"}
        # the same query on one core, and the line-for-line WGSL transcription on all cores and on one
        v1, f1, d1 = cpu_leg(SCENE, args.cpu_seconds / 2, 1, reference_query=True, frame=args.warmup)[:3]
        cpu["single_core"] = {"value": round(v1, 3), "unit": UNIT, "cores": 1, "sample": f"{f1} frame(s) in {d1:.1f} s"}
        vw, fw, dw = cpu_leg(SCENE, args.cpu_seconds / 2, threads, reference_query=False, frame=args.warmup)[:3]
        vw1, fw1, dw1 = cpu_leg(SCENE, args.cpu_seconds / 2, 1, reference_query=False, frame=args.warmup)[:3]
        cpu["wgsl_transcription"] = {
            "value": round(vw, 3), "unit": UNIT, "cores": threads, "sample": f"{fw} frame(s) in {dw:.1f} s",
            "single_core": round(vw1, 3),
            "what": "the oracle's line-for-line C transcription of trace_world_64tree_from (traversal64.wgsl:226-556) "
                    "and the primary / GI passes, on the same frames"}
        bpp = bytes_per_pixel(world, cam, threads)
    peak, peak_kind = _peaks()
    avg_ms = total_ms / args.steps if ws == 1 else statistics.mean(ms)
    roofline = None
    if bpp is not None:
        achieved = bpp * npx / (statistics.mean(ms) * 1e-3) / 1e9
        traffic = _profile_traffic("frame_persistent_kernel" if cfg.variant == 1 else "frame_plain_kernel")
        roofline = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": traffic, "peak_kind": peak_kind,
                    "algorithmic_bytes_per_pixel": round(bpp, 2)}
        if l2_gbs:
            roofline["l2"] = {"peak": round(l2_gbs, 1), "frac": round(achieved / l2_gbs, 4),
                              "peak_kind": "measured by this run: 50 copies of 32 MiB resident in L2, one CUDA graph"}
    # row bands of a device frame (arc_set_frame_bands; the library's rule: default 4, at most one per
    # 64 rows, one launch for the persistent kernel and the frame-wide variants)
    bands = 1
    if cfg.variant == 0 and not (cfg.features & (4 | 8 | 16)):
        bands = max(1, min(args.frame_bands if args.frame_bands else 4, H_ // 64))
    line = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(avg_ms, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+u32", "data": "synthetic (seeded heightfield + caves)",
        "config": {"workload": WORKLOAD, "scene": SCENE, "width": WIDTH, "height": HEIGHT,
                   "parallelism": f"replicas x{ws}", "l2": "flushed before every timed frame (256 MiB write)",
                   "kernel": "persistent" if cfg.variant == 1 else "plain",
                   "autotuned": tuned_ms is not None,
                   "launch": {"block_threads": cfg.block_threads, "blocks_per_sm": cfg.blocks_per_sm,
                              "tile": [cfg.tile_w, cfg.tile_h], "refill_threshold": cfg.refill_threshold,
                              "reg_blocks": cfg.reg_blocks, "order": "morton" if cfg.order else "row-major",
                              "features": cfg.features, "row_bands": bands}},
        "default_config": {"value": round(plain_value, 3), "unit": UNIT, "ms_per_step": round(statistics.mean(plain_ms), 4),
                           "frames": np_frames},
        "e2e": {"value": round(e2e_value, 3), "unit": UNIT, "h2d_bytes_per_step": 480,
                "d2h_bytes_per_step": npx * 60 + 8 + 16},
        # per timed frame: the persistent kernel, or the plain kernel's primary instance + the GI pass
        # (one kernel, or four with the GI rays sorted over the frame: keys, scan, scatter, trace),
        # once per concurrent row band
        "gpu_launches": args.steps * (1 if cfg.variant == 1 else (5 if cfg.features & 4 else 2 * bands)),
        "roofline": roofline,
        "cpu_baseline": cpu,
        "nrc": nrc,
        "batched": batched,
        "restir_gi_temporal": restir,
        "c5": c5,
        "clocks": clk,
    }
    if nrc is not None:
        # the cache comparison at its operating point in both modes, last so that a tail of the line keeps it
        ov, se = nrc, nrc["serial"]
        line["c4"] = {
            "workload": "NRC vs SHARC at the GI hits of 1920x1080 frames of the 1024^3 caves world, 300 static frames",
            "operating_point": {"train_samples": 32768, "adam_steps_per_frame": 4, "lr": ov["lr"]},
            "overlapped": {"nrc_ms": ov["nrc_ms_per_frame"], "sharc_ms": ov["sharc_ms_per_frame"],
                           "rel_mse_nrc": round(ov["rel_mse_nrc"], 4), "rel_mse_sharc": round(ov["rel_mse_sharc"], 4)},
            "serial": {"nrc_ms": se["nrc_ms_per_frame"], "sharc_ms": se["sharc_ms_per_frame"],
                       "rel_mse_nrc": se["rel_mse_nrc"], "rel_mse_sharc": se["rel_mse_sharc"]},
            "nrc_faster_and_better_in_both": bool(ov["nrc_ms_per_frame"] < ov["sharc_ms_per_frame"]
                                                  and se["nrc_ms_per_frame"] < se["sharc_ms_per_frame"]
                                                  and ov["rel_mse_nrc"] <= ov["rel_mse_sharc"]
                                                  and se["rel_mse_nrc"] <= se["rel_mse_sharc"]),
            "reference_spp": 4096,
            "static_curve": [[c["frame"], round(c["rel_mse_nrc"], 3), round(c["rel_mse_sharc"], 3)] for c in ov["convergence"]],
            "moving_c5_path": ([[c["frame"], c["rel_mse_nrc"], c["rel_mse_sharc"]] for c in c5["cache_scores_along_path"]]
                               if c5 and "cache_scores_along_path" in c5 else None),
            "c5_cache_ms_4k": ({"nrc": c5["median_ms"]["nrc_ms"], "sharc": c5.get("sharc_ms_median")} if c5 else None)}
    print(json.dumps(line), flush=True)


def main():
    args = _args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
