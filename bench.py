#!/usr/bin/env python
"""Benchmark of the GB300 ray-query path on the procedural-asteroid workload.

One step = one render request (2048^2, 1 spp: primary + sun shadow ray) and one LiDAR scan
(1024^2 beams, range + triangle id) on the device-resident BVH of the 2M-triangle asteroid.
`value` is Mrays/s (primary + shadow + LiDAR rays) with inputs resident on the device and
outputs left in device memory, timed with CUDA events on the library's stream, an L2 flush
(256 MiB write) between steps outside the timed events.  `e2e` is the same workload through the
public `crt` API (BodyFixedGroup.render / lidar_scan) returning numpy arrays.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

--impl reference times the CPU oracle (FP64 C restatement of the reference path, all host cores).
Multi-GPU (torchrun): every rank runs the same workload on its own GPU (replicas; weak scaling).
"""
import argparse
import datetime
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(REPO, "ceres-raytracer_gb300")
for _p in (PKG, REPO):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mrays/s and p50/p99 request latency, batched/served vs per-call GPU, one GB300"
UNIT = "Mrays/s"
# algorithmic bytes per unit of work: an 8-wide node's planes as bytes (80 B), a triangle (48 B), a ray
# (32 B) and its hit (16 B); the node as stored is 128 B (planes as halves: NODE_BYTES_STORED)
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES = 80, 48, 32, 16
NODE_BYTES_STORED = 128


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--faces", type=int, default=2_000_000)
    ap.add_argument("--res", type=int, default=2048)
    ap.add_argument("--lidar", type=int, default=1024)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--served-seconds", type=float, default=60.0,
                    help="length of the Poisson request stream (the configuration's 60 s)")
    ap.add_argument("--served-rate", type=float, default=200.0)
    ap.add_argument("--served-lanes", type=int, default=4)
    ap.add_argument("--served-wave-paths", type=int, default=1 << 22)
    ap.add_argument("--served-budget-mib", type=int, default=4096)
    ap.add_argument("--no-srp", action="store_true")
    ap.add_argument("--no-cornell", action="store_true")
    ap.add_argument("--srp-attitudes", type=int, default=256)
    ap.add_argument("--probe", type=int, default=0,
                    help="profiling aid (the commands of the ncu summaries under profiles/ run it): only run "
                         "the --probe-kind workload this many times")
    ap.add_argument("--probe-kind", default="closest", choices=["closest", "batched", "srp", "step"],
                    help="closest: crt_trace_closest on the 2048^2 primary rays; batched: one crt_batch of the "
                         "64-request mix; srp: 8 attitudes x 4096^2 rays x 2 bounces with per-facet flux; step: "
                         "the bench's step (L2 flush, render, LiDAR scan) with device outputs")
    return ap.parse_args()


def probe(args):
    """Profiling aid used by the commands of the ncu summaries under profiles/: the 2M-triangle asteroid
    resident (about 330 MB with the rays, larger than L2) and `--probe` launches of crt_trace_closest on
    the 2048^2 primary camera rays (or of the batched mix / SRP batch, --probe-kind)."""
    import torch
    from crt_gb300 import build, lib, workloads
    build.build()
    ents = workloads.asteroid_entities(args.faces)
    cfg = workloads.asteroid_config(args.res, args.lidar)
    ctx = lib.Context(0)
    if args.probe_kind == "srp":
        s = workloads.srp_config(n_att=8)
        scs = ctx.scene(s["entities"])
        for _ in range(args.probe):
            f, t, fp = scs.srp(s["sun"], s["quaternions"], s["grid"], num_bounces=s["num_bounces"], facet_power=True)
        print(json.dumps({"probe_launches": args.probe, "kind": "srp", "force0": f[0].tolist()}))
        scs.close()
        ctx.close()
        return
    if args.probe_kind == "batched":
        ctx.set_tuning(collapse_tri_cost=0.5)   # as the bench's batched measurement builds its scene
    sc = ctx.scene(ents)
    ctx.set_tuning()
    if args.probe_kind == "step":
        lid = cfg["lidar"]
        rgba = torch.empty((args.res, args.res, 4), dtype=torch.uint8, device="cuda")
        rng = torch.empty((lid["ny"], lid["nx"]), dtype=torch.float64, device="cuda")
        prim = torch.empty((lid["ny"], lid["nx"]), dtype=torch.int32, device="cuda")
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        for _ in range(args.probe):
            flush.zero_()
            sc.render(cfg["camera"], cfg["lights"], 1, 1, 1.0, cfg["bounces"], want_radiance=False, out_rgba=rgba)
            sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"],
                          out_range=rng, out_prim=prim)
        ctx.synchronize()
        print(json.dumps({"probe_launches": args.probe, "kind": "step"}))
        ctx.close()
        return
    if args.probe_kind == "batched":
        reqs = []
        for q in workloads.batched_config(seed=1):
            if q["kind"] == "render":
                reqs.append(dict(kind="render", scene=sc, camera=q["camera"], lights=q["lights"],
                                 min_samples=q["spp"], max_samples=q["spp"], noise_threshold=0.0,
                                 num_bounces=q["bounces"], seed=1, request=q["request"]))
            else:
                reqs.append(dict(kind="lidar", scene=sc, position=q["position"], rotation=q["rotation"], nx=q["nx"],
                                 ny=q["ny"], half_x=q["half_x"], half_y=q["half_y"]))
        for _ in range(args.probe):
            _, st = ctx.batch(reqs)
        print(json.dumps({"probe_launches": args.probe, "kind": "batched", "waves": st["waves"]}))
        ctx.close()
        return
    rays = torch.from_numpy(scenes_camera_rays(cfg["camera"])).cuda()
    hits = torch.empty((rays.shape[0], 4), dtype=torch.float32, device="cuda")
    for _ in range(args.probe):
        sc.trace_closest(rays, out=hits)
    ctx.synchronize()
    miss = (hits[:, 3].view(torch.int32) == -1).float().mean().item()
    print(json.dumps({"probe_launches": args.probe, "rays": int(rays.shape[0]), "miss_fraction": miss}))
    ctx.close()


def dist_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_throughput(ms, rays_per_step, world, device):
    """Whole-job throughput of `world` replicas (one per GPU, no data-path collective): the step
    time is the maximum over ranks, the rays are every rank's.  Returns (max ms, Mrays/s)."""
    if world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    return ms, rays_per_step * world / (ms / 1e3) / 1e6


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q / 100.0
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region: sampling starts before it (the
    tool's start-up can hold this process's CUDA driver calls for tens of milliseconds) and only the
    samples stamped between start() returning and stop() are summarised."""
    FIELDS = "timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active," \
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap,utilization.gpu"

    def __init__(self, device, settle_s=1.5):
        self.device = device
        self.settle_s = settle_s
        self.proc = None
        self.path = None
        self.t0 = self.t1 = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200", "-f", self.path],
                                         stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t = time.perf_counter()
        while time.perf_counter() - t < self.settle_s and self.proc.poll() is None:
            time.sleep(0.02)
        self.t0 = time.time()

    def stop(self):
        if not self.proc:
            return None
        self.t1 = time.time()
        time.sleep(0.25)   # the sample that covers the end of the window
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 10:
                    rows.append(parts)
        os.unlink(self.path)

        def stamp(r):
            try:
                return datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except ValueError:
                return None
        inside = [r for r in rows if stamp(r) is not None and self.t0 - 0.2 <= stamp(r) <= self.t1 + 0.2]
        rows = inside or rows
        if not rows:
            return None
        num = lambda x: x.replace(".", "").isdigit()
        sm = [float(r[2]) for r in rows if num(r[2])]
        mx = [float(r[3]) for r in rows if num(r[3])]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[6 + k].lower().startswith("active")})
        util = [float(r[10]) for r in rows if len(r) > 10 and num(r[10])]
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window_s": round(self.t1 - self.t0, 3),
                "gpu_busy_pct": round(statistics.mean(util), 1) if util else None}


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


PROFILE = os.path.join("profiles", "trace_closest_asteroid2M.md")


def profiled_counters():
    """Per-launch counters of the primary trace kernel on the bench's rays from the committed ncu
    summary (its `key = value` lines): dram_bytes, lts_bytes, warp_inst, issue_active_pct, rays.  ncu
    cannot run inside the timed bench, so these are the capture's figures for the same kernel, BVH and
    rays; bench.py divides them by the kernel time it measures."""
    path = os.path.join(REPO, PROFILE)
    out = {}
    if not os.path.exists(path):
        return out
    for line in open(path):
        line = line.strip().strip("`")
        if line.startswith("counter ") and "=" in line:
            k, v = line[len("counter "):].split("=", 1)
            try:
                out[k.strip()] = float(v.split()[0])
            except (IndexError, ValueError):
                pass
    return out


def read_peaks(ctx, dev):
    """Streaming-read bandwidth measured here with the library's read kernel (crt_measure_read, at
    least 1 GiB read per launch): the best of 64, 80 and 96 MiB buffers, which stay in the L2 cache
    after the first pass (the plateau of a 4 MiB .. 4 GiB sweep on this GPU; 128 MiB no longer fits),
    and a 4 GiB buffer read from HBM.  GB/s."""
    import torch
    l2 = 0.0
    for mib in (64, 80, 96):
        b = torch.ones(mib << 20, dtype=torch.uint8, device=dev)
        l2 = max(l2, b.numel() / ctx.measure_read(b, reps=5) / 1e6)
        del b
    big = torch.ones(4 << 30, dtype=torch.uint8, device=dev)
    ms_hbm = ctx.measure_read(big, reps=5)
    out = {"l2_read_gbs": round(l2, 1), "hbm_read_gbs": round(big.numel() / ms_hbm / 1e6, 1)}
    del big
    torch.cuda.empty_cache()
    return out


# ------------------------------------------------------------------ CPU (oracle port) timing
def cpu_measure(ents, cfg, budget_s):
    """Time the CPU oracle on the step's workload with all host threads; returns (Mrays/s, detail)."""
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o = oracle.Scene(ents, nthreads=threads)
    build_s = time.perf_counter() - t0
    cam, lights = cfg["camera"], cfg["lights"]
    W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
    from crt_gb300 import workloads
    lid_rays = workloads.lidar_grid_rays(cfg["lidar"])
    # probe: 16 rows of the image + 1/64 of the beams, then scale the sample to ~budget_s
    rows = 16
    t = time.perf_counter()
    o.render(cam, lights, 1, 1, 1.0, cfg["bounces"], row0=0, row1=rows)
    o.trace_closest(lid_rays[: len(lid_rays) // 64])
    probe = time.perf_counter() - t
    frac = min(1.0, max(rows / H, (budget_s / max(probe, 1e-3)) * rows / H))
    rows = max(16, min(H, int(H * frac)))
    nl = max(1024, int(len(lid_rays) * rows / H))
    _, ids, _, _ = o.passes(cam, 0, rows)
    shadow = int((ids > 0).sum()) * len(lights)
    reps, el = 0, 0.0
    while reps == 0 or (el < 0.5 * budget_s and reps < 8):
        t = time.perf_counter()
        o.render(cam, lights, 1, 1, 1.0, cfg["bounces"], row0=0, row1=rows)
        o.trace_closest(lid_rays[:nl])
        el += time.perf_counter() - t
        reps += 1
    rays = (rows * W + shadow + nl) * reps
    return rays / el / 1e6, dict(cores=threads, seconds=el, rays=rays, build_s=build_s,
                                 sample=f"{reps} x (rows 0..{rows} of the {W}x{H} render, primary + shadow, and {nl} "
                                        f"of {len(lid_rays)} LiDAR beams); BVH built once (untimed)")


def step_workload(args):
    """Name of the asteroid step at the given sizes (both arms report the same name)."""
    faces = "2M" if args.faces == 2_000_000 else str(args.faces)
    return (f"asteroid-{faces}: render {args.res}^2 1 spp (primary + sun shadow) + LiDAR {args.lidar}^2 "
            "(range + triangle id)")


# ------------------------------------------------------------------ reference arm
def reference_arm(args):
    rank, world, _ = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
        if rank != 0:
            dist.barrier()
            return
    from crt_gb300 import build, workloads
    build.build()
    ents = workloads.asteroid_entities(args.faces)
    cfg = workloads.asteroid_config(args.res, args.lidar)
    # one bounded sample (about --cpu-seconds of work) of the step's workload; the BVH build is not timed
    mr, det = cpu_measure(ents, cfg, args.cpu_seconds)
    line = {"impl": "reference", "metric": METRIC, "value": round(mr, 3), "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": step_workload(args), "path": "CPU oracle port, all host threads, bounded sample",
                       "triangles": args.faces},
            "cpu_baseline": {"value": round(mr, 3), "unit": UNIT, "cores": det["cores"], "kind": "port",
                             "sample": det["sample"]},
            "e2e": {"value": round(mr, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    rays_step = args.res * args.res * 2 + args.lidar * args.lidar
    line["ms_per_step"] = round(rays_step / (mr * 1e6) * 1e3, 3)
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ GPU arm
def gpu_arm(args):
    import torch
    from crt_gb300 import build, lib, scenes, workloads
    build.build()
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://", device_id=torch.device("cuda", local))

    ents = workloads.asteroid_entities(args.faces)
    cfg = workloads.asteroid_config(args.res, args.lidar)
    cam, lights, lid = cfg["camera"], cfg["lights"], cfg["lidar"]
    ctx = lib.Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    sc = ctx.scene(ents)
    st = sc.stats()
    W = H = args.res
    dev = torch.device("cuda", local)
    rgba = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    rng_out = torch.empty((lid["ny"], lid["nx"]), dtype=torch.float64, device=dev)
    prim_out = torch.empty((lid["ny"], lid["nx"]), dtype=torch.int32, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def render():
        sc.render(cam, lights, 1, 1, 1.0, cfg["bounces"], want_radiance=False, out_rgba=rgba)

    def scan():
        sc.lidar_grid(lid["position"], lid["rotation"], lid["nx"], lid["ny"], lid["half_x"], lid["half_y"],
                      out_range=rng_out, out_prim=prim_out)

    # rays per step: primary + shadow (one per primary hit, one light) + LiDAR beams
    with torch.cuda.stream(stream):
        ctx.reset_counters()
        ctx.set_counting(True)
        render()
        c_render = ctx.counters()
        ctx.reset_counters()
        scan()
        c_scan = ctx.counters()
        ctx.set_counting(False)
        ctx.synchronize()
    rays_step = int(c_render["answered"] + c_scan["answered"])

    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            flush.zero_()
            render()
            scan()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ctx.reset_counters()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(args.steps):
            flush.zero_()
            a, b, c = ev[k]
            a.record(stream)
            render()
            b.record(stream)
            scan()
            c.record(stream)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t_wall
    launches = ctx.counters()["launches"]
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    # the K-step window is short (tens of ms); clocks over ~2 s of the same step, right after it
    sustained = ClockSampler(local)
    sustained.start()
    t_s = time.perf_counter()
    with torch.cuda.stream(stream):
        while time.perf_counter() - t_s < 2.0:
            for _ in range(20):
                flush.zero_()
                render()
                scan()
            torch.cuda.synchronize()
    clk_sustained = sustained.stop()
    lat_render = [a.elapsed_time(b) for a, b, c in ev]
    lat_lidar = [b.elapsed_time(c) for a, b, c in ev]
    step_ms = [a.elapsed_time(c) for a, b, c in ev]
    ms, value = replica_throughput(float(np.mean(step_ms)), rays_step, world, dev)

    # ---- roofline of the dominant kernel: closest-hit traversal of the primary camera rays
    rays64 = scenes_camera_rays(cam)
    rays_dev = torch.from_numpy(rays64).to(dev)
    hits_dev = torch.empty((rays64.shape[0], 4), dtype=torch.float32, device=dev)
    with torch.cuda.stream(stream):
        ctx.reset_counters()
        ctx.set_counting(True)
        sc.trace_closest(rays_dev, out=hits_dev)
        cnt = ctx.counters()
        ctx.set_counting(False)
        times = []
        for _ in range(max(5, min(20, args.steps))):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            sc.trace_closest(rays_dev, out=hits_dev)
            b.record(stream)
            times.append((a, b))
    torch.cuda.synchronize()
    t_kernel = float(np.mean([a.elapsed_time(b) for a, b in times])) / 1e3
    nodes_ray = cnt["nodes"] / cnt["rays"]
    tris_ray = cnt["tris"] / cnt["rays"]
    b_ray = NODE_BYTES * nodes_ray + TRI_BYTES * tris_ray + RAY_BYTES + HIT_BYTES
    achieved = b_ray * cnt["rays"] / t_kernel / 1e9
    peak, peak_kind = measured_peak()
    pk = read_peaks(ctx, dev)
    prof = profiled_counters()
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 4), "traffic": prof.get("dram_bytes"), "peak_source": peak_kind,
            "kernel": "k_trace<closest> on 2048^2 primary camera rays in 8x4 tiles (crt_trace_closest)",
            "bytes_per_ray": round(b_ray, 1), "nodes_per_ray": round(nodes_ray, 2), "tris_per_ray": round(tris_ray, 2),
            "kernel_ms": round(t_kernel * 1e3, 3), "kernel_mrays_s": round(cnt["rays"] / t_kernel / 1e6, 1),
            "bytes_per_ray_stored": round(NODE_BYTES_STORED * nodes_ray + TRI_BYTES * tris_ray + RAY_BYTES + HIT_BYTES, 1),
            "frac_note": "algorithmic bytes (80 B per node: its planes as bytes, as the node is 128 B stored with "
                         "planes as halves; 48 B per triangle, 48 B ray + hit) over the measured HBM copy "
                         "bandwidth; most are served from L1 / L2, see dram_frac / l2_frac",
            "read_peaks_gbs": pk}
    if prof.get("dram_bytes") and prof.get("lts_bytes"):
        # the ncu capture's bytes for one launch of this kernel on these rays, over the time measured here
        dram_gbs = prof["dram_bytes"] / t_kernel / 1e9
        l2_gbs = prof["lts_bytes"] / t_kernel / 1e9
        roof.update(traffic_source="ncu capture of the same kernel, BVH and rays (" + PROFILE + ", counters "
                                   "dram__bytes_read.sum + dram__bytes_write.sum, lts__t_bytes.sum) over the "
                                   "kernel time measured in this run",
                    dram_gbs=round(dram_gbs, 1), dram_frac=round(dram_gbs / peak, 4),
                    l2_gbs=round(l2_gbs, 1), l2_frac=round(l2_gbs / pk["l2_read_gbs"], 4))
    if prof.get("warp_inst") and prof.get("rays"):
        roof.update(warp_inst_per_32_rays=round(prof["warp_inst"] / (prof["rays"] / 32.0), 1),
                    issue_active_pct=prof.get("issue_active_pct"),
                    binding="SM instruction issue (ncu issue-active % above; DRAM and L2 fractions low)")

    # ---- end to end through the public crt API (host numpy outputs), right after the step it repeats
    e2e = None
    if not args.no_e2e and rank == 0:
        e2e = e2e_measure(args, ents, cfg, rays_step)

    # ---- batched vs per-call on the config-3 request set
    batched = None
    if not args.no_batched and rank == 0:
        batched = batched_measure(ctx, ents, stream)

    srp = None
    if not args.no_srp and rank == 0:
        srp = srp_measure(args, ctx, stream)

    cornell = None
    if not args.no_cornell and rank == 0:
        cornell = cornell_measure(ctx, stream, cpu=not args.no_cpu)

    served = None
    if not args.no_served and rank == 0:
        served = served_measure(args, local)

    line = None
    if rank == 0:
        line = {"metric": METRIC, "value": round(value, 2), "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": round(ms, 4), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": step_workload(args), "path": "per-call GPU, resident BVH",
                           "triangles": st["n_tris"], "wide_nodes": st["n_nodes"], "bvh_depth": st["depth"],
                           "bvh_build_ms": round(st["build_ms"], 2), "rays_per_step": rays_step,
                           "l2": "256 MiB buffer written between steps (outside the timed events)",
                           "wall_s": round(wall, 3)},
                "latency_ms": {"render_p50": round(percentile(lat_render, 50), 3),
                               "render_p99": round(percentile(lat_render, 99), 3),
                               "lidar_p50": round(percentile(lat_lidar, 50), 3),
                               "lidar_p99": round(percentile(lat_lidar, 99), 3),
                               "step_p50": round(percentile(step_ms, 50), 3),
                               "step_max": round(max(step_ms), 3)},
                "roofline": roof, "gpu_launches": int(launches), "clocks": clk,
                "clocks_sustained": clk_sustained, "e2e": e2e, "batched": batched,
                "served": served, "srp": srp, "cornell": cornell}
        if world == 1 and not args.no_cpu:
            mr, det = cpu_measure(ents, cfg, args.cpu_seconds)
            line["cpu_baseline"] = {"value": round(mr, 3), "unit": UNIT, "cores": det["cores"], "kind": "port",
                                    "sample": det["sample"]}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()
    ctx.close()


def batched_measure(ctx, ents, stream, reps=1):
    """Config-3 workload on the resident asteroid: 64 requests (32 renders, 2 bounces, resolution
    128^2..2048^2, 1..64 spp; 32 LiDAR scans 64^2..1024^2) as per-call GPU requests (one library call
    each, in sequence) and as one crt_batch; device outputs in both cases.  Returns a dict."""
    import torch
    from crt_gb300 import workloads
    # a scene built for multi-bounce path tracing: smaller leaves (collapse triangle cost 0.5), which
    # incoherent bounce rays traverse faster; both arms below use it
    ctx.set_tuning(collapse_tri_cost=0.5)
    sc = ctx.scene(ents)
    ctx.set_tuning()
    reqs = workloads.batched_config(seed=1)
    dev = torch.device("cuda", torch.cuda.current_device())
    outs, breqs = [], []
    for q in reqs:
        if q["kind"] == "render":
            W, H = q["camera"]["resolution"]
            outs.append((torch.empty((H, W, 4), dtype=torch.uint8, device=dev), None))
            breqs.append(dict(kind="render", scene=sc, camera=q["camera"], lights=q["lights"], min_samples=q["spp"],
                              max_samples=q["spp"], noise_threshold=0.0, num_bounces=q["bounces"], seed=1,
                              request=q["request"]))
        else:
            outs.append((torch.empty((q["ny"], q["nx"]), dtype=torch.float64, device=dev),
                         torch.empty((q["ny"], q["nx"]), dtype=torch.int32, device=dev)))
            breqs.append(dict(kind="lidar", scene=sc, position=q["position"], rotation=q["rotation"], nx=q["nx"],
                              ny=q["ny"], half_x=q["half_x"], half_y=q["half_y"]))

    def per_call(events=None):
        for k, (q, o) in enumerate(zip(breqs, outs)):
            if events is not None:
                events[k][0].record(stream)
            if q["kind"] == "render":
                sc.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], 0.0, q["num_bounces"],
                          seed=q["seed"], request=q["request"], want_radiance=False, out_rgba=o[0])
            else:
                sc.lidar_grid(q["position"], q["rotation"], q["nx"], q["ny"], q["half_x"], q["half_y"],
                              out_range=o[0], out_prim=o[1])
            if events is not None:
                events[k][1].record(stream)

    from crt_gb300 import autotune
    with torch.cuda.stream(stream):
        # wave size and queue chunk picked by the autotuner on this request set (both paths use them)
        knobs, rep = autotune.tune(ctx, lambda: ctx.batch(breqs, outputs=outs), "batched-64", sc.stats()["n_tris"],
                                   grid={"queue_chunk": (1, 2), "wave_paths": (1 << 22, 1 << 23, 1 << 24),
                                         "use_graphs": (True,)}, use_cache=False)
        # rays actually traced (counting build), identical for both paths
        ctx.reset_counters()
        ctx.set_counting(True)
        ctx.batch(breqs, outputs=outs)
        rays = ctx.counters()["answered"]
        ctx.set_counting(False)
        ctx.batch(breqs, outputs=outs)      # warm-up (scratch sized, graph path exercised)
        per_call()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in breqs]
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        per_call(ev)
        t1.record(stream)
        b0 = torch.cuda.Event(enable_timing=True)
        b1 = torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        for _ in range(reps):
            _, st = ctx.batch(breqs, outputs=outs)
        b1.record(stream)
    torch.cuda.synchronize()
    pc_ms = t0.elapsed_time(t1)
    bt_ms = b0.elapsed_time(b1) / reps
    lat = [a.elapsed_time(b) for a, b in ev]
    # per-call latency of a request submitted with the whole set: its completion time in the sequence
    done = np.cumsum(lat)
    mixed = mixed_measure(ctx, breqs, outs, stream)
    sc.close()
    return {"mixed": mixed,
            "workload": "64 requests on the 2M asteroid: 32 renders (128^2..2048^2, 1..64 spp, 2 bounces, "
                        "sun light) + 32 LiDAR scans (64^2..1024^2); scene built with collapse_tri_cost 0.5",
            "rays": int(rays), "per_call_mrays_s": round(rays / (pc_ms / 1e3) / 1e6, 1),
            "batched_mrays_s": round(rays / (bt_ms / 1e3) / 1e6, 1), "speedup": round(pc_ms / bt_ms, 3),
            "per_call_ms": round(pc_ms, 2), "batched_ms": round(bt_ms, 2), "waves": st["waves"],
            "per_call_request_ms_p50": round(percentile(lat, 50), 3),
            "per_call_request_ms_p99": round(percentile(lat, 99), 3),
            "per_call_completion_ms_p50": round(percentile(list(done), 50), 2),
            "per_call_completion_ms_p99": round(percentile(list(done), 99), 2),
            "batched_completion_ms": round(bt_ms, 2),
            "tuning": knobs, "tuning_trials_ms": [[t[0]["queue_chunk"], t[0]["wave_paths"], round(t[1], 2)]
                                                  for t in rep["trials"]]}


def mixed_measure(ctx, breqs, outs, stream):
    """The 64 requests above plus 16 SRP queries on the spacecraft (grid 512^2..2048^2, 1..4 attitudes,
    2 specular bounces) as per-call GPU requests (crt_render / crt_lidar_grid / crt_srp, in sequence)
    and as one crt_batch_mixed, whose waves carry the SRP sun rays in their primary traces; device
    outputs in both cases."""
    import torch
    from crt_gb300 import scenes
    craft = ctx.scene(scenes.spacecraft())
    rng = np.random.Generator(np.random.PCG64(11))
    dev = torch.device("cuda", torch.cuda.current_device())
    sreqs, souts = [], []
    for k in range(16):
        q = scenes.random_quaternions(int(rng.integers(1, 5)), seed=500 + k)
        sreqs.append(dict(kind="srp", scene=craft, sun_dir=[1.0, 0.0, 0.0], quaternions=q,
                          grid=int(rng.choice([512, 1024, 2048])), num_bounces=2))
        souts.append((torch.empty((len(q), 3), dtype=torch.float64, device=dev),
                      torch.empty((len(q), 3), dtype=torch.float64, device=dev)))
    mreqs, mouts = list(breqs), list(outs)
    for k, (q, o) in enumerate(zip(sreqs, souts)):   # spread the SRP queries through the request list
        at = (k * len(mreqs)) // len(sreqs) + k
        mreqs.insert(at, q)
        mouts.insert(at, o)
    sc = next(q["scene"] for q in breqs)

    def per_call():
        for q, o in zip(mreqs, mouts):
            if q["kind"] == "render":
                sc.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], 0.0, q["num_bounces"],
                          seed=q["seed"], request=q["request"], want_radiance=False, out_rgba=o[0])
            elif q["kind"] == "lidar":
                sc.lidar_grid(q["position"], q["rotation"], q["nx"], q["ny"], q["half_x"], q["half_y"],
                              out_range=o[0], out_prim=o[1])
            else:
                craft.srp_into(q["sun_dir"], q["quaternions"], q["grid"], o[0], o[1], num_bounces=q["num_bounces"])

    with torch.cuda.stream(stream):
        ctx.reset_counters()
        ctx.set_counting(True)
        _, st = ctx.batch(mreqs, outputs=mouts)
        rays = ctx.counters()["answered"]
        ctx.set_counting(False)
        ctx.batch(mreqs, outputs=mouts)      # warm-up
        per_call()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record(stream)
        per_call()
        ev[1].record(stream)
        ev[2].record(stream)
        _, st = ctx.batch(mreqs, outputs=mouts)
        ev[3].record(stream)
    torch.cuda.synchronize()
    pc_ms, bt_ms = ev[0].elapsed_time(ev[1]), ev[2].elapsed_time(ev[3])
    craft.close()
    return {"workload": "the 64 requests + 16 SRP queries on the spacecraft (48,728 triangles; grid 512^2..2048^2, "
                        "1..4 attitudes, 2 bounces; 46 attitudes), one crt_batch_mixed vs per-call",
            "rays": int(rays), "per_call_ms": round(pc_ms, 2), "batched_ms": round(bt_ms, 2),
            "per_call_mrays_s": round(rays / (pc_ms / 1e3) / 1e6, 1),
            "batched_mrays_s": round(rays / (bt_ms / 1e3) / 1e6, 1), "speedup": round(pc_ms / bt_ms, 3),
            "waves": st["waves"]}


def served_measure(args, device):
    """Served stream: Poisson arrivals (200 req/s by default) over four resident asteroids (100k, 500k,
    2M, 8M triangles), 50 % renders / 30 % LiDAR / 20 % SRP, host (numpy) outputs as a user gets them.

    open loop   requests are submitted at their arrival times; latency = completion - arrival.  The
                server (continuous batching over `lanes` concurrent lanes) and the per-call drop-in
                (one blocking library call per request, in arrival order) serve the same stream.
    closed loop every request is submitted at once: makespan throughput of both paths.
    Rays come from a counting pass over the same requests (identical for both paths)."""
    import threading
    from crt_gb300 import lib, workloads
    stream = workloads.served_stream(args.served_rate, args.served_seconds)
    srv = lib.Server(device, lanes=args.served_lanes, lane_budget_bytes=args.served_budget_mib << 20, max_batch=256,
                     wave_paths=args.served_wave_paths)
    t0 = time.perf_counter()
    ents = workloads.served_bodies()
    t_gen = time.perf_counter() - t0
    bodies = [srv.scene(e) for e in ents]
    items = [(t, dict(q, scene=bodies[q["body"]])) for t, q in stream]

    def call(q):
        sc = q["scene"]
        if q["kind"] == "render":
            sc.render(q["camera"], q["lights"], q["min_samples"], q["max_samples"], 0.0, q["num_bounces"],
                      seed=q["seed"], request=q["request"], want_radiance=False)
        elif q["kind"] == "lidar":
            sc.lidar_grid(q["position"], q["rotation"], q["nx"], q["ny"], q["half_x"], q["half_y"])
        else:
            sc.srp(q["sun_dir"], q["quaternions"], q["grid"], num_bounces=q["num_bounces"])

    # rays of the whole stream (counting build, context of the scenes)
    srv.ctx.reset_counters()
    srv.ctx.set_counting(True)
    for _, q in items:
        call(q)
    rays = int(srv.ctx.counters()["answered"])
    srv.ctx.set_counting(False)
    for _, q in items[:64]:                       # warm-up of both paths
        call(q)
    for tk in [srv.submit(q) for _, q in items[:64]]:
        srv.wait(tk)

    def served(open_loop):
        tickets = [None] * len(items)
        start = time.perf_counter() + 0.05

        def submitter():
            for i, (t, q) in enumerate(items):
                if open_loop:
                    d = start + t - time.perf_counter()
                    if d > 0:
                        time.sleep(d)
                tickets[i] = srv.submit(q)

        s0 = srv.stats()
        th = threading.Thread(target=submitter)
        th.start()
        res = []
        for i in range(len(items)):
            while tickets[i] is None:
                time.sleep(0.0002)
            res.append(srv.wait(tickets[i])[0])
        th.join()
        s1 = srv.stats()
        lat = [1e3 * (r["end_s"] - r["submit_s"]) for r in res]
        span = max(r["end_s"] for r in res) - min(r["submit_s"] for r in res)
        return lat, span, (s1["batches"] - s0["batches"]), res

    def per_call(open_loop):
        lat = []
        start = time.perf_counter() + 0.05
        t_first = None
        for t, q in items:
            arrive = start + t if open_loop else None
            if open_loop:
                d = arrive - time.perf_counter()
                if d > 0:
                    time.sleep(d)
            a = time.perf_counter()
            t_first = t_first or a
            call(q)
            e = time.perf_counter()
            lat.append(1e3 * (e - (arrive if open_loop else t_first)))
        return lat, time.perf_counter() - t_first

    small = [q.get("size", 0) <= 1024 for _, q in items]
    kinds = [q["kind"] for _, q in items]

    def summary(lat, span):
        ls = [x for x, f in zip(lat, small) if f]
        by_kind = {}
        for k in ("render", "lidar", "srp"):
            lk = [x for x, f, kk in zip(lat, small, kinds) if f and kk == k]
            if lk:
                by_kind[k] = round(percentile(lk, 99), 2)
        return {"mrays_s": round(rays / span / 1e6, 1), "span_s": round(span, 3),
                "p50_ms": round(percentile(lat, 50), 2), "p99_ms": round(percentile(lat, 99), 2),
                "p50_ms_le1024": round(percentile(ls, 50), 2), "p99_ms_le1024": round(percentile(ls, 99), 2),
                "p99_ms_le1024_by_kind": by_kind}

    def clocked(fn, *a):
        cs = ClockSampler(device)
        cs.start()
        r = fn(*a)
        return r, cs.stop()

    (lat_s, span_s, nb_s, res_s), clk_s = clocked(served, True)
    (lat_p, span_p), clk_p = clocked(per_call, True)
    (clat_s, cspan_s, cnb_s, _), cclk_s = clocked(served, False)
    (clat_p, cspan_p), cclk_p = clocked(per_call, False)
    out = {"workload": "served stream: Poisson %.0f req/s for %.0f s (%d requests) over 4 resident asteroids "
                       "(100k/500k/2M/8M triangles); 50%% renders 128^2..2048^2 x 1..16 spp (primary + sun "
                       "shadow), 30%% LiDAR 64^2..1024^2, 20%% SRP 512^2..2048^2 x 2 bounces; host outputs"
                       % (args.served_rate, args.served_seconds, len(items)),
           "rays": rays, "offered_mrays_s": round(rays / args.served_seconds / 1e6, 1),
           "lanes": args.served_lanes, "lane_budget_mib": args.served_budget_mib,
           "wave_paths": args.served_wave_paths,
           "open_loop": {"kind": "latency: requests submitted at their Poisson arrival times, so mrays_s is "
                                 "the offered load, not a throughput figure",
                         "served": dict(summary(lat_s, span_s), waves=nb_s, clocks=clk_s),
                         "per_call": dict(summary(lat_p, span_p), clocks=clk_p)},
           "closed_loop": {"kind": "throughput: every request submitted at once, makespan Mrays/s",
                           "served": dict(summary(clat_s, cspan_s), waves=cnb_s, clocks=cclk_s),
                           "per_call": dict(summary(clat_p, cspan_p), clocks=cclk_p),
                           "speedup": round(cspan_p / cspan_s, 3)},
           "body_generation_s": round(t_gen, 1)}
    srv.close()
    return out


def cornell_measure(ctx, stream, cpu=True):
    """Cornell box (36 triangles): 256^2 render, 16 spp, 3 bounces, area light, seed 0, and the
    depth / normal / instance passes -- on the GPU (CUDA events, device outputs) and, for the render,
    the CPU oracle on all host cores (same Philox streams, so the same paths and ray count)."""
    import torch
    from crt_gb300 import scenes
    ents, cam, lights = scenes.cornell()
    sc = ctx.scene(ents)
    W, H = int(cam["resolution"][0]), int(cam["resolution"][1])
    dev = torch.device("cuda", torch.cuda.current_device())
    rgba = torch.empty((H, W, 4), dtype=torch.uint8, device=dev)
    xyz = torch.empty((H, W, 3), dtype=torch.float64, device=dev)
    ids = torch.empty((H, W), dtype=torch.int32, device=dev)
    nrm = torch.empty((H, W, 3), dtype=torch.float64, device=dev)

    def render():
        sc.render(cam, lights, 16, 16, 0.0, 3, seed=0, want_radiance=False, out_rgba=rgba)

    def passes():
        sc.passes(cam, xyz=xyz, ids=ids, normals=nrm)

    with torch.cuda.stream(stream):
        ctx.reset_counters()
        ctx.set_counting(True)
        render()
        rays = int(ctx.counters()["answered"])
        ctx.set_counting(False)
        times = {}
        for name, fn, reps in (("render", render, 10), ("passes", passes, 20)):
            fn()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(reps):
                fn()
            b.record(stream)
            torch.cuda.synchronize()
            times[name] = a.elapsed_time(b) / reps
    out = {"workload": "Cornell box 36 triangles: render %dx%d, 16 spp, 3 bounces, area light, seed 0; "
                       "depth + normal + instance passes" % (W, H),
           "rays": rays, "gpu_render_ms": round(times["render"], 3), "gpu_passes_ms": round(times["passes"], 3),
           "gpu_mrays_s": round(rays / times["render"] / 1e3, 1)}
    if cpu:
        import oracle
        o = oracle.Scene(ents, nthreads=os.cpu_count() or 1)
        t = time.perf_counter()
        o.render(cam, lights, 16, 16, 0.0, 3, seed=0)
        cs = time.perf_counter() - t
        out.update(cpu_render_s=round(cs, 3), cpu_mrays_s=round(rays / cs / 1e6, 2), cpu_cores=os.cpu_count() or 1,
                   gpu_speedup=round(cs * 1e3 / times["render"], 1))
    sc.close()
    return out


def srp_measure(args, ctx, stream):
    """SRP batch: spacecraft (box bus, two panels, parabolic dish), N random attitudes, 4096^2 parallel
    sun rays each, 2 specular bounces, FP64 force / torque and per-facet absorbed power on the device."""
    import torch
    from crt_gb300 import workloads
    cfg = workloads.srp_config(n_att=args.srp_attitudes)
    sc = ctx.scene(cfg["entities"])
    n_tris = sc.stats()["n_tris"]
    q = torch.from_numpy(np.ascontiguousarray(cfg["quaternions"])).cuda()
    n = q.shape[0]
    f = torch.empty((n, 3), dtype=torch.float64, device=q.device)
    t = torch.empty((n, 3), dtype=torch.float64, device=q.device)
    fp = torch.empty((n, n_tris), dtype=torch.float64, device=q.device)

    def run(facet):
        sc.srp_into(cfg["sun"], q, cfg["grid"], f, t, fp if facet else None, num_bounces=cfg["num_bounces"])

    with torch.cuda.stream(stream):
        # rays (counting build): every sun ray of the grids, traced or resolved as a miss by the
        # scene-box test, and the specular continuations
        ctx.reset_counters()
        ctx.set_counting(True)
        run(True)
        cnt = ctx.counters()
        ctx.set_counting(False)
        run(True)
        res = {}
        for facet in (False, True):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            run(facet)
            b.record(stream)
            torch.cuda.synchronize()
            res[facet] = a.elapsed_time(b) / 1e3
        # the allocation-free entry point on the first 16 attitudes, beside crt_srp on the same ones
        ns = min(16, n)
        qh = np.ascontiguousarray(cfg["quaternions"][:ns])
        fs = torch.empty((ns, 3), dtype=torch.float64, device=q.device)
        ts = torch.empty((ns, 3), dtype=torch.float64, device=q.device)
        sc.srp_static_into(cfg["sun"], qh, cfg["grid"], fs, ts, num_bounces=cfg["num_bounces"])   # warm-up
        st_ms = {}
        for name, fn in (("crt_srp", lambda: sc.srp_into(cfg["sun"], qh, cfg["grid"], fs, ts,
                                                         num_bounces=cfg["num_bounces"])),
                         ("crt_srp_static", lambda: sc.srp_static_into(cfg["sun"], qh, cfg["grid"], fs, ts,
                                                                       num_bounces=cfg["num_bounces"]))):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            st_ms[name] = (time.perf_counter() - t0) * 1e3 / ns
    sc.close()
    return {"workload": "SRP batch: spacecraft %d triangles, %d attitudes x %d^2 sun rays, %d bounces"
                        % (n_tris, n, cfg["grid"], cfg["num_bounces"]),
            "rays": int(cnt["answered"]), "mrays_s": round(cnt["answered"] / res[True] / 1e6, 1),
            "rays_traversed": int(cnt["rays"]),
            "rays_note": "sun rays of the grids (traced, or resolved as misses by the scene-box test) + "
                         "specular continuations traced",
            "ms": round(res[True] * 1e3, 2), "ms_without_facet_power": round(res[False] * 1e3, 2),
            "ms_per_attitude": round(res[True] * 1e3 / n, 3), "nodes_per_ray": round(cnt["nodes"] / cnt["rays"], 2),
            "static_vs_allocating": {"attitudes": ns, "host_quaternions_device_outputs": True,
                                     "wall_ms_per_attitude": {k: round(v, 3) for k, v in st_ms.items()}}}


def tile_order(W, H):
    """Pixel index of each path slot in the order the render path traces camera rays: 8 x 4 tiles in
    row-major tile order (rows in bands of 4, the last band lower when H % 4 != 0, each band's last
    tile W % 8 wide)."""
    j = np.arange(W * H, dtype=np.int64)
    y0 = j // (4 * W) * 4
    hb = np.minimum(4, H - y0)
    r = j - y0 * W
    full = W >> 3
    tx = np.minimum(r // (8 * hb), full)
    rr = r - tx * 8 * hb
    wt = np.where(tx < full, 8, max(W - 8 * full, 1))
    return (y0 + rr // wt) * W + tx * 8 + rr % wt


def scenes_camera_rays(cam):
    """FP32 camera rays in crt_ray layout (o.xyz, tmin, d.xyz, tmax) as an [n, 8] float32 array in the
    render path's 8 x 4 tile order, for the roofline probe (workloads.camera_rays gives FP64 rays laid
    out o.xyz, d.xyz, tmin, tmax, one per pixel in row-major order)."""
    from crt_gb300 import workloads
    r64 = workloads.camera_rays(cam)[tile_order(int(cam["resolution"][0]), int(cam["resolution"][1]))]
    r = np.empty((r64.shape[0], 8), dtype=np.float32)
    r[:, 0:3] = r64[:, 0:3]
    r[:, 3] = 0.0
    r[:, 4:7] = r64[:, 3:6]
    r[:, 7] = np.finfo(np.float32).max
    return r


def e2e_measure(args, ents, cfg, rays_step):
    import crt
    from crt.body_fixed import BodyFixedEntity, BodyFixedGroup
    from crt.cameras import SimpleCamera
    from crt.lidars import SimpleLidar
    from crt.lights import PointLight
    from crt_gb300 import scenes
    cache = os.environ.get("CRT_SCENE_CACHE", "/tmp/crt_scene_cache")
    os.makedirs(cache, exist_ok=True)
    path = os.path.join(cache, f"asteroid_{args.faces}.obj")
    if not os.path.exists(path):
        scenes.write_obj_fast(ents[0].mesh, path + ".tmp")
        os.replace(path + ".tmp", path)
    group = BodyFixedGroup([BodyFixedEntity(path, color=[0.1, 0.1, 0.1])])
    cam = cfg["camera"]
    camera = SimpleCamera(cam["focal_length"], cam["resolution"], cam["sensor_size"], False,
                          position=cam["position"], rotation=cam["rotation"])
    light = PointLight(cfg["lights"][0]["intensity"], position=cfg["lights"][0]["position"])
    lid = cfg["lidar"]
    lidar = SimpleLidar(False, position=lid["position"], rotation=lid["rotation"])
    lidar.set_beam_grid(lid["nx"], lid["ny"], lid["half_x"], lid["half_y"])
    for _ in range(max(3, args.warmup)):
        img = group.render(camera, light, 1, 1, 1.0, cfg["bounces"])
        rng, prim = group.lidar_scan(lidar)
    n = max(3, min(args.steps, 50))
    t = time.perf_counter()
    for _ in range(n):
        img = group.render(camera, light, 1, 1, 1.0, cfg["bounces"])
        rng, prim = group.lidar_scan(lidar)
    el = (time.perf_counter() - t) / n
    d2h = img.nbytes + rng.nbytes + prim.nbytes
    h2d = 3 * 160   # camera, light and LiDAR descriptors (kernel parameters); the BVH stays resident
    return {"value": round(rays_step / el / 1e6, 2), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": int(d2h), "ms_per_step": round(el * 1e3, 3), "api": "crt.BodyFixedGroup"}


def main():
    args = parse()
    if args.probe:
        probe(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
