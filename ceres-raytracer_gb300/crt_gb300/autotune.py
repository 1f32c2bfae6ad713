"""Autotuner for the persistent-kernel and wavefront knobs of a context (crt_tuning).

Knobs: queue_chunk (32-ray groups a warp takes per atomic grab of the ray queue), wave_paths
(camera paths per wavefront wave: larger waves amortise launches, smaller ones keep the path
buffers in L2) and use_graphs (replay one captured wave per wave).  The traversal stack depth is a
compile-time constant (8 shared-memory entries per thread and a 64-entry local spill; an 8-wide
tree over 8M triangles is about 10 levels deep), so it is not searched.

`tune(ctx, run)` times `run()` (one representative call, e.g. one crt_batch of the workload) for
each candidate with CUDA events on the context stream, after a warm-up call, and keeps the fastest.
Results are cached in a JSON file keyed by GPU name, SM count, a scene-size class and the caller's
workload name, so a server tunes once per GPU type and workload.
"""
import json
import os
import time

CANDIDATES = {
    "queue_chunk": (1, 2, 4),
    "wave_paths": (1 << 21, 1 << 22, 1 << 23, 1 << 24),
    "use_graphs": (True, False),
}


def cache_path():
    return os.environ.get("CRT_TUNE_CACHE", os.path.join(os.path.expanduser("~"), ".cache", "crt_gb300_tune.json"))


def scene_class(n_tris):
    """Order of magnitude of the triangle count (tuning transfers within a class)."""
    c = 0
    while n_tris >= 10 ** (c + 1):
        c += 1
    return "1e%d" % c


def device_key():
    import torch
    p = torch.cuda.get_device_properties(torch.cuda.current_device())
    return "%s/%dsm" % (p.name, p.multi_processor_count)


def load_cache(path=None):
    path = path or cache_path()
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def save_cache(cache, path=None):
    path = path or cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def candidates(grid=None):
    grid = grid or CANDIDATES
    for qc in grid["queue_chunk"]:
        for wp in grid["wave_paths"]:
            for g in grid["use_graphs"]:
                yield {"queue_chunk": qc, "wave_paths": wp, "use_graphs": g}


def time_call(ctx, run, reps=1):
    """Device time (ms) of `reps` calls of run(), CUDA events recorded on the context stream."""
    import torch
    h = ctx.stream_handle()
    s = torch.cuda.ExternalStream(h) if h else torch.cuda.default_stream()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(reps):
        run()
    b.record(s)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def tune(ctx, run, workload, n_tris, grid=None, reps=1, use_cache=True, path=None, timer=None, device=None):
    """Best crt_tuning for `run` on this GPU; applies it to ctx and returns (knobs, report).

    report: {"cached": bool, "trials": [(knobs, ms), ...], "seconds": wall time of the search}.
    `timer(ctx, run, reps) -> ms` and `device` (cache key of the GPU) default to CUDA-event timing
    on the context stream and the current device."""
    timer = timer or time_call
    key = "%s|%s|%s" % (device or device_key(), scene_class(n_tris), workload)
    cache = load_cache(path) if use_cache else {}
    if key in cache:
        best = cache[key]["knobs"]
        ctx.set_tuning(**best)
        return best, {"cached": True, "trials": cache[key].get("trials", []), "seconds": 0.0}
    t0 = time.perf_counter()
    trials = []
    for k in candidates(grid):
        ctx.set_tuning(**k)
        run()   # warm-up: scratch sized for this wave size, graph path exercised
        trials.append((k, timer(ctx, run, reps)))
    best = min(trials, key=lambda t: t[1])[0]
    ctx.set_tuning(**best)
    report = {"cached": False, "trials": trials, "seconds": time.perf_counter() - t0}
    if use_cache:
        cache = load_cache(path)
        cache[key] = {"knobs": best, "trials": trials}
        save_cache(cache, path)
    return best, report
