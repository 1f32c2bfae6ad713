"""Autotuner host logic (no GPU): candidate grid, best choice, cache round trip, scene classes."""
from crt_gb300 import autotune


class FakeCtx:
    def __init__(self):
        self.knobs = None
        self.calls = 0

    def set_tuning(self, **k):
        self.knobs = dict(k)


def cost(ctx, run, reps):
    # a made-up cost surface: best at queue_chunk 2, 4M-path waves, graphs on
    k = ctx.knobs
    run()
    return (abs(k["queue_chunk"] - 2) + abs(k["wave_paths"].bit_length() - 23) + (0 if k["use_graphs"] else 0.5))


def test_tune_picks_minimum_and_caches(tmp_path):
    path = str(tmp_path / "tune.json")
    ctx = FakeCtx()
    runs = []
    best, rep = autotune.tune(ctx, lambda: runs.append(1), "mix", 2_000_000, path=path, timer=cost, device="gpu")
    assert best == {"queue_chunk": 2, "wave_paths": 1 << 22, "use_graphs": True}
    assert ctx.knobs == best and not rep["cached"]
    n = len(list(autotune.candidates()))
    assert len(rep["trials"]) == n and len(runs) == 2 * n      # warm-up + timed call per candidate
    ctx2 = FakeCtx()
    best2, rep2 = autotune.tune(ctx2, lambda: None, "mix", 3_000_000, path=path, timer=cost, device="gpu")
    assert rep2["cached"] and best2 == best and ctx2.knobs == best
    # another scene class or workload is tuned separately
    _, rep3 = autotune.tune(FakeCtx(), lambda: None, "mix", 20_000_000, path=path, timer=cost, device="gpu")
    assert not rep3["cached"]


def test_scene_class():
    assert autotune.scene_class(36) == "1e1"
    assert autotune.scene_class(2_000_000) == "1e6"
    assert autotune.scene_class(8_000_000) == "1e6"
    assert autotune.scene_class(10_000_000) == "1e7"
