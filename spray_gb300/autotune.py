"""Autotuner of the tracer's launch shapes, wavefront size and out-of-core
batching.

For a benchmark workload (`spray_gb300.scenes.CONFIGS`) it times whole frames
on the GPU (device time from the tracer's own events, median of `frames`
frames after `warmup`) and runs coordinate descent over

  trace_blocks_per_sm    CTAs per SM of the traversal launches (packets in flight)
  sched_chunks_per_warp  ray chunks per scheduling warp (queue-chunk size)
  wave_samples           samples per wavefront (0 = the library default)
  ooc_batch, ooc_inplace out of core only: domains per batch (prefetch depth)
                         and the in-place tracing threshold

starting from the library defaults.  The result goes to
`spray_gb300/tuned/<workload>.json` (`<workload>_policy<p>.json` when tuned
for a schedule policy other than the workload's), which bench.py applies;
every trial is kept in the file.  Images do not depend on these settings.

    python -m spray_gb300.autotune --config c2
"""
from __future__ import annotations

import argparse
import json
import statistics
from pathlib import Path

TUNED = Path(__file__).resolve().parent / "tuned"

SPACE = {
    "trace_blocks_per_sm": [2, 3, 4, 6, 8],
    "sched_chunks_per_warp": [2, 4, 8, 16],
    "wave_samples": [0, 16 << 20, 32 << 20],
}
OOC_SPACE = {
    "ooc_batch": [0, 32, 64],
    "ooc_inplace": [4096, 16384, 65536],
}


def _path(name: str, policy: int | None) -> Path:
    return TUNED / (f"{name}.json" if policy is None else f"{name}_policy{policy}.json")


def load(name: str, policy: int | None = None) -> dict | None:
    """The committed tuning of a workload for a schedule policy (falling back
    to the workload's own), or None."""
    for p in ([_path(name, policy)] if policy is not None else []) + [_path(name, None)]:
        try:
            return json.loads(p.read_text())
        except Exception:
            continue
    return None


def _frame_ms(scene, cfg: dict, cam, frames: int, warmup: int, views: list | None = None) -> float:
    """Median frame time; a multi-view workload traces its whole view batch."""
    import spray_gb300 as sg
    t = sg.Tracer(cfg)
    t.set_scene(scene)
    t.set_camera(*cam)
    frame = (lambda: t.trace_views(views)) if views else t.trace
    for _ in range(warmup):
        frame()
    ms = [frame()[1]["frame_ms"] for _ in range(frames)]
    t.close()
    return statistics.median(ms)


def tune(name: str, frames: int | None = None, warmup: int | None = None, policy: int | None = None,
         rounds: int = 1, write: bool = True) -> dict:
    """frames / warmup default to 3 / 2 in core and 10 / 5 out of core, where the
    domain cache settles over several frames (with fewer, the early frames'
    loads mislead the comparison)."""
    import spray_gb300 as sg
    from spray_gb300 import scenes
    path, _ = scenes.benchmark_scene(name)
    scene = sg.Scene.load(path, path.parent)
    spec, cfg = scenes.workload_config(name, scene)
    if policy is not None:
        cfg["schedule_policy"] = policy
    ooc = 0 < cfg.get("cache_size", -1) < len(scene.domains)
    if frames is None:
        frames = 10 if ooc else 3
    if warmup is None:
        warmup = 5 if ooc else 2
    space = dict(SPACE)
    if ooc:
        space.update(OOC_SPACE)
    cam = scenes.orbit_camera(scene)
    views = scenes.c5_views(scene, spec["views"], spec["view_seed"]) if "views" in spec else None
    best = {k: 0 for k in space}
    best.update({"trace_blocks_per_sm": 4, "sched_chunks_per_warp": 8, "wave_samples": 0})
    if ooc:
        best.update({"ooc_batch": 0, "ooc_inplace": 16384})
    trials = []

    def run(params):
        ms = _frame_ms(scene, dict(cfg, **params), cam, frames, warmup, views)
        trials.append({"params": dict(params), "frame_ms": ms})
        return ms

    default_ms = best_ms = run(best)
    for _ in range(rounds):
        for key, values in space.items():
            for v in values:
                if v == best[key]:
                    continue
                cand = dict(best, **{key: v})
                ms = run(cand)
                if ms < best_ms:
                    best, best_ms = cand, ms
    out = {"workload": name, "policy": cfg.get("schedule_policy", 0), "params": best, "frame_ms": best_ms,
           "default_frame_ms": default_ms, "frames": frames, "warmup": warmup, "trials": trials}
    try:
        import torch
        out["gpu"] = torch.cuda.get_device_name(0)
    except Exception:
        pass
    if write:
        TUNED.mkdir(exist_ok=True)
        _path(name, policy).write_text(json.dumps(out, indent=1) + "\n")
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", default="c2")
    ap.add_argument("--frames", type=int, default=None, help="timed frames per trial (3; 10 out of core)")
    ap.add_argument("--warmup", type=int, default=None, help="warm-up frames per trial (2; 5 out of core)")
    ap.add_argument("--policy", type=int, default=None)
    ap.add_argument("--rounds", type=int, default=1)
    args = ap.parse_args()
    r = tune(args.config, args.frames, args.warmup, args.policy, args.rounds)
    print(json.dumps({k: r[k] for k in ("workload", "params", "frame_ms", "default_frame_ms")}))


if __name__ == "__main__":
    main()
