"""Benchmark of the speculative domain-parallel tracer (one frame = one step).

Default workload (the configuration the headline metric is quoted on): the
64-domain wavelet grid (4x4x4 cells, 64^3 isosurfaces), path tracing,
1920x1080, 16 spp, 5 bounces with Russian roulette from bounce 3, per-domain
albedo, one emissive quad light, seeded orbit camera.  Prints one JSON line.

  value         Mrays/s of all logical rays (primary + shadow + bounce), frames
                timed with CUDA events on the tracer's stream, scene resident
  e2e           the same metric through spray_gpu_trace with the image copied
                to pinned host memory every frame (wall clock around the call)
  roofline      closest-hit traversal kernel: algorithmic bytes / kernel time
  accuracy      the GPU renders the CPU baseline's reduced frame too: image
                RMSE against the reference loop restated on the CPU (oracle
                mode A), bit equality with the wavefront restatement (mode B),
                hit and occlusion agreement of every depth's rays
  c3_schedulers the 512-domain out-of-core workload (C3) under the plain
                speculative order, batched passes and the learned proposal:
                Mrays/s by ray class, domain loads, bytes copied and bytes read
                in place from host memory per frame
  cpu_baseline  the CPU restatement of the reference loop (speculative queues,
                DomainStats order, VBuf history) on a downscaled frame, all cores

--impl reference times that CPU restatement alone on the same workload and the
same full frame.  It loads the scene with the oracle's own reader and never
loads the CUDA library (the reference binary itself needs Embree 2.17, glm,
glog and MPI, which are not available).  Rank 0 only.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s at <=1e-3 image RMSE, learned vs plain scheduler; domain loads/frame"
POLICIES = {"plain": (0, "plain speculative"), "resident": (1, "resident domains first"),
            "batched": (2, "batched passes (shadow b + radiance b+1), culled domains not loaded"),
            "learned": (3, "learned domain-order proposal (online-trained MLP) + batched passes"),
            "nonspec": (4, "non-speculative LoadAnyOnce: one pass per list position, most pending rays first"),
            "rounds": (5, "the reference's non-speculative image tracer: one domain per round, the one "
                          "holding the most queued rays (LoadAnyOnceImageSched)")}
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0
NODE_BYTES, TRI_BYTES, ENTRY_BYTES, RAY_BYTES, HIT_BYTES = 128, 48, 8, 32, 24


def describe(name: str, spec: dict, cfg: dict) -> str:
    g = spec["grid"]
    if name == "c5":
        return (f"c5: {g}x{g}x{g} wavelet domains ({spec['samples']}^3 isosurfaces), {spec['views']} views "
                "of mixed size (256..2048 squared), spp (1, 4, 16) and shader (AO / 4-bounce path tracing) "
                "in one frame")
    mode = "AO" if cfg.get("ao_mode") else "path tracing"
    return (f"{name}: {g}x{g}x{g} wavelet domains ({spec['samples']}^3 isosurfaces), {mode}, "
            f"{cfg['image_w']}x{cfg['image_h']}, {cfg['pixel_samples']} spp, {cfg['bounces']} bounces")


def scene_file(name: str) -> Path:
    """The workload's .spray file, generated once.  Generation uses the
    library's wavelet generator; a process that must not load the library
    (the reference arm) runs it in a child process."""
    from spray_gb300 import scenes
    spec = scenes.CONFIGS[name]
    d = scenes.scene_dir(name)
    if not (d / "scene.spray").exists():
        subprocess.run([sys.executable, "-c",
                        f"import sys; sys.path.insert(0, {str(ROOT)!r}); "
                        f"from spray_gb300 import scenes; scenes.benchmark_scene({name!r})"], check=True)
    return d / "scene.spray"


def bench_config(name: str, spec: dict, cfg: dict, scene, policy: str, tuned, world: int,
                 views=None) -> dict:
    """The `config` object of the JSON line, from host-side facts only, so
    that both arms print the same one."""
    W, H = cfg["image_w"], cfg["image_h"]
    c = {"workload": describe(name, spec, cfg), "scheduler": POLICIES[policy][1],
         "domains": len(scene.domains), "triangles": int(sum(len(d.faces) for d in scene.domains)),
         "image": [W, H], "spp": cfg["pixel_samples"], "bounces": cfg["bounces"],
         "l2": "256 MiB buffer written before every timed frame; ray state > L2",
         "parallelism": f"replicas x{world} (one view per GPU)", "tuned": tuned}
    if views is not None:
        c["views"] = {"count": len(views), "pixels": sum(v["image_w"] * v["image_h"] for v in views),
                      "samples": sum(v["image_w"] * v["image_h"] * v["pixel_samples"] for v in views),
                      "ao_views": sum(1 for v in views if v["ao_mode"]),
                      "sizes": sorted({v["image_w"] for v in views})}
    return c


def clock_sampler(out: Path):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(out, "w")
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                              "-lms", "50"], stdout=f, stderr=subprocess.DEVNULL)
    except Exception:
        return None, None
    # the timed region starts once the sampler writes (its start-up takes
    # longer than a few frames)
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < 3.0 and p.poll() is None:
        f.flush()
        if out.stat().st_size > 0:
            break
        time.sleep(0.01)
    return p, f


def smi_index(local: int) -> int:
    """nvidia-smi index of this process's CUDA device (CUDA_VISIBLE_DEVICES may remap it)."""
    vis = [v.strip() for v in os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",") if v.strip()]
    if local < len(vis) and vis[local].isdigit():
        return int(vis[local])
    return local


def clock_summary(path: Path, device: int) -> dict | None:
    try:
        rows = [l.split(",") for l in path.read_text().splitlines() if l.strip()]
    except Exception:
        return None
    rows = [[c.strip() for c in r] for r in rows if len(r) >= 9 and r[0].strip() == str(device)]
    if not rows:
        return None
    sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
    mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
            "reasons": reasons, "samples": len(rows)}


def hbm_peak():
    try:
        d = json.loads(MEASURED_PEAKS.read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def load_profile_traffic(name: str):
    """DRAM bytes per algorithmic byte of the closest-hit kernel, from the committed ncu summary."""
    p = ROOT / "profiles" / f"trace_closest_{name}.json"
    try:
        return json.loads(p.read_text())
    except Exception:
        return None


def oracle_config(cfg: dict, scale: int) -> dict:
    c = dict(cfg)
    c["image_w"] = max(8, cfg["image_w"] // scale)
    c["image_h"] = max(8, cfg["image_h"] // scale)
    c.setdefault("history_size", 4)
    c.setdefault("list_size", 16)
    c.setdefault("cache_size", -1)
    c.setdefault("max_samples_per_rank", 1 << 20)
    c.setdefault("num_ranks", 1)
    c.setdefault("rank", 0)
    return c


def cpu_speculative(scene, cfg, threads: int, scale: int, frame: int = 0):
    """The reference loop restated on the CPU (oracle mode A), on a frame
    downscaled by `scale` per axis.  Returns (rays, seconds, config, stats,
    image, oracle)."""
    from oracle import oracle as O
    from spray_gb300 import scenes
    c = oracle_config(cfg, scale)
    o = O.Oracle(c, scene)
    o.set_camera(*scenes.orbit_camera(scene, frame=frame))
    t0 = time.perf_counter()
    img, st = o.render_speculative(threads)
    dt = time.perf_counter() - t0
    rays = st["rays_primary"] + st["rays_shadow"] + st["rays_bounce"]
    return rays, dt, c, st, img, o


def run_reference(args, rank):
    """Times the CPU restatement of the reference loop on the full workload
    frame.  Never loads the CUDA library: the scene comes from the oracle's
    own .spray/PLY reader."""
    if rank != 0:
        return
    from oracle import scene_io
    from spray_gb300 import autotune, scenes
    path = scene_file(args.config)
    scene = scene_io.load(path, path.parent)
    spec, cfg = scenes.workload_config(args.config, scene)
    if args.config == "c5":
        print(json.dumps({"impl": "reference", "unavailable": "the multi-view batch has no counterpart in "
                          "the reference loop (one camera per renderer)"}), flush=True)
        return
    t = autotune.load(args.config, POLICIES[args.policy][0]) if args.tuned else None
    tuned = dict(t["params"]) if t else None
    threads = os.cpu_count() or 1
    scale = args.ref_scale
    for _ in range(args.warmup):
        cpu_speculative(scene, cfg, threads, scale)
    rays_t, secs, st_last, c = 0, 0.0, None, None
    for _ in range(args.steps):
        rays, dt, c, st, _, o = cpu_speculative(scene, cfg, threads, scale)
        o.close()
        rays_t += rays
        secs += dt
        st_last = st
    v = rays_t / secs / 1e6
    sample = (f"the full {c['image_w']}x{c['image_h']} frame per step" if scale == 1 else
              f"{c['image_w']}x{c['image_h']} frame (1/{scale} per axis)") + \
        f" of the same scene, camera, spp and bounces; speculative loop with {threads} OpenMP threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * secs / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded wavelet isosurface scene, seeded orbit camera)",
        "config": bench_config(args.config, spec, cfg, scene, args.policy, tuned, args.gpus),
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "rays_per_frame": {k: st_last[f"rays_{k}"] for k in ("primary", "shadow", "bounce")},
        "domain_loads_per_frame": st_last["domain_loads"],
        "note": "reference binary unbuildable here (Embree 2.17, glm, glog, MPI absent); timed the CPU "
                "restatement of its speculative loop (oracle mode A), scene read by the oracle's own loader",
    }
    print(json.dumps(line), flush=True)


def accuracy_report(scene, cfg, cam, mode_a_img, oracle_obj, device: int) -> dict:
    """The GPU renders the CPU baseline's reduced frame with its stage
    buffers kept, and is compared with the oracle (image, hits, occlusion)."""
    import spray_gb300 as sg
    from oracle import accuracy as A
    c = dict(cfg)
    c["debug_capture"] = 1
    t = sg.Tracer(c, device=device)
    t.set_scene(scene)
    t.set_camera(*cam)
    img, st = t.trace()
    # the oracle walks the same hierarchies the GPU built (front to back,
    # culled by the hit so far) and counts that walk's nodes and triangles
    for d in range(len(scene.domains)):
        oracle_obj.set_bvh4(d, t.debug(sg.DBG_NODES, d), t.debug(sg.DBG_TRIS, d))
    mode_b, ost = oracle_obj.render_wavefront()
    hits, shadows = {}, {}
    for b in range(cfg["bounces"]):
        rays = t.debug(sg.DBG_RAYS, b)
        if len(rays) == 0:
            break
        h = t.debug(sg.DBG_HITS, b)
        hits[str(b)] = A.hit_agreement(rays, h, oracle_obj)
        shadows[str(b)] = A.shadow_agreement(t.debug(sg.DBG_SHADOWS, b), h, oracle_obj)
    t.close()
    rep = A.frame_report(img, mode_a_img, mode_b, hits, shadows)
    rep["frame"] = [c["image_w"], c["image_h"]]
    gpu_bytes = (st["visits_radiance"] * (RAY_BYTES + ENTRY_BYTES + HIT_BYTES)
                 + st["nodes_radiance"] * NODE_BYTES + st["tris_radiance"] * TRI_BYTES)
    orc_bytes = (ost["bvh4_visits"] * (RAY_BYTES + ENTRY_BYTES + HIT_BYTES)
                 + ost["bvh4_nodes"] * NODE_BYTES + ost["bvh4_tris"] * TRI_BYTES)
    rep["closest_hit_traversal"] = {
        "gpu": {"visits": st["visits_radiance"], "nodes": st["nodes_radiance"], "tris": st["tris_radiance"]},
        "oracle": {"visits": ost["bvh4_visits"], "nodes": ost["bvh4_nodes"], "tris": ost["bvh4_tris"],
                   "hit_mismatches": ost["bvh4_mismatches"]},
        "oracle_to_gpu_bytes": orc_bytes / gpu_bytes if gpu_bytes else None}
    return rep


def c3_schedulers_block(args, device: int) -> dict:
    """C3 (512 domains out of core) under the plain speculative order, the
    batched passes, the learned proposal, the non-speculative passes and the
    reference's non-speculative round loop: the metric's comparison."""
    import spray_gb300 as sg
    from spray_gb300 import autotune, scenes
    from oracle import accuracy as A
    path, spec = scenes.benchmark_scene("c3")
    scene = sg.Scene.load(path, path.parent)
    _, cfg0 = scenes.workload_config("c3", scene)
    cam = scenes.orbit_camera(scene)
    prep = Path(tempfile.gettempdir()) / f"spray_c3_prepared_{os.getpid()}"
    sg.prepare_scene(scene, prep)
    out = {"workload": describe("c3", spec, cfg0), "policies": {}}
    frames = max(args.steps, args.c3_frames)
    ref_img = None
    small = None
    for name in ("plain", "batched", "learned", "nonspec", "rounds"):
        cfg = dict(cfg0)
        pol = POLICIES[name][0]
        cfg["schedule_policy"] = pol
        t = autotune.load("c3", pol) if args.tuned else None
        if t and t.get("policy") == pol:
            cfg.update(t["params"])
        if name == "learned":
            cfg["learn_frames"] = 1
        tr = sg.Tracer(cfg, device=device)
        tr.set_scene_prepared(prep, len(scene.domains), scene.lights)
        tr.set_camera(*cam)
        img = np.empty((cfg["image_h"], cfg["image_w"], 4), np.float32)
        # the round loop runs thousands of rounds per frame: fewer frames (it
        # is deterministic, so frames differ only in the cache's warmth)
        nwarm, ntimed = (1, min(frames, 3)) if name == "rounds" else (max(args.warmup, 3), frames)
        warm = [tr.trace(img)[1] for _ in range(nwarm)]
        sts = [tr.trace(img)[1] for _ in range(ntimed)]
        if ref_img is None:
            ref_img = img.copy()
        ms = sum(s["frame_ms"] for s in sts)
        rays = {k: sum(s[f"rays_{k}"] for s in sts) for k in ("primary", "shadow", "bounce")}
        n = len(sts)
        vis = sum(s["visits_radiance"] + s["visits_shadow"] for s in sts)
        r = {"scheduler": POLICIES[name][1], "frames": n, "ms_per_frame": ms / n,
             "mrays_per_s": sum(rays.values()) / (ms * 1e-3) / 1e6,
             "mrays_per_s_by_class": {k: v / (ms * 1e-3) / 1e6 for k, v in rays.items()},
             "visits_per_ray": vis / max(sum(rays.values()), 1),
             "radiance_visits_per_frame": sum(s["visits_radiance"] for s in sts) / n,
             "shadow_visits_per_frame": sum(s["visits_shadow"] for s in sts) / n,
             "domain_loads_per_frame": sum(s["domain_loads"] for s in sts) / n,
             "h2d_bytes_per_frame": sum(s["h2d_bytes"] for s in sts) / n,
             "inplace_bytes_per_frame": sum(s["inplace_bytes"] for s in sts) / n,
             "inplace_domains_per_frame": sum(s["inplace_domains"] for s in sts) / n,
             "image_equals_plain": bool(A.bit_exact(img, ref_img)),
             "tuned": t["params"] if t and t.get("policy") == pol else None}
        if name == "rounds":
            # the baseline tracer numbers samples across the whole image
            # (samid = spp * pixel + s, baseline_insitu_tracer.inl:407-440) where
            # the speculative tracer numbers them per tile, so the two images
            # carry different sample noise: compare their mean radiance, and
            # the loop itself with the oracle below
            mean = lambda x: float(np.mean(x[..., :3], dtype=np.float64))
            r["mean_radiance_rel_diff_vs_plain"] = abs(mean(img) - mean(ref_img)) / max(mean(ref_img), 1e-30)
            r["rounds_per_frame"] = sum(s["rounds"] for s in sts) / n
            r["shading_only_visits_per_frame"] = sum(s["visits_shade"] for s in sts) / n
            r["cold_cache_domain_loads"] = warm[0]["domain_loads"]
        if name == "learned":
            w0 = next((w for w in warm if w["learn_ms"] > 0), None)
            r["learn"] = {"trained_before_timing": bool(warm[-1]["learn_trained"]),
                          "pairs": warm[-1]["learn_pairs"], "train_ms": w0["learn_ms"] if w0 else None,
                          "loss": w0["learn_loss"] if w0 else None,
                          "held_out_pairs": w0["learn_eval_pairs"] if w0 else 0,
                          "top1_accuracy": w0["learn_top1"] if w0 else None,
                          "top1_accuracy_nearest_candidate": w0["learn_top1_nearest"] if w0 else None}
        s0 = sts[-1]
        out["cache"] = {"slots": s0["cache_slots"], "slot_bytes": s0["cache_slot_bytes"],
                        "cache_bytes": s0["cache_slots"] * s0["cache_slot_bytes"],
                        "scene_bytes": s0["scene_bytes"], "scene_triangles": s0["scene_triangles"],
                        "fraction_of_scene": s0["cache_slots"] * s0["cache_slot_bytes"] / max(s0["scene_bytes"], 1),
                        "note": "the cache holds half of the domains, the 8 GiB of ~16 GB ratio of the "
                                "workload description; the generated scene is smaller than its estimate"}
        out["policies"][name] = r
        tr.close()
    p, b, l = (out["policies"][k] for k in ("plain", "batched", "learned"))
    out["nonspec_vs_plain"] = {"speedup": out["policies"]["nonspec"]["mrays_per_s"] / p["mrays_per_s"]}
    rd = out["policies"]["rounds"]
    out["learned_vs_reference_nonspeculative_loop"] = {
        "speedup": l["mrays_per_s"] / rd["mrays_per_s"],
        "domain_load_reduction": 1 - l["domain_loads_per_frame"] / max(rd["domain_loads_per_frame"], 1e-9),
        "radiance_visits_ratio": l["radiance_visits_per_frame"] / max(rd["radiance_visits_per_frame"], 1e-9)}
    out["learned_vs_plain"] = {"speedup": l["mrays_per_s"] / p["mrays_per_s"],
                               "domain_load_reduction": 1 - l["domain_loads_per_frame"] / max(p["domain_loads_per_frame"], 1e-9),
                               "bytes_moved_reduction": 1 - (l["h2d_bytes_per_frame"] + l["inplace_bytes_per_frame"]) /
                               max(p["h2d_bytes_per_frame"] + p["inplace_bytes_per_frame"], 1e-9)}
    out["learned_vs_batched"] = {"speedup": l["mrays_per_s"] / b["mrays_per_s"],
                                 "visits_per_ray_ratio": l["visits_per_ray"] / b["visits_per_ray"]}
    # accuracy at this scene's settings on a reduced frame (all 512 domains,
    # list size 22, 8 spp, 4 bounces): the learned order against the oracle
    if not args.no_cpu_baseline:
        cfg = dict(cfg0)
        cfg["schedule_policy"] = POLICIES["learned"][0]
        cfg["learn_frames"] = 1
        threads = os.cpu_count() or 1
        scale = max(1, cfg0["image_w"] // args.c3_accuracy_size)
        _, _, c, _, mode_a, o = cpu_speculative(scene, cfg, threads, scale)
        tr = sg.Tracer(dict(c, schedule_policy=3, learn_frames=1), device=device)
        tr.set_scene_prepared(prep, len(scene.domains), scene.lights)
        tr.set_camera(*cam)
        tr.trace()
        img, _ = tr.trace()  # trained after the first frame
        tr.close()
        mode_b, _ = o.render_wavefront()
        out["accuracy"] = {"frame": [c["image_w"], c["image_h"]],
                           "image_rmse_vs_oracle": A.image_rmse(img, mode_a),
                           "bit_exact_vs_wavefront_oracle": A.bit_exact(img, mode_b)}
        o.close()
        # the round loop against the oracle's restatement of the reference's
        # baseline tracer (mode C) on a small frame: the same rounds, loads
        # and visits from a cold cache; the image up to the order of additions
        rc = dict(cfg0, image_w=args.c3_rounds_size, image_h=args.c3_rounds_size)
        oc = dict(rc)
        for k, v in dict(history_size=4, max_samples_per_rank=1 << 20, num_ranks=1, rank=0).items():
            oc.setdefault(k, v)
        from oracle import oracle as O
        o = O.Oracle(oc, scene)
        o.set_camera(*cam)
        want, ws, sched = o.render_baseline()
        o.close()
        tr = sg.Tracer(dict(rc, schedule_policy=POLICIES["rounds"][0]), device=device)
        tr.set_scene_prepared(prep, len(scene.domains), scene.lights)
        tr.set_camera(*cam)
        img, st = tr.trace()
        log = tr.debug(sg.DBG_LOADS, 0)
        tr.close()
        out["rounds_accuracy"] = {
            "frame": [rc["image_w"], rc["image_h"]], "oracle": "mode C (reference baseline loop, one thread)",
            "rounds": [st["rounds"], ws["rounds"]], "domain_loads": [st["domain_loads"], ws["domain_loads"]],
            "schedule_equal": bool(np.array_equal(log["domain"], sched)),
            "visits_equal": all(st[k] == ws[k] for k in ("visits_radiance", "visits_shadow", "visits_shade",
                                                          "rays_shadow", "rays_bounce")),
            "image_rmse_vs_oracle": A.image_rmse(img, want)}
    import shutil
    shutil.rmtree(prep, ignore_errors=True)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c5"])
    ap.add_argument("--cpu-scale", type=int, default=2, help="CPU baseline frame downscale per axis")
    ap.add_argument("--ref-scale", type=int, default=1,
                    help="--impl reference: frame downscale per axis (1 = the workload's full frame)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-flush", action="store_true")
    ap.add_argument("--policy", default="plain", choices=list(POLICIES),
                    help="out-of-core domain order (plain: the reference's DomainStats order)")
    ap.add_argument("--ooc-batch", type=int, default=None, help="domains per batch under --policy batched")
    ap.add_argument("--ooc-inplace", type=int, default=None,
                    help="trace a non-resident domain in place from host memory when a batch holds at "
                         "most this many of its live entries (batched and learned policies)")
    ap.add_argument("--graphs", type=int, default=1, choices=[0, 1],
                    help="1: replay the in-core frame as a captured CUDA graph; 0: direct launches "
                         "(kernel profilers)")
    ap.add_argument("--tuned", type=int, default=1, choices=[0, 1],
                    help="apply the committed autotuner result for the workload (spray_gb300/tuned)")
    ap.add_argument("--scale", type=int, default=1,
                    help="divide the image size (profiling captures on a small frame only)")
    ap.add_argument("--c3-schedulers", type=int, default=1, choices=[0, 1],
                    help="1: also run C3 under every scheduler (plain, batched, learned, non-speculative, "
                         "the reference's round loop; rank 0 of a single-GPU run)")
    ap.add_argument("--c3-frames", type=int, default=15, help="timed C3 frames per scheduler")
    ap.add_argument("--c3-rounds-size", type=int, default=64,
                    help="image size of the round loop's comparison with the oracle")
    ap.add_argument("--c3-accuracy-size", type=int, default=256, help="C3 accuracy frame width")
    ap.add_argument("--accuracy", type=int, default=1, choices=[0, 1],
                    help="1: compare the GPU with the oracle on the CPU baseline's reduced frame")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank)
        return

    import torch
    import torch.distributed as dist
    import spray_gb300 as sg
    from spray_gb300 import scenes

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            dist.barrier()

    def allmax(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    def allsum(x: float) -> float:
        if world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        return float(t.item())

    if rank == 0:
        scenes.benchmark_scene(args.config)
    barrier()
    path, _ = scenes.benchmark_scene(args.config)
    scene = sg.Scene.load(path, path.parent)
    spec, cfg = scenes.workload_config(args.config, scene)
    base_cfg = dict(cfg)
    if args.scale > 1:
        cfg["image_w"] = max(8, cfg["image_w"] // args.scale)
        cfg["image_h"] = max(8, cfg["image_h"] // args.scale)
    tuned = None
    if args.tuned:
        from spray_gb300 import autotune
        t = autotune.load(args.config, POLICIES[args.policy][0])
        if t:
            tuned = dict(t["params"])
            cfg.update(tuned)
    cfg["graphs"] = args.graphs
    cfg["schedule_policy"] = POLICIES[args.policy][0]
    if args.ooc_batch is not None:
        cfg["ooc_batch"] = args.ooc_batch
    if args.ooc_inplace is not None:
        cfg["ooc_inplace"] = args.ooc_inplace
    if args.policy == "learned":
        cfg["learn_frames"] = 1  # collect during the first warm-up frame, train after it
    tracer = sg.Tracer(cfg, device=local)
    tracer.set_scene(scene)
    # weak scaling: each rank renders its own seeded view of the scene
    cam = scenes.orbit_camera(scene, frame=rank)
    tracer.set_camera(*cam)
    W, H = cfg["image_w"], cfg["image_h"]
    views = None
    if args.config == "c5":
        # the uneven multi-view batch: every view of the batch traced in one frame
        views = scenes.c5_views(scene, spec["views"], spec["view_seed"] + rank)
        if args.scale > 1:
            for v in views:
                v["image_w"] = max(8, v["image_w"] // args.scale)
                v["image_h"] = max(8, v["image_h"] // args.scale)
        npix = sum(v["image_w"] * v["image_h"] for v in views)
    else:
        npix = W * H
    img_dev = torch.empty(npix * 4, dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # 256 MiB > 129 MB L2

    def frame_device():
        if not args.no_flush:
            flush.fill_(1)
            torch.cuda.synchronize()
        if views is not None:
            return tracer.trace_views_device(views, img_dev.data_ptr())
        return tracer.trace_device(img_dev.data_ptr())

    warm = [frame_device() for _ in range(args.warmup)]
    learn = None
    if args.policy == "learned":
        w0 = next((w for w in warm if w["learn_ms"] > 0), None)
        learn = {"trained_before_timing": bool(warm[-1]["learn_trained"]) if warm else False,
                 "pairs": warm[-1]["learn_pairs"] if warm else 0,
                 "train_ms": w0["learn_ms"] if w0 else None, "loss": w0["learn_loss"] if w0 else None}

    clk_path = Path(tempfile.gettempdir()) / f"spray_bench_clocks_rank{rank}_{os.getpid()}.csv"
    proc, fh = clock_sampler(clk_path)
    barrier()
    torch.cuda.synchronize()
    stats = [frame_device() for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()

    rays = sum(s["rays_primary"] + s["rays_shadow"] + s["rays_bounce"] for s in stats)
    dev_ms = sum(s["frame_ms"] for s in stats)
    t_max = allmax(dev_ms)
    rays_all = allsum(rays)
    value = rays_all / (t_max * 1e-3) / 1e6

    # end to end through the C ABI: image to pinned host memory every frame
    host = torch.empty(npix * 4, dtype=torch.float32, pin_memory=True)
    host_np = host.numpy().reshape(npix, 1, 4) if views is not None else host.numpy().reshape(H, W, 4)
    e2e_rays, e2e_s, h2d, d2h = 0, 0.0, 0, 0
    barrier()
    for _ in range(args.steps):
        if not args.no_flush:
            flush.fill_(1)
            torch.cuda.synchronize()
        t0 = time.perf_counter()
        if views is not None:
            _, st = tracer.trace_views(views)
        else:
            _, st = tracer.trace(host_np)
        e2e_s += time.perf_counter() - t0
        e2e_rays += st["rays_primary"] + st["rays_shadow"] + st["rays_bounce"]
        h2d, d2h = st["h2d_bytes"], st["d2h_bytes"]
    barrier()
    e2e_value = allsum(e2e_rays) / allmax(e2e_s) / 1e6
    if proc is not None:
        proc.terminate()
        proc.wait()
        fh.close()
    clocks = clock_summary(clk_path, smi_index(local))
    tracer.close()
    del flush

    s0 = stats[-1]
    peak, peak_kind = hbm_peak()
    trace_bytes = (s0["visits_radiance"] * (RAY_BYTES + ENTRY_BYTES + HIT_BYTES)
                   + s0["nodes_radiance"] * NODE_BYTES + s0["tris_radiance"] * TRI_BYTES)
    occl_bytes = (s0["visits_shadow"] * (RAY_BYTES + ENTRY_BYTES)
                  + s0["nodes_shadow"] * NODE_BYTES + s0["tris_shadow"] * TRI_BYTES)
    if s0["trace_ms"] >= s0["occlude_ms"]:
        kname, kbytes, kms, klaunch = "closest-hit traversal", trace_bytes, s0["trace_ms"], s0["trace_launches"]
        kvisits = s0["visits_radiance"]
        kmin = kvisits * (RAY_BYTES + ENTRY_BYTES + HIT_BYTES)
    else:
        kname, kbytes, kms, klaunch = "occlusion traversal", occl_bytes, s0["occlude_ms"], s0["occlude_launches"]
        kvisits = s0["visits_shadow"]
        kmin = kvisits * (RAY_BYTES + ENTRY_BYTES)
    achieved = kbytes / (kms * 1e-3) / 1e9 if kms > 0 else 0.0
    prof = load_profile_traffic(args.config)
    traffic = None
    if prof and prof.get("kernel") == kname and "dram_bytes_per_algorithmic_byte" in prof:
        # ncu DRAM bytes of a small frame, scaled by the units processed
        traffic = prof["dram_bytes_per_algorithmic_byte"] * kbytes

    nrays = s0["rays_primary"] + s0["rays_shadow"] + s0["rays_bounce"]
    out = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": allmax(dev_ms / args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded wavelet isosurface scene, seeded orbit camera)",
        "config": bench_config(args.config, spec, cfg, scene, args.policy, tuned, world, views),
        "rays_per_frame": {"primary": s0["rays_primary"], "shadow": s0["rays_shadow"],
                           "bounce": s0["rays_bounce"]},
        "mrays_per_s_by_class": {k: s0[f"rays_{k}"] / (s0["frame_ms"] * 1e-3) / 1e6
                                 for k in ("primary", "shadow", "bounce")},
        "visits_per_ray": (s0["visits_radiance"] + s0["visits_shadow"]) / max(nrays, 1),
        "visits_culled": s0["visits_culled"],
        # primary rays (included in rays_per_frame) whose 16x16 screen bin no
        # domain box's projection touches: misses, resolved at generation
        "eyes_culled_per_frame": s0.get("eyes_culled", 0),
        "domain_loads_per_frame": s0["domain_loads"],
        "inplace_domains_per_frame": s0["inplace_domains"],
        "inplace_bytes_per_frame": s0["inplace_bytes"],
        "breakdown_ms_per_frame": {k: s0[f"{k}_ms"] for k in ("frame", "schedule", "trace", "occlude", "h2d")},
        "h2d_bytes_per_frame": s0["h2d_bytes"],
        "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
        "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        # The traversal is bound by latency and SIMT divergence, not by DRAM:
        # its node and triangle reads are served mostly by L1/L2.  `achieved`
        # is the algorithmic bytes the walk requested (its own node and
        # triangle counts) per second against the HBM copy peak;
        # `achieved_floor` counts only the bytes every visit must move (ray,
        # queue entry, hit record), a lower bound independent of the walk.
        "roofline": {"bound": "latency", "peak_kind": "hbm", "kernel": kname, "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                     "traffic": traffic, "algorithmic_bytes_per_frame": kbytes,
                     "achieved_floor": kmin / (kms * 1e-3) / 1e9 if kms > 0 else 0.0,
                     "frac_floor": (kmin / (kms * 1e-3) / 1e9) / peak if kms > 0 else 0.0,
                     "launches_per_frame": klaunch, "kernel_ms_per_frame": kms},
        "clocks": clocks,
    }
    if learn is not None:
        out["learn"] = learn
    if rank == 0 and not args.no_cpu_baseline and views is None:
        threads = os.cpu_count() or 1
        ocfg = dict(base_cfg)
        ocfg["schedule_policy"] = POLICIES[args.policy][0]
        r, dt, c, _, mode_a, o = cpu_speculative(scene, ocfg, threads, args.cpu_scale)
        out["cpu_baseline"] = {
            "value": r / dt / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{c['image_w']}x{c['image_h']} frame (1/{args.cpu_scale} per axis), same scene, "
                      f"camera, spp and bounces; speculative loop, {threads} OpenMP threads"}
        if args.accuracy:
            gcfg = dict(cfg)
            gcfg.update(image_w=c["image_w"], image_h=c["image_h"], graphs=0)
            out["accuracy"] = accuracy_report(scene, gcfg, cam, mode_a, o, local)
            tr = out["accuracy"]["closest_hit_traversal"]
            rl = out["roofline"]
            if rl["kernel"] == "closest-hit traversal" and tr["oracle_to_gpu_bytes"]:
                # the algorithmic bytes with node and triangle counts from the
                # oracle's ordered walk of the same hierarchies (measured on the
                # accuracy frame, scaled to this frame by the ratio of the walks)
                ob = rl["algorithmic_bytes_per_frame"] * tr["oracle_to_gpu_bytes"]
                ach = ob / (rl["kernel_ms_per_frame"] * 1e-3) / 1e9
                rl["oracle_counted"] = {"algorithmic_bytes_per_frame": ob, "achieved": ach,
                                        "frac": ach / rl["peak"], "ratio_to_kernel_counts": tr["oracle_to_gpu_bytes"],
                                        "sample": f"{c['image_w']}x{c['image_h']} frame of the same workload"}
        o.close()
    if rank == 0 and world == 1 and args.c3_schedulers and args.config == "c2":
        out["c3_schedulers"] = c3_schedulers_block(args, local)
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
