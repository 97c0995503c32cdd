"""Autotuner logic without a GPU: the frame timer is replaced by a model of the
frame time, the benchmark scene by a stub with the workload's domain count."""
import types

import pytest

import spray_gb300 as sg
from spray_gb300 import autotune, scenes


@pytest.fixture
def stubbed(monkeypatch, tmp_path):
    calls = []

    def fake_scene(name):
        return tmp_path / f"{name}.spray", None

    def fake_load(path, base):
        n = {"c2": 64, "c3": 512, "c5": 64}[path.stem]
        return types.SimpleNamespace(domains=[None] * n)

    def fake_frame_ms(scene, cfg, cam, frames, warmup, views=None):
        calls.append(dict(cfg=dict(cfg), frames=frames, warmup=warmup, views=views))
        # a frame-time model with its minimum at 6 CTAs per SM and 16 chunks per warp
        return (10.0 + abs(cfg["trace_blocks_per_sm"] - 6) + 0.5 * abs(cfg["sched_chunks_per_warp"] - 16)
                + (0.25 if cfg["wave_samples"] else 0.0))

    monkeypatch.setattr(scenes, "benchmark_scene", fake_scene)
    monkeypatch.setattr(sg.Scene, "load", staticmethod(fake_load))
    monkeypatch.setattr(scenes, "orbit_camera", lambda scene, frame=0: ((0, 0, 5), (0, 0, 0), (0, 1, 0), 60.0))
    monkeypatch.setattr(scenes, "c5_views", lambda scene, n, seed: [{"view": k, "seed": seed} for k in range(n)])
    monkeypatch.setattr(autotune, "_frame_ms", fake_frame_ms)
    return calls


def test_coordinate_descent_finds_the_model_minimum(stubbed):
    r = autotune.tune("c2", write=False)
    assert r["params"] == {"trace_blocks_per_sm": 6, "sched_chunks_per_warp": 16, "wave_samples": 0}
    assert r["frame_ms"] == 10.0 and r["default_frame_ms"] == 10.0 + 2 + 4
    assert len(r["trials"]) == len(stubbed)
    # in core: 3 timed frames after 2 warm-up frames, one view
    assert all(c["frames"] == 3 and c["warmup"] == 2 and c["views"] is None for c in stubbed)


def test_out_of_core_trials_are_longer_and_search_the_cache_knobs(stubbed):
    r = autotune.tune("c3", policy=2, write=False)
    assert r["policy"] == 2 and "ooc_batch" in r["params"] and "ooc_inplace" in r["params"]
    assert all(c["frames"] == 10 and c["warmup"] == 5 for c in stubbed)
    assert {c["cfg"]["ooc_inplace"] for c in stubbed} >= set(autotune.OOC_SPACE["ooc_inplace"])


def test_multi_view_workload_times_its_view_batch(stubbed):
    autotune.tune("c5", write=False)
    spec = scenes.CONFIGS["c5"]
    assert all(c["views"] is not None and len(c["views"]) == spec["views"] for c in stubbed)
    assert all(c["views"][0]["seed"] == spec["view_seed"] for c in stubbed)
