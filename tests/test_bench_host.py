"""Host-side logic of bench.py that needs no GPU: the nvidia-smi index of the
process's device and the clock summary of a sampled CSV."""
import importlib.util
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("visible,local,want", [
    ("", 0, 0), ("", 3, 3),            # no remapping: the local index
    ("3,5", 0, 3), ("3,5", 1, 5),      # remapped numeric ids
    ("GPU-1a2b", 0, 0),                # UUIDs cannot be mapped: the local index
    ("2", 1, 1),                       # more ranks than listed ids
])
def test_smi_index_follows_cuda_visible_devices(bench, monkeypatch, visible, local, want):
    monkeypatch.setenv("CUDA_VISIBLE_DEVICES", visible)
    assert bench.smi_index(local) == want


def test_clock_summary_reads_only_its_device(bench, tmp_path):
    # index, sm, max sm, power, active, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    rows = [
        "0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "1, 1200, 2070, 300.0, 0x4, Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 950.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 940.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    f = tmp_path / "clocks.csv"
    f.write_text("\n".join(rows) + "\n")
    c0 = bench.clock_summary(f, 0)
    assert c0["samples"] == 3 and c0["sm_mhz"] == 2070.0 and c0["sm_max_mhz"] == 2070.0
    assert c0["reasons"] == ["sw_power_cap"]
    c1 = bench.clock_summary(f, 1)
    assert c1["samples"] == 1 and c1["sm_mhz"] == 1200.0 and c1["reasons"] == ["hw_slowdown"]
    assert bench.clock_summary(f, 7) is None
    assert bench.clock_summary(tmp_path / "missing.csv", 0) is None


def test_both_arms_describe_the_same_workload(bench, lib_built):
    # the GPU arm loads the scene with the library, the reference arm with the
    # oracle's own reader; the `config` objects they print must be identical
    import spray_gb300 as sg
    from oracle import scene_io
    from spray_gb300 import autotune, scenes
    path = bench.scene_file("c2")
    t = autotune.load("c2", 0)
    tuned = dict(t["params"]) if t else None
    got = []
    for scene in (sg.Scene.load(path, path.parent), scene_io.load(path, path.parent)):
        spec, cfg = scenes.workload_config("c2", scene)
        got.append(bench.bench_config("c2", spec, cfg, scene, "plain", tuned, 1))
    want = got[0]
    assert got[1] == want
    assert want["image"] == [1920, 1080] and want["spp"] == 16 and want["bounces"] == 5
    assert want["domains"] == 64 and want["triangles"] > 1_000_000


def test_reference_arm_runs_without_the_cuda_library(tmp_path):
    # a child process runs the reference arm on a small frame and lists the
    # repository libraries it mapped: the oracle's, never libspray_gpu.so
    import subprocess
    import sys
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '0', '--ref-scale', '16'];\n"
            "runpy.run_path(%r, run_name='__main__')\n"
            "maps = open('/proc/self/maps').read()\n"
            "print('MAPPED', sorted({l.split()[-1] for l in maps.splitlines() if l.endswith('.so')}))"
            % str(ROOT / "bench.py"))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = next(l for l in r.stdout.splitlines() if l.startswith("{"))
    import json
    d = json.loads(line)
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    mapped = next(l for l in r.stdout.splitlines() if l.startswith("MAPPED"))
    assert "libspray_gpu.so" not in mapped and "liboracle.so" in mapped
