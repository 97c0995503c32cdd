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
