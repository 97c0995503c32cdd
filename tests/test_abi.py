"""The C-ABI library loads and exports every entry point include/*.h declares."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(spray_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "spray_gpu_create" in names and "spray_gpu_trace" in names
    assert len(names) >= 15


def test_library_exports_every_declared_symbol(lib_built):
    missing = [n for n in declared_functions() if not hasattr(lib_built, n)]
    assert not missing, missing


def test_config_defaults_match_reference(lib_built):
    import spray_gb300 as sg
    d = sg.default_config()
    # Config::Config() (src/render/config.cc:33-73)
    assert d["image_w"] == 400 and d["image_h"] == 400
    assert d["ao_samples"] == 8 and d["pixel_samples"] == 4 and d["bounces"] == 1
    assert d["fov"] == 90.0 and d["cache_size"] == -1 and d["ao_mode"] == 0
    assert d["max_samples_per_rank"] == 1024 * 1024
    assert d["list_size"] == 16 and d["history_size"] == 4


def test_errors_without_gpu_are_reported(lib_built):
    """With no GPU, creating a tracer fails with a CUDA error code and a message."""
    import spray_gb300 as sg
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        pytest.skip("GPU present")
    with pytest.raises(sg.SprayError) as e:
        sg.Tracer(image_w=8, image_h=8)
    assert e.value.code == sg.ECUDA


def test_invalid_config_rejected(lib_built):
    import spray_gb300 as sg
    with pytest.raises(sg.SprayError) as e:
        sg.Tracer(image_w=0, image_h=8)
    assert e.value.code in (sg.EINVAL, sg.ECUDA)


@pytest.mark.parametrize("kw", [dict(schedule_policy=6), dict(schedule_policy=-1), dict(ooc_batch=-1),
                                dict(schedule_policy=5, num_ranks=2, rank=0),
                                dict(schedule_policy=3, learn_batch=0), dict(schedule_policy=3, learn_lr=0.0),
                                dict(schedule_policy=3, learn_frames=0), dict(ooc_inplace=-1),
                                dict(trace_blocks_per_sm=33), dict(sched_chunks_per_warp=-1),
                                dict(bucket_launches=2)])
def test_out_of_core_options_validated(lib_built, kw):
    """Options are checked before any device is touched."""
    import spray_gb300 as sg
    with pytest.raises(sg.SprayError) as e:
        sg.Tracer(image_w=8, image_h=8, **kw)
    assert e.value.code == sg.EINVAL
