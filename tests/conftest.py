import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


@pytest.fixture(scope="session")
def lib_built():
    from spray_gb300 import build as B
    B.build()
    import spray_gb300 as sg
    return sg.lib()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle as O
    O.build()
    return O


def small_config(**kw):
    cfg = dict(image_w=64, image_h=48, ao_mode=1, ao_samples=4, pixel_samples=1, bounces=1,
               fov=60.0, cache_size=-1, max_samples_per_rank=1 << 20, list_size=16, history_size=4,
               num_ranks=1, rank=0)
    cfg.update(kw)
    return cfg
