"""The allocation-free scheduling entry point against the regular one.

spray_gpu_schedule_static serves callers that cannot allocate device memory
while they run (a renderer with a fixed device budget reserved at start-up, a
runtime that hands out GPU memory from its own pool): its scratch is one
static device array.  Its queues must equal, entry for entry, the queues the regular
path (spray_gpu_trace, read back through spray_gpu_debug_copy) builds from the
same rays -- on two calls in a row, since calls share and reuse the scratch.
This file is collected last so that a failure here does not hide the others.
"""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config

pytestmark = pytest.mark.gpu


def test_static_scratch_schedule_matches_regular_path(lib_built):
    torch = pytest.importorskip("torch")
    scene = scenes.wavelet_grid(2, 24, colors="albedo", light="point")
    cfg = small_config(image_w=96, image_h=64, cull=0, debug_capture=1)
    t = sg.Tracer(cfg)
    t.set_scene(scene)
    t.set_camera(*scenes.orbit_camera(scene))
    t.trace()
    rays = t.debug(sg.DBG_RAYS, 0)
    want = t.debug(sg.DBG_RQUEUES, 0)
    n, D = len(rays), len(scene.domains)
    assert np.array_equal(rays["sample"], np.arange(n)) and len(want) > 0

    dev = torch.device("cuda:0")
    org = torch.zeros((n, 4), dtype=torch.float32)
    dr = torch.zeros((n, 4), dtype=torch.float32)
    org[:, :3] = torch.from_numpy(np.ascontiguousarray(rays["org"]))
    dr[:, :3] = torch.from_numpy(np.ascontiguousarray(rays["dir"]))
    org, dr = org.to(dev), dr.to(dev)
    bounds = torch.from_numpy(np.stack([d.bounds for d in scene.domains]).astype(np.float32)).to(dev)
    cap = 4 * len(want) + 64
    entries = torch.zeros((cap, 2), dtype=torch.int32, device=dev)
    starts = torch.zeros(D + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    for call in range(2):
        entries.fill_(-1)
        starts.fill_(-1)
        torch.cuda.synchronize()
        k = sg.schedule_static(bounds.data_ptr(), D, org.data_ptr(), dr.data_ptr(), n, cfg["list_size"],
                               entries.data_ptr(), cap, starts.data_ptr())
        assert k == len(want), (call, k, len(want))
        e = entries[:k].cpu().numpy().view(np.uint32)
        ks = starts.cpu().numpy().astype(np.int64)
        assert ks[0] == 0 and ks[-1] == k and np.all(np.diff(ks) >= 0)
        dom = np.repeat(np.arange(D), np.diff(ks))
        assert np.array_equal(dom, want["domain"])
        assert np.array_equal(e[:, 0] & ((1 << 26) - 1), want["ray"])
        assert np.array_equal((e[:, 0] >> 26) & 31, want["depth"])
        assert np.array_equal(e[:, 1], want["tdom"].view(np.uint32))


def test_static_scratch_rejects_oversize_requests(lib_built):
    with pytest.raises(sg.SprayError) as e:
        sg.schedule_static(16, 257, 16, 16, 1, 16, 16, 1, 16)
    assert e.value.code == sg.EINVAL and "num_domains" in str(e.value)
    with pytest.raises(sg.SprayError) as e:
        sg.schedule_static(16, 8, 16, 16, (1 << 18) + 1, 16, 16, 1, 16)
    assert e.value.code == sg.EINVAL and "num_rays" in str(e.value)


def _device_rays(torch, n):
    dev = torch.device("cuda:0")
    return (torch.zeros((max(n, 1), 4), dtype=torch.float32, device=dev),
            torch.zeros((max(n, 1), 4), dtype=torch.float32, device=dev))


def test_static_scratch_reports_small_entry_capacity(lib_built):
    # the device detects that the queues need more entries than the caller's
    # output holds; the scatter never writes past entry_capacity
    torch = pytest.importorskip("torch")
    scene = scenes.wavelet_grid(2, 24, colors="albedo", light="point")
    cfg = small_config(image_w=48, image_h=32, cull=0, debug_capture=1)
    t = sg.Tracer(cfg)
    t.set_scene(scene)
    t.set_camera(*scenes.orbit_camera(scene))
    t.trace()
    rays = t.debug(sg.DBG_RAYS, 0)
    want = t.debug(sg.DBG_RQUEUES, 0)
    n, D = len(rays), len(scene.domains)
    dev = torch.device("cuda:0")
    org, dr = _device_rays(torch, n)
    org[:, :3] = torch.from_numpy(np.ascontiguousarray(rays["org"])).to(dev)
    dr[:, :3] = torch.from_numpy(np.ascontiguousarray(rays["dir"])).to(dev)
    bounds = torch.from_numpy(np.stack([d.bounds for d in scene.domains]).astype(np.float32)).to(dev)
    cap = len(want) - 1
    entries = torch.full((cap + 1, 2), -7, dtype=torch.int32, device=dev)
    starts = torch.zeros(D + 1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    with pytest.raises(sg.SprayError) as e:
        sg.schedule_static(bounds.data_ptr(), D, org.data_ptr(), dr.data_ptr(), n, cfg["list_size"],
                           entries.data_ptr(), cap, starts.data_ptr())
    assert e.value.code == sg.EOVERFLOW and "entry_capacity" in str(e.value)
    # the guard row past the capacity is untouched
    assert entries[cap].cpu().tolist() == [-7, -7]
    # and the scratch is usable again afterwards with a large enough output
    entries = torch.zeros((len(want), 2), dtype=torch.int32, device=dev)
    k = sg.schedule_static(bounds.data_ptr(), D, org.data_ptr(), dr.data_ptr(), n, cfg["list_size"],
                           entries.data_ptr(), len(want), starts.data_ptr())
    assert k == len(want)


def test_static_scratch_zero_rays(lib_built):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    D = 8
    bounds = torch.zeros((D, 6), dtype=torch.float32, device=dev)
    bounds[:, 3:] = 1.0
    org, dr = _device_rays(torch, 0)
    entries = torch.zeros((4, 2), dtype=torch.int32, device=dev)
    starts = torch.full((D + 1,), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    for _ in range(2):
        k = sg.schedule_static(bounds.data_ptr(), D, org.data_ptr(), dr.data_ptr(), 0, 16,
                               entries.data_ptr(), 4, starts.data_ptr())
        assert k == 0
        assert np.array_equal(starts.cpu().numpy(), np.zeros(D + 1, np.int32))


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_static_schedule_matches_the_oracle_on_degenerate_inputs(lib_built, oracle_mod, seed):
    # boxes that overlap, touch, are flat in one or two axes or are points;
    # rays with zero direction components (infinite inverse), starting inside
    # boxes, on their faces and on shared faces: the slab tests, the (t, id)
    # order and the queue positions must equal the oracle's bit for bit
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(seed)
    D = 48
    lo = np.round(rng.uniform(-4, 4, (D, 3)) * 2) / 2
    ext = np.round(rng.uniform(0, 3, (D, 3)) * 2) / 2
    ext[rng.random((D, 3)) < 0.15] = 0.0  # flat sides, some boxes points
    lo[D // 2:D // 2 + 4] = lo[0]          # identical boxes
    ext[D // 2:D // 2 + 4] = ext[0]
    bounds = np.concatenate([lo, lo + ext], 1).astype(np.float32)
    n = 20000
    org = rng.uniform(-5, 5, (n, 3)).astype(np.float32)
    pick = rng.integers(0, D, n)
    face = rng.random(n) < 0.3               # start on a box's face or corner
    org[face] = np.where(rng.random((face.sum(), 3)) < 0.5, bounds[pick[face], :3], bounds[pick[face], 3:])
    inside = rng.random(n) < 0.2
    org[inside] = (bounds[pick[inside], :3] + bounds[pick[inside], 3:]) * 0.5
    dr = rng.normal(size=(n, 3)).astype(np.float32)
    dr[rng.random((n, 3)) < 0.2] = 0.0       # axis-parallel rays
    dr[np.all(dr == 0, 1)] = (1, 0, 0)
    dr = (dr / np.linalg.norm(dr, axis=1, keepdims=True)).astype(np.float32)
    # the oracle's queues: one Oracle with these boxes as its domains
    doms = [sg.Domain(np.array([b[:3], b[3:], b[:3]], np.float32), np.array([[0, 1, 2]], np.uint32),
                      bounds=b) for b in bounds]
    o = oracle_mod.Oracle(small_config(), sg.Scene(doms, [sg.Light(0, (0, 0, 9))]))
    want, _ = o.schedule(org, dr)
    o.close()
    order = np.lexsort((want["depth"], want["ray"], want["domain"]))  # queue order: domain, then ray
    want = want[order]
    dev = torch.device("cuda:0")
    to4 = lambda a: torch.from_numpy(np.concatenate([a, np.zeros((len(a), 1), np.float32)], 1)).to(dev)
    bnd = torch.from_numpy(bounds).to(dev)
    cap = len(want) + 64
    entries = torch.zeros((cap, 2), dtype=torch.int32, device=dev)
    starts = torch.zeros(D + 1, dtype=torch.int32, device=dev)
    o4, d4 = to4(org), to4(dr)  # kept alive: the call takes raw device pointers
    torch.cuda.synchronize()
    k = sg.schedule_static(bnd.data_ptr(), D, o4.data_ptr(), d4.data_ptr(), n, 16,
                           entries.data_ptr(), cap, starts.data_ptr())
    assert k == len(want) and k > n // 4
    e = entries[:k].cpu().numpy().view(np.uint32)
    ks = starts.cpu().numpy().astype(np.int64)
    dom = np.repeat(np.arange(D), np.diff(ks))
    assert np.array_equal(dom, want["domain"])
    assert np.array_equal(e[:, 0] & ((1 << 26) - 1), want["ray"])
    assert np.array_equal((e[:, 0] >> 26) & 31, want["depth"])
    assert np.array_equal(e[:, 1], want["tdom"].view(np.uint32))
