"""The non-speculative round loop on the GPU (schedule_policy 5) against the
oracle's restatement of the same loop (mode C): the reference's baseline
image tracer (src/baseline/baseline_image_tracer.inl:28-131) with
LoadAnyOnceImageSched (baseline_schedulers.cc:43-62).

The GPU runs each round's rays in parallel and the oracle one by one, but
what a round queues depends only on each ray's own state, so the two must
agree exactly on the sequence of rounds (the domain of every round, from the
load log), the cache loads, the closest-hit, occlusion and shading-only
visits and the rays spawned; the images agree up to the order of the
additions per pixel."""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config
from oracle import accuracy as A

pytestmark = pytest.mark.gpu

ORDER_RMSE = 1e-6
COUNTS = ("rays_primary", "rays_shadow", "rays_bounce", "visits_radiance", "visits_shadow", "visits_shade",
          "rounds")


def _compare(oracle_mod, sc, cfg, frames=1, rel=None):
    cam = scenes.orbit_camera(sc)
    t = sg.Tracer(dict(cfg, schedule_policy=5))
    t.set_scene(sc)
    t.set_camera(*cam)
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*cam)
    want, ws, sched = o.render_baseline()
    for frame in range(frames):
        img, st = t.trace()
        log = t.debug(sg.DBG_LOADS, 0)
        assert np.array_equal(log["domain"], sched), frame
        assert np.array_equal(log["pass"], np.arange(1, len(sched) + 1))
        for k in COUNTS:
            assert st[k] == ws[k], (frame, k, st[k], ws[k])
        if rel is None:
            assert A.image_rmse(img, want) <= ORDER_RMSE, (frame, A.image_rmse(img, want))
        else:  # unbounded radiance (delta BSDFs): relative to the pixel
            assert np.all(np.abs(img - want) <= rel * np.maximum(np.abs(want), 1.0)), frame
        if cfg["cache_size"] > 0 and frame == 0:
            # a cold cache: the loads of the oracle's LRU over the same rounds
            assert st["domain_loads"] == ws["domain_loads"] == int(np.sum(log["outcome"] == 0))
    t.close()
    return st, ws


@pytest.mark.parametrize("mode,spp,cache", [("pt", 1, -1), ("pt", 2, 8), ("ao", 1, 8), ("ao", 2, -1),
                                            ("pt", 3, 5), ("pt", 1, 1)])
def test_rounds_match_the_oracle_loop(lib_built, oracle_mod, mode, spp, cache):
    sc = scenes.wavelet_grid(3, 16, colors="albedo", light="point+diffuse" if mode == "pt" else "point")
    cfg = small_config(image_w=48, image_h=36, ao_mode=int(mode == "ao"), ao_samples=2, pixel_samples=spp,
                       bounces=1 if mode == "ao" else 3, cache_size=cache)
    st, ws = _compare(oracle_mod, sc, cfg, frames=2)
    assert st["rounds"] > len(sc.domains) // 2 and st["visits_radiance"] > 0


def test_rounds_send_rays_back_to_shade(lib_built, oracle_mod):
    # two copies of a grid, the second shifted by a quarter of the scene:
    # overlapping domains, so rays move on past a hit and come back to shade
    sc = scenes.wavelet_grid(2, 14, colors="albedo", light="point")
    lo, hi = scenes.scene_box(sc)
    shift = ((np.asarray(hi) - np.asarray(lo)) * 0.25).astype(np.float32)
    doms = list(sc.domains) + [sg.Domain(d.vertices + shift, d.faces, d.colors) for d in sc.domains]
    sc2 = sg.Scene(doms, sc.lights)
    cfg = small_config(image_w=40, image_h=30, ao_mode=0, pixel_samples=1, bounces=2, cache_size=3)
    st, ws = _compare(oracle_mod, sc2, cfg)
    assert st["visits_shade"] > 0


def test_rounds_on_the_out_of_core_workload(lib_built, oracle_mod):
    # C3's 512 domains, list size 22, 8 spp, 4 bounces, the 256-domain cache
    path, _ = scenes.benchmark_scene("c3")
    sc = sg.Scene.load(path, path.parent)
    _, c3 = scenes.workload_config("c3", sc)
    cfg = dict(c3, image_w=48, image_h=48)
    for k, v in dict(history_size=4, max_samples_per_rank=1 << 20, num_ranks=1, rank=0).items():
        cfg.setdefault(k, v)
    assert cfg["cache_size"] == 256 and len(sc.domains) == 512
    st, ws = _compare(oracle_mod, sc, cfg)
    assert st["domain_loads"] > 0 and st["rounds"] >= st["domain_loads"]
    print(f"C3 48x48 rounds {st['rounds']}, loads {st['domain_loads']}, "
          f"visits/ray {st['visits_radiance'] / max(1, st['rays_primary'] + st['rays_bounce']):.3f}")


def test_rounds_with_delta_bsdfs(lib_built, oracle_mod):
    # mirror, glass and transmission domains: bounce rays leave the hit's
    # domain on delta paths (weights up to 1e5 at grazing angles)
    sc = scenes.wavelet_grid(2, 24, colors="albedo", light="point+diffuse")
    params = {1: (1, 1, 1), 2: (1.0, 1.5, 0.0), 3: (1.0, 1.33, 0.0)}
    for i, d in enumerate(sc.domains):
        d.bsdf_type = i % 4
        d.bsdf_params = np.asarray(params.get(i % 4, (1, 1, 1)), np.float32)
    cfg = small_config(image_w=48, image_h=36, ao_mode=0, ao_samples=2, pixel_samples=2, bounces=4,
                       cache_size=5)
    _compare(oracle_mod, sc, cfg, rel=1e-6)


def test_rounds_with_the_ao_workload_settings(lib_built, oracle_mod):
    # C1's AO: 8 rays within 5 % of the diagonal, plus the light's shadow ray
    path, _ = scenes.benchmark_scene("c1")
    sc = sg.Scene.load(path, path.parent)
    _, c1 = scenes.workload_config("c1", sc)
    cfg = dict(c1, image_w=64, image_h=48, cache_size=24)
    for k, v in dict(history_size=4, list_size=16, max_samples_per_rank=1 << 20, num_ranks=1, rank=0).items():
        cfg.setdefault(k, v)
    assert cfg["ao_samples"] == 8 and cfg["ao_light_shadow"] == 1 and cfg["ao_max_distance"] > 0
    st, ws = _compare(oracle_mod, sc, cfg)
    assert st["domain_loads"] > 0


def test_rounds_reject_several_views(lib_built):
    sc = scenes.wavelet_grid(2, 12, colors="albedo", light="point")
    t = sg.Tracer(small_config(schedule_policy=5))
    t.set_scene(sc)
    views = []
    for k in range(2):
        pos, look, up = scenes.orbit_camera(sc, frame=k)
        views.append(dict(position=pos, lookat=look, up=up, vfov=60.0))
    with pytest.raises(sg.SprayError) as e:
        t.trace_views(views)
    assert e.value.code == sg.EINVAL
    t.close()


def test_rounds_when_every_ray_misses(lib_built):
    sc = scenes.wavelet_grid(2, 12, colors="albedo", light="point")
    t = sg.Tracer(small_config(image_w=32, image_h=16, schedule_policy=5))
    t.set_scene(sc)
    t.set_camera((0, 0, 50), (0, 0, 100), (0, 1, 0))  # looking away from the grid
    img, st = t.trace()
    assert not img.any() and st["rounds"] == 0 and st["visits_radiance"] == 0
    assert len(t.debug(sg.DBG_LOADS, 0)) == 0
    t.close()


def test_rounds_on_one_domain(lib_built, oracle_mod):
    # one domain: every list holds it alone (no domain hierarchy), and a ray
    # spawned on its surface may start outside its box
    v = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0], [0, 0, 1]], np.float32)
    f = np.array([[0, 1, 2], [0, 1, 3], [1, 2, 3], [2, 0, 3]], np.uint32)
    sc = sg.Scene([sg.Domain(v, f, np.full(4, 0x80a0c0, np.uint32))], [sg.Light(0, (0, 0, 5))])
    cfg = small_config(image_w=37, image_h=23, ao_mode=0, pixel_samples=3, bounces=3)
    cam = ((0.1, 0.2, 3), (0, 0, 0), (0, 1, 0))
    t = sg.Tracer(dict(cfg, schedule_policy=5))
    t.set_scene(sc)
    t.set_camera(*cam)
    img, st = t.trace()
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*cam)
    want, ws, sched = o.render_baseline()
    for k in COUNTS:
        assert st[k] == ws[k], (k, st[k], ws[k])
    assert A.image_rmse(img, want) <= ORDER_RMSE and img[..., :3].max() > 0
    t.close()
