"""The CUDA path against the oracle at the benchmarked workloads' settings.

The other parity tests use small scenes; these run each benchmark workload's
own scene and render settings on a reduced image (the scene, spp, bounces,
lights, AO range, Russian roulette, list size and cache are the workload's):

  C2  64 domains (64^3 isosurfaces), quad light, 16 spp, 5 bounces, Russian
      roulette from bounce 3, the committed launch tuning
  C1  the same grid in grey, AO with 8 rays, range 5 % of the diagonal, the
      light ray, 1 spp
  C3  512 domains (128^3 phase-shifted isosurfaces), list size 22, 8 spp,
      4 bounces; in core, and out of core with the 256-domain cache under
      every scheduling policy

Each compares the GPU image with the oracle's wavefront restatement (mode B)
bit for bit, with the restated reference loop (mode A) at image RMSE <= 1e-3,
and every depth's closest hits and occlusion flags with the oracle's
(>= 99.99 % agreement, hit t within 1e-5 relative).
"""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import autotune, scenes
from oracle import accuracy as A

pytestmark = pytest.mark.gpu


def _oracle_cfg(cfg):
    c = dict(cfg)
    for k, v in dict(history_size=4, list_size=16, cache_size=-1, max_samples_per_rank=1 << 20,
                     num_ranks=1, rank=0).items():
        c.setdefault(k, v)
    return c


def _workload(name, w, h, **over):
    path, spec = scenes.benchmark_scene(name)
    scene = sg.Scene.load(path, path.parent)
    _, cfg = scenes.workload_config(name, scene)
    cfg.update(image_w=w, image_h=h, **over)
    return scene, _oracle_cfg(cfg)


def _check_frame(scene, cfg, oracle_mod, gpu_extra=None, threads=8):
    cam = scenes.orbit_camera(scene)
    t = sg.Tracer(dict(cfg, debug_capture=1, **(gpu_extra or {})))
    t.set_scene(scene)
    t.set_camera(*cam)
    img, st = t.trace()
    o = oracle_mod.Oracle(cfg, scene)
    o.set_camera(*cam)
    wb, sb = o.render_wavefront()
    assert A.bit_exact(img, wb), float(np.abs(img - wb).max())
    assert st["rays_shadow"] == sb["rays_shadow"] and st["rays_bounce"] == sb["rays_bounce"]
    wa, _ = o.render_speculative(threads)
    rmse = A.image_rmse(img, wa)
    assert rmse <= A.IMG_RMSE, rmse
    nhit = 0
    for b in range(cfg["bounces"]):
        rays = t.debug(sg.DBG_RAYS, b)
        if len(rays) == 0:
            break
        h = t.debug(sg.DBG_HITS, b)
        ha = A.hit_agreement(rays, h, o)
        assert ha["agree"] >= A.HIT_AGREE, (b, ha)
        assert ha["t_max_rel_err"] <= A.T_RTOL, (b, ha)
        nhit += ha["hits"]
        sa = A.shadow_agreement(t.debug(sg.DBG_SHADOWS, b), h, o)
        assert sa["agree"] >= A.HIT_AGREE, (b, sa)
    assert nhit > 1000 and img[..., :3].max() > 0
    t.close()
    return img, st, o


def test_c2_settings_match_the_oracle(lib_built, oracle_mod):
    scene, cfg = _workload("c2", 160, 90)
    tuned = autotune.load("c2", 0)
    img, st, o = _check_frame(scene, cfg, oracle_mod, dict(tuned["params"]) if tuned else None)
    assert cfg["pixel_samples"] == 16 and cfg["bounces"] == 5 and cfg["rr_depth"] == 3
    assert scene.lights[0].type == sg.Light.QUAD and st["rays_bounce"] > 0


def test_c1_settings_match_the_oracle(lib_built, oracle_mod):
    scene, cfg = _workload("c1", 256, 256)
    assert cfg["ao_samples"] == 8 and cfg["ao_light_shadow"] == 1 and cfg["ao_max_distance"] > 0
    img, st, o = _check_frame(scene, cfg, oracle_mod)
    assert st["rays_shadow"] > 8 * 0.1 * st["rays_primary"]


@pytest.fixture(scope="module")
def c3_small():
    scene, cfg = _workload("c3", 128, 128)
    assert len(scene.domains) == 512 and cfg["list_size"] == 22 and cfg["cache_size"] == 256
    return scene, cfg


def test_c3_settings_match_the_oracle_in_core(lib_built, oracle_mod, c3_small):
    scene, cfg = c3_small
    incore = dict(cfg, cache_size=-1)
    img, st, o = _check_frame(scene, incore, oracle_mod)
    assert st["list_overflows"] == 0


@pytest.mark.parametrize("policy", [0, 2, 3, 4])
def test_c3_out_of_core_policies_render_the_in_core_image(lib_built, oracle_mod, c3_small, policy):
    scene, cfg = c3_small
    cam = scenes.orbit_camera(scene)
    o = oracle_mod.Oracle(dict(cfg, cache_size=-1), scene)
    o.set_camera(*cam)
    wb, _ = o.render_wavefront()
    t = sg.Tracer(dict(cfg, schedule_policy=policy, learn_frames=1))
    t.set_scene(scene)
    t.set_camera(*cam)
    for frame in range(2):  # the learned order is trained after the first frame
        img, st = t.trace()
        assert A.bit_exact(img, wb), (policy, frame, float(np.abs(img - wb).max()))
        assert st["cache_slots"] == 256 and st["cache_slot_bytes"] > 0
        assert st["domain_loads"] + st["inplace_domains"] > 0
        assert st["h2d_bytes"] >= st["domain_loads"] * 1  # every load copies its domain
        if st["inplace_domains"] > 0:
            assert st["inplace_bytes"] > 0
    t.close()
