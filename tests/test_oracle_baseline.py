"""Oracle mode C, the reference's non-speculative image tracer
(src/baseline/baseline_image_tracer.inl:28-131 with LoadAnyOnceImageSched,
baseline_schedulers.cc:43-62), against the oracle's other two modes.

Mode C shades the same hits with the same sample streams as the speculative
loop (mode A) and the wavefront (mode B).  Its image differs from theirs in
the order of the floating-point additions per pixel and where the reference
loop itself loses a ray: a bounce ray first runs in the domain that spawned
it (temp_q, baseline_insitu_tracer.inl:620-635), at list position 0 even
when its list starts with another domain, so a ray whose origin rounds to
just outside the spawning domain's box and whose list holds one other
domain ends there without visiting it.  Its scheduler is pinned to the
reference's compiled scheduleImage by the golden vectors (tests/golden, group
load_any_once)."""
import numpy as np
import pytest

from oracle import accuracy as A
from spray_gb300 import scenes
from conftest import small_config

# per-pixel sums in another order: a few ulp of the pixel values
ORDER_RMSE = 1e-6


def _render(oracle_mod, sc, cfg):
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*scenes.orbit_camera(sc))
    ia, sa = o.render_speculative(1)
    ib, sb = o.render_wavefront()
    ic, stc, sched = o.render_baseline()
    return (ia, sa), (ib, sb), (ic, stc, sched)


@pytest.mark.parametrize("mode,spp,cache", [("pt", 1, -1), ("pt", 2, 8), ("ao", 1, 8), ("ao", 2, -1)])
def test_baseline_loop_renders_the_speculative_image(oracle_mod, mode, spp, cache):
    sc = scenes.wavelet_grid(3, 16, colors="albedo", light="point+diffuse" if mode == "pt" else "point")
    cfg = small_config(image_w=48, image_h=36, ao_mode=int(mode == "ao"), ao_samples=2, pixel_samples=spp,
                       bounces=1 if mode == "ao" else 3, cache_size=cache)
    (ia, sa), (ib, sb), (ic, stc, sched) = _render(oracle_mod, sc, cfg)
    assert ic[..., :3].max() > 0
    assert stc["rays_primary"] == sb["rays_primary"]
    # bounce rays the reference loop loses (never more than it spawns)
    lost = sb["rays_bounce"] - stc["rays_bounce"]
    assert 0 <= lost <= 0.01 * sb["rays_bounce"]
    # a lost ray changes its own pixel only; elsewhere the images differ in
    # the order of additions
    bad = np.abs(ic - ib)[..., :3].max(-1) > 1e-5 * np.maximum(1.0, np.abs(ib)[..., :3].max(-1))
    assert bad.sum() <= lost
    assert A.image_rmse(np.where(bad[..., None], ib, ic), ib) <= ORDER_RMSE
    assert A.image_rmse(np.where(bad[..., None], ia, ic), ia) <= ORDER_RMSE
    if lost == 0:
        # the same rays: every occlusion test of the wavefront is made once
        # (the shading domain first, then the list in order until an occluder)
        assert stc["rays_shadow"] == sb["rays_shadow"]
        assert stc["visits_shadow"] == sb["visits_shadow"]
    # a radiance ray stops at the first domain whose hit no later domain can
    # beat; the wavefront walks every domain of the list
    assert 0 < stc["visits_radiance"] <= sb["visits_radiance"]
    # one domain per round; every round's domain held queued rays
    assert stc["rounds"] == len(sched) and len(sched) >= len(set(sched.tolist()))
    hits = oracle_mod.lru_trace(len(sc.domains), cache, sched)
    assert stc["domain_loads"] == int(np.sum(hits == 0))
    if cache < 0:
        assert stc["domain_loads"] == len(set(sched.tolist()))


def test_baseline_loop_sends_rays_back_to_shade(oracle_mod):
    # overlapping domains: two copies of a grid, the second shifted by half a
    # cell, so that a ray often finds a hit in one domain that a later,
    # overlapping domain could still beat; the ray then moves on and, when the
    # later domain holds no nearer hit, returns to the first for shading
    sc = scenes.wavelet_grid(2, 14, colors="albedo", light="point")
    import spray_gb300 as sg
    lo, hi = scenes.scene_box(sc)
    shift = (np.asarray(hi) - np.asarray(lo)) * 0.25
    doms = list(sc.domains) + [sg.Domain(d.vertices + shift.astype(np.float32), d.faces, d.colors)
                               for d in sc.domains]
    sc2 = sg.Scene(doms, sc.lights)
    cfg = small_config(image_w=40, image_h=30, ao_mode=0, pixel_samples=1, bounces=2, cache_size=-1)
    (ia, sa), (ib, sb), (ic, stc, sched) = _render(oracle_mod, sc2, cfg)
    assert stc["visits_shade"] > 0
    assert A.image_rmse(ic, ib) <= A.IMG_RMSE
    assert stc["rays_shadow"] > 0
