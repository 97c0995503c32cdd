"""Eye culling by the screen bins: the samples of pixels whose 16x16 bin no domain box's projection touches stop at generation
(no domain list is possible for them) and never enter the alive list.

The debug capture keeps every sample alive, so the same frame traced with and
without it must give the bit-identical image and the same ray counts, for one
view and for a multi-view batch (each view has its own bins); the
culled samples must be among those the capture shows without any queue entry;
and the culled frame must equal the oracle's wavefront image bit for bit."""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config

pytestmark = pytest.mark.gpu

RAYS = ("rays_primary", "rays_shadow", "rays_bounce")


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _frame(sc, cfg, cam, **kw):
    t = sg.Tracer(cfg, **kw)
    t.set_scene(sc)
    t.set_camera(*cam)
    img, st = t.trace()
    return t, img, st


@pytest.mark.parametrize("mode,spp,waves", [("pt", 2, 0), ("ao", 1, 0), ("pt", 3, 2500)])
def test_culled_eyes_keep_the_image_and_the_counts(lib_built, oracle_mod, mode, spp, waves):
    sc = scenes.wavelet_grid(3, 16, colors="albedo", light="point+diffuse" if mode == "pt" else "point")
    cfg = small_config(image_w=176, image_h=128, ao_mode=int(mode == "ao"), ao_samples=2, pixel_samples=spp,
                       bounces=3 if mode == "pt" else 1, max_samples_per_rank=4096)
    pos, look, up = scenes.orbit_camera(sc)
    pos = look + 1.6 * (pos - look)  # farther out: the grid leaves empty bins around it
    cam = (pos, look, up)
    kw = dict(wave_samples=waves) if waves else {}
    t, img, st = _frame(sc, cfg, cam, **kw)
    t.close()
    tc, imgc, stc = _frame(sc, cfg, cam, debug_capture=1, **kw)
    npix = cfg["image_w"] * cfg["image_h"]
    assert stc["eyes_culled"] == 0
    assert 0 < st["eyes_culled"] < npix * spp
    assert st["eyes_culled"] % spp == 0  # whole pixels
    assert np.array_equal(bits(img), bits(imgc))
    for k in RAYS:
        assert st[k] == stc[k], k
    # culled samples have no depth-0 entry in the full (capture) frame
    q = tc.debug(sg.DBG_RQUEUES, 0)
    listed = np.unique(q["ray"]).size
    assert st["eyes_culled"] <= npix * spp - listed
    tc.close()
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*cam)
    want, ws = o.render_wavefront()
    assert np.array_equal(bits(img), bits(want))
    for k in RAYS:
        assert st[k] == ws[k], k
    o.close()


def test_culled_eyes_in_a_multi_view_batch(lib_built):
    # each view has its own bins; the batch equals the same views traced with
    # every sample alive (debug capture), view by view and bit for bit
    sc = scenes.wavelet_grid(3, 14, colors="albedo", light="point+diffuse")
    views = []
    for k, (w, h, spp, ao) in enumerate([(96, 64, 2, 0), (64, 64, 1, 1), (128, 80, 3, 0)]):
        pos, look, up = scenes.orbit_camera(sc, frame=k)
        views.append(dict(position=look + 1.5 * (pos - look), lookat=look, up=up, vfov=60.0, image_w=w,
                          image_h=h, pixel_samples=spp, ao_mode=ao, bounces=1 if ao else 3, ao_samples=2))
    out = []
    for kw in ({}, dict(debug_capture=1)):
        t = sg.Tracer(small_config(max_samples_per_rank=4096), **kw)
        t.set_scene(sc)
        out.append(t.trace_views(views))
        t.close()
    (imgs, st), (imgs_c, st_c) = out
    assert st_c["eyes_culled"] == 0 and st["eyes_culled"] > 0
    for a, b in zip(imgs, imgs_c):
        assert np.array_equal(bits(a), bits(b))
    for k in RAYS:
        assert st[k] == st_c[k], k
