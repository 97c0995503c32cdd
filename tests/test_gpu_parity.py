"""CUDA path vs the CPU oracle, stage by stage and image by image.

Every check calls the GPU through the C ABI (spray_gb300 -> libspray_gpu.so)
and compares with the oracle on the same seeded inputs:
  eye rays, per-domain queues, domain scores    bit-exact
  closest hits (hit, domain, prim, t, colour, Ns)  bit-exact (>= 99.99% required)
  shadow and bounce rays from the shaders       bit-exact
  occlusion flags                               bit-exact (>= 99.99% required)
  images vs the wavefront oracle                bit-exact (same accumulation order)
  images vs the speculative loop (mode A)       max abs 1e-5 (float accumulation order)
"""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config

pytestmark = pytest.mark.gpu

HIT_AGREE = 0.9999   # required agreement on hit/miss, domain and primitive
T_RTOL = 1e-5        # required relative agreement of hit distances
IMG_RMSE = 1e-3      # required image agreement (RMSE on [0,1] radiance)


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


@pytest.fixture(scope="module")
def scene8():
    return scenes.wavelet_grid(2, 24, colors="albedo", light="point+diffuse")


@pytest.fixture(scope="module")
def scene64():
    return scenes.wavelet_grid(4, 32, colors="albedo", light="point")


def run(cfg, scene, grid, oracle_mod, **gpu_kw):
    cam = scenes.orbit_camera(scene)
    t = sg.Tracer(cfg, debug_capture=1, **gpu_kw)
    t.set_scene(scene)
    t.set_camera(*cam)
    img, st = t.trace()
    o = oracle_mod.Oracle(cfg, scene)
    o.set_camera(*cam)
    return t, img, st, o


def test_eye_rays_bit_exact(lib_built, oracle_mod, scene8):
    for spp in (1, 4):
        cfg = small_config(pixel_samples=spp, image_w=40, image_h=30, max_samples_per_rank=1024)
        t, img, st, o = run(cfg, scene8, 2, oracle_mod)
        r = t.debug(sg.DBG_RAYS, 0)
        ntiles = len(o.tiles())
        org, dr, pix, sam = o.eyes(0, ntiles)
        assert len(r) == len(org) == 40 * 30 * spp
        assert np.array_equal(r["sample"], np.arange(len(r)))
        assert np.array_equal(bits(r["org"]), bits(org))
        assert np.array_equal(bits(r["dir"]), bits(dr))
        assert np.array_equal(r["pixid"], pix) and np.array_equal(r["samid"], sam)


def _queues_by_domain(e):
    order = np.lexsort((e["ray"], e["domain"]))
    e = e[order]
    return e["domain"], e["ray"], bits(e["tdom"]), e["depth"], e["origin"]


@pytest.mark.parametrize("cull", [0, 1])
def test_radiance_queues_bit_exact(lib_built, oracle_mod, scene64, cull):
    cfg = small_config(image_w=80, image_h=60)
    t, img, st, o = run(cfg, scene64, 4, oracle_mod, cull=cull)
    rays = t.debug(sg.DBG_RAYS, 0)
    q = t.debug(sg.DBG_RQUEUES, 0)
    oq, dstats = o.schedule(rays["org"], rays["dir"])
    oq["ray"] = rays["sample"][oq["ray"]]
    assert len(q) == len(oq) > 0
    if cull == 0:
        # domain-major order, each queue in push (ray) order: the exact sequence
        assert np.array_equal(q["domain"], oq["domain"]) and np.array_equal(q["ray"], oq["ray"])
        assert np.array_equal(bits(q["tdom"]), bits(oq["tdom"]))
        assert np.array_equal(q["depth"], oq["depth"])
    for a, b in zip(_queues_by_domain(q), _queues_by_domain(oq)):
        assert np.array_equal(a, b)
    # DomainStats scores and the processing order
    sc = t.debug(sg.DBG_SCORES, 0)
    osc, oorder = o.scores(dstats)
    assert np.array_equal(sc["score"], osc)
    assert np.array_equal(np.argsort(sc["order"]), oorder)


def test_many_domains_queues_and_image(lib_built, oracle_mod):
    # 125 domains: 500 scheduler keys, so the histogram scan runs over several
    # key tiles and key-scan blocks; radiance queues and the path-traced image
    # (shadow queues sorted by list position, 500 keys too) stay bit-exact
    sc = scenes.wavelet_grid(5, 16, colors="albedo", light="point+diffuse")
    cfg = small_config(image_w=80, image_h=60, ao_mode=0, ao_samples=2, pixel_samples=2, bounces=3)
    t, img, st, o = run(cfg, sc, 5, oracle_mod, cull=0)
    rays = t.debug(sg.DBG_RAYS, 0)
    q = t.debug(sg.DBG_RQUEUES, 0)
    oq, _ = o.schedule(rays["org"], rays["dir"])
    oq["ray"] = rays["sample"][oq["ray"]]
    assert len(q) == len(oq) > 0
    assert np.array_equal(q["domain"], oq["domain"]) and np.array_equal(q["ray"], oq["ray"])
    assert np.array_equal(bits(q["tdom"]), bits(oq["tdom"]))
    assert np.array_equal(q["depth"], oq["depth"])
    wb, sb = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb))
    assert st["rays_shadow"] == sb["rays_shadow"] and st["rays_bounce"] == sb["rays_bounce"]
    assert img[..., :3].max() > 0


def _hits_match(h, oh):
    same = (h["hit"] == oh["hit"]) & (h["domain"] == oh["domain"]) & (h["prim"] == oh["prim"])
    return same


def test_closest_hits_bit_exact(lib_built, oracle_mod, scene64):
    cfg = small_config(image_w=96, image_h=72, ao_mode=0, pixel_samples=2, bounces=3)
    t, img, st, o = run(cfg, scene64, 4, oracle_mod)
    total = 0
    for b in range(3):
        rays = t.debug(sg.DBG_RAYS, b)
        h = t.debug(sg.DBG_HITS, b)
        assert np.array_equal(h["sample"], rays["sample"])
        oh = o.closest(rays["org"], rays["dir"])
        same = _hits_match(h, oh)
        assert same.mean() >= HIT_AGREE, (b, same.mean())
        hit = (h["hit"] == 1) & same
        assert np.allclose(h["t"][hit], oh["t"][hit], rtol=T_RTOL, atol=0)
        # the same watertight test on both sides: identical bits
        assert same.all(), np.nonzero(~same)[0][:10]
        assert np.array_equal(bits(h["t"][hit]), bits(oh["t"][hit]))
        assert np.array_equal(h["color"][hit], oh["color"][hit])
        assert np.array_equal(bits(h["ns"][hit]), bits(oh["ns"][hit]))
        total += hit.sum()
    assert total > 1000


def _shade_check(t, o, b, S):
    rays = t.debug(sg.DBG_RAYS, b)
    h = t.debug(sg.DBG_HITS, b)
    sh = t.debug(sg.DBG_SHADOWS, b)
    m = h["hit"] == 1
    r, hh = rays[m], h[m]
    out = o.shade(b, r["org"], r["dir"], r["w"], r["pixid"], r["samid"], hh["t"], hh["domain"],
                  hh["color"], hh["ns"])
    # expected shadow rays, ordered (sample, slot)
    samp = np.repeat(r["sample"], S)
    slot = np.tile(np.arange(S), len(r))
    valid = out["svalid"].reshape(-1).astype(bool)
    exp_s, exp_k = samp[valid], slot[valid]
    assert np.array_equal(sh["sample"], exp_s) and np.array_equal(sh["slot"], exp_k)
    assert np.array_equal(bits(sh["dir"]), bits(out["sdir"].reshape(-1, 3)[valid]))
    assert np.array_equal(bits(sh["w"]), bits(out["sw"].reshape(-1, 3)[valid]))
    assert np.array_equal(bits(sh["tmax"]), bits(out["stmax"].reshape(-1)[valid]))
    # bounce rays become the rays of the next depth
    if b + 1 < t.config["bounces"]:
        nxt = t.debug(sg.DBG_RAYS, b + 1)
        bv = out["bvalid"].astype(bool)
        assert np.array_equal(nxt["sample"], r["sample"][bv])
        assert np.array_equal(bits(nxt["dir"]), bits(out["bdir"][bv]))
        assert np.array_equal(bits(nxt["w"]), bits(out["bw"][bv]))
        pos = r["dir"] * hh["t"][:, None] + r["org"]
        assert np.array_equal(bits(nxt["org"]), bits(pos[bv].astype(np.float32)))
    return sh, h


@pytest.mark.parametrize("mode", ["ao", "pt"])
def test_shaders_bit_exact(lib_built, oracle_mod, scene8, mode):
    cfg = small_config(image_w=64, image_h=48, ao_mode=int(mode == "ao"), ao_samples=3,
                       pixel_samples=2, bounces=3, ks=[0.4, 0.4, 0.4], shininess=10.0)
    t, img, st, o = run(cfg, scene8, 2, oracle_mod)
    S = o.slots()
    for b in range(3):
        _shade_check(t, o, b, S)


def test_occlusion_and_shadow_queues(lib_built, oracle_mod, scene64):
    cfg = small_config(image_w=80, image_h=60, ao_mode=1, ao_samples=4, bounces=2)
    t, img, st, o = run(cfg, scene64, 4, oracle_mod)
    S = o.slots()
    for b in range(2):
        sh = t.debug(sg.DBG_SHADOWS, b)
        h = t.debug(sg.DBG_HITS, b)
        rays = t.debug(sg.DBG_RAYS, b)
        dom_of = dict(zip(h["sample"].tolist(), h["domain"].tolist()))
        origin = np.array([dom_of[s] for s in sh["sample"]], np.int32)
        occ = o.occluded(sh["org"], sh["dir"], sh["tmax"], origin)
        agree = (occ == sh["occluded"]).mean()
        assert agree >= HIT_AGREE and agree == 1.0
        # shadow queues: ray id = alive index * slots + slot
        alive = {s: i for i, s in enumerate(rays["sample"].tolist())}
        sid = np.array([alive[s] * S + k for s, k in zip(sh["sample"].tolist(), sh["slot"].tolist())],
                       np.uint32)
        q = t.debug(sg.DBG_SQUEUES, b)
        oq, _ = o.schedule(sh["org"], sh["dir"], sh["tmax"], origin)
        oq["ray"] = sid[oq["ray"]]
        for a, c in zip(_queues_by_domain(q), _queues_by_domain(oq)):
            assert np.array_equal(a, c)


@pytest.mark.parametrize("mode,spp,bounces,light", [
    ("ao", 1, 1, "point"), ("ao", 2, 2, "point"), ("pt", 1, 1, "point"),
    ("pt", 2, 3, "point+diffuse"), ("pt", 4, 4, "point+diffuse"), ("pt", 2, 3, "quad"),
    ("pt", 32, 2, "point"),  # 256 pixels x 32 spp: retire reads alive indices unstaged
])
def test_image_matches_oracles(lib_built, oracle_mod, mode, spp, bounces, light):
    sc = scenes.wavelet_grid(2, 24, colors="albedo", light=light)
    cfg = small_config(image_w=72, image_h=54, ao_mode=int(mode == "ao"), ao_samples=3,
                       pixel_samples=spp, bounces=bounces, max_samples_per_rank=4096)
    t, img, st, o = run(cfg, sc, 2, oracle_mod)
    wb, sb = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb))           # same order of every float add
    assert st["rays_primary"] == sb["rays_primary"]
    assert st["rays_shadow"] == sb["rays_shadow"] and st["rays_bounce"] == sb["rays_bounce"]
    wa, sa = o.render_speculative(2)
    assert np.abs(img - wa).max() <= 1e-5
    assert np.sqrt(np.mean((img[..., :3] - wa[..., :3]) ** 2)) < IMG_RMSE
    assert img[..., :3].max() > 0


def test_extensions_match_wavefront_oracle(lib_built, oracle_mod):
    sc = scenes.wavelet_grid(2, 24, colors="albedo", light="quad")
    diag = scenes.scene_diagonal(sc)
    for cfg in (small_config(ao_mode=1, ao_samples=4, ao_max_distance=0.05 * diag, ao_light_shadow=1),
                small_config(ao_mode=0, ao_samples=2, pixel_samples=2, bounces=5, rr_depth=3)):
        t, img, st, o = run(cfg, sc, 2, oracle_mod)
        wb, _ = o.render_wavefront()
        assert np.array_equal(bits(img), bits(wb))


def test_waves_and_culling_do_not_change_the_image(lib_built, oracle_mod, scene64):
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3,
                       max_samples_per_rank=2048)
    cam = scenes.orbit_camera(scene64)
    imgs = []
    for kw in (dict(cull=1, bucket_launches=4), dict(cull=0), dict(cull=1, wave_samples=3000, bucket_launches=4),
               dict(cull=0, wave_samples=2048), dict(cull=1)):
        t = sg.Tracer(cfg, **kw)
        t.set_scene(scene64)
        t.set_camera(*cam)
        img, st = t.trace()
        imgs.append(img)
        if kw.get("bucket_launches") == 4:
            assert st["visits_culled"] > 0  # one launch per bucket: nearer hits always seen
    for im in imgs[1:]:
        assert np.array_equal(bits(im), bits(imgs[0]))


def test_large_wavefront_ray_ids(lib_built, scene64):
    # 1024 x 1024 x 8 spp AO with 8 AO rays and the light ray: 9 shadow slots,
    # so one wavefront numbers its shadow rays up to ~75 M (beyond 2^26); the
    # image equals, bit for bit, the same frame cut into 1 M-sample wavefronts
    diag = scenes.scene_diagonal(scene64)
    cfg = small_config(image_w=1024, image_h=1024, ao_mode=1, ao_samples=8, pixel_samples=8,
                       ao_max_distance=0.05 * diag, ao_light_shadow=1)
    cam = scenes.orbit_camera(scene64)
    imgs, stats = [], []
    for kw in (dict(), dict(wave_samples=1 << 20)):
        t = sg.Tracer(cfg, **kw)
        t.set_scene(scene64)
        t.set_camera(*cam)
        img, st = t.trace()
        imgs.append(img)
        stats.append(st)
        del t
    assert stats[0]["rays_primary"] == 1024 * 1024 * 8  # one wavefront: ids up to 9 x 8.4 M
    assert stats[0]["rays_shadow"] == stats[1]["rays_shadow"] > 0
    assert np.array_equal(bits(imgs[0]), bits(imgs[1]))
    assert imgs[0][..., :3].max() > 0


@pytest.mark.parametrize("launches", [1, 4])
def test_deterministic_frames(lib_built, scene64, launches):
    """Images and ray counts repeat exactly; with one launch per depth bucket the
    visit counts do too."""
    t = sg.Tracer(small_config(image_w=64, image_h=64, ao_mode=0, pixel_samples=2, bounces=2),
                  bucket_launches=launches)
    t.set_scene(scene64)
    t.set_camera(*scenes.orbit_camera(scene64))
    a, sa = t.trace()
    b, sb = t.trace()
    assert np.array_equal(bits(a), bits(b))
    keys = ["rays_primary", "rays_shadow", "rays_bounce", "visits_shadow"]
    if launches == 4:
        keys.append("visits_radiance")
        assert sa["trace_launches"] == 4 * 2
    for k in keys:
        assert sa[k] == sb[k]


def test_all_rays_miss(lib_built, scene8):
    t = sg.Tracer(small_config(image_w=32, image_h=16))
    t.set_scene(scene8)
    t.set_camera((0, 0, 50), (0, 0, 100), (0, 1, 0))  # looking away from the grid
    img, st = t.trace()
    assert not img.any() and st["rays_shadow"] == 0 and st["visits_radiance"] == 0


def test_single_triangle_and_ragged_tiles(lib_built, oracle_mod):
    v = np.array([[-1, -1, 0], [1, -1, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.uint32)
    sc = sg.Scene([sg.Domain(v, f, np.full(3, 0x80a0c0, np.uint32))], [sg.Light(0, (0, 0, 5))])
    cfg = small_config(image_w=37, image_h=23, ao_mode=0, pixel_samples=3, max_samples_per_rank=500)
    t = sg.Tracer(cfg)
    t.set_scene(sc)
    t.set_camera((0.1, 0.2, 3), (0, 0, 0), (0, 1, 0))
    img, st = t.trace()
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera((0.1, 0.2, 3), (0, 0, 0), (0, 1, 0))
    assert len(o.tiles()) > 5
    wb, _ = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb)) and img[..., :3].max() > 0


def test_errors(lib_built, scene8):
    t = sg.Tracer(small_config())
    with pytest.raises(sg.SprayError) as e:
        t.trace()
    assert e.value.code == sg.ESTATE
    t.set_scene(scene8)
    with pytest.raises(sg.SprayError) as e:
        t.trace()
    assert e.value.code == sg.ESTATE  # no camera yet
    pt = sg.Tracer(small_config(ao_mode=0))
    with pytest.raises(sg.SprayError) as e:
        pt.set_scene(sg.Scene(scene8.domains, []))
    assert e.value.code == sg.EINVAL
    with pytest.raises(sg.SprayError) as e:
        sg.Tracer(small_config(list_size=64))
    assert e.value.code == sg.EINVAL


def test_domain_list_overflow_reported(lib_built):
    # 40 unit boxes in a row: a ray along the row overlaps all of them
    v0 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    f = np.array([[0, 1, 2]], np.uint32)
    doms = [sg.Domain(v0 + [2 * i, 0, 0], f, bounds=[2 * i, 0, 0, 2 * i + 1, 1, 1]) for i in range(40)]
    t = sg.Tracer(small_config(image_w=4, image_h=4))
    t.set_scene(sg.Scene(doms, [sg.Light(0, (0, 5, 0))]))
    t.set_camera((-5, 0.5, 0.5), (100, 0.5, 0.5), (0, 1, 0), 1.0)
    with pytest.raises(sg.SprayError) as e:
        t.trace()
    assert e.value.code == sg.EOVERFLOW


def test_scene_file_path(lib_built, oracle_mod, tmp_path):
    p = scenes.write_wavelet_grid(tmp_path, grid=2, samples=16, colors="albedo", light="point")
    sc = sg.Scene.load(p, p.parent)
    cfg = small_config(ao_mode=0, pixel_samples=2, bounces=2)
    t, img, st, o = run(cfg, sc, 2, oracle_mod)
    wb, _ = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb))


@pytest.mark.parametrize("kw", [dict(cache_size=16), dict(cache_size=5), dict(cache_bytes=3 << 20),
                                dict(cache_size=16, schedule_policy=1),
                                dict(cache_size=16, schedule_policy=2, ooc_inplace=0),
                                dict(cache_size=5, schedule_policy=2, ooc_batch=1, ooc_inplace=0),
                                dict(cache_size=1, schedule_policy=2, ooc_inplace=0),
                                dict(cache_bytes=3 << 20, schedule_policy=2, ooc_batch=3, ooc_inplace=0),
                                dict(cache_size=16, schedule_policy=2, ooc_inplace=200),
                                dict(cache_size=16, schedule_policy=2, ooc_inplace=1 << 30),
                                dict(cache_size=16, schedule_policy=2),
                                dict(cache_size=16, schedule_policy=4, ooc_inplace=0),
                                dict(cache_size=5, schedule_policy=4, ooc_batch=2)])
def test_out_of_core_cache_gives_the_in_core_image(lib_built, scene64, kw):
    """Streaming domains through a small LRU cache changes loads, never the image."""
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3)
    cam = scenes.orbit_camera(scene64)
    ref = sg.Tracer(cfg, bucket_launches=4)
    ref.set_scene(scene64)
    ref.set_camera(*cam)
    want, st0 = ref.trace()
    assert st0["domain_loads"] == 0
    t = sg.Tracer(cfg, **kw)
    t.set_scene(scene64)
    t.set_camera(*cam)
    got, st = t.trace()
    assert np.array_equal(bits(got), bits(want))
    inplace = kw.get("ooc_inplace", 16384) if kw.get("schedule_policy", 0) in (2, 3, 4) else 0
    if inplace >= 1 << 30:
        assert st["domain_loads"] == 0 and st["inplace_domains"] > 0  # every domain read in place
    elif inplace == 0:
        assert st["domain_loads"] > 0 and st["h2d_bytes"] > 0 and st["inplace_domains"] == 0
    else:
        assert st["domain_loads"] + st["inplace_domains"] > 0
    if 0 < inplace < 1 << 30 and "ooc_inplace" in kw:
        assert st["inplace_domains"] > 0 and st["domain_loads"] > 0
    assert st["rays_shadow"] == st0["rays_shadow"] and st["visits_radiance"] >= st0["visits_radiance"] - st0["visits_culled"]
    got2, st2 = t.trace()  # the cache stays warm across frames
    assert np.array_equal(bits(got2), bits(want))


def test_out_of_core_queues_match_oracle(lib_built, oracle_mod, scene64):
    cfg = small_config(image_w=80, image_h=60, cache_size=8)
    t, img, st, o = run(cfg, scene64, 4, oracle_mod)
    rays = t.debug(sg.DBG_RAYS, 0)
    q = t.debug(sg.DBG_RQUEUES, 0)
    oq, _ = o.schedule(rays["org"], rays["dir"])
    oq["ray"] = rays["sample"][oq["ray"]]
    assert np.array_equal(q["domain"], oq["domain"]) and np.array_equal(q["ray"], oq["ray"])
    wb, _ = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb))


def test_cache_aware_order_needs_fewer_loads(lib_built, scene64):
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=4, cache_size=24)
    cam = scenes.orbit_camera(scene64)
    loads = []
    for pol in (0, 1, 2):
        t = sg.Tracer(cfg, schedule_policy=pol, ooc_inplace=0)
        t.set_scene(scene64)
        t.set_camera(*cam)
        t.trace()
        _, st = t.trace()
        loads.append(st["domain_loads"])
    assert loads[1] < loads[0]
    assert loads[2] < loads[1]


def test_batched_pass_skips_fully_culled_domains(lib_built, scene64):
    """Batched out-of-core passes trace no more entries than the plain order and
    never load a domain whose entries were all culled, with the same image."""
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3, cache_size=16)
    cam = scenes.orbit_camera(scene64)
    out = {}
    for pol, batch in ((0, 0), (2, 2)):
        t = sg.Tracer(cfg, schedule_policy=pol, ooc_batch=batch, ooc_inplace=0)
        t.set_scene(scene64)
        t.set_camera(*cam)
        out[pol] = t.trace()
    (img0, st0), (img2, st2) = out[0], out[2]
    assert np.array_equal(bits(img0), bits(img2))
    assert st2["rays_shadow"] == st0["rays_shadow"] and st2["rays_bounce"] == st0["rays_bounce"]
    assert st2["visits_radiance"] <= st0["visits_radiance"]
    assert st2["visits_shadow"] <= st0["visits_shadow"]
    assert st2["domain_loads"] < st0["domain_loads"]



LEARN = dict(schedule_policy=3, learn_frames=1, learn_batch=8192, learn_epochs=8)


@pytest.mark.parametrize("kw", [dict(), dict(cache_size=16), dict(cache_size=5, ooc_batch=1)])
def test_learned_proposal_keeps_the_image(lib_built, kw):
    """The learned order changes which entries are traced when, never the image."""
    scene = scenes.wavelet_grid(4, 32, colors="albedo", light="quad")
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=4, rr_depth=3)
    cam = scenes.orbit_camera(scene)
    ref = sg.Tracer(cfg)
    ref.set_scene(scene)
    ref.set_camera(*cam)
    want, _ = ref.trace()
    t = sg.Tracer(cfg, **LEARN, **kw)
    t.set_scene(scene)
    t.set_camera(*cam)
    img1, st1 = t.trace()  # collects pairs, trains after the frame
    assert st1["learn_trained"] == 1 and st1["learn_pairs"] > 1000 and st1["learn_ms"] > 0
    assert np.isfinite(st1["learn_loss"]) and st1["learn_loss"] < np.log(8)
    img2, st2 = t.trace()  # ordered by the trained proposal
    img3, _ = t.trace()
    for img in (img1, img2, img3):
        assert np.array_equal(bits(img), bits(want))
    assert st2["learn_ms"] == 0


def test_learned_proposal_against_the_method_without_it(lib_built):
    """The learned proposal (policy 3) against the same batched out-of-core
    passes without the network (policy 2) and with the untrained network.

    What the network gains is prediction: on held-out (ray, winning candidate)
    pairs its top-1 accuracy beats the nearest-candidate guess (the
    front-to-back order's) and the untrained network.  The image never
    changes.  Its effect on work is reported against policy 2 (visits, loads,
    frame time): each ray keeps its front-to-back order inside a batch, where
    that order is already visit-optimal (a candidate in front of the hit can
    never be culled), so only the cross-batch domain order can move."""
    scene = scenes.wavelet_grid(4, 32, colors="albedo", light="quad")
    cfg = small_config(image_w=320, image_h=240, ao_mode=0, pixel_samples=4, bounces=4, rr_depth=3,
                       cache_size=16, ooc_inplace=0)
    cam = scenes.orbit_camera(scene)
    out = {}
    for name, kw in (("batched", dict(schedule_policy=2)), ("untrained", dict(LEARN, learn_epochs=0)),
                     ("trained", LEARN)):
        t = sg.Tracer(cfg, **kw)
        t.set_scene(scene)
        t.set_camera(*cam)
        _, s1 = t.trace()
        img, st = t.trace()
        st["first"] = s1
        out[name] = (img, st)
        t.close()
    (ib, sb), (iu, su), (it, s_t) = out["batched"], out["untrained"], out["trained"]
    assert np.array_equal(bits(ib), bits(it)) and np.array_equal(bits(iu), bits(it))
    tr, un = s_t["first"], su["first"]
    assert tr["learn_trained"] == 1 and tr["learn_eval_pairs"] > 1000
    assert tr["learn_top1"] > tr["learn_top1_nearest"] + 0.03, (tr["learn_top1"], tr["learn_top1_nearest"])
    assert tr["learn_top1"] > un["learn_top1"] + 0.1, (tr["learn_top1"], un["learn_top1"])
    # the trained order culls more than the untrained network's
    assert s_t["visits_radiance"] < su["visits_radiance"]
    print("learned vs batched: radiance visits %d vs %d, loads %d vs %d, %.2f vs %.2f ms; top-1 %.3f "
          "(nearest %.3f, untrained %.3f)" % (s_t["visits_radiance"], sb["visits_radiance"],
                                               s_t["domain_loads"], sb["domain_loads"], s_t["frame_ms"],
                                               sb["frame_ms"], tr["learn_top1"], tr["learn_top1_nearest"],
                                               un["learn_top1"]))


def test_graph_replay_follows_camera_and_matches_direct_launches(lib_built, scene64):
    """The in-core frame captured as a CUDA graph renders what direct launches
    render, across camera moves and several wavefronts per frame."""
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3, wave_samples=5000,
                       bucket_launches=4)
    tg = sg.Tracer(cfg, graphs=1)
    td = sg.Tracer(cfg, graphs=0)
    for t in (tg, td):
        t.set_scene(scene64)
    for frame in range(3):
        cam = scenes.orbit_camera(scene64, frame=frame)
        out = []
        for t in (tg, td):
            t.set_camera(*cam)
            out.append(t.trace())
        (ig, sgr), (idr, sd) = out
        assert np.array_equal(bits(ig), bits(idr)), frame
        for k in ("rays_primary", "rays_shadow", "rays_bounce", "visits_radiance", "visits_shadow",
                  "kernel_launches", "trace_launches"):
            assert sgr[k] == sd[k], (frame, k)
        assert sgr["trace_ms"] > 0 and sgr["frame_ms"] > 0


@pytest.mark.parametrize("kw", [dict(), dict(cache_size=3, schedule_policy=2)])
def test_prepared_blobs_render_the_same_image(lib_built, scene64, tmp_path, kw):
    """A scene set from prepared-domain blobs renders bit-identically to set_scene."""
    sg.prepare_scene(scene64, tmp_path)
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3)
    cam = scenes.orbit_camera(scene64)
    imgs = []
    for prepared in (False, True):
        t = sg.Tracer(cfg, **kw)
        if prepared:
            t.set_scene_prepared(tmp_path, len(scene64.domains), scene64.lights)
        else:
            t.set_scene(scene64)
        t.set_camera(*cam)
        img, st = t.trace()
        imgs.append((img, st))
    assert np.array_equal(bits(imgs[0][0]), bits(imgs[1][0]))
    assert imgs[0][1]["scene_triangles"] == imgs[1][1]["scene_triangles"]


def test_non_speculative_order_visits_least(lib_built, scene64):
    """The LoadAnyOnce restatement traces each ray only in domains it reaches
    without a nearer hit: no more radiance visits than the speculative passes."""
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3, cache_size=16,
                       ooc_inplace=0)
    cam = scenes.orbit_camera(scene64)
    out = {}
    for pol in (0, 4):
        t = sg.Tracer(cfg, schedule_policy=pol)
        t.set_scene(scene64)
        t.set_camera(*cam)
        out[pol] = t.trace()
    (i0, s0), (i4, s4) = out[0], out[4]
    assert np.array_equal(bits(i0), bits(i4))
    assert s4["visits_radiance"] <= s0["visits_radiance"]


def _mixed_views(scene):
    """An uneven batch: different sizes, spp, AO or path tracing, bounces."""
    specs = [dict(image_w=64, image_h=48, pixel_samples=1, ao_mode=1, ao_samples=4, bounces=1),
             dict(image_w=96, image_h=64, pixel_samples=4, ao_mode=0, ao_samples=2, bounces=3),
             dict(image_w=40, image_h=40, pixel_samples=2, ao_mode=0, ao_samples=1, bounces=4, rr_depth=2),
             dict(image_w=128, image_h=32, pixel_samples=1, ao_mode=1, ao_samples=2, bounces=2,
                  ao_light_shadow=1)]
    views = []
    for k, sp in enumerate(specs):
        pos, look, up = scenes.orbit_camera(scene, frame=k)
        views.append(dict(sp, position=pos, lookat=look, up=up, vfov=60.0))
    return views


@pytest.mark.parametrize("kw", [dict(), dict(cache_size=16, schedule_policy=2),
                                dict(wave_samples=3000, graphs=1)])
def test_multi_view_batch_matches_single_views(lib_built, kw):
    """Views of one multi-view frame equal single-view renders of each, bit for bit."""
    scene = scenes.wavelet_grid(4, 32, colors="albedo", light="point")
    views = _mixed_views(scene)
    base = small_config()
    t = sg.Tracer(base, **kw)
    t.set_scene(scene)
    for rep in range(2):  # the second frame replays whatever was captured
        imgs, st = t.trace_views(views)
        total_primary = 0
        for v, img in zip(views, imgs):
            cfg = dict(base, **{k: v[k] for k in v if k not in ("position", "lookat", "up", "vfov")}, fov=60.0)
            r = sg.Tracer(cfg, **kw)
            r.set_scene(scene)
            r.set_camera(v["position"], v["lookat"], v["up"], 60.0)
            want, sr = r.trace()
            assert np.array_equal(bits(img), bits(want)), (rep, v["image_w"])
            total_primary += sr["rays_primary"]
        assert st["rays_primary"] == total_primary


def _delta_scene():
    """Eight domains cycling diffuse, mirror, glass (1 | 1.5) and
    transmission (1 | 1.33): every delta branch of the PT shader."""
    sc = scenes.wavelet_grid(2, 24, colors="albedo", light="point+diffuse")
    params = {1: (1, 1, 1), 2: (1.0, 1.5, 0.0), 3: (1.0, 1.33, 0.0)}
    for i, d in enumerate(sc.domains):
        d.bsdf_type = i % 4
        d.bsdf_params = np.asarray(params.get(i % 4, (1, 1, 1)), np.float32)
    return sc


@pytest.mark.parametrize("spp,bounces", [(2, 3), (1, 5)])
def test_delta_bsdfs_match_oracles(lib_built, oracle_mod, spp, bounces):
    """Mirror, glass and transmission (reflection.h:126-174, 264-364; the
    weight Lin * fr / |cos| of ooc_shader_pt.h:181-210, so pixels reach 1e5 and
    more at grazing angles): bit-exact against the wavefront oracle, and
    within float accumulation order of the speculative loop."""
    sc = _delta_scene()
    cfg = small_config(image_w=72, image_h=54, ao_mode=0, ao_samples=2, pixel_samples=spp, bounces=bounces,
                       max_samples_per_rank=4096)
    t, img, st, o = run(cfg, sc, 2, oracle_mod)
    wb, sb = o.render_wavefront()
    assert np.array_equal(bits(img), bits(wb))
    assert st["rays_shadow"] == sb["rays_shadow"] and st["rays_bounce"] == sb["rays_bounce"]
    wa, _ = o.render_speculative(2)
    assert np.all(np.abs(img - wa) <= 1e-6 * np.maximum(np.abs(wa), 1.0))
    assert img[..., :3].max() > 0
