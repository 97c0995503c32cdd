"""The per-domain BVH built on the GPU (binned SAH, 4-wide nodes) against the
host builder.

SpRay rebuilds each domain's Embree BVH on load (TriMeshBuffer::load,
src/render/trimesh_buffer.cc:104,222-224); here set_scene builds every
domain's BVH on the device (bvh_device = 1, the default) or on the host cores
(bvh_device = 0).  The traced answer does not depend on the tree: hits are
the minimum of (t, triangle) over the exact triangle tests, and node boxes
are exact unions of the triangles' float boxes.  So images, hits and queues
must be bit-identical between the two builders, in core and out of core, and
the device tree's quality (nodes and triangles visited) close to the host's.
"""
import time

import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config

pytestmark = pytest.mark.gpu


def bits(a):
    return np.ascontiguousarray(a, np.float32).view(np.uint32)


def _trace(scene, cfg, **kw):
    t = sg.Tracer(cfg, **kw)
    t0 = time.perf_counter()
    t.set_scene(scene)
    build_s = time.perf_counter() - t0
    t.set_camera(*scenes.orbit_camera(scene))
    img, st = t.trace()
    return t, img, st, build_s


def _degenerate_scene():
    """Domains that stress the builder: one triangle, two, a stack of 600
    identical triangles (every centroid equal: split by halves), a fan of
    300 triangles sharing a vertex, and an ordinary wavelet mesh."""
    doms = []
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    doms.append(sg.Domain(tri + [0, 0, 0], [[0, 1, 2]], np.full(3, 0x808080, np.uint32)))
    two = np.concatenate([tri, tri + [0, 0, 0.5]])
    doms.append(sg.Domain(two + [2, 0, 0], [[0, 1, 2], [3, 4, 5]], np.full(6, 0x80a080, np.uint32)))
    stack = np.tile(tri, (600, 1)) + [4, 0, 0]
    doms.append(sg.Domain(stack, np.arange(1800).reshape(600, 3), np.full(1800, 0xa08080, np.uint32)))
    ang = np.linspace(0, 2 * np.pi, 301)[:-1]
    ring = np.stack([np.cos(ang), np.sin(ang), 0.2 * np.sin(5 * ang)], 1).astype(np.float32) + [6, 0.5, 0]
    fan_v = np.concatenate([[[6, 0.5, 0.3]], ring]).astype(np.float32)
    fan_f = np.stack([np.zeros(300), 1 + np.arange(300), 1 + (np.arange(300) + 1) % 300], 1).astype(np.uint32)
    doms.append(sg.Domain(fan_v, fan_f, np.full(len(fan_v), 0x8080a0, np.uint32)))
    v, f = sg.generate_wavelet(28)
    doms.append(sg.Domain(v * 0.9 + [8.5, 0.5, 0], f, np.full(len(v), 0xc0c0c0, np.uint32)))
    sc = sg.Scene(doms, [])
    sc.lights = scenes.make_lights("point+diffuse", *scenes.scene_box(sc))
    return sc


@pytest.mark.parametrize("which", ["grid64", "grid8", "degenerate"])
def test_device_bvh_traces_the_host_bvh_image(lib_built, which):
    if which == "grid64":
        sc = scenes.wavelet_grid(4, 32, colors="albedo", light="quad")
    elif which == "grid8":
        sc = scenes.wavelet_grid(2, 24, colors="albedo", light="point+diffuse")
    else:
        sc = _degenerate_scene()
    cfg = small_config(image_w=96, image_h=72, ao_mode=0, ao_samples=2, pixel_samples=2, bounces=3, cull=0,
                       debug_capture=1)
    th, ih, sh, _ = _trace(sc, cfg, bvh_device=0)
    td, idv, sd, _ = _trace(sc, cfg, bvh_device=1)
    assert np.array_equal(bits(ih), bits(idv)), float(np.abs(ih - idv).max())
    for b in range(3):
        hh, hd = th.debug(sg.DBG_HITS, b), td.debug(sg.DBG_HITS, b)
        assert np.array_equal(hh, hd), b
    assert sh["rays_shadow"] == sd["rays_shadow"] and sh["rays_bounce"] == sd["rays_bounce"]
    # tree quality: the device's binned SAH walks about as many nodes as the host's
    assert sd["nodes_radiance"] <= 1.25 * sh["nodes_radiance"], (sd["nodes_radiance"], sh["nodes_radiance"])
    assert sd["tris_radiance"] <= 1.25 * sh["tris_radiance"], (sd["tris_radiance"], sh["tris_radiance"])
    assert ih[..., :3].max() > 0


@pytest.mark.parametrize("policy", [0, 2])
def test_device_bvh_out_of_core(lib_built, policy):
    sc = scenes.wavelet_grid(4, 24, colors="albedo", light="quad")
    cfg = small_config(image_w=96, image_h=72, ao_mode=0, pixel_samples=2, bounces=3, cache_size=10,
                       schedule_policy=policy)
    _, ih, _, _ = _trace(sc, cfg, bvh_device=0)
    _, idv, _, _ = _trace(sc, cfg, bvh_device=1)
    assert np.array_equal(bits(ih), bits(idv))


def test_device_bvh_on_the_out_of_core_workload(lib_built):
    # C3's 512 domains (38.5 M triangles): build time on the device against
    # the host cores, and the same image
    path, _ = scenes.benchmark_scene("c3")
    sc = sg.Scene.load(path, path.parent)
    _, c3 = scenes.workload_config("c3", sc)
    cfg = dict(c3, image_w=128, image_h=128)
    th, ih, sh, host_s = _trace(sc, cfg, bvh_device=0)
    th.close()
    td, idv, sd, dev_s = _trace(sc, cfg, bvh_device=1)
    td.close()
    assert np.array_equal(bits(ih), bits(idv))
    print(f"C3 set_scene: host BVH {host_s:.2f} s, device BVH {dev_s:.2f} s; nodes visited "
          f"{sd['nodes_radiance']} vs {sh['nodes_radiance']}")
    assert dev_s < host_s


@pytest.mark.parametrize("cache", [-1, 10])
def test_oracle_walks_the_gpu_hierarchy(lib_built, oracle_mod, cache):
    # the hierarchies set_scene built on the device, read back through the
    # debug hook (from the device in core, from pinned host memory out of
    # core), give every ray the oracle's own closest hit; the kernel's node
    # and triangle counts are close to those of the oracle's ordered walk
    # (front to back over the domains, culled by the hit so far)
    sc = scenes.wavelet_grid(4, 24, colors="albedo", light="quad")
    cfg = small_config(image_w=96, image_h=72, ao_mode=0, pixel_samples=2, bounces=3, cache_size=cache,
                       bucket_launches=4)
    t, img, st, _ = _trace(sc, cfg)
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*scenes.orbit_camera(sc))
    for d in range(len(sc.domains)):
        nodes, tris = t.debug(sg.DBG_NODES, d), t.debug(sg.DBG_TRIS, d)
        assert len(tris) == len(sc.domains[d].faces) and len(nodes) >= 1
        assert np.all(np.isin(np.sort(tris["v"][:, 0, 3].view(np.uint32)),
                              np.arange(len(tris), dtype=np.uint32)))
        o.set_bvh4(d, nodes, tris)
    want, ost = o.render_wavefront()
    assert np.array_equal(bits(img), bits(want))
    assert ost["bvh4_mismatches"] == 0
    # out of core the queues run domain by domain in score order, so fewer
    # entries see a nearer hit before they start
    hi = 1.25 if cache < 0 else 2.0
    for k, g in (("bvh4_nodes", "nodes_radiance"), ("bvh4_tris", "tris_radiance"),
                 ("bvh4_visits", "visits_radiance")):
        r = st[g] / ost[k]
        print(f"{g}: gpu {st[g]} oracle {ost[k]} ratio {r:.4f}")
        assert 0.9 <= r <= hi, (g, st[g], ost[k])
    t.close()
