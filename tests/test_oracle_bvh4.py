"""The oracle's ordered walk over the product's 4-wide BVH layout, the counts
behind the traversal roofline's oracle-counted bytes.

The hierarchies come from prepared domain blobs (spray_scene_prepare, built on
the host cores; no GPU needed).  Walking them must give every ray exactly the
oracle's own closest hit (its independent binary BVH and the same watertight
triangle test), so a corrupt layout or a wrong reading of it shows up as
mismatches; the counted work is then that of the product's hierarchy."""
import numpy as np
import pytest

import spray_gb300 as sg
from oracle import oracle as O
from spray_gb300 import scenes
from conftest import small_config


@pytest.fixture(scope="module")
def grid_blobs(lib_built, tmp_path_factory):
    sc = scenes.wavelet_grid(3, 16, colors="albedo", light="point+diffuse")
    where = tmp_path_factory.mktemp("blobs")
    sg.prepare_scene(sc, where)
    return sc, where


def test_walk_over_the_product_layout_finds_the_oracle_hits(oracle_mod, grid_blobs):
    sc, where = grid_blobs
    cfg = small_config(image_w=48, image_h=36, ao_mode=0, ao_samples=2, pixel_samples=2, bounces=3)
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*scenes.orbit_camera(sc))
    plain, st0 = o.render_wavefront()
    assert st0["bvh4_nodes"] == 0
    for d in range(len(sc.domains)):
        nodes, tris = O.read_blob_bvh(where / f"domain_{d:05d}.sdom")
        o.set_bvh4(d, nodes, tris)
    img, st = o.render_wavefront()
    assert np.array_equal(img.view(np.uint32), plain.view(np.uint32))
    assert st["bvh4_mismatches"] == 0
    # the walk skips domains whose entry lies beyond the hit found so far
    assert 0 < st["bvh4_visits"] <= st["visits_radiance"]
    assert st["bvh4_nodes"] > st["bvh4_visits"] and st["bvh4_tris"] > 0
    o.close()


def test_a_corrupt_hierarchy_is_caught(oracle_mod, grid_blobs):
    # a node box shrunk to nothing hides its subtree: rays whose hit lies
    # there find another (or none), which the comparison reports
    sc, where = grid_blobs
    cfg = small_config(image_w=48, image_h=36, ao_mode=1, ao_samples=1, pixel_samples=1, bounces=1)
    o = oracle_mod.Oracle(cfg, sc)
    o.set_camera(*scenes.orbit_camera(sc))
    org, dir, _, _ = o.eyes(0, len(o.tiles()))
    h = o.closest(org, dir)
    seen = np.bincount(h["domain"][h["hit"] == 1], minlength=len(sc.domains))
    victim = int(np.argmax(seen))  # the domain that holds the most primary hits
    assert seen[victim] > 0
    for d in range(len(sc.domains)):
        nodes, tris = O.read_blob_bvh(where / f"domain_{d:05d}.sdom")
        nodes = nodes.copy().reshape(-1, 32)
        if d == victim:
            nodes[0, 0:4] = np.inf   # lo x of the root's children
            nodes[0, 4:8] = -np.inf  # hi x
        o.set_bvh4(d, nodes, tris)
    _, st = o.render_wavefront()
    assert st["bvh4_mismatches"] > 0
    o.close()
