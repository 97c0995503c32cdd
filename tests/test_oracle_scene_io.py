"""The oracle's own scene reader (oracle/scene_io.py) against the reference's
loader outputs and against the product's loader.

The reference-timing arm of bench.py loads its scene through this reader so
that it never maps the CUDA library; these checks show it sees the scene the
product traces: the same world-space vertices and bounds bit for bit, faces,
colours, materials and lights.
"""
import json

import numpy as np

from golden import refvec as V
from oracle import scene_io
from spray_gb300 import scenes


def _scene_files(tmp_path):
    doc = json.loads(V.SCENE_FIXTURE.read_text())
    files = {k: V.decode(a).tobytes() for k, a in doc["files"].items()}
    return V.write_scene_files(files, tmp_path), {k: V.decode(a) for k, a in doc["out"].items()}


def test_oracle_reader_matches_reference_vectors(tmp_path):
    # rotations about x, y and z, scales, chained and negative transforms,
    # binary and ASCII PLY, every material kind, point and hemisphere lights
    spray, ref = _scene_files(tmp_path)
    V.compare_scene(ref, V.oracle_scene_outputs(spray))


def test_oracle_reader_matches_product_loader(lib_built, tmp_path):
    import spray_gb300 as sg
    spray, _ = _scene_files(tmp_path)
    a, b = scene_io.load(spray, spray.parent), sg.Scene.load(spray, spray.parent)
    for x, y in zip(a.domains, b.domains):
        assert x.bsdf_type == y.bsdf_type
        assert np.array_equal(x.bsdf_params.view(np.uint32), y.bsdf_params.view(np.uint32))
    # a benchmark-style scene: quad light extension, packed grid, albedo colours
    path = scenes.write_wavelet_grid(tmp_path / "grid", 2, 12, colors="albedo", light="quad")
    a, b = scene_io.load(path, path.parent), sg.Scene.load(path, path.parent)
    assert len(a.domains) == len(b.domains) == 8
    for x, y in zip(a.domains, b.domains):
        assert np.array_equal(x.vertices.view(np.uint32), y.vertices.view(np.uint32))
        assert np.array_equal(x.bounds.view(np.uint32), y.bounds.view(np.uint32))
        assert np.array_equal(x.faces, y.faces) and np.array_equal(x.colors, y.colors)
    assert len(a.lights) == len(b.lights) == 1
    for f in ("type", "position", "radiance", "edge1", "edge2"):
        assert np.array_equal(np.asarray(getattr(a.lights[0], f)), np.asarray(getattr(b.lights[0], f))), f


def test_oracle_reader_catches_a_moved_vertex(tmp_path):
    spray, ref = _scene_files(tmp_path)
    out = V.oracle_scene_outputs(spray)
    out["vertices"] = np.array(out["vertices"], copy=True)
    out["vertices"].view(np.uint32)[5, 1] += 1
    try:
        V.compare_scene(ref, out)
    except AssertionError:
        return
    raise AssertionError("a one-ulp vertex change went unnoticed")
