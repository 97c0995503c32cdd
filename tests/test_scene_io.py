"""Scene file grammar, PLY reading/writing and the wavelet generator."""
import math
import os
from pathlib import Path

import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from golden import refvec

REF_EXAMPLES = refvec.REFERENCE_SOURCES / "examples"


def test_wavelet_mesh_is_watertight_and_oriented(lib_built):
    v, f = sg.generate_wavelet(40)
    assert len(f) > 1000
    e = np.sort(np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]]), axis=1)
    _, c = np.unique(e, axis=0, return_counts=True)
    assert set(c.tolist()) == {2}  # every edge shared by exactly two triangles
    de = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    _, c2 = np.unique(de, axis=0, return_counts=True)
    assert c2.max() == 1  # consistent winding
    assert np.all(np.abs(v) <= 1.0)


def test_wavelet_deterministic_and_phase_dependent(lib_built):
    a = sg.generate_wavelet(32, 157.0, (0, 0, 0))
    b = sg.generate_wavelet(32, 157.0, (0, 0, 0))
    c = sg.generate_wavelet(32, 157.0, (1.0, 2.0, 3.0))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert len(c[1]) != len(a[1]) or not np.array_equal(c[0], a[0])


def test_ply_roundtrip_binary(lib_built, tmp_path):
    v, f = sg.generate_wavelet(20)
    col = (np.arange(len(v)) * 2654435761 % (1 << 24)).astype(np.uint32)
    p = tmp_path / "m.ply"
    sg.write_ply(p, v, f, col)
    spray = tmp_path / "s.spray"
    spray.write_text("domain\nfile m.ply\nmtl diffuse 1 1 1\nbound -1 -1 -1 1 1 1\n"
                     f"face {len(f)}\nvertex {len(v)}\n")
    s = sg.Scene.load(spray, tmp_path)
    d = s.domains[0]
    assert np.array_equal(d.vertices, v) and np.array_equal(d.faces, f)
    assert np.array_equal(d.colors, col)


def test_ply_ascii_and_transforms(lib_built, tmp_path):
    (tmp_path / "tri.ply").write_text(
        "ply\nformat ascii 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
        "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\n"
        "element face 1\nproperty list uchar int vertex_indices\nend_header\n"
        "0 0 0 255 0 0\n1 0 0 0 255 0\n0 1 0 0 0 255\n3 0 1 2\n")
    (tmp_path / "s.spray").write_text(
        "# comment\nlight point 1 2 3 0.5 0.5 0.5\nlight diffuse .1 .2 .3\n\n"
        "domain\nfile tri.ply\nmtl mirror 1 1 1\nbound 0 0 0 1 1 0\nscale 2 2 2\n"
        "translate 1 0 0\nface 1\nvertex 3\n"
        "domain\nfile tri.ply\nmtl glass 1 1.5\nbound 0 0 0 1 1 0\nrotate z 90\nface 1\nvertex 3\n")
    s = sg.Scene.load(tmp_path / "s.spray", tmp_path)
    assert len(s.domains) == 2 and len(s.lights) == 2
    assert s.lights[0].type == sg.Light.POINT and np.allclose(s.lights[0].position, [1, 2, 3])
    assert s.lights[1].type == sg.Light.DIFFUSE
    d0, d1 = s.domains
    # glm order: scale then translate in object space -> x' = 2x + 2
    assert np.allclose(d0.vertices, [[2, 0, 0], [4, 0, 0], [2, 2, 0]])
    assert np.allclose(d0.bounds, [2, 0, 0, 4, 2, 0])
    assert d0.bsdf_type == 1 and d1.bsdf_type == 2
    assert np.allclose(d1.bsdf_params[:2], [1, 1.5])
    assert np.allclose(d1.vertices, [[0, 0, 0], [0, 1, 0], [-1, 0, 0]], atol=1e-6)
    assert np.array_equal(d0.colors, [0xff0000, 0x00ff00, 0x0000ff])


@pytest.mark.parametrize("text,frag", [
    ("domain\nfile x.ply\nbogus 1\n", "unknown tag"),
    ("domain\nmtl plastic 1 1 1\n", "unknown material"),
    ("file x.ply\n", "before 'domain'"),
    ("light point 1 2 3\n", "light point"),
    ("# only a comment\n", "no domains"),
])
def test_malformed_scene_rejected(lib_built, tmp_path, text, frag):
    p = tmp_path / "bad.spray"
    p.write_text(text)
    with pytest.raises(sg.SprayError) as e:
        sg.Scene.load(p)
    assert e.value.code == sg.EIO and frag in str(e.value)


def test_truncated_ply_rejected(lib_built, tmp_path):
    v, f = sg.generate_wavelet(12)
    sg.write_ply(tmp_path / "m.ply", v, f)
    data = (tmp_path / "m.ply").read_bytes()
    (tmp_path / "m.ply").write_bytes(data[: len(data) // 2])
    (tmp_path / "s.spray").write_text("domain\nfile m.ply\nbound -1 -1 -1 1 1 1\n")
    with pytest.raises(sg.SprayError):
        sg.Scene.load(tmp_path / "s.spray", tmp_path)


def test_written_grid_matches_in_memory_scene(lib_built, tmp_path):
    p = scenes.write_wavelet_grid(tmp_path, grid=2, samples=16, colors="albedo", light="point")
    a = sg.Scene.load(p, p.parent)
    b = scenes.wavelet_grid(2, 16, colors="albedo", light="point")
    assert len(a.domains) == 8
    for da, db in zip(a.domains, b.domains):
        assert np.array_equal(da.faces, db.faces) and np.array_equal(da.colors, db.colors)
        assert np.allclose(da.vertices, db.vertices, atol=0, rtol=0) or np.allclose(da.vertices, db.vertices)
        assert np.allclose(da.bounds, db.bounds, atol=1e-6)


@pytest.mark.skipif(not REF_EXAMPLES.exists(), reason="reference examples not mounted")
def test_reference_example_scenes_parse(lib_built):
    s = sg.Scene.load(REF_EXAMPLES / "wavelets64" / "wavelets64.spray", REF_EXAMPLES)
    assert len(s.domains) == 64 and len(s.lights) == 1
    assert all(len(d.faces) == 5480 and len(d.vertices) == 2840 for d in s.domains)
    assert np.allclose(s.domains[1].bounds, [10, -10, -10, 30, 9.324713, 10], atol=1e-5)
    s2 = sg.Scene.load(REF_EXAMPLES / "wavelet" / "wavelet_example.spray", REF_EXAMPLES / "wavelet")
    assert len(s2.domains) == 2 and [l.type for l in s2.lights] == [0, 1]
    assert len(s2.domains[0].faces) == 1748 and len(s2.domains[1].faces) == 1684


def test_ppm_writer_semantics(tmp_path):
    from spray_gb300 import image
    img = np.zeros((2, 3, 4), np.float32)
    img[0, 0, :3] = [0.5, 2.0, -1.0]       # bottom-left pixel
    img[1, 2, :3] = [0.001, 0.9999, 1.0]    # top-right pixel
    data = image.ppm_bytes(img).decode().split("\n")
    assert data[:3] == ["P3", "3 2", "1023"]
    # rows from y = H-1 down; clamp(v * 1023) truncated (image.h:193-200)
    assert data[3 + 2] == "1 1022 1023"
    assert data[3 + 3] == "511 1023 0"
    assert np.array_equal(image.read_ppm_bytes(image.ppm_bytes(img))[0, 0], [511, 1023, 0])


def test_prepared_domain_blobs_round_trip(lib_built, tmp_path):
    """spray_scene_prepare writes one self-describing blob per domain (no GPU)."""
    import struct
    import spray_gb300 as sg
    from spray_gb300 import scenes
    scene = scenes.wavelet_grid(2, 16, colors="albedo", light="point")
    sg.prepare_scene(scene, tmp_path)
    files = sorted(tmp_path.glob("domain_*.sdom"))
    assert len(files) == len(scene.domains)
    for d, f in enumerate(files):
        raw = f.read_bytes()
        assert raw[:8] == b"SPRAYDOM"
        version, bsdf = struct.unpack_from("<Ii", raw, 8)
        bounds = struct.unpack_from("<6f", raw, 16)
        nv, nf, nn = struct.unpack_from("<3q", raw, 16 + 24 + 12 + 4)
        offs = struct.unpack_from("<6Q", raw, 16 + 24 + 12 + 4 + 24)
        dom = scene.domains[d]
        assert version == 1 and nv == len(dom.vertices) and nf == len(dom.faces) and nn > 0
        assert np.array_equal(np.float32(bounds), dom.bounds)
        assert offs[-1] == len(raw)
        faces = np.frombuffer(raw, np.uint32, 3 * nf, offs[2]).reshape(-1, 3)
        assert np.array_equal(faces, dom.faces)


def test_prepared_blob_errors(lib_built, tmp_path):
    import spray_gb300 as sg
    bad = tmp_path / "domain_00000.sdom"
    bad.write_bytes(b"not a blob" * 40)
    try:
        t = sg.Tracer(image_w=8, image_h=8)
    except sg.SprayError:
        pytest.skip("no GPU: the loader runs inside a tracer")
    with pytest.raises(sg.SprayError) as e:
        t.set_scene_prepared(tmp_path, 1)
    assert e.value.code == sg.EIO
