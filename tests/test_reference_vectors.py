"""The oracle, and the product's scene loader, against the reference's own
code, function by function.

tests/golden/refvec.py lists the groups, the reference function each pins
(file:line) and its match rule; tests/golden/reference_vectors.json holds the
reference's outputs for seeded inputs (tests/golden/make_reference_vectors.py
wrote it from oracle/_ref, which oracle/build_ref.sh compiles from the
reference's sources).  Where oracle/_ref exists, the oracle is also checked
against the live libraries on fresh inputs.  The product's scene loader is
held to the reference's SceneLoader, PlyLoader and vertex transform on the
scene of tests/golden/reference_scene.json and on the reference's example
scenes."""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from golden import refvec as V

LIBS = V.load_reference()
needs_ref = pytest.mark.skipif(LIBS is None, reason="oracle/_ref not built (reference sources absent)")


@pytest.fixture(scope="module")
def vectors(oracle_mod):
    doc = json.loads(V.FIXTURE.read_text())
    cases = {g: {k: V.decode(a) for k, a in d["in"].items()} for g, d in doc["groups"].items()}
    ref = {g: {k: V.decode(a) for k, a in d["out"].items()} for g, d in doc["groups"].items()}
    return cases, ref, V.oracle_outputs(cases)


def test_fixture_covers_every_group(vectors):
    cases, ref, _ = vectors
    assert sorted(ref) == sorted(V.GROUPS)
    assert all(ref[g] for g in V.GROUPS)


@pytest.mark.parametrize("group", V.GROUPS)
def test_oracle_matches_reference_vectors(vectors, group):
    cases, ref, orc = vectors
    V.compare(group, cases, ref, orc)


@needs_ref
def test_fixture_matches_the_reference_libraries(vectors):
    """The committed outputs are what the reference's code returns today."""
    cases, ref, _ = vectors
    live = V.reference_outputs(cases, LIBS)
    for g in V.GROUPS:
        for k, a in ref[g].items():
            assert np.array_equal(np.ascontiguousarray(live[g][k]).view(np.uint8),
                                  np.ascontiguousarray(a).view(np.uint8)), (g, k)


@needs_ref
@pytest.mark.parametrize("seed", [7, 11])
def test_oracle_matches_reference_code_on_fresh_inputs(oracle_mod, seed):
    cases = V.make_cases(seed, 8)
    ref = V.reference_outputs(cases, LIBS)
    orc = V.oracle_outputs(cases)
    for g in V.GROUPS:
        V.compare(g, cases, ref, orc)


def test_a_planted_oracle_error_is_caught(vectors):
    """The comparison is not vacuous: one ulp moved in an oracle output of
    each bit-exact group fails it."""
    cases, ref, orc = vectors
    for g, k in [("camera", "dir"), ("slab", "tmin_tmax"), ("fr_dielectric", "wt"), ("unpack", "rgb"),
                 ("local_to_world", "out"), ("rng", "floats")]:
        bad = {gg: {kk: np.array(a, copy=True) for kk, a in d.items()} for gg, d in orc.items()}
        flat = bad[g][k].reshape(-1).view(np.uint32)
        i = int(np.flatnonzero(flat)[0])
        flat[i] += 1
        with pytest.raises(AssertionError):
            V.compare(g, cases, ref, bad)


@pytest.fixture(scope="module")
def scene_vectors():
    doc = json.loads(V.SCENE_FIXTURE.read_text())
    files = {k: V.decode(a).tobytes() for k, a in doc["files"].items()}
    return files, {k: V.decode(a) for k, a in doc["out"].items()}


def test_scene_loader_matches_reference_vectors(lib_built, scene_vectors, tmp_path):
    """World-space vertices and bounds bit for bit (rotations, scales,
    translations, binary and ASCII PLY), faces, colours, materials, lights."""
    files, ref = scene_vectors
    V.compare_scene(ref, V.product_scene_outputs(V.write_scene_files(files, tmp_path)))


def test_scene_comparison_catches_a_left_to_right_transform(scene_vectors):
    """Summing m * (x, y, z, 1) left to right instead of in glm's pairwise
    order moves vertices of the domains rotated about y and translated; the
    comparison fails on it (as it did on the product's earlier transform)."""
    files, ref = scene_vectors
    raw = files["bin.ply"]
    body = raw[raw.index(b"end_header\n") + len(b"end_header\n"):]
    nv = int(ref["nverts"][0])
    obj = np.frombuffer(body[:nv * 15], [("p", "<f4", 3), ("c", "u1", 3)])["p"].astype(np.float32)
    names = [ln.split()[1] for ln in files["scene.spray"].decode().splitlines() if ln.startswith("file ")]
    offs = np.concatenate([[0], np.cumsum(ref["nverts"])])
    bad = {k: np.array(a, copy=True) for k, a in ref.items()}
    changed = 0
    for i, name in enumerate(names):
        M = ref["transform"][i].reshape(4, 4)
        if name != "bin.ply" or np.array_equal(M, np.eye(4, dtype=np.float32)):
            continue
        x, y, z = obj[:, 0:1], obj[:, 1:2], obj[:, 2:3]
        l2r = ((M[0, :3] * x + M[1, :3] * y) + M[2, :3] * z) + M[3, :3]
        seg = bad["vertices"][offs[i]:offs[i + 1]]
        changed += int(np.any(l2r.view(np.uint32) != seg.view(np.uint32)))
        seg[:] = l2r
    assert changed >= 1
    with pytest.raises(AssertionError):
        V.compare_scene(ref, bad)


@needs_ref
def test_scene_fixture_matches_the_reference_libraries(scene_vectors, tmp_path):
    files, ref = scene_vectors
    live = V.reference_scene_outputs(V.write_scene_files(files, tmp_path), LIBS)
    for k, a in ref.items():
        assert np.array_equal(np.ascontiguousarray(live[k]).view(np.uint8), np.ascontiguousarray(a).view(np.uint8)), k


REF_EXAMPLES = V.REFERENCE_SOURCES / "examples"


@needs_ref
@pytest.mark.skipif(not REF_EXAMPLES.exists(), reason="reference examples absent")
@pytest.mark.parametrize("spray,ply_dir", [("wavelets64/wavelets64.spray", "."),
                                           ("wavelet/wavelet_example.spray", "wavelet")])
def test_reference_example_scenes_load_like_the_reference(lib_built, spray, ply_dir):
    ref = V.reference_scene_outputs(REF_EXAMPLES / spray, LIBS, REF_EXAMPLES / ply_dir)
    V.compare_scene(ref, V.product_scene_outputs(REF_EXAMPLES / spray, REF_EXAMPLES / ply_dir))
