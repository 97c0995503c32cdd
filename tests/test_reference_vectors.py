"""The oracle against the reference's own code, function by function.

tests/golden/refvec.py lists the groups, the reference function each pins
(file:line) and its match rule; tests/golden/reference_vectors.json holds the
reference's outputs for seeded inputs (tests/golden/make_reference_vectors.py
wrote it from oracle/_ref, which oracle/build_ref.sh compiles from the
reference's sources).  Where oracle/_ref exists, the oracle is also checked
against the live libraries on fresh inputs."""
import json

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
