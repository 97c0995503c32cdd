"""Writes reference_vectors.json (seeded inputs and what the reference's own
code returns for them, per hot-path function: the groups of refvec.py) and
reference_scene.json (a .spray scene with its PLY files, and what the
reference's scene and PLY loaders make of them).

TEST INFRASTRUCTURE ONLY.  Run it where the reference sources are present:

    python tests/golden/make_reference_vectors.py [--reference-dir DIR]

It builds oracle/_ref with oracle/build_ref.sh (the reference's sources are
compiled where they lie; nothing is copied), calls those libraries on the
inputs of refvec.make_cases(seed=2024, scale=1) and stores both as base64
arrays.  tests/test_reference_vectors.py checks the oracle against the file.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE.parent))

import numpy as np  # noqa: E402

from golden import refvec as V  # noqa: E402

SEED, SCALE = 2024, 1


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--reference-dir", default=str(V.REFERENCE_SOURCES))
    args = ap.parse_args()
    env = dict(os.environ, SPRAY_REFERENCE_DIR=args.reference_dir)
    subprocess.run(["sh", str(ROOT / "oracle" / "build_ref.sh")], check=True, env=env)
    libs = V.load_reference()
    if libs is None:
        print("reference sources absent: nothing written", file=sys.stderr)
        return 1
    cases = V.make_cases(SEED, SCALE)
    ref = V.reference_outputs(cases, libs)
    doc = {
        "about": "inputs and outputs of the reference's own hot-path functions, compiled from its sources "
                 "by oracle/build_ref.sh; made by tests/golden/make_reference_vectors.py",
        "seed": SEED,
        "scale": SCALE,
        "groups": {g: {"in": {k: V.encode(a) for k, a in cases[g].items()} if g in cases else {},
                       "out": {k: V.encode(a) for k, a in ref[g].items()}} for g in V.GROUPS},
    }
    # refract reads the fr_dielectric inputs
    doc["groups"]["refract"]["in"] = {}
    V.FIXTURE.write_text(json.dumps(doc, indent=1, sort_keys=True) + "\n")
    print(f"{V.FIXTURE}: {V.FIXTURE.stat().st_size} bytes, {len(V.GROUPS)} groups")

    files = V.make_scene_files()
    with tempfile.TemporaryDirectory() as tmp:
        out = V.reference_scene_outputs(V.write_scene_files(files, Path(tmp)), libs)
    scene = {
        "about": "a .spray scene and its PLY files, and what the reference's SceneLoader, PlyLoader and "
                 "TriMeshBuffer vertex transform make of them; made by tests/golden/make_reference_vectors.py",
        "files": {k: V.encode(np.frombuffer(b, np.uint8)) for k, b in files.items()},
        "out": {k: V.encode(a) for k, a in out.items()},
    }
    V.SCENE_FIXTURE.write_text(json.dumps(scene, indent=1, sort_keys=True) + "\n")
    print(f"{V.SCENE_FIXTURE}: {V.SCENE_FIXTURE.stat().st_size} bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
