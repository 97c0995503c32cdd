"""The C++ film-mode driver (spray_ooc's command line over the C ABI)."""
import subprocess

import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import build as B
from spray_gb300 import image, scenes
from conftest import small_config

pytestmark = pytest.mark.gpu


def test_film_driver_matches_library(lib_built, tmp_path):
    path = scenes.write_wavelet_grid(tmp_path, grid=2, samples=20, colors="albedo", light="point")
    scene = sg.Scene.load(path, path.parent)
    pos, look, _ = scenes.orbit_camera(scene)
    out = tmp_path / "out.ppm"
    cmd = [str(B.FILM), "--mode", "film", "--frames", "2", "-w", "80", "-h", "60", "--pixel-samples", "2",
           "--bounces", "3", "--ao-samples", "2", "--fov", "60", "--blinn", "0.4", "0.4", "0.4", "10",
           "--camera", *[f"{v:.9g}" for v in (*pos, *look)], "--ply-path", str(path.parent),
           "-o", str(out), str(path)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert "Mrays/s" in r.stdout
    t = sg.Tracer(small_config(image_w=80, image_h=60, ao_mode=0, pixel_samples=2, bounces=3, ao_samples=2,
                               fov=60.0, ks=[0.4, 0.4, 0.4], shininess=10.0))
    t.set_scene(scene)
    cam = [float(f"{v:.9g}") for v in (*pos, *look)]
    t.set_camera(cam[:3], cam[3:], (0, 1, 0))
    img, _ = t.trace()
    assert np.array_equal(image.read_ppm(out), image.read_ppm_bytes(image.ppm_bytes(img)))


def test_film_driver_rejects_interactive_mode(lib_built, tmp_path):
    r = subprocess.run([str(B.FILM), "--mode", "glfw", "x.spray"], capture_output=True, text=True)
    assert r.returncode == 2 and "unavailable" in r.stderr
