"""Benchmark and test scenes in SpRay's format.

The benchmark scenes are grids of domains, each the wavelet isosurface
f = 255 exp(-(x^2+y^2+z^2)/(2*0.5^2)) + 10 sin(60x+p0) + 18 sin(30y+p1)
    + 5 cos(40z+p2) = 157
on [-1,1]^3, translated into its cell of a g^3 grid whose cell size is the
largest domain extent, as the reference's example scene packs 64 copies of one
wavelet mesh at its bounding-box size (examples/wavelets64/wavelets64.spray:
bound -10..10, translate steps of 20), so neighbouring domain boxes touch.  Domain bounds are the object-space
AABB of the vertices, as ply_header_reader computes them
(src/apps/ply_header_reader.cc:86-103).  Colours are per-vertex uchar RGB
because the reference shades with vertex colour, not the mtl albedo
(src/render/trimesh_buffer.cc:328-350).
"""
from __future__ import annotations

import math
import os
from pathlib import Path

import numpy as np

from . import Domain, Light, Scene, generate_wavelet, write_ply

REPO = Path(__file__).resolve().parent.parent
SCENE_CACHE = Path(os.environ.get("SPRAY_SCENE_CACHE", REPO / "_scenes"))

# Workloads.  "reference" keys are the reference's Config fields; "ext" keys
# are the extensions, all off for reference-exact parity runs.
CONFIGS = {
    # 4x4x4 grid, AO, 1024^2, 1 spp, 8 AO rays, AO max distance 5% of the
    # diagonal plus one shadow ray toward the light
    "c1": dict(grid=4, samples=64, colors="grey", light="point", phase_seed=None,
               cfg=dict(image_w=1024, image_h=1024, ao_mode=1, ao_samples=8, pixel_samples=1,
                        bounces=1, fov=60.0),
               ext=dict(ao_max_distance_frac=0.05, ao_light_shadow=1)),
    # same scene, path tracing, per-domain albedo, quad light, 5 bounces with
    # Russian roulette after bounce 3, 16 spp, 1920x1080
    "c2": dict(grid=4, samples=64, colors="albedo", light="quad", phase_seed=None,
               cfg=dict(image_w=1920, image_h=1080, ao_mode=0, ao_samples=1, pixel_samples=16,
                        bounces=5, fov=60.0),
               ext=dict(rr_depth=3)),
    # 8x8x8 grid of phase-shifted 128^3 isosurfaces, path tracing, 2048^2,
    # 8 spp, 4 bounces; the device cache holds half of the domains (the
    # 8 GiB-of-16 GiB ratio of the workload description; the generated scene
    # is smaller, so the cap is given in domains like SpRay's --cache-size)
    "c3": dict(grid=8, samples=128, colors="albedo", light="quad", phase_seed=2024,
               cfg=dict(image_w=2048, image_h=2048, ao_mode=0, ao_samples=1, pixel_samples=8,
                        bounces=4, fov=60.0, list_size=22, cache_size=256),
               ext=dict()),
    # uneven multi-view batch over the C2 scene: 24 seeded views, resolutions
    # from {256, 512, 1024, 2048}^2, spp from {1, 4, 16}, half AO-only (8 rays,
    # max distance 5% of the diagonal, one light ray), half path tracing with
    # 4 bounces and Russian roulette after bounce 3 (views: c5_views)
    "c5": dict(grid=4, samples=64, colors="albedo", light="quad", phase_seed=None,
               cfg=dict(image_w=256, image_h=256, ao_mode=0, ao_samples=1, pixel_samples=1,
                        bounces=4, fov=60.0),
               ext=dict(), views=24, view_seed=5),
}

GREY = 200
ALBEDO_SEED = 7
CAMERA_SEED = 11


def _color(rgb) -> int:
    r, g, b = (int(v) for v in rgb)
    return (r << 16) | (g << 8) | b


def domain_albedo(n: int, seed: int = ALBEDO_SEED) -> np.ndarray:
    """Per-domain albedo drawn from U[0.3, 0.9], quantised to uchar."""
    rng = np.random.default_rng(seed)
    a = rng.uniform(0.3, 0.9, size=(n, 3))
    return np.clip(np.rint(a * 255.0), 0, 255).astype(np.uint32)


def domain_phases(n: int, seed: int | None) -> np.ndarray:
    if seed is None:
        return np.zeros((n, 3))
    return np.random.default_rng(seed).uniform(0.0, 2.0 * math.pi, size=(n, 3))


def grid_translations(grid: int, cell: float) -> np.ndarray:
    """Domain d = i + g*j + g*g*k sits at cell (i, j, k)."""
    t = []
    for k in range(grid):
        for j in range(grid):
            for i in range(grid):
                t.append((cell * i, cell * j, cell * k))
    return np.asarray(t, np.float32)


def domain_meshes(grid: int, samples: int, phase_seed: int | None):
    """Per-domain object-space meshes and the grid cell size (largest extent)."""
    n = grid ** 3
    phases = domain_phases(n, phase_seed)
    if phase_seed is None:
        base = generate_wavelet(samples, 157.0, (0.0, 0.0, 0.0))
        meshes = [base] * n
    else:
        # the generator runs in C++ without the GIL: one thread per core
        from concurrent.futures import ThreadPoolExecutor
        with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
            meshes = list(ex.map(lambda d: generate_wavelet(samples, 157.0, tuple(phases[d])), range(n)))
    cell = max(float((v.max(0) - v.min(0)).max()) for v, _ in meshes[: (1 if phase_seed is None else n)])
    cell = float(np.float32(cell))
    return meshes, cell


def scene_box(scene: Scene):
    b = np.array([d.bounds for d in scene.domains], np.float64)
    return b[:, :3].min(0), b[:, 3:].max(0)


def make_lights(kind: str, lo, hi) -> list[Light]:
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    c = 0.5 * (lo + hi)
    ext = hi - lo
    if kind == "point":
        return [Light(Light.POINT, position=(c[0], hi[1] + 2.0 * ext[1], c[2] + ext[2]),
                      radiance=(1.0, 1.0, 1.0))]
    if kind == "quad":
        s = 0.5 * ext[0]
        p0 = (c[0] - 0.5 * s, hi[1] + 0.5 * ext[1], c[2] - 0.5 * s)
        return [Light(Light.QUAD, position=p0, radiance=(2.0, 2.0, 2.0), edge1=(s, 0, 0),
                      edge2=(0, 0, s))]
    if kind == "point+diffuse":
        return [Light(Light.POINT, position=(c[0], hi[1] + 2.0 * ext[1], c[2] + ext[2]),
                      radiance=(0.6, 0.6, 0.6)),
                Light(Light.DIFFUSE, radiance=(0.3, 0.3, 0.3))]
    raise ValueError(kind)


def orbit_camera(scene: Scene, seed: int = CAMERA_SEED, frame: int = 0):
    """Pinhole on a seeded orbit around the scene centre, radius 1.2 x diagonal."""
    lo, hi = scene_box(scene)
    c = 0.5 * (lo + hi)
    diag = float(np.linalg.norm(hi - lo))
    rng = np.random.default_rng(seed + 7919 * frame)
    phi = rng.uniform(0.0, 2.0 * math.pi)
    elev = math.radians(rng.uniform(15.0, 40.0))
    r = 1.2 * diag
    pos = c + r * np.array([math.cos(elev) * math.sin(phi), math.sin(elev),
                            math.cos(elev) * math.cos(phi)])
    return pos.astype(np.float32), c.astype(np.float32), np.array([0, 1, 0], np.float32)


def scene_diagonal(scene: Scene) -> float:
    lo, hi = scene_box(scene)
    return float(np.linalg.norm(hi - lo))


def wavelet_grid(grid: int = 4, samples: int = 64, colors: str = "grey", light: str = "point",
                 phase_seed: int | None = None) -> Scene:
    """In-memory scene: the same domains the .spray writer produces."""
    n = grid ** 3
    meshes, cell = domain_meshes(grid, samples, phase_seed)
    trans = grid_translations(grid, cell)
    alb = domain_albedo(n) if colors == "albedo" else None
    domains = []
    for d in range(n):
        v, f = meshes[d]
        col = _color(alb[d]) if alb is not None else _color((GREY, GREY, GREY))
        obj_lo, obj_hi = v.min(0), v.max(0)
        wv = (v + trans[d]).astype(np.float32)  # one float add per coordinate, as the loader does
        bounds = np.concatenate([obj_lo + trans[d], obj_hi + trans[d]]).astype(np.float32)
        domains.append(Domain(wv, f, np.full(len(v), col, np.uint32), bounds))
    sc = Scene(domains, [])
    sc.lights = make_lights(light, *scene_box(sc))
    return sc


def write_wavelet_grid(out_dir: Path, grid: int = 4, samples: int = 64, colors: str = "grey",
                       light: str = "point", phase_seed: int | None = None) -> Path:
    """Writes PLY files and a .spray scene file; returns the .spray path."""
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    spray = out_dir / "scene.spray"
    if spray.exists():
        return spray
    n = grid ** 3
    meshes, cell = domain_meshes(grid, samples, phase_seed)
    trans = grid_translations(grid, cell)
    alb = domain_albedo(n) if colors == "albedo" else None
    lo = np.min([meshes[d][0].min(0) + trans[d] for d in range(n)], axis=0)
    hi = np.max([meshes[d][0].max(0) + trans[d] for d in range(n)], axis=0)
    lines = []
    for l in make_lights(light, lo, hi):
        if l.type == Light.POINT:
            lines.append("light point %.9g %.9g %.9g %.9g %.9g %.9g" % (*l.position, *l.radiance))
        elif l.type == Light.DIFFUSE:
            lines.append("light diffuse %.9g %.9g %.9g" % tuple(l.radiance))
        else:
            lines.append("light quad " + " ".join("%.9g" % x for x in (*l.position, *l.edge1, *l.edge2,
                                                                      *l.radiance)))
    written = {}
    jobs = []
    for d in range(n):
        v, f = meshes[d]
        col = _color(alb[d]) if alb is not None else _color((GREY, GREY, GREY))
        key = (d if phase_seed is not None else -1, col)
        if key not in written:
            name = f"wavelet_{d:04d}.ply"
            jobs.append((out_dir / name, v, f, np.full(len(v), col, np.uint32)))
            written[key] = (name, v.min(0), v.max(0), len(v), len(f))
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        list(ex.map(lambda j: write_ply(*j), jobs))
    for d in range(n):
        v, f = meshes[d]
        col = _color(alb[d]) if alb is not None else _color((GREY, GREY, GREY))
        key = (d if phase_seed is not None else -1, col)
        name, blo, bhi, nv, nf = written[key]
        lines += ["", f"# domain {d}", "domain", f"file {name}", "mtl diffuse 1 1 1",
                  "bound %.9g %.9g %.9g %.9g %.9g %.9g" % (*blo, *bhi), f"face {nf}", f"vertex {nv}",
                  "translate %.9g %.9g %.9g" % tuple(trans[d])]
    tmp = spray.with_suffix(".tmp")
    tmp.write_text("\n".join(lines) + "\n")
    tmp.replace(spray)
    return spray


def scene_dir(name: str) -> Path:
    """Directory of a benchmark workload's generated .spray and PLY files."""
    spec = CONFIGS[name]
    return SCENE_CACHE / f"{name}_g{spec['grid']}_s{spec['samples']}_{spec['colors']}_{spec['light']}_packed"


def benchmark_scene(name: str) -> tuple[Path, dict]:
    """Generates (once) and returns the .spray file of a benchmark workload."""
    spec = CONFIGS[name]
    path = write_wavelet_grid(scene_dir(name), spec["grid"], spec["samples"], spec["colors"], spec["light"],
                              spec["phase_seed"])
    return path, spec


def c5_views(scene, n: int = 24, seed: int = 5) -> list[dict]:
    """The uneven multi-view batch: seeded orbit cameras, sizes, spp and shaders."""
    rng = np.random.default_rng(seed)
    diag = scene_diagonal(scene)
    views = []
    for k in range(n):
        pos, look, up = orbit_camera(scene, frame=k)
        res = int(rng.choice([256, 512, 1024, 2048]))
        spp = int(rng.choice([1, 4, 16]))
        v = dict(position=pos, lookat=look, up=up, vfov=60.0, image_w=res, image_h=res, pixel_samples=spp)
        if k % 2 == 0:
            v.update(ao_mode=1, ao_samples=8, bounces=1, ao_light_shadow=1, ao_max_distance=0.05 * diag,
                     rr_depth=0)
        else:
            v.update(ao_mode=0, ao_samples=1, bounces=4, rr_depth=3, ao_light_shadow=0, ao_max_distance=0.0)
        views.append(v)
    return views


def workload_config(name: str, scene=None) -> tuple[dict, dict]:
    """(spec, tracer configuration) of a benchmark workload; the AO range is a
    fraction of the scene diagonal, so it needs the scene."""
    spec = CONFIGS[name]
    cfg = dict(spec["cfg"])
    ext = dict(spec["ext"])
    frac = ext.pop("ao_max_distance_frac", None)
    if frac is not None and scene is not None:
        cfg["ao_max_distance"] = frac * scene_diagonal(scene)
    cfg.update({k: v for k, v in ext.items() if k != "cache_bytes"})
    return spec, cfg
