"""Oracle known-answer tests: RNG, sin/cos, slab test, triangle test, LRU
cache, blocking tiles, and mode A (speculative loop) vs mode B (wavefront)."""
import math
from pathlib import Path

import numpy as np
import pytest

from spray_gb300 import scenes
from conftest import small_config

M32 = 0xFFFFFFFF


def py_rng(seed, n):
    """RandomSampler restated in Python (deps/embree/random_sampler.h:34-108)."""
    k = (seed & M32) * 0xcc9e2d51 & M32
    k = ((k << 15) | (k >> 17)) & M32
    k = k * 0x1b873593 & M32
    h = 0 ^ k
    h = ((((h << 13) | (h >> 19)) & M32) * 5 + 0xe6546b64) & M32
    h ^= h >> 16
    h = h * 0x85ebca6b & M32
    h ^= h >> 13
    h = h * 0xc2b2ae35 & M32
    h ^= h >> 16
    out = []
    for _ in range(n):
        h = (h * 1664525 + 1013904223) & M32
        out.append(np.float32(np.float32(h >> 1) * np.float32(4.656612873077392578125e-10)))
    return np.array(out, np.float32)


@pytest.mark.parametrize("seed", [0, 1, 7, 1023, 123456, -5, 2**31 - 1])
def test_rng_matches_formula(oracle_mod, seed):
    assert np.array_equal(oracle_mod.rng_floats(seed, 16), py_rng(seed, 16))


def test_rng_range(oracle_mod):
    x = oracle_mod.rng_floats(42, 100000)
    assert x.min() >= 0.0 and x.max() < 1.0 and abs(x.mean() - 0.5) < 0.01


def test_sincos_accuracy(oracle_mod):
    x = np.linspace(0.0, 2 * math.pi, 200001, dtype=np.float32)
    s, c = oracle_mod.sincos(x)
    xs = x.astype(np.float64)
    assert np.abs(s - np.sin(xs)).max() < 4e-7
    assert np.abs(c - np.cos(xs)).max() < 4e-7


def py_slab(b, o, d, t0=np.float32(0.001), t1=np.float32(np.inf)):
    """aabb.h:139-169 in numpy float32."""
    f = np.float32
    with np.errstate(all="ignore"):
        inv = [f(1.0) / f(x) for x in d]
        sg = [int(i < 0) for i in inv]
        lo, hi = [f(x) for x in b[:3]], [f(x) for x in b[3:]]
        bnd = [lo, hi]
        tmin = (bnd[sg[0]][0] - f(o[0])) * inv[0]
        tmax = (bnd[1 - sg[0]][0] - f(o[0])) * inv[0]
        tymin = (bnd[sg[1]][1] - f(o[1])) * inv[1]
        tymax = (bnd[1 - sg[1]][1] - f(o[1])) * inv[1]
        if tmin > tymax or tymin > tmax:
            return False, None
        if tymin > tmin:
            tmin = tymin
        if tymax < tmax:
            tmax = tymax
        tzmin = (bnd[sg[2]][2] - f(o[2])) * inv[2]
        tzmax = (bnd[1 - sg[2]][2] - f(o[2])) * inv[2]
        if tmin > tzmax or tzmin > tmax:
            return False, None
        if tzmin > tmin:
            tmin = tzmin
        if tzmax < tmax:
            tmax = tzmax
        return bool(tmin < t1 and tmax > t0), tmin


SLAB_CASES = [
    ([0, 0, 0, 1, 1, 1], [-1, 0.5, 0.5], [1, 0, 0]),          # zero y, z components
    ([0, 0, 0, 1, 1, 1], [-1, 0.0, 0.5], [1, 0, 0]),          # origin on the y = 0 plane
    ([0, 0, 0, 1, 1, 1], [-1, 1.0, 0.5], [1, -0.0, 0]),       # on the upper plane, -0 direction
    ([0, 0, 0, 1, 1, 1], [0.5, 0.5, 0.5], [0.3, 0.4, 0.5]),   # origin inside: tmin < 0
    ([0, 0, 0, 1, 1, 1], [2, 2, 2], [1, 1, 1]),               # box behind
    ([0, 0, 0, 1, 1, 1], [-1, -1, -1], [1, 1, 1]),            # diagonal through corners
    ([0, 0, 0, 1, 1, 1], [1.0005, 0.5, 0.5], [1, 0, 0]),      # exit before t0
    ([0, 0, 0, 1, 1, 1], [0.5, 2, 0.5], [0, -1, 0]),
    ([-3, -2, 5, 4, 7, 9], [0.1, 0.2, -10], [0.01, 0.02, 1]),
    ([0, 0, 0, 1, 1, 1], [0, 0, 0], [0, 0, 0]),               # degenerate direction
]


@pytest.mark.parametrize("b,o,d", SLAB_CASES)
def test_slab_matches_reference_formula(oracle_mod, b, o, d):
    hit, tmin, _ = oracle_mod.slab(b, o, d)
    ph, pt = py_slab(b, o, d)
    assert hit == ph
    if hit:
        assert np.float32(tmin).tobytes() == np.float32(pt).tobytes()


def test_triangle_known_answers(oracle_mod):
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    hit, t, u, v = oracle_mod.triangle([0.25, 0.5, -2], [0, 0, 1], tri)
    assert hit and t == 2.0 and u == 0.25 and v == 0.5
    assert not oracle_mod.triangle([0.75, 0.75, -2], [0, 0, 1], tri)[0]       # outside
    assert not oracle_mod.triangle([0.25, 0.25, 1], [0, 0, 1], tri)[0]        # behind
    assert not oracle_mod.triangle([0.25, 0.25, -0.0005], [0, 0, 1], tri)[0]  # t < 1e-3
    assert oracle_mod.triangle([0.25, 0.25, 2], [0, 0, -1], tri)[0]           # back face
    # watertight: a ray through the shared edge of two triangles hits one of them
    tri2 = np.array([[1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    for x in np.linspace(0.01, 0.99, 37, dtype=np.float32):
        o = [x, np.float32(1) - x, -1]
        assert oracle_mod.triangle(o, [0, 0, 1], tri)[0] or oracle_mod.triangle(o, [0, 0, 1], tri2)[0]


def test_lru_trace(oracle_mod):
    # lru_cache.cc:65-171: capacity 2, LRU at the front
    ids = [0, 1, 0, 2, 1, 3, 0, 3, 3]
    assert oracle_mod.lru_trace(4, 2, ids).tolist() == [0, 0, 1, 0, 0, 0, 0, 1, 1]
    # capacity >= domains behaves like the infinite cache
    assert oracle_mod.lru_trace(3, -1, [0, 1, 2, 0, 1, 2]).tolist() == [0, 0, 0, 1, 1, 1]
    assert oracle_mod.lru_trace(3, 1, [0, 0, 1, 0]).tolist() == [0, 1, 0, 0]


@pytest.mark.parametrize("w,h,spp,expect", [
    (1024, 1024, 1, [(0, 0, 1024, 1024)]),
    (1920, 1080, 16, [(0, 33 * i, 1920, 33) for i in range(32)] + [(0, 1056, 1920, 24)]),
    (2048, 2048, 8, [(0, 64 * i, 2048, 64) for i in range(32)]),
    (400, 400, 4, [(0, 0, 400, 400)]),
])
def test_blocking_tiles(oracle_mod, w, h, spp, expect):
    sc = scenes.wavelet_grid(1, 8)
    o = oracle_mod.Oracle(small_config(image_w=w, image_h=h, pixel_samples=spp), sc)
    assert [tuple(t) for t in o.tiles()] == expect


def test_vertical_stripes(oracle_mod):
    sc = scenes.wavelet_grid(1, 8)
    got = []
    for r in range(3):
        o = oracle_mod.Oracle(small_config(image_w=100, image_h=10, num_ranks=3, rank=r), sc)
        got.append([tuple(t) for t in o.tiles()])
    assert got == [[(0, 0, 33, 10)], [(33, 0, 33, 10)], [(66, 0, 34, 10)]]


def _modes(oracle_mod, scene, cfg, threads=1):
    o = oracle_mod.Oracle(cfg, scene)
    pos, look, up = scenes.orbit_camera(scene)
    o.set_camera(pos, look, up)
    a, sa = o.render_speculative(threads)
    b, sb = o.render_wavefront()
    return a, b, sa, sb


@pytest.mark.parametrize("mode,spp,bounces,light,threads", [
    ("ao", 1, 1, "point", 1), ("ao", 2, 2, "point", 2), ("pt", 1, 1, "point", 1),
    ("pt", 2, 3, "point+diffuse", 1), ("pt", 2, 4, "point+diffuse", 3), ("pt", 1, 2, "quad", 1),
])
def test_speculative_loop_equals_wavefront(oracle_mod, mode, spp, bounces, light, threads):
    """Mode A (the reference loop) and mode B (wavefront) render the same image
    up to float accumulation order whenever no ray passes the history wrap."""
    sc = scenes.wavelet_grid(2, 20, colors="albedo", light=light)
    cfg = small_config(ao_mode=int(mode == "ao"), pixel_samples=spp, bounces=bounces, ao_samples=3,
                       max_samples_per_rank=2048)
    a, b, sa, sb = _modes(oracle_mod, sc, cfg, threads)
    assert sa["rays_primary"] == sb["rays_primary"]
    assert np.abs(a - b).max() <= 1e-6
    assert b[..., :3].max() > 0


def test_history_wrap_stays_within_tolerance(oracle_mod):
    """Beyond SPRAY_HISTORY_SIZE bounces the reference also continues wrong-path
    rays from its pending queue; the images still agree within 1e-3 RMSE."""
    sc = scenes.wavelet_grid(2, 20, colors="albedo", light="quad")
    cfg = small_config(ao_mode=0, pixel_samples=16, bounces=5, rr_depth=3, ao_samples=1,
                       max_samples_per_rank=8192)
    a, b, _, _ = _modes(oracle_mod, sc, cfg, threads=2)
    rmse = np.sqrt(np.mean((a[..., :3] - b[..., :3]) ** 2))
    assert 0 < rmse < 1e-3


def test_ao_of_open_plane_is_vertex_color(oracle_mod):
    """AO of an unoccluded plane: sum of cos/(pi N pdf) weights = albedo."""
    import spray_gb300 as sg
    v = np.array([[-10, 0, -10], [10, 0, -10], [10, 0, 10], [-10, 0, 10]], np.float32)
    f = np.array([[0, 1, 2], [0, 2, 3]], np.uint32)
    col = np.full(4, (200 << 16) | (100 << 8) | 50, np.uint32)
    sc = sg.Scene([sg.Domain(v, f, col)], [sg.Light(0, (0, 10, 0))])
    o = oracle_mod.Oracle(small_config(image_w=16, image_h=16, ao_samples=16), sc)
    o.set_camera((0.3, 5, 0.2), (0, 0, 0), (0, 0, 1), 40.0)
    img, _ = o.render_wavefront()
    # the hit colour is interpolated and truncated to integers
    # (trimesh_buffer.cc:345-350), so a channel can read one step lower
    c = np.array([200, 100, 50], np.float64)
    hi = c * 0.00392156862745098
    lo = (c - 1) * 0.00392156862745098
    px = img[..., :3].astype(np.float64)
    assert np.all(px <= hi * (1 + 3e-6)) and np.all(px >= lo * (1 - 3e-6))
    assert np.mean(np.abs(px - hi) <= hi * 3e-6) > 0.8


REF_RNG = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "libref_rng.so"


@pytest.mark.skipif(not REF_RNG.exists(), reason="reference sampler not built (reference tree absent)")
def test_rng_matches_the_reference_sampler():
    """The oracle's sampler equals the reference's own RandomSampler
    (deps/embree/random_sampler.h, built by oracle/build_ref.sh), bit for bit,
    for the seed forms the tracer uses: tile-local sample ids (eye jitter),
    pixel * (l + 1) (AO), sample * depth (bounces) and their wrap-arounds."""
    import ctypes as C
    from oracle import oracle as O
    L = C.CDLL(str(REF_RNG))
    L.ref_rng.argtypes = [C.c_int32, C.c_int32, C.c_void_p]
    rng = np.random.default_rng(3)
    seeds = [0, 1, -1, 2 ** 31 - 1, -(2 ** 31)] + list(rng.integers(-(2 ** 31), 2 ** 31, 200))
    seeds += [p * (l + 1) for p in (0, 5, 1919, 2073599) for l in range(8)]
    for seed in seeds:
        seed = int(np.int32(np.int64(seed) & 0xFFFFFFFF if seed >= 0 else seed))
        want = np.zeros(16, np.float32)
        L.ref_rng(seed, 16, want.ctypes.data)
        got = O.rng_floats(seed, 16)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), seed
