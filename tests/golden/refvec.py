"""Known-answer vectors from the reference's own code, and the rules that
compare the oracle with them.

TEST INFRASTRUCTURE ONLY.  ``oracle/build_ref.sh`` compiles the reference's
hot-path functions from its sources (``oracle/_ref/libref_path.so``,
``oracle/_ref/libref_rng.so``).  This module makes seeded inputs for each
function, runs them through those libraries (``reference_outputs``) or through
the oracle (``oracle_outputs``), and checks one against the other
(``compare``).  ``make_reference_vectors.py`` stores inputs and reference
outputs in ``reference_vectors.json`` so that the check runs where the
reference sources are absent.

Each group names the reference function it pins (file:line within the
reference's ``src/`` or ``deps/``):

============== ==================================================== =========
group          reference                                            match
============== ==================================================== =========
rng            RandomSampler_init/get1D, embree/random_sampler.h    bit-exact
slab           intersectAabb (float arrays), render/aabb.h:139-169  bit-exact
camera         Camera::init/generateRay, render/camera.h:128-209    bit-exact
disk           ConcentricDiskSampling, render/sampler.h:49-92       cos/sin
local_to_world localToWorld, render/sampler.h:101-110               bit-exact
cosine         getCosineHemisphereSample, render/sampler.cc:54-60   cos/sin
diffuse_light  DiffuseHemisphereLight::sampleArea, light.h:80-85    cos/sin
point_light    PointLight::sample, render/light.h:47-52             bit-exact
blinn_phong    blinnPhong, render/reflection.h:202-214              pow
reflect        Reflect, render/reflection.h:126-128                 bit-exact
fr_dielectric  FrDielectric, render/reflection.h:134-158            bit-exact
refract        Refract, render/reflection.h:160-174                 bit-exact
unpack         util::unpack, utils/util.h:75-79                     bit-exact
lru            LruCache::init/load, render/lru_cache.cc:41-171      exact
tiles          ImageScheduleTileList::init, render/tile.cc:317-391  exact
domain_order   DomainStats::schedule, ooc/ooc_domain_stats.cc:60-111 ties
vbuf           VBuf::update/correct, ooc/ooc_vbuf.cc:41-112          exact
hdr_add        HdrImage::add (double scale), display/image.h:99-109 bit-exact
ppm            HdrImage::writePpm, display/image.h:183-204         bytes (*)
domain_list    DomainList::push/sort, render/rays.h:57-93           exact
mesh           TriMeshBuffer::computeNormals/updateIntersection,    bit-exact
               render/trimesh_buffer.cc:267-360
load_any_once  LoadAnyOnceSched::scheduleImage,                     exact
               baseline/baseline_schedulers.cc:43-62
============== ==================================================== =========

(*) ppm holds the product's writer (spray_gb300.image), not the oracle, to the
reference's bytes; NaN is included (the reference writes 0 on x86).

"cos/sin": the reference calls libm's cosf/sinf through glm; the oracle (and
the CUDA path, which equals the oracle bit for bit) uses its own Cody-Waite +
Taylor sinCos.  The disk point then differs by at most 2^-23 and everything
downstream of it is bit-exact wherever the disk point agrees.  "pow": glm::pow
is powf; the oracle raises to the integral shininess by binary
exponentiation (relative difference below 1e-5).  "ties": the reference
orders equal scores with an unstable std::sort, the oracle by domain id; the
score sequence of the schedule must agree.
"""
from __future__ import annotations

import base64
import ctypes as C
import os
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
# the reference source tree these helpers read (oracle/build_ref.sh uses the same variable)
REFERENCE_SOURCES = Path(os.environ.get("SPRAY_REFERENCE_DIR", "/root/reference"))
REF_DIR = ROOT / "oracle" / "_ref"
FIXTURE = Path(__file__).resolve().parent / "reference_vectors.json"
LIST_SIZE = 16  # SPRAY_RAY_DOMAIN_LIST_SIZE in the reference's CMake defaults

P = C.c_void_p
I64 = C.c_int64

# tolerances of the groups that are not bit-exact (see the module docstring)
DISK_ABS = 2.0 ** -23
# A disk point off by e <= 2^-23 moves z = sqrt(1 - x^2 - y^2) by at most
# sqrt(4 e) at the rim (z -> 0) and by about e * r / z elsewhere; wi is a
# rotation of (x, y, z) and pdf = z / pi.
COSINE_RIM_ABS = (4 * DISK_ABS) ** 0.5
COSINE_ABS = 2e-6      # where z > 0.1 (r / z < 10)
BLINN_REL = 1e-5

GROUPS = ["rng", "slab", "camera", "disk", "local_to_world", "cosine", "diffuse_light", "point_light",
          "blinn_phong", "reflect", "fr_dielectric", "refract", "unpack", "lru", "tiles", "domain_order",
          "vbuf", "hdr_add", "ppm", "domain_list", "mesh", "load_any_once"]
VBUF_SAMPLES, HISTORY = 8, 4  # SPRAY_SPECU_HISTORY_SIZE in the reference's CMake defaults
HDR_W, HDR_H = 13, 7


def _p(a):
    return a.ctypes.data_as(P)


# ------------------------------------------------------------------ encoding
def encode(a: np.ndarray) -> dict:
    a = np.ascontiguousarray(a)
    return {"dtype": a.dtype.str, "shape": list(a.shape), "b64": base64.b64encode(a.tobytes()).decode()}


def decode(d: dict) -> np.ndarray:
    return np.frombuffer(base64.b64decode(d["b64"]), np.dtype(d["dtype"])).reshape(d["shape"]).copy()


# ------------------------------------------------------------------ inputs
def _unit(rng, n):
    v = rng.normal(size=(n, 3))
    return (v / np.linalg.norm(v, axis=1, keepdims=True)).astype(np.float32)


def make_cases(seed: int = 2024, scale: int = 1) -> dict:
    """Seeded inputs per group; ``scale`` multiplies the random part."""
    rng = np.random.default_rng(seed)
    f32 = np.float32
    c = {}

    seeds = [0, 1, -1, 2 ** 31 - 1, -(2 ** 31), 7, 1023, 123456]
    seeds += [p * (l + 1) for p in (0, 5, 1919, 2073599) for l in range(8)]  # AO: pixel * (l + 1)
    seeds += [s * d for s in (3, 4095, 2 ** 20 + 7) for d in range(1, 6)]     # bounces: sample * depth
    seeds += rng.integers(-(2 ** 31), 2 ** 31, 40 * scale).tolist()
    c["rng"] = {"seed": np.array([np.int64(s) for s in seeds], np.int64).astype(np.int32)}

    # slab: edge cases first (zero and -0 direction components, origin on a
    # plane, origin inside, degenerate direction, flat boxes), then random
    inf = np.inf
    edge = [
        ([0, 0, 0, 1, 1, 1], [0.5, 0.5, -1], [0, 0, 1]),
        ([0, 0, 0, 1, 1, 1], [0.5, 0.5, -1], [-0.0, 0, 1]),
        ([0, 0, 0, 1, 1, 1], [0.5, 0.5, -1], [0.0, -0.0, 1]),
        ([0, 0, 0, 1, 1, 1], [0, 0.5, -1], [0, 0, 1]),
        ([0, 0, 0, 1, 1, 1], [1, 1, -1], [0, 0, 1]),
        ([0, 0, 0, 1, 1, 1], [0.5, 0.5, 0.5], [1, 2, 3]),
        ([0, 0, 0, 1, 1, 1], [0.5, 0.5, 0.5], [0, 0, 0]),
        ([0, 0, 0, 1, 1, 1], [2, 2, 2], [1, 1, 1]),
        ([0, 0, 0, 1, 1, 1], [-1, -1, -1], [1, 1, 1]),
        ([0, 0, 0, 1, 0, 1], [0.5, -1, 0.5], [0, 1, 0]),
        ([0, 0, 0, 0, 0, 0], [-1, 0, 0], [1, 0, 0]),
        ([-3, -2, -1, 3, 2, 1], [10, 0, 0], [-1, 1e-30, 0]),
        ([-3, -2, -1, 3, 2, 1], [0, 0, 0], [1e-38, 1, 0]),
    ]
    nr = 200 * scale
    lo = rng.uniform(-4, 4, (nr, 3))
    hi = lo + rng.uniform(0, 3, (nr, 3)) * (rng.random((nr, 1)) > 0.05)
    org = rng.uniform(-8, 8, (nr, 3))
    tgt = rng.uniform(lo, np.maximum(hi, lo + 1e-3))
    d = tgt - org + rng.normal(0, 0.5, (nr, 3)) * (rng.random((nr, 1)) < 0.5)
    d[rng.random(nr) < 0.1, rng.integers(0, 3)] = 0.0
    box = np.concatenate([np.array([e[0] for e in edge]), np.concatenate([lo, hi], 1)]).astype(f32)
    c["slab"] = {
        "box": box,
        "org": np.concatenate([np.array([e[1] for e in edge]), org]).astype(f32),
        "dir": np.concatenate([np.array([e[2] for e in edge]), d]).astype(f32),
        "t": np.stack([np.where(rng.random(len(box)) < 0.8, f32(0.001), f32(0.0)),
                       np.where(rng.random(len(box)) < 0.8, f32(inf), rng.uniform(0.5, 12, len(box)).astype(f32))],
                      1).astype(f32),
    }

    # camera: the workload resolutions and odd ones; integer pixels and jitter
    views = [(1920, 1080, 60.0), (1024, 1024, 90.0), (2048, 2048, 60.0), (64, 48, 45.0), (7, 5, 30.0),
             (256, 256, 60.0)]
    cams, xy = [], []
    for (w, h, fov) in views:
        pos = rng.uniform(-12, 12, 3)
        look = rng.uniform(-1, 1, 3)
        m = 32 * scale
        odd = np.arange(m) % 2  # odd entries jittered like multi-sample eye rays
        p = np.stack([rng.integers(0, w, m) + rng.random(m) * odd, rng.integers(0, h, m) + rng.random(m) * odd], 1)
        p[:4] = [[0, 0], [w - 1, h - 1], [w / 2, h / 2], [0, h - 1]]
        cams.append(np.concatenate([pos, look, [0, 1, 0], [fov, w, h]]))
        xy.append(p)
    c["camera"] = {"view": np.array(cams, f32), "xy": np.array(xy, f32)}

    # disk: the region boundaries (sx = 0, sy = 0, sx = +-sy) and the corners
    g = np.array([0.0, 0.25, 0.5, 0.75, 1.0], f32)
    uu = np.stack(np.meshgrid(g, g), -1).reshape(-1, 2)
    t = rng.random(48 * scale).astype(f32)
    uu = np.concatenate([uu, np.stack([t, t], 1), np.stack([t, f32(1) - t], 1),
                         rng.random((160 * scale, 2)).astype(f32)]).astype(f32)
    c["disk"] = {"u": uu}

    axes = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0], [0, 0, -1],
                     [0.6, 0.8, 0], [0, 0.6, 0.8], [0.8, 0, 0.6]], f32)
    nn = np.concatenate([axes, _unit(rng, 96 * scale)])
    c["local_to_world"] = {"n": nn, "v": _unit(rng, len(nn))}

    cu = np.concatenate([uu[:40], rng.random((200 * scale, 2)).astype(f32)])
    c["cosine"] = {"u": cu, "n": np.concatenate([np.repeat(axes, 5, 0)[:len(cu)], _unit(rng, len(cu))])[:len(cu)]}

    dseeds = np.array([p * (l + 1) for p in rng.integers(0, 2 ** 21, 12 * scale) for l in range(8)], np.int64)
    c["diffuse_light"] = {"seed": dseeds.astype(np.int32), "n": _unit(rng, len(dseeds))}

    npt = 64 * scale
    c["point_light"] = {"light": rng.uniform(-100, 1000, (npt, 3)).astype(f32),
                        "p": rng.uniform(-2, 2, (npt, 3)).astype(f32)}

    nb = 96 * scale
    shin = np.concatenate([[1, 2, 3, 8, 16, 64, 127, 200], rng.integers(1, 129, nb - 8)]).astype(f32)
    c["blinn_phong"] = {"args": np.concatenate([
        rng.random((nb, 1)), rng.random((nb, 3)), rng.random((nb, 3)), shin[:, None],
        rng.random((nb, 3)) * 3, _unit(rng, nb), _unit(rng, nb), _unit(rng, nb)], 1).astype(f32)}

    nrf = 96 * scale
    c["reflect"] = {"wo": _unit(rng, nrf), "n": _unit(rng, nrf)}

    nd = 160 * scale
    cos_i = np.concatenate([[1, -1, 0, 1e-4, -1e-4, 0.5, -0.5, 0.2], rng.uniform(-1, 1, nd - 8)])
    eta = np.concatenate([np.array([[1, 1.5], [1.5, 1], [1, 1], [2.4, 1], [1, 2.4], [1.33, 1], [1, 1.33],
                                    [1.5, 1]]), rng.choice([1.0, 1.33, 1.5, 2.4], (nd - 8, 2))])
    c["fr_dielectric"] = {"args": np.concatenate([cos_i[:, None], eta, _unit(rng, nd), _unit(rng, nd)],
                                                 1).astype(f32)}

    grey = (np.arange(256, dtype=np.uint32) * 0x010101).astype(np.uint32)
    c["unpack"] = {"color": np.concatenate([grey, rng.integers(0, 2 ** 32, 64 * scale, dtype=np.uint64)
                                            .astype(np.uint32)])}

    traces = []
    for (ndom, cap) in [(8, 1), (8, 3), (8, 8), (8, -1), (64, 16), (512, 57)]:
        ids = rng.integers(0, ndom, 150 * scale)
        ids[40:60] = ids[0]  # repeated hits
        traces.append((ndom, cap, ids))
    c["lru"] = {"config": np.array([(a, b) for a, b, _ in traces], np.int32),
                "ids": np.array([t for _, _, t in traces], np.int32)}

    # tiles: (w, h, spp, ranks, rank, max samples per rank), every tile height > 0
    c["tiles"] = {"config": np.array([
        (1024, 1024, 1, 1, 0, 1 << 20), (1920, 1080, 16, 1, 0, 1 << 20), (2048, 2048, 8, 1, 0, 1 << 20),
        (400, 400, 4, 1, 0, 1 << 20), (100, 10, 1, 3, 0, 1 << 20), (100, 10, 1, 3, 1, 1 << 20),
        (100, 10, 1, 3, 2, 1 << 20), (1920, 1080, 16, 3, 2, 1 << 20), (1000, 7, 4, 2, 1, 5000),
        (640, 480, 64, 5, 4, 100000), (3, 1000, 1, 8, 7, 17), (7, 5, 2, 1, 0, 30)], np.int64)}

    orders = []
    for (ndom, hi_, zero) in [(64, 50, 0.0), (64, 3, 0.5), (128, 20, 0.7), (8, 2, 0.3)]:
        cnt = rng.integers(0, hi_, (ndom, LIST_SIZE)).astype(np.int64)
        cnt[rng.random(ndom) < zero] = 0
        orders.append(cnt)
    c["domain_order"] = {"counts": np.concatenate([o.reshape(-1) for o in orders]),
                         "ndomains": np.array([len(o) for o in orders], np.int32)}

    # speculation history: few samples and few distinct t values, so that
    # equal, smaller and larger histories all occur
    nv_ = 600 * scale
    tv = np.array([0.5, 1, 2, 3, np.inf], f32)
    c["vbuf"] = {"op": (rng.random(nv_) < 0.3).astype(np.uint8),
                 "samid": rng.integers(0, VBUF_SAMPLES, nv_).astype(np.int32),
                 "depth": rng.integers(0, HISTORY, nv_).astype(np.int32),
                 "hist": tv[rng.integers(0, len(tv), (nv_, HISTORY))],
                 "t": np.array([0.25, 0.5, 1, 1.5, 2, 3], f32)[rng.integers(0, 6, nv_)]}

    # retire: radiance of every magnitude added into few pixels, at the 1/spp
    # scales of the workloads (and 1/7, inexact in binary)
    nh = 1500 * scale
    c["hdr_add"] = {"pixid": rng.integers(0, HDR_W * HDR_H, nh).astype(np.int32),
                    "rgb": (rng.random((nh, 3)) * rng.choice([1e-4, 1, 1e3, 1e6], (nh, 1))).astype(f32),
                    "scale": np.array([1.0, 1 / 8, 1 / 16, 1 / 7], np.float64)}

    # PPM: truncation boundaries k / 1023, clamping, infinities and NaN
    img = rng.uniform(-0.2, 1.3, (HDR_H, HDR_W, 4)).astype(f32)
    k = rng.integers(0, 1024, 24)
    edge = np.concatenate([k / 1023.0, np.nextafter((k / 1023.0).astype(f32), f32(0)), [0, -0.0, 1, 1.0000001,
                           np.inf, -np.inf, np.nan, 1e-30, 0.99999994]]).astype(f32)
    img.reshape(-1)[:len(edge)] = edge
    c["ppm"] = {"rgba": img}

    # domain lists of up to 22 hits (the C3 list size) pushed in any order:
    # distances quantised so that ties are common, negative entries (origin
    # inside a box), +0 and -0; ids unique per list
    nl = 120 * scale
    sizes = rng.integers(1, 23, nl)
    ids, ts = [], []
    for n in sizes:
        ids.append(rng.permutation(512)[:n].astype(np.int32))
        t = np.round(rng.uniform(-2, 6, n) * 4) / 4
        t[rng.random(n) < 0.1] = 0.0
        t = t.astype(f32)
        t[rng.random(n) < 0.05] = f32(-0.0)
        ts.append(t)
    c["domain_list"] = {"size": sizes.astype(np.int32), "ids": np.concatenate(ids), "ts": np.concatenate(ts)}

    # a mesh with per-vertex colours (every byte value occurs), queried at
    # its triangles' corners, edges and random barycentrics
    mv, mf = _sphere(14, 24)
    ncol = len(mv)
    col = rng.integers(0, 256, (ncol, 3)).astype(np.uint32)
    col[:3] = [[0, 0, 0], [255, 255, 255], [255, 0, 128]]
    nq = 1000 * scale
    prim = rng.integers(0, len(mf), nq).astype(np.uint32)
    uu = rng.random(nq).astype(f32)
    vv = (rng.random(nq) * (1 - uu)).astype(f32)
    corners = np.array([[0, 0], [1, 0], [0, 1], [0.5, 0.5]], f32)
    k = len(corners) * len(mf)
    prim = np.concatenate([np.repeat(np.arange(len(mf), dtype=np.uint32), len(corners)), prim])
    uu = np.concatenate([np.tile(corners[:, 0], len(mf)), uu])
    vv = np.concatenate([np.tile(corners[:, 1], len(mf)), vv])
    c["mesh"] = {"vertices": mv, "faces": mf, "colors": (col[:, 0] << 16) | (col[:, 1] << 8) | col[:, 2],
                 "prim": prim, "u": uu, "v": vv, "corner_queries": np.array([k], np.int64)}

    # one round's per-domain queue counts: 1 to 600 domains (std::sort's
    # insertion-sort and introsort ranges), few distinct values so that the
    # largest count is usually tied, and all-zero rounds (the frame is done)
    nr = 300 * scale
    nds = rng.integers(1, 601, nr)
    nds[:4] = [1, 16, 17, 512]
    counts = []
    for k, n in enumerate(nds):
        hi = int(rng.integers(1, 5)) if k % 3 else int(rng.integers(1, 10_000))
        cnt = rng.integers(0, hi, n).astype(np.int64)
        if k % 17 == 5:
            cnt[:] = 0
        counts.append(cnt)
    c["load_any_once"] = {"ndomains": nds.astype(np.int32), "counts": np.concatenate(counts)}
    return c


# ------------------------------------------------------------------ reference
def load_reference():
    """(libref_path, libref_rng) as ctypes libraries, or None where
    oracle/build_ref.sh has not built them (reference sources absent)."""
    lp, lr = REF_DIR / "libref_path.so", REF_DIR / "libref_rng.so"
    if not (lp.exists() and lr.exists()):
        return None
    R, G = C.CDLL(str(lp)), C.CDLL(str(lr))
    G.ref_rng.argtypes = [C.c_int32, C.c_int32, P]
    R.ref_slab.argtypes = [P, P, P, C.c_float, C.c_float, P, P]
    R.ref_camera_rays.argtypes = [P, P, P, C.c_float, C.c_int32, C.c_int32, I64, P, P]
    for name in ("disk", "unpack_color", "blinn_phong"):
        getattr(R, "ref_" + name).argtypes = [I64, P, P]
    for name in ("local_to_world", "reflect", "fr_dielectric", "refract", "point_light"):
        getattr(R, "ref_" + name).argtypes = [I64, P, P, P]
    for name in ("cosine_sample", "diffuse_light"):
        getattr(R, "ref_" + name).argtypes = [I64, P, P, P, P]
    R.ref_lru_trace.argtypes = [C.c_int32, C.c_int32, I64, P, P]
    R.ref_tiles.argtypes = [I64, I64, I64, I64, C.c_int32, I64, P, C.c_int32]
    R.ref_tiles.restype = C.c_int32
    R.ref_domain_order.argtypes = [C.c_int32, P, P]
    return R, G


def _tile_height(w, h, spp, nr, rk, mx):
    """Tile height ImageScheduleTileList::init would compute (None for an
    empty stripe), so that no case reaches its division by zero."""
    sw = max(int(w) // int(nr), 1)
    x = int(rk) * sw
    if x >= w:
        return None
    vw = w - x if (x + sw > w or rk == nr - 1) else sw
    ntiles = (vw * h * spp + mx - 1) // mx
    return int(h) // int(ntiles)


def _vec_call(fn, n, *arrays, outs):
    res = [np.zeros(s, dt) for s, dt in outs]
    fn(n, *[_p(np.ascontiguousarray(a)) for a in arrays], *[_p(r) for r in res])
    return res


def reference_outputs(cases: dict, libs) -> dict:
    R, G = libs
    f32, out = np.float32, {}
    s = cases["rng"]["seed"]
    r = np.zeros((len(s), 16), f32)
    for i, sd in enumerate(s):
        G.ref_rng(int(sd), 16, _p(r[i]))
    out["rng"] = {"floats": r}

    b = cases["slab"]
    n = len(b["box"])
    hit, tt = np.zeros(n, np.uint8), np.zeros((n, 2), f32)
    for i in range(n):
        lo, hi = np.zeros(1, f32), np.zeros(1, f32)
        hit[i] = R.ref_slab(_p(b["box"][i]), _p(b["org"][i]), _p(b["dir"][i]), b["t"][i, 0], b["t"][i, 1],
                            _p(lo), _p(hi))
        tt[i] = lo[0], hi[0]
    out["slab"] = {"hit": hit, "tmin_tmax": tt}

    cm = cases["camera"]
    dirs = np.zeros(cm["xy"].shape[:2] + (3,), f32)
    for k, v in enumerate(cm["view"]):
        R.ref_camera_rays(_p(v[0:3].copy()), _p(v[3:6].copy()), _p(v[6:9].copy()), v[9], int(v[10]), int(v[11]),
                          cm["xy"].shape[1], _p(cm["xy"][k]), _p(dirs[k]))
    out["camera"] = {"dir": dirs}

    u = cases["disk"]["u"]
    out["disk"] = {"d": _vec_call(R.ref_disk, len(u), u, outs=[((len(u), 2), f32)])[0]}

    lw = cases["local_to_world"]
    out["local_to_world"] = {"out": _vec_call(R.ref_local_to_world, len(lw["n"]), lw["n"], lw["v"],
                                              outs=[((len(lw["n"]), 3), f32)])[0]}

    cs = cases["cosine"]
    m = len(cs["u"])
    wi, pdf = _vec_call(R.ref_cosine_sample, m, cs["u"], cs["n"], outs=[((m, 3), f32), (m, f32)])
    dd = _vec_call(R.ref_disk, m, cs["u"], outs=[((m, 2), f32)])[0]
    out["cosine"] = {"wi": wi, "pdf": pdf, "disk": dd}

    dl = cases["diffuse_light"]
    m = len(dl["seed"])
    wi, pdf = _vec_call(R.ref_diffuse_light, m, dl["seed"], dl["n"], outs=[((m, 3), f32), (m, f32)])
    uu = np.zeros((m, 2), f32)
    for i, sd in enumerate(dl["seed"]):
        G.ref_rng(int(sd), 2, _p(uu[i]))
    dd = _vec_call(R.ref_disk, m, uu, outs=[((m, 2), f32)])[0]
    out["diffuse_light"] = {"wi": wi, "pdf": pdf, "disk": dd}

    pl = cases["point_light"]
    out["point_light"] = {"wi": _vec_call(R.ref_point_light, len(pl["p"]), pl["light"], pl["p"],
                                          outs=[((len(pl["p"]), 3), f32)])[0]}

    a = cases["blinn_phong"]["args"]
    out["blinn_phong"] = {"out": _vec_call(R.ref_blinn_phong, len(a), a, outs=[((len(a), 3), f32)])[0]}

    rf = cases["reflect"]
    out["reflect"] = {"out": _vec_call(R.ref_reflect, len(rf["wo"]), rf["wo"], rf["n"],
                                       outs=[((len(rf["wo"]), 3), f32)])[0]}

    a = cases["fr_dielectric"]["args"]
    fr, wt = _vec_call(R.ref_fr_dielectric, len(a), a, outs=[(len(a), f32), ((len(a), 3), f32)])
    ok, wt2 = _vec_call(R.ref_refract, len(a), a, outs=[(len(a), np.uint8), ((len(a), 3), f32)])
    out["fr_dielectric"] = {"fr": fr, "wt": wt}
    out["refract"] = {"ok": ok, "wt": wt2}

    col = cases["unpack"]["color"]
    out["unpack"] = {"rgb": _vec_call(R.ref_unpack_color, len(col), col, outs=[((len(col), 3), f32)])[0]}

    lr = cases["lru"]
    hits = np.zeros(lr["ids"].shape, np.uint8)
    for k, (ndom, cap) in enumerate(lr["config"]):
        R.ref_lru_trace(int(ndom), int(cap), lr["ids"].shape[1], _p(np.ascontiguousarray(lr["ids"][k])), _p(hits[k]))
    out["lru"] = {"hits": hits}

    tiles = []
    for (w, h, spp, nr, rk, mx) in cases["tiles"]["config"]:
        if _tile_height(w, h, spp, nr, rk, mx) == 0:
            raise ValueError("tile height 0: the reference divides by it")
        buf = np.zeros(4 * 4096, np.int32)
        k = R.ref_tiles(int(w), int(h), int(spp), int(nr), int(rk), int(mx), _p(buf), 4096)
        tiles.append(buf[:4 * k].reshape(-1, 4))
    out["tiles"] = {"count": np.array([len(t) for t in tiles], np.int32),
                    "tiles": np.concatenate(tiles).astype(np.int32)}

    do = cases["domain_order"]
    orders, off = [], 0
    for ndom in do["ndomains"]:
        cnt = np.ascontiguousarray(do["counts"][off:off + ndom * LIST_SIZE])
        od = np.zeros(ndom, np.int32)
        R.ref_domain_order(int(ndom), _p(cnt), _p(od))
        orders.append(od)
        off += ndom * LIST_SIZE
    out["domain_order"] = {"order": np.concatenate(orders)}

    vb = cases["vbuf"]
    R.ref_vbuf_trace.argtypes = [C.c_int32, I64, P, P, P, P, P, P]
    hist = np.array(vb["hist"], f32, copy=True)
    res = np.zeros(len(vb["op"]), np.uint8)
    R.ref_vbuf_trace(VBUF_SAMPLES, len(vb["op"]), _p(vb["op"]), _p(vb["samid"]), _p(vb["depth"]), _p(hist),
                     _p(vb["t"]), _p(res))
    out["vbuf"] = {"result": res, "hist": hist}

    R.ref_hdr_add.argtypes = [C.c_int32, C.c_int32, I64, P, P, C.c_double, P]
    R.ref_write_ppm.argtypes = [C.c_int32, C.c_int32, P, C.c_char_p]
    hd = cases["hdr_add"]
    imgs = []
    for sc_ in hd["scale"]:
        buf = np.zeros((HDR_W * HDR_H, 4), f32)
        R.ref_hdr_add(HDR_W, HDR_H, len(hd["pixid"]), _p(hd["pixid"]), _p(hd["rgb"]), float(sc_), _p(buf))
        imgs.append(buf)
    out["hdr_add"] = {"rgba": np.stack(imgs)}

    import tempfile
    img = np.ascontiguousarray(cases["ppm"]["rgba"])
    with tempfile.TemporaryDirectory() as tmp:
        path = Path(tmp) / "ref.ppm"
        R.ref_write_ppm(img.shape[1], img.shape[0], _p(img), str(path).encode())
        out["ppm"] = {"bytes": np.frombuffer(path.read_bytes(), np.uint8).copy()}

    R.ref_domain_list_sort.argtypes = [C.c_int32, P, P, P, P]
    dl = cases["domain_list"]
    oi, ot = np.zeros_like(dl["ids"]), np.zeros_like(dl["ts"])
    off = 0
    for n in dl["size"]:
        R.ref_domain_list_sort(int(n), _p(dl["ids"][off:]), _p(dl["ts"][off:]), _p(oi[off:]), _p(ot[off:]))
        off += int(n)
    out["domain_list"] = {"ids": oi, "ts": ot}

    R.ref_load_any_once.argtypes = [C.c_int32, P, P, P]
    la = cases["load_any_once"]
    ids = np.zeros(len(la["ndomains"]), np.int32)
    done = np.zeros(len(la["ndomains"]), np.uint8)
    off = 0
    for k, n in enumerate(la["ndomains"]):
        R.ref_load_any_once(int(n), _p(la["counts"][off:]), _p(ids[k:]), _p(done[k:]))
        off += int(n)
    out["load_any_once"] = {"id": ids, "done": done}

    R.ref_mesh_attributes.argtypes = [C.c_char_p, I64, I64, I64, P, P, P, P, P]
    ms = cases["mesh"]
    col = np.zeros(len(ms["prim"]), np.uint32)
    ns = np.zeros((len(ms["prim"]), 3), f32)
    with tempfile.TemporaryDirectory() as tmp:
        ply = Path(tmp) / "mesh.ply"
        ply.write_bytes(_ply_binary(ms["vertices"], ms["faces"], ms["colors"]))
        R.ref_mesh_attributes(str(ply).encode(), len(ms["vertices"]), len(ms["faces"]), len(ms["prim"]),
                              _p(ms["prim"]), _p(ms["u"]), _p(ms["v"]), _p(col), _p(ns))
    out["mesh"] = {"color": col, "ns": ns}
    return out


# ------------------------------------------------------------------ oracle
def oracle_outputs(cases: dict) -> dict:
    from oracle import oracle as O
    from spray_gb300 import scenes

    f32, out = np.float32, {}
    out["rng"] = {"floats": np.stack([O.rng_floats(int(s), 16) for s in cases["rng"]["seed"]])}

    b = cases["slab"]
    res = [O.slab(b["box"][i], b["org"][i], b["dir"][i], b["t"][i, 0], b["t"][i, 1]) for i in range(len(b["box"]))]
    out["slab"] = {"hit": np.array([r[0] for r in res], np.uint8),
                   "tmin_tmax": np.array([(r[1], r[2]) for r in res], f32)}

    cm = cases["camera"]
    out["camera"] = {"dir": np.stack([O.camera_rays(v[0:3], v[3:6], v[6:9], v[9], int(v[10]), int(v[11]), cm["xy"][k])
                                      for k, v in enumerate(cm["view"])])}
    out["disk"] = {"d": O.disk(cases["disk"]["u"])}
    lw = cases["local_to_world"]
    out["local_to_world"] = {"out": O.local_to_world(lw["n"], lw["v"])}

    cs = cases["cosine"]
    wi, pdf = O.cosine_sample(cs["u"], cs["n"])
    out["cosine"] = {"wi": wi, "pdf": pdf, "disk": O.disk(cs["u"])}

    # the hemisphere light draws two floats from RandomSampler_init(seed)
    # (RandomSampler_get2D) and takes a cosine sample around the normal
    dl = cases["diffuse_light"]
    uu = np.stack([O.rng_floats(int(s), 2) for s in dl["seed"]])
    wi, pdf = O.cosine_sample(uu, dl["n"])
    out["diffuse_light"] = {"wi": wi, "pdf": pdf, "disk": O.disk(uu)}

    pl = cases["point_light"]
    out["point_light"] = {"wi": O.point_light(pl["light"], pl["p"])}

    out["blinn_phong"] = {"out": O.blinn_phong(cases["blinn_phong"]["args"])}
    rf = cases["reflect"]
    out["reflect"] = {"out": O.reflect(rf["wo"], rf["n"])}
    fr, wt = O.fr_dielectric(cases["fr_dielectric"]["args"])
    out["fr_dielectric"] = {"fr": fr, "wt": wt}
    ok, wt2 = O.refract(cases["fr_dielectric"]["args"])
    out["refract"] = {"ok": ok, "wt": wt2}
    out["unpack"] = {"rgb": O.unpack_color(cases["unpack"]["color"])}

    lr = cases["lru"]
    out["lru"] = {"hits": np.stack([O.lru_trace(int(nd), int(cap), lr["ids"][k])
                                    for k, (nd, cap) in enumerate(lr["config"])])}

    sc = scenes.wavelet_grid(1, 8)
    tiles = []
    for (w, h, spp, nr, rk, mx) in cases["tiles"]["config"]:
        o = O.Oracle(_config(image_w=int(w), image_h=int(h), pixel_samples=int(spp), num_ranks=int(nr),
                             rank=int(rk), max_samples_per_rank=int(mx)), sc)
        tiles.append(np.asarray(o.tiles(), np.int32).reshape(-1, 4))
    out["tiles"] = {"count": np.array([len(t) for t in tiles], np.int32),
                    "tiles": np.concatenate(tiles).astype(np.int32)}

    do = cases["domain_order"]
    orders, scores, off = [], [], 0
    for ndom in do["ndomains"]:
        cnt = do["counts"][off:off + ndom * LIST_SIZE]
        grid = scenes.wavelet_grid(1, 8)
        grid.domains = grid.domains * int(ndom)
        o = O.Oracle(_config(list_size=LIST_SIZE), grid)
        s, od = o.scores(cnt)
        orders.append(od)
        scores.append(s)
        off += ndom * LIST_SIZE
    out["domain_order"] = {"order": np.concatenate(orders), "score": np.concatenate(scores)}

    vb = cases["vbuf"]
    res, hist = O.vbuf_trace(VBUF_SAMPLES, HISTORY, vb["op"], vb["samid"], vb["depth"], vb["hist"], vb["t"])
    out["vbuf"] = {"result": res, "hist": hist}

    hd = cases["hdr_add"]
    out["hdr_add"] = {"rgba": np.stack([O.hdr_add(np.zeros((HDR_W * HDR_H, 4), f32), hd["pixid"], hd["rgb"],
                                                  float(sc_)) for sc_ in hd["scale"]])}
    from spray_gb300 import image
    out["ppm"] = {"bytes": np.frombuffer(image.ppm_bytes(cases["ppm"]["rgba"]), np.uint8).copy()}
    dl = cases["domain_list"]
    ids, ts, off = [], [], 0
    for n in dl["size"]:
        a, b = O.domain_list_sort(dl["ids"][off:off + n], dl["ts"][off:off + n])
        ids.append(a)
        ts.append(b)
        off += int(n)
    out["domain_list"] = {"ids": np.concatenate(ids), "ts": np.concatenate(ts)}
    ms = cases["mesh"]
    nrm, col, ns = O.mesh_attributes(ms["vertices"], ms["faces"], ms["colors"], ms["prim"], ms["u"], ms["v"])
    out["mesh"] = {"color": col, "ns": ns, "normals": nrm}
    la = cases["load_any_once"]
    ids, done, off = [], [], 0
    for n in la["ndomains"]:
        i, d = O.load_any_once(la["counts"][off:off + n])
        ids.append(i)
        done.append(d)
        off += int(n)
    out["load_any_once"] = {"id": np.array(ids, np.int32), "done": np.array(done, np.uint8)}
    return out


def _config(**kw):
    cfg = dict(image_w=64, image_h=48, ao_mode=1, ao_samples=1, pixel_samples=1, bounces=1, fov=60.0,
               cache_size=-1, max_samples_per_rank=1 << 20, list_size=16, history_size=4, num_ranks=1, rank=0)
    cfg.update(kw)
    return cfg


# ------------------------------------------------------------------ comparison
def _bits(a):
    return np.ascontiguousarray(a).view(np.uint32)


def _same(a, b):
    return np.array_equal(_bits(np.asarray(a, np.float32)), _bits(np.asarray(b, np.float32)))


def compare(group: str, cases: dict, ref: dict, orc: dict) -> None:
    """Asserts the oracle's outputs `orc` against the reference's `ref` for one
    group, by the rule the module docstring gives for it."""
    r, o = ref[group], orc[group]
    if group in ("rng", "camera", "local_to_world", "point_light", "reflect", "unpack"):
        (k,) = [k for k in r]
        assert _same(r[k], o[k]), f"{group}: {np.sum(_bits(r[k]) != _bits(o[k]))} values differ"
    elif group == "slab":
        assert np.array_equal(r["hit"], o["hit"])
        assert _same(r["tmin_tmax"], o["tmin_tmax"])
    elif group == "disk":
        assert np.all(np.abs(r["d"] - o["d"]) <= DISK_ABS), np.abs(r["d"] - o["d"]).max()
    elif group in ("cosine", "diffuse_light"):
        assert np.all(np.abs(r["disk"] - o["disk"]) <= DISK_ABS)
        agree = np.all(_bits(r["disk"]) == _bits(o["disk"]), axis=1)
        assert agree.mean() > 0.5  # most sin/cos values agree; those cases are bit-exact downstream
        assert _same(r["wi"][agree], o["wi"][agree]) and _same(r["pdf"][agree], o["pdf"][agree])
        dw = np.abs(r["wi"] - o["wi"]).max(axis=1)
        dp = np.abs(r["pdf"] - o["pdf"])
        assert np.all(dw <= COSINE_RIM_ABS) and np.all(dp <= COSINE_RIM_ABS)
        inner = r["pdf"] * np.float32(np.pi) > 0.1
        assert np.all(dw[inner] <= COSINE_ABS) and np.all(dp[inner] <= COSINE_ABS)
    elif group == "blinn_phong":
        rel = np.abs(r["out"] - o["out"]) / np.maximum(np.abs(r["out"]), np.float32(1e-30))
        assert np.all(rel <= BLINN_REL), rel.max()
    elif group == "vbuf":
        assert np.array_equal(r["result"], o["result"]) and _same(r["hist"], o["hist"])
        assert 0 < r["result"].mean() < 1  # both outcomes occur
    elif group == "hdr_add":
        assert _same(r["rgba"], o["rgba"])
    elif group == "ppm":
        assert r["bytes"].tobytes() == o["bytes"].tobytes()
    elif group == "fr_dielectric":
        assert _same(r["fr"], o["fr"]) and _same(r["wt"], o["wt"])
    elif group == "refract":
        assert np.array_equal(r["ok"], o["ok"]) and _same(r["wt"], o["wt"])
    elif group == "lru":
        assert np.array_equal(r["hits"], o["hits"])
    elif group == "domain_list":
        assert np.array_equal(r["ids"], o["ids"]) and _same(r["ts"], o["ts"])
    elif group == "load_any_once":
        # the same domain on ties too: both sort with std::sort over ids
        # ascending, by count descending
        assert np.array_equal(r["id"], o["id"]) and np.array_equal(r["done"], o["done"])
        assert 0 < r["done"].mean() < 1
    elif group == "mesh":
        assert np.array_equal(r["color"], o["color"]), int(np.sum(r["color"] != o["color"]))
        assert _same(r["ns"], o["ns"]), int(np.sum(np.any(_bits(r["ns"]) != _bits(o["ns"]), 1)))
        # the reference's vertex normals, read at the triangles' corners
        # (w, u, v = 1, 0, 0 / 0, 1, 0 / 0, 0, 1), equal the oracle's
        ms = cases["mesh"]
        k = int(ms["corner_queries"][0])
        nc = 4
        f = ms["faces"]
        for corner, vi in ((0, 0), (1, 1), (2, 2)):
            got = r["ns"][:k].reshape(-1, nc, 3)[:, corner]
            want = o["normals"][f[:, vi]]
            assert np.array_equal(got, want)  # values (+0 and -0 equal)
    elif group == "tiles":
        assert np.array_equal(r["count"], o["count"]) and np.array_equal(r["tiles"], o["tiles"])
    elif group == "domain_order":
        off = 0
        for ndom in cases["domain_order"]["ndomains"]:
            ro, oo = r["order"][off:off + ndom], o["order"][off:off + ndom]
            sc = o["score"][off:off + ndom]
            assert np.array_equal(np.sort(ro), np.arange(ndom))
            # the same score at every position of the schedule; equal scores
            # in any order (unstable sort in the reference, by id in the oracle)
            assert np.array_equal(sc[ro], sc[oo])
            assert np.all(np.diff(sc[oo]) <= 0)
            # no ties: the same order
            if len(np.unique(sc)) == ndom:
                assert np.array_equal(ro, oo)
            off += ndom
    else:
        raise KeyError(group)


# ------------------------------------------------------------------ scene files
# SceneLoader::load (io/scene_loader.cc:311-358), PlyLoader::load
# (io/ply_loader.cc:179-204) and the vertex transform of TriMeshBuffer::load
# (render/trimesh_buffer.cc:141-153) against the product's scene loader
# (spray_scene_load): world-space vertices and world bounds bit-exact, faces,
# colours, materials and light radiance equal.
SCENE_FIXTURE = Path(__file__).resolve().parent / "reference_scene.json"
_XFORMS = ["", "translate 1.5 -2.25 3", "scale 2 0.5 3|rotate x 30|translate 0.1 0.2 0.3",
           "rotate y 47.5|translate -4 5 6.125", "rotate z 90", "rotate x 13|rotate y -71|rotate z 200|"
           "scale 1.1 1.2 1.3|translate 7 8 9", "translate 3 3 3|rotate y 33", "scale -1 1 1|rotate x -90"]
_MTLS = ["", "mtl diffuse 0.5 0.25 0.75", "mtl mirror 1 1 1", "mtl glass 1 1.5", "mtl transmission 1 1.33"]


def _sphere(nt=10, nph=20, r=1.3, c=(0.2, -0.1, 0.05)):
    th = np.linspace(0.15, np.pi - 0.15, nt)
    ph = np.linspace(0, 2 * np.pi, nph, endpoint=False)
    T, PH = np.meshgrid(th, ph, indexing="ij")
    v = np.stack([np.sin(T) * np.cos(PH), np.cos(T), np.sin(T) * np.sin(PH)], -1).reshape(-1, 3) * r + c
    f = []
    for i in range(nt - 1):
        for j in range(nph):
            a, b = i * nph + j, i * nph + (j + 1) % nph
            f += [(a, b, a + nph), (b, b + nph, a + nph)]
    return v.astype(np.float32), np.array(f, np.uint32)


def _ply_binary(v, f, col):
    head = ("ply\nformat binary_little_endian 1.0\nelement vertex %d\nproperty float x\nproperty float y\n"
            "property float z\nproperty uchar red\nproperty uchar green\nproperty uchar blue\n"
            "element face %d\nproperty list uchar int vertex_indices\nend_header\n" % (len(v), len(f))).encode()
    vr = np.zeros(len(v), [("p", "<f4", 3), ("c", "u1", 3)])
    vr["p"] = v
    vr["c"] = np.stack([(col >> 16) & 255, (col >> 8) & 255, col & 255], 1)
    fr = np.zeros(len(f), [("n", "u1"), ("i", "<i4", 3)])
    fr["n"] = 3
    fr["i"] = f
    return head + vr.tobytes() + fr.tobytes()


def _ply_ascii(v, f, col=None):
    lines = ["ply", "format ascii 1.0", f"element vertex {len(v)}", "property float x", "property float y",
             "property float z"]
    if col is not None:
        lines += ["property uchar red", "property uchar green", "property uchar blue"]
    lines += [f"element face {len(f)}", "property list uchar int vertex_indices", "end_header"]
    for k, p in enumerate(v):
        s = " ".join(repr(float(x)) for x in p)
        if col is not None:
            s += " %d %d %d" % ((col[k] >> 16) & 255, (col[k] >> 8) & 255, col[k] & 255)
        lines.append(s)
    lines += ["3 %d %d %d" % tuple(t) for t in f]
    return ("\n".join(lines) + "\n").encode()


def make_scene_files(seed: int = 5) -> dict:
    """A .spray scene (every material kind, translate/scale/rotate chains,
    point and hemisphere lights) and the PLY files it names: binary
    little-endian with colour, ASCII with and without colour."""
    rng = np.random.default_rng(seed)
    v, f = _sphere()
    col = rng.integers(0, 1 << 24, len(v)).astype(np.uint32)
    jitter = (v + rng.normal(0, 0.01, v.shape)).astype(np.float32)
    files = {"bin.ply": _ply_binary(v, f, col), "asc.ply": _ply_ascii(jitter, f, col),
             "plain.ply": _ply_ascii(v[:40], f[(f < 40).all(1)])}
    plys = ["bin.ply", "asc.ply", "plain.ply"]
    txt = ["# scene for the loader comparison", "light point 1 2 3 0.5 0.25 0.125", "light diffuse .1 .2 .3", ""]
    for i, x in enumerate(_XFORMS):
        name = plys[i % 3]
        vv = v if name == "bin.ply" else (jitter if name == "asc.ply" else v[:40])
        lo, hi = vv.min(0), vv.max(0)
        txt += ["domain", f"file {name}"] + ([_MTLS[i % 5]] if _MTLS[i % 5] else [])
        txt += ["bound " + " ".join(repr(float(a)) for a in np.concatenate([lo, hi]))]
        txt += [t for t in x.split("|") if t]
        nf = len(f) if name != "plain.ply" else int((f < 40).all(1).sum())
        txt += [f"face {nf}", f"vertex {len(vv)}", ""]
    files["scene.spray"] = ("\n".join(txt) + "\n").encode()
    return files


def write_scene_files(files: dict, where: Path) -> Path:
    for name, data in files.items():
        (where / name).write_bytes(data)
    return where / "scene.spray"


def reference_scene_outputs(spray: Path, libs, ply_dir: Path | None = None) -> dict:
    R, _ = libs
    R.ref_scene_load.argtypes = [C.c_char_p, C.c_char_p, C.c_int32, P, P, P, P, P, C.c_int32, P, P, P]
    R.ref_scene_load.restype = C.c_int32
    R.ref_ply_load.argtypes = [C.c_char_p, I64, I64, P, P, P, P]
    R.ref_ply_load.restype = I64
    R.ref_transform_points.argtypes = [P, I64, P]
    cap, lcap = 4096, 64
    T = np.zeros((cap, 16), np.float32)
    ob, wb = np.zeros((cap, 6), np.float32), np.zeros((cap, 6), np.float32)
    cnt, kind = np.zeros((cap, 2), np.int64), np.zeros(cap, np.int32)
    nl, lk, lr = np.zeros(1, np.int32), np.zeros(lcap, np.int32), np.zeros((lcap, 3), np.float32)
    ply_dir = Path(ply_dir or spray.parent)
    n = R.ref_scene_load(str(spray).encode(), str(ply_dir).encode(), cap, _p(T), _p(ob), _p(wb), _p(cnt), _p(kind), lcap,
                         _p(nl), _p(lk), _p(lr))
    if n < 0:
        raise ValueError("scene larger than the comparison buffers")
    names = [ln.split()[1] for ln in spray.read_text().splitlines() if ln.startswith("file ")]
    verts, faces, cols = [], [], []
    for i in range(n):
        path = str(ply_dir / names[i]).encode()
        nvh, nfh = _ply_counts(ply_dir / names[i])
        vb = np.zeros((nvh + 1, 3), np.float32)
        fb = np.zeros((nfh + 1, 3), np.uint32)
        cb = np.zeros(nvh + 1, np.uint32)
        nf = np.zeros(1, np.int64)
        nv = R.ref_ply_load(path, len(vb), len(fb), _p(vb), _p(fb), _p(cb), _p(nf))
        vb, fb, cb = vb[:nv], fb[:nf[0]], cb[:nv]
        mat = np.ascontiguousarray(T[i])
        if not np.array_equal(mat.reshape(4, 4), np.eye(4, dtype=np.float32)):  # render/scene.inl:151
            R.ref_transform_points(_p(mat), len(vb), _p(vb))
        verts.append(vb)
        faces.append(fb)
        cols.append(cb)
    return {"world_bounds": wb[:n], "object_bounds": ob[:n], "transform": T[:n], "counts": cnt[:n],
            "bsdf_kind": kind[:n], "light_kind": lk[:nl[0]], "light_radiance": lr[:nl[0]],
            "nverts": np.array([len(v) for v in verts], np.int64), "vertices": np.concatenate(verts),
            "faces": np.concatenate(faces), "colors": np.concatenate(cols)}


def _ply_counts(path: Path) -> tuple[int, int]:
    nv = nf = 0
    with open(path, "rb") as fh:
        for line in fh:
            w = line.split()
            if w[:2] == [b"element", b"vertex"]:
                nv = int(w[2])
            elif w[:2] == [b"element", b"face"]:
                nf = int(w[2])
            elif w[:1] == [b"end_header"]:
                break
    return nv, nf


def product_scene_outputs(spray: Path, ply_dir: Path | None = None) -> dict:
    import spray_gb300 as sg
    s = sg.Scene.load(spray, ply_dir or spray.parent)
    return {"world_bounds": np.stack([d.bounds for d in s.domains]),
            "bsdf_kind": np.array([d.bsdf_type for d in s.domains], np.int32),
            "light_kind": np.array([l.type for l in s.lights], np.int32),
            "light_radiance": np.stack([l.radiance for l in s.lights]).astype(np.float32),
            "nverts": np.array([len(d.vertices) for d in s.domains], np.int64),
            "vertices": np.concatenate([d.vertices for d in s.domains]),
            "faces": np.concatenate([d.faces for d in s.domains]),
            "colors": np.concatenate([d.colors for d in s.domains])}


def oracle_scene_outputs(spray: Path, ply_dir: Path | None = None) -> dict:
    """The same fields from the oracle's own reader (oracle/scene_io.py)."""
    from oracle import scene_io
    s = scene_io.load(spray, ply_dir or spray.parent)
    return {"world_bounds": np.stack([d.bounds for d in s.domains]),
            "bsdf_kind": np.array([d.bsdf_type for d in s.domains], np.int32),
            "light_kind": np.array([l.type for l in s.lights], np.int32),
            "light_radiance": np.stack([l.radiance for l in s.lights]).astype(np.float32),
            "nverts": np.array([len(d.vertices) for d in s.domains], np.int64),
            "vertices": np.concatenate([d.vertices for d in s.domains]),
            "faces": np.concatenate([d.faces for d in s.domains]),
            "colors": np.concatenate([d.colors for d in s.domains])}


def compare_scene(ref: dict, prod: dict) -> None:
    assert np.array_equal(ref["nverts"], prod["nverts"])
    assert _same(ref["vertices"], prod["vertices"]), \
        f"{int(np.sum(np.any(_bits(ref['vertices']) != _bits(prod['vertices']), 1)))} vertices differ"
    assert _same(ref["world_bounds"], prod["world_bounds"])
    assert np.array_equal(ref["faces"], prod["faces"]) and np.array_equal(ref["colors"], prod["colors"])
    # no mtl line: the reference leaves the BSDF unset, the product takes the diffuse default
    assert np.array_equal(np.maximum(ref["bsdf_kind"], 0), prod["bsdf_kind"])
    # light kinds: the reference's point / hemisphere, the product's POINT = 0, DIFFUSE = 1
    assert np.array_equal(ref["light_kind"], prod["light_kind"])
    assert _same(ref["light_radiance"], prod["light_radiance"])
