"""ctypes wrapper of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: the CPU restatement of SpRay's speculative
domain-parallel ray-tracing loop that the CUDA path is checked against.  Only
tests, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.
The reference binary cannot be built here (Embree 2.17, MPI and GLFW are
absent) and ships no golden vectors; its hot-path functions that compile alone
(oracle/build_ref.sh) pin the oracle function by function
(tests/test_reference_vectors.py).  Traversal and the loop as a whole stay
unpinned.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "oracle.cpp"
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"

_lib = None


def build(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force or not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime,
                                                               (HERE / "oracle.h").stat().st_mtime):
        tmp = LIB.with_suffix(".tmp.so")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-o", str(tmp), str(SRC)]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout)
        tmp.replace(LIB)
    return LIB


class OrcConfig(C.Structure):
    _fields_ = [
        ("image_w", C.c_int32), ("image_h", C.c_int32), ("ao_mode", C.c_int32),
        ("ao_samples", C.c_int32), ("pixel_samples", C.c_int32), ("bounces", C.c_int32),
        ("ks", C.c_float * 3), ("shininess", C.c_float), ("fov", C.c_float),
        ("cache_size", C.c_int32), ("max_samples_per_rank", C.c_int32), ("list_size", C.c_int32),
        ("history_size", C.c_int32), ("num_ranks", C.c_int32), ("rank", C.c_int32),
        ("ao_light_shadow", C.c_int32), ("ao_max_distance", C.c_float), ("rr_depth", C.c_int32),
    ]


class OrcStats(C.Structure):
    _fields_ = [(k, C.c_int64) for k in ("rays_primary", "rays_shadow", "rays_bounce",
                                         "visits_radiance", "visits_shadow", "domain_loads",
                                         "rounds", "visits_shade", "bvh4_visits", "bvh4_nodes",
                                         "bvh4_tris", "bvh4_mismatches")]

    def asdict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.orc_create.restype = P
        L.orc_create.argtypes = [C.POINTER(OrcConfig), C.c_int32]
        L.orc_destroy.argtypes = [P]
        L.orc_set_domain.argtypes = [P, C.c_int32, P, C.c_int64, P, C.c_int64, P, P, C.c_int32, P]
        L.orc_set_lights.argtypes = [P, C.c_int32, P]
        L.orc_build.argtypes = [P]
        L.orc_set_camera.argtypes = [P, P, P, P, C.c_float]
        L.orc_normals.argtypes = [P, C.c_int32, P]
        L.orc_tiles.argtypes = [P, P, C.c_int32]
        L.orc_tiles.restype = C.c_int32
        L.orc_gen_eyes.argtypes = [P, C.c_int32, C.c_int32, P, P, P, P]
        L.orc_gen_eyes.restype = C.c_int64
        L.orc_schedule.argtypes = [P, C.c_int64, P, P, P, P, P, C.c_int64, P]
        L.orc_schedule.restype = C.c_int64
        L.orc_scores.argtypes = [P, P, P, P]
        L.orc_closest.argtypes = [P, C.c_int64, P, P, P, P, P, P, P, P, P, P]
        L.orc_occluded.argtypes = [P, C.c_int64, P, P, P, P, P]
        L.orc_slots.argtypes = [P]
        L.orc_slots.restype = C.c_int32
        L.orc_shade.argtypes = [P, C.c_int32, C.c_int64] + [P] * 16
        L.orc_rng.argtypes = [C.c_int32, C.c_int32, P]
        L.orc_sincos.argtypes = [C.c_int64, P, P, P]
        L.orc_slab.argtypes = [P, P, P, C.c_float, C.c_float, P, P]
        L.orc_triangle.argtypes = [P, P, P, C.c_float, C.c_float, P, P, P]
        L.orc_lru_trace.argtypes = [C.c_int32, C.c_int32, C.c_int64, P, P, P]
        L.orc_camera_rays.argtypes = [P, P, P, C.c_float, C.c_int32, C.c_int32, C.c_int64, P, P]
        for name in ("disk", "unpack_color", "blinn_phong"):
            getattr(L, "orc_" + name).argtypes = [C.c_int64, P, P]
        for name in ("local_to_world", "reflect", "fr_dielectric", "refract", "point_light"):
            getattr(L, "orc_" + name).argtypes = [C.c_int64, P, P, P]
        L.orc_cosine_sample.argtypes = [C.c_int64, P, P, P, P]
        L.orc_hdr_add.argtypes = [C.c_int64, P, P, C.c_double, P]
        L.orc_vbuf_trace.argtypes = [C.c_int32, C.c_int32, C.c_int64, P, P, P, P, P, P]
        L.orc_domain_list_sort.argtypes = [C.c_int32, P, P, P, P]
        L.orc_mesh_attributes.argtypes = [P, C.c_int64, P, C.c_int64, P, C.c_int64, P, P, P, P, P, P]
        L.orc_render_wavefront.argtypes = [P, P, C.POINTER(OrcStats)]
        L.orc_render_speculative.argtypes = [P, C.c_int32, P, C.POINTER(OrcStats)]
        L.orc_render_baseline.argtypes = [P, P, C.POINTER(OrcStats)]
        L.orc_set_bvh4.argtypes = [P, C.c_int32, P, C.c_int64, P, C.c_int64]
        L.orc_baseline_schedule.argtypes = [P, P, C.c_int64]
        L.orc_baseline_schedule.restype = C.c_int64
        L.orc_load_any_once.argtypes = [C.c_int32, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, np.float32)


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


ORACLE_FIELDS = [f for f, _ in OrcConfig._fields_]


def rng_floats(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().orc_rng(seed, n, _p(out))
    return out


def sincos(x) -> tuple[np.ndarray, np.ndarray]:
    x = _f32(x)
    s = np.zeros_like(x)
    c = np.zeros_like(x)
    lib().orc_sincos(len(x), _p(x), _p(s), _p(c))
    return s, c


def slab(bounds, org, dir, t0=0.001, t1=np.inf):
    tmin = np.zeros(1, np.float32)
    tmax = np.zeros(1, np.float32)
    hit = lib().orc_slab(_p(_f32(bounds)), _p(_f32(org)), _p(_f32(dir)), t0, t1, _p(tmin), _p(tmax))
    return bool(hit), float(tmin[0]), float(tmax[0])


def triangle(org, dir, verts, tnear=0.001, tfar=np.inf):
    t = np.zeros(1, np.float32)
    u = np.zeros(1, np.float32)
    v = np.zeros(1, np.float32)
    hit = lib().orc_triangle(_p(_f32(org)), _p(_f32(dir)), _p(_f32(verts).reshape(9)), tnear, tfar,
                             _p(t), _p(u), _p(v))
    return bool(hit), float(t[0]), float(u[0]), float(v[0])


def lru_trace(num_domains: int, cache_size: int, ids, with_evicted: bool = False):
    """Replays loads through LruCache: hits (1 = hit), and with_evicted also
    the domain each miss displaced (-1: none)."""
    ids = _i32(ids)
    hits = np.zeros(len(ids), np.uint8)
    ev = np.zeros(len(ids), np.int32)
    lib().orc_lru_trace(num_domains, cache_size, len(ids), _p(ids), _p(hits), _p(ev))
    return (hits, ev) if with_evicted else hits


def read_blob_bvh(path) -> tuple[np.ndarray, np.ndarray]:
    """The BVH nodes (32 float32 each) and leaf-ordered triangles (12 float32
    each) of a prepared domain blob (`domain_NNNNN.sdom`: a 128-byte header --
    magic SPRAYDOM, version, BSDF, bounds, BSDF parameters, BVH depth, vertex,
    face and node counts, array offsets -- then 256-byte-aligned arrays)."""
    raw = np.fromfile(path, np.uint8)
    if raw[:8].tobytes() != b"SPRAYDOM":
        raise ValueError(f"{path}: not a prepared domain")
    nv, nf, nn = raw[56:80].view(np.int64)
    off_nodes, off_tris = raw[80:96].view(np.uint64)
    nodes = raw[int(off_nodes):int(off_nodes) + 128 * int(nn)].view(np.float32)
    tris = raw[int(off_tris):int(off_tris) + 48 * int(nf)].view(np.float32)
    return nodes, tris


def load_any_once(counts) -> tuple[int, bool]:
    """LoadAnyOnceSched::scheduleImage on per-domain queue counts: the domain
    processed next, and whether every queue is empty."""
    counts = np.ascontiguousarray(counts, np.int64)
    i, d = C.c_int32(0), C.c_uint8(0)
    if lib().orc_load_any_once(len(counts), _p(counts), C.byref(i), C.byref(d)) != 0:
        raise ValueError("empty domain count array")
    return int(i.value), bool(d.value)


def domain_list_sort(ids, ts) -> tuple[np.ndarray, np.ndarray]:
    """DomainList::sort of (id, tnear) pairs pushed in the given order."""
    ids, ts = _i32(ids), _f32(ts)
    oi, ot = np.zeros_like(ids), np.zeros_like(ts)
    lib().orc_domain_list_sort(len(ids), _p(ids), _p(ts), _p(oi), _p(ot))
    return oi, ot


def mesh_attributes(vertices, faces, colors, prim, u, v):
    """Vertex normals and (colour, shading normal) at n (triangle, u, v)."""
    vv = _f32(vertices).reshape(-1, 3)
    ff = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    cc = np.ascontiguousarray(colors, np.uint32)
    pr = np.ascontiguousarray(prim, np.uint32)
    col = np.zeros(len(pr), np.uint32)
    ns = np.zeros((len(pr), 3), np.float32)
    nrm = np.zeros((len(vv), 3), np.float32)
    lib().orc_mesh_attributes(_p(vv), len(vv), _p(ff), len(ff), _p(cc), len(pr), _p(pr), _p(_f32(u)), _p(_f32(v)),
                              _p(col), _p(ns), _p(nrm))
    return nrm, col, ns


def camera_rays(pos, lookat, up, vfov, image_w, image_h, xy) -> np.ndarray:
    """Camera::init + generateRay at image coordinates xy[n, 2] -> dir[n, 3]."""
    xy = _f32(xy).reshape(-1, 2)
    out = np.zeros((len(xy), 3), np.float32)
    lib().orc_camera_rays(_p(_f32(pos)), _p(_f32(lookat)), _p(_f32(up)), vfov, image_w, image_h, len(xy),
                          _p(xy), _p(out))
    return out


def disk(u) -> np.ndarray:
    """ConcentricDiskSampling of u[n, 2] -> [n, 2]."""
    u = _f32(u).reshape(-1, 2)
    out = np.zeros_like(u)
    lib().orc_disk(len(u), _p(u), _p(out))
    return out


def local_to_world(normal, v) -> np.ndarray:
    normal, v = _f32(normal).reshape(-1, 3), _f32(v).reshape(-1, 3)
    out = np.zeros_like(v)
    lib().orc_local_to_world(len(v), _p(normal), _p(v), _p(out))
    return out


def cosine_sample(u, normal) -> tuple[np.ndarray, np.ndarray]:
    """getCosineHemisphereSample(u1, u2, N) -> (wi[n, 3], pdf[n])."""
    u, normal = _f32(u).reshape(-1, 2), _f32(normal).reshape(-1, 3)
    wi = np.zeros((len(u), 3), np.float32)
    pdf = np.zeros(len(u), np.float32)
    lib().orc_cosine_sample(len(u), _p(u), _p(normal), _p(wi), _p(pdf))
    return wi, pdf


def point_light(light, p) -> np.ndarray:
    """Shadow-ray direction toward point lights: normalize(light - p)."""
    light, p = _f32(light).reshape(-1, 3), _f32(p).reshape(-1, 3)
    out = np.zeros_like(p)
    lib().orc_point_light(len(p), _p(light), _p(p), _p(out))
    return out


def vbuf_trace(nsamples: int, history: int, op, samid, depth, hist, t) -> tuple[np.ndarray, np.ndarray]:
    """VBuf operations in order (op 0 = update(t, ray), 1 = correct(ray)) ->
    (returned flags, ray histories afterwards)."""
    op = np.ascontiguousarray(op, np.uint8)
    hist = np.array(hist, np.float32, copy=True).reshape(-1, history)
    res = np.zeros(len(op), np.uint8)
    lib().orc_vbuf_trace(nsamples, history, len(op), _p(op), _p(_i32(samid)), _p(_i32(depth)), _p(hist),
                         _p(_f32(t)), _p(res))
    return res, hist


def hdr_add(rgba, pixid, rgb, scale: float) -> np.ndarray:
    """HdrImage::add(pixid[i], rgb[i], scale) in order on a copy of rgba[P, 4]."""
    out = np.array(rgba, np.float32, copy=True).reshape(-1, 4)
    pixid, rgb = _i32(pixid), _f32(rgb).reshape(-1, 3)
    lib().orc_hdr_add(len(pixid), _p(pixid), _p(rgb), scale, _p(out))
    return out


def blinn_phong(args) -> np.ndarray:
    """args[n, 20] = costheta, kd, ks, shininess, li, wi, n_hat, wo -> [n, 3]."""
    args = _f32(args).reshape(-1, 20)
    out = np.zeros((len(args), 3), np.float32)
    lib().orc_blinn_phong(len(args), _p(args), _p(out))
    return out


def unpack_color(colors) -> np.ndarray:
    colors = np.ascontiguousarray(colors, np.uint32)
    out = np.zeros((len(colors), 3), np.float32)
    lib().orc_unpack_color(len(colors), _p(colors), _p(out))
    return out


def reflect(wo, normal) -> np.ndarray:
    wo, normal = _f32(wo).reshape(-1, 3), _f32(normal).reshape(-1, 3)
    out = np.zeros_like(wo)
    lib().orc_reflect(len(wo), _p(wo), _p(normal), _p(out))
    return out


def fr_dielectric(args) -> tuple[np.ndarray, np.ndarray]:
    """args[n, 9] = cos_theta_i, eta_i, eta_t, wo, n -> (fr[n], wt[n, 3])."""
    args = _f32(args).reshape(-1, 9)
    fr = np.zeros(len(args), np.float32)
    wt = np.zeros((len(args), 3), np.float32)
    lib().orc_fr_dielectric(len(args), _p(args), _p(fr), _p(wt))
    return fr, wt


def refract(args) -> tuple[np.ndarray, np.ndarray]:
    """Same layout as fr_dielectric -> (ok[n] as uint8, wt[n, 3])."""
    args = _f32(args).reshape(-1, 9)
    ok = np.zeros(len(args), np.uint8)
    wt = np.zeros((len(args), 3), np.float32)
    lib().orc_refract(len(args), _p(args), _p(ok), _p(wt))
    return ok, wt


class Oracle:
    """CPU oracle for one configuration and scene (see oracle.h)."""

    def __init__(self, config: dict, scene):
        c = OrcConfig()
        for k in ORACLE_FIELDS:
            if k == "ks":
                c.ks = (C.c_float * 3)(*config.get("ks", (0, 0, 0)))
            elif k in config:
                setattr(c, k, config[k])
        self.config = dict(config)
        self.scene = scene
        self.L = lib()
        self.h = self.L.orc_create(C.byref(c), len(scene.domains))
        if not self.h:
            raise RuntimeError("orc_create failed")
        for i, d in enumerate(scene.domains):
            self.L.orc_set_domain(self.h, i, _p(d.vertices), len(d.vertices), _p(d.faces), len(d.faces),
                                  _p(d.colors), _p(d.bounds), d.bsdf_type, _p(d.bsdf_params))
        lf = np.zeros((max(len(scene.lights), 1), 13), np.float32)
        for i, l in enumerate(scene.lights):
            lf[i, 0] = l.type
            lf[i, 1:4] = l.position
            lf[i, 4:7] = l.radiance
            lf[i, 7:10] = l.edge1
            lf[i, 10:13] = l.edge2
        self.L.orc_set_lights(self.h, len(scene.lights), _p(lf))
        self.L.orc_build(self.h)
        self.D = len(scene.domains)

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_camera(self, pos, lookat, up=(0, 1, 0), vfov=None):
        fov = self.config.get("fov", 90.0) if vfov is None else vfov
        self.L.orc_set_camera(self.h, _p(_f32(pos)), _p(_f32(lookat)), _p(_f32(up)), float(fov))

    def normals(self, d):
        out = np.zeros((len(self.scene.domains[d].vertices), 3), np.float32)
        self.L.orc_normals(self.h, d, _p(out))
        return out

    def tiles(self):
        out = np.zeros((4096, 4), np.int32)
        n = self.L.orc_tiles(self.h, _p(out), 4096)
        return out[:n]

    def eyes(self, first_tile, num_tiles):
        t = self.tiles()[first_tile:first_tile + num_tiles]
        n = int((t[:, 2].astype(np.int64) * t[:, 3]).sum() * self.config["pixel_samples"])
        org = np.zeros((n, 3), np.float32)
        dr = np.zeros((n, 3), np.float32)
        pix = np.zeros(n, np.int32)
        sam = np.zeros(n, np.int32)
        self.L.orc_gen_eyes(self.h, first_tile, num_tiles, _p(org), _p(dr), _p(pix), _p(sam))
        return org, dr, pix, sam

    def schedule(self, org, dir, tmax=None, origin=None, capacity=None):
        org, dir = _f32(org), _f32(dir)
        n = len(org)
        cap = capacity or max(64, n * 40)
        ent = np.zeros((cap, 5), np.int32)
        L = self.config.get("list_size", 16)
        dstats = np.zeros((self.D, L), np.int64)
        tm = None if tmax is None else _f32(tmax)
        og = None if origin is None else _i32(origin)
        k = self.L.orc_schedule(self.h, n, _p(org), _p(dir), _p(tm), _p(og), _p(ent), cap, _p(dstats))
        if k < 0:
            raise RuntimeError("schedule capacity too small")
        ent = ent[:k]
        out = np.zeros(k, [("domain", "<i4"), ("ray", "<u4"), ("tdom", "<f4"), ("depth", "<i4"),
                           ("origin", "<i4")])
        out["domain"] = ent[:, 0]
        out["ray"] = ent[:, 1].view(np.uint32)
        out["tdom"] = ent[:, 2].view(np.float32)
        out["depth"] = ent[:, 3]
        out["origin"] = ent[:, 4]
        return out, dstats

    def scores(self, dstats):
        sc = np.zeros(self.D, np.int64)
        od = np.zeros(self.D, np.int32)
        self.L.orc_scores(self.h, _p(np.ascontiguousarray(dstats, np.int64)), _p(sc), _p(od))
        return sc, od

    def closest(self, org, dir):
        org, dir = _f32(org), _f32(dir)
        n = len(org)
        hit = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        dom = np.zeros(n, np.int32)
        prim = np.zeros(n, np.int32)
        u = np.zeros(n, np.float32)
        v = np.zeros(n, np.float32)
        col = np.zeros(n, np.uint32)
        ns = np.zeros((n, 3), np.float32)
        self.L.orc_closest(self.h, n, _p(org), _p(dir), _p(hit), _p(t), _p(dom), _p(prim), _p(u), _p(v),
                           _p(col), _p(ns))
        return dict(hit=hit, t=t, domain=dom, prim=prim, u=u, v=v, color=col, ns=ns)

    def occluded(self, org, dir, tmax, origin):
        org, dir = _f32(org), _f32(dir)
        occ = np.zeros(len(org), np.uint8)
        self.L.orc_occluded(self.h, len(org), _p(org), _p(dir), _p(_f32(tmax)), _p(_i32(origin)), _p(occ))
        return occ

    def slots(self):
        return int(self.L.orc_slots(self.h))

    def shade(self, depth, org, dir, w, pixid, samid, t, domain, color, ns):
        n = len(org)
        S = self.slots()
        sdir = np.zeros((n, S, 3), np.float32)
        sw = np.zeros((n, S, 3), np.float32)
        stmax = np.zeros((n, S), np.float32)
        sval = np.zeros((n, S), np.uint8)
        bdir = np.zeros((n, 3), np.float32)
        bw = np.zeros((n, 3), np.float32)
        bval = np.zeros(n, np.uint8)
        self.L.orc_shade(self.h, depth, n, _p(_f32(org)), _p(_f32(dir)), _p(_f32(w)), _p(_i32(pixid)),
                         _p(_i32(samid)), _p(_f32(t)), _p(_i32(domain)),
                         _p(np.ascontiguousarray(color, np.uint32)), _p(_f32(ns)), _p(sdir), _p(sw),
                         _p(stmax), _p(sval), _p(bdir), _p(bw), _p(bval))
        return dict(sdir=sdir, sw=sw, stmax=stmax, svalid=sval, bdir=bdir, bw=bw, bvalid=bval)

    def _image(self):
        return np.zeros((self.config["image_h"], self.config["image_w"], 4), np.float32)

    def render_wavefront(self):
        img = self._image()
        st = OrcStats()
        if self.L.orc_render_wavefront(self.h, _p(img), C.byref(st)) != 0:
            raise RuntimeError("oracle wavefront render failed")
        return img, st.asdict()

    def set_bvh4(self, d: int, nodes, tris):
        """Domain d's 4-wide BVH in the product's layout (128-byte nodes and
        leaf-ordered triangles of three float4, as spray_gpu_debug returns
        them or a prepared blob holds them); once every domain has one,
        render_wavefront also counts an ordered walk over them."""
        nodes = np.ascontiguousarray(nodes).view(np.float32).reshape(-1)
        tris = np.ascontiguousarray(tris).view(np.float32).reshape(-1)
        if nodes.size % 32 or tris.size % 12:
            raise ValueError("nodes must be 128-byte records, triangles 48-byte records")
        rc = self.L.orc_set_bvh4(self.h, d, _p(nodes), nodes.size // 32, _p(tris), tris.size // 12)
        if rc != 0:
            raise ValueError(f"domain {d}: BVH rejected ({rc})")

    def render_baseline(self):
        """Mode C, the reference's non-speculative image tracer on one
        process: the image, the stats and the domain scheduled in every
        round."""
        img = self._image()
        st = OrcStats()
        if self.L.orc_render_baseline(self.h, _p(img), C.byref(st)) != 0:
            raise RuntimeError("oracle baseline render failed")
        n = self.L.orc_baseline_schedule(self.h, None, 0)
        sched = np.zeros(n, np.int32)
        self.L.orc_baseline_schedule(self.h, _p(sched), n)
        return img, st.asdict(), sched

    def render_speculative(self, nthreads=1):
        img = self._image()
        st = OrcStats()
        if self.L.orc_render_speculative(self.h, nthreads, _p(img), C.byref(st)) != 0:
            raise RuntimeError("oracle speculative render failed")
        return img, st.asdict()
