"""spray_gb300: GB300-native speculative domain-parallel ray tracer.

Python view of the C ABI in include/spray_gpu.h (ctypes; no torch types).  The
classes mirror SpRay's film-mode pieces: `Config` (src/render/config.h),
`Scene` (the .spray loader, src/io/scene_loader.cc), `Tracer` (the
ooc::Tracer concept, src/ooc/ooc_tracer.h).  Every call goes to the CUDA
library; there is no CPU fallback and importing fails loudly when the library
has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libspray_gpu.so"

OK, EINVAL, ECUDA, EIO, ESTATE, EOVERFLOW, ENOMEM, ETIMEOUT = range(8)
DBG_RAYS, DBG_RQUEUES, DBG_HITS, DBG_SHADOWS, DBG_SQUEUES, DBG_SCORES, DBG_LOADS, DBG_NODES, DBG_TRIS = range(9)


class SprayError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class ConfigC(C.Structure):
    _fields_ = [
        ("image_w", C.c_int32), ("image_h", C.c_int32), ("ao_mode", C.c_int32),
        ("ao_samples", C.c_int32), ("pixel_samples", C.c_int32), ("bounces", C.c_int32),
        ("ks", C.c_float * 3), ("shininess", C.c_float), ("fov", C.c_float),
        ("cache_size", C.c_int32), ("max_samples_per_rank", C.c_int32), ("list_size", C.c_int32),
        ("history_size", C.c_int32), ("nthreads", C.c_int32), ("num_ranks", C.c_int32),
        ("rank", C.c_int32), ("ao_light_shadow", C.c_int32), ("ao_max_distance", C.c_float),
        ("rr_depth", C.c_int32), ("cull", C.c_int32), ("cache_bytes", C.c_int64),
        ("wave_samples", C.c_int64), ("debug_capture", C.c_int32), ("device", C.c_int32),
        ("schedule_policy", C.c_int32),
        ("ooc_batch", C.c_int32), ("learn_samples", C.c_int64), ("learn_batch", C.c_int32),
        ("learn_epochs", C.c_int32), ("learn_lr", C.c_float), ("learn_seed", C.c_int32),
        ("learn_frames", C.c_int32), ("graphs", C.c_int32), ("ooc_inplace", C.c_int32),
        ("trace_blocks_per_sm", C.c_int32), ("sched_chunks_per_warp", C.c_int32),
        ("bucket_launches", C.c_int32), ("learn_buckets", C.c_int32), ("bvh_device", C.c_int32),
    ]


class DomainC(C.Structure):
    _fields_ = [
        ("vertices", C.POINTER(C.c_float)), ("faces", C.POINTER(C.c_uint32)),
        ("colors", C.POINTER(C.c_uint32)), ("num_vertices", C.c_int64), ("num_faces", C.c_int64),
        ("world_bounds", C.c_float * 6), ("bsdf_type", C.c_int32), ("bsdf_params", C.c_float * 3),
    ]


class LightC(C.Structure):
    _fields_ = [("type", C.c_int32), ("position", C.c_float * 3), ("radiance", C.c_float * 3),
                ("edge1", C.c_float * 3), ("edge2", C.c_float * 3)]


class ViewC(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("lookat", C.c_float * 3), ("up", C.c_float * 3),
                ("vfov", C.c_float), ("image_w", C.c_int32), ("image_h", C.c_int32),
                ("pixel_samples", C.c_int32), ("ao_mode", C.c_int32), ("ao_samples", C.c_int32),
                ("bounces", C.c_int32), ("rr_depth", C.c_int32), ("ao_light_shadow", C.c_int32),
                ("ao_max_distance", C.c_float)]


class StatsC(C.Structure):
    _fields_ = [
        ("rays_primary", C.c_int64), ("rays_shadow", C.c_int64), ("rays_bounce", C.c_int64),
        ("visits_radiance", C.c_int64), ("visits_shadow", C.c_int64), ("visits_culled", C.c_int64),
        ("domain_loads", C.c_int64), ("h2d_bytes", C.c_int64), ("d2h_bytes", C.c_int64),
        ("kernel_launches", C.c_int64), ("list_overflows", C.c_int64), ("frame_ms", C.c_double),
        ("trace_ms", C.c_double), ("occlude_ms", C.c_double), ("schedule_ms", C.c_double),
        ("trace_launches", C.c_int64), ("occlude_launches", C.c_int64),
        ("nodes_radiance", C.c_int64), ("tris_radiance", C.c_int64), ("nodes_shadow", C.c_int64),
        ("tris_shadow", C.c_int64), ("scene_triangles", C.c_int64), ("scene_bytes", C.c_int64),
        ("h2d_ms", C.c_double), ("learn_pairs", C.c_int64), ("learn_trained", C.c_int64),
        ("learn_ms", C.c_double), ("learn_loss", C.c_double), ("inplace_domains", C.c_int64),
        ("inplace_bytes", C.c_int64), ("cache_slots", C.c_int64), ("cache_slot_bytes", C.c_int64),
        ("learn_eval_pairs", C.c_int64), ("learn_top1", C.c_double), ("learn_top1_nearest", C.c_double),
        ("exchange_bytes", C.c_int64), ("rounds", C.c_int64), ("visits_shade", C.c_int64),
        ("eyes_culled", C.c_int64),
    ]

    def asdict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


# spray_gpu_reduce_ops: element-wise reductions across the ranks of a
# domain-parallel tracer (pointer, count, stream) -> 0 on success
REDUCE_U64 = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint64), C.c_int64, C.c_void_p)
REDUCE_U8 = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_uint8), C.c_int64, C.c_void_p)


class ReduceOpsC(C.Structure):
    _fields_ = [("user", C.c_void_p), ("host_buffers", C.c_int32), ("min_u64", REDUCE_U64),
                ("max_u8", REDUCE_U8)]


DBG_DTYPES = {
    DBG_RAYS: np.dtype([("sample", "<u4"), ("pixid", "<i4"), ("samid", "<i4"), ("org", "<f4", 3),
                        ("dir", "<f4", 3), ("w", "<f4", 3)]),
    DBG_RQUEUES: np.dtype([("domain", "<i4"), ("ray", "<u4"), ("tdom", "<f4"), ("depth", "<i4"),
                           ("origin", "<i4")]),
    DBG_HITS: np.dtype([("sample", "<u4"), ("hit", "<i4"), ("t", "<f4"), ("domain", "<i4"),
                        ("prim", "<i4"), ("color", "<u4"), ("ns", "<f4", 3)]),
    DBG_SHADOWS: np.dtype([("sample", "<u4"), ("slot", "<i4"), ("org", "<f4", 3), ("dir", "<f4", 3),
                           ("w", "<f4", 3), ("tmax", "<f4"), ("occluded", "<i4")]),
    DBG_SQUEUES: np.dtype([("domain", "<i4"), ("ray", "<u4"), ("tdom", "<f4"), ("depth", "<i4"),
                           ("origin", "<i4")]),
    DBG_SCORES: np.dtype([("domain", "<i4"), ("pad", "<i4"), ("score", "<i8"), ("order", "<i4"),
                          ("pad2", "<i4")]),
    DBG_LOADS: np.dtype([("domain", "<i4"), ("outcome", "<i4"), ("evicted", "<i4"), ("pass", "<i4")]),
    # one BVH node (BvhNode4) and one leaf-ordered triangle of a domain (bounce = the domain)
    # box rows: lo x, hi x, lo y, hi y, lo z, hi z of the four children
    DBG_NODES: np.dtype([("box", "<f4", (6, 4)), ("child", "<i4", 4), ("pad", "<i4", 4)]),
    DBG_TRIS: np.dtype([("v", "<f4", (3, 4))]),
}

_lib_handle = None

EXPORTED_SYMBOLS = [
    "spray_gpu_config_defaults", "spray_gpu_last_error", "spray_gpu_create", "spray_gpu_destroy",
    "spray_gpu_set_scene", "spray_gpu_set_camera", "spray_gpu_trace", "spray_gpu_trace_device",
    "spray_scene_load", "spray_scene_free", "spray_scene_counts", "spray_scene_domains",
    "spray_scene_lights", "spray_write_ply", "spray_generate_wavelet", "spray_gpu_debug_count",
    "spray_gpu_debug_copy", "spray_gpu_schedule_static", "spray_gpu_set_insitu", "spray_gpu_insitu_partition",
]


def lib() -> C.CDLL:
    """The loaded CUDA library; raises when it has not been built."""
    global _lib_handle
    if _lib_handle is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        P = C.c_void_p
        L.spray_gpu_last_error.restype = C.c_char_p
        L.spray_gpu_config_defaults.argtypes = [C.POINTER(ConfigC)]
        L.spray_gpu_create.argtypes = [C.POINTER(ConfigC), C.POINTER(P)]
        L.spray_gpu_destroy.argtypes = [P]
        L.spray_gpu_set_scene.argtypes = [P, C.POINTER(DomainC), C.c_int32, C.POINTER(LightC), C.c_int32]
        L.spray_gpu_set_camera.argtypes = [P, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                           C.POINTER(C.c_float), C.c_float]
        L.spray_gpu_trace.argtypes = [P, P, C.POINTER(StatsC)]
        L.spray_gpu_trace_device.argtypes = [P, P, C.POINTER(StatsC)]
        L.spray_gpu_debug_count.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(C.c_int64)]
        L.spray_gpu_debug_copy.argtypes = [P, C.c_int32, C.c_int32, P, C.c_int64]
        L.spray_scene_load.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(P)]
        L.spray_scene_free.argtypes = [P]
        L.spray_scene_counts.argtypes = [P, C.POINTER(C.c_int32), C.POINTER(C.c_int32)]
        L.spray_scene_domains.argtypes = [P, C.POINTER(DomainC), C.c_int32]
        L.spray_scene_lights.argtypes = [P, C.POINTER(LightC), C.c_int32]
        L.spray_write_ply.argtypes = [C.c_char_p, P, C.c_int64, P, P, C.c_int64]
        L.spray_generate_wavelet.argtypes = [C.c_int32, C.c_double, C.POINTER(C.c_double), P, C.c_int64,
                                             P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64)]
        L.spray_gpu_schedule_static.argtypes = [P, C.c_int32, P, P, C.c_int32, C.c_int32, P, C.c_int64, P,
                                                C.POINTER(C.c_int64), P]
        L.spray_gpu_trace_views.argtypes = [P, C.POINTER(ViewC), C.c_int32, P, C.POINTER(StatsC)]
        L.spray_gpu_trace_views_device.argtypes = [P, C.POINTER(ViewC), C.c_int32, P, C.POINTER(StatsC)]
        L.spray_scene_prepare.argtypes = [C.POINTER(DomainC), C.c_int32, C.c_char_p]
        L.spray_gpu_set_insitu.argtypes = [P, C.c_int32, C.c_int32, C.POINTER(ReduceOpsC)]
        L.spray_gpu_insitu_partition.argtypes = [P, C.c_int32, C.c_int32, P]
        L.spray_gpu_set_scene_prepared.argtypes = [P, C.c_char_p, C.c_int32, C.POINTER(LightC), C.c_int32]
        F4 = C.POINTER(C.c_float)
        L.spray_mlp_param_count.restype = C.c_int32
        L.spray_mlp_forward_dev.argtypes = [P, P, F4, P, C.c_int64, P, P, C.c_int32]
        L.spray_mlp_grad_dev.argtypes = [P, P, F4, P, C.c_int64, P, C.c_int32]
        L.spray_mlp_train_dev.argtypes = [P, P, P, P, F4, P, C.c_int64, C.c_int32, C.c_float, C.c_int32,
                                          C.c_int32, P, C.c_int32]
        _lib_handle = L
    return _lib_handle


def _check(code: int) -> None:
    if code != OK:
        raise SprayError(code, lib().spray_gpu_last_error().decode(errors="replace"))


def default_config(**overrides) -> dict:
    c = ConfigC()
    lib().spray_gpu_config_defaults(C.byref(c))
    d = {k: (list(getattr(c, k)) if k == "ks" else getattr(c, k)) for k, _ in ConfigC._fields_}
    for k, v in overrides.items():
        if k not in d:
            raise KeyError(f"unknown config field {k}")
        d[k] = v
    return d


def _config_struct(cfg: dict) -> ConfigC:
    c = ConfigC()
    lib().spray_gpu_config_defaults(C.byref(c))
    for k, v in cfg.items():
        if k == "ks":
            c.ks = (C.c_float * 3)(*v)
        else:
            setattr(c, k, v)
    return c


class Domain:
    """One domain: world-space mesh, AABB, material."""

    def __init__(self, vertices, faces, colors=None, bounds=None, bsdf_type=0, bsdf_params=(1, 1, 1)):
        self.vertices = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, dtype=np.uint32).reshape(-1, 3)
        if colors is None:
            colors = np.zeros(len(self.vertices), np.uint32)
        self.colors = np.ascontiguousarray(colors, dtype=np.uint32).reshape(-1)
        if bounds is None:
            bounds = np.concatenate([self.vertices.min(0), self.vertices.max(0)])
        self.bounds = np.asarray(bounds, dtype=np.float32).reshape(6)
        self.bsdf_type = int(bsdf_type)
        self.bsdf_params = np.asarray(bsdf_params, dtype=np.float32).reshape(3)


class Light:
    POINT, DIFFUSE, QUAD = 0, 1, 2

    def __init__(self, type, position=(0, 0, 0), radiance=(1, 1, 1), edge1=(0, 0, 0), edge2=(0, 0, 0)):
        self.type = int(type)
        self.position = np.asarray(position, np.float32)
        self.radiance = np.asarray(radiance, np.float32)
        self.edge1 = np.asarray(edge1, np.float32)
        self.edge2 = np.asarray(edge2, np.float32)


class Scene:
    """Domains and lights; load a .spray file or build from arrays."""

    def __init__(self, domains: list[Domain], lights: list[Light]):
        self.domains = domains
        self.lights = lights

    @staticmethod
    def load(spray_file: str | os.PathLike, ply_path: str | os.PathLike | None = None) -> "Scene":
        L = lib()
        h = C.c_void_p()
        _check(L.spray_scene_load(str(spray_file).encode(), str(ply_path).encode() if ply_path else None,
                                  C.byref(h)))
        try:
            nd, nl = C.c_int32(), C.c_int32()
            _check(L.spray_scene_counts(h, C.byref(nd), C.byref(nl)))
            doms = (DomainC * nd.value)()
            _check(L.spray_scene_domains(h, doms, nd.value))
            lts = (LightC * max(nl.value, 1))()
            _check(L.spray_scene_lights(h, lts, nl.value))
            domains = []
            for d in doms:
                nv, nf = d.num_vertices, d.num_faces
                v = np.ctypeslib.as_array(d.vertices, shape=(nv * 3,)).copy()
                f = np.ctypeslib.as_array(d.faces, shape=(nf * 3,)).copy()
                c = np.ctypeslib.as_array(d.colors, shape=(nv,)).copy()
                domains.append(Domain(v, f, c, list(d.world_bounds), d.bsdf_type, list(d.bsdf_params)))
            lights = [Light(l.type, list(l.position), list(l.radiance), list(l.edge1), list(l.edge2))
                      for l in lts[: nl.value]]
        finally:
            L.spray_scene_free(h)
        return Scene(domains, lights)

    def domain_structs(self):
        arr = (DomainC * len(self.domains))()
        for i, d in enumerate(self.domains):
            a = arr[i]
            a.vertices = d.vertices.ctypes.data_as(C.POINTER(C.c_float))
            a.faces = d.faces.ctypes.data_as(C.POINTER(C.c_uint32))
            a.colors = d.colors.ctypes.data_as(C.POINTER(C.c_uint32))
            a.num_vertices = len(d.vertices)
            a.num_faces = len(d.faces)
            a.world_bounds = (C.c_float * 6)(*d.bounds.tolist())
            a.bsdf_type = d.bsdf_type
            a.bsdf_params = (C.c_float * 3)(*d.bsdf_params.tolist())
        return arr

    def light_structs(self):
        arr = (LightC * max(len(self.lights), 1))()
        for i, l in enumerate(self.lights):
            a = arr[i]
            a.type = l.type
            a.position = (C.c_float * 3)(*l.position.tolist())
            a.radiance = (C.c_float * 3)(*l.radiance.tolist())
            a.edge1 = (C.c_float * 3)(*l.edge1.tolist())
            a.edge2 = (C.c_float * 3)(*l.edge2.tolist())
        return arr


class Tracer:
    """GPU tracer for one configuration (Tracer::init/trace)."""

    def __init__(self, config: dict | None = None, **overrides):
        cfg = default_config(**(config or {}))
        cfg.update(overrides)
        self.config = cfg
        self._c = _config_struct(cfg)
        self._h = C.c_void_p()
        _check(lib().spray_gpu_create(C.byref(self._c), C.byref(self._h)))

    def close(self) -> None:
        if self._h:
            lib().spray_gpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_scene(self, scene: Scene) -> None:
        doms = scene.domain_structs()
        lts = scene.light_structs()
        self._scene_ref = scene
        _check(lib().spray_gpu_set_scene(self._h, doms, len(scene.domains), lts, len(scene.lights)))

    def set_scene_prepared(self, directory, num_domains: int, lights=()) -> None:
        """set_scene from prepared-domain blobs (see prepare_scene)."""
        lts = Scene([], list(lights)).light_structs()
        _check(lib().spray_gpu_set_scene_prepared(self._h, str(directory).encode(), num_domains, lts,
                                                  len(lights)))

    def set_insitu(self, num_ranks: int, rank: int, min_u64=None, max_u8=None, host_buffers: bool = True) -> None:
        """Domain-parallel tracing (spray_gpu_set_insitu), before set_scene.

        min_u64(array) and max_u8(array) reduce a numpy array in place across
        all ranks (element-wise unsigned minimum of uint64, maximum of uint8)
        when host_buffers is true; otherwise they receive (device pointer, n,
        stream) and must order their work on that stream."""
        ops = ReduceOpsC()
        ops.host_buffers = 1 if host_buffers else 0
        if num_ranks > 1:
            def wrap(fn, dtype):
                def call(user, ptr, n, stream):
                    try:
                        if host_buffers:
                            addr = C.cast(ptr, C.c_void_p).value
                            buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(addr)
                            fn(np.frombuffer(buf, dtype=dtype, count=n))
                        else:
                            fn(C.cast(ptr, C.c_void_p).value, n, stream)
                        return 0
                    except Exception:  # no exception may cross the C boundary
                        import traceback
                        traceback.print_exc()
                        return 1
                return call
            ops.min_u64 = REDUCE_U64(wrap(min_u64, np.uint64))
            ops.max_u8 = REDUCE_U8(wrap(max_u8, np.uint8))
        self._reduce_ops = ops  # the callbacks must outlive the tracer's use of them
        _check(lib().spray_gpu_set_insitu(self._h, num_ranks, rank, C.byref(ops)))

    def set_camera(self, pos, lookat, up=(0, 1, 0), vfov=None) -> None:
        f3 = lambda x: (C.c_float * 3)(*[float(v) for v in x])
        fov = self.config["fov"] if vfov is None else vfov
        _check(lib().spray_gpu_set_camera(self._h, f3(pos), f3(lookat), f3(up), float(fov)))

    def trace(self, out: np.ndarray | None = None) -> tuple[np.ndarray, dict]:
        """One frame into host memory: (H, W, 4) float32 image and stats."""
        W, H = self.config["image_w"], self.config["image_h"]
        if out is None:
            out = np.empty((H, W, 4), np.float32)
        assert out.dtype == np.float32 and out.flags.c_contiguous and out.size == W * H * 4
        st = StatsC()
        _check(lib().spray_gpu_trace(self._h, out.ctypes.data_as(C.c_void_p), C.byref(st)))
        return out, st.asdict()

    def _view_array(self, views: list[dict]):
        arr = (ViewC * len(views))()
        for i, v in enumerate(views):
            c = arr[i]
            c.position = (C.c_float * 3)(*[float(x) for x in v["position"]])
            c.lookat = (C.c_float * 3)(*[float(x) for x in v["lookat"]])
            c.up = (C.c_float * 3)(*[float(x) for x in v.get("up", (0, 1, 0))])
            c.vfov = float(v.get("vfov", self.config["fov"]))
            for k in ("image_w", "image_h", "pixel_samples", "ao_mode", "ao_samples", "bounces", "rr_depth",
                      "ao_light_shadow"):
                setattr(c, k, int(v.get(k, self.config[k])))
            c.ao_max_distance = float(v.get("ao_max_distance", self.config["ao_max_distance"]))
        return arr

    def trace_views_device(self, views: list[dict], dev_ptr: int) -> dict:
        """trace_views into device memory at dev_ptr (the views' images back to back)."""
        st = StatsC()
        _check(lib().spray_gpu_trace_views_device(self._h, self._view_array(views), len(views),
                                                  C.c_void_p(dev_ptr), C.byref(st)))
        return st.asdict()

    def trace_views(self, views: list[dict]) -> tuple[list[np.ndarray], dict]:
        """Several views in one frame (multi-view batch).  Each view is a dict with
        position, lookat, up, vfov and any of image_w, image_h, pixel_samples,
        ao_mode, ao_samples, bounces, rr_depth, ao_light_shadow, ao_max_distance
        (defaults: this tracer's configuration).  Returns one (H, W, 4) image per
        view and the frame's stats."""
        arr = self._view_array(views)
        shapes = [(arr[q].image_h, arr[q].image_w) for q in range(len(views))]
        out = np.empty(sum(h * w for h, w in shapes) * 4, np.float32)
        st = StatsC()
        _check(lib().spray_gpu_trace_views(self._h, arr, len(views), out.ctypes.data_as(C.c_void_p), C.byref(st)))
        imgs, off = [], 0
        for h, w in shapes:
            imgs.append(out[off:off + h * w * 4].reshape(h, w, 4))
            off += h * w * 4
        return imgs, st.asdict()

    def trace_device(self, dev_ptr: int) -> dict:
        """One frame into device memory at dev_ptr (W*H*4 floats)."""
        st = StatsC()
        _check(lib().spray_gpu_trace_device(self._h, C.c_void_p(dev_ptr), C.byref(st)))
        return st.asdict()

    def debug(self, what: int, bounce: int = 0) -> np.ndarray:
        n = C.c_int64()
        _check(lib().spray_gpu_debug_count(self._h, what, bounce, C.byref(n)))
        out = np.zeros(n.value, DBG_DTYPES[what])
        if n.value:
            _check(lib().spray_gpu_debug_copy(self._h, what, bounce, out.ctypes.data_as(C.c_void_p),
                                              out.nbytes))
        return out


def schedule_static(domain_bounds_ptr: int, num_domains: int, org_ptr: int, dir_ptr: int, num_rays: int,
                    list_size: int, entries_ptr: int, entry_capacity: int, domain_start_ptr: int,
                    stream: int | None = None) -> int:
    """spray_gpu_schedule_static on device pointers; returns the entry count."""
    n = C.c_int64()
    _check(lib().spray_gpu_schedule_static(C.c_void_p(domain_bounds_ptr), num_domains, C.c_void_p(org_ptr),
                                           C.c_void_p(dir_ptr), num_rays, list_size,
                                           C.c_void_p(entries_ptr), entry_capacity,
                                           C.c_void_p(domain_start_ptr), C.byref(n),
                                           C.c_void_p(stream) if stream else None))
    return n.value


def insitu_partition(bounds, num_ranks: int) -> np.ndarray:
    """Rank of each domain under SpRay's in-situ partition (host only)."""
    b = np.ascontiguousarray(bounds, np.float32).reshape(-1, 6)
    out = np.zeros(len(b), np.int32)
    _check(lib().spray_gpu_insitu_partition(b.ctypes.data_as(C.c_void_p), len(b), num_ranks,
                                            out.ctypes.data_as(C.c_void_p)))
    return out


def prepare_scene(scene: "Scene", directory) -> None:
    """Writes one prepared-domain blob per domain (normals, BVH, leaf-ordered
    triangles) into `directory`; needs no GPU."""
    Path(directory).mkdir(parents=True, exist_ok=True)
    _check(lib().spray_scene_prepare(scene.domain_structs(), len(scene.domains), str(directory).encode()))


# spray_mlp_sample
MLP_SAMPLE_DTYPE = np.dtype([("org", "<f4", 3), ("dir", "<f4", 3), ("cand", "<u2", 8), ("ncand", "<i4"),
                             ("label", "<i4")])


def mlp_param_count() -> int:
    return int(lib().spray_mlp_param_count())


def _norm(norm) -> C.Array:
    return (C.c_float * 4)(*[float(x) for x in norm])


def mlp_forward(params_ptr: int, boxes_ptr: int, norm, samples_ptr: int, n: int, logits_ptr: int,
                pred_ptr: int, device: int = 0) -> None:
    """Learned proposal forward pass on device buffers (spray_mlp_forward_dev)."""
    P = C.c_void_p
    _check(lib().spray_mlp_forward_dev(P(params_ptr), P(boxes_ptr), _norm(norm), P(samples_ptr), n,
                                       P(logits_ptr), P(pred_ptr), device))


def mlp_grad(params_ptr: int, boxes_ptr: int, norm, samples_ptr: int, n: int, grad_ptr: int,
             device: int = 0) -> None:
    """Mean cross-entropy gradient, loss sum and labelled count (spray_mlp_grad_dev)."""
    P = C.c_void_p
    _check(lib().spray_mlp_grad_dev(P(params_ptr), P(boxes_ptr), _norm(norm), P(samples_ptr), n,
                                    P(grad_ptr), device))


def mlp_train(params_ptr: int, m_ptr: int, v_ptr: int, boxes_ptr: int, norm, samples_ptr: int, n: int,
              batch: int, lr: float, steps: int, first_step: int = 1, losses_ptr: int = 0,
              device: int = 0) -> None:
    """Adam steps over consecutive batches (spray_mlp_train_dev)."""
    P = C.c_void_p
    _check(lib().spray_mlp_train_dev(P(params_ptr), P(m_ptr), P(v_ptr), P(boxes_ptr), _norm(norm),
                                     P(samples_ptr), n, batch, lr, steps, first_step,
                                     P(losses_ptr) if losses_ptr else None, device))


def generate_wavelet(samples: int = 64, iso: float = 157.0, phase=(0.0, 0.0, 0.0)):
    """Wavelet isosurface on [-1,1]^3: (vertices (n,3) float32, faces (m,3) uint32)."""
    L = lib()
    nv, nf = C.c_int64(), C.c_int64()
    ph = (C.c_double * 3)(*phase)
    code = L.spray_generate_wavelet(samples, iso, ph, None, 0, None, 0, C.byref(nv), C.byref(nf))
    if code not in (OK, EOVERFLOW):
        _check(code)
    v = np.empty((nv.value, 3), np.float32)
    f = np.empty((nf.value, 3), np.uint32)
    _check(L.spray_generate_wavelet(samples, iso, ph, v.ctypes.data_as(C.c_void_p), nv.value,
                                    f.ctypes.data_as(C.c_void_p), nf.value, C.byref(nv), C.byref(nf)))
    return v, f


def write_ply(path, vertices, faces, colors=None) -> None:
    v = np.ascontiguousarray(vertices, np.float32)
    f = np.ascontiguousarray(faces, np.uint32)
    c = None if colors is None else np.ascontiguousarray(colors, np.uint32)
    _check(lib().spray_write_ply(str(path).encode(), v.ctypes.data_as(C.c_void_p), len(v.reshape(-1, 3)),
                                 None if c is None else c.ctypes.data_as(C.c_void_p),
                                 f.ctypes.data_as(C.c_void_p), len(f.reshape(-1, 3))))
