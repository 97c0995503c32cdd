"""The oracle's own reader of SpRay scene files (.spray + PLY).

TEST INFRASTRUCTURE ONLY.  A numpy restatement of the reference's scene
loading so that the oracle (and bench.py's reference arm, which must run
without the CUDA library) can load a scene by itself:

  .spray grammar      src/io/scene_loader.cc:42-270 (tags, materials, lights,
                      bound, scale/rotate/translate, face/vertex counts)
  world bounds        src/io/scene_loader.cc:351-357 (the transform applied to
                      the two object-space corners)
  PLY                 src/io/ply_loader.cc:179-324 (binary little endian or
                      ascii; float x y z, optional uchar r g b packed as
                      r << 16 | g << 8 | b; triangle lists)
  vertex transform    src/render/trimesh_buffer.cc:141-153, applied only when
                      the matrix is not the identity (src/render/scene.inl:178)

Matrix arithmetic follows glm's operation order in float32 (the same order
the reference build's glm stand-in, oracle/ref_shim/glm, restates):
translate adds m0 x + m1 y + m2 z + m3 left to right, rotate builds the 3x3
rotation from cosf/sinf of the float angle, and mat4 * vec4 sums pairwise,
(m0 x + m1 y) + (m2 z + m3 w).  The one extension the benchmark scenes use,
`light quad p0 edge1 edge2 radiance`, is read as the product reads it.
"""
from __future__ import annotations

import ctypes
import ctypes.util
import math
from pathlib import Path

import numpy as np

F32 = np.float32
BSDF = {"diffuse": 0, "mirror": 1, "glass": 2, "transmission": 3}
LIGHT_POINT, LIGHT_DIFFUSE, LIGHT_QUAD = 0, 1, 2

_libm = None


def _cosf_sinf(x: float) -> tuple[np.float32, np.float32]:
    """glm::cos/sin of a float angle: the C library's cosf and sinf."""
    global _libm
    if _libm is None:
        _libm = ctypes.CDLL(ctypes.util.find_library("m") or "libm.so.6")
        for n in ("cosf", "sinf"):
            getattr(_libm, n).restype = ctypes.c_float
            getattr(_libm, n).argtypes = [ctypes.c_float]
    return F32(_libm.cosf(float(x))), F32(_libm.sinf(float(x)))


class Domain:
    """One domain in world space, with the fields the oracle reads."""

    def __init__(self, vertices, faces, colors, bounds, bsdf_type=0, bsdf_params=(1, 1, 1)):
        self.vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
        self.faces = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
        self.colors = np.ascontiguousarray(colors, np.uint32).reshape(-1)
        self.bounds = np.asarray(bounds, np.float32).reshape(6)
        self.bsdf_type = int(bsdf_type)
        self.bsdf_params = np.asarray(bsdf_params, np.float32).reshape(3)


class Light:
    def __init__(self, type, position=(0, 0, 0), radiance=(0, 0, 0), edge1=(0, 0, 0), edge2=(0, 0, 0)):
        self.type = int(type)
        self.position = np.asarray(position, np.float32)
        self.radiance = np.asarray(radiance, np.float32)
        self.edge1 = np.asarray(edge1, np.float32)
        self.edge2 = np.asarray(edge2, np.float32)


class Scene:
    def __init__(self, domains, lights):
        self.domains = domains
        self.lights = lights


# ---------------------------------------------------------------- glm order
def _identity() -> np.ndarray:
    return np.eye(4, dtype=np.float32)  # [column][row], column-major like glm


def _translate(m: np.ndarray, v) -> np.ndarray:
    r = m.copy()
    x, y, z = (F32(a) for a in v)
    r[3] = ((m[0] * x + m[1] * y) + m[2] * z) + m[3]
    return r


def _scale(m: np.ndarray, v) -> np.ndarray:
    r = m.copy()
    for i in range(3):
        r[i] = m[i] * F32(v[i])
    return r


def _rotate(m: np.ndarray, angle: np.float32, axis_index: int) -> np.ndarray:
    c, s = _cosf_sinf(angle)
    axis = np.zeros(3, np.float32)
    axis[axis_index] = 1.0
    # normalize(v) = v * (1 / sqrt(dot(v, v))) with dot = (xx + yy) + zz
    d = (axis[0] * axis[0] + axis[1] * axis[1]) + axis[2] * axis[2]
    axis = axis * (F32(1.0) / F32(math.sqrt(float(d))))
    temp = (F32(1.0) - c) * axis
    R = np.zeros((3, 3), np.float32)
    R[0, 0] = c + temp[0] * axis[0]
    R[0, 1] = temp[0] * axis[1] + s * axis[2]
    R[0, 2] = temp[0] * axis[2] - s * axis[1]
    R[1, 0] = temp[1] * axis[0] - s * axis[2]
    R[1, 1] = c + temp[1] * axis[1]
    R[1, 2] = temp[1] * axis[2] + s * axis[0]
    R[2, 0] = temp[2] * axis[0] + s * axis[1]
    R[2, 1] = temp[2] * axis[1] - s * axis[0]
    R[2, 2] = c + temp[2] * axis[2]
    r = m.copy()
    for i in range(3):
        r[i] = (m[0] * R[i, 0] + m[1] * R[i, 1]) + m[2] * R[i, 2]
    r[3] = m[3]
    return r


def transform_points(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    """mat4 * vec4(p, 1) for p[n, 3], pairwise: (m0 x + m1 y) + (m2 z + m3)."""
    p = np.ascontiguousarray(p, np.float32).reshape(-1, 3)
    x, y, z = p[:, 0:1], p[:, 1:2], p[:, 2:3]
    add0 = m[0][None, :] * x + m[1][None, :] * y
    add1 = m[2][None, :] * z + m[3][None, :] * F32(1.0)
    return (add0 + add1)[:, :3].astype(np.float32)


# ---------------------------------------------------------------- .spray
def _atof(tok: str) -> np.float32:
    return F32(float(tok))


def parse_spray(path, ply_path=None) -> tuple[list[dict], list[Light]]:
    """Domain records (file, material, bounds, transform) and lights of a .spray file."""
    doms: list[dict] = []
    lights: list[Light] = []
    for lineno, raw in enumerate(Path(path).read_text().splitlines(), 1):
        t = [w for w in raw.rstrip("\r").split(" ") if w]  # strtok(" ")
        if not t or t[0][0] == "#":
            continue
        tag = t[0]

        def need(n):
            if len(t) != n:
                raise ValueError(f"{path}:{lineno}: '{tag}' expects {n - 1} tokens")

        if tag == "domain":
            doms.append(dict(file=None, bsdf=0, params=np.ones(3, np.float32), bound=np.zeros(6, np.float32),
                             m=_identity()))
            continue
        if tag == "light":
            kind = t[1] if len(t) > 1 else ""
            if kind == "point":
                need(8)
                lights.append(Light(LIGHT_POINT, [_atof(x) for x in t[2:5]], [_atof(x) for x in t[5:8]]))
            elif kind == "diffuse":
                need(5)
                lights.append(Light(LIGHT_DIFFUSE, radiance=[_atof(x) for x in t[2:5]]))
            elif kind == "quad":
                need(14)
                v = [_atof(x) for x in t[2:14]]
                lights.append(Light(LIGHT_QUAD, v[0:3], v[9:12], v[3:6], v[6:9]))
            else:
                raise ValueError(f"{path}:{lineno}: unknown light source {kind}")
            continue
        if not doms:
            raise ValueError(f"{path}:{lineno}: '{tag}' before 'domain'")
        d = doms[-1]
        if tag == "file":
            need(2)
            d["file"] = t[1] if not ply_path else f"{ply_path}/{t[1]}"
        elif tag == "mtl":
            if t[1] in ("diffuse", "mirror"):
                need(5)
                d["bsdf"], d["params"] = BSDF[t[1]], np.array([_atof(x) for x in t[2:5]], np.float32)
            elif t[1] in ("glass", "transmission"):
                need(4)
                d["bsdf"], d["params"] = BSDF[t[1]], np.array([_atof(t[2]), _atof(t[3]), 0.0], np.float32)
            else:
                raise ValueError(f"{path}:{lineno}: unknown material type {t[1]}")
        elif tag == "bound":
            need(7)
            d["bound"] = np.array([_atof(x) for x in t[1:7]], np.float32)
        elif tag == "scale":
            need(4)
            d["m"] = _scale(d["m"], [_atof(x) for x in t[1:4]])
        elif tag == "rotate":
            need(3)
            axis = {"x": 0, "y": 1, "z": 2}.get(t[1])
            if axis is None:
                raise ValueError(f"{path}:{lineno}: invalid axis name {t[1]}")
            # glm::radians on the double from atof, then (float)
            d["m"] = _rotate(d["m"], F32(float(t[2]) * 0.01745329251994329576923690768489), axis)
        elif tag == "translate":
            need(4)
            d["m"] = _translate(d["m"], [_atof(x) for x in t[1:4]])
        elif tag in ("face", "vertex"):
            need(2)
        else:
            raise ValueError(f"{path}:{lineno}: unknown tag name {tag}")
    if not doms:
        raise ValueError(f"no domains in {path}")
    return doms, lights


# ---------------------------------------------------------------- PLY
_PLY_TYPES = {"char": "i1", "int8": "i1", "uchar": "u1", "uint8": "u1", "short": "<i2", "int16": "<i2",
              "ushort": "<u2", "uint16": "<u2", "int": "<i4", "int32": "<i4", "uint": "<u4",
              "uint32": "<u4", "float": "<f4", "float32": "<f4", "double": "<f8", "float64": "<f8"}


def read_ply(path) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """(vertices [n, 3] float32, faces [m, 3] uint32, colours [n] uint32)."""
    data = Path(path).read_bytes()
    end = data.index(b"end_header")
    end = data.index(b"\n", end) + 1
    header = data[:end].decode("ascii", "replace").splitlines()
    if header[0].strip() != "ply":
        raise ValueError(f"{path}: unknown file type")
    fmt, elems, cur = None, [], None
    for line in header[1:]:
        w = line.split()
        if not w:
            continue
        if w[0] == "format":
            fmt = w[1]
        elif w[0] == "element":
            cur = dict(name=w[1], n=int(w[2]), props=[])
            elems.append(cur)
        elif w[0] == "property":
            cur["props"].append(w[1:])
    if fmt not in ("ascii", "binary_little_endian"):
        raise ValueError(f"{path}: unsupported ply format {fmt}")
    verts = faces = cols = None
    body = data[end:]
    off = 0
    text = body.decode("ascii", "replace").splitlines() if fmt == "ascii" else None
    row = 0
    for e in elems:
        if e["name"] == "vertex":
            names = [p[1] for p in e["props"]]
            has_color = all(c in names for c in ("red", "green", "blue"))
            if fmt == "binary_little_endian":
                # the reference reads x y z as float, then r g b as uchar
                dt = [("xyz", "<f4", 3)] + ([("rgb", "u1", 3)] if has_color else [])
                a = np.frombuffer(body, np.dtype(dt), e["n"], off)
                off += a.nbytes
                verts = a["xyz"].astype(np.float32)
                rgb = a["rgb"].astype(np.uint32) if has_color else None
            else:
                rows = np.array([text[row + i].split()[: 6 if has_color else 3] for i in range(e["n"])],
                                dtype=np.float64)
                row += e["n"]
                verts = rows[:, :3].astype(np.float32)
                rgb = rows[:, 3:6].astype(np.uint32) if has_color else None
            cols = ((rgb[:, 0] << 16) | (rgb[:, 1] << 8) | rgb[:, 2]) if has_color else \
                np.zeros(len(verts), np.uint32)
        elif e["name"] == "face":
            p = e["props"][0]
            if p[0] != "list":
                raise ValueError(f"{path}: face property must be a list")
            if fmt == "binary_little_endian":
                dt = np.dtype([("n", _PLY_TYPES[p[1]]), ("i", _PLY_TYPES[p[2]], 3)])
                a = np.frombuffer(body, dt, e["n"], off)
                off += a.nbytes
                if np.any(a["n"] != 3):
                    raise ValueError(f"{path}: only triangle faces are supported")
                faces = a["i"].astype(np.uint32)
            else:
                rows = np.array([text[row + i].split()[:4] for i in range(e["n"])], dtype=np.int64)
                row += e["n"]
                if np.any(rows[:, 0] != 3):
                    raise ValueError(f"{path}: only triangle faces are supported")
                faces = rows[:, 1:4].astype(np.uint32)
    if verts is None or faces is None:
        raise ValueError(f"{path}: malformed ply")
    return verts, faces, cols


def load(spray_file, ply_path=None) -> Scene:
    """SceneLoader::load + TriMeshBuffer::load for every domain."""
    recs, lights = parse_spray(spray_file, None if ply_path is None else str(ply_path))
    domains = []
    for r in recs:
        v, f, c = read_ply(r["file"])
        m = r["m"]
        if not np.array_equal(m, _identity()):
            v = transform_points(m, v)
        lo = transform_points(m, r["bound"][:3])[0]
        hi = transform_points(m, r["bound"][3:])[0]
        domains.append(Domain(v, f, c, np.concatenate([lo, hi]), r["bsdf"], r["params"]))
    return Scene(domains, lights)
