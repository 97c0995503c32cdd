"""CPU restatement (numpy) of the learned domain-order proposal.

TEST INFRASTRUCTURE ONLY: the checker of the tensor-core MLP kernels in
spray_gb300/csrc/mlp.cu.  SpRay has no learned component, so there is no
reference file to follow; the network, its features and its training rule
are the ones the CUDA path states: 54 features (normalised origin and
direction, then six per candidate of the first eight: distance along the ray
to the point closest to the box centre, distance from the centre there, box
half diagonal, their two ratios, presence), three ReLU
layers of 64, eight logits masked to the present candidates, mean softmax
cross-entropy over labelled rows, Adam (beta1 0.9, beta2 0.999, eps 1e-8).

The GPU rounds to bfloat16 (round to nearest even) at fixed points: the
features, the weights, every hidden activation after ReLU and every
back-propagated dZ before it enters a tensor-core product; products
accumulate in fp32.  `rounding=True` reproduces those points (sums in
float64, then float32); `rounding=False` runs the same algebra in float64,
which the finite-difference test uses to pin the back-propagation itself.
"""
from __future__ import annotations

import numpy as np

CAND = 8
K = 64
HID = 64
OUT_PAD = 16
W1, B1 = 0, HID * K
W2, B2 = B1 + HID, B1 + HID + HID * HID
W3, B3 = B2 + HID, B2 + HID + HID * HID
W4, B4 = B3 + HID, B3 + HID + OUT_PAD * HID
PARAMS = B4 + OUT_PAD

SAMPLE_DTYPE = np.dtype([("org", "<f4", 3), ("dir", "<f4", 3), ("cand", "<u2", 8), ("ncand", "<i4"),
                         ("label", "<i4")])


def bf16(x: np.ndarray) -> np.ndarray:
    """float32 -> nearest bfloat16 (ties to even), returned as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32).reshape(x.shape)


def init_params(seed: int) -> np.ndarray:
    """He-uniform weights, zero biases, zero padding (seeded test parameters)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS, np.float32)

    def put(off, rows, cols, fan_in, real_rows=None, real_cols=None):
        real_rows = rows if real_rows is None else real_rows
        real_cols = cols if real_cols is None else real_cols
        lim = np.sqrt(6.0 / fan_in)
        w = np.zeros((rows, cols), np.float32)
        w[:real_rows, :real_cols] = rng.uniform(-lim, lim, (real_rows, real_cols))
        p[off:off + rows * cols] = w.ravel()

    put(W1, HID, K, 54, real_cols=54)
    put(W2, HID, HID, HID)
    put(W3, HID, HID, HID)
    put(W4, OUT_PAD, HID, HID, real_rows=CAND)
    return p


def unpack(p: np.ndarray):
    return (p[W1:B1].reshape(HID, K), p[B1:W2], p[W2:B2].reshape(HID, HID), p[B2:W3],
            p[W3:B3].reshape(HID, HID), p[B3:W4], p[W4:B4].reshape(OUT_PAD, HID), p[B4:PARAMS])


def features(samples: np.ndarray, boxes: np.ndarray, norm) -> np.ndarray:
    """(n, 64) float32 features, the same float32 operations as the kernel:
    normalised origin, direction, and per candidate (zeros when absent) the
    distance along the ray to the point closest to the box centre, the ray's
    distance from the centre there, the box half diagonal, their two ratios
    (miss / r at most 4, along / r within [-4, 4]) and a presence flag."""
    n = len(samples)
    c = np.asarray(norm[:3], np.float32)
    s = np.float32(norm[3])
    f = np.zeros((n, K), np.float32)
    on = ((samples["org"] - c) * s).astype(np.float32)
    d = np.asarray(samples["dir"], np.float32)
    f[:, 0:3] = on
    f[:, 3:6] = d
    nc = np.minimum(samples["ncand"], CAND)
    bx = np.asarray(boxes, np.float32).reshape(-1, 6)
    half = np.float32(0.5)
    for j in range(CAND):
        present = j < nc
        b = bx[np.where(present, samples["cand"][:, j].astype(np.int64), 0)]
        lo = ((b[:, 0:3] - c) * s).astype(np.float32)
        hi = ((b[:, 3:6] - c) * s).astype(np.float32)
        pc = ((lo + hi) * half - on).astype(np.float32)
        hh = ((hi - lo) * half).astype(np.float32)
        along = (pc[:, 0] * d[:, 0] + pc[:, 1] * d[:, 1]) + pc[:, 2] * d[:, 2]
        pp = (pc[:, 0] * pc[:, 0] + pc[:, 1] * pc[:, 1]) + pc[:, 2] * pc[:, 2]
        miss = np.sqrt(np.maximum(pp - along * along, np.float32(0.0))).astype(np.float32)
        r = np.sqrt((hh[:, 0] * hh[:, 0] + hh[:, 1] * hh[:, 1]) + hh[:, 2] * hh[:, 2]).astype(np.float32)
        with np.errstate(divide="ignore"):
            ir = np.where(r > 0, np.float32(1.0) / np.where(r > 0, r, np.float32(1.0)), np.float32(0.0))
        ir = ir.astype(np.float32)
        cols = [along, miss, r, np.minimum(miss * ir, np.float32(4.0)),
                np.minimum(np.maximum(along * ir, np.float32(-4.0)), np.float32(4.0)), np.ones(n, np.float32)]
        for k, v in enumerate(cols):
            f[:, 6 + 6 * j + k] = np.where(present, v, np.float32(0.0))
    return f


def _mm(a, b, rounding):
    if rounding:
        return (a.astype(np.float64) @ b.astype(np.float64)).astype(np.float32)
    return a @ b


def forward(params: np.ndarray, samples: np.ndarray, boxes, norm, rounding: bool = True):
    """Returns (logits (n, 8) with -inf for absent candidates, cache for backward)."""
    r = bf16 if rounding else (lambda x: np.asarray(x, np.float64))
    w1, b1, w2, b2, w3, b3, w4, b4 = unpack(np.asarray(params, np.float32 if rounding else np.float64))
    x = r(features(samples, boxes, norm))
    w1r, w2r, w3r, w4r = r(w1), r(w2), r(w3), r(w4)

    def layer(h, w, b):
        z = _mm(h, w.T, rounding)
        if rounding:
            z = (z + b.astype(np.float32)).astype(np.float32)
        else:
            z = z + b
        return r(np.maximum(z, 0.0))

    h1 = layer(x, w1r, b1)
    h2 = layer(h1, w2r, b2)
    h3 = layer(h2, w3r, b3)
    z4 = _mm(h3, w4r.T, rounding)[:, :CAND] + b4[:CAND]
    nc = np.minimum(samples["ncand"], CAND)
    valid = np.arange(CAND)[None, :] < nc[:, None]
    logits = np.where(valid, z4, -np.inf)
    return logits, (x, h1, h2, h3, (w1r, w2r, w3r, w4r), valid)


def predict(params, samples, boxes, norm) -> np.ndarray:
    logits, _ = forward(params, samples, boxes, norm)
    return np.argmax(logits, axis=1)


def grad(params: np.ndarray, samples: np.ndarray, boxes, norm, rounding: bool = True):
    """(gradient [PARAMS], loss sum, labelled count) of the mean cross-entropy."""
    r = bf16 if rounding else (lambda x: np.asarray(x, np.float64))
    dt = np.float32 if rounding else np.float64
    logits, (x, h1, h2, h3, (w1r, w2r, w3r, w4r), valid) = forward(params, samples, boxes, norm, rounding)
    n = len(samples)
    nc = np.minimum(samples["ncand"], CAND)
    lab = samples["label"]
    labelled = (lab >= 0) & (lab < nc)
    cnt = int(labelled.sum())
    inv = dt(1.0 / cnt) if cnt else dt(0.0)
    m = np.max(np.where(valid, logits, -np.inf), axis=1, initial=-np.inf)
    m = np.where(np.isfinite(m), m, 0.0)
    e = np.where(valid, np.exp(np.where(valid, logits, 0.0) - m[:, None]), 0.0)
    ssum = e.sum(axis=1)
    loss = 0.0
    dz4 = np.zeros((n, OUT_PAD), dt)
    rows = np.nonzero(labelled)[0]
    if len(rows):
        li = lab[rows]
        loss = float(np.sum(np.log(ssum[rows]) - (logits[rows, li] - m[rows])))
        p = e[rows] / ssum[rows, None]
        oh = np.zeros_like(p)
        oh[np.arange(len(rows)), li] = 1.0
        dz4[rows, :CAND] = ((p - oh) * inv).astype(dt)
    g = np.zeros(PARAMS, np.float64)
    d4 = r(dz4)
    g[W4:B4] = _mm(d4.T, h3, rounding).ravel()
    g[B4:PARAMS] = d4.sum(axis=0)
    dh3 = _mm(d4, w4r, rounding)
    d3 = r(np.where(h3 > 0, dh3, 0.0))
    g[W3:B3] = _mm(d3.T, h2, rounding).ravel()
    g[B3:W4] = d3.sum(axis=0)
    dh2 = _mm(d3, w3r, rounding)
    d2 = r(np.where(h2 > 0, dh2, 0.0))
    g[W2:B2] = _mm(d2.T, h1, rounding).ravel()
    g[B2:W3] = d2.sum(axis=0)
    dh1 = _mm(d2, w2r, rounding)
    d1 = r(np.where(h1 > 0, dh1, 0.0))
    g[W1:B1] = _mm(d1.T, x, rounding).ravel()
    g[B1:W2] = d1.sum(axis=0)
    return g, loss, cnt


def mean_loss(params: np.ndarray, samples: np.ndarray, boxes, norm) -> float:
    """float64 mean cross-entropy without rounding (finite-difference target)."""
    _, loss, cnt = grad(params, samples, boxes, norm, rounding=False)
    return loss / max(cnt, 1)


def adam(params, m, v, g, lr: float, step: int):
    """One Adam step in float32, the kernel's operation order."""
    g = np.asarray(g, np.float32)
    m[:] = np.float32(0.9) * m + np.float32(0.1) * g
    v[:] = np.float32(0.999) * v + np.float32(0.001) * (g * g)
    mh = m / np.float32(1.0 - 0.9 ** step)
    vh = v / np.float32(1.0 - 0.999 ** step)
    params[:] = params - np.float32(lr) * mh / (np.sqrt(vh) + np.float32(1e-8))
    return params
