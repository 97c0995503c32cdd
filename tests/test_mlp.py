"""The learned domain-order proposal: the numpy oracle's back-propagation is
pinned by finite differences (CPU), then the tensor-core forward pass,
gradient and Adam steps are checked against it (GPU)."""
import numpy as np
import pytest

from oracle import mlp as om

NORM = (2.0, 2.0, 2.0, 0.5)


def grid_boxes(n=4):
    b = []
    for z in range(n):
        for y in range(n):
            for x in range(n):
                b.append([x, y, z, x + 1, y + 1, z + 1])
    return np.asarray(b, np.float32)


def make_samples(n, seed, nd=64, labelled=0.8):
    rng = np.random.default_rng(seed)
    s = np.zeros(n, om.SAMPLE_DTYPE)
    s["org"] = rng.uniform(-1.0, 5.0, (n, 3))
    d = rng.normal(size=(n, 3))
    s["dir"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    s["ncand"] = rng.integers(0, 9, n)
    for i in range(n):
        s["cand"][i] = rng.choice(nd, 8, replace=False)
    lab = rng.integers(0, 8, n) % np.maximum(s["ncand"], 1)
    keep = (rng.uniform(size=n) < labelled) & (s["ncand"] > 0)
    s["label"] = np.where(keep, lab, -1)
    return s


def test_sample_layout_matches_header():
    import spray_gb300 as sg
    assert om.SAMPLE_DTYPE.itemsize == 48 and sg.MLP_SAMPLE_DTYPE == om.SAMPLE_DTYPE
    assert om.PARAMS == 13520


def test_oracle_backprop_matches_finite_differences():
    boxes = grid_boxes()
    s = make_samples(48, 1)
    p = om.init_params(3).astype(np.float64)
    p[om.B1:om.W2] = 0.05  # keep units active so the check sees every layer
    g, loss, cnt = om.grad(p, s, boxes, NORM, rounding=False)  # already the mean's gradient
    rng = np.random.default_rng(0)
    idx = np.concatenate([rng.integers(om.W1, om.W1 + 64 * 54, 6), rng.integers(om.W2, om.B2, 6),
                          rng.integers(om.W3, om.B3, 6), om.W4 + rng.integers(0, 8 * 64, 6),
                          np.arange(om.B1, om.B1 + 3), np.arange(om.B4, om.B4 + 3)])
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp = om.mean_loss(q, s, boxes, NORM)
        q[i] -= 2 * eps
        lm = om.mean_loss(q, s, boxes, NORM)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_oracle_bf16_rounding_is_nearest_even():
    # bf16 spacing at 1.0 is 2^-7: 1 + 2^-8 is a tie (to even: 1.0), 1 + 3 * 2^-8 a tie to 1 + 2^-6
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -8 + 2 ** -12, -2.5], np.float32)
    r = om.bf16(x)
    assert list(r) == [1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, -2.5]


torch = pytest.importorskip("torch")


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


def ptr(t):
    return t.data_ptr()


@pytest.mark.gpu
def test_forward_matches_oracle(lib_built):
    import spray_gb300 as sg
    boxes = grid_boxes()
    s = make_samples(1000, 2)
    p = om.init_params(5)
    p[om.B1:om.W2] = 0.02
    logits = torch.zeros(len(s) * 8, dtype=torch.float32, device="cuda")
    pred = torch.zeros(len(s), dtype=torch.int32, device="cuda")
    dp, db, ds = dev(p), dev(boxes), dev(s)
    sg.mlp_forward(ptr(dp), ptr(db), NORM, ptr(ds), len(s), ptr(logits), ptr(pred))
    got = logits.cpu().numpy().reshape(-1, 8)
    want, _ = om.forward(p, s, boxes, NORM)
    fin = np.isfinite(want)
    assert np.array_equal(np.isfinite(got), fin)
    assert np.allclose(got[fin], want[fin], atol=2e-2, rtol=2e-2), np.abs(got[fin] - want[fin]).max()
    has = s["ncand"] > 0
    agree = (pred.cpu().numpy()[has] == np.argmax(want, axis=1)[has]).mean()
    assert agree >= 0.99


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 127, 128, 4096 + 37])
def test_gradient_matches_oracle(lib_built, n):
    import spray_gb300 as sg
    boxes = grid_boxes()
    s = make_samples(n, 10 + n)
    p = om.init_params(7)
    p[om.B1:om.W2] = 0.02
    grad = torch.zeros(om.PARAMS + 2, dtype=torch.float32, device="cuda")
    dp, db, ds = dev(p), dev(boxes), dev(s)
    sg.mlp_grad(ptr(dp), ptr(db), NORM, ptr(ds), n, ptr(grad))
    g = grad.cpu().numpy()
    want, loss, cnt = om.grad(p, s, boxes, NORM)
    assert g[om.PARAMS + 1] == cnt
    assert abs(g[om.PARAMS] - loss) <= 1e-3 * max(1.0, abs(loss))
    if cnt == 0:
        assert not np.any(g[:om.PARAMS])
        return
    for name, a, b in (("W1", om.W1, om.B1), ("b1", om.B1, om.W2), ("W2", om.W2, om.B2),
                       ("b2", om.B2, om.W3), ("W3", om.W3, om.B3), ("b3", om.B3, om.W4),
                       ("W4", om.W4, om.B4), ("b4", om.B4, om.PARAMS)):
        ref = want[a:b]
        err = np.linalg.norm(g[a:b] - ref) / max(np.linalg.norm(ref), 1e-12)
        assert err < 3e-2, (name, err)
    # padding receives no gradient
    assert not np.any(g[om.W1:om.B1].reshape(64, 64)[:, 54:])
    assert not np.any(g[om.W4:om.B4].reshape(16, 64)[8:])


@pytest.mark.gpu
def test_adam_steps_match_oracle_and_reduce_loss(lib_built):
    import spray_gb300 as sg
    boxes = grid_boxes()
    rng = np.random.default_rng(4)
    s = make_samples(4096, 4, labelled=1.0)
    # a learnable rule: the candidate whose box centre is nearest the origin
    c = boxes[s["cand"].astype(np.int64)][:, :, :3] + 0.5
    dist = np.linalg.norm(c - s["org"][:, None, :], axis=2)
    dist[np.arange(8)[None, :] >= s["ncand"][:, None]] = np.inf
    s["label"] = np.where(s["ncand"] > 0, np.argmin(dist, axis=1), -1)
    p = om.init_params(9)
    dp, db, ds = dev(p), dev(boxes), dev(s)
    m = torch.zeros(om.PARAMS, dtype=torch.float32, device="cuda")
    v = torch.zeros_like(m)
    losses = torch.zeros(300, dtype=torch.float32, device="cuda")
    # first step against the oracle: Adam on the oracle's gradient
    sg.mlp_train(ptr(dp), ptr(m), ptr(v), ptr(db), NORM, ptr(ds), len(s), 1024, 1e-3, 1, 1, ptr(losses))
    p1 = dp.cpu().numpy().view(np.float32)
    g0, _, cnt = om.grad(p, s[:1024], boxes, NORM)
    want = om.adam(p.copy(), np.zeros_like(p), np.zeros_like(p), (g0 / 1.0).astype(np.float32), 1e-3, 1)
    moved = np.abs(want - p) > 0
    # Adam's first step is lr * sign(g) wherever the gradient is clearly nonzero
    big = np.abs(g0) > 1e-4 * np.abs(g0).max()
    assert np.mean(np.sign(p1 - p)[big] == np.sign(want - p)[big]) > 0.98
    assert not np.any((p1 != p)[~moved & (g0 == 0)])
    sg.mlp_train(ptr(dp), ptr(m), ptr(v), ptr(db), NORM, ptr(ds), len(s), 1024, 1e-3, 300, 2, ptr(losses))
    L = losses.cpu().numpy()
    assert L[-20:].mean() < 0.6 * L[:20].mean(), (L[:5], L[-5:])
    acc = (om.predict(dp.cpu().numpy().view(np.float32), s, boxes, NORM) == s["label"]).mean()
    assert acc > 0.6
