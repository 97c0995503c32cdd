"""Domain-parallel (in-situ) execution: SpRay's domain partition and the
per-depth reductions that join the ranks (src/render/data_partition.h:60-137,
src/insitu/insitu_vbuf.h:109-129).

CPU: the product's partition equals the oracle's restatement; the reduction
callbacks (unsigned 64-bit minimum, byte maximum) give the element-wise
results across three gloo ranks.  GPU: two and three ranks, each a process
with its own tracer on the one GPU holding and traversing only its domains,
joined by those gloo reductions on the host, each end with the single-rank
image bit for bit.  The ranks' kernels never wait on each other (the only
exchange is the host-side gloo call between stages).  Unmeasured on several
GPUs: every run here has one.
"""
import os

import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config
from oracle import partition as P

SIGN = np.int64(-2 ** 63)


def gloo_reductions(dist, torch):
    """min_u64 / max_u8 callbacks over a gloo group (host buffers)."""
    def min_u64(a):
        # unsigned order of the keys = signed order with the top bit flipped
        t = torch.from_numpy(a.view(np.int64) ^ SIGN)
        dist.all_reduce(t, op=dist.ReduceOp.MIN)
        a.view(np.int64)[:] = t.numpy() ^ SIGN

    def max_u8(a):
        t = torch.from_numpy(a.astype(np.int32))
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        a[:] = t.numpy().astype(np.uint8)
    return min_u64, max_u8


@pytest.mark.parametrize("grid,samples,seed", [(4, 16, None), (8, 12, 3), (3, 10, None)])
def test_partition_matches_the_oracle(lib_built, grid, samples, seed):
    sc = scenes.wavelet_grid(grid, samples, phase_seed=seed)
    b = np.stack([d.bounds for d in sc.domains])
    for ranks in range(1, 8):
        got = sg.insitu_partition(b, ranks)
        want = P.insitu_partition(b, ranks)
        assert np.array_equal(got, want), ranks
        counts = np.bincount(got, minlength=ranks)
        shares = len(b) // ranks
        assert counts.min() >= shares and counts.sum() == len(b)


def test_partition_of_random_boxes(lib_built):
    rng = np.random.default_rng(5)
    lo = rng.uniform(-10, 10, (37, 3)).astype(np.float32)
    b = np.concatenate([lo, lo + rng.uniform(0.1, 3, (37, 3)).astype(np.float32)], 1)
    for ranks in (1, 2, 5, 36, 40):
        assert np.array_equal(sg.insitu_partition(b, ranks), P.insitu_partition(b, ranks))


def _reduce_rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mn, mx = gloo_reductions(dist, torch)
    rng = np.random.default_rng(rank)
    keys = rng.integers(0, 2 ** 64 - 1, 1000, dtype=np.uint64, endpoint=True)
    keys[rank::world] = np.uint64(2 ** 64 - 1)  # misses on this rank
    b = rng.integers(0, 256, 1000).astype(np.uint8)
    k0, b0 = keys.copy(), b.copy()
    mn(keys)
    mx(b)
    q.put((rank, k0, b0, keys, b))
    dist.barrier()
    dist.destroy_process_group()


def test_reduction_callbacks_on_cpu_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 3, 29900 + os.getpid() % 1000
    procs = [ctx.Process(target=_reduce_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(world)], key=lambda x: x[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    kmin = np.minimum.reduce([r[1] for r in res])
    bmax = np.maximum.reduce([r[2] for r in res])
    for _, _, _, k, b in res:
        assert np.array_equal(k, kmin) and np.array_equal(b, bmax)


def _render(cfg, scene):
    t = sg.Tracer(cfg)
    t.set_scene(scene)
    t.set_camera(*scenes.orbit_camera(scene))
    img, st = t.trace()
    return t, img, st


CASES = {"pt": dict(image_w=64, image_h=48, ao_mode=0, ao_samples=2, pixel_samples=2, bounces=3),
         "ao": dict(image_w=64, image_h=48, ao_mode=1, ao_samples=4, pixel_samples=2, bounces=2)}


def _insitu_rank(rank, world, port, q, case):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mn, mx = gloo_reductions(dist, torch)
    sc = scenes.wavelet_grid(4, 16, colors="albedo", light="point+diffuse")
    t = sg.Tracer(small_config(**CASES[case]))
    t.set_insitu(world, rank, mn, mx)
    t.set_scene(sc)
    t.set_camera(*scenes.orbit_camera(sc))
    img, st = t.trace()
    img2, _ = t.trace()  # a second frame reuses the buffers
    q.put((rank, img, img2, st))
    t.close()
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.gpu
@pytest.mark.parametrize("world,case", [(2, "pt"), (3, "pt"), (2, "ao")])
def test_domain_parallel_ranks_render_the_single_rank_image(lib_built, world, case):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29950 + (os.getpid() + world * 7) % 1000
    procs = [ctx.Process(target=_insitu_rank, args=(r, world, port, q, case)) for r in range(world)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=600) for _ in range(world)], key=lambda x: x[0])
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sc = scenes.wavelet_grid(4, 16, colors="albedo", light="point+diffuse")
    _, want, st1 = _render(small_config(**CASES[case]), sc)
    bits = lambda a: np.ascontiguousarray(a, np.float32).view(np.uint32)
    owned = np.bincount(sg.insitu_partition(np.stack([d.bounds for d in sc.domains]), world))
    for rank, img, img2, st in res:
        assert np.array_equal(bits(img), bits(want)), (rank, float(np.abs(img - want).max()))
        assert np.array_equal(bits(img2), bits(want))
        assert st["exchange_bytes"] > 0 and st["rays_primary"] == st1["rays_primary"]
        # each rank holds only its own domains' triangles
        assert 0 < st["scene_triangles"] < st1["scene_triangles"]
        assert st["rays_shadow"] == st1["rays_shadow"] and st["rays_bounce"] == st1["rays_bounce"]
    assert sum(r[3]["scene_triangles"] for r in res) == st1["scene_triangles"]
    assert len(owned) == world and owned.min() > 0
    assert want[..., :3].max() > 0
