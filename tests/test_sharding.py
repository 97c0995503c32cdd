"""Image-space sharding (the reference's multi-rank scheme): rank r renders
vertical stripe r (src/render/tile.cc:214-235) and the float4 images are
summed to rank 0 (HdrImage::composite, src/display/image.h:167-181).  Two gloo
ranks on CPU, each rendering its stripe with the oracle, must reproduce the
single-rank image."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from spray_gb300 import scenes
from conftest import small_config


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    sc = scenes.wavelet_grid(2, 16, colors="albedo", light="point")
    cfg = small_config(image_w=45, image_h=30, num_ranks=world, rank=rank, ao_samples=3)
    o = O.Oracle(cfg, sc)
    o.set_camera(*scenes.orbit_camera(sc))
    img, _ = o.render_wavefront()
    t = torch.from_numpy(img.copy())
    dist.reduce(t, dst=0, op=dist.ReduceOp.SUM)
    if rank == 0:
        q.put(t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_stripes_compose_to_single_rank_image(oracle_mod):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    composed = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    sc = scenes.wavelet_grid(2, 16, colors="albedo", light="point")
    o = oracle_mod.Oracle(small_config(image_w=45, image_h=30, ao_samples=3), sc)
    o.set_camera(*scenes.orbit_camera(sc))
    single, _ = o.render_wavefront()
    assert np.array_equal(composed.view(np.uint32), single.view(np.uint32))
    assert single[..., :3].max() > 0
