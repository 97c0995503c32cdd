"""Image-space sharding through the CUDA library (the reference's multi-rank
scheme on spray_ooc): rank r renders vertical stripe r of the image
(src/render/tile.cc:214-235, with its blocking tiles, tile.cc:317-391) and
the float4 images are summed to rank 0 (HdrImage::composite,
src/display/image.h:167-181).

Each stripe equals the oracle's render of the same (num_ranks, rank) bit for
bit.  For AO at one sample per pixel no random stream depends on the tiling
(eye rays through pixel corners, AO seeds from the pixel id), so the summed
stripes equal the single-rank image bit for bit as well.  Jitter and
path-tracing seeds follow the tile-local sample numbers, as in the reference
(ooc_tracer.inl:138-152, ooc_shader_pt.h:130,217), so there the stripes and
the whole image differ in their noise only.
"""
import os

import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config
from oracle import accuracy as A

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.wavelet_grid(2, 16, colors="albedo", light="point")


def _gpu(cfg, scene):
    t = sg.Tracer(cfg)
    t.set_scene(scene)
    t.set_camera(*scenes.orbit_camera(scene))
    img, st = t.trace()
    t.close()
    return img, st


@pytest.mark.parametrize("spp,mode", [(1, "ao"), (4, "ao"), (1, "pt"), (4, "pt")])
def test_stripes_match_the_oracle(lib_built, oracle_mod, spp, mode):
    sc = _scene()
    world = 3
    parts = []
    for rank in range(world):
        cfg = small_config(image_w=45, image_h=30, num_ranks=world, rank=rank, pixel_samples=spp,
                           ao_mode=int(mode == "ao"), ao_samples=3, bounces=1 if mode == "ao" else 3,
                           max_samples_per_rank=512)
        img, st = _gpu(cfg, sc)
        o = oracle_mod.Oracle(cfg, sc)
        o.set_camera(*scenes.orbit_camera(sc))
        want, _ = o.render_wavefront()
        assert A.bit_exact(img, want), (rank, float(np.abs(img - want).max()))
        parts.append(img)
    # every pixel belongs to exactly one stripe
    covered = sum((p[..., 3] != 0) | np.any(p[..., :3] != 0, -1) for p in parts)
    assert covered.max() <= 1
    if spp == 1 and mode == "ao":
        single, _ = _gpu(small_config(image_w=45, image_h=30, pixel_samples=1, ao_mode=int(mode == "ao"),
                                      ao_samples=3, bounces=1 if mode == "ao" else 3,
                                      max_samples_per_rank=512), sc)
        assert A.bit_exact(sum(parts), single)


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sc = _scene()
    cfg = small_config(image_w=45, image_h=30, num_ranks=world, rank=rank, ao_samples=3, device=0)
    img, _ = _gpu(cfg, sc)
    t = torch.from_numpy(img.copy())
    dist.reduce(t, dst=0, op=dist.ReduceOp.SUM)
    if rank == 0:
        q.put(t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_compose_the_single_rank_image(lib_built):
    # two processes share the one GPU; their kernels never wait on each other
    # (the only exchange is the host-side gloo reduction of the images)
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29700 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    composed = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    single, _ = _gpu(small_config(image_w=45, image_h=30, ao_samples=3), _scene())
    assert A.bit_exact(composed, single)
    assert single[..., :3].max() > 0
