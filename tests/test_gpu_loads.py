"""Out-of-core domain loads of the CUDA tracer against the oracle.

Every frame the tracer logs each domain it asks its device cache for (domain,
hit or miss, the domain a miss evicted, the pass).  These requests, replayed
through the oracle's LruCache -- which equals the reference's compiled
lru_cache.cc (tests/test_reference_vectors.py) -- give the same hits, the
same evictions and hence the same number of loads (LruCache::load,
src/render/lru_cache.cc:65-171, called from the round loop,
src/ooc/ooc_pcontext.h:147-153).  Under the plain policy the requests of
every pass follow the DomainStats order of the depth (scores and order are
bit-exact against the oracle, ooc_domain_stats.cc:60-111), restricted to the
domains that hold queue entries.  The cache persists across frames, so the
replay runs over consecutive frames.

The totals are not compared with the oracle's speculative loop (mode A): the
GPU traces a depth's radiance and shadow queues in separate passes over the
domains and loads every domain holding entries, while the reference visits
each domain once per round for both queue sets and skips domains whose
entries its speculative filters dropped, so the two loops request different
sequences by construction.
"""
import numpy as np
import pytest

import spray_gb300 as sg
from spray_gb300 import scenes
from conftest import small_config

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid():
    return scenes.wavelet_grid(4, 24, colors="albedo", light="quad")


@pytest.mark.parametrize("policy,extra", [(0, {}), (1, {}), (2, dict(ooc_inplace=0)), (2, {}),
                                          (3, dict(learn_frames=1)), (4, dict(ooc_inplace=0))])
def test_domain_requests_replay_through_the_reference_lru(lib_built, oracle_mod, grid, policy, extra):
    cache = 12
    cfg = small_config(image_w=160, image_h=120, ao_mode=0, pixel_samples=2, bounces=3, rr_depth=3,
                       cache_size=cache, schedule_policy=policy, **extra)
    t = sg.Tracer(cfg)
    t.set_scene(grid)
    t.set_camera(*scenes.orbit_camera(grid))
    reqs, loads, inplace = [], 0, 0
    for frame in range(3):
        _, st = t.trace()
        log = t.debug(sg.DBG_LOADS, 0)
        cached = log[log["outcome"] != 2]  # traced in place: the cache is not asked
        assert st["domain_loads"] == int(np.sum(cached["outcome"] == 0)), frame
        assert st["inplace_domains"] == int(np.sum(log["outcome"] == 2))
        reqs.append(cached)
        loads += st["domain_loads"]
        inplace += st["inplace_domains"]
    allr = np.concatenate(reqs)
    if extra.get("ooc_inplace", 1) != 0 and policy in (2, 3):
        # with in-place tracing this small frame may never ask the cache
        assert len(allr) + inplace > 0
        if len(allr) == 0:
            return
    else:
        assert len(allr) > 0 and loads > 0 and inplace == 0
    hits, evicted = oracle_mod.lru_trace(len(grid.domains), cache, allr["domain"], with_evicted=True)
    assert np.array_equal(hits.astype(np.int32), allr["outcome"])
    assert np.array_equal(evicted, allr["evicted"])
    t.close()


def test_plain_policy_requests_domains_in_score_order(lib_built, oracle_mod, grid):
    # with the stage buffers kept, the first wave's per-depth DomainStats
    # order is available; every pass of depth b asks for a subsequence of it
    cfg = small_config(image_w=96, image_h=64, ao_mode=0, pixel_samples=2, bounces=3, rr_depth=3,
                       cache_size=12, schedule_policy=0, debug_capture=1, max_samples_per_rank=1 << 20)
    t = sg.Tracer(cfg)
    t.set_scene(grid)
    t.set_camera(*scenes.orbit_camera(grid))
    t.trace()
    log = t.debug(sg.DBG_LOADS, 0)
    passes = sorted(set(log["pass"].tolist()))
    assert len(passes) >= 2
    checked = 0
    for b in range(cfg["bounces"]):
        try:
            sc = t.debug(sg.DBG_SCORES, b)
        except sg.SprayError:
            break
        if len(sc) == 0:
            break
        rank = np.empty(len(sc), np.int64)
        rank[sc["domain"]] = sc["order"]
        # radiance pass 2b + 1 and shadow pass 2b + 2 of the depth
        for p in (2 * b + 1, 2 * b + 2):
            seq = log["domain"][log["pass"] == p]
            if len(seq) == 0:
                continue
            assert np.all(np.diff(rank[seq]) > 0), (b, p)
            checked += 1
    assert checked >= 2
