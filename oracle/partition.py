"""SpRay's in-situ domain partition, restated in numpy.

TEST INFRASTRUCTURE ONLY (the checker of the product's partition in
spray_gb300/csrc/insitu.cu).  InsituPartition::partition
(src/render/data_partition.h:60-137) with Morton::compute
(src/render/morton.h:33-52), in float32 and the reference's operation order:

  scene box = union of the domains' world boxes
  scale = 1 / (max - min) per axis, offset = 0 - min * scale
  centre = 0.5 * (lo + hi) per domain, mapped to c = centre * scale + offset
  code = interleave(10-bit x, y, z), each min(max(c * 1024, 0), 1023) truncated
  domains sorted by code, then ndomains / ranks consecutive domains per rank,
  the remainder wrapping to rank 0 onwards

The reference sorts with std::sort (equal codes in no defined order); here
equal codes keep domain order, as in the product.
"""
from __future__ import annotations

import numpy as np

F = np.float32


def _spread(v: np.ndarray) -> np.ndarray:
    """Insert two zero bits after each of the low ten bits (uint32 arithmetic)."""
    v = v.astype(np.uint64)
    m = np.uint64(0xFFFFFFFF)
    v = ((v * np.uint64(0x00010001)) & m) & np.uint64(0xFF0000FF)
    v = ((v * np.uint64(0x00000101)) & m) & np.uint64(0x0F00F00F)
    v = ((v * np.uint64(0x00000011)) & m) & np.uint64(0xC30C30C3)
    v = ((v * np.uint64(0x00000005)) & m) & np.uint64(0x49249249)
    return v


def morton(c: np.ndarray) -> np.ndarray:
    q = np.minimum(np.maximum(c.astype(F) * F(1024.0), F(0.0)), F(1023.0)).astype(np.uint32)
    code = _spread(q[:, 0]) * np.uint64(4) + _spread(q[:, 1]) * np.uint64(2) + _spread(q[:, 2])
    return (code & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def insitu_partition(bounds, num_ranks: int) -> np.ndarray:
    b = np.asarray(bounds, F).reshape(-1, 6)
    nd = len(b)
    lo, hi = b[:, :3].min(0), b[:, 3:].max(0)
    scale = (F(1.0) / (hi - lo)).astype(F)
    offset = (F(0.0) - lo * scale).astype(F)
    centre = ((b[:, :3] + b[:, 3:]) * F(0.5)).astype(F)
    c = (centre * scale + offset).astype(F)
    order = np.argsort(morton(c), kind="stable")
    shares = max(nd // num_ranks, 1)
    owner = np.zeros(nd, np.int32)
    rank = s = 0
    for d in order:
        owner[d] = rank
        s += 1
        if s == shares:
            s = 0
            rank += 1
            if rank == num_ranks:
                rank = 0
    return owner
