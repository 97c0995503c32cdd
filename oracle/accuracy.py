"""Accuracy measures of a GPU frame against the oracle.

TEST INFRASTRUCTURE ONLY (tests/ and bench.py's accuracy report).  The
tolerances are the ones the tracer is held to:

  hits            >= 99.99 % of rays agree on hit or miss, domain and
                  primitive; hit t within 1e-5 relative where they agree
  occlusion       >= 99.99 % of AO/shadow rays agree on occluded or not
  image           RMSE <= 1e-3 over the RGB channels of radiance clipped to
                  [0, 1] (the displayable range)

Every function takes plain numpy arrays (the GPU side comes from the
library's debug hooks), so this module never loads the CUDA library.
"""
from __future__ import annotations

import numpy as np

HIT_AGREE = 0.9999
T_RTOL = 1e-5
IMG_RMSE = 1e-3


def image_rmse(a: np.ndarray, b: np.ndarray, clip: bool = True) -> float:
    """RMSE over the RGB channels of two (H, W, 4) radiance images."""
    x = np.asarray(a, np.float64)[..., :3]
    y = np.asarray(b, np.float64)[..., :3]
    if clip:
        x, y = np.clip(x, 0.0, 1.0), np.clip(y, 0.0, 1.0)
    return float(np.sqrt(np.mean((x - y) ** 2)))


def bit_exact(a: np.ndarray, b: np.ndarray) -> bool:
    return np.array_equal(np.ascontiguousarray(a, np.float32).view(np.uint32),
                          np.ascontiguousarray(b, np.float32).view(np.uint32))


def hit_agreement(rays: np.ndarray, hits: np.ndarray, oracle) -> dict:
    """GPU closest hits of one depth's rays (debug records) against the
    oracle's closest hit of the same rays."""
    n = len(rays)
    if n == 0:
        return {"rays": 0, "agree": 1.0, "t_max_rel_err": 0.0, "t_bit_exact": 1.0}
    oh = oracle.closest(rays["org"], rays["dir"])
    same = (hits["hit"] == oh["hit"]) & (hits["domain"] == oh["domain"]) & (hits["prim"] == oh["prim"])
    both = same & (hits["hit"] == 1)
    t0 = hits["t"][both].astype(np.float64)
    t1 = oh["t"][both].astype(np.float64)
    rel = np.abs(t0 - t1) / np.maximum(np.abs(t1), 1e-30)
    return {"rays": int(n), "agree": float(same.mean()),
            "t_max_rel_err": float(rel.max()) if len(rel) else 0.0,
            "t_bit_exact": float(np.mean(hits["t"][both].view(np.uint32) == oh["t"][both].view(np.uint32)))
            if both.any() else 1.0,
            "hits": int(both.sum())}


def shadow_agreement(shadows: np.ndarray, hits: np.ndarray, oracle) -> dict:
    """GPU occlusion flags of one depth's shadow rays against the oracle's.
    The shadow ray's origin domain is the domain of its parent's hit."""
    if len(shadows) == 0:
        return {"rays": 0, "agree": 1.0}
    order = np.argsort(hits["sample"], kind="stable")
    pos = np.searchsorted(hits["sample"][order], shadows["sample"])
    origin = hits["domain"][order][pos].astype(np.int32)
    occ = oracle.occluded(shadows["org"], shadows["dir"], shadows["tmax"], origin)
    agree = occ.astype(np.int64) == shadows["occluded"].astype(np.int64)
    return {"rays": int(len(shadows)), "agree": float(agree.mean()),
            "occluded": float(np.mean(occ != 0))}


def frame_report(gpu_img: np.ndarray, mode_a_img: np.ndarray, mode_b_img: np.ndarray | None,
                 hits_by_depth: dict, shadows_by_depth: dict) -> dict:
    """One dictionary for the bench line: image RMSE against the reference
    loop restated (mode A) and the wavefront restatement (mode B), and hit
    and occlusion agreement per depth."""
    out = {"image_rmse_vs_oracle": image_rmse(gpu_img, mode_a_img),
           "image_rmse_unclipped": image_rmse(gpu_img, mode_a_img, clip=False),
           "image_rmse_tolerance": IMG_RMSE}
    if mode_b_img is not None:
        out["bit_exact_vs_wavefront_oracle"] = bit_exact(gpu_img, mode_b_img)
        out["max_abs_diff_vs_wavefront_oracle"] = float(np.abs(np.asarray(gpu_img, np.float64)
                                                               - np.asarray(mode_b_img, np.float64)).max())
    rays = sum(h["rays"] for h in hits_by_depth.values())
    agree = sum(h["agree"] * h["rays"] for h in hits_by_depth.values())
    out["hit_agreement"] = agree / rays if rays else 1.0
    out["hit_agreement_by_depth"] = hits_by_depth
    srays = sum(s["rays"] for s in shadows_by_depth.values())
    sagree = sum(s["agree"] * s["rays"] for s in shadows_by_depth.values())
    out["shadow_agreement"] = sagree / srays if srays else 1.0
    out["shadow_agreement_by_depth"] = shadows_by_depth
    out["t_max_rel_err"] = max([h["t_max_rel_err"] for h in hits_by_depth.values()] + [0.0])
    return out
