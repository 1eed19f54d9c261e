"""Seeded in-place edit batches: carved spheres and recoloured bricks at surfaces the camera sees.

An edit lands where a primary ray hit (hit records of the previous frame), the way gameplay edits
land where the player aims. ``batch_from_hits`` turns hit records into ``layout.EDIT_DTYPE`` records:
a fraction ``recolor`` of them recolour the hit voxel's brick to a random material 1..16, the rest
carve a sphere of radius U[r_min, r_max] voxels centred at a random point of the hit voxel.
``ops_for_brick_budget`` sizes a batch so that about a given number of bricks is rewritten.
"""
from __future__ import annotations

import numpy as np

from .layout import EDIT_CARVE, EDIT_DTYPE, EDIT_RECOLOR, HIT_DTYPE


def batch_from_hits(hits: np.ndarray, n_ops: int, rng: np.random.Generator, recolor: float = 0.5, r_min: float = 2.0,
                    r_max: float = 16.0) -> np.ndarray:
    hits = np.ascontiguousarray(hits).view(HIT_DTYPE)
    cand = np.nonzero(hits["flags"] & 1)[0]
    ops = np.zeros(n_ops if len(cand) else 0, EDIT_DTYPE)
    if not len(ops):
        return ops
    pick = cand[rng.integers(0, len(cand), n_ops)]
    vox = hits["voxel"][pick].astype(np.int64)
    is_recolor = rng.random(n_ops) < recolor
    ops["kind"] = np.where(is_recolor, EDIT_RECOLOR, EDIT_CARVE)
    ops["material"] = np.where(is_recolor, rng.integers(1, 17, n_ops), 0)
    ops["brick"] = np.where(is_recolor[:, None], vox >> 2, 0).astype(np.uint32)
    ops["center"] = np.where(is_recolor[:, None], 0.0, vox + rng.random((n_ops, 3))).astype(np.float32)
    ops["radius"] = np.where(is_recolor, 0.0, rng.uniform(r_min, r_max, n_ops)).astype(np.float32)
    return ops


def ops_for_brick_budget(bricks_target: int, bricks_per_op: float) -> int:
    """Number of edits expected to rewrite about `bricks_target` bricks, given the measured mean."""
    return max(1, int(round(bricks_target / max(bricks_per_op, 1e-3))))
