"""Rigid voxel bodies on the host: putting a body's 64-tree into the world pools and packing its
GpuRigidBodyInstance record (layout.RIGID_BODY_DTYPE) for ``arc_set_rigid_bodies``.

``register_dynamic_tree`` follows WorldMap::register_dynamic_tree (crates/arcadia-world/src/world_map.rs:
623-703) with relocate_chunk_nodes (705-735), appending instead of reusing free spans: the tree's
nodes and bricks go to the end of the pools, child pointers of internal nodes move by the node base,
brick pointers of non-uniform leaves by the brick base, empty nodes stay empty; the body's root is
its tree's first node.

``body_instance`` follows RigidVoxelBody::to_gpu_instance (crates/arcadia-physics/src/rigid_voxel/
transform.rs:80-111): local -> world = T(x_com) R(q) T(-c_local) (body-local meters in
[0, dims_v / 16]), its inverse, the previous frame's local -> world, the local box with the root
index's bit pattern, and the bounding sphere at x_com + R (half_extents - c_local) with radius
|half_extents| + 1/16 m.
"""
from __future__ import annotations

import numpy as np

from . import layout as L

VOXEL_SIZE = 0.0625
IS_LEAF = 0x80000000
IS_UNIFORM = 0x40000000
PTR_MASK = 0x3FFFFFFF


def register_dynamic_tree(nodes: np.ndarray, bricks: np.ndarray, tree_nodes: np.ndarray, tree_bricks: np.ndarray):
    """Pools with the tree appended, and the body's root node index."""
    tn = np.ascontiguousarray(tree_nodes).view(L.NODE_DTYPE).copy()
    node_base, brick_base = len(nodes), len(bricks)
    empty = (tn["mask_low"] == 0) & (tn["mask_high"] == 0)
    ptr = tn["child_ptr"].astype(np.uint64)
    flags = ptr & (IS_LEAF | IS_UNIFORM)
    local = ptr & PTR_MASK
    leaf = (ptr & IS_LEAF) != 0
    uniform = (ptr & IS_UNIFORM) != 0
    new = np.where(leaf, np.where(uniform, flags, flags | (brick_base + local)), flags | (node_base + local))
    tn["child_ptr"] = new.astype(np.uint32)
    tn[empty] = np.zeros(1, L.NODE_DTYPE)
    out_nodes = np.concatenate([np.ascontiguousarray(nodes).view(L.NODE_DTYPE), tn])
    out_bricks = np.concatenate([np.ascontiguousarray(bricks).view(L.BRICK_DTYPE),
                                 np.ascontiguousarray(tree_bricks).view(L.BRICK_DTYPE)])
    return out_nodes, out_bricks, node_base


def quat_matrix(q) -> np.ndarray:
    """3x3 rotation of a unit quaternion (x, y, z, w)."""
    x, y, z, w = (float(v) for v in q)
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def _local_to_world(position, q, com_local_m) -> np.ndarray:
    r = quat_matrix(q)
    m = np.eye(4)
    m[:3, :3] = r
    m[:3, 3] = np.asarray(position, np.float64) - r @ np.asarray(com_local_m, np.float64)
    return m


def body_instance(position, orientation, com_local_m, dims_v, root: int, prev_position=None, prev_orientation=None):
    """One RIGID_BODY_DTYPE record (column-major matrices)."""
    l2w = _local_to_world(position, orientation, com_local_m)
    w2l = np.linalg.inv(l2w)
    pl2w = _local_to_world(position if prev_position is None else prev_position,
                           orientation if prev_orientation is None else prev_orientation, com_local_m)
    dims = np.asarray(dims_v, np.float64)
    half = dims * (0.5 * VOXEL_SIZE)
    centre = np.asarray(position, np.float64) + quat_matrix(orientation) @ (half - np.asarray(com_local_m, np.float64))
    rec = np.zeros(1, L.RIGID_BODY_DTYPE)
    rec["world_to_local"][0] = w2l.T.reshape(16)
    rec["local_to_world"][0] = l2w.T.reshape(16)
    rec["prev_local_to_world"][0] = pl2w.T.reshape(16)
    rec["local_bounds_and_root"][0, :3] = dims * VOXEL_SIZE
    rec["local_bounds_and_root"][0, 3] = np.array([root], np.uint32).view(np.float32)[0]
    rec["world_sphere"][0] = [centre[0], centre[1], centre[2], np.linalg.norm(half) + VOXEL_SIZE]
    return rec
