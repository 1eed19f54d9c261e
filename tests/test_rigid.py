"""Rigid voxel bodies on CPU: the host helpers (tree registration, instance packing) and the oracle's
restatement of trace_rigid_bodies (traversal64.wgsl:1006-1244) against the body's dense volume.

Every body hit must name a solid voxel of the body's volume with that voxel's material, its point
must lie on that voxel's face in body-local space, and a ray stopped short of the hit must miss."""
import numpy as np

from arcadia_gb300 import layout as L
from arcadia_gb300 import rigid

DIMS = (24, 16, 20)  # body box in voxels (x, y, z)


def body_volume():
    """(z, y, x) u8 volume of the test body: a stone block (material 5) with a chequer of pillars on
    top (cells removed where y >= 12), a mirror layer (material 28) at y = 11 for x < 8 and a
    grass-coloured layer (material 9) at y = 0."""
    vol = np.zeros((256, 256, 256), np.uint8)
    sub = vol[: DIMS[2], : DIMS[1], : DIMS[0]]
    sub[...] = 5
    zz, yy, xx = np.meshgrid(np.arange(DIMS[2]), np.arange(DIMS[1]), np.arange(DIMS[0]), indexing="ij")
    sub[(yy >= 12) & (((xx // 3) + (zz // 3)) % 2 == 0)] = 0
    sub[:, 11, :8] = 28
    sub[:, 0, :] = 9
    return vol


def world_with_bodies(orc, world, n=3, seed=11, eye=(8.0, 13.75, 8.0)):
    """The world's pools with the test body's tree registered once and n instances of it placed in
    front of the benchmark camera of the 256^3 world, each moving and turning a little per frame."""
    nodes_t, bricks_t = orc.build_chunk_dense(body_volume(), world.palette)
    nodes, bricks, root = rigid.register_dynamic_tree(world.nodes, world.bricks, nodes_t, bricks_t)
    rng = np.random.default_rng(seed)
    com = np.array(DIMS, np.float64) * (0.5 * rigid.VOXEL_SIZE)
    bodies = []
    for i in range(n):
        pos = np.array(eye) + np.array([-2.0 + 2.0 * i, -2.2 - 0.4 * i, -4.5 - 1.5 * i]) + rng.uniform(-0.3, 0.3, 3)
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        ang = rng.uniform(0.2, 1.2)
        q = np.concatenate([axis * np.sin(ang / 2), [np.cos(ang / 2)]])
        pq = np.concatenate([axis * np.sin((ang - 0.05) / 2), [np.cos((ang - 0.05) / 2)]])
        bodies.append(rigid.body_instance(pos, q, com, DIMS, root, prev_position=pos - np.array([0.03, 0.0, 0.02]),
                                          prev_orientation=pq))
    bodies = np.concatenate(bodies)
    return orc.World(world.grid, world.roots, nodes, bricks, world.palette, bodies), root


def test_register_dynamic_tree_relocates():
    base_nodes = np.zeros(5, L.NODE_DTYPE)
    base_bricks = np.zeros(3, L.BRICK_DTYPE)
    t = np.zeros(3, L.NODE_DTYPE)
    t[0] = (1, 0, 1, 0)                          # internal, children at local 1
    t[1] = (3, 0, rigid.IS_LEAF | 0, 7)          # leaf with brick 0
    t[2] = (0, 0, 0, 0)                          # empty
    nodes, bricks, root = rigid.register_dynamic_tree(base_nodes, base_bricks, t, np.zeros(1, L.BRICK_DTYPE))
    assert root == 5 and len(nodes) == 8 and len(bricks) == 4
    assert nodes[5]["child_ptr"] == 6 and nodes[6]["child_ptr"] == (rigid.IS_LEAF | 3) and nodes[7]["child_ptr"] == 0


def test_body_instance_round_trip():
    q = np.array([0.2, 0.5, -0.1, 0.0])
    q[3] = np.sqrt(1 - (q[:3] ** 2).sum())
    rec = rigid.body_instance([1.0, 2.0, 3.0], q, [0.5, 0.25, 0.6], DIMS, 42)[0]
    l2w = rec["local_to_world"].reshape(4, 4).T.astype(np.float64)
    w2l = rec["world_to_local"].reshape(4, 4).T.astype(np.float64)
    assert np.allclose(l2w @ w2l, np.eye(4), atol=1e-5)
    assert rec["local_bounds_and_root"][3:].view(np.uint32)[0] == 42
    # the centre of mass maps to the body's position
    assert np.allclose((l2w @ np.array([0.5, 0.25, 0.6, 1.0]))[:3], [1.0, 2.0, 3.0], atol=1e-5)


def test_oracle_rigid_march_hits_solid_voxels(orc, world_cache):
    w, _ = world_with_bodies(orc, world_cache("c1_256"))
    cam = L.default_camera_for(L.SCENES["c1_256"], 64, 36, quality=L.quality_high())
    cam[0]["point_light_count"][1] = len(w.bodies) << 16
    vol = body_volume()
    rng = np.random.default_rng(2)
    rays = np.zeros(6000, L.RAY_DTYPE)
    for i in range(len(rays)):
        b = w.bodies[i % len(w.bodies)]
        l2w = b["local_to_world"].reshape(4, 4).T.astype(np.float64)
        target = (l2w @ np.append(rng.uniform(0, 1, 3) * np.array(DIMS) * 0.0625, 1.0))[:3]
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        rays[i]["origin_m"] = target - d * 3.0
        rays[i]["dir"] = d
    hits, det = orc.trace_rigid_rays(w, cam, rays, 20.0, threads=4)
    hit = (hits["flags"] & 1).astype(bool)
    assert 0.3 < hit.mean() < 1.0
    assert np.all((hits["flags"][hit] & 0x10) != 0)  # ARC_HIT_FLAG_RIGID
    v = hits["voxel"][hit]
    assert np.all(vol[v[:, 2], v[:, 1], v[:, 0]] == hits["mat"][hit])
    # the hit point, taken back to body-local voxels, lies on the hit voxel's boundary
    body = (hits["flags"][hit] >> 8) & 31
    ok = 0
    for bi, vv, p in zip(body, v, det[hit, :3]):
        w2l = w.bodies[bi]["world_to_local"].reshape(4, 4).T.astype(np.float64)
        lp = (w2l @ np.append(p.astype(np.float64), 1.0))[:3] * 16.0
        ok += bool(np.all(lp >= vv - 1e-3) and np.all(lp <= vv + 1 + 1e-3))
    assert ok >= 0.99 * hit.sum()
    # stopped short of the hit: no hit
    short = np.minimum(hits["depth_m"][hit] - 0.01, 20.0)
    idx = np.nonzero(hit)[0][:500]
    h2 = [orc.trace_rigid_rays(w, cam, rays[i:i + 1], float(s), threads=1)[0] for i, s in zip(idx, short[:500])]
    assert not any(int(h["flags"][0]) & 1 for h in h2)
