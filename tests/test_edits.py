"""In-place edits in the oracle (CPU): the sequential restatement of the reference edit path
(crates/arcadia-core/src/chunk_tree/edit/carve.rs:39-176, set.rs:244-618) checked against a dense
expectation computed independently in numpy, and against a fresh build of the edited volume."""
import numpy as np
import pytest

from arcadia_gb300.layout import EDIT_CARVE, EDIT_DTYPE, EDIT_RECOLOR, SCENES, SceneParams


def surface_points(vol, rng, n):
    """(x, y, z) of the top solid voxel of n random columns of a dense (z, y, x) chunk volume."""
    pts = []
    while len(pts) < n:
        x, z = rng.integers(0, 256, 2)
        col = np.nonzero(vol[z, :, x])[0]
        if len(col):
            pts.append((int(x), int(col[-1]), int(z)))
    return pts


def make_ops(vol, rng, n, origin=(0, 0, 0)):
    ops = np.zeros(n, EDIT_DTYPE)
    for i, (x, y, z) in enumerate(surface_points(vol, rng, n)):
        x, y, z = x + origin[0], y + origin[1], z + origin[2]
        if i % 3 == 2:
            ops[i]["kind"] = EDIT_RECOLOR
            ops[i]["brick"] = (x >> 2, y >> 2, z >> 2)
            ops[i]["material"] = int(rng.integers(1, 17))
        else:
            ops[i]["kind"] = EDIT_CARVE
            ops[i]["center"] = np.array([x, y, z], np.float32) + rng.random(3).astype(np.float32)
            ops[i]["radius"] = np.float32(rng.uniform(2.0, 16.0))
    return ops


def expected_volume(vol, ops, origin=(0, 0, 0)):
    """Dense result of the edits on one chunk: carve clears solid voxels whose centre is within r
    (f32 ((dx*dx + dy*dy) + dz*dz)); recolour sets the solid voxels of a brick."""
    out = vol.copy()
    z, y, x = np.meshgrid(np.arange(256), np.arange(256), np.arange(256), indexing="ij")
    for op in ops:
        if op["kind"] == EDIT_CARVE:
            c = op["center"].astype(np.float32) - np.array(origin, np.float32)
            r = np.float32(op["radius"])
            lo = np.maximum(np.floor(c - r).astype(int) - 1, 0)
            hi = np.minimum(np.ceil(c + r).astype(int) + 2, 256)
            sl = (slice(lo[2], hi[2]), slice(lo[1], hi[1]), slice(lo[0], hi[0]))
            dx = c[0] - (x[sl].astype(np.float32) + np.float32(0.5))
            dy = c[1] - (y[sl].astype(np.float32) + np.float32(0.5))
            dz = c[2] - (z[sl].astype(np.float32) + np.float32(0.5))
            inside = ((dx * dx + dy * dy) + dz * dz) <= r * r
            out[sl][inside] = 0
        else:
            b = op["brick"].astype(int) - np.array(origin) // 4
            if np.any(b < 0) or np.any(b >= 64):
                continue
            blk = out[b[2] * 4:b[2] * 4 + 4, b[1] * 4:b[1] * 4 + 4, b[0] * 4:b[0] * 4 + 4]
            blk[blk != 0] = op["material"]
    return out


@pytest.mark.parametrize("scene", ["c1_256", "caves256"])
def test_oracle_edits_match_dense_expectation(orc, scene):
    s = SCENES["c1_256"] if scene == "c1_256" else SceneParams(grid=(1, 1, 1), seed=21, caves=True)
    w = orc.build_world(s)
    vol = orc.scene_volume(s)
    rng = np.random.default_rng(7)
    ops = make_ops(vol, rng, 40)
    e = orc.apply_edits(w, ops)
    got = orc.chunk_volume(e.grid, e.roots, e.nodes, e.bricks, (0, 0, 0))
    want = expected_volume(vol, ops)
    assert np.array_equal(got, want), int((got != want).sum())
    assert (want != vol).sum() > 1000  # the edits changed something
    assert len(e.nodes) > len(w.nodes)  # uncollapsed branches appended


def test_oracle_edited_tree_equals_fresh_build(orc):
    """The edited tree, node by node in child order, equals ChunkTree64::from_generator over the edited
    volume: masks, LOD payloads and voxel materials. The reference never turns a brick leaf whose
    remaining voxels share one material back into a uniform leaf (a fresh build does), so the leaf
    form is not compared."""
    s = SCENES["c1_256"]
    w = orc.build_world(s)
    vol = orc.scene_volume(s)
    ops = make_ops(vol, np.random.default_rng(8), 30)
    ops = ops[ops["kind"] == EDIT_CARVE]
    e = orc.apply_edits(w, ops)
    fresh_nodes, fresh_bricks = orc.build_chunk_dense(expected_volume(vol, ops))
    f = orc.world_from_chunk(fresh_nodes, fresh_bricks)
    assert orc.tree_compare(e.roots[0], e.nodes, e.bricks, f.roots[0], f.nodes, f.bricks, leaf_form=False) == 0
    assert orc.tree_compare(e.roots[0], e.nodes, e.bricks, f.roots[0], f.nodes, f.bricks) != 0  # kept bricks


def test_oracle_edits_across_chunks(orc):
    """A sphere on a chunk boundary carves both chunks (per-chunk local centres)."""
    s = SceneParams(grid=(2, 1, 1), seed=3, caves=False)
    w = orc.build_world(s)
    vols = [orc.scene_volume(s, (cx, 0, 0)) for cx in range(2)]
    col = np.nonzero(vols[0][100, :, 255])[0]
    y = int(col[-1])
    ops = np.zeros(1, EDIT_DTYPE)
    ops[0]["kind"] = EDIT_CARVE
    ops[0]["center"] = (256.25, y + 0.5, 100.5)
    ops[0]["radius"] = 9.0
    e = orc.apply_edits(w, ops)
    for cx in range(2):
        got = orc.chunk_volume(e.grid, e.roots, e.nodes, e.bricks, (cx, 0, 0))
        want = expected_volume(vols[cx], ops, origin=(256 * cx, 0, 0))
        assert np.array_equal(got, want)
        assert (want != vols[cx]).any()
