"""In-place edits on the GPU (arc_apply_edits) against the oracle's sequential restatement of the
reference edit path: the edited trees are equal node for node (masks, flags, LOD payloads, brick
materials; only pool positions differ), and frames traced on the edited worlds are bit-exact."""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L
from arcadia_gb300.layout import EDIT_DTYPE, SceneParams

from test_edits import make_ops

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8


def _ops_for_world(orc, scene, rng, per_chunk):
    """Edits at surface points of every non-empty chunk column (chunk-local surfaces, world coords)."""
    gx, gy, gz = scene.grid
    out = []
    for cz in range(gz):
        for cx in range(gx):
            for cy in range(gy - 1, -1, -1):
                vol = orc.scene_volume(scene, (cx, cy, cz))
                if vol.any():
                    out.append(make_ops(vol, rng, per_chunk, origin=(256 * cx, 256 * cy, 256 * cz)))
                    break
    ops = np.concatenate(out)
    return ops[rng.permutation(len(ops))]


def _compare_trees(orc, ow, roots, nodes, bricks):
    assert np.array_equal(roots, ow.roots)
    for i, r in enumerate(ow.roots):
        pos = orc.tree_compare(r, ow.nodes, ow.bricks, roots[i], nodes, bricks)
        assert pos == 0, f"chunk {i}: first difference at depth-first node {pos}"


@pytest.mark.parametrize("scene_name", ["c1_256", "band512"])
def test_gpu_edit_batches_match_oracle(orc, native_lib, scene_name):
    scene = L.SCENES[scene_name]
    ow = orc.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(ow.grid, ow.roots, ow.nodes, ow.bricks, ow.palette, node_headroom=1 << 20, brick_headroom=1 << 17)
        rng = np.random.default_rng(11)
        total = 0
        for batch in range(3):
            ops = _ops_for_world(orc, scene, rng, 12)
            ow = orc.apply_edits(ow, ops)
            total = t.apply_edits(ops, sync=True)
            roots, nodes, bricks = t.download_world()
            _compare_trees(orc, ow, roots, nodes, bricks)
        assert total > 100
        st = t.edit_stats()
        assert st["overflow"] == 0 and st["next_node"] == len(ow.nodes) and st["next_brick"] == len(ow.bricks)
        # frames on the edited world: G-buffer, hits and GI hits bit-exact against the oracle
        cam = L.default_camera_for(scene, 640, 360, quality=L.quality_parity(512), frame_index=2)
        t.set_camera(cam)
        gdm, gnm, gaa, hits, gi, _ = t.trace_frame()
        ogdm, ognm, ogaa, ohits, _ = orc.primary(ow, cam, threads=THREADS)
        _, ogi, _ = orc.gi_rays(ow, cam, ogdm, ognm, threads=THREADS)
        np.testing.assert_array_equal(gdm, ogdm)
        np.testing.assert_array_equal(gnm, ognm)
        np.testing.assert_array_equal(gaa, ogaa)
        assert hits.tobytes() == ohits.tobytes()
        assert gi.tobytes() == ogi.tobytes()
        assert t.stats().device_status == 0
    finally:
        t.close()


def test_gpu_edit_capacity_and_validation(orc, native_lib):
    from arcadia_gb300.native import ArcError

    scene = L.SCENES["c1_256"]
    ow = orc.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(ow.grid, ow.roots, ow.nodes, ow.bricks, ow.palette)  # no headroom
        bad = np.zeros(1, EDIT_DTYPE)
        for kind, field, value in ((0, "radius", 0.0), (0, "radius", 17.0), (1, "material", 0), (1, "brick", (64, 0, 0)),
                                   (7, "radius", 1.0)):
            bad[:] = 0
            bad[0]["kind"] = kind
            bad[0]["material"] = 3
            bad[0]["radius"] = 4.0
            bad[0][field] = value
            with pytest.raises(ArcError):
                t.apply_edits(bad, sync=True)
        ops = _ops_for_world(orc, scene, np.random.default_rng(5), 20)
        with pytest.raises(ArcError) as e:
            t.apply_edits(ops, sync=True)
        assert "headroom" in str(e.value)
        assert t.edit_stats()["overflow"] != 0
        # the pools stay traversable: a frame runs and no range check fires
        cam = L.default_camera_for(scene, 320, 180, quality=L.quality_parity(512))
        t.set_camera(cam)
        t.trace_frame()
        assert t.stats().device_status == 0
    finally:
        t.close()


def test_gpu_empty_chunks_and_boundary_spheres(orc, native_lib):
    """Spheres reaching into empty chunks (above the terrain) and straddling chunk faces."""
    scene = SceneParams(grid=(2, 2, 1), seed=9, caves=False, height_lo=0.30, height_hi=0.45)
    ow = orc.build_world(scene)
    assert (ow.roots == L.EMPTY_CHUNK).any()
    t = native_lib.Tracer(0)
    try:
        t.upload_world(ow.grid, ow.roots, ow.nodes, ow.bricks, ow.palette, node_headroom=1 << 18, brick_headroom=1 << 15)
        ops = np.zeros(4, EDIT_DTYPE)
        for i, c in enumerate([(255.6, 200.0, 100.0), (256.0, 256.0, 128.0), (100.0, 255.9, 200.0), (10.0, 300.0, 10.0)]):
            ops[i]["kind"] = L.EDIT_CARVE
            ops[i]["center"] = c
            ops[i]["radius"] = 16.0
        ow = orc.apply_edits(ow, ops)
        t.apply_edits(ops, sync=True)
        roots, nodes, bricks = t.download_world()
        _compare_trees(orc, ow, roots, nodes, bricks)
    finally:
        t.close()
