"""The full per-frame pipeline (edits -> trace -> GI points -> NRC) on a small editable world: it runs,
rewrites bricks every frame, and the world it leaves equals the oracle replaying the same edit
batches (trees node for node, a frame bit-exact)."""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8


def test_pipeline_frames_and_replay(orc, native_lib):
    from arcadia_gb300.pipeline import FullPipeline, path_camera

    scene = L.SCENES["band512"]
    ow = orc.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(ow.grid, ow.roots, ow.nodes, ow.bricks, ow.palette, node_headroom=1 << 20, brick_headroom=1 << 17)
        p = FullPipeline(t, scene, 320, 180, n_bricks=len(ow.bricks), n_frames=8, edit_fraction=0.01, keep_ops=True)
        s = p.run(warmup=1)
        assert s["frames"] == 8 and s["overflow"] == 0 and s["device_status"] == 0
        assert s["bricks_rewritten_per_frame"] > 0 and s["gi_hits_per_frame"] > 100
        assert all(r["ops"] > 0 for r in p.records[1:])
        for ops in p.ops_log:
            ow = orc.apply_edits(ow, ops)
        roots, nodes, bricks = t.download_world()
        for i, r in enumerate(ow.roots):
            assert orc.tree_compare(r, ow.nodes, ow.bricks, roots[i], nodes, bricks) == 0, i
        cam = path_camera(scene, 320, 180, 7, 8, L.quality_high())
        t.set_camera(cam)
        gdm, gnm, gaa, hits, gi, _ = t.trace_frame()
        ogdm, ognm, ogaa, ohits, _ = orc.primary(ow, cam, threads=THREADS)
        np.testing.assert_array_equal(gdm, ogdm)
        assert hits.tobytes() == ohits.tobytes()
        out = p.nrc_out.cpu().numpy()[p.valid.cpu().numpy().astype(bool)]
        assert np.isfinite(out).all()
    finally:
        t.close()
