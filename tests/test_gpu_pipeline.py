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


def test_pipeline_4096_matches_oracle(orc, native_lib, world_cache):
    """The 4096^3 world of the full pipeline (16^3 chunks, 16.6M nodes, 1.56M bricks), at a reduced
    960x540 resolution so the oracle replay stays short: 8 pipeline frames (edits rewriting 1 % of the
    bricks per frame, trace, GI points, NRC) on the GPU, then the oracle replays the same edit batches.
    Every chunk's tree equals the oracle's node for node, and frames traced on the edited world at
    960x540 and at the workload's 3840x2160 (primary G-buffer, primary and GI hit records, high_quality
    preset with LOD on) are bit-exact against the oracle's trace of its own edited world."""
    from arcadia_gb300.pipeline import FullPipeline, path_camera

    scene = L.SCENES["c5_4096"]
    ow = world_cache("c5_4096")
    nr, nn, nb, _ = native_lib.build_world(scene)  # the pipeline's own builder gives the oracle's pools
    assert nr.tobytes() == ow.roots.tobytes() and nn.tobytes() == ow.nodes.tobytes() and nb.tobytes() == ow.bricks.tobytes()
    W, H, F = 960, 540, 8
    t = native_lib.Tracer(0)
    try:
        t.upload_world(ow.grid, ow.roots, ow.nodes, ow.bricks, ow.palette, node_headroom=1 << 22, brick_headroom=1 << 19)
        p = FullPipeline(t, scene, W, H, n_bricks=len(ow.bricks), n_frames=F, edit_fraction=0.01, keep_ops=True)
        s = p.run(warmup=1)
        assert s["frames"] == F and s["overflow"] == 0 and s["device_status"] == 0
        assert s["bricks_rewritten_per_frame"] > 0.5 * s["brick_target_per_frame"]
        for ops in p.ops_log:
            ow = orc.apply_edits(ow, ops, node_headroom=1 << 22, brick_headroom=1 << 19)
        roots, nodes, bricks = t.download_world()
        assert (roots == 0xFFFFFFFF).sum() == (ow.roots == 0xFFFFFFFF).sum()
        for i, r in enumerate(ow.roots):
            assert orc.tree_compare(r, ow.nodes, ow.bricks, roots[i], nodes, bricks) == 0, i
        cam = path_camera(scene, W, H, F - 1, F, L.quality_high())
        t.set_camera(cam)
        gdm, gnm, gaa, hits, gi, n_gi = t.trace_frame()
        ogdm, ognm, ogaa, ohits, _ = orc.primary(ow, cam, threads=THREADS)
        _, ogi, _ = orc.gi_rays(ow, cam, ogdm, ognm, threads=THREADS)
        np.testing.assert_array_equal(gdm, ogdm)
        np.testing.assert_array_equal(gnm, ognm)
        np.testing.assert_array_equal(gaa, ogaa)
        assert hits.tobytes() == ohits.tobytes()
        assert gi.tobytes() == ogi.tobytes()
        assert n_gi == int((ohits["flags"] & 1).sum()) > 0.2 * W * H
        # the same edited world at the workload's own 3840x2160
        cam4 = path_camera(scene, 3840, 2160, F - 1, F, L.quality_high())
        t.set_camera(cam4)
        gdm, gnm, gaa, hits, gi, n_gi = t.trace_frame()
        ogdm, ognm, ogaa, ohits, _ = orc.primary(ow, cam4, threads=THREADS)
        _, ogi, _ = orc.gi_rays(ow, cam4, ogdm, ognm, threads=THREADS)
        np.testing.assert_array_equal(gdm, ogdm)
        np.testing.assert_array_equal(gnm, ognm)
        np.testing.assert_array_equal(gaa, ogaa)
        assert hits.tobytes() == ohits.tobytes()
        assert gi.tobytes() == ogi.tobytes()
        assert n_gi == int((ohits["flags"] & 1).sum())
    finally:
        t.close()
