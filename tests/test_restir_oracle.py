"""ReSTIR GI temporal pass of the oracle (orc_restir.c) on CPU: invariants of temporal_main
(lighting_restir_gi.wgsl:61-336) that hold whatever the radiance: sky pixels get the empty reservoir,
a first frame (empty history) gives M = 1, age 0 and the pixel's own depth, and a second frame from
the same camera reuses the history (M = 2) wherever the candidate or the history has weight."""
import numpy as np

from arcadia_gb300 import layout as L


def test_restir_oracle_first_and_second_frame(orc, world_cache):
    w = world_cache("c1_256")
    W, H = 160, 90
    cam = L.default_camera_for(L.SCENES["c1_256"], W, H, quality=L.quality_high(), frame_index=2)
    gdm, gnm, _, _, _ = orc.primary(w, cam, threads=4)
    resolved = np.zeros(131072, L.SHARC_SLOT_DTYPE)  # empty cache: the radiance buffer stands in
    rng = np.random.default_rng(3)
    radiance = rng.random((W * H, 3), dtype=np.float32)
    r1 = orc.restir_gi_temporal(w, cam, resolved, gdm, gnm, L.empty_reservoirs(W * H), radiance=radiance, threads=4)
    depth = gdm[:, 0].view(np.float32)
    hit = depth < 1e4
    assert 0.1 < hit.mean() < 1.0
    assert np.all(r1["primary_depth"][~hit] == np.float32(1e5)) and np.all(r1["norm_m_flags"][~hit] == 0)
    assert np.array_equal(r1["primary_depth"][hit], depth[hit])
    nmf = r1["norm_m_flags"][hit]
    assert np.all(((nmf >> 16) & 0xFF) == 1) and np.all(((nmf >> 24) & 0x7F) == 0)
    # same camera again (motion vectors of a static camera, prev_cam_pos = eye): the history validates
    # almost everywhere (not where rounding of the reprojection lands across a depth edge)
    r2 = orc.restir_gi_temporal(w, cam, resolved, gdm, gnm, r1, radiance=radiance, threads=4)
    m2 = (r2["norm_m_flags"][hit] >> 16) & 0xFF
    assert set(np.unique(m2)) <= {1, 2} and (m2 == 2).mean() > 0.95
    # the shadow average counts two samples exactly where the history was valid
    sm = r2["shadow_vis_m"][hit] >> 16
    assert np.array_equal(sm == np.float16(2.0).view(np.uint16), m2 == 2)
