"""Radiance caches at secondary hits: what the trained network gains, and how SHARC compares (GPU).

Both caches learn the one-bounce radiance at GI hits on the 1024^3 caves scene; quality is the relative
MSE against a 4096-spp reference (FP64 host accumulation), at the benchmark's own setting (1920x1080,
static camera, 300 frames, which take a few seconds). The trained network must beat the method without
the learned part (the same network untrained) and SHARC, the cache it replaces.
"""
import pytest

pytestmark = pytest.mark.gpu


def test_trained_nrc_beats_untrained_and_sharc(native_lib):
    pytest.importorskip("torch")
    from arcadia_gb300 import gi_cache, layout as L

    scene = L.SCENES["c2_1024_caves"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        r = gi_cache.run_comparison(t, width=1920, height=1080, frames=300, eval_points=8192, curve=())
    finally:
        t.close()
    print(r)
    assert r["eval_points"] > 1000
    assert r["rel_mse_nrc"] < 0.8 * r["rel_mse_untrained_nrc"]
    assert r["rel_mse_nrc"] < r["rel_mse_sharc"]
    assert 0.0 < r["sharc_hit_fraction"] <= 1.0


def _points(native_lib, w=320, h=180):
    """c1_256 frame: G-buffer, GI hit points and their compacted list on the GPU."""
    import torch
    from arcadia_gb300 import gi_cache, layout as L

    scene = L.SCENES["c1_256"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
    cc = gi_cache.CacheComparison(t, scene, w, h)
    cc.shared(3)
    return t, cc


def test_gi_points_list_is_the_valid_set(native_lib):
    import numpy as np

    t, cc = _points(native_lib)
    try:
        valid = cc.valid.cpu().numpy()
        n = int(cc.n_valid.item())
        lst = cc.list.cpu().numpy()[:n]
        assert n == int(valid.sum()) > 100
        assert np.array_equal(np.sort(lst), np.nonzero(valid)[0])
    finally:
        t.close()


def test_list_queries_match_dense_queries(native_lib):
    """NRC and SHARC queries over the compacted list write exactly the listed pixels, with the dense
    query's values there."""
    import numpy as np
    import torch
    from arcadia_gb300.native import lib

    t, cc = _points(native_lib)
    try:
        L_ = lib()
        n_px = cc.w * cc.h
        assert L_.arc_nrc_init(t.ctx, 5) == 0
        assert L_.arc_sharc_set_mode(t.ctx, 1) == 0
        t.sharc_reset()
        assert L_.arc_sharc_update_dev(t.ctx, cc.w, cc.h, cc.gdm.data_ptr(), cc.gnm.data_ptr()) == 0
        assert L_.arc_sharc_resolve(t.ctx) == 0
        dense_n = torch.zeros((n_px, 3), dtype=torch.float32, device="cuda")
        dense_s = torch.zeros((n_px, 4), dtype=torch.float32, device="cuda")
        assert L_.arc_nrc_query_dev(t.ctx, cc.nin.data_ptr(), cc.alb.data_ptr(), n_px, dense_n.data_ptr()) == 0
        assert L_.arc_sharc_query_dev(t.ctx, cc.pos.data_ptr(), cc.nrm.data_ptr(), None, n_px, dense_s.data_ptr()) == 0
        list_n = torch.full((n_px, 3), -7.0, dtype=torch.float32, device="cuda")
        list_s = torch.full((n_px, 4), -7.0, dtype=torch.float32, device="cuda")
        assert L_.arc_nrc_query_list_dev(t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n_px, cc.nin.data_ptr(),
                                         cc.alb.data_ptr(), list_n.data_ptr()) == 0
        assert L_.arc_sharc_query_list_dev(t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n_px, cc.pos.data_ptr(),
                                           cc.nrm.data_ptr(), list_s.data_ptr()) == 0
        t.synchronize()
        v = cc.valid.cpu().numpy().astype(bool)
        for got, want in ((list_n, dense_n), (list_s, dense_s)):
            g, w_ = got.cpu().numpy(), want.cpu().numpy()
            np.testing.assert_array_equal(g[v], w_[v])
            assert (g[~v] == -7.0).all()
        assert (dense_s.cpu().numpy()[v][:, 3] > 0.5).any()  # some cached entries found
        assert L_.arc_sharc_set_mode(t.ctx, 0) == 0
    finally:
        t.close()


def test_train_frame_updates_weights_and_skips_empty_frames(native_lib):
    import numpy as np
    import torch
    from arcadia_gb300.native import lib

    t, cc = _points(native_lib)
    try:
        L_ = lib()
        assert L_.arc_nrc_init(t.ctx, 5) == 0
        w0 = np.zeros(30400, np.float32)
        assert L_.arc_nrc_get_weights(t.ctx, w0.ctypes.data) == 0
        zero = torch.zeros(1, dtype=torch.int64, device="cuda")
        args = (cc.list.data_ptr(), zero.data_ptr(), cc.pos.data_ptr(), cc.nrm.data_ptr(), cc.nin.data_ptr(), 11, 4096, 2, 1e-3)
        assert L_.arc_nrc_train_frame_dev(t.ctx, *args) == 0
        w1 = np.zeros(30400, np.float32)
        assert L_.arc_nrc_get_weights(t.ctx, w1.ctypes.data) == 0
        assert np.array_equal(w0, w1)  # no GI hit: nothing to learn
        args = (cc.list.data_ptr(), cc.n_valid.data_ptr()) + args[2:]
        assert L_.arc_nrc_train_frame_dev(t.ctx, *args) == 0
        assert L_.arc_nrc_get_weights(t.ctx, w1.ctypes.data) == 0
        assert np.isfinite(w1).all() and np.abs(w1 - w0).max() > 1e-4
        bad = args[:7] + (0,) + args[8:]
        assert L_.arc_nrc_train_frame_dev(t.ctx, *bad) != 0  # steps = 0
    finally:
        t.close()


def test_gi_points_from_hit_records(native_lib):
    """Points from the frame kernel's GI hit records: the same hit pixels as re-tracing the GI rays, the
    same normals and albedos, positions on the hit cell's entry face."""
    import numpy as np
    import torch
    from arcadia_gb300 import gi_cache, layout as L
    from arcadia_gb300.native import lib

    scene = L.SCENES["c1_256"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        w, h = 320, 180
        cc = gi_cache.CacheComparison(t, scene, w, h)
        t.set_camera(cc.camera(4))
        hits = torch.zeros(w * h * 5, dtype=torch.int32, device="cuda")
        gi = torch.zeros(w * h * 5, dtype=torch.int32, device="cuda")
        t.trace_frame_dev(w, h, cc.gdm.data_ptr(), cc.gnm.data_ptr(), cc.gaa.data_ptr(), hits.data_ptr(), gi.data_ptr())
        assert lib().arc_gi_points_dev(t.ctx, w, h, cc.gdm.data_ptr(), cc.gnm.data_ptr(), cc.pos.data_ptr(), cc.nrm.data_ptr(),
                                       cc.alb.data_ptr(), cc.nin.data_ptr(), cc.valid.data_ptr(), cc.n_valid.data_ptr(),
                                       cc.list.data_ptr()) == 0
        t.synchronize()
        ref = [x.cpu().numpy().copy() for x in (cc.pos, cc.nrm, cc.alb, cc.valid)]
        assert lib().arc_gi_points_from_hits_dev(t.ctx, w, h, cc.gdm.data_ptr(), cc.gnm.data_ptr(), gi.data_ptr(),
                                                 cc.pos.data_ptr(), cc.nrm.data_ptr(), cc.alb.data_ptr(), cc.nin.data_ptr(),
                                                 cc.valid.data_ptr(), cc.n_valid.data_ptr(), cc.list.data_ptr()) == 0
        t.synchronize()
        pos, nrm, alb, valid = [x.cpu().numpy() for x in (cc.pos, cc.nrm, cc.alb, cc.valid)]
        v = ref[3].astype(bool)
        assert v.sum() > 1000 and np.array_equal(valid.astype(bool), v)
        assert int(cc.n_valid.item()) == int(v.sum())
        np.testing.assert_array_equal(nrm[v], ref[1][v])
        np.testing.assert_array_equal(alb[v], ref[2][v])
        span = 1 << (2 * ((gi.cpu().numpy().view(L.HIT_DTYPE)["flags"][v] >> 1) & 7))
        # on the entry face: within half a cell of its centre per axis; a GI ray that starts inside a
        # solid voxel hits at its own origin, off the face (a few points)
        d = np.abs(pos[v] - ref[0][v]).max(1)
        assert np.mean(d <= 0.0625 * span * 0.5 + 1e-4) >= 0.99, np.mean(d <= 0.0625 * span * 0.5 + 1e-4)
        assert np.all(d <= 0.0625 * span * 2.0), d.max()
        nin = cc.nin.cpu().numpy()[v]
        np.testing.assert_allclose(np.linalg.norm(nin[:, 6:9], axis=1), 1.0, atol=1e-5)
    finally:
        t.close()


def test_overlapped_cache_frames_query_the_previous_state(native_lib):
    """arc_nrc_frame_dev / arc_sharc_frame_dev run each cache's query beside its update: the query's
    output equals a query issued before the update (bit-exact), and the update still happens."""
    import ctypes as C

    import numpy as np
    import torch

    t, cc = _points(native_lib)
    lib, n = cc.lib, cc.w * cc.h
    try:
        # NRC
        assert lib.arc_nrc_init(t.ctx, 5) == 0
        before = torch.zeros_like(cc.nrc_out)
        assert lib.arc_nrc_query_list_dev(t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n, cc.nin.data_ptr(),
                                          cc.alb.data_ptr(), before.data_ptr()) == 0
        w0 = np.zeros(200000, np.float32)
        assert lib.arc_nrc_get_weights(t.ctx, w0.ctypes.data) == 0
        assert lib.arc_nrc_frame_dev(t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n, cc.pos.data_ptr(), cc.nrm.data_ptr(),
                                     cc.nin.data_ptr(), cc.alb.data_ptr(), cc.nrc_out.data_ptr(), 77, 8192, 2,
                                     C.c_float(1e-3)) == 0
        t.synchronize()
        assert torch.equal(cc.nrc_out, before)
        w1 = np.zeros(200000, np.float32)
        assert lib.arc_nrc_get_weights(t.ctx, w1.ctypes.data) == 0
        assert not np.array_equal(w0, w1)
        # SHARC: fill the cache for one frame, then the overlapped frame queries that resolve
        t.sharc_reset()
        cc.sharc_frame()
        before = cc.sharc_out.clone()
        assert (before[:, 3] > 0.5).any()
        cc.shared(4)
        assert lib.arc_sharc_query_list_dev(t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), n, cc.pos.data_ptr(),
                                            cc.nrm.data_ptr(), before.data_ptr()) == 0
        res0 = t.sharc_download()[2].copy()
        cc.sharc_frame(overlap=True)
        assert torch.equal(cc.sharc_out, before)
        assert not np.array_equal(t.sharc_download()[2], res0)  # the update and resolve ran
    finally:
        t.close()
