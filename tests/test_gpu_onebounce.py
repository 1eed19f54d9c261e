"""The one-bounce estimator of the cache comparison against its oracle restatement (GPU).

Every radiance number the cache comparison reports is built on this estimator (sun term with
trace_shadow_vis, shaders/common/traversal64.wgsl:571-773, from x + 0.10 n as in sharc_shade_surface,
shaders/sharc_update.wgsl:68-105; sky term through one cosine ray, types.wgsl:531-545): the GI hit points
the caches are queried at, the NRC's training targets, SHARC's mode-1 deposits and the 4096-spp
reference that scores both caches. Each is checked here bit for bit against the oracle on the 1024^3
caves world (high_quality preset).
"""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
W, H = 640, 360


@pytest.fixture(scope="module")
def frame(orc, native_lib, world_cache):
    """GPU frame of the caves world: G-buffer, GI hit points, their compacted list (device tensors)."""
    pytest.importorskip("torch")
    from arcadia_gb300 import gi_cache

    w = world_cache("c2_1024_caves")
    t = native_lib.Tracer(0)
    t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
    cc = gi_cache.CacheComparison(t, L.SCENES["c2_1024_caves"], W, H)
    cc.shared(4)
    t.synchronize()
    yield w, t, cc
    t.close()


def _np(x):
    return x.cpu().numpy()


def test_gi_points_match_oracle(orc, frame):
    """arc_gi_points_dev (GI ray traced again from the G-buffer): valid mask, point, normal, albedo and
    network inputs of every pixel bit-exact; the compacted list holds exactly the valid pixels."""
    w, t, cc = frame
    cam = cc.camera(4)
    gdm, gnm = _np(cc.gdm).view(np.uint32), _np(cc.gnm).view(np.uint32)
    pos, nrm, alb, nin, valid = orc.gi_points(w, cam, gdm, gnm, threads=THREADS)
    gvalid = _np(cc.valid).view(np.uint32)
    np.testing.assert_array_equal(gvalid, valid)
    m = valid.astype(bool)
    assert m.sum() > 0.05 * W * H
    for got, want in ((cc.pos, pos), (cc.nrm, nrm), (cc.alb, alb), (cc.nin, nin)):
        np.testing.assert_array_equal(_np(got)[m].view(np.uint32), want[m].view(np.uint32))
    n = int(cc.n_valid.item())
    assert np.array_equal(np.sort(_np(cc.list)[:n].view(np.uint32)), np.nonzero(m)[0])


def test_gi_points_from_hits_match_oracle(orc, native_lib, frame):
    """arc_gi_points_from_hits_dev (points from the frame kernel's GI hit records) bit-exact."""
    import torch

    w, t, cc = frame
    cam = cc.camera(4)
    t.set_camera(cam)
    n = W * H
    bufs = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (2 * n, 2 * n, n, 5 * n, 5 * n)]
    t.trace_frame_dev(W, H, *[b.data_ptr() for b in bufs])
    pos, nrm, alb, nin = (torch.zeros((n, k), dtype=torch.float32, device="cuda") for k in (3, 3, 3, 9))
    valid = torch.zeros(n, dtype=torch.int32, device="cuda")
    n_valid = torch.zeros(1, dtype=torch.int64, device="cuda")
    lst = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert native_lib.lib().arc_gi_points_from_hits_dev(
        t.ctx, W, H, bufs[0].data_ptr(), bufs[1].data_ptr(), bufs[4].data_ptr(), pos.data_ptr(), nrm.data_ptr(),
        alb.data_ptr(), nin.data_ptr(), valid.data_ptr(), n_valid.data_ptr(), lst.data_ptr()) == 0
    t.synchronize()
    gdm, gnm = _np(bufs[0]).view(np.uint32), _np(bufs[1]).view(np.uint32)
    ogi = _np(bufs[4]).view(L.HIT_DTYPE)
    opos, onrm, oalb, onin, ovalid = orc.gi_points_from_hits(cam, gdm, gnm, ogi)
    np.testing.assert_array_equal(_np(valid).view(np.uint32), ovalid)
    m = ovalid.astype(bool)
    assert m.sum() > 0.05 * n and int(n_valid.item()) == int(m.sum())
    for got, want in ((pos, opos), (nrm, onrm), (alb, oalb), (nin, onin)):
        np.testing.assert_array_equal(_np(got)[m].view(np.uint32), want[m].view(np.uint32))


@pytest.mark.parametrize("spp", [1, 4])
def test_onebounce_matches_oracle(orc, native_lib, frame, spp):
    """arc_onebounce_dev at 20,000 GI hit points: the mean of spp samples bit-exact, then accumulated
    into the same buffer by a second call with another seed."""
    import torch

    w, t, cc = frame
    t.set_camera(cc.camera(4))
    valid = _np(cc.valid).astype(bool)
    idx = np.nonzero(valid)[0][::3][:20000].astype(np.uint32)
    d_idx = torch.from_numpy(idx.view(np.int32)).cuda()
    out = torch.zeros((len(idx), 3), dtype=torch.float32, device="cuda")
    lib = native_lib.lib()
    assert lib.arc_onebounce_dev(t.ctx, d_idx.data_ptr(), len(idx), cc.pos.data_ptr(), cc.nrm.data_ptr(),
                                 cc.alb.data_ptr(), spp, 77, 0, out.data_ptr()) == 0
    t.synchronize()
    pos, nrm, alb = _np(cc.pos), _np(cc.nrm), _np(cc.alb)
    want = orc.onebounce(w, cc.camera(4), pos, nrm, alb, spp, 77, idx=idx, threads=THREADS)
    got = _np(out)
    np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))
    assert (got > 0).any(axis=1).mean() > 0.3 and (got == 0).all(axis=1).any()  # lit and fully dark points
    assert lib.arc_onebounce_dev(t.ctx, d_idx.data_ptr(), len(idx), cc.pos.data_ptr(), cc.nrm.data_ptr(),
                                 cc.alb.data_ptr(), spp, 78, 1, out.data_ptr()) == 0
    t.synchronize()
    want = orc.onebounce(w, cc.camera(4), pos, nrm, alb, spp, 78, idx=idx, accumulate_into=want, threads=THREADS)
    np.testing.assert_array_equal(_np(out).view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("cluster", [1, 32])
def test_training_batch_matches_oracle(orc, native_lib, frame, cluster):
    """arc_nrc_train_samples_dev, the batch arc_nrc_train_frame_dev trains on: 32,768 samples in 4
    interleaved slices, each its own stratum or in runs of 32 list entries, inputs and 1-spp targets
    bit-exact (the oracle draws from the same compacted list, whose order the GPU's warp-aggregated
    appends decide)."""
    import torch

    w, t, cc = frame
    t.set_camera(cc.camera(4))
    assert native_lib.lib().arc_nrc_set_sample_cluster(t.ctx, cluster) == 0
    n_samples, steps, seed = 32768, 4, 0xC0FFEE
    tin = torch.zeros((n_samples, 9), dtype=torch.float32, device="cuda")
    tt = torch.zeros((n_samples, 3), dtype=torch.float32, device="cuda")
    assert native_lib.lib().arc_nrc_train_samples_dev(
        t.ctx, cc.list.data_ptr(), cc.n_valid.data_ptr(), cc.pos.data_ptr(), cc.nrm.data_ptr(), cc.nin.data_ptr(), seed,
        n_samples, steps, tin.data_ptr(), tt.data_ptr()) == 0
    t.synchronize()
    n_valid = int(cc.n_valid.item())
    lst = _np(cc.list).view(np.uint32)[:n_valid]
    assert native_lib.lib().arc_nrc_set_sample_cluster(t.ctx, 1) == 0
    oin, ot = orc.train_samples(w, cc.camera(4), lst, n_valid, _np(cc.pos), _np(cc.nrm), _np(cc.nin), seed, n_samples,
                                steps, threads=THREADS, cluster=cluster)
    np.testing.assert_array_equal(_np(tin).view(np.uint32), oin.view(np.uint32))
    np.testing.assert_array_equal(_np(tt).view(np.uint32), ot.view(np.uint32))
    assert (ot > 0).any(axis=1).mean() > 0.3


def test_reference_scores_match_oracle(orc, frame):
    """The 4096-spp reference that scores both caches (64 launches of 64 spp, accumulated in FP64 on the
    host): at 64 points every launch is bit-exact against the oracle's, so the reference equals the oracle's
    FP64 accumulation exactly."""
    from arcadia_gb300 import gi_cache

    w, t, cc = frame
    t.set_camera(cc.camera(4))
    idx = np.nonzero(_np(cc.valid).astype(bool))[0][::997][:64]
    ref = cc.reference(idx, seed=4242)
    pos, nrm, alb = _np(cc.pos), _np(cc.nrm), _np(cc.alb)
    acc = np.zeros((len(idx), 3), np.float64)
    for k in range(gi_cache.REF_LAUNCHES):
        acc += orc.onebounce(w, cc.camera(4), pos, nrm, alb, gi_cache.REF_SPP_PER_LAUNCH, 4242 + 7919 * k,
                             idx=idx.astype(np.uint32), threads=THREADS).astype(np.float64)
    np.testing.assert_array_equal(ref, acc / gi_cache.REF_LAUNCHES)
    assert (ref > 0).any()


def test_sharc_mode1_update_matches_oracle(orc, native_lib, frame):
    """SHARC's update pass in mode 1 (the estimator at the path vertex, as the cache comparison runs it):
    per-key fixed-point sums and counts equal the oracle's sequential replay."""
    w, t, cc = frame
    cam = cc.camera(4)
    t.set_camera(cam)
    lib = native_lib.lib()
    assert lib.arc_sharc_set_mode(t.ctx, 1) == 0
    try:
        t.sharc_reset()
        t.sharc_update_dev(W, H, cc.gdm.data_ptr(), cc.gnm.data_ptr())
        keys, accum, _ = t.sharc_download()
    finally:
        lib.arc_sharc_set_mode(t.ctx, 0)
    osh = orc.Sharc()
    tk, tb, tr, tv = osh.update(w, cam, _np(cc.gdm).view(np.uint32), _np(cc.gnm).view(np.uint32), mode=1)
    assert tv.sum() > 100

    def per_key(k, a):
        a = a.reshape(-1, 4)
        return {int(x): tuple(int(v) for v in a[i]) for i, x in enumerate(k) if x}

    per_bucket = {}
    for k, b in zip(tk[tv == 1], tb[tv == 1]):
        per_bucket.setdefault(int(b), set()).add(int(k))
    crowded = {k for ks in per_bucket.values() if len(ks) > 4 for k in ks}
    g, o = per_key(keys, accum), per_key(osh.keys, osh.accum)
    assert set(g) - crowded == set(o) - crowded
    for k in set(o) - crowded:
        assert g[k] == o[k], (k, g[k], o[k])
