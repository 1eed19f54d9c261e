"""Failure detection on the GPU, without a GPU fault (failures injected from the host side).

The reference renderer has no device-side checks (it handles only swapchain loss,
crates/arcadia-render/src/renderer.rs:368-378); this library's are exercised here:
  * a tensor-core pipeline wait that runs out of its cycle budget: through arc_debug_set the NRC
    kernels arm the barrier of their weight copy without issuing the copy (a flag that nothing sets)
    and the budget is shrunk to 0.1 ms; the kernel sets status bit 31, frees TMEM and returns, the
    call fails with ARC_E_DEVICE_CHECK, and the next call on the same context works and gives the
    earlier results;
  * a corrupt pool that reaches the kernels (upload validation switched off through arc_debug_set):
    the range checks read the bad nodes as empty and the bad bricks as air, exactly as the oracle's
    ReadZeroSkipWrite reads, and the status readback reports ARC_E_DEVICE_CHECK;
  * NaN, infinite, zero-length and huge rays, and empty batches, bit-exact against the oracle.
No test here faults, traps or hangs the device: every wait has a bound and every index a range check.
"""
import ctypes
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
ARC_DEBUG_TC_WAIT_BUDGET = 1
ARC_DEBUG_SKIP_POOL_VALIDATION = 2
ARC_DEBUG_TC_STALL = 3
ARC_E_DEVICE_CHECK = -6


def _fp(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _err(t):
    return t.last_error()


def test_tc_wait_timeout_is_reported_and_context_recovers(native_lib, world_cache):
    lib = native_lib.lib()
    w = world_cache("c1_256")
    t = native_lib.Tracer(0)
    try:
        t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
        t.set_camera(L.default_camera_for(L.SCENES["c1_256"], 64, 64))
        assert lib.arc_nrc_init(t.ctx, 5) == 0
        rng = np.random.default_rng(1)
        n = 5000
        x = rng.random((n, 9), dtype=np.float32)
        tgt = rng.random((n, 3), dtype=np.float32)
        base = np.zeros((n, 3), np.float32)
        assert lib.arc_nrc_query(t.ctx, _fp(x), None, n, _fp(base)) == 0, _err(t)
        assert np.isfinite(base).all() and np.abs(base).max() > 0
        # the weight barrier is armed but never fed; its wait gives up after 200,000 cycles
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_WAIT_BUDGET, 200000) == 0
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_STALL, 1) == 0
        out = np.zeros((n, 3), np.float32)
        assert lib.arc_nrc_query(t.ctx, _fp(x), None, n, _fp(out)) == ARC_E_DEVICE_CHECK
        assert "tensor-core pipeline wait timed out" in _err(t)
        # the hook switched off and the budget restored, the same context answers again with the same results
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_STALL, 0) == 0
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_WAIT_BUDGET, 0) == 0
        again = np.zeros((n, 3), np.float32)
        assert lib.arc_nrc_query(t.ctx, _fp(x), None, n, _fp(again)) == 0, _err(t)
        np.testing.assert_array_equal(again, base)
        # the training kernel's wait runs out the same way
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_WAIT_BUDGET, 200000) == 0
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_STALL, 1) == 0
        loss = ctypes.c_float(0.0)
        assert lib.arc_nrc_train_step(t.ctx, _fp(x), _fp(tgt), n, ctypes.c_float(1e-3), ctypes.byref(loss)) == ARC_E_DEVICE_CHECK
        assert "tensor-core pipeline wait timed out" in _err(t)
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_STALL, 0) == 0
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_WAIT_BUDGET, 0) == 0
        assert lib.arc_nrc_init(t.ctx, 5) == 0
        assert lib.arc_nrc_query(t.ctx, _fp(x), None, n, _fp(again)) == 0, _err(t)
        np.testing.assert_array_equal(again, base)
        assert lib.arc_nrc_train_step(t.ctx, _fp(x), _fp(tgt), n, ctypes.c_float(1e-3), ctypes.byref(loss)) == 0, _err(t)
        assert np.isfinite(loss.value) and loss.value > 0
        assert t.stats().device_status == 0
        # the traversal kernels on the same context are unaffected
        hits = t.trace_rays(np.zeros(0, L.RAY_DTYPE), 10.0)
        assert hits.size == 0
        t.trace_frame()
        assert lib.arc_debug_set(t.ctx, 99, 0) == -1
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_TC_WAIT_BUDGET, -5) == -1
    finally:
        t.close()


def _corrupt(orc, w, rng):
    """Copies of the pools with 12 internal nodes pointing past the node pool and 12 mixed leaves past
    the brick pool; the nodes picked are children of chunk roots, so primary rays descend into them."""
    nodes = w.nodes.copy()
    cp = nodes["child_ptr"].astype(np.int64)
    internal = np.nonzero(((cp & 0x80000000) == 0) & ((nodes["mask_low"] | nodes["mask_high"]) != 0))[0]
    mixed = np.nonzero((cp & 0xC0000000) == 0x80000000)[0]
    near_top = internal[(internal > 0) & (internal < 64)]
    bad_n = rng.choice(near_top, min(12, len(near_top)), replace=False)
    bad_b = rng.choice(mixed, 12, replace=False)
    nodes["child_ptr"][bad_n] = len(nodes) + 1000 + np.arange(len(bad_n))
    nodes["child_ptr"][bad_b] = 0x80000000 | (len(w.bricks) + 50 + np.arange(len(bad_b)))
    return orc.World(w.grid, w.roots, nodes, w.bricks, w.palette)


def test_corrupt_pool_reads_as_empty_and_is_reported(orc, native_lib, world_cache):
    import torch

    lib = native_lib.lib()
    w = world_cache("c1_256")
    bad = _corrupt(orc, w, np.random.default_rng(2))
    Wd, Hd = 640, 360
    cam = L.default_camera_for(L.SCENES["c1_256"], Wd, Hd, quality=L.quality_parity(512), frame_index=2)
    t = native_lib.Tracer(0)
    try:
        with pytest.raises(native_lib.ArcError) as e:
            t.upload_world(bad.grid, bad.roots, bad.nodes, bad.bricks, bad.palette)
        assert e.value.code == -4  # validation on: rejected on the host
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_SKIP_POOL_VALIDATION, 1) == 0
        t.upload_world(bad.grid, bad.roots, bad.nodes, bad.bricks, bad.palette)  # no headroom: the pointers are out of range
        assert lib.arc_debug_set(t.ctx, ARC_DEBUG_SKIP_POOL_VALIDATION, 0) == 0
        t.set_camera(cam)
        n = Wd * Hd
        bufs = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (2 * n, 2 * n, n, 5 * n, 5 * n)]
        t.trace_frame_dev(Wd, Hd, *[b.data_ptr() for b in bufs])
        rc = lib.arc_synchronize(t.ctx)
        assert rc == ARC_E_DEVICE_CHECK, rc
        assert "range check" in _err(t)
        ogdm, ognm, ogaa, ohits, _ = orc.primary(bad, cam, threads=THREADS)
        _, ogi, _ = orc.gi_rays(bad, cam, ogdm, ognm, threads=THREADS)
        for got, want in zip(bufs, (ogdm, ognm, ogaa, ohits, ogi)):
            assert np.array_equal(got.cpu().numpy().view(np.uint32), np.ascontiguousarray(want).view(np.uint32).reshape(-1))
        # the bad pointers changed the picture: the good world's frame differs
        gdm_good = orc.primary(w, cam, threads=THREADS)[0]
        assert not np.array_equal(gdm_good, ogdm)
        # the status was cleared by the readback; a valid world on the same context traces cleanly
        t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
        t.set_camera(cam)
        t.trace_frame_dev(Wd, Hd, *[b.data_ptr() for b in bufs])
        t.synchronize()
        assert np.array_equal(bufs[0].cpu().numpy().view(np.uint32), gdm_good.reshape(-1))
    finally:
        t.close()


def _odd_rays(rng):
    nan, inf = np.float32(np.nan), np.float32(np.inf)
    o = [(8, 13.75, 8)] * 12 + [(nan, 5, 5), (5, nan, 5), (nan, nan, nan), (inf, 5, 5), (-inf, 5, 5), (5, -inf, 5),
                                (1e30, 5, 5), (-1e30, -1e30, -1e30), (8, 13.75, 8), (8, 13.75, 8), (0, 0, 0), (16, 16, 16)]
    d = [(0, 0, 0), (nan, 0, 0), (0, nan, 0), (nan, nan, nan), (inf, 0, 0), (0, -inf, 0), (inf, inf, -inf),
         (1e-30, -1e-30, 0), (-0.0, -1, -0.0), (1e-45, -1, 0), (3e38, -3e38, 1), (0, -1e-8, 0)] + \
        [(0, -1, 0), (0, -1, 0), (0, -1, 0), (1, 0, 0), (1, 0, 0), (0, 1, 0), (1, 0, 0), (1, 1, 1), (nan, -1, 0),
         (0, -1, inf), (1, 1, 1), (-1, -1, -1)]
    rays = np.zeros(len(o) + 2000, L.RAY_DTYPE)
    rays["origin_m"][: len(o)] = np.array(o, np.float32)
    rays["dir"][: len(o)] = np.array(d, np.float32)
    # plus random rays with random components replaced by NaN / inf / 0 / denormals
    k = 2000
    ro = (rng.random((k, 3)) * 20 - 2).astype(np.float32)
    rd = rng.standard_normal((k, 3)).astype(np.float32)
    special = np.array([np.nan, np.inf, -np.inf, 0.0, -0.0, 1e-40, 1e30], np.float32)
    for arr in (ro, rd):
        m = rng.random(arr.shape) < 0.08
        arr[m] = rng.choice(special, int(m.sum()))
    rays["origin_m"][len(o):] = ro
    rays["dir"][len(o):] = rd
    return rays


def _same_records(a, b):
    a = a.view(np.uint32).reshape(len(a), -1).copy()
    b = b.view(np.uint32).reshape(len(b), -1).copy()
    fa, fb = a[:, 4].view(np.float32), b[:, 4].view(np.float32)
    both_nan = np.isnan(fa) & np.isnan(fb)
    a[both_nan, 4] = b[both_nan, 4] = 0  # a NaN depth is a NaN whatever its payload bits
    return np.array_equal(a, b)


@pytest.mark.parametrize("lod_bias,water", [(0, False), (2, True)])
def test_nan_inf_and_degenerate_rays_match_oracle(orc, native_lib, world_cache, lod_bias, water):
    w = world_cache("c1_256")
    cam = L.default_camera_for(L.SCENES["c1_256"], 64, 64, quality=L.quality_high())
    t = native_lib.Tracer(0)
    try:
        t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
        t.set_camera(cam)
        rays = _odd_rays(np.random.default_rng(7 + lod_bias))
        for max_d in (0.0, 3.0, 80.0, np.float32(np.inf)):
            g = t.trace_rays(rays, float(max_d), lod_bias, water)
            o = orc.trace_rays(w, cam, rays, float(max_d), lod_bias, water, threads=THREADS)
            assert _same_records(g, o), max_d
        assert t.stats().device_status == 0
        # empty batches: host and device forms
        assert t.trace_rays(rays[:0], 10.0).size == 0
        assert native_lib.lib().arc_trace_rays_dev(t.ctx, None, 0, ctypes.c_float(10.0), 0, 0, None) == 0
        t.synchronize()
    finally:
        t.close()


def test_degenerate_shadow_rays_match_oracle(orc, native_lib, world_cache):
    import torch

    w = world_cache("c1_256")
    cam = L.default_camera_for(L.SCENES["c1_256"], 64, 64, quality=L.quality_high())
    t = native_lib.Tracer(0)
    try:
        t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
        t.set_camera(cam)
        rays = _odd_rays(np.random.default_rng(11))[:400]
        d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
        vis = torch.zeros(len(rays), dtype=torch.float32, device="cuda")
        t.shadow_rays_dev(d_rays.data_ptr(), len(rays), 32.0, vis.data_ptr())
        t.synchronize()
        want = np.array([orc.shadow_vis(w, cam, r["origin_m"], r["dir"], 32.0) for r in rays], np.float32)
        np.testing.assert_array_equal(vis.cpu().numpy(), want)
    finally:
        t.close()
