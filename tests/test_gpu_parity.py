"""GPU parity: libarc_trace.so (sm_103a) against the CPU oracle on identical inputs, through the C ABI.

Bar: hit voxel, face, material, G-buffer words and hit records bit-exact; depth within 1e-5 relative
(plus 1e-6 m absolute for hits at the origin) of the FP64 plane-entry distance.
"""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
DEPTH_RTOL = 1e-5
DEPTH_ATOL_M = 1e-6


@pytest.fixture(scope="module")
def tracer(native_lib):
    t = native_lib.Tracer(0)
    yield t
    t.close()


def _load(t, w, cam):
    t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette, node_headroom=4096, brick_headroom=1024)
    t.set_camera(cam)


def _assert_hits_equal(a, b, what):
    if a.tobytes() != b.tobytes():
        bad = np.nonzero(a.view(np.uint8).reshape(len(a), -1).any(1) != b.view(np.uint8).reshape(len(b), -1).any(1)
                         | (a.view(np.uint32).reshape(len(a), -1) != b.view(np.uint32).reshape(len(b), -1)).any(1))[0]
        raise AssertionError(f"{what}: {len(bad)} of {len(a)} records differ; first {bad[:5]}: gpu {a[bad[:3]]} oracle {b[bad[:3]]}")


def _check_depth_fp64(orc, rays_o, rays_d, hits, stride=97):
    idx = np.nonzero(hits["flags"] & 1)[0][::stride]
    for i in idx:
        shift = int((hits["flags"][i] >> 1) & 7) * 2
        span = 1 << shift
        cmin = hits["voxel"][i] & ~(span - 1)
        d64 = orc.depth_fp64(rays_o[i], rays_d[i], cmin, span) / 16.0
        d = float(hits["depth_m"][i])
        assert abs(d - d64) <= DEPTH_RTOL * d64 + DEPTH_ATOL_M, (i, d, d64)


def _camera_rays(cam, w, h):
    """Primary ray directions as the oracle computes them (float64 here only for the FP64 depth)."""
    from oracle import pyorc  # noqa: F401  (oracle import keeps the checker on the test side)

    c = cam[0]
    x = (np.arange(w, dtype=np.float32) + np.float32(0.5)) / np.float32(w)
    y = (np.arange(h, dtype=np.float32) + np.float32(0.5)) / np.float32(h)
    nx, ny = x * 2 - 1, 1 - y * 2
    th, asp = c["cam_forward_fov"][3], c["cam_right_aspect"][3]
    sx = (nx * asp) * th
    sy = ny * th
    f, r, u = c["cam_forward_fov"][:3], c["cam_right_aspect"][:3], c["cam_up_frame"][:3]
    d = (f[None, None, :] + r[None, None, :] * sx[None, :, None]) + u[None, None, :] * sy[:, None, None]
    d = d / np.sqrt((d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2])[..., None]
    return d.reshape(-1, 3).astype(np.float32)


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("quality", ["parity", "high"])
def test_frame_c1_bitexact(orc, tracer, world_cache, variant, quality):
    """256^3 world, 1280x720 primary + GI rays: every G-buffer word and hit record bit-exact."""
    w = world_cache("c1_256")
    q = L.quality_parity(512) if quality == "parity" else L.quality_high()
    cam = L.default_camera_for(L.SCENES["c1_256"], 1280, 720, quality=q, frame_index=3)
    _load(tracer, w, cam)
    tracer.set_launch_config(variant=variant)
    gdm, gnm, gaa, hits, gi, n_gi = tracer.trace_frame()
    ogdm, ognm, ogaa, ohits, _ = orc.primary(w, cam, threads=THREADS)
    _, ogi, _ = orc.gi_rays(w, cam, ogdm, ognm, threads=THREADS)
    np.testing.assert_array_equal(gdm, ogdm)
    np.testing.assert_array_equal(gnm, ognm)
    np.testing.assert_array_equal(gaa, ogaa)
    _assert_hits_equal(hits, ohits, "primary hits")
    _assert_hits_equal(gi, ogi, "GI hits")
    assert n_gi == int((ohits["flags"] & 1).sum())
    assert (hits["flags"] & 1).mean() > 0.15
    eye = np.broadcast_to(cam[0]["cam_pos_time"][:3], (len(hits), 3))
    _check_depth_fp64(orc, eye, _camera_rays(cam, 1280, 720), hits)


def test_primary_then_secondary_matches_fused(orc, tracer, world_cache):
    w = world_cache("c1_256")
    cam = L.default_camera_for(L.SCENES["c1_256"], 640, 360, quality=L.quality_high(), frame_index=9)
    _load(tracer, w, cam)
    gdm, gnm, gaa, hits = tracer.trace_primary()
    gi = tracer.trace_secondary(gdm, gnm)
    fgdm, fgnm, fgaa, fhits, fgi, _ = tracer.trace_frame()
    np.testing.assert_array_equal(gdm, fgdm)
    _assert_hits_equal(hits, fhits, "primary")
    _assert_hits_equal(gi, fgi, "GI")
    # the GI pass repacking its running rays every 4 steps
    from arcadia_gb300 import native

    tracer.set_launch_config(features=native.ARC_FEAT_GI_REPACK, refill_threshold=4)
    try:
        _assert_hits_equal(tracer.trace_secondary(gdm, gnm), fgi, "GI repacked")
    finally:
        tracer.set_launch_config(features=0, refill_threshold=24)


@pytest.mark.parametrize("quality", ["parity", "high"])
def test_frame_c2_1024_caves_full(orc, tracer, world_cache, quality, native_lib):
    """1024^3 caves world at 1920x1080 (the headline workload): the whole frame, every G-buffer word,
    primary hit record and GI hit record of all 2,073,600 pixels, bit-exact against the oracle for both
    kernel variants (plain kernel + GI pass, persistent queue kernel) and the plain kernel's traversal
    variants (Morton block order, one node per loop iteration, warp-shared node fetch, GI rays sorted over
    the whole frame, resident CTAs with and without the top tree levels staged in shared memory,
    per-ray constants computed once, the GI pass repacking its running rays every 1, 8 or 32 steps),
    through the host-buffer entry point and the device-buffer one (one launch, or concurrent row bands),
    in parity mode
    (up to 512 steps, LOD out of reach) and with the high_quality preset (LOD on)."""
    native_lib_feat = native_lib
    w = world_cache("c2_1024_caves")
    q = L.quality_parity(512) if quality == "parity" else L.quality_high()
    cam = L.default_camera_for(L.SCENES["c2_1024_caves"], 1920, 1080, quality=q, frame_index=1)
    _load(tracer, w, cam)
    ogdm, ognm, ogaa, ohits, _ = orc.primary(w, cam, threads=THREADS)
    _, ogi, _ = orc.gi_rays(w, cam, ogdm, ognm, threads=THREADS)
    n_hit = int((ohits["flags"] & 1).sum())
    assert n_hit > 0.3 * 1920 * 1080
    configs = [dict(variant=0), dict(variant=1),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_NODE_VISIT, reg_blocks=3),
               dict(variant=0, order=0, features=native_lib_feat.ARC_FEAT_WARP_FETCH, reg_blocks=2),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_WARP_FETCH | native_lib_feat.ARC_FEAT_NODE_VISIT,
                    reg_blocks=2, block_threads=64),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_GI_SORT, reg_blocks=3, block_threads=128),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_TOP_TABLE, reg_blocks=3, block_threads=256),
               dict(variant=0, order=0, features=native_lib_feat.ARC_FEAT_GRID_STRIDE, reg_blocks=2, block_threads=128),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_PRECOMP, reg_blocks=3, block_threads=64),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_GI_REPACK, reg_blocks=3, refill_threshold=8),
               dict(variant=0, order=0, features=native_lib_feat.ARC_FEAT_GI_REPACK, reg_blocks=4, refill_threshold=1),
               dict(variant=0, order=1, features=native_lib_feat.ARC_FEAT_GI_REPACK | native_lib_feat.ARC_FEAT_PRECOMP,
                    reg_blocks=2, refill_threshold=32, block_threads=64)]
    for cfg in configs:
        tracer.set_launch_config(**cfg)
        gdm, gnm, gaa, hits, gi, n_gi = tracer.trace_frame()
        np.testing.assert_array_equal(gdm, ogdm)
        np.testing.assert_array_equal(gnm, ognm)
        np.testing.assert_array_equal(gaa, ogaa)
        _assert_hits_equal(hits, ohits, f"primary {cfg}")
        _assert_hits_equal(gi, ogi, f"GI {cfg}")
        assert n_gi == n_hit
    tracer.set_launch_config(variant=0, order=0, features=0, reg_blocks=3, block_threads=128, refill_threshold=24)
    # the device-buffer entry point, in one launch and in concurrent row bands (default 4)
    import torch

    n = 1920 * 1080
    bufs = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (2 * n, 2 * n, n, 5 * n, 5 * n)]
    n_gi_dev = torch.zeros(1, dtype=torch.int64, device="cuda")
    try:
        for bands, order in ((1, 1), (2, 0), (0, 1), (8, 1)):
            assert native_lib.lib().arc_set_frame_bands(tracer.ctx, bands) == 0
            tracer.set_launch_config(order=order)
            for x in bufs:
                x.fill_(-1)
            tracer.trace_frame_dev(1920, 1080, *[x.data_ptr() for x in bufs], n_gi_dev.data_ptr())
            tracer.synchronize()
            got = [x.cpu().numpy().view(np.uint32) for x in bufs]
            np.testing.assert_array_equal(got[0].reshape(-1, 2), ogdm)
            np.testing.assert_array_equal(got[1].reshape(-1, 2), ognm)
            np.testing.assert_array_equal(got[2], ogaa)
            _assert_hits_equal(got[3].view(L.HIT_DTYPE), ohits, f"primary, device frame in {bands} bands")
            _assert_hits_equal(got[4].view(L.HIT_DTYPE), ogi, f"GI, device frame in {bands} bands")
            assert int(n_gi_dev.item()) == n_hit
    finally:
        native_lib.lib().arc_set_frame_bands(tracer.ctx, 0)
        tracer.set_launch_config(order=0)
    eye = np.broadcast_to(cam[0]["cam_pos_time"][:3], (len(ohits), 3))
    _check_depth_fp64(orc, eye, _camera_rays(cam, 1920, 1080), ohits, stride=401)


def _random_rays(n, grid, rng, outside_frac=0.2):
    ext = np.array(grid, np.float32) * 16.0
    o = rng.random((n, 3)).astype(np.float32) * ext
    k = int(n * outside_frac)
    o[:k] = (rng.random((k, 3)).astype(np.float32) * 3 - 1) * ext   # many start outside the world
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d[n // 10: n // 5, rng.integers(0, 3)] = 0.0                    # zero components (1e-7 clamp)
    d[n // 5: n // 4, :] *= np.float32([0, 1, 0])                    # axis-aligned
    d[n // 5: n // 4, 1] = np.where(d[n // 5: n // 4, 1] == 0, 1.0, d[n // 5: n // 4, 1])
    d /= np.sqrt((d * d).sum(1, keepdims=True)).astype(np.float32)
    rays = np.zeros(n, L.RAY_DTYPE)
    rays["origin_m"] = o
    rays["dir"] = d
    return rays


@pytest.mark.parametrize("lod_bias,water", [(0, False), (1, False), (2, True), (0, True)])
def test_trace_rays_random(orc, tracer, world_cache, lod_bias, water):
    w = world_cache("c2_1024_caves")
    cam = L.default_camera_for(L.SCENES["c2_1024_caves"], 64, 64, quality=L.quality_high())
    _load(tracer, w, cam)
    rng = np.random.default_rng(100 + lod_bias)
    rays = _random_rays(60000, w.grid, rng)
    g = tracer.trace_rays(rays, 120.0, lod_bias, water)
    o = orc.trace_rays(w, cam, rays, 120.0, lod_bias, water, threads=THREADS)
    _assert_hits_equal(g, o, f"rays lod={lod_bias} water={water}")
    if lod_bias == 0:
        _check_depth_fp64(orc, rays["origin_m"], rays["dir"], g, stride=13)


def test_trace_rays_edge_cases(orc, tracer, world_cache):
    w = world_cache("c1_256")
    cam = L.default_camera_for(L.SCENES["c1_256"], 64, 64, quality=L.quality_parity(512))
    _load(tracer, w, cam)
    rays = np.zeros(9, L.RAY_DTYPE)
    rays["origin_m"] = [[8, 13.75, 8], [8, 2, 8], [-5, 8, 8], [8, 13.75, 8], [16, 16, 16], [0, 0, 0], [8, 6, 8],
                        [15.99, 3.0, 0.01], [8, 13.75, 8]]
    rays["dir"] = [[0, -1, 0], [0, 1, 0], [1, 0, 0], [0, 0, 1], [-0.57735, -0.57735, -0.57735], [1, 0, 0], [0, -1, 0],
                   [-1, 0, 0], [0, -1, 0]]
    for max_d in (0.0, 0.01, 5.0, 250.0):
        g = tracer.trace_rays(rays, max_d, 0, False)
        o = orc.trace_rays(w, cam, rays, max_d, 0, False, threads=1)
        _assert_hits_equal(g, o, f"edge max_d={max_d}")
    assert tracer.trace_rays(rays[:0], 10.0).size == 0


def _water_world(orc):
    """One chunk: stone floor (y < 40), a water layer (40 <= y < 80) with mixed water/stone bricks at its
    rim, so both the uniform-water skip and the per-voxel water test are exercised."""
    vol = np.zeros((256, 256, 256), np.uint8)
    vol[:, :40, :] = 2
    vol[:, 40:80, :] = 18
    vol[:, 40:80, 100:104] = 5
    vol[120:123, 60:90, 30:33] = 7
    n, b = orc.build_chunk_dense(vol)
    return orc.world_from_chunk(n, b)


def test_water_paths(orc, tracer):
    w = _water_world(orc)
    cam = L.camera_uniforms((1, 1, 1), 64, 64, (8.0, 7.0, 8.0), quality=L.quality_high())
    _load(tracer, w, cam)
    rays = _random_rays(40000, (1, 1, 1), np.random.default_rng(5), outside_frac=0.05)
    for lod, water in ((0, True), (0, False), (2, True), (1, True)):
        g = tracer.trace_rays(rays, 40.0, lod, water)
        o = orc.trace_rays(w, cam, rays, 40.0, lod, water, threads=THREADS)
        _assert_hits_equal(g, o, f"water lod={lod} ignore={water}")


def test_shadow_rays(orc, tracer, world_cache):
    import torch

    w = world_cache("c2_1024_caves")
    cam = L.default_camera_for(L.SCENES["c2_1024_caves"], 64, 64, quality=L.quality_high())
    _load(tracer, w, cam)
    rays = _random_rays(20000, w.grid, np.random.default_rng(9), outside_frac=0.1)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_vis = torch.zeros(len(rays), dtype=torch.float32, device="cuda")
    tracer.shadow_rays_dev(d_rays.data_ptr(), len(rays), 32.0, d_vis.data_ptr())
    tracer.synchronize()
    vis = d_vis.cpu().numpy()
    ovis = np.array([orc.shadow_vis(w, cam, r["origin_m"], r["dir"], 32.0) for r in rays[:4000]], np.float32)
    np.testing.assert_array_equal(vis[:4000], ovis)
    assert 0.0 < vis.mean() < 1.0


def test_persistent_schedules_agree(tracer, world_cache):
    w = world_cache("c1_256")
    cam = L.default_camera_for(L.SCENES["c1_256"], 800, 450, quality=L.quality_high(), frame_index=2)
    _load(tracer, w, cam)
    ref = None
    for cfg in [dict(variant=0, block_threads=64), dict(variant=1, block_threads=256, tile_w=8, tile_h=4, refill_threshold=8),
                dict(variant=1, block_threads=128, tile_w=4, tile_h=8, refill_threshold=1),
                dict(variant=1, block_threads=64, tile_w=16, tile_h=2, refill_threshold=32, blocks_per_sm=3)]:
        tracer.set_launch_config(**cfg)
        out = tracer.trace_frame()
        if ref is None:
            ref = out
        else:
            for a, b in zip(out[:5], ref[:5]):
                assert a.tobytes() == b.tobytes(), cfg
    tracer.set_launch_config(variant=1, block_threads=256, tile_w=8, tile_h=4, refill_threshold=8, blocks_per_sm=0)


def test_invalid_pools_rejected(orc, tracer, world_cache, native_lib):
    w = world_cache("c1_256")
    bad = w.nodes.copy()
    internal = np.nonzero(((bad["child_ptr"] & 0x80000000) == 0) & (bad["mask_low"] | bad["mask_high"] != 0))[0]
    bad["child_ptr"][internal[3]] = len(bad) + 5
    with pytest.raises(native_lib.ArcError) as e:
        tracer.upload_world(w.grid, w.roots, bad, w.bricks, w.palette)
    assert e.value.code == -4
    bad = w.nodes.copy()
    mixed = np.nonzero(((bad["child_ptr"] & 0xC0000000) == 0x80000000))[0]
    bad["child_ptr"][mixed[0]] = 0x80000000 | (len(w.bricks) + 2)
    with pytest.raises(native_lib.ArcError):
        tracer.upload_world(w.grid, w.roots, bad, w.bricks, w.palette)
    with pytest.raises(native_lib.ArcError):
        tracer.upload_world(w.grid, np.array([len(w.nodes) + 9], np.uint32), w.nodes, w.bricks, w.palette)


def test_patch_application(orc, tracer, world_cache):
    """A GpuPatch (world_map.rs:20-27) that appends a rebuilt chunk tree, then one that empties a chunk."""
    base = world_cache("s512")
    cam = L.default_camera_for(L.SCENES["s512"], 320, 200, quality=L.quality_high())
    tracer.upload_world(base.grid, base.roots, base.nodes, base.bricks, base.palette, node_headroom=400000,
                        brick_headroom=100000)
    tracer.set_camera(cam)
    vol = orc.scene_volume(L.SceneParams(grid=(1, 1, 1), seed=77), (0, 0, 0))
    vol[:, 120:, :] = 0
    pn, pb = orc.build_chunk_dense(vol)
    node_off, brick_off = len(base.nodes), len(base.bricks)
    rel = pn.copy()
    ptr = rel["child_ptr"].astype(np.int64)
    leaf, uni = (ptr & 0x80000000) != 0, (ptr & 0x40000000) != 0
    loc = ptr & 0x3FFFFFFF
    rel["child_ptr"] = np.where(leaf, np.where(uni, ptr & 0xC0000000, (ptr & 0xC0000000) | (loc + brick_off)),
                                loc + node_off).astype(np.uint32)
    chunk = 3
    tracer.apply_patch(chunk, node_off, node_off, rel, brick_off, pb)
    roots = base.roots.copy()
    roots[chunk] = node_off
    patched = orc.World(base.grid, roots, np.concatenate([base.nodes, rel]), np.concatenate([base.bricks, pb]))
    rays = _random_rays(30000, base.grid, np.random.default_rng(3))
    _assert_hits_equal(tracer.trace_rays(rays, 60.0), orc.trace_rays(patched, cam, rays, 60.0, 0, False, threads=THREADS),
                       "after append patch")
    tracer.apply_patch(1, 0xFFFFFFFF, 0, np.zeros(0, L.NODE_DTYPE), 0, np.zeros(0, L.BRICK_DTYPE))
    roots[1] = 0xFFFFFFFF
    patched = orc.World(base.grid, roots, patched.nodes, patched.bricks)
    _assert_hits_equal(tracer.trace_rays(rays, 60.0), orc.trace_rays(patched, cam, rays, 60.0, 0, False, threads=THREADS),
                       "after empty patch")


def test_shadow_rays_di(orc, tracer, world_cache):
    """trace_shadow_vis_di: rays between nearby visible surface points, 30 % of the visible bricks
    recoloured to the emissive ids, each ray with its own target distance. Bit-exact against the
    oracle; both outcomes occur, and some rays are visible only because their target is emissive
    (the emitter early-out)."""
    import torch
    from arcadia_gb300.layout import EDIT_DTYPE, EDIT_RECOLOR
    from arcadia_gb300.native import lib

    W, H = 320, 180
    w = world_cache("c2_1024_caves")
    cam = L.default_camera_for(L.SCENES["c2_1024_caves"], W, H, quality=L.quality_high())
    _load(tracer, w, cam)
    hits = tracer.trace_frame()[3]
    rng = np.random.default_rng(31)
    is_hit = (hits["flags"] & 1).astype(bool)
    vox = hits["voxel"].astype(np.int64)
    hit_px = np.nonzero(is_hit)[0]
    emit_px = rng.choice(hit_px, int(0.3 * len(hit_px)), replace=False)
    ops = np.zeros(len(emit_px), EDIT_DTYPE)
    ops["kind"] = EDIT_RECOLOR
    ops["brick"] = (vox[emit_px] >> 2).astype(np.uint32)
    ops["material"] = rng.choice([19, 20, 21, 22, 24, 27], len(emit_px))
    ew = orc.apply_edits(w, ops)
    # ray pairs: a hit pixel and a hit pixel within +-12 pixels of it
    src = rng.choice(hit_px, 8000)
    sx, sy = src % W + rng.integers(-12, 13, len(src)), src // W + rng.integers(-12, 13, len(src))
    ok = (sx >= 0) & (sx < W) & (sy >= 0) & (sy < H)
    src, dst = src[ok], (sy * W + sx)[ok]
    ok = is_hit[dst] & (np.abs(vox[src] - vox[dst]).max(1) > 2)
    src, dst = src[ok], dst[ok]
    o = (vox[src].astype(np.float32) + np.float32(0.5)) * np.float32(0.0625) + np.array([0, 0.04, 0], np.float32)
    tgt = (vox[dst].astype(np.float32) + np.float32(0.5)) * np.float32(0.0625)
    d = tgt - o
    dist = np.sqrt((d * d).sum(1)).astype(np.float32)
    d = (d / dist[:, None]).astype(np.float32)
    rays = np.zeros(len(o), L.RAY_DTYPE)
    rays["origin_m"] = o
    rays["dir"] = d
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_max = torch.from_numpy(dist.copy()).cuda()

    def gpu_vis(world):
        _load(tracer, world, cam)
        out = torch.zeros(len(rays), dtype=torch.float32, device="cuda")
        assert lib().arc_shadow_rays_di_dev(tracer.ctx, d_rays.data_ptr(), d_max.data_ptr(), len(rays), out.data_ptr()) == 0
        tracer.synchronize()
        return out.cpu().numpy()

    vis = gpu_vis(ew)
    ovis = np.array([orc.shadow_vis_di(ew, cam, r["origin_m"], r["dir"], float(m)) for r, m in zip(rays, dist)], np.float32)
    np.testing.assert_array_equal(vis, ovis)
    assert 0.05 < vis.mean() < 0.95, vis.mean()
    plain = gpu_vis(w)  # same rays, no emitters in the world
    assert np.all(plain <= vis) and (vis > plain).sum() > 20


def test_host_frame_into_pinned_buffers(tracer, world_cache):
    """arc_trace_frame into page-locked host buffers and into pageable buffers (both filled by the
    library's banded device-to-host copies) and arc_trace_frame_dev on the device: identical results."""
    import torch

    w = world_cache("c1_256")
    W, H = 480, 270
    cam = L.default_camera_for(L.SCENES["c1_256"], W, H, quality=L.quality_high(), frame_index=5)
    _load(tracer, w, cam)
    pageable = tracer.trace_frame()
    pinned = [torch.zeros(m, dtype=torch.int32).pin_memory() for m in (W * H * 2, W * H * 2, W * H, W * H * 5, W * H * 5)]
    import ctypes

    from arcadia_gb300.native import lib

    n = ctypes.c_uint64(0)
    assert lib().arc_trace_frame(tracer.ctx, W, H, *[p.data_ptr() for p in pinned], ctypes.byref(n)) == 0
    dev = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (W * H * 2, W * H * 2, W * H, W * H * 5, W * H * 5)]
    tracer.trace_frame_dev(W, H, *[d.data_ptr() for d in dev])
    tracer.synchronize()
    for a, b, c in zip(pageable[:5], pinned, dev):
        a = np.ascontiguousarray(a).view(np.int32).reshape(-1)
        assert np.array_equal(a, b.numpy()) and np.array_equal(a, c.cpu().numpy())
    assert n.value == pageable[5]


def test_banded_device_frame_in_cuda_graph(orc, tracer, world_cache, native_lib):
    """arc_trace_frame_dev in four concurrent row bands, captured into a CUDA graph on the library's
    stream after one direct call (which creates the band streams): the replay writes the same words as
    the direct call, and those equal the oracle's."""
    torch = pytest.importorskip("torch")
    w = world_cache("c1_256")
    W, H = 1280, 720
    cam = L.default_camera_for(L.SCENES["c1_256"], W, H, quality=L.quality_high(), frame_index=5)
    _load(tracer, w, cam)
    n = W * H
    bufs = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (2 * n, 2 * n, n, 5 * n, 5 * n)]
    n_gi = torch.zeros(1, dtype=torch.int64, device="cuda")
    ptrs = [x.data_ptr() for x in bufs] + [n_gi.data_ptr()]
    assert native_lib.lib().arc_set_frame_bands(tracer.ctx, 4) == 0
    try:
        tracer.trace_frame_dev(W, H, *ptrs)
        tracer.synchronize()
        direct = [x.clone() for x in bufs]
        n_direct = int(n_gi.item())
        for x in bufs:
            x.fill_(-1)
        n_gi.zero_()
        stream = torch.cuda.ExternalStream(tracer.stream())
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            g.capture_begin(capture_error_mode="thread_local")
            tracer.trace_frame_dev(W, H, *ptrs)
            g.capture_end()
        for x in bufs:  # nothing ran during the capture
            assert (x == -1).all()
        g.replay()
        torch.cuda.synchronize()
        for got, want in zip(bufs, direct):
            assert torch.equal(got, want)
        assert int(n_gi.item()) == n_direct
    finally:
        native_lib.lib().arc_set_frame_bands(tracer.ctx, 0)
    ogdm, ognm, ogaa, ohits, _ = orc.primary(w, cam, threads=THREADS)
    _, ogi, _ = orc.gi_rays(w, cam, ogdm, ognm, threads=THREADS)
    got = [x.cpu().numpy().view(np.uint32) for x in bufs]
    np.testing.assert_array_equal(got[0].reshape(-1, 2), ogdm)
    np.testing.assert_array_equal(got[2], ogaa)
    _assert_hits_equal(got[3].view(L.HIT_DTYPE), ohits, "primary, graph replay")
    _assert_hits_equal(got[4].view(L.HIT_DTYPE), ogi, "GI, graph replay")
