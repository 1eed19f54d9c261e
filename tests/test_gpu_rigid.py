"""Rigid voxel bodies on the GPU against the oracle (trace_rigid_bodies, traversal64.wgsl:1006-1244,
and its callers: primary_gbuffer.wgsl:121-136 and 183-253, lighting_restir_gi.wgsl:209-224).

Three instances of one body tree (stone block with a pillar chequer, a mirror layer) in front of the
256^3 world's camera, moving and turning between frames. Bar: hit records (with the rigid flag,
body index and body-local voxel), per-ray hit points and normals, every G-buffer word, GI hit
records and ReSTIR reservoirs bit-exact against the oracle.
"""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

from test_rigid import world_with_bodies

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
W, H = 640, 360


@pytest.fixture(scope="module")
def tracer(native_lib):
    t = native_lib.Tracer(0)
    yield t
    t.close()


@pytest.fixture(scope="module")
def body_world(orc, world_cache):
    return world_with_bodies(orc, world_cache("c1_256"))[0]


def _load(t, w, cam):
    t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette, node_headroom=4096, brick_headroom=1024)
    t.set_rigid_bodies(w.bodies)
    t.set_camera(cam)


def _cam(n_bodies, width=W, height=H, frame=3, underwater=False):
    cam = L.default_camera_for(L.SCENES["c1_256"], width, height, quality=L.quality_high(), frame_index=frame)
    cam[0]["point_light_count"][1] = (n_bodies << 16) | (1 if underwater else 0)
    cam[0]["cam_pos_time"][3] = 4.0
    return cam


def _same(got, want, what):
    g, o = np.asarray(got).view(np.uint32).reshape(-1), np.asarray(want).view(np.uint32).reshape(-1)
    bad = np.nonzero(g != o)[0]
    assert len(bad) == 0, f"{what}: {len(bad)} words differ, first {bad[:5]}: gpu {g[bad[:3]]} oracle {o[bad[:3]]}"


def test_rigid_rays_bitexact(orc, tracer, body_world):
    import torch

    w = body_world
    cam = _cam(len(w.bodies))
    _load(tracer, w, cam)
    rng = np.random.default_rng(9)
    rays = np.zeros(20000, L.RAY_DTYPE)
    eye = cam[0]["cam_pos_time"][:3].astype(np.float64)
    for i in range(len(rays)):
        b = w.bodies[i % len(w.bodies)]
        l2w = b["local_to_world"].reshape(4, 4).T.astype(np.float64)
        target = (l2w @ np.append(rng.uniform(-0.1, 1.1, 3) * np.array([24, 16, 20]) * 0.0625, 1.0))[:3]
        o = eye + rng.normal(scale=1.5, size=3)
        d = target - o
        rays[i]["origin_m"] = o
        rays[i]["dir"] = d / np.linalg.norm(d)
    d_rays = torch.from_numpy(rays.view(np.uint8).copy()).cuda()
    d_hits = torch.zeros(len(rays) * 20, dtype=torch.uint8, device="cuda")
    d_det = torch.zeros(len(rays) * 9, dtype=torch.float32, device="cuda")
    tracer.trace_rigid_bodies_dev(d_rays.data_ptr(), len(rays), 30.0, d_hits.data_ptr(), d_det.data_ptr())
    tracer.synchronize()
    hits = d_hits.cpu().numpy().view(L.HIT_DTYPE)
    ohits, odet = orc.trace_rigid_rays(w, cam, rays, 30.0, threads=THREADS)
    _same(hits, ohits, "hit records")
    _same(d_det.cpu().numpy(), odet, "hit point / previous point / normal")
    hit = (hits["flags"] & 1).astype(bool)
    assert 0.3 < hit.mean() < 0.98
    assert len(np.unique((hits["flags"][hit] >> 8) & 31)) == len(w.bodies)


@pytest.mark.parametrize("variant", [0, 1])
def test_frame_with_rigid_bodies_bitexact(orc, tracer, body_world, variant):
    w = body_world
    cam = _cam(len(w.bodies))
    _load(tracer, w, cam)
    tracer.set_launch_config(variant=variant)
    gdm, gnm, gaa, hits, gi, _ = tracer.trace_frame()
    ogdm, ognm, ogaa, ohits, _ = orc.primary(w, cam, threads=THREADS)
    _, ogi, _ = orc.gi_rays(w, cam, ogdm, ognm, threads=THREADS)
    for g, o, what in ((gdm, ogdm, "gbuf_depth_mat"), (gnm, ognm, "gbuf_norm_motion"), (gaa, ogaa, "gbuf_albedo_ao"),
                       (hits, ohits, "hits"), (gi, ogi, "gi_hits")):
        _same(g, o, what)
    rigid_px = (gdm[:, 1] >> 16) == 1
    assert rigid_px.sum() > 2000, rigid_px.sum()
    assert ((hits["flags"] & 0x10) != 0).sum() == rigid_px.sum()
    assert ((gi["flags"] & 0x10) != 0).sum() > 50
    # a camera that names no bodies runs the regular frame kernels: no pixel is a body
    tracer.set_camera(_cam(0))
    g0 = tracer.trace_frame()[0]
    assert ((g0[:, 1] >> 16) == 0).all()


def test_surface_rays_see_rigid_bodies(orc, tracer, body_world):
    """Water in the world, mirror voxels on the bodies: refraction, reflection and mirror rays all
    trace the bodies after the world (primary_gbuffer.wgsl:183, 223, 253)."""
    from arcadia_gb300.layout import EDIT_DTYPE, EDIT_RECOLOR

    w = body_world
    cam = _cam(len(w.bodies))
    _load(tracer, w, cam)
    hits = tracer.trace_frame()[3]
    world_hit = ((hits["flags"] & 1) != 0) & ((hits["flags"] & 0x10) == 0)
    bricks = np.unique(hits["voxel"][world_hit].astype(np.int64) >> 2, axis=0)
    rng = np.random.default_rng(4)
    pick = bricks[rng.choice(len(bricks), len(bricks) // 2, replace=False)]
    ops = np.zeros(len(pick), EDIT_DTYPE)
    ops["kind"] = EDIT_RECOLOR
    ops["brick"] = pick.astype(np.uint32)
    ops["material"] = np.where(rng.random(len(pick)) < 0.7, 18, 28)
    ew = orc.apply_edits(w, ops).with_bodies(w.bodies)
    for pitch in (-30.0, -14.0):
        cam = L.default_camera_for(L.SCENES["c1_256"], W, H, quality=L.quality_high(), frame_index=5, pitch_deg=pitch)
        cam[0]["point_light_count"][1] = len(w.bodies) << 16
        _load(tracer, ew, cam)
        gdm, gnm, gaa, h, gi, _ = tracer.trace_frame()
        ogdm, ognm, ogaa, ohits, _ = orc.primary(ew, cam, threads=THREADS)
        _, ogi, _ = orc.gi_rays(ew, cam, ogdm, ognm, threads=THREADS)
        for g, o, what in ((gdm, ogdm, "gbuf_depth_mat"), (gnm, ognm, "gbuf_norm_motion"), (gaa, ogaa, "gbuf_albedo_ao"),
                           (h, ohits, "hits"), (gi, ogi, "gi_hits")):
            _same(g, o, what)
        mat = gdm[:, 1] & 0xFFFF
        assert (mat == 18).sum() > 500 and (mat == 28).sum() > 200


def test_restir_with_rigid_bodies(orc, tracer, body_world):
    import torch

    w = body_world
    npx = W * H
    dev = torch.device("cuda")
    gdm, gnm = (torch.zeros(npx * 2, dtype=torch.int32, device=dev) for _ in range(2))
    gaa = torch.zeros(npx, dtype=torch.int32, device=dev)
    hits, gi = (torch.zeros(npx * 5, dtype=torch.int32, device=dev) for _ in range(2))
    res = [torch.from_numpy(L.empty_reservoirs(npx).view(np.uint8).copy()).to(dev) for _ in range(2)]
    rng = np.random.default_rng(8)
    _load(tracer, w, _cam(len(w.bodies)))
    tracer.sharc_reset()
    for f in range(3):
        cam = _cam(len(w.bodies), frame=f + 1)
        tracer.set_camera(cam)
        tracer.trace_frame_dev(W, H, gdm.data_ptr(), gnm.data_ptr(), gaa.data_ptr(), hits.data_ptr(), gi.data_ptr())
        tracer.sharc_update_dev(W, H, gdm.data_ptr(), gnm.data_ptr())
        tracer.sharc_resolve()
        radiance = None
        d_rad = None
        if f == 2:
            radiance = rng.random((npx, 3), dtype=np.float32)
            d_rad = torch.from_numpy(radiance).to(dev)
        r_in, r_out = res[f % 2], res[(f + 1) % 2]
        tracer.restir_gi_temporal_dev(W, H, gdm.data_ptr(), gnm.data_ptr(), gi.data_ptr(), r_in.data_ptr(), r_out.data_ptr(),
                                      d_rad.data_ptr() if d_rad is not None else 0)
        tracer.synchronize()
        want = orc.restir_gi_temporal(w, cam, tracer.sharc_download()[2], gdm.cpu().numpy(), gnm.cpu().numpy(),
                                      r_in.cpu().numpy().view(L.RESERVOIR_DTYPE), radiance=radiance, threads=THREADS)
        _same(r_out.cpu().numpy(), want, f"reservoirs, frame {f}")


def test_batched_views_reject_rigid_cameras(native_lib, tracer, body_world):
    import torch

    w = body_world
    _load(tracer, w, _cam(len(w.bodies)))
    table = np.zeros(1, L.VIEW_DTYPE)
    bufs = [torch.zeros(n, dtype=torch.int32, device="cuda") for n in (W * H * 2, W * H * 2, W * H, W * H * 5, W * H * 5)]
    table[0]["world_slot"] = 0
    table[0]["width"], table[0]["height"] = W, H
    table[0]["cam"] = _cam(len(w.bodies))[0]
    for f, b in zip(("gbuf_depth_mat", "gbuf_norm_motion", "gbuf_albedo_ao", "hits", "gi_hits"), bufs):
        table[0][f] = b.data_ptr()
    with pytest.raises(native_lib.ArcError):
        tracer.trace_views_dev(table, use_graph=False)
    table[0]["cam"] = _cam(0)[0]
    tracer.trace_views_dev(table, use_graph=False)
    tracer.synchronize()
    tracer.set_rigid_bodies(np.zeros(0, L.RIGID_BODY_DTYPE))
