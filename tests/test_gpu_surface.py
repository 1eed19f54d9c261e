"""Primary-pass surface branches (primary_gbuffer.wgsl:163-295) on the GPU against the oracle.

A water hit (material 18) traces a refraction ray to the bed and, at grazing angles, a reflection
ray, and stores the up normal (which the GI ray then starts from); a mirror hit (material 28) traces
a reflection ray (and a second one past its own seam); an underwater camera gives every hit caustics
and absorption. Worlds get water and mirrors by recolour edits applied on both sides (the oracle's
restatement of the reference edit path is node-for-node equal to the GPU's). Bar: every G-buffer
word and hit record bit-exact, on every frame entry point (device, host banded, allocation-free,
batched views).
"""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
W, H = 640, 360


@pytest.fixture(scope="module")
def tracer(native_lib):
    t = native_lib.Tracer(0)
    yield t
    t.close()


def _load(t, w, cam):
    t.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette, node_headroom=4096, brick_headroom=1024)
    t.set_camera(cam)


def _cam(width=W, height=H, frame=3, underwater=False, yaw=0.0, pitch=-30.0):
    """The benchmark camera of the 256^3 world at t = 12.5 s, with three point lights in front of it."""
    scene = L.SCENES["c1_256"]
    cam = L.default_camera_for(scene, width, height, quality=L.quality_high(), frame_index=frame, yaw_deg=yaw,
                               pitch_deg=pitch)
    c = cam[0]
    c["cam_pos_time"][3] = 12.5
    eye, fwd = c["cam_pos_time"][:3].copy(), c["cam_forward_fov"][:3].copy()
    c["point_light_count"][0] = 3
    for i, (dist, side) in enumerate(((4.0, -2.0), (7.0, 1.5), (10.0, 0.0))):
        c["point_light"][i] = [eye[0] + fwd[0] * dist + side, eye[1] + fwd[1] * dist, eye[2] + fwd[2] * dist, 2.0 + i]
    if underwater:
        c["point_light_count"][1] = 1
    return cam


@pytest.fixture(scope="module")
def surface_world(orc, world_cache, tracer):
    """The 256^3 world with 40 % of the bricks the camera sees recoloured: three quarters to water,
    one quarter to mirror chrome."""
    from arcadia_gb300.layout import EDIT_DTYPE, EDIT_RECOLOR

    w = world_cache("c1_256")
    _load(tracer, w, _cam())
    hits = tracer.trace_frame()[3]
    vox = hits["voxel"][(hits["flags"] & 1).astype(bool)].astype(np.int64)
    bricks = np.unique(vox >> 2, axis=0)
    rng = np.random.default_rng(41)
    pick = bricks[rng.choice(len(bricks), int(0.4 * len(bricks)), replace=False)]
    ops = np.zeros(len(pick), EDIT_DTYPE)
    ops["kind"] = EDIT_RECOLOR
    ops["brick"] = pick.astype(np.uint32)
    ops["material"] = np.where(rng.random(len(pick)) < 0.75, 18, 28)
    return orc.apply_edits(w, ops)


def _oracle_frame(orc, w, cam):
    ogdm, ognm, ogaa, ohits, _ = orc.primary(w, cam, threads=THREADS)
    _, ogi, _ = orc.gi_rays(w, cam, ogdm, ognm, threads=THREADS)
    return ogdm, ognm, ogaa, ohits, ogi


def _assert_frame_equal(got, want):
    for g, o, what in zip(got, want, ("gbuf_depth_mat", "gbuf_norm_motion", "gbuf_albedo_ao", "hits", "gi_hits")):
        g = np.asarray(g).view(np.uint32).reshape(-1)
        o = np.asarray(o).view(np.uint32).reshape(-1)
        bad = np.nonzero(g != o)[0]
        assert len(bad) == 0, f"{what}: {len(bad)} words differ, first {bad[:5]}: gpu {g[bad[:3]]} oracle {o[bad[:3]]}"


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("pitch", [-30.0, -12.0])
def test_water_and_mirror_bitexact(orc, tracer, surface_world, variant, pitch):
    """At -12 degrees most water hits are grazing enough to trace the reflection ray as well."""
    cam = _cam(pitch=pitch)
    _load(tracer, surface_world, cam)
    tracer.set_launch_config(variant=variant)
    gdm, gnm, gaa, hits, gi, _ = tracer.trace_frame()
    want = _oracle_frame(orc, surface_world, cam)
    _assert_frame_equal((gdm, gnm, gaa, hits, gi), want)
    mat = gdm[:, 1] & 0xFFFF
    water, mirror = mat == 18, mat == 28
    assert water.sum() > 2000 and mirror.sum() > 500, (water.sum(), mirror.sum())
    assert len(np.unique(gaa[water] & 0xFFFFFF)) > 20
    # water stores the up normal (octahedral (0, 1) -> snorm words 0, 32767)
    up = np.uint32(0) | (np.uint32(32767) << 16)
    assert np.all(gnm[water, 0] == up)
    # the branches replaced the palette albedo (water 0.06, 0.28, 0.38 -> about 15, 71, 97)
    rgb = np.stack([(gaa >> s) & 0xFF for s in (0, 8, 16)], 1).astype(np.int32)
    plain = np.abs(rgb[water] - np.array([15, 71, 97])).max(1) <= 3
    assert plain.mean() < 0.5, plain.mean()
    assert len(np.unique(rgb[mirror], axis=0)) > 50


def test_underwater_camera_bitexact(orc, tracer, world_cache):
    w = world_cache("c1_256")
    cam = _cam(underwater=True)
    _load(tracer, w, cam)
    tracer.set_launch_config(variant=0)
    got = tracer.trace_frame()
    _assert_frame_equal((got[0], got[1], got[2], got[3], got[4]), _oracle_frame(orc, w, cam))
    dry = _cam()
    tracer.set_camera(dry)
    plain = tracer.trace_frame()[2]
    hit = (got[0][:, 0] != np.float32(1e5).view(np.uint32))
    changed = ((got[2] ^ plain) & 0x00FFFFFF) != 0
    assert changed[hit].mean() > 0.9, changed[hit].mean()


def test_surface_on_every_frame_entry_point(native_lib, tracer, surface_world):
    """Device, host (banded, concurrent and sequential bands) and allocation-free frames agree; the
    allocation-free one needs the surface list reserved."""
    import torch

    npx = W * H
    cam = _cam(frame=7)

    def dev_bufs():
        return [torch.zeros(n, dtype=torch.int32, device="cuda") for n in (npx * 2, npx * 2, npx, npx * 5, npx * 5)]

    fresh = native_lib.Tracer(0)
    try:
        _load(fresh, surface_world, cam)
        out = dev_bufs()
        with pytest.raises(native_lib.ArcError) as e:
            fresh.trace_frame_noalloc(W, H, *[b.data_ptr() for b in out])
        assert e.value.code == -8, e.value
        fresh.reserve_surface_list(npx)
        fresh.trace_frame_noalloc(W, H, *[b.data_ptr() for b in out])
        fresh.synchronize()
        noalloc = [b.cpu().numpy() for b in out]
    finally:
        fresh.close()
    results = [noalloc]
    for variant in (0, 1):
        _load(tracer, surface_world, cam)
        tracer.set_launch_config(variant=variant)
        ref = dev_bufs()
        tracer.trace_frame_dev(W, H, *[b.data_ptr() for b in ref])
        tracer.synchronize()
        results.append([b.cpu().numpy() for b in ref])
        host = tracer.trace_frame()
        results.append([host[i] for i in range(5)])
    for r in results[1:]:
        _assert_frame_equal(r, results[0])


@pytest.mark.parametrize("use_graph", [False, True])
def test_surface_batched_views(native_lib, tracer, surface_world, use_graph):
    """Two views of the water/mirror world in one batched launch equal two single-view frames."""
    import torch

    shapes = [(640, 360, 0.0, -30.0), (320, 240, 25.0, -40.0)]
    _load(tracer, surface_world, _cam())
    tracer.set_launch_config(variant=0)
    table = np.zeros(len(shapes), L.VIEW_DTYPE)
    bufs, cams = [], []
    for i, (w, h, yaw, pitch) in enumerate(shapes):
        cam = _cam(w, h, frame=2, yaw=yaw, pitch=pitch)
        cams.append(cam)
        b = [torch.zeros(n, dtype=torch.int32, device="cuda") for n in (w * h * 2, w * h * 2, w * h, w * h * 5, w * h * 5)]
        bufs.append(b)
        table[i]["world_slot"] = 0
        table[i]["width"], table[i]["height"] = w, h
        table[i]["cam"] = cam[0]
        for f, buf in zip(("gbuf_depth_mat", "gbuf_norm_motion", "gbuf_albedo_ao", "hits", "gi_hits"), b):
            table[i][f] = buf.data_ptr()
    for _ in range(2):  # a replayed graph re-shades the list of its own launch
        tracer.trace_views_dev(table, use_graph=use_graph)
        tracer.synchronize()
    for (w, h, _, _), cam, b in zip(shapes, cams, bufs):
        tracer.set_camera(cam)
        ref = [torch.zeros_like(x) for x in b]
        tracer.trace_frame_dev(w, h, *[x.data_ptr() for x in ref])
        tracer.synchronize()
        _assert_frame_equal([x.cpu().numpy() for x in b], [x.cpu().numpy() for x in ref])
        mat = b[0].cpu().numpy().reshape(-1, 2)[:, 1] & 0xFFFF
        assert (mat == 18).sum() > 100
