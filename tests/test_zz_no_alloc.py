"""The allocation-free frame entry point against the regular one, through the C ABI.

arc_trace_frame_noalloc serves callers that cannot allocate device memory while they trace (a frame
loop under a no-allocation rule or a fixed memory budget): its kernels keep their scratch in a static
device array instead of context memory. It must produce exactly what arc_trace_frame_dev produces
(all outputs are integer words, so the tolerance is zero) on consecutive calls, since every call
reuses the same array. This file sorts last so a failure here comes after every other test has run.
"""
import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu


def _outputs(torch, npx):
    dev = torch.device("cuda")
    return [torch.zeros(n, dtype=torch.int32, device=dev) for n in (npx * 2, npx * 2, npx, npx * 5, npx * 5)] + [
        torch.zeros(1, dtype=torch.int64, device=dev)]


@pytest.mark.parametrize("variant", [0, 1])
def test_noalloc_frame_matches_regular_entry_point(native_lib, variant):
    """variant 0: the plain kernel, then the frame's GI pass over the G-buffer rows (both entry points
    run the same row GI pass, so this compares the scratch placement, not two GI strategies);
    variant 1: the persistent kernel, whose queue head lives in the scratch."""
    torch = pytest.importorskip("torch")
    scene = L.SCENES["c1_256"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        t.set_launch_config(variant=variant)
        w, h = 640, 360
        for frame in (5, 6):  # two calls in a row: the shared static scratch must be cleared each time
            t.set_camera(L.default_camera_for(scene, w, h, quality=L.quality_high(), frame_index=frame))
            ref = _outputs(torch, w * h)
            t.trace_frame_dev(w, h, *[x.data_ptr() for x in ref])
            t.synchronize()
            out = _outputs(torch, w * h)
            torch.cuda.synchronize()
            free_before = torch.cuda.mem_get_info()[0]
            t.trace_frame_noalloc(w, h, *[x.data_ptr() for x in out])
            t.synchronize()
            # the first call on a device looks up the static array (the driver may load its module then);
            # from the second call on nothing may change device memory
            if frame == 6:
                assert torch.cuda.mem_get_info()[0] == free_before, "the allocation-free entry point allocated memory"
            for a, b in zip(out, ref):
                assert torch.equal(a, b)
            assert int(out[5].item()) > 0
    finally:
        t.close()


def test_noalloc_rejects_oversize_frames(native_lib):
    pytest.importorskip("torch")
    scene = L.SCENES["c1_256"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        t.set_camera(L.default_camera_for(scene, 9000, 8000, quality=L.quality_high()))
        with pytest.raises(native_lib.ArcError) as e:
            t.trace_frame_noalloc(9000, 8000, 16, 16, 16)  # rejected before any pointer is used
        assert e.value.code == -8 and "allocation-free limit" in str(e.value)
    finally:
        t.close()


def test_noalloc_surface_list(native_lib):
    """A world with water and mirror voxels (recoloured by the library's own edit path) and an underwater
    camera: both need the surface list of the shading branches. Before it is reserved the allocation-free
    call fails with ARC_E_CAPACITY (it may not allocate the list itself); after arc_reserve_surface_list
    it matches arc_trace_frame_dev word for word on consecutive calls, whose surface-entry counter lives
    in the shared static array."""
    torch = pytest.importorskip("torch")
    from arcadia_gb300.layout import EDIT_DTYPE, EDIT_RECOLOR

    scene = L.SCENES["c1_256"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    w, h = 640, 360
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette(), node_headroom=4096,
                       brick_headroom=4096)
        cam = L.default_camera_for(scene, w, h, quality=L.quality_high(), frame_index=3)
        t.set_camera(cam)
        hits = t.trace_frame()[3]
        vox = hits["voxel"][(hits["flags"] & 1).astype(bool)].astype(np.int64)
        picked = np.unique(vox >> 2, axis=0)
        rng = np.random.default_rng(43)
        picked = picked[rng.choice(len(picked), int(0.4 * len(picked)), replace=False)]
        ops = np.zeros(len(picked), EDIT_DTYPE)
        ops["kind"] = EDIT_RECOLOR
        ops["brick"] = picked.astype(np.uint32)
        ops["material"] = np.where(rng.random(len(picked)) < 0.75, 18, 28)
        t.apply_edits(ops)
        t.synchronize()
        out = _outputs(torch, w * h)
        with pytest.raises(native_lib.ArcError) as e:
            t.trace_frame_noalloc(w, h, *[x.data_ptr() for x in out])
        assert e.value.code == -8 and "surface list" in str(e.value)
        assert native_lib.lib().arc_reserve_surface_list(t.ctx, w * h) == 0
        for frame, underwater in ((5, False), (6, False), (7, True), (8, True)):
            c = L.default_camera_for(scene, w, h, quality=L.quality_high(), frame_index=frame)
            if underwater:
                c[0]["point_light_count"][1] = 1
            t.set_camera(c)
            ref = _outputs(torch, w * h)
            t.trace_frame_dev(w, h, *[x.data_ptr() for x in ref])
            t.synchronize()
            out = _outputs(torch, w * h)
            t.trace_frame_noalloc(w, h, *[x.data_ptr() for x in out])
            t.synchronize()
            for a, b in zip(out, ref):
                assert torch.equal(a, b), (frame, underwater)
            if frame == 6:
                mats = ref[0].cpu().numpy().view(np.uint32).reshape(-1, 2)[:, 1] & 0xFF
                assert ((mats == 18) | (mats == 28)).sum() > 1000  # the branches ran on many pixels
    finally:
        t.close()
