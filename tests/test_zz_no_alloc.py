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
    """variant 0: the plain kernel, whose GI pass runs over the G-buffer rows here (no GI list to
    allocate) and over the listed hit pixels in arc_trace_frame_dev; variant 1: the persistent kernel."""
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
