"""ReSTIR GI temporal pass (temporal_main, lighting_restir_gi.wgsl:61-336) on the GPU against the oracle.

Five frames along a moving camera (motion vectors and prev_cam_pos from the previous camera), each:
frame kernel -> SHARC update + resolve -> temporal pass with the previous frame's reservoirs. The GPU
pass reuses the frame kernel's GI hit records; the oracle traces the GI ray again, as the reference
does. Bar: every 32 B reservoir bit-exact, given the same G-buffer, history and SHARC state.
"""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu
THREADS = os.cpu_count() or 8
W, H = 480, 270


@pytest.fixture(scope="module")
def tracer(native_lib):
    t = native_lib.Tracer(0)
    yield t
    t.close()


def _path_cameras(scene, q, n):
    """n cameras drifting right and turning 1.5 degrees per frame, each carrying the previous one's
    view-projection and position."""
    gx, gy, gz = scene.grid
    base = np.array([gx * 256 * 0.5, gy * 256 * (220.0 / 256.0), gz * 256 * 0.5]) * 0.0625
    cams, prev_vp, prev_eye = [], None, None
    for f in range(n):
        eye = base + np.array([0.06 * f, 0.0, 0.04 * f])
        cam = L.camera_uniforms(scene.grid, W, H, eye, yaw_deg=1.5 * f, pitch_deg=-30.0, quality=q, frame_index=f + 1,
                                prev_eye_m=prev_eye, prev_view_proj=prev_vp)
        cams.append(cam)
        prev_vp = cam[0]["curr_view_proj"].reshape(4, 4).T.copy()
        prev_eye = eye
    return cams


@pytest.mark.parametrize("mode", ["sharc", "sharc_low_taps_shadow_vis", "radiance_buffer"])
def test_restir_gi_temporal_matches_oracle(orc, tracer, world_cache, mode):
    import torch

    scene = L.SCENES["c2_1024_caves"]
    w = world_cache("c2_1024_caves")
    q = L.quality_high()
    if mode == "sharc_low_taps_shadow_vis":
        q.denoiser_taps = 8  # checkerboard half rate
        q.shadow_mode = 1    # trace_shadow_vis for the sun ray
    tracer.upload_world(w.grid, w.roots, w.nodes, w.bricks, w.palette)
    tracer.set_launch_config(variant=0)
    tracer.sharc_reset()
    npx = W * H
    dev = torch.device("cuda")
    gdm, gnm = (torch.zeros(npx * 2, dtype=torch.int32, device=dev) for _ in range(2))
    gaa = torch.zeros(npx, dtype=torch.int32, device=dev)
    hits, gi = (torch.zeros(npx * 5, dtype=torch.int32, device=dev) for _ in range(2))
    res = [torch.from_numpy(L.empty_reservoirs(npx).view(np.uint8).copy()).to(dev) for _ in range(2)]
    rng = np.random.default_rng(5)
    stats = []
    for f, cam in enumerate(_path_cameras(scene, q, 5)):
        tracer.set_camera(cam)
        tracer.trace_frame_dev(W, H, gdm.data_ptr(), gnm.data_ptr(), gaa.data_ptr(), hits.data_ptr(), gi.data_ptr())
        radiance, d_rad = None, None
        if mode == "radiance_buffer":
            radiance = rng.random((npx, 3), dtype=np.float32) * np.float32(2.0)
            d_rad = torch.from_numpy(radiance).to(dev)
        else:
            tracer.sharc_update_dev(W, H, gdm.data_ptr(), gnm.data_ptr())
            tracer.sharc_resolve()
        r_in, r_out = res[f % 2], res[(f + 1) % 2]
        tracer.restir_gi_temporal_dev(W, H, gdm.data_ptr(), gnm.data_ptr(), gi.data_ptr(), r_in.data_ptr(),
                                      r_out.data_ptr(), d_rad.data_ptr() if d_rad is not None else 0)
        tracer.synchronize()
        got = r_out.cpu().numpy().view(L.RESERVOIR_DTYPE)
        resolved = tracer.sharc_download()[2]
        want = orc.restir_gi_temporal(w, cam, resolved, gdm.cpu().numpy(), gnm.cpu().numpy(),
                                      r_in.cpu().numpy().view(L.RESERVOIR_DTYPE), radiance=radiance, threads=THREADS)
        gw, ow = got.view(np.uint32).reshape(npx, 8), want.view(np.uint32).reshape(npx, 8)
        bad = np.nonzero((gw != ow).any(1))[0]
        assert len(bad) == 0, f"frame {f}: {len(bad)} reservoirs differ, first {bad[:4]}: gpu {gw[bad[:2]]} oracle {ow[bad[:2]]}"
        nmf = got["norm_m_flags"]
        hit = got["primary_depth"] < 1e4
        stats.append(dict(m_gt1=float((((nmf >> 16) & 0xFF) > 1)[hit].mean()), aged=int(((nmf >> 24) & 0x7F)[hit].astype(bool).sum()),
                          sky=int((nmf >> 31)[hit].sum()), lit=float((got["lo_rg"] != 0)[hit].mean())))
    assert stats[0]["m_gt1"] == 0.0
    assert all(s["m_gt1"] > 0.3 for s in stats[1:]), stats
    assert all(s["sky"] > 100 for s in stats), stats
    assert stats[-1]["aged"] > 100, stats
    assert all(s["lit"] > 0.3 for s in stats), stats
