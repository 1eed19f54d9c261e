"""Batched multi-view launch (several worlds, mixed resolutions, one persistent launch, CUDA graph):
every view's G-buffer and hit records equal a single-view trace of the same camera, bit for bit."""
import os

import numpy as np
import pytest

from arcadia_gb300 import layout as L

pytestmark = pytest.mark.gpu


def _single(native_lib, world, scene, cam, w, h):
    import torch

    t = native_lib.Tracer(0)
    try:
        roots, nodes, bricks = world
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        t.set_camera(cam)
        out = [torch.zeros(m, dtype=torch.int32, device="cuda") for m in (w * h * 2, w * h * 2, w * h, w * h * 5, w * h * 5)]
        t.trace_frame_dev(w, h, *[o.data_ptr() for o in out])
        t.synchronize()
        return [o.cpu() for o in out]
    finally:
        t.close()


def test_batched_views_match_single_view(native_lib):
    torch = pytest.importorskip("torch")
    from arcadia_gb300.batch import Batch

    scenes = ["c1_256", "s512"]
    worlds = [native_lib.build_world(L.SCENES[s])[:3] for s in scenes]
    t = native_lib.Tracer(0)
    try:
        b = Batch(t, scenes, 3, resolutions=[(96, 64), (160, 90), (200, 120)], worlds=worlds, seed=5)
        n_gi = torch.zeros(1, dtype=torch.int64, device="cuda")
        runs = ((0, False, 1, 1), (1, True, 1, 0), (2, True, 1, 1), (3, False, 0, 1), (4, True, 0, 0))
        for frame, use_graph, variant, order in runs:
            # persistent, then plain (one thread per queue slot); Morton or row-major tile order
            t.set_launch_config(variant=variant, order=order)
            b.set_frame(frame)
            b.trace(n_gi.data_ptr(), use_graph=use_graph)
            t.synchronize()
            total_gi = 0
            for i, v in enumerate(b.views):
                ref = _single(native_lib, worlds[v["slot"]], v["scene"], b.camera(i, frame), v["w"], v["h"])
                for got, want in zip(b.buffers[i], ref):
                    assert torch.equal(got.cpu(), want), (frame, i)
                hits = ref[3].numpy().view(L.HIT_DTYPE)
                total_gi += int((hits["flags"] & 1).sum())
            assert int(n_gi.item()) == total_gi
        t.set_launch_config(variant=0, order=1)
    finally:
        t.close()


def test_batched_autotune_keeps_results(native_lib):
    pytest.importorskip("torch")
    from arcadia_gb300.batch import Batch

    t = native_lib.Tracer(0)
    try:
        b = Batch(t, ["c1_256"], 4, resolutions=[(128, 96), (64, 64)], seed=9)
        b.trace(use_graph=False)
        t.synchronize()
        before = [[x.cpu() for x in bufs] for bufs in b.buffers]
        best, ms = t.autotune_views_dev(b.table, frames=2)
        assert ms > 0 and best.variant in (0, 1)
        b.trace(use_graph=True)
        t.synchronize()
        for bufs, ref in zip(b.buffers, before):
            for x, y in zip(bufs, ref):
                assert (x.cpu() == y).all()
    finally:
        t.close()


def test_bench_batch_matches_oracle(orc, native_lib, world_cache):
    """The benchmark batch itself (256^3, 512^3, 1024^3 and 1024^3-caves worlds, 16 views each, 320x240 up
    to 2560x1440, seeded poses), replayed from its CUDA graph with both kernel variants and both tile
    orders (Morton super-tiles, row-major): every view's G-buffer words, primary hit records and GI hit
    records bit-exact against the oracle's trace of the same camera, and the batch's GI-ray count equal
    to the oracle's number of primary hits."""
    torch = pytest.importorskip("torch")
    from arcadia_gb300.batch import BENCH_SCENES, Batch

    threads = os.cpu_count() or 8
    worlds = [world_cache(s) for s in BENCH_SCENES]
    t = native_lib.Tracer(0)
    try:
        b = Batch(t, BENCH_SCENES, 16, worlds=[(w.roots, w.nodes, w.bricks) for w in worlds])
        assert {(v["w"], v["h"]) for v in b.views} >= {(1920, 1080), (2560, 1440)}
        expect = []
        for i, v in enumerate(b.views):
            w = worlds[v["slot"]]
            cam = b.camera(i, 1)
            gdm, gnm, gaa, hits, _ = orc.primary(w, cam, threads=threads)
            _, gi, _ = orc.gi_rays(w, cam, gdm, gnm, threads=threads)
            expect.append((gdm, gnm, gaa, hits, gi))
        n_hit = sum(int((e[3]["flags"] & 1).sum()) for e in expect)
        n_gi = torch.zeros(1, dtype=torch.int64, device="cuda")
        for variant, order in ((0, 1), (1, 1), (0, 0)):  # Morton tile order (default) and row-major
            t.set_launch_config(variant=variant, order=order)
            for bufs in b.buffers:
                for x in bufs:
                    x.fill_(-1)
            b.set_frame(1)
            b.trace(n_gi.data_ptr(), use_graph=True)
            t.synchronize()
            assert int(n_gi.item()) == n_hit, (variant, order)
            for i, (bufs, e) in enumerate(zip(b.buffers, expect)):
                for got, want, what in zip(bufs, e, ("depth/material", "normal/motion", "albedo/ao", "hits", "GI hits")):
                    got = got.cpu().numpy().view(np.uint32)
                    want = np.ascontiguousarray(want).view(np.uint32).reshape(-1)
                    if not np.array_equal(got, want):
                        bad = np.nonzero(got != want)[0]
                        raise AssertionError(f"variant {variant} order {order} view {i} ({b.views[i]['w']}x{b.views[i]['h']}, "
                                             f"world {BENCH_SCENES[b.views[i]['slot']]}) {what}: {len(bad)} words differ, "
                                             f"first at {bad[:4]}")
        t.set_launch_config(variant=0, order=1)
    finally:
        t.close()
