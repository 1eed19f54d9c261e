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
