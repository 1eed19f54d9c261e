"""Radiance caches at secondary hits: what the trained network gains, and how SHARC compares (GPU).

Both caches learn the one-bounce radiance at GI hits on the 1024^3 caves scene; quality is the relative
MSE against a 4096-spp reference (FP64 host accumulation). A smaller frame than the benchmark keeps the
test short. The trained network must beat the method without it: the untrained network and the
per-pixel 1-spp estimate.
"""
import pytest

pytestmark = pytest.mark.gpu


def test_trained_nrc_beats_untrained_and_one_sample(native_lib):
    pytest.importorskip("torch")
    from arcadia_gb300 import gi_cache, layout as L

    scene = L.SCENES["c2_1024_caves"]
    roots, nodes, bricks, _ = native_lib.build_world(scene)
    t = native_lib.Tracer(0)
    try:
        t.upload_world(scene.grid, roots, nodes, bricks, native_lib.default_palette())
        r = gi_cache.run_comparison(t, width=640, height=360, frames=40, eval_points=4096)
    finally:
        t.close()
    print(r)
    assert r["eval_points"] > 1000
    assert r["rel_mse_nrc"] < 0.5 * r["rel_mse_untrained_nrc"]
    assert r["rel_mse_nrc"] < r["rel_mse_1spp"]
    assert 0.0 < r["sharc_hit_fraction"] <= 1.0
