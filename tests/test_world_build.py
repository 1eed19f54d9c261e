"""World pools: the native builder (libarc_trace.so, C++) against the oracle's recursive builder.

The layout is the drop-in contract (BFS level order, uniform collapse, lod payloads, Morton chunk
order, relocated pointers; crates/arcadia-core/src/chunk_tree/builder.rs:86-378,
crates/arcadia-world/src/world_map.rs:158-205), so the pools must be identical byte for byte.
"""
import dataclasses

import numpy as np
import pytest

from arcadia_gb300.layout import SCENES, SceneParams


def _same(orc_world, native):
    roots, nodes, bricks, solid = native
    np.testing.assert_array_equal(roots, orc_world.roots)
    assert len(nodes) == len(orc_world.nodes)
    assert nodes.tobytes() == orc_world.nodes.tobytes()
    assert bricks.tobytes() == orc_world.bricks.tobytes()
    assert solid == orc_world.solid_voxels


def test_palette_matches(orc, native_lib):
    a = native_lib.default_palette()
    b = orc.default_palette()
    assert a[:29].tobytes() == b[:29].tobytes()
    np.testing.assert_allclose(a["albedo_roughness"], b["albedo_roughness"], atol=1e-6)


@pytest.mark.parametrize("name", ["c1_256", "s512"])
def test_native_builder_matches_oracle(orc, native_lib, world_cache, name):
    _same(world_cache(name), native_lib.build_world(SCENES[name], orc.default_palette()))


def test_native_builder_caves_small(orc, native_lib):
    s = SceneParams(grid=(2, 2, 2), seed=11, caves=True)
    _same(orc.build_world(s), native_lib.build_world(s, orc.default_palette()))


def test_native_builder_cave_band(orc, native_lib):
    """Caves limited to a band under the surface: the native builder's region classification (band
    bounds from the per-block height minima and maxima) gives the oracle's per-voxel pools."""
    s = SceneParams(grid=(2, 2, 2), seed=12, caves=True, cave_depth=24)
    _same(orc.build_world(s), native_lib.build_world(s, orc.default_palette()))
    full = orc.build_world(dataclasses.replace(s, cave_depth=0))
    assert orc.build_world(s).solid_voxels > full.solid_voxels  # the band carves less


@pytest.mark.slow
def test_native_builder_caves_1024(orc, native_lib, world_cache):
    _same(world_cache("c2_1024_caves"), native_lib.build_world(SCENES["c2_1024_caves"], orc.default_palette()))


def test_oracle_region_hint_is_exact(orc, world_cache):
    """The oracle's air-above-terrain hint gives the same chunk as evaluating every voxel."""
    vol = orc.scene_volume(SCENES["c1_256"])
    nodes, bricks = orc.build_chunk_dense(vol)
    w = orc.world_from_chunk(nodes, bricks)
    ref = world_cache("c1_256")
    assert w.nodes.tobytes() == ref.nodes.tobytes()
    assert w.bricks.tobytes() == ref.bricks.tobytes()


def test_cave_fraction_near_spec(orc, world_cache):
    """1024^3 caves scene: ~20% of solids carved (noise > 0.6)."""
    s = SCENES["c2_1024_caves"]
    carved = 1.0 - world_cache("c2_1024_caves").solid_voxels / orc.build_world(dataclasses.replace(s, caves=False)).solid_voxels
    assert 0.15 < carved < 0.30


def test_pool_invariants(world_cache):
    """Every internal child slice and brick index lies inside the pools; node 0 / brick 0 are the
    reserved empty entries (world_map.rs:167-169)."""
    w = world_cache("c2_1024_caves")
    n = w.nodes
    assert n[0].tobytes() == bytes(16) and w.bricks[0].tobytes() == bytes(64)
    mask = n["mask_low"].astype(np.uint64) | (n["mask_high"].astype(np.uint64) << np.uint64(32))
    live = mask != 0
    leaf = (n["child_ptr"] & 0x80000000) != 0
    uni = (n["child_ptr"] & 0x40000000) != 0
    ptr = n["child_ptr"] & 0x3FFFFFFF
    cnt = np.array([bin(int(m)).count("1") for m in mask[live & ~leaf]])
    assert np.all(ptr[live & ~leaf].astype(np.int64) + cnt <= len(n))
    assert np.all(ptr[live & leaf & ~uni] < len(w.bricks))
    r = w.roots[w.roots != 0xFFFFFFFF]
    assert np.all(r < len(n))
