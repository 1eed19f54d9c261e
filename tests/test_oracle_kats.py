"""The oracle pinned against the reference's own known-answer tests (CPU only).

Sources of the expectations:
  crates/arcadia-core/src/raycast_cpu.rs:334-446   four raycast KATs
  crates/arcadia-core/src/node64.rs:165-186        popcount slot offsets, brick pack/unpack
  crates/arcadia-core/src/coord.rs:111-133         child bit index round trip
  crates/arcadia-render/src/camera.rs:160-163      480 B CameraUniforms
  crates/arcadia-render/src/sharc.rs:441-475       SHARC sizes and tile grids
  crates/arcadia-render/tests/sharc_gpu.rs:261-350 SHARC deposit / resolve / query / EMA / eviction
"""
import numpy as np
import pytest

from arcadia_gb300 import layout as L

FLOOR = 2  # MAT_STONE_DEEP


@pytest.fixture(scope="module")
def floor_world(orc):
    vol = np.zeros((256, 256, 256), np.uint8)
    vol[:, :32, :] = FLOOR
    n, b = orc.build_chunk_dense(vol)
    return orc.world_from_chunk(n, b)


def _single(orc, voxels):
    vol = np.zeros((256, 256, 256), np.uint8)
    for (x, y, z) in voxels:
        vol[z, y, x] = FLOOR
    n, b = orc.build_chunk_dense(vol)
    return orc.world_from_chunk(n, b)


def _norm(d):
    d = np.asarray(d, np.float32)
    return d / np.float32(np.sqrt(np.float32(d @ d)))


# ---- raycast_cpu.rs KATs through the reference CPU raycaster restatement -----------------------

def test_kat_floor_hit(orc, floor_world):
    h = orc.raycast_chunk_local(floor_world, (128.5, 50.0, 128.5), (0.0, -1.0, 0.0), 100.0)
    assert h["mat"] == FLOOR and h["voxel"][1] == 31 and h["normal"] == (0.0, 1.0, 0.0)
    assert abs(h["distance"] - 18.0) < 0.05


def test_kat_grazing(orc, floor_world):
    assert orc.raycast_chunk_local(floor_world, (10.0, 32.0001, 10.0), (1.0, 0.0, 0.0), 100.0) is None
    h = orc.raycast_chunk_local(floor_world, (10.0, 32.5, 10.0), _norm((1.0, -0.005, 0.0)), 200.0)
    assert h["mat"] == FLOOR and h["voxel"][1] == 31 and h["normal"] == (0.0, 1.0, 0.0)


def test_kat_row_skipping(orc):
    w = _single(orc, [(3, 0, 0)])
    h = orc.raycast_chunk_local(w, (0.1, 0.5, 0.5), (1.0, 0.0, 0.0), 10.0)
    assert h["voxel"] == (3, 0, 0) and h["normal"] == (-1.0, 0.0, 0.0) and abs(h["distance"] - 2.9) < 1e-3
    h = orc.raycast_chunk_local(w, (3.9, 0.5, 0.5), (-1.0, 0.0, 0.0), 10.0)
    assert h["voxel"] == (3, 0, 0) and h["normal"] == (1.0, 0.0, 0.0)
    w = _single(orc, [(3, 0, 0), (0, 0, 0)])
    h = orc.raycast_chunk_local(w, (1.1, 0.5, 0.5), (1.0, 0.0, 0.0), 10.0)
    assert h["voxel"] == (3, 0, 0) and h["normal"] == (-1.0, 0.0, 0.0) and abs(h["distance"] - 1.9) < 1e-3


def test_kat_brick_crossing(orc):
    w = _single(orc, [(5, 0, 0)])
    h = orc.raycast_chunk_local(w, (0.5, 0.5, 0.5), (1.0, 0.0, 0.0), 20.0)
    assert h["voxel"] == (5, 0, 0) and h["normal"] == (-1.0, 0.0, 0.0) and abs(h["distance"] - 4.5) < 1e-3


# ---- the same KATs through the WGSL traversal restatement (the parity oracle) ------------------

def _cam1():
    return L.camera_uniforms((1, 1, 1), 16, 16, (8.0, 8.0, 8.0), quality=L.quality_parity(512))


def _trace(orc, world, origin_v, d, max_v, lod=0, water=False):
    rays = np.zeros(1, L.RAY_DTYPE)
    rays["origin_m"][0] = np.asarray(origin_v, np.float32) / np.float32(16.0)
    rays["dir"][0] = np.asarray(d, np.float32)
    return orc.trace_rays(world, _cam1(), rays, max_v / 16.0, lod, water, threads=1)[0]


@pytest.mark.parametrize("origin,d,maxv,voxel,face,dist", [
    ((128.5, 50.0, 128.5), (0.0, -1.0, 0.0), 100.0, (128, 31, 128), 2, 18.0),
])
def test_wgsl_kat_floor(orc, floor_world, origin, d, maxv, voxel, face, dist):
    h = _trace(orc, floor_world, origin, d, maxv)
    assert tuple(h["voxel"]) == voxel and h["face"] == face and h["mat"] == FLOOR
    assert abs(h["depth_m"] * 16.0 - dist) < 1e-4


def test_wgsl_kat_grazing(orc, floor_world):
    h = _trace(orc, floor_world, (10.0, 32.0001, 10.0), (1.0, 0.0, 0.0), 100.0)
    assert h["flags"] & 1 == 0
    h = _trace(orc, floor_world, (10.0, 32.5, 10.0), _norm((1.0, -0.005, 0.0)), 200.0)
    assert h["voxel"][1] == 31 and h["face"] == 2


def test_wgsl_kat_rows(orc):
    w = _single(orc, [(3, 0, 0)])
    h = _trace(orc, w, (0.1, 0.5, 0.5), (1.0, 0.0, 0.0), 10.0)
    assert tuple(h["voxel"]) == (3, 0, 0) and h["face"] == 1 and abs(h["depth_m"] * 16 - 2.9) < 1e-4
    h = _trace(orc, w, (3.9, 0.5, 0.5), (-1.0, 0.0, 0.0), 10.0)
    assert tuple(h["voxel"]) == (3, 0, 0) and h["face"] == 0
    w = _single(orc, [(3, 0, 0), (0, 0, 0)])
    h = _trace(orc, w, (1.1, 0.5, 0.5), (1.0, 0.0, 0.0), 10.0)
    assert tuple(h["voxel"]) == (3, 0, 0) and h["face"] == 1 and abs(h["depth_m"] * 16 - 1.9) < 1e-4
    w = _single(orc, [(5, 0, 0)])
    h = _trace(orc, w, (0.5, 0.5, 0.5), (1.0, 0.0, 0.0), 20.0)
    assert tuple(h["voxel"]) == (5, 0, 0) and h["face"] == 1 and abs(h["depth_m"] * 16 - 4.5) < 1e-4


# ---- node64.rs / coord.rs / layout KATs -------------------------------------------------------

def test_popcount_slot_offsets(orc):
    """node64.rs:165-174: children {0,5,19,63} at base 100 sit at 100..103; checked by tracing into
    each child of a hand-built root whose children are uniform leaves of distinct materials."""
    nodes = np.zeros(104, L.NODE_DTYPE)
    mask = (1 << 0) | (1 << 5) | (1 << 19) | (1 << 63)
    nodes[1] = (mask & 0xFFFFFFFF, mask >> 32, 100, 0)
    for k, mat in enumerate((3, 4, 5, 6)):
        nodes[100 + k] = (0xFFFFFFFF, 0xFFFFFFFF, L.IS_LEAF_FLAG | L.IS_UNIFORM_FLAG, mat << 24)
    w = orc.World((1, 1, 1), np.array([1], np.uint32), nodes, np.zeros(1, L.BRICK_DTYPE))
    for bit, mat in zip((0, 5, 19, 63), (3, 4, 5, 6)):
        cx, cy, cz = bit & 3, (bit >> 2) & 3, (bit >> 4) & 3
        centre = np.array([cx * 64 + 32.5, cy * 64 + 32.5, cz * 64 + 32.5], np.float32)
        h = _trace(orc, w, centre + np.float32([0, 0, 0]), (0.0, -1.0, 0.0), 10.0)
        assert h["mat"] == mat and h["flags"] & 1


def test_child_bit_index_roundtrip():
    seen = 0
    for z in range(4):
        for y in range(4):
            for x in range(4):
                b = (z << 4) | (y << 2) | x
                assert (b & 3, (b >> 2) & 3, (b >> 4) & 3) == (x, y, z)
                seen |= 1 << b
    assert seen == (1 << 64) - 1


def test_layout_sizes():
    assert L.CAMERA_DTYPE.itemsize == 480
    assert L.NODE_DTYPE.itemsize == 16 and L.BRICK_DTYPE.itemsize == 64 and L.MATERIAL_DTYPE.itemsize == 32
    assert L.SHARC_SLOT_DTYPE.itemsize == 16
    assert L.SHARC_SLOTS * 4 + L.SHARC_SLOTS * 16 + L.SHARC_SLOTS * 16 == 4_718_592


def test_sharc_tile_grids():
    def grid(w, h, t):
        return ((w + t - 1) // t) * ((h + t - 1) // t)
    assert grid(1920, 1080, 16) == 8_160 and grid(1920, 1080, 8) == 32_400


# ---- sharc_gpu.rs scenario on the oracle -------------------------------------------------------

TEST_POS = (40.13, 12.07, 55.31)
TEST_CAM = (41.0, 13.0, 56.0)
PX, NX, PY = (1.0, 0.0, 0.0), (-1.0, 0.0, 0.0), (0.0, 1.0, 0.0)


def test_sharc_scenario_oracle(orc):
    s = orc.Sharc()
    for i in range(64):  # test_deposit_first: 4 workgroups x 16 threads
        s.deposit(TEST_POS, PX, TEST_CAM, (1.0, 2.0, 3.0))
        if i % 2 == 0:
            s.deposit(TEST_POS, NX, TEST_CAM, (0.25, 0.5, 0.75))
    assert np.count_nonzero(s.keys) == 2
    counts = sorted(c for c in s.accum.reshape(-1, 4)[:, 3] if c > 0)
    assert counts == [32, 64]
    s.resolve(1)
    assert not s.accum.any()

    def q():
        far = tuple(np.float32(TEST_POS) + np.float32([50, 0, 0]))
        return [s.query(TEST_POS, PX, TEST_CAM), s.query(TEST_POS, PX, TEST_CAM, (0.9, -0.8)),
                s.query(TEST_POS, NX, TEST_CAM), s.query(far, PX, TEST_CAM), s.query(TEST_POS, PY, TEST_CAM)]

    r = q()
    np.testing.assert_allclose(r[0], [1, 2, 3, 1], atol=1e-3)
    np.testing.assert_allclose(r[1], [1, 2, 3, 1], atol=1e-3)
    np.testing.assert_allclose(r[2], [0.25, 0.5, 0.75, 1], atol=1e-3)
    np.testing.assert_allclose(r[3], [0, 0, 0, 0], atol=1e-3)
    np.testing.assert_allclose(r[4], [0, 0, 0, 0], atol=1e-3)
    for _ in range(16):  # test_deposit_second
        s.deposit(TEST_POS, PX, TEST_CAM, (3.0, 2.0, 1.0))
    s.resolve(1)
    r = q()
    np.testing.assert_allclose(r[0], [2, 2, 2, 1], atol=1e-3)
    np.testing.assert_allclose(r[2], [0.25, 0.5, 0.75, 1], atol=1e-3)
    s.resolve(63)
    r = q()
    np.testing.assert_allclose(r[2], [0.25, 0.5, 0.75, 1], atol=1e-3)
    np.testing.assert_allclose(r[0], [2, 2, 2, 1], atol=1e-3)
    s.resolve(1)
    r = q()
    np.testing.assert_allclose(r[2], [0, 0, 0, 0], atol=1e-3)
    np.testing.assert_allclose(r[0], [2, 2, 2, 1], atol=1e-3)
    assert np.count_nonzero(s.keys) == 1


# ---- canonical arithmetic of the oracle --------------------------------------------------------

def test_canonical_sincos_error_bound(orc):
    x = np.linspace(0.0, 6.2831853, 200001, dtype=np.float32)
    s, c = orc.sincos(x)
    xd = x.astype(np.float64)
    assert np.max(np.abs(s - np.sin(xd))) < 4e-7
    assert np.max(np.abs(c - np.cos(xd))) < 4e-7


def test_canonical_exp2_log2_pow_error_bounds(orc):
    x = np.linspace(-40.0, 40.0, 200001, dtype=np.float32)
    e2, _ = orc.exp2_log2(x)
    ref = np.exp2(x.astype(np.float64))
    assert np.max(np.abs(e2 / ref - 1.0)) < 4e-7
    assert orc.exp2_log2(np.float32([-127.0, -200.0]))[0].tolist() == [0.0, 0.0]
    y = np.concatenate([np.linspace(1e-6, 4.0, 200001, dtype=np.float32), np.float32([1.0, 2.0, 0.5, 1e-30, 3e38])])
    _, l2 = orc.exp2_log2(y)
    err = np.abs(l2 - np.log2(y.astype(np.float64)))
    assert np.max(err / np.maximum(np.abs(np.log2(y.astype(np.float64))), 1.0)) < 4e-7
    assert l2[-5] == 0.0 and l2[-4] == 1.0 and l2[-3] == -1.0
    p = np.linspace(0.0, 1.0, 100001, dtype=np.float32)
    for e in (2.2, 2.5):
        got = orc.pow_canon(p, e)
        want = p.astype(np.float64) ** e
        assert np.max(np.abs(got - want)) < 2e-6
    assert orc.pow_canon(np.float32([0.0, -1.0]), 2.2).tolist() == [0.0, 0.0]


def test_f16_packing_matches_ieee_rne(orc):
    rng = np.random.default_rng(7)
    x = np.concatenate([
        rng.standard_normal(100000).astype(np.float32) * np.float32(10.0),
        (rng.random(20000) * 1e-4).astype(np.float32),                      # f16 subnormals
        np.float32([0.0, -0.0, 65504.0, 65520.0, 1e9, -1e9, 2.0**-25, 2.0**-24, 3 * 2.0**-26]),
    ])
    ref = x.astype(np.float16).view(np.uint16)
    np.testing.assert_array_equal(orc.f16_bits(x), ref)


def test_powi_exact_small(orc):
    x = np.float32([0.0, 0.5, 1.0, 0.75, 0.999])
    np.testing.assert_allclose(orc.powi(x, 14), x.astype(np.float64) ** 14, rtol=2e-6, atol=1e-30)
    np.testing.assert_allclose(orc.powi(x, 3), x.astype(np.float64) ** 3, rtol=1e-6, atol=1e-30)


def _pack4x8unorm_wgsl(x):
    """WGSL pack4x8unorm by the specification's definition: byte i = floor(0.5 + 255 * min(1, max(0, e[i])))."""
    f = np.float32
    x = np.asarray(x, np.float32).reshape(-1, 4)
    v = np.floor(f(0.5) + f(255.0) * np.minimum(f(1.0), np.maximum(f(0.0), x))).astype(np.uint32)
    return v[:, 0] | (v[:, 1] << 8) | (v[:, 2] << 16) | (v[:, 3] << 24)


def _pack2x16snorm_wgsl(x):
    """WGSL pack2x16snorm by the specification's definition: half i = floor(0.5 + 32767 * min(1, max(-1, e[i])))
    as a 16-bit two's complement integer."""
    f = np.float32
    x = np.asarray(x, np.float32).reshape(-1, 2)
    v = np.floor(f(0.5) + f(32767.0) * np.minimum(f(1.0), np.maximum(f(-1.0), x))).astype(np.int64) & 0xFFFF
    return (v[:, 0] | (v[:, 1] << 16)).astype(np.uint32)


def _oct_encode_wgsl(n):
    """oct_encode / oct_wrap (shaders/common/types.wgsl:108-119) in float32."""
    f = np.float32
    n = np.asarray(n, np.float32).reshape(-1, 3)
    l1 = (np.abs(n[:, 0]) + np.abs(n[:, 1])) + np.abs(n[:, 2])
    p = n[:, :2] * (f(1.0) / np.maximum(l1, f(1e-6)))[:, None]
    wrapped = (f(1.0) - np.abs(p[:, ::-1])) * np.where(p >= 0, f(1.0), f(-1.0))
    return np.where((n[:, 2] < 0)[:, None], wrapped, p).astype(np.float32)


def test_gbuffer_packing_matches_wgsl_definitions(orc):
    """The G-buffer words (normal and albedo/AO packing) pinned to the WGSL definitions: the oracle's
    pack4x8unorm and pack2x16snorm equal the specification's formulas bit for bit, including the clamps
    and the values on rounding midpoints, and its octahedral encoding equals types.wgsl's in float32.
    The GPU writes the same words as the oracle (every frame parity test), so both sides are pinned."""
    rng = np.random.default_rng(11)
    mids = ((np.arange(256, dtype=np.float64) + 0.5) / 255.0).astype(np.float32)
    u = np.concatenate([rng.uniform(-0.5, 1.5, 400000).astype(np.float32), mids, np.nextafter(mids, np.float32(0)),
                        np.nextafter(mids, np.float32(2)), np.float32([0.0, -0.0, 1.0, -1.0, 2.0, 1e-30, 1e30, -1e30])])
    u = u[: len(u) // 4 * 4]
    np.testing.assert_array_equal(orc.pack4x8unorm(u), _pack4x8unorm_wgsl(u))
    smid = ((np.arange(-32767, 32767, 7, dtype=np.float64) + 0.5) / 32767.0).astype(np.float32)
    s = np.concatenate([rng.uniform(-1.5, 1.5, 400000).astype(np.float32), smid, np.nextafter(smid, np.float32(-2)),
                        np.float32([0.0, -0.0, 1.0, -1.0, 3.0, -3.0])])
    s = s[: len(s) // 2 * 2]
    np.testing.assert_array_equal(orc.pack2x16snorm(s), _pack2x16snorm_wgsl(s))
    d = rng.standard_normal((200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    axes = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [0.0, -0.0, -1.0],
                     [-0.0, 0.0, -1.0]], np.float64)
    n = np.concatenate([d, axes]).astype(np.float32)
    got = orc.oct_encode(n)
    np.testing.assert_array_equal(got.view(np.uint32), _oct_encode_wgsl(n).view(np.uint32))
    np.testing.assert_array_equal(got[-8:-2], np.float32([[1, 0], [-1, 0], [0, 1], [0, -1], [0, 0], [1, 1]]))
