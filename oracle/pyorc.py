"""ctypes front end of the CPU oracle (``oracle/_build/liborc.so``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg
of ``bench.py``. The product (``arcadia_gb300``) never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

from arcadia_gb300.layout import (
    BRICK_DTYPE,
    CAMERA_DTYPE,
    EDIT_DTYPE,
    HIT_DTYPE,
    MATERIAL_DTYPE,
    NODE_DTYPE,
    RAY_DTYPE,
    SHARC_SLOT_DTYPE,
    IS_LEAF_FLAG,
    IS_UNIFORM_FLAG,
    PTR_INDEX_MASK,
    SceneParams,
)

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liborc.so")
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Scene(C.Structure):
    _fields_ = [
        ("grid", C.c_uint32 * 3),
        ("seed", C.c_uint32),
        ("caves", C.c_uint32),
        ("cave_threshold", C.c_float),
        ("height_lo", C.c_float),
        ("height_hi", C.c_float),
        ("cave_depth", C.c_uint32),
    ]


class _Pools(C.Structure):
    _fields_ = [
        ("grid", C.c_uint32 * 3),
        ("n_chunks", C.c_uint32),
        ("roots", C.POINTER(C.c_uint32)),
        ("nodes", C.c_void_p),
        ("n_nodes", C.c_uint32),
        ("bricks", C.c_void_p),
        ("n_bricks", C.c_uint32),
        ("solid_voxels", C.c_uint64),
    ]


class _World(C.Structure):
    _fields_ = [
        ("roots", C.c_void_p),
        ("nodes", C.c_void_p),
        ("n_nodes", C.c_uint32),
        ("bricks", C.c_void_p),
        ("n_bricks", C.c_uint32),
        ("palette", C.c_void_p),
        ("bodies", C.c_void_p),
        ("n_bodies", C.c_uint32),
    ]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        _lib = C.CDLL(_LIB_PATH)
        vp, u32, f32, i32 = C.c_void_p, C.c_uint32, C.c_float, C.c_int
        _lib.orc_build_world.argtypes = [C.POINTER(_Scene), C.POINTER(_Pools)]
        _lib.orc_free_pools.argtypes = [C.POINTER(_Pools)]
        _lib.orc_default_palette.argtypes = [vp]
        _lib.orc_build_chunk_dense.argtypes = [vp, vp, vp, C.POINTER(u32), vp, C.POINTER(u32)]
        _lib.orc_trace_rays.argtypes = [C.POINTER(_World), vp, vp, u32, f32, u32, i32, vp, vp, i32]
        _lib.orc_primary.argtypes = [C.POINTER(_World), vp, u32, u32, u32, u32, vp, vp, vp, vp, vp, i32]
        _lib.orc_gi_rays.argtypes = [C.POINTER(_World), vp, u32, u32, u32, u32, vp, vp, vp, vp, vp, i32]
        _lib.orc_restir_gi_temporal.argtypes = [C.POINTER(_World), vp, vp, vp, vp, vp, vp, vp, i32]
        _lib.orc_trace_rigid_rays.argtypes = [C.POINTER(_World), vp, vp, u32, f32, vp, vp, i32]
        _lib.orc_frame_sample.argtypes = [C.POINTER(_World), vp, u32, i32, vp, vp, vp]
        _lib.orc_frame_sample.restype = C.c_uint64
        _lib.orc_cpu_frame_sample.argtypes = [C.POINTER(_World), vp, u32, i32, vp, vp, vp]
        _lib.orc_cpu_frame_sample.restype = C.c_uint64
        _lib.orc_cpu_raycast.argtypes = [C.POINTER(_World), vp, vp, u32, f32, vp, i32]
        _lib.orc_raycast_chunk_local.argtypes = [C.POINTER(_World), u32, vp, vp, f32, vp, vp, vp]
        _lib.orc_raycast_chunk_local.restype = C.c_int
        _lib.orc_depth_fp64.argtypes = [vp, vp, vp, u32]
        _lib.orc_depth_fp64.restype = C.c_double
        _lib.orc_sharc_make_key.argtypes = [vp, vp, vp, vp, vp, vp]
        _lib.orc_sharc_deposit.argtypes = [vp, vp, u32, u32, vp]
        _lib.orc_sharc_deposit.restype = u32
        _lib.orc_sharc_resolve.argtypes = [vp, vp, vp]
        _lib.orc_sharc_query.argtypes = [vp, vp, vp, vp, vp, vp]
        _lib.orc_sharc_update.argtypes = [C.POINTER(_World), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib.orc_sharc_update_mode.argtypes = [C.POINTER(_World), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32]
        _lib.orc_cmp_albedo.argtypes = [u32, vp]
        _lib.orc_onebounce.argtypes = [C.POINTER(_World), vp, vp, u32, vp, vp, vp, u32, u32, i32, vp, i32]
        _lib.orc_train_samples.argtypes = [C.POINTER(_World), vp, vp, C.c_uint64, vp, vp, vp, u32, u32, u32, u32, vp, vp, i32]
        _lib.orc_gi_points.argtypes = [C.POINTER(_World), vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, i32]
        _lib.orc_gi_points_from_hits.argtypes = [vp, u32, u32, vp, vp, vp, vp, vp, vp, vp, vp]
        _lib.orc_shadow_vis.argtypes = [C.POINTER(_World), vp, vp, vp, f32, vp]
        _lib.orc_shadow_vis.restype = f32
        _lib.orc_shadow_vis_di.argtypes = [C.POINTER(_World), vp, vp, vp, f32]
        _lib.orc_shadow_vis_di.restype = f32
        _lib.orc_test_sincos.argtypes = [vp, u32, vp, vp]
        _lib.orc_test_f16.argtypes = [vp, u32, vp]
        _lib.orc_test_pack4x8unorm.argtypes = [vp, u32, vp]
        _lib.orc_test_pack2x16snorm.argtypes = [vp, u32, vp]
        _lib.orc_test_oct_encode.argtypes = [vp, u32, vp]
        _lib.orc_test_powi.argtypes = [vp, u32, u32, vp]
        _lib.orc_test_exp2_log2.argtypes = [vp, u32, vp, vp]
        _lib.orc_test_pow.argtypes = [vp, u32, C.c_float, vp]
        _lib.orc_scene_heightmap.argtypes = [C.POINTER(_Scene), vp]
        _lib.orc_scene_voxel.argtypes = [C.POINTER(_Scene), vp, u32, u32, u32]
        _lib.orc_scene_voxel.restype = u32
        _lib.orc_test_scene_volume.argtypes = [C.POINTER(_Scene), u32, u32, u32, vp]
        _lib.orc_nrc_param_count.restype = u32
        _lib.orc_nrc_forward.argtypes = [vp, vp, u32, vp, vp]
        _lib.orc_nrc_grad.argtypes = [vp, vp, vp, u32, vp]
        _lib.orc_nrc_grad.restype = C.c_double
        _lib.orc_nrc_adam.argtypes = [vp, vp, vp, vp, u32, u32, f32]
        _lib.orc_apply_edits.argtypes = [vp, vp, vp, C.POINTER(u32), u32, vp, C.POINTER(u32), u32, vp, vp, u32]
        _lib.orc_pool_chunk_volume.argtypes = [vp, vp, vp, vp, u32, u32, u32, vp]
        _lib.orc_tree_compare.argtypes = [u32, vp, vp, u32, vp, vp, C.c_int]
        _lib.orc_tree_compare.restype = C.c_uint64
    return _lib


def _p(a: np.ndarray | None):
    """Pointer to the array's data that keeps the array alive (a temporary made by a dtype
    conversion in the call expression must outlive the C call)."""
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def default_palette() -> np.ndarray:
    pal = np.zeros(256, MATERIAL_DTYPE)
    lib().orc_default_palette(_p(pal))
    return pal


class World:
    """Flat GPU-ready pools (chunk roots, Node64 pool, LeafBrick64 pool, palette)."""

    def __init__(self, grid, roots, nodes, bricks, palette=None, bodies=None):
        from arcadia_gb300.layout import RIGID_BODY_DTYPE

        self.grid = tuple(int(g) for g in grid)
        self.roots = np.ascontiguousarray(roots, np.uint32)
        self.nodes = np.ascontiguousarray(nodes).view(NODE_DTYPE)
        self.bricks = np.ascontiguousarray(bricks).view(BRICK_DTYPE)
        self.palette = default_palette() if palette is None else np.ascontiguousarray(palette).view(MATERIAL_DTYPE)
        self.bodies = np.zeros(0, RIGID_BODY_DTYPE) if bodies is None else np.ascontiguousarray(bodies).view(RIGID_BODY_DTYPE)
        self._w = _World(
            _p(self.roots), _p(self.nodes), len(self.nodes), _p(self.bricks), len(self.bricks), _p(self.palette),
            _p(self.bodies) if len(self.bodies) else None, len(self.bodies)
        )

    def with_bodies(self, bodies) -> "World":
        """The same pools with a rigid-body table."""
        return World(self.grid, self.roots, self.nodes, self.bricks, self.palette, bodies)

    @property
    def cw(self):
        return C.byref(self._w)


def build_world(scene: SceneParams) -> World:
    s = _Scene((C.c_uint32 * 3)(*scene.grid), scene.seed, int(scene.caves), scene.cave_threshold, scene.height_lo,
               scene.height_hi, scene.cave_depth)
    p = _Pools()
    lib().orc_build_world(C.byref(s), C.byref(p))
    n_ch = p.n_chunks
    roots = np.ctypeslib.as_array(p.roots, shape=(n_ch,)).copy()
    nodes = np.frombuffer((C.c_char * (16 * p.n_nodes)).from_address(p.nodes), dtype=NODE_DTYPE).copy()
    bricks = np.frombuffer((C.c_char * (64 * p.n_bricks)).from_address(p.bricks), dtype=BRICK_DTYPE).copy()
    solid = p.solid_voxels
    lib().orc_free_pools(C.byref(p))
    w = World(scene.grid, roots, nodes, bricks)
    w.solid_voxels = solid
    return w


def apply_edits(world: World, ops: np.ndarray, node_headroom: int = 1 << 20, brick_headroom: int = 1 << 18) -> World:
    """A copy of `world` with the edit records `ops` (layout.EDIT_DTYPE) applied in order by the
    sequential restatement of the reference edit path (orc_edit.c)."""
    ops = np.ascontiguousarray(ops).view(EDIT_DTYPE)
    nodes = np.zeros(len(world.nodes) + node_headroom, NODE_DTYPE)
    nodes[: len(world.nodes)] = world.nodes
    bricks = np.zeros(len(world.bricks) + brick_headroom, BRICK_DTYPE)
    bricks[: len(world.bricks)] = world.bricks
    nn, nb = C.c_uint32(len(world.nodes)), C.c_uint32(len(world.bricks))
    grid = np.array(world.grid, np.uint32)
    rc = lib().orc_apply_edits(_p(grid), _p(world.roots), _p(nodes), C.byref(nn), len(nodes), _p(bricks), C.byref(nb),
                               len(bricks), _p(world.palette), _p(ops), len(ops))
    if rc:
        raise RuntimeError("orc_apply_edits: pool headroom exhausted")
    return World(world.grid, world.roots.copy(), nodes[: nn.value].copy(), bricks[: nb.value].copy(), world.palette)


def chunk_volume(grid, roots, nodes, bricks, chunk) -> np.ndarray:
    """Dense (z, y, x) u8 materials of one chunk of a flattened pool, by point descent."""
    vol = np.zeros((256, 256, 256), np.uint8)
    g = np.array(grid, np.uint32)
    lib().orc_pool_chunk_volume(_p(g), _p(np.ascontiguousarray(roots, np.uint32)), _p(np.ascontiguousarray(nodes)),
                                _p(np.ascontiguousarray(bricks)), chunk[0], chunk[1], chunk[2], _p(vol))
    return vol


def tree_compare(root_a, nodes_a, bricks_a, root_b, nodes_b, bricks_b, leaf_form: bool = True) -> int:
    """0 when two chunk trees are equal node by node in child order (masks, flags, lod payloads, voxel
    materials under leaf masks), wherever their nodes sit; else the position of the first difference.
    leaf_form=False lets a brick leaf equal a uniform leaf with the same voxels."""
    return int(lib().orc_tree_compare(int(root_a), _p(np.ascontiguousarray(nodes_a)), _p(np.ascontiguousarray(bricks_a)),
                                      int(root_b), _p(np.ascontiguousarray(nodes_b)), _p(np.ascontiguousarray(bricks_b)),
                                      1 if leaf_form else 0))


def build_chunk_dense(vol: np.ndarray, palette: np.ndarray | None = None):
    """ChunkTree64::from_generator over a dense (z, y, x) u8 volume with no region hint."""
    vol = np.ascontiguousarray(vol, np.uint8)
    assert vol.shape == (256, 256, 256)
    pal = default_palette() if palette is None else palette
    nn, nb = C.c_uint32(0), C.c_uint32(0)
    lib().orc_build_chunk_dense(_p(vol), _p(pal), None, C.byref(nn), None, C.byref(nb))
    nodes = np.zeros(nn.value, NODE_DTYPE)
    bricks = np.zeros(max(nb.value, 1), BRICK_DTYPE)
    lib().orc_build_chunk_dense(_p(vol), _p(pal), _p(nodes), C.byref(nn), _p(bricks), C.byref(nb))
    return nodes, bricks[: nb.value]


def world_from_chunk(nodes: np.ndarray, bricks: np.ndarray, palette=None) -> World:
    """One-chunk world: relocate a chunk's local tree behind the reserved empty node/brick 0
    (world_map.rs:167-203)."""
    out = np.zeros(len(nodes) + 1, NODE_DTYPE)
    rel = nodes.copy()
    ptr = rel["child_ptr"].astype(np.uint64)
    flags = ptr & (IS_LEAF_FLAG | IS_UNIFORM_FLAG)
    local = ptr & PTR_INDEX_MASK
    is_leaf = (ptr & IS_LEAF_FLAG) != 0
    is_uni = (ptr & IS_UNIFORM_FLAG) != 0
    new = np.where(is_leaf, np.where(is_uni, flags, flags | (local + 1)), flags | (local + 1))
    empty = (rel["mask_low"] == 0) & (rel["mask_high"] == 0)
    new = np.where(empty, 0, new)
    rel["child_ptr"] = new.astype(np.uint32)
    rel["lod_payload"] = np.where(empty, 0, rel["lod_payload"])
    out[1:] = rel
    b = np.zeros(len(bricks) + 1, BRICK_DTYPE)
    b[1:] = bricks
    roots = np.array([1 if not empty[0] else 0xFFFFFFFF], np.uint32)
    return World((1, 1, 1), roots, out, b, palette)


def trace_rays(world: World, cam: np.ndarray, rays: np.ndarray, max_dist_m: float, lod_bias: int, ignore_water: bool,
               threads: int = 8, want_bytes: bool = False):
    n = len(rays)
    hits = np.zeros(n, HIT_DTYPE)
    by = np.zeros(n, np.uint32) if want_bytes else None
    lib().orc_trace_rays(world.cw, _p(cam), _p(np.ascontiguousarray(rays, RAY_DTYPE)), n, max_dist_m, lod_bias,
                         int(ignore_water), _p(hits), _p(by), threads)
    return (hits, by) if want_bytes else hits


def primary(world: World, cam: np.ndarray, rect=None, threads: int = 8):
    w = int(cam["world_grid_dims"][0][3] & 0xFFFF)
    h = int(cam["world_grid_dims"][0][3] >> 16)
    x0, y0, x1, y1 = rect or (0, 0, w, h)
    gdm = np.zeros((h * w, 2), np.uint32)
    gnm = np.zeros((h * w, 2), np.uint32)
    gaa = np.zeros(h * w, np.uint32)
    hits = np.zeros(h * w, HIT_DTYPE)
    by = np.zeros(h * w, np.uint32)
    lib().orc_primary(world.cw, _p(cam), x0, y0, x1, y1, _p(gdm), _p(gnm), _p(gaa), _p(hits), _p(by), threads)
    return gdm, gnm, gaa, hits, by


def gi_rays(world: World, cam: np.ndarray, gdm, gnm, rect=None, threads: int = 8):
    w = int(cam["world_grid_dims"][0][3] & 0xFFFF)
    h = int(cam["world_grid_dims"][0][3] >> 16)
    x0, y0, x1, y1 = rect or (0, 0, w, h)
    rays = np.zeros(h * w, RAY_DTYPE)
    hits = np.zeros(h * w, HIT_DTYPE)
    by = np.zeros(h * w, np.uint32)
    lib().orc_gi_rays(world.cw, _p(cam), x0, y0, x1, y1, _p(gdm), _p(gnm), _p(rays), _p(hits), _p(by), threads)
    return rays, hits, by


def trace_rigid_rays(world: World, cam: np.ndarray, rays: np.ndarray, max_dist_m: float, threads: int = 8):
    """trace_rigid_bodies over a ray batch: (hit records, (n, 9) hit point / previous point / normal)."""
    rays = np.ascontiguousarray(rays).view(RAY_DTYPE)
    hits = np.zeros(len(rays), HIT_DTYPE)
    detail = np.zeros((len(rays), 9), np.float32)
    lib().orc_trace_rigid_rays(world.cw, _p(cam), _p(rays), len(rays), max_dist_m, _p(hits), _p(detail), threads)
    return hits, detail


def restir_gi_temporal(world: World, cam: np.ndarray, resolved: np.ndarray, gdm, gnm, res_in: np.ndarray,
                       radiance=None, threads: int = 8) -> np.ndarray:
    """GI part of temporal_main for every pixel: this frame's reservoirs from the previous frame's
    (``res_in``), the G-buffer and the resolved SHARC slots (or a per-pixel radiance buffer)."""
    from arcadia_gb300.layout import RESERVOIR_DTYPE

    w = int(cam["world_grid_dims"][0][3] & 0xFFFF)
    h = int(cam["world_grid_dims"][0][3] >> 16)
    res_in = np.ascontiguousarray(res_in).view(RESERVOIR_DTYPE)
    out = np.zeros(h * w, RESERVOIR_DTYPE)
    rad = None if radiance is None else np.ascontiguousarray(radiance, np.float32)
    lib().orc_restir_gi_temporal(world.cw, _p(cam), _p(np.ascontiguousarray(resolved)), _p(rad),
                                 _p(np.ascontiguousarray(gdm, np.uint32)), _p(np.ascontiguousarray(gnm, np.uint32)),
                                 _p(res_in), _p(out), threads)
    return out


def frame_sample(world: World, cam: np.ndarray, stride: int, threads: int, cpu_query: bool = False):
    """Primary + GI rays of every ``stride``-th pixel; returns (rays, primary, gi, checksum, bytes).

    ``cpu_query`` selects the reference CPU ray query (raycast_meters) instead of the WGSL
    transcription; bytes (the instrumented algorithmic byte count) are only counted for the latter."""
    npri, ngi, cs = np.zeros(1, np.uint64), np.zeros(1, np.uint64), np.zeros(1, np.uint64)
    fn = lib().orc_cpu_frame_sample if cpu_query else lib().orc_frame_sample
    total = fn(world.cw, _p(cam), stride, threads, _p(npri), _p(ngi), _p(cs))
    by = 0 if cpu_query else int(C.c_uint64.in_dll(lib(), "orc_last_sample_bytes").value)
    return int(total), int(npri[0]), int(ngi[0]), int(cs[0]), by


def cpu_raycast(world: World, rays: np.ndarray, max_dist_m: float, threads: int = 8):
    hits = np.zeros(len(rays), HIT_DTYPE)
    grid = np.array(world.grid, np.uint32)
    lib().orc_cpu_raycast(world.cw, _p(grid), _p(np.ascontiguousarray(rays, RAY_DTYPE)), len(rays), max_dist_m,
                          _p(hits), threads)
    return hits


def raycast_chunk_local(world: World, origin_v, dir_, max_dist_v):
    o = np.asarray(origin_v, np.float32)
    d = np.asarray(dir_, np.float32)
    out = np.zeros(4, np.float32)
    vox = np.zeros(3, np.int32)
    mat = np.zeros(1, np.uint32)
    ok = lib().orc_raycast_chunk_local(world.cw, int(world.roots[0]), _p(o), _p(d), max_dist_v, _p(out), _p(vox),
                                       _p(mat))
    if not ok:
        return None
    return {"distance": float(out[0]), "normal": tuple(float(v) for v in out[1:]), "voxel": tuple(int(v) for v in vox),
            "mat": int(mat[0])}


def depth_fp64(origin_m, dir_, cell_min, span: int) -> float:
    o = np.asarray(origin_m, np.float32)
    d = np.asarray(dir_, np.float32)
    c = np.asarray(cell_min, np.int32)
    return lib().orc_depth_fp64(_p(o), _p(d), _p(c), span)


def shadow_vis(world: World, cam, origin_m, dir_, max_dist_m) -> float:
    o = np.asarray(origin_m, np.float32)
    d = np.asarray(dir_, np.float32)
    return lib().orc_shadow_vis(world.cw, _p(cam), _p(o), _p(d), max_dist_m, None)


def shadow_vis_di(world: World, cam, origin_m, dir_, max_dist_m) -> float:
    o = np.asarray(origin_m, np.float32)
    d = np.asarray(dir_, np.float32)
    return lib().orc_shadow_vis_di(world.cw, _p(cam), _p(o), _p(d), max_dist_m)


class Sharc:
    """Host-side SHARC state (keys, fixed-point accumulators, resolved slots)."""

    def __init__(self):
        self.keys = np.zeros(131072, np.uint32)
        self.accum = np.zeros(131072 * 4, np.uint32)
        self.resolved = np.zeros(131072, SHARC_SLOT_DTYPE)

    def make_key(self, pos, normal, cam_pos, jitter=(0.0, 0.0)):
        b, k = np.zeros(1, np.uint32), np.zeros(1, np.uint32)
        args = [np.asarray(v, np.float32) for v in (pos, normal, cam_pos, jitter)]
        lib().orc_sharc_make_key(*[_p(a) for a in args], _p(b), _p(k))
        return int(b[0]), int(k[0])

    def deposit(self, pos, normal, cam_pos, rad):
        b, k = self.make_key(pos, normal, cam_pos)
        r = np.asarray(rad, np.float32)
        return lib().orc_sharc_deposit(_p(self.keys), _p(self.accum), b, k, _p(r))

    def resolve(self, passes: int = 1):
        for _ in range(passes):
            lib().orc_sharc_resolve(_p(self.keys), _p(self.accum), _p(self.resolved))

    def query(self, pos, normal, cam_pos, jitter=(0.0, 0.0)):
        out = np.zeros(4, np.float32)
        args = [np.asarray(v, np.float32) for v in (pos, normal, cam_pos, jitter)]
        lib().orc_sharc_query(_p(self.resolved), *[_p(a) for a in args], _p(out))
        return out

    def update(self, world: World, cam, gdm, gnm, resolved_prev=None, mode: int = 0):
        w = int(cam["world_grid_dims"][0][3] & 0xFFFF)
        h = int(cam["world_grid_dims"][0][3] >> 16)
        tile = 16 if (int(cam["quality_flags"][0][3]) & 0xFF) <= 12 else 8
        nt = ((w + tile - 1) // tile) * ((h + tile - 1) // tile)
        tk, tb, tv = np.zeros(nt, np.uint32), np.zeros(nt, np.uint32), np.zeros(nt, np.uint32)
        tr = np.zeros((nt, 3), np.float32)
        prev = self.resolved if resolved_prev is None else resolved_prev
        lib().orc_sharc_update_mode(world.cw, _p(cam), _p(gdm), _p(gnm), _p(prev), _p(self.keys), _p(self.accum), _p(tk),
                                    _p(tb), _p(tr), _p(tv), mode)
        return tk, tb, tr, tv


def _frame_size(cam):
    return int(cam["world_grid_dims"][0][3] & 0xFFFF), int(cam["world_grid_dims"][0][3] >> 16)


def cmp_albedo(mat: int) -> np.ndarray:
    out = np.zeros(3, np.float32)
    lib().orc_cmp_albedo(int(mat), _p(out))
    return out


def onebounce(world: World, cam, pos, nrm, alb, spp: int, seed: int, idx=None, accumulate_into=None, threads: int = 8):
    """Mean of spp one-bounce samples at points idx (or every point): (n, 3) float32, as arc_onebounce_dev."""
    pos = np.ascontiguousarray(pos, np.float32)
    nrm = np.ascontiguousarray(nrm, np.float32)
    alb = np.ascontiguousarray(alb, np.float32)
    idx_a = None if idx is None else np.ascontiguousarray(idx, np.uint32)
    n = len(pos) if idx_a is None else len(idx_a)
    out = np.zeros((n, 3), np.float32) if accumulate_into is None else accumulate_into
    lib().orc_onebounce(world.cw, _p(cam), _p(idx_a), n, _p(pos), _p(nrm), _p(alb), spp, seed & 0xFFFFFFFF,
                        int(accumulate_into is not None), _p(out), threads)
    return out


def train_samples(world: World, cam, lst, n_valid: int, pos, nrm, nrc_in, seed: int, n_samples: int, steps: int,
                  threads: int = 8, cluster: int = 1):
    """The training batch of arc_nrc_train_samples_dev: (inputs (n, 9), targets (n, 3))."""
    tin = np.zeros((n_samples, 9), np.float32)
    tt = np.zeros((n_samples, 3), np.float32)
    lib().orc_train_samples(world.cw, _p(cam), _p(np.ascontiguousarray(lst, np.uint32)), n_valid,
                            _p(np.ascontiguousarray(pos, np.float32)), _p(np.ascontiguousarray(nrm, np.float32)),
                            _p(np.ascontiguousarray(nrc_in, np.float32)), seed & 0xFFFFFFFF, n_samples, steps, cluster,
                            _p(tin), _p(tt), threads)
    return tin, tt


def gi_points(world: World, cam, gdm, gnm, threads: int = 8):
    """GI hit points traced from the G-buffer: (pos, nrm, alb, nrc_in, valid), as arc_gi_points_dev."""
    w, h = _frame_size(cam)
    n = w * h
    pos, nrm, alb = (np.zeros((n, 3), np.float32) for _ in range(3))
    nin = np.zeros((n, 9), np.float32)
    valid = np.zeros(n, np.uint32)
    lib().orc_gi_points(world.cw, _p(cam), w, h, _p(np.ascontiguousarray(gdm)), _p(np.ascontiguousarray(gnm)), _p(pos),
                        _p(nrm), _p(alb), _p(nin), _p(valid), threads)
    return pos, nrm, alb, nin, valid


def gi_points_from_hits(cam, gdm, gnm, gi_hits):
    """GI hit points from GI hit records: (pos, nrm, alb, nrc_in, valid), as arc_gi_points_from_hits_dev."""
    w, h = _frame_size(cam)
    n = w * h
    pos, nrm, alb = (np.zeros((n, 3), np.float32) for _ in range(3))
    nin = np.zeros((n, 9), np.float32)
    valid = np.zeros(n, np.uint32)
    lib().orc_gi_points_from_hits(_p(cam), w, h, _p(np.ascontiguousarray(gdm)), _p(np.ascontiguousarray(gnm)),
                                  _p(np.ascontiguousarray(gi_hits).view(HIT_DTYPE)), _p(pos), _p(nrm), _p(alb), _p(nin),
                                  _p(valid))
    return pos, nrm, alb, nin, valid


def sincos(x: np.ndarray):
    x = np.ascontiguousarray(x, np.float32)
    s, c = np.zeros_like(x), np.zeros_like(x)
    lib().orc_test_sincos(_p(x), len(x), _p(s), _p(c))
    return s, c


def pack4x8unorm(x: np.ndarray) -> np.ndarray:
    """The oracle's WGSL pack4x8unorm over rows of 4 floats."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 4)
    out = np.zeros(len(x), np.uint32)
    lib().orc_test_pack4x8unorm(_p(x), len(x), _p(out))
    return out


def pack2x16snorm(x: np.ndarray) -> np.ndarray:
    """The oracle's WGSL pack2x16snorm over rows of 2 floats."""
    x = np.ascontiguousarray(x, np.float32).reshape(-1, 2)
    out = np.zeros(len(x), np.uint32)
    lib().orc_test_pack2x16snorm(_p(x), len(x), _p(out))
    return out


def oct_encode(n: np.ndarray) -> np.ndarray:
    """The oracle's octahedral encoding of unit normals (rows of 3 floats) into rows of 2 floats."""
    n = np.ascontiguousarray(n, np.float32).reshape(-1, 3)
    out = np.zeros((len(n), 2), np.float32)
    lib().orc_test_oct_encode(_p(n), len(n), _p(out))
    return out


def f16_bits(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros(len(x), np.uint16)
    lib().orc_test_f16(_p(x), len(x), _p(out))
    return out


def powi(x: np.ndarray, e: int) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    lib().orc_test_powi(_p(x), len(x), e, _p(out))
    return out


def exp2_log2(x: np.ndarray):
    """Canonical 2^x and log2(x) (log2 only where x > 0, else 0)."""
    x = np.ascontiguousarray(x, np.float32)
    e2, l2 = np.zeros_like(x), np.zeros_like(x)
    lib().orc_test_exp2_log2(_p(x), len(x), _p(e2), _p(l2))
    return e2, l2


def pow_canon(x: np.ndarray, y: float) -> np.ndarray:
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros_like(x)
    lib().orc_test_pow(_p(x), len(x), float(y), _p(out))
    return out


def scene_volume(scene: SceneParams, chunk=(0, 0, 0)) -> np.ndarray:
    """Dense (z, y, x) u8 materials of one chunk of a synthetic scene (per-voxel evaluation)."""
    s = _Scene((C.c_uint32 * 3)(*scene.grid), scene.seed, int(scene.caves), scene.cave_threshold, scene.height_lo,
               scene.height_hi, scene.cave_depth)
    vol = np.zeros((256, 256, 256), np.uint8)
    lib().orc_test_scene_volume(C.byref(s), chunk[0], chunk[1], chunk[2], _p(vol))
    return vol


NRC_PARAMS = 30400


def nrc_forward(weights: np.ndarray, inputs: np.ndarray) -> np.ndarray:
    """FP64 reference of the NRC forward pass (FP16-quantised weights and activations)."""
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(inputs, np.float32)
    out = np.zeros((len(x), 3), np.float64)
    lib().orc_nrc_forward(_p(w), _p(x), len(x), _p(out), None)
    return out


def nrc_grad(weights: np.ndarray, inputs: np.ndarray, targets: np.ndarray):
    """(loss, gradient) of the mean relative-L2 loss in FP64."""
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(inputs, np.float32)
    t = np.ascontiguousarray(targets, np.float32)
    g = np.zeros(NRC_PARAMS, np.float64)
    loss = lib().orc_nrc_grad(_p(w), _p(x), _p(t), len(x), _p(g))
    return loss, g


def nrc_adam(weights, m, v, grad, step: int, lr: float):
    for a in (weights, m, v):
        assert a.dtype == np.float32 and a.flags.c_contiguous
    g = np.ascontiguousarray(grad, np.float32)
    lib().orc_nrc_adam(_p(weights), _p(m), _p(v), _p(g), NRC_PARAMS, step, lr)
