"""ctypes front end of ``libarc_trace.so`` (the C ABI in ``include/arc/arc_trace.h``).

``Tracer`` wraps one ``arc_ctx``. Host-array methods take numpy arrays with the dtypes of
``arcadia_gb300.layout``; ``*_dev`` methods take raw device pointers (e.g. ``torch.Tensor.data_ptr()``).
The library must be built (``python -m arcadia_gb300.build``): there is no fallback path, a missing
library or a failing call raises ``ArcError``.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from .layout import (
    BRICK_DTYPE,
    CAMERA_DTYPE,
    EDIT_DTYPE,
    HIT_DTYPE,
    MATERIAL_DTYPE,
    NODE_DTYPE,
    RAY_DTYPE,
    SHARC_SLOT_DTYPE,
    SceneParams,
)

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libarc_trace.so")

ARC_OK = 0
ARC_FEAT_WARP_FETCH = 1
ARC_FEAT_NODE_VISIT = 2
ARC_FEAT_GI_SORT = 4
ARC_FEAT_TOP_TABLE = 8
ARC_FEAT_GRID_STRIDE = 16
ARC_FEAT_PRECOMP = 32
ARC_FEAT_GI_REPACK = 64
ERRORS = {
    -1: "ARC_E_INVALID_ARG",
    -2: "ARC_E_CUDA",
    -3: "ARC_E_NO_WORLD",
    -4: "ARC_E_INVALID_POOL",
    -5: "ARC_E_OUT_OF_MEMORY",
    -6: "ARC_E_DEVICE_CHECK",
    -7: "ARC_E_NO_CAMERA",
    -8: "ARC_E_CAPACITY",
}

# Every entry point include/arc/*.h declares, with its ctypes signature.
_vp, _u32, _u64, _f32, _i32, _sz = C.c_void_p, C.c_uint32, C.c_uint64, C.c_float, C.c_int, C.c_size_t
SIGNATURES = {
    "arc_create": [_i32, C.POINTER(_vp)],
    "arc_destroy": [_vp],
    "arc_last_error": [_vp, C.c_char_p, _sz],
    "arc_synchronize": [_vp],
    "arc_get_stream": [_vp, C.POINTER(_vp)],
    "arc_set_launch_config": [_vp, _vp],
    "arc_set_frame_bands": [_vp, _u32],
    "arc_autotune_frame_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _u32, _vp, _vp],
    "arc_get_launch_config": [_vp, _vp],
    "arc_get_stats": [_vp, _vp],
    "arc_debug_set": [_vp, _i32, C.c_longlong],
    "arc_upload_world": [_vp, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp, _u32, _u32],
    "arc_apply_patch": [_vp, _u32, _u32, _u32, _vp, _u32, _u32, _vp, _u32],
    "arc_set_camera": [_vp, _vp],
    "arc_upload_world_slot": [_vp, _u32, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp],
    "arc_trace_views_dev": [_vp, _vp, _u32, _vp, _i32],
    "arc_autotune_views_dev": [_vp, _vp, _u32, _u32, _vp, _vp],
    "arc_trace_primary": [_vp, _u32, _u32, _vp, _vp, _vp, _vp],
    "arc_trace_primary_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp],
    "arc_trace_secondary": [_vp, _u32, _u32, _vp, _vp, _vp],
    "arc_trace_secondary_dev": [_vp, _u32, _u32, _vp, _vp, _vp],
    "arc_trace_frame": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_trace_frame_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_trace_frame_noalloc": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_reserve_surface_list": [_vp, _u64],
    "arc_set_rigid_bodies": [_vp, _vp, _u32],
    "arc_trace_rigid_bodies_dev": [_vp, _vp, _u32, _f32, _vp, _vp],
    "arc_restir_gi_temporal_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_trace_rays": [_vp, _vp, _u32, _f32, _u32, _i32, _vp],
    "arc_trace_rays_dev": [_vp, _vp, _u32, _f32, _u32, _i32, _vp],
    "arc_shadow_rays_dev": [_vp, _vp, _u32, _f32, _vp],
    "arc_sharc_reset": [_vp],
    "arc_sharc_update_dev": [_vp, _u32, _u32, _vp, _vp],
    "arc_sharc_resolve": [_vp],
    "arc_sharc_query_dev": [_vp, _vp, _vp, _vp, _u32, _vp],
    "arc_sharc_query": [_vp, _vp, _vp, _vp, _u32, _vp],
    "arc_sharc_download": [_vp, _vp, _vp, _vp],
    "arc_sharc_upload": [_vp, _vp, _vp, _vp],
    "arc_sharc_deposit_dev": [_vp, _vp, _vp, _vp, _vp, _u32],
    "arc_sharc_set_mode": [_vp, _u32],
    "arc_gi_points_from_hits_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_gi_points_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
    "arc_onebounce_dev": [_vp, _vp, _u32, _vp, _vp, _vp, _u32, _u32, _i32, _vp],
    "arc_apply_edits": [_vp, _vp, _u32, _vp],
    "arc_edit_stats": [_vp, _vp, _vp, _vp, _vp],
    "arc_download_world": [_vp, _vp, _vp, _u32, _vp, _u32, _vp, _vp],
    "arc_shadow_rays_di_dev": [_vp, _vp, _vp, _u32, _vp],
    "arc_nrc_init": [_vp, _u32],
    "arc_nrc_set_weights": [_vp, _vp],
    "arc_nrc_get_weights": [_vp, _vp],
    "arc_nrc_set_ema_decay": [_vp, _f32],
    "arc_nrc_set_ema_warmup": [_vp, _u32],
    "arc_nrc_set_output_clamp": [_vp, _i32],
    "arc_nrc_set_sample_cluster": [_vp, _u32],
    "arc_nrc_set_adam_betas": [_vp, _f32, _f32],
    "arc_set_cache_launch_overlap": [_vp, _i32],
    "arc_nrc_set_infer_path": [_vp, C.c_int],
    "arc_nrc_set_train_path": [_vp, C.c_int],
    "arc_nrc_get_ema_weights": [_vp, _vp],
    "arc_nrc_query_list_dev": [_vp, _vp, _vp, _u32, _vp, _vp, _vp],
    "arc_nrc_train_frame_dev": [_vp, _vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _f32],
    "arc_nrc_frame_dev": [_vp, _vp, _vp, _u32, _vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _f32],
    "arc_sharc_frame_dev": [_vp, _u32, _u32, _vp, _vp, _vp, _vp, _u32, _vp, _vp, _vp],
    "arc_sharc_query_list_dev": [_vp, _vp, _vp, _u32, _vp, _vp, _vp],
    "arc_nrc_query_dev": [_vp, _vp, _vp, _u32, _vp],
    "arc_nrc_query": [_vp, _vp, _vp, _u32, _vp],
    "arc_nrc_train_samples_dev": [_vp, _vp, _vp, _vp, _vp, _vp, _u32, _u32, _u32, _vp, _vp],
    "arc_nrc_grad_dev": [_vp, _vp, _vp, _u32, _vp],
    "arc_nrc_train_step_dev": [_vp, _vp, _vp, _u32, _f32, _vp],
    "arc_nrc_train_step": [_vp, _vp, _vp, _u32, _f32, _vp],
    "arc_default_palette": [_vp],
    "arc_world_build": [_vp, _vp, _i32, C.POINTER(_vp)],
    "arc_world_info": [_vp, C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u32), C.POINTER(_u64)],
    "arc_world_copy": [_vp, _vp, _vp, _vp],
    "arc_world_free": [_vp],
}

_lib = None


class ArcError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class LaunchConfig(C.Structure):
    _fields_ = [
        ("variant", C.c_uint32),
        ("block_threads", C.c_uint32),
        ("blocks_per_sm", C.c_uint32),
        ("tile_w", C.c_uint32),
        ("tile_h", C.c_uint32),
        ("refill_threshold", C.c_uint32),
        ("reg_blocks", C.c_uint32),
        ("order", C.c_uint32),
        ("features", C.c_uint32),
    ]


class Stats(C.Structure):
    _fields_ = [("last_kernel_ms", C.c_float), ("rays_traced", C.c_uint64), ("device_status", C.c_uint32),
                ("n_sm", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("grid", C.c_uint32 * 3), ("seed", C.c_uint32), ("caves", C.c_uint32), ("cave_threshold", C.c_float),
                ("height_lo", C.c_float), ("height_hi", C.c_float), ("cave_depth", C.c_uint32)]


def lib() -> C.CDLL:
    """Loads libarc_trace.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ArcError(-2, f"{LIB_PATH} is missing: build it with `python -m arcadia_gb300.build`")
        L = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            fn = getattr(L, name, None)
            if fn is None:
                continue
            fn.argtypes = args
            fn.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    """Pointer argument: None, a device address (int) or a host array. The array's pointer object
    keeps the array alive, so a temporary made by a dtype conversion in the call expression outlives
    the C call."""
    if a is None:
        return None
    if isinstance(a, int):
        return a
    return a.ctypes.data_as(C.c_void_p)


def default_palette() -> np.ndarray:
    pal = np.zeros(256, MATERIAL_DTYPE)
    rc = lib().arc_default_palette(_p(pal))
    if rc:
        raise ArcError(rc, "arc_default_palette")
    return pal


def build_world(scene: SceneParams, palette: np.ndarray | None = None, threads: int = 0):
    """Native world build: returns (roots, nodes, bricks, solid_voxels)."""
    d = SceneDesc((C.c_uint32 * 3)(*scene.grid), scene.seed, int(scene.caves), scene.cave_threshold, scene.height_lo,
                  scene.height_hi, scene.cave_depth)
    h = C.c_void_p()
    pal = None if palette is None else np.ascontiguousarray(palette).view(MATERIAL_DTYPE)
    rc = lib().arc_world_build(C.byref(d), _p(pal), threads, C.byref(h))
    if rc:
        raise ArcError(rc, "arc_world_build")
    try:
        nr, nn, nb, solid = C.c_uint32(), C.c_uint32(), C.c_uint32(), C.c_uint64()
        lib().arc_world_info(h, C.byref(nr), C.byref(nn), C.byref(nb), C.byref(solid))
        roots = np.zeros(nr.value, np.uint32)
        nodes = np.zeros(nn.value, NODE_DTYPE)
        bricks = np.zeros(nb.value, BRICK_DTYPE)
        lib().arc_world_copy(h, _p(roots), _p(nodes), _p(bricks))
    finally:
        lib().arc_world_free(h)
    return roots, nodes, bricks, int(solid.value)


class Tracer:
    """One arc_ctx: pools + camera + SHARC cache on one device and stream."""

    def __init__(self, device: int = 0):
        self._ctx = C.c_void_p()
        self._check(lib().arc_create(device, C.byref(self._ctx)), "arc_create")

    def close(self):
        if self._ctx:
            lib().arc_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def ctx(self):
        return self._ctx

    def last_error(self) -> str:
        buf = C.create_string_buffer(512)
        lib().arc_last_error(self._ctx, buf, 512)
        return buf.value.decode(errors="replace")

    def _check(self, rc: int, what: str):
        if rc != ARC_OK:
            msg = self.last_error() if self._ctx else what
            raise ArcError(rc, f"{what}: {msg}")

    # pools / camera -----------------------------------------------------------------------------
    def upload_world(self, grid, roots, nodes, bricks, palette, node_headroom=0, brick_headroom=0):
        g = np.asarray(grid, np.uint32)
        self._roots = np.ascontiguousarray(roots, np.uint32)
        nodes = np.ascontiguousarray(nodes).view(NODE_DTYPE)
        bricks = np.ascontiguousarray(bricks).view(BRICK_DTYPE)
        pal = np.ascontiguousarray(palette).view(MATERIAL_DTYPE)
        self._check(lib().arc_upload_world(self._ctx, _p(g), _p(self._roots), len(self._roots), _p(nodes), len(nodes),
                                           _p(bricks), len(bricks), _p(pal), node_headroom, brick_headroom),
                    "arc_upload_world")

    def apply_patch(self, chunk, new_root, node_offset, nodes, brick_offset, bricks):
        nodes = np.ascontiguousarray(nodes).view(NODE_DTYPE)
        bricks = np.ascontiguousarray(bricks).view(BRICK_DTYPE)
        self._check(lib().arc_apply_patch(self._ctx, chunk, new_root, node_offset, _p(nodes) if len(nodes) else None,
                                          len(nodes), brick_offset, _p(bricks) if len(bricks) else None, len(bricks)),
                    "arc_apply_patch")

    def apply_edits(self, ops: np.ndarray, sync: bool = False):
        """In-place edits (layout.EDIT_DTYPE records, applied in order) on the device; with sync=True
        returns the running count of rewritten bricks."""
        ops = np.ascontiguousarray(ops).view(EDIT_DTYPE)
        out = C.c_uint32(0)
        self._check(lib().arc_apply_edits(self._ctx, _p(ops) if len(ops) else None, len(ops),
                                          C.byref(out) if sync else None), "arc_apply_edits")
        return out.value if sync else None

    def download_world(self):
        """(roots, nodes, bricks) as the device holds them, up to the last written node and brick."""
        nn, nb = C.c_uint32(0), C.c_uint32(0)
        self._check(lib().arc_download_world(self._ctx, None, None, 0, None, 0, C.byref(nn), C.byref(nb)), "arc_download_world")
        roots = np.zeros(len(self._roots), np.uint32)
        nodes = np.zeros(nn.value, NODE_DTYPE)
        bricks = np.zeros(nb.value, BRICK_DTYPE)
        self._check(lib().arc_download_world(self._ctx, _p(roots), _p(nodes), nn.value, _p(bricks), nb.value, None, None),
                    "arc_download_world")
        return roots, nodes, bricks

    def edit_stats(self):
        v = [C.c_uint32(0) for _ in range(4)]
        self._check(lib().arc_edit_stats(self._ctx, *[C.byref(x) for x in v]), "arc_edit_stats")
        return {"next_node": v[0].value, "next_brick": v[1].value, "bricks_rewritten": v[2].value, "overflow": v[3].value}

    def set_camera(self, cam: np.ndarray):
        cam = np.ascontiguousarray(cam).view(CAMERA_DTYPE)
        self._check(lib().arc_set_camera(self._ctx, _p(cam)), "arc_set_camera")
        self._cam = cam

    def set_launch_config(self, **kw):
        cfg = self.launch_config()
        for k, v in kw.items():
            setattr(cfg, k, v)
        self._check(lib().arc_set_launch_config(self._ctx, C.byref(cfg)), "arc_set_launch_config")

    def autotune_frame_dev(self, w, h, gdm, gnm, gaa, hits=0, gi=0, frames=3):
        best = LaunchConfig()
        ms = C.c_float()
        self._check(lib().arc_autotune_frame_dev(self._ctx, w, h, gdm, gnm, gaa, hits or None, gi or None, frames,
                                                 C.byref(best), C.byref(ms)), "arc_autotune_frame_dev")
        return best, ms.value

    def launch_config(self) -> LaunchConfig:
        cfg = LaunchConfig()
        self._check(lib().arc_get_launch_config(self._ctx, C.byref(cfg)), "arc_get_launch_config")
        return cfg

    def stats(self) -> Stats:
        s = Stats()
        self._check(lib().arc_get_stats(self._ctx, C.byref(s)), "arc_get_stats")
        return s

    def stream(self) -> int:
        s = C.c_void_p()
        self._check(lib().arc_get_stream(self._ctx, C.byref(s)), "arc_get_stream")
        return s.value or 0

    def synchronize(self):
        self._check(lib().arc_synchronize(self._ctx), "arc_synchronize")

    # passes (host arrays) -----------------------------------------------------------------------
    def _dims(self):
        wd = int(self._cam["world_grid_dims"][0][3])
        return wd & 0xFFFF, wd >> 16

    def trace_primary(self, want_hits=True):
        w, h = self._dims()
        gdm = np.zeros((h * w, 2), np.uint32)
        gnm = np.zeros((h * w, 2), np.uint32)
        gaa = np.zeros(h * w, np.uint32)
        hits = np.zeros(h * w, HIT_DTYPE) if want_hits else None
        self._check(lib().arc_trace_primary(self._ctx, w, h, _p(gdm), _p(gnm), _p(gaa), _p(hits)), "arc_trace_primary")
        return gdm, gnm, gaa, hits

    def trace_secondary(self, gdm, gnm):
        w, h = self._dims()
        gi = np.zeros(h * w, HIT_DTYPE)
        self._check(lib().arc_trace_secondary(self._ctx, w, h, _p(np.ascontiguousarray(gdm, np.uint32)),
                                              _p(np.ascontiguousarray(gnm, np.uint32)), _p(gi)), "arc_trace_secondary")
        return gi

    def trace_frame(self, want_hits=True, want_gi=True):
        w, h = self._dims()
        gdm = np.zeros((h * w, 2), np.uint32)
        gnm = np.zeros((h * w, 2), np.uint32)
        gaa = np.zeros(h * w, np.uint32)
        hits = np.zeros(h * w, HIT_DTYPE) if want_hits else None
        gi = np.zeros(h * w, HIT_DTYPE) if want_gi else None
        n_gi = C.c_uint64()
        self._check(lib().arc_trace_frame(self._ctx, w, h, _p(gdm), _p(gnm), _p(gaa), _p(hits), _p(gi), C.byref(n_gi)),
                    "arc_trace_frame")
        return gdm, gnm, gaa, hits, gi, int(n_gi.value)

    def trace_rays(self, rays, max_dist_m, lod_bias=0, ignore_water=False):
        rays = np.ascontiguousarray(rays).view(RAY_DTYPE)
        hits = np.zeros(len(rays), HIT_DTYPE)
        self._check(lib().arc_trace_rays(self._ctx, _p(rays), len(rays), max_dist_m, lod_bias, int(ignore_water), _p(hits)),
                    "arc_trace_rays")
        return hits

    def upload_world_slot(self, slot, grid, roots, nodes, bricks, palette):
        g = np.asarray(grid, np.uint32)
        roots = np.ascontiguousarray(roots, np.uint32)
        nodes = np.ascontiguousarray(nodes).view(NODE_DTYPE)
        bricks = np.ascontiguousarray(bricks).view(BRICK_DTYPE)
        pal = np.ascontiguousarray(palette).view(MATERIAL_DTYPE)
        self._check(lib().arc_upload_world_slot(self._ctx, slot, _p(g), _p(roots), len(roots), _p(nodes), len(nodes),
                                                _p(bricks), len(bricks), _p(pal)), "arc_upload_world_slot")

    def trace_views_dev(self, views: np.ndarray, n_gi=0, use_graph=True):
        """views: numpy array of layout.VIEW_DTYPE (device output pointers filled in)."""
        self._views = np.ascontiguousarray(views)
        self._check(lib().arc_trace_views_dev(self._ctx, _p(self._views), len(self._views), n_gi or None,
                                              int(use_graph)), "arc_trace_views_dev")

    def autotune_views_dev(self, views: np.ndarray, frames=3):
        best = LaunchConfig()
        ms = C.c_float()
        self._views = np.ascontiguousarray(views)
        self._check(lib().arc_autotune_views_dev(self._ctx, _p(self._views), len(self._views), frames, C.byref(best),
                                                 C.byref(ms)), "arc_autotune_views_dev")
        return best, ms.value

    # passes (device pointers) -------------------------------------------------------------------
    def trace_frame_dev(self, w, h, gdm, gnm, gaa, hits=0, gi=0, n_gi=0):
        self._check(lib().arc_trace_frame_dev(self._ctx, w, h, gdm, gnm, gaa, hits or None, gi or None, n_gi or None),
                    "arc_trace_frame_dev")

    def trace_frame_noalloc(self, w, h, gdm, gnm, gaa, hits=0, gi=0, n_gi=0):
        self._check(lib().arc_trace_frame_noalloc(self._ctx, w, h, gdm, gnm, gaa, hits or None, gi or None,
                                                  n_gi or None), "arc_trace_frame_noalloc")

    def restir_gi_temporal_dev(self, w, h, gdm, gnm, gi_hits, res_in, res_out, radiance=0):
        """ReSTIR GI temporal pass over a traced frame (device pointers; reservoirs of layout.RESERVOIR_DTYPE)."""
        self._check(lib().arc_restir_gi_temporal_dev(self._ctx, w, h, gdm, gnm, gi_hits, res_in, res_out, radiance or None),
                    "arc_restir_gi_temporal_dev")

    def set_rigid_bodies(self, bodies):
        """Rigid-body table (layout.RIGID_BODY_DTYPE records; their trees must be in the node pool)."""
        from .layout import RIGID_BODY_DTYPE

        self._bodies = np.ascontiguousarray(bodies).view(RIGID_BODY_DTYPE)
        self._check(lib().arc_set_rigid_bodies(self._ctx, _p(self._bodies) if len(self._bodies) else None,
                                               len(self._bodies)), "arc_set_rigid_bodies")

    def trace_rigid_bodies_dev(self, rays, n, max_dist_m, hits, detail=0):
        self._check(lib().arc_trace_rigid_bodies_dev(self._ctx, rays, n, max_dist_m, hits, detail or None),
                    "arc_trace_rigid_bodies_dev")

    def reserve_surface_list(self, max_pixels: int):
        """Surface list (water / mirror / underwater branches) for frames of up to max_pixels pixels."""
        self._check(lib().arc_reserve_surface_list(self._ctx, int(max_pixels)), "arc_reserve_surface_list")

    def trace_primary_dev(self, w, h, gdm, gnm, gaa, hits=0):
        self._check(lib().arc_trace_primary_dev(self._ctx, w, h, gdm, gnm, gaa, hits or None), "arc_trace_primary_dev")

    def trace_secondary_dev(self, w, h, gdm, gnm, gi):
        self._check(lib().arc_trace_secondary_dev(self._ctx, w, h, gdm, gnm, gi), "arc_trace_secondary_dev")

    def trace_rays_dev(self, rays, n, max_dist_m, lod_bias, ignore_water, hits):
        self._check(lib().arc_trace_rays_dev(self._ctx, rays, n, max_dist_m, lod_bias, int(ignore_water), hits),
                    "arc_trace_rays_dev")

    def shadow_rays_dev(self, rays, n, max_dist_m, vis):
        self._check(lib().arc_shadow_rays_dev(self._ctx, rays, n, max_dist_m, vis), "arc_shadow_rays_dev")

    # SHARC --------------------------------------------------------------------------------------
    def sharc_reset(self):
        self._check(lib().arc_sharc_reset(self._ctx), "arc_sharc_reset")

    def sharc_update_dev(self, w, h, gdm, gnm):
        self._check(lib().arc_sharc_update_dev(self._ctx, w, h, gdm, gnm), "arc_sharc_update_dev")

    def sharc_resolve(self, passes: int = 1):
        for _ in range(passes):
            self._check(lib().arc_sharc_resolve(self._ctx), "arc_sharc_resolve")

    def sharc_query_dev(self, pos, normal, jitter, n, out):
        self._check(lib().arc_sharc_query_dev(self._ctx, pos, normal, jitter, n, out), "arc_sharc_query_dev")

    def sharc_deposit(self, pos, normal, cam_pos, rad, n_threads):
        args = [np.asarray(v, np.float32) for v in (pos, normal, cam_pos, rad)]
        self._check(lib().arc_sharc_deposit_dev(self._ctx, *[_p(a) for a in args], n_threads), "arc_sharc_deposit_dev")

    def sharc_download(self):
        keys = np.zeros(131072, np.uint32)
        accum = np.zeros(131072 * 4, np.uint32)
        res = np.zeros(131072, SHARC_SLOT_DTYPE)
        self._check(lib().arc_sharc_download(self._ctx, _p(keys), _p(accum), _p(res)), "arc_sharc_download")
        return keys, accum, res

    def sharc_upload(self, keys=None, accum=None, resolved=None):
        k = None if keys is None else np.ascontiguousarray(keys, np.uint32)
        a = None if accum is None else np.ascontiguousarray(accum, np.uint32)
        r = None if resolved is None else np.ascontiguousarray(resolved).view(SHARC_SLOT_DTYPE)
        self._check(lib().arc_sharc_upload(self._ctx, _p(k), _p(a), _p(r)), "arc_sharc_upload")
