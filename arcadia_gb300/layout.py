"""numpy mirrors of the byte layouts in ``include/arc/layout.h`` plus the camera-uniform builder.

The structured dtypes let Python hand pools, cameras and ray batches to the C ABI without
copies. ``camera_uniforms`` mirrors ``Renderer::prepare_camera_uniforms``
(crates/arcadia-render/src/renderer.rs:513-649) for a pinhole camera given by yaw/pitch, and
``quality_high`` / ``quality_parity`` are the ``RaymarchQualitySettings`` presets it packs
(crates/arcadia-render/src/quality.rs:101-134).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

VOXEL_SIZE = np.float32(0.0625)
CHUNK_DIM = 256
EMPTY_CHUNK = 0xFFFFFFFF
IS_LEAF_FLAG = 0x80000000
IS_UNIFORM_FLAG = 0x40000000
PTR_INDEX_MASK = 0x3FFFFFFF
SHARC_BUCKETS = 32768
SHARC_WAYS = 4
SHARC_SLOTS = 131072
FACE_NONE = 0xFF

NODE_DTYPE = np.dtype([("mask_low", "<u4"), ("mask_high", "<u4"), ("child_ptr", "<u4"), ("lod_payload", "<u4")])
BRICK_DTYPE = np.dtype([("packed_materials", "<u4", (16,))])
MATERIAL_DTYPE = np.dtype([("albedo_roughness", "<f4", (4,)), ("emission_meta", "<f4", (4,))])
SHARC_SLOT_DTYPE = np.dtype([("key", "<u4"), ("rad_rg", "<u4"), ("rad_b_meta", "<u4"), ("pad", "<u4")])
RAY_DTYPE = np.dtype([("origin_m", "<f4", (3,)), ("dir", "<f4", (3,))])
HIT_DTYPE = np.dtype(
    [("voxel", "<i4", (3,)), ("face", "u1"), ("mat", "u1"), ("flags", "<u2"), ("depth_m", "<f4")]
)
CAMERA_DTYPE = np.dtype(
    [
        ("cam_pos_time", "<f4", (4,)),
        ("cam_forward_fov", "<f4", (4,)),
        ("cam_right_aspect", "<f4", (4,)),
        ("cam_up_frame", "<f4", (4,)),
        ("prev_view_proj", "<f4", (16,)),
        ("curr_view_proj", "<f4", (16,)),
        ("world_grid_dims", "<u4", (4,)),
        ("sun_dir_intensity", "<f4", (4,)),
        ("jitter_brush_dt", "<f4", (4,)),
        ("target_voxel_info", "<f4", (4,)),
        ("point_light_count", "<u4", (4,)),
        ("point_light", "<f4", (8, 4)),
        ("ray_steps", "<u4", (4,)),
        ("ray_distances", "<f4", (4,)),
        ("lod_settings", "<f4", (4,)),
        ("quality_flags", "<u4", (4,)),
        ("prev_cam_pos", "<f4", (4,)),
    ]
)
VIEW_DTYPE = np.dtype(
    [
        ("world_slot", "<u4"), ("width", "<u4"), ("height", "<u4"), ("pad", "<u4"), ("cam", CAMERA_DTYPE),
        ("gbuf_depth_mat", "<u8"), ("gbuf_norm_motion", "<u8"), ("gbuf_albedo_ao", "<u8"), ("hits", "<u8"),
        ("gi_hits", "<u8"),
    ]
)
RESERVOIR_DTYPE = np.dtype(
    [("sample_pos", "<f4", (3,)), ("norm_m_flags", "<u4"), ("lo_rg", "<u4"), ("lo_b_w", "<u4"), ("primary_depth", "<f4"),
     ("shadow_vis_m", "<u4")]
)


def empty_reservoirs(n: int) -> np.ndarray:
    """create_empty_reservoir (types.wgsl:187-196) for n pixels."""
    r = np.zeros(n, RESERVOIR_DTYPE)
    r["primary_depth"] = 1e5
    return r


RIGID_BODY_DTYPE = np.dtype(
    [("world_to_local", "<f4", (16,)), ("local_to_world", "<f4", (16,)), ("prev_local_to_world", "<f4", (16,)),
     ("local_bounds_and_root", "<f4", (4,)), ("world_sphere", "<f4", (4,))]
)

EDIT_CARVE = 0
EDIT_RECOLOR = 1
EDIT_DTYPE = np.dtype(
    [("kind", "<u4"), ("material", "<u4"), ("brick", "<u4", (3,)), ("center", "<f4", (3,)), ("radius", "<f4"),
     ("pad", "<u4")]
)
assert EDIT_DTYPE.itemsize == 40 and RESERVOIR_DTYPE.itemsize == 32 and RIGID_BODY_DTYPE.itemsize == 224
assert VIEW_DTYPE.itemsize == 536
assert NODE_DTYPE.itemsize == 16 and BRICK_DTYPE.itemsize == 64 and MATERIAL_DTYPE.itemsize == 32
assert CAMERA_DTYPE.itemsize == 480 and SHARC_SLOT_DTYPE.itemsize == 16
assert RAY_DTYPE.itemsize == 24 and HIT_DTYPE.itemsize == 20


@dataclass
class Quality:
    """Subset of ``RaymarchQualitySettings`` that the traversal path reads (quality.rs:6-81)."""

    primary_max_steps: int = 200
    sec_max_steps: int = 72
    gi_max_steps: int = 48
    shadow_max_steps: int = 72
    water_refr_dist: float = 140.0
    mirror_refl_dist: float = 120.0
    gi_max_dist: float = 26.0
    shadow_max_dist: float = 88.0
    primary_lod_dist: float = 120.0
    primary_lod_step: int = 155
    sec_lod_dist: float = 28.0
    sec_lod_step: int = 60
    gi_lod_dist: float = 24.0
    gi_lod_step: int = 48
    shadow_jitter: float = 0.018
    shadow_mode: int = 0
    denoiser_taps: int = 16
    mirror_adaptive: int = 0
    dither_mode: int = 3
    tonemapper_mode: int = 0
    ambient_floor: float = 0.005
    contact_ao_dist: float = 24.0


def quality_high() -> Quality:
    """``RaymarchQualitySettings::high_quality`` (quality.rs:101-134)."""
    return Quality()


def quality_parity(max_steps: int = 512) -> Quality:
    """Parity mode A: up to ``max_steps`` DDA steps for every ray class and LOD pushed out of reach.

    The GI LOD step threshold is an 8-bit field of ``quality_flags.w`` (traversal64.wgsl:275), so
    GI rays still switch to 0.25 m cells after step 255.
    """
    q = Quality()
    q.primary_max_steps = q.sec_max_steps = q.gi_max_steps = max_steps
    q.primary_lod_dist = q.sec_lod_dist = q.gi_lod_dist = 1.0e9
    q.primary_lod_step = q.sec_lod_step = 0xFFFFFFFF
    q.gi_lod_step = 255
    return q


def _look_to_rh(eye, fwd, up):
    f = np.asarray(fwd, np.float64)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3] = s
    m[1, :3] = u
    m[2, :3] = -f
    m[0, 3] = -np.dot(s, eye)
    m[1, 3] = -np.dot(u, eye)
    m[2, 3] = np.dot(f, eye)
    return m


def _perspective_infinite_reverse_rh(fov_y, aspect, z_near):
    f = 1.0 / math.tan(0.5 * fov_y)
    m = np.zeros((4, 4))
    m[0, 0] = f / aspect
    m[1, 1] = f
    m[2, 3] = z_near
    m[3, 2] = -1.0
    return m


def camera_uniforms(
    grid,
    width: int,
    height: int,
    eye_m,
    yaw_deg: float = 0.0,
    pitch_deg: float = -30.0,
    fov_y_deg: float = 70.0,
    quality: Quality | None = None,
    frame_index: int = 0,
    sun_dir=(0.35, 0.80, 0.25),
    sun_intensity: float = 3.0,
    jitter=(0.0, 0.0),
    prev_eye_m=None,
    prev_view_proj=None,
) -> np.ndarray:
    """Builds one ``CameraUniforms`` record the way ``prepare_camera_uniforms`` packs it."""
    q = quality or quality_high()
    yaw, pitch = math.radians(yaw_deg), math.radians(pitch_deg)
    fwd = np.array([math.cos(pitch) * math.sin(yaw), math.sin(pitch), -math.cos(pitch) * math.cos(yaw)], np.float32)
    fwd /= np.linalg.norm(fwd)
    right = np.array([math.cos(yaw), 0.0, math.sin(yaw)], np.float32)
    right /= np.linalg.norm(right)
    up = np.cross(right, fwd).astype(np.float32)
    up /= np.linalg.norm(up)
    aspect = np.float32(width) / np.float32(height)
    tan_half = np.float32(math.tan(math.radians(fov_y_deg) * 0.5))
    view = _look_to_rh(np.asarray(eye_m, np.float64), fwd.astype(np.float64), up.astype(np.float64))
    proj = _perspective_infinite_reverse_rh(math.radians(fov_y_deg), float(aspect), 0.1)
    vp = (proj @ view).astype(np.float32)
    sd = np.asarray(sun_dir, np.float32)
    sd = sd / np.linalg.norm(sd)

    c = np.zeros(1, CAMERA_DTYPE)
    c["cam_pos_time"][0] = [eye_m[0], eye_m[1], eye_m[2], 0.0]
    c["cam_forward_fov"][0] = [fwd[0], fwd[1], fwd[2], tan_half]
    c["cam_right_aspect"][0] = [right[0], right[1], right[2], aspect]
    c["cam_up_frame"][0, :3] = up
    c["cam_up_frame"][0, 3] = np.array([frame_index & 0xFFFFFFFF], np.uint32).view(np.float32)[0]
    # column-major matrices (glam to_cols_array_2d)
    c["curr_view_proj"][0] = vp.T.reshape(16)
    pvp = vp if prev_view_proj is None else np.asarray(prev_view_proj, np.float32)
    c["prev_view_proj"][0] = pvp.T.reshape(16)
    c["world_grid_dims"][0] = [grid[0], grid[1], grid[2], (width & 0xFFFF) | ((height & 0xFFFF) << 16)]
    c["sun_dir_intensity"][0] = [sd[0], sd[1], sd[2], sun_intensity]
    c["jitter_brush_dt"][0] = [jitter[0], jitter[1], 0.0, 0.016]
    c["point_light_count"][0] = [
        0,
        0,
        np.array([q.ambient_floor], np.float32).view(np.uint32)[0],
        np.array([q.contact_ao_dist], np.float32).view(np.uint32)[0],
    ]
    c["ray_steps"][0] = [q.primary_max_steps, q.sec_max_steps, q.gi_max_steps, q.shadow_max_steps]
    c["ray_distances"][0] = [q.water_refr_dist, q.mirror_refl_dist, q.gi_max_dist, q.shadow_max_dist]
    c["lod_settings"][0] = [q.primary_lod_dist, q.sec_lod_dist, q.gi_lod_dist, q.shadow_jitter]
    c["quality_flags"][0] = [
        q.primary_lod_step & 0xFFFFFFFF,
        q.sec_lod_step & 0xFFFFFFFF,
        q.shadow_mode,
        (q.denoiser_taps | (q.mirror_adaptive << 8) | ((q.gi_lod_step & 0xFF) << 16) | ((q.dither_mode & 7) << 24)
         | ((q.tonemapper_mode & 1) << 27)),
    ]
    pe = eye_m if prev_eye_m is None else prev_eye_m
    c["prev_cam_pos"][0] = [pe[0], pe[1], pe[2], 0.0]
    return c


@dataclass
class SceneParams:
    """Seeded synthetic world: 2D value-noise heightfield and optional 3D value-noise caves."""

    grid: tuple = (1, 1, 1)
    seed: int = 1
    caves: bool = False
    cave_threshold: float = 0.6
    height_lo: float = 0.25
    height_hi: float = 0.75
    cave_depth: int = 0  # caves only within this many voxels below the surface (0 = at any depth)


SCENES = {
    # 256^3, one chunk (4-level 64-tree), heightfield only
    "c1_256": SceneParams(grid=(1, 1, 1), seed=1, caves=False),
    # 512^3 (2^3 chunks)
    "s512": SceneParams(grid=(2, 2, 2), seed=2, caves=False),
    # 1024^3 (4^3 chunks), heightfield + caves
    "c2_1024_caves": SceneParams(grid=(4, 4, 4), seed=3, caves=True),
    # 1024^3 heightfield only
    "s1024": SceneParams(grid=(4, 4, 4), seed=4, caves=False),
    # 512^3 with caves in a 40-voxel band under the surface (small case of the 4096^3 scene's structure)
    "band512": SceneParams(grid=(2, 2, 2), seed=6, caves=True, cave_depth=40),
    # 4096^3 = 16^3 chunks (6-level 64-tree), sparse: terrain between 20 % and 35 % of the height,
    # caves in a 48-voxel band under the surface
    "c5_4096": SceneParams(grid=(16, 16, 16), seed=5, caves=True, height_lo=0.20, height_hi=0.35, cave_depth=48),
}


def default_camera_for(scene: SceneParams, width: int, height: int, quality: Quality | None = None, **kw):
    """Camera of the benchmark configs: above the centre of the world, looking down 30 degrees.

    For the 256^3 world this is (128, 220, 128) voxels = (8, 13.75, 8) m with FOV_y 70 degrees; larger
    worlds scale the position with the world size.
    """
    gx, gy, gz = scene.grid
    eye = (gx * 256 * 0.5 * 0.0625, gy * 256 * (220.0 / 256.0) * 0.0625, gz * 256 * 0.5 * 0.0625)
    kw.setdefault("pitch_deg", -30.0)
    kw.setdefault("fov_y_deg", 70.0)
    return camera_uniforms(scene.grid, width, height, eye, quality=quality, **kw)
