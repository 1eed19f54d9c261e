/*
 * arc/layout.h — byte layouts shared by the host, the CUDA kernels and the CPU oracle.
 *
 * Every struct here is a drop-in mirror of a buffer element of the Arcadia renderer, so a
 * pool that Arcadia's `WorldMap` packs (or that its `queue.write_buffer` uploads) can be handed
 * to this library unchanged:
 *
 *   arc_node64            crates/arcadia-core/src/node64.rs:27-36, shaders/common/types.wgsl:65-70
 *   arc_brick64           crates/arcadia-core/src/node64.rs:118-120, shaders/common/types.wgsl:72-74
 *   arc_material          crates/arcadia-core/src/material.rs:42-47, shaders/common/types.wgsl:76-79
 *   arc_camera_uniforms   crates/arcadia-render/src/camera.rs:11-38, shaders/common/types.wgsl:19-63
 *   arc_sharc_slot        crates/arcadia-render/src/sharc.rs:49-54, shaders/common/sharc.wgsl:16-21
 *   arc_gi_reservoir      shaders/common/types.wgsl:90-106 (GiReservoir, 32 B)
 *   arc_rigid_body        crates/arcadia-physics/src/rigid_voxel/types.rs:20-31, shaders/common/types.wgsl:220-226
 *   G-buffer words        shaders/common/types.wgsl:292-332 (20 B per pixel in three arrays)
 *
 * Two records have no buffer counterpart in the reference and are this library's own:
 * arc_ray (a 24 B ray for the batch-ray entry point) and arc_hit_record (a 20 B per-ray hit:
 * global voxel i32x3, face id, material, flags, depth in meters).
 *
 * Plain C11 so the oracle (gcc, C) and the product (g++/nvcc, C++17) include the same file.
 */
#ifndef ARC_LAYOUT_H
#define ARC_LAYOUT_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#define ARC_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define ARC_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif

/* Scale constants: shaders/common/types.wgsl:4-8, crates/arcadia-core/src/coord.rs:7-16. */
#define ARC_VOXEL_SIZE 0.0625f
#define ARC_VOXELS_PER_METER 16.0f
#define ARC_CHUNK_DIM 256u
#define ARC_CHUNK_DIM_F 256.0f
#define ARC_EMPTY_CHUNK 0xFFFFFFFFu

/* Node flags: crates/arcadia-core/src/node64.rs:9-16. */
#define ARC_IS_LEAF_FLAG 0x80000000u
#define ARC_IS_UNIFORM_FLAG 0x40000000u
#define ARC_PTR_INDEX_MASK 0x3FFFFFFFu

/* Material ids that change traversal or shading: crates/arcadia-core/src/material.rs:8-36. */
#define ARC_MAT_AIR 0u
#define ARC_MAT_WATER_CRYSTAL 18u
#define ARC_MAT_POINT_LIGHT 27u
#define ARC_MAT_MIRROR_CHROME 28u

/* Face ids in the order of `sharc_norm_id` (shaders/common/sharc.wgsl:48-57). */
#define ARC_FACE_POS_X 0u
#define ARC_FACE_NEG_X 1u
#define ARC_FACE_POS_Y 2u
#define ARC_FACE_NEG_Y 3u
#define ARC_FACE_POS_Z 4u
#define ARC_FACE_NEG_Z 5u
#define ARC_FACE_NONE 0xFFu

/* SHARC constants: shaders/common/sharc.wgsl:4-12, crates/arcadia-render/src/sharc.rs:7-19. */
#define ARC_SHARC_BUCKETS 32768u
#define ARC_SHARC_WAYS 4u
#define ARC_SHARC_SLOTS 131072u
#define ARC_SHARC_NO_SLOT 0xFFFFFFFFu
#define ARC_SHARC_FIXED_SCALE 1024.0f
#define ARC_SHARC_MAX_RADIANCE 32.0f
#define ARC_SHARC_STALE_EVICT_AGE 64u
#define ARC_SHARC_HISTORY_CAP 16.0f
#define ARC_SHARC_KEY_VALID_BIT 0x80000000u

/* One 64-tree node (16 B). Internal: mask = child occupancy, child_ptr = base of the contiguous
 * child slice in the node pool. Leaf: mask = 4x4x4 voxel occupancy, child_ptr = brick index or
 * uniform flag. lod_payload = RGB8 average | primary material << 24. */
typedef struct arc_node64 {
    uint32_t mask_low;
    uint32_t mask_high;
    uint32_t child_ptr;
    uint32_t lod_payload;
} arc_node64;

/* 4x4x4 u8 materials packed into 16 u32 words; voxel b lives in word b>>2 at bit (b&3)*8. */
typedef struct arc_brick64 {
    uint32_t packed_materials[16];
} arc_brick64;

typedef struct arc_material {
    float albedo_roughness[4];
    float emission_meta[4];
} arc_material;

/* 480 B per-frame parameter block, field for field the WGSL `CameraUniforms`. The traversal reads
 * world_grid_dims, ray_steps, ray_distances, lod_settings, quality_flags and point_light_count. */
typedef struct arc_camera_uniforms {
    float cam_pos_time[4];       /* xyz eye (m), w time (s) */
    float cam_forward_fov[4];    /* xyz unit forward, w tan(fov_y/2) */
    float cam_right_aspect[4];   /* xyz unit right, w aspect */
    float cam_up_frame[4];       /* xyz unit up, w bitcast(frame_index) */
    float prev_view_proj[16];    /* column-major */
    float curr_view_proj[16];    /* column-major */
    uint32_t world_grid_dims[4]; /* xyz chunk grid, w = width | height << 16 */
    float sun_dir_intensity[4];
    float jitter_brush_dt[4];
    float target_voxel_info[4];
    uint32_t point_light_count[4]; /* x lights, y underwater | rb_count<<16, z ambient bits, w contact_ao_dist bits */
    float point_light[8][4];
    uint32_t ray_steps[4];     /* primary, secondary, gi, shadow */
    float ray_distances[4];    /* water_refr, mirror_refl, gi_max, shadow_max (m) */
    float lod_settings[4];     /* primary_lod, sec_lod, gi_lod (m), shadow_jitter */
    uint32_t quality_flags[4]; /* primary_lod_step, sec_lod_step, shadow_mode, taps | mirror<<8 | gi_lod_step<<16 | ... */
    float prev_cam_pos[4];
} arc_camera_uniforms;

typedef struct arc_sharc_slot {
    uint32_t key;
    uint32_t rad_rg;
    uint32_t rad_b_meta;
    uint32_t pad;
} arc_sharc_slot;

/* ReSTIR GI reservoir of one pixel. norm_m_flags: bits 0..15 octahedral normal of the sample
 * (2 x 8 bit), 16..23 M, 24..30 sample age, 31 sample is sky; lo_rg / lo_b_w: f16 outgoing radiance
 * of the sample and f16 RIS weight W; primary_depth: the pixel's primary hit distance (1e5 when the
 * reservoir is empty); shadow_vis_m: f16 temporal sun visibility and its sample count. */
typedef struct arc_gi_reservoir {
    float sample_pos[3];
    uint32_t norm_m_flags;
    uint32_t lo_rg;
    uint32_t lo_b_w;
    float primary_depth;
    uint32_t shadow_vis_m;
} arc_gi_reservoir;

/* One rigid voxel body (GpuRigidBodyInstance, 224 B): column-major 4x4 matrices world -> body-local
 * meters, body-local -> world meters now and in the previous frame; local_bounds_and_root.xyz the
 * body's local box in meters (at most 16 m: its tree is one 256^3 chunk tree in the node pool) and .w
 * the bit pattern of its root node index; world_sphere its bounding sphere (centre, radius) in
 * meters. The camera's point_light_count.y >> 16 says how many of the uploaded bodies are traced. */
#define ARC_MAX_RIGID_BODIES 32u
typedef struct arc_rigid_body {
    float world_to_local[16];
    float local_to_world[16];
    float prev_local_to_world[16];
    float local_bounds_and_root[4];
    float world_sphere[4];
} arc_rigid_body;

/* A ray in world meters: origin xyz, unit direction xyz. */
typedef struct arc_ray {
    float origin_m[3];
    float dir[3];
} arc_ray;

/* Per-ray hit. voxel = global voxel coordinate of the hit cell's DDA position, face = ARC_FACE_*,
 * flags bit 0 = hit, bits 1..3 = level shift / 2 of the cell that was hit (0 = single voxel).
 * depth_m = distance along the ray in meters (plane-entry distance; 250 m style max on a miss). */
typedef struct arc_hit_record {
    int32_t voxel[3];
    uint8_t face;
    uint8_t mat;
    uint16_t flags;
    float depth_m;
} arc_hit_record;

#define ARC_HIT_FLAG_HIT 1u
/* A hit on a rigid body: voxel is the body-local voxel, face the dominant axis of the world normal,
 * flags bits 8..12 the body index. */
#define ARC_HIT_FLAG_RIGID 0x10u

ARC_STATIC_ASSERT(sizeof(arc_node64) == 16, "Node64 is 16 B");
ARC_STATIC_ASSERT(sizeof(arc_brick64) == 64, "LeafBrick64 is 64 B");
ARC_STATIC_ASSERT(sizeof(arc_material) == 32, "Material is 32 B");
ARC_STATIC_ASSERT(sizeof(arc_camera_uniforms) == 480, "CameraUniforms is 480 B");
ARC_STATIC_ASSERT(sizeof(arc_sharc_slot) == 16, "SharcResolvedSlot is 16 B");
ARC_STATIC_ASSERT(sizeof(arc_ray) == 24, "ray is 24 B");
ARC_STATIC_ASSERT(sizeof(arc_hit_record) == 20, "hit record is 20 B");
ARC_STATIC_ASSERT(sizeof(arc_gi_reservoir) == 32, "GiReservoir is 32 B");
ARC_STATIC_ASSERT(sizeof(arc_rigid_body) == 224, "GpuRigidBodyInstance is 224 B");

/* One in-place world edit. The reference has no edit record: its callers invoke
 * ChunkTree64::carve_sphere_tracked (crates/arcadia-core/src/chunk_tree/edit/carve.rs:39-176) and
 * mutate_brick_in_place (edit/set.rs:244-319) directly; this record names those two operations.
 *   ARC_EDIT_CARVE    clear every solid voxel whose centre lies within `radius` of `center` (world
 *                     voxel units; voxel v spans [v, v + 1)); no scorch rim
 *   ARC_EDIT_RECOLOR  set every solid voxel of world brick `brick` (voxel coordinates >> 2) to `material` */
#define ARC_EDIT_CARVE 0u
#define ARC_EDIT_RECOLOR 1u
typedef struct arc_edit_op {
    uint32_t kind;
    uint32_t material;
    uint32_t brick[3];
    float center[3];
    float radius;
    uint32_t pad;
} arc_edit_op;
ARC_STATIC_ASSERT(sizeof(arc_edit_op) == 40, "edit record is 40 B");

#ifdef __cplusplus
}
#endif

#endif /* ARC_LAYOUT_H */
