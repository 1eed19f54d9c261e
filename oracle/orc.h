/*
 * orc.h — CPU oracle of the 64-tree traversal path.
 *
 * TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load this library, and only as the checker or the timed host-core baseline. Nothing in the
 * product links or calls it.
 *
 * It restates, in plain C with the canonical arithmetic of orc_math.h:
 *   - the synthetic scene (seeded heightfield + 3D value-noise caves, in the style of
 *     crates/arcadia-world/src/generator.rs:656-694);
 *   - ChunkTree64::from_generator / build_recursive / pack_build_tree
 *     (crates/arcadia-core/src/chunk_tree/builder.rs:86-378);
 *   - WorldMap::rebuild_all_gpu_pools / morton3d / relocate_chunk_nodes
 *     (crates/arcadia-world/src/world_map.rs:158-205,689-735);
 *   - trace_world_64tree_from and trace_shadow_vis (shaders/common/traversal64.wgsl:226-773);
 *   - primary_raymarch G-buffer output (shaders/primary_gbuffer.wgsl:93-312);
 *   - the Pass-2A GI secondary ray (shaders/lighting_restir_gi.wgsl:20-54,195-209);
 *   - SHARC key/claim/deposit/update/resolve/query (shaders/common/sharc.wgsl,
 *     shaders/common/sharc_query.wgsl, shaders/sharc_update.wgsl, shaders/sharc_resolve.wgsl);
 *   - the reference CPU ray query raycast_meters -> raycast_chunk_tree
 *     (crates/arcadia-world/src/world_map.rs:464-545, crates/arcadia-core/src/raycast_cpu.rs:28-327);
 *   - an FP64 plane-entry depth and a per-ray algorithmic byte counter.
 */
#ifndef ORC_H
#define ORC_H

#include <stdint.h>
#include "../include/arc/layout.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_scene_params {
    uint32_t grid[3];      /* chunks per axis */
    uint32_t seed;
    uint32_t caves;        /* 1 = carve 3D value-noise caves */
    float cave_threshold;  /* empty where cave noise > threshold (0.6) */
    float height_lo;       /* terrain height range as a fraction of world height */
    float height_hi;
    uint32_t cave_depth;   /* caves only within this many voxels below the surface (0 = at any depth) */
} orc_scene_params;

typedef struct orc_pools {
    uint32_t grid[3];
    uint32_t n_chunks;
    uint32_t* roots;
    arc_node64* nodes;
    uint32_t n_nodes;
    arc_brick64* bricks;
    uint32_t n_bricks;
    uint64_t solid_voxels;
} orc_pools;

typedef struct orc_world {
    const uint32_t* roots;
    const arc_node64* nodes;
    uint32_t n_nodes;
    const arc_brick64* bricks;
    uint32_t n_bricks;
    const arc_material* palette; /* 256 entries */
    const arc_rigid_body* bodies; /* rigid bodies (their trees live in the node pool), may be NULL */
    uint32_t n_bodies;
} orc_world;

/* Per-ray outcome in the form the CUDA kernels report it. */
typedef struct orc_trace_out {
    uint32_t hit;
    float t_voxels;
    float hit_pos_m[3];
    float normal[3];
    uint32_t mat_id;
    float lod_rgb[3];
    uint32_t voxel_hash;
    float contact_ao;
    uint32_t vi[3];
    uint32_t shift;
    uint32_t steps;
    uint32_t bytes;
} orc_trace_out;

/* world */
int orc_build_world(const orc_scene_params* p, orc_pools* out);
void orc_free_pools(orc_pools* p);
void orc_default_palette(arc_material out[256]);
uint32_t orc_scene_voxel(const orc_scene_params* p, const float* heightmap, uint32_t x, uint32_t y, uint32_t z);
void orc_scene_heightmap(const orc_scene_params* p, float* out_heights);
/* Build one chunk from a dense 256^3 u8 material volume (x fastest), as ChunkTree64::from_generator
 * with no region hint; returns node/brick counts, fills caller buffers when non-null. */
int orc_build_chunk_dense(const uint8_t* vol, const arc_material* palette, arc_node64* nodes_out, uint32_t* n_nodes,
                          arc_brick64* bricks_out, uint32_t* n_bricks);
uint32_t orc_morton3d(uint32_t x, uint32_t y, uint32_t z);

/* traversal */
void orc_trace(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
               float start_t_m, float max_dist_m, uint32_t lod_bias, int ignore_water, orc_trace_out* out);
float orc_shadow_vis_di(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
                        float max_dist_m);
float orc_shadow_vis(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
                     float max_dist_m, uint32_t* bytes);
uint32_t orc_face_id(const float n[3]);

/* Rigid-body hit (RigidTraceResult) with the body-local voxel, its cell level and the body index. */
typedef struct orc_rigid_out {
    uint32_t hit;
    float t_voxels;
    float hit_pos_m[3];
    float prev_hit_pos_m[3];
    float normal[3];
    uint32_t mat_id;
    uint32_t voxel_hash;
    float contact_ao;
    uint32_t vi[3];
    uint32_t shift;
    uint32_t body;
} orc_rigid_out;
void orc_trace_rigid_bodies(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3],
                            const float dir[3], float max_dist_m, orc_rigid_out* best);
uint32_t orc_rigid_count(const orc_world* w, const arc_camera_uniforms* cam);
void orc_trace_rigid_rays(const orc_world* w, const arc_camera_uniforms* cam, const arc_ray* rays, uint32_t n,
                          float max_dist_m, arc_hit_record* hits, float* detail, int threads);
int orc_trace_scene(const orc_world* w, const arc_camera_uniforms* cam, const float o[3], const float d[3],
                    float max_dist_m, uint32_t lod_bias, int ignore_water, orc_trace_out* r);
/* GI ray of a hit pixel from its G-buffer words and what temporal_main reuses of its setup. */
typedef struct orc_gi_ray {
    float hit_dist;
    float ray_dir[3];
    float hit_pos[3];
    float normal[3];
    float smooth_n[3];
    float xi[2];
    int guided;
    float origin[3];
    float dir[3];
} orc_gi_ray;
int orc_gi_setup(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                 uint32_t gd0, uint32_t gn0, orc_gi_ray* g, uint32_t* bytes);
void orc_ign(float px, float py, uint32_t frame, float out[2]);
void orc_oct_decode_packed(uint32_t packed, float n[3]);
/* test hooks of the G-buffer packing (orc_test.c, orc_trace.c) */
void orc_test_pack4x8unorm(const float* x, uint32_t n, uint32_t* out);
void orc_test_pack2x16snorm(const float* x, uint32_t n, uint32_t* out);
void orc_test_oct_encode(const float* nrm, uint32_t n, float* out);
void orc_sky_radiance(const float dir[3], const float sun[3], float out[3]);

/* ReSTIR GI temporal pass (orc_restir.c): res_in is the previous frame's reservoirs, res_out this
 * frame's; radiance (3 floats per pixel, may be NULL) replaces the SHARC query at secondary hits. */
void orc_restir_gi_temporal(const orc_world* w, const arc_camera_uniforms* cam, const arc_sharc_slot* resolved,
                            const float* radiance, const uint32_t* gdm, const uint32_t* gnm, const arc_gi_reservoir* res_in,
                            arc_gi_reservoir* res_out, int threads);

/* primary-pass surface branches (orc_surface.c): 1 when the hit takes one (underwater camera, water,
 * mirror); orc_surface_shade rewrites albedo (and, for water, the normal) of that hit. */
int orc_surface_special(const arc_camera_uniforms* cam, uint32_t mat);
void orc_surface_shade(const orc_world* w, const arc_camera_uniforms* cam, const float ray_dir[3],
                       const orc_trace_out* p, float albedo[3], float normal[3], uint32_t* bytes);

/* batch entry points (OpenMP over rays when threads > 1) */
void orc_trace_rays(const orc_world* w, const arc_camera_uniforms* cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                    uint32_t lod_bias, int ignore_water, arc_hit_record* hits, uint32_t* bytes_out, int threads);
void orc_primary(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                 uint32_t* gbuf_depth_mat, uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits,
                 uint32_t* bytes_out, int threads);
void orc_gi_rays(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                 const uint32_t* gbuf_depth_mat, const uint32_t* gbuf_norm_motion, arc_ray* gi_rays_out,
                 arc_hit_record* gi_hits, uint32_t* bytes_out, int threads);
/* every `stride`-th pixel of the frame, primary + GI, for the CPU throughput baseline */
uint64_t orc_frame_sample(const orc_world* w, const arc_camera_uniforms* cam, uint32_t stride, int threads,
                          uint64_t* n_primary, uint64_t* n_gi, uint64_t* checksum);

/* algorithmic bytes of the last orc_frame_sample (sum over sampled pixels, primary + GI) */
extern uint64_t orc_last_sample_bytes;

/* reference CPU ray query (raycast_meters); one hit per ray */
void orc_cpu_raycast(const orc_world* w, const uint32_t grid[3], const arc_ray* rays, uint32_t n, float max_dist_m,
                     arc_hit_record* hits, int threads);
uint64_t orc_cpu_frame_sample(const orc_world* w, const arc_camera_uniforms* cam, uint32_t stride, int threads,
                              uint64_t* n_primary, uint64_t* n_gi, uint64_t* checksum);

int orc_raycast_chunk_local(const orc_world* w, uint32_t root_idx, const float origin_v[3], const float dir[3],
                            float max_dist_v, float out[4], int32_t voxel[3], uint32_t* mat);

/* FP64 plane-entry distance (voxels) of the cell [cmin, cmin+span)^3 along the ray, clamped at 0 */
double orc_depth_fp64(const float origin_m[3], const float dir[3], const int32_t cell_min[3], uint32_t span);

/* SHARC */
void orc_sharc_make_key(const float pos[3], const float normal[3], const float cam_pos[3], const float jitter[2],
                        uint32_t* bucket, uint32_t* key);
uint32_t orc_sharc_deposit(uint32_t* keys, uint32_t* accum, uint32_t bucket, uint32_t key, const float rad[3]);
void orc_sharc_resolve(uint32_t* keys, uint32_t* accum, arc_sharc_slot* resolved);
void orc_sharc_query(const arc_sharc_slot* resolved, const float pos[3], const float normal[3], const float cam_pos[3],
                     const float jitter[2], float out[4]);
/* One SHARC update pass (sharc_update.wgsl main) over the tile grid, sequential in tile order.
 * Writes per-tile records: key, bucket, radiance (NaN-free), valid flag. */
void orc_sharc_update(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* gbuf_depth_mat,
                      const uint32_t* gbuf_norm_motion, const arc_sharc_slot* resolved_prev, uint32_t* keys,
                      uint32_t* accum, uint32_t* tile_key, uint32_t* tile_bucket, float* tile_rad, uint32_t* tile_valid);

void orc_sharc_update_mode(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* gbuf_depth_mat,
                           const uint32_t* gbuf_norm_motion, const arc_sharc_slot* resolved_prev, uint32_t* keys,
                           uint32_t* accum, uint32_t* tile_key, uint32_t* tile_bucket, float* tile_rad,
                           uint32_t* tile_valid, uint32_t mode);

/* one-bounce estimator of the cache comparison and the points / training batch built on it */
void orc_cmp_albedo(uint32_t mat, float out[3]);
void orc_onebounce_sun(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float n[3], float out[3]);
void orc_onebounce_sky(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float n[3],
                       uint32_t seed, float out[3]);
void orc_onebounce(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* idx, uint32_t n, const float* pos,
                   const float* nrm, const float* alb, uint32_t spp, uint32_t seed, int accumulate, float* out, int threads);
void orc_train_samples(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* list, uint64_t n_valid,
                       const float* pos, const float* nrm, const float* nrc_in, uint32_t seed, uint32_t n_samples,
                       uint32_t steps, uint32_t cluster, float* train_in, float* train_t, int threads);
void orc_gi_points(const orc_world* w, const arc_camera_uniforms* cam, uint32_t W, uint32_t H, const uint32_t* gdm,
                   const uint32_t* gnm, float* pos, float* nrm, float* alb, float* nrc_in, uint32_t* valid, int threads);
void orc_gi_points_from_hits(const arc_camera_uniforms* cam, uint32_t W, uint32_t H, const uint32_t* gdm, const uint32_t* gnm,
                             const arc_hit_record* gi_hits, float* pos, float* nrm, float* alb, float* nrc_in,
                             uint32_t* valid);

#ifdef __cplusplus
}
#endif

#endif /* ORC_H */
