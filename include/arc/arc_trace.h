/*
 * arc/arc_trace.h — C ABI of the GB300 64-tree traversal library (libarc_trace.so).
 *
 * The library stands in for three WGSL compute passes of Arcadia's renderer and the pool uploads
 * that feed them. Each entry point names the reference interface it replaces:
 *
 *   arc_upload_world     Group0 pool upload: create_group0_resources
 *                        (crates/arcadia-render/src/gpu_pools.rs:124-261) of the WorldMap pools
 *                        (crates/arcadia-world/src/world_map.rs:37-42, 158-205)
 *   arc_apply_patch      Renderer::apply_world_patches (crates/arcadia-render/src/renderer.rs:147-315)
 *                        of one GpuPatch (crates/arcadia-world/src/world_map.rs:20-27)
 *   arc_set_camera       queue.write_buffer of CameraUniforms (renderer.rs:362-366)
 *   arc_trace_primary    record_primary_raymarch_pass (crates/arcadia-render/src/pipeline.rs:150-166)
 *                        -> primary_raymarch (shaders/primary_gbuffer.wgsl:93-312)
 *   arc_trace_secondary  the Pass-2A GI secondary ray (shaders/lighting_restir_gi.wgsl:195-209)
 *   arc_trace_frame      primary + GI secondary of a whole frame (no reference counterpart: the two
 *                        passes above in one call; by default the primary kernel, then the frame's
 *                        GI rays as a pass of their own; arc_set_launch_config variant 1 = one
 *                        persistent launch for both)
 *   arc_trace_rays       trace_world_64tree (shaders/common/traversal64.wgsl:559-567) on a ray batch
 *   arc_sharc_update     record_sharc_update_pass (crates/arcadia-render/src/sharc.rs:225-241)
 *                        -> sharc_update.wgsl main (shaders/sharc_update.wgsl:148-191)
 *   arc_sharc_resolve    record_sharc_resolve_pass (sharc.rs:244-256) -> sharc_resolve.wgsl:13-70
 *   arc_sharc_query      query_sharc (shaders/common/sharc_query.wgsl:21-29) on a batch
 *   arc_nrc_query        the neural radiance cache in place of query_sharc at secondary hits
 *                        (lighting_restir_gi.wgsl:249, sharc_update.wgsl:94); no reference counterpart
 *   arc_nrc_train_step   one Adam step of that cache on a batch of radiance samples (no counterpart)
 *
 * Conventions: library-owned device memory lives behind an opaque arc_ctx; caller-owned host
 * memory is copied in and out inside the call (the *_dev variants take device pointers and
 * copy nothing). Every function returns an int status, 0 = ARC_OK, negative = ARC_E_*; no C++
 * exception crosses the ABI. One CUDA stream per context. A context is thread-compatible, not
 * thread-safe: calls on one context must not overlap.
 */
#ifndef ARC_TRACE_H
#define ARC_TRACE_H

#include <stddef.h>
#include <stdint.h>
#include "layout.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ARC_OK 0
#define ARC_E_INVALID_ARG -1
#define ARC_E_CUDA -2
#define ARC_E_NO_WORLD -3
#define ARC_E_INVALID_POOL -4
#define ARC_E_OUT_OF_MEMORY -5
#define ARC_E_DEVICE_CHECK -6 /* a device-side range check found an index outside the pools */
#define ARC_E_NO_CAMERA -7
#define ARC_E_CAPACITY -8

typedef struct arc_ctx arc_ctx;

/* Scheduling of the traversal kernels. variant 0 (the default: 128 threads, reg_blocks 3) = one
 * thread per pixel on a 2D grid for the primary rays, then the frame's GI rays as a pass of their own
 * (one thread per pixel, octant-sorted per block); variant 1 = persistent warps that refill idle lanes
 * from a global ray queue and trace each GI ray right after its primary ray. */
typedef struct arc_launch_config {
    uint32_t variant;
    uint32_t block_threads;    /* threads per CTA (multiple of 32) */
    uint32_t blocks_per_sm;    /* persistent variant: resident CTAs per SM (0 = occupancy maximum) */
    uint32_t tile_w, tile_h;   /* pixel tile a warp's 32 consecutive queue entries cover (tile_w*tile_h = 32) */
    uint32_t refill_threshold; /* persistent variant: refill when at least this many lanes are idle */
    uint32_t reg_blocks;       /* register budget: kernel built for at least this many 256-thread CTAs per SM (1-4) */
    uint32_t order;            /* variant 0: order of the pixel blocks (primary kernel and GI pass): 0 row-major,
                                  1 Morton (Z) order inside super-tiles of 8 x 8 blocks; batched views (both
                                  variants): the same two orders of each view's 32-pixel tiles */
    uint32_t features;         /* traversal variants of variant 0's primary-only kernel and GI pass (register
                                  budgets 2 and 3), ARC_FEAT_* bits; every variant gives the same results */
} arc_launch_config;

#define ARC_FEAT_WARP_FETCH 1u  /* lanes of a warp that descend into the same node load it once (match + shuffle) */
#define ARC_FEAT_NODE_VISIT 2u  /* one node evaluation per loop iteration instead of a per-step descent loop */
#define ARC_FEAT_GI_SORT 4u     /* arc_trace_frame_dev: the frame's GI rays sorted over the whole frame by
                                   (direction octant, origin cell on a 16^3 grid over the world) before they
                                   are traced (one thread per sorted ray); other entry points sort per block */
#define ARC_FEAT_TOP_TABLE 8u   /* the primary kernel as resident CTAs that loop over the pixel blocks, each CTA
                                   staging every chunk root and its level-1 children (at most 48 KB, else
                                   read from the pool) in shared memory once */
#define ARC_FEAT_GRID_STRIDE 16u /* the same resident-CTA primary kernel without the staged table (the
                                    control of ARC_FEAT_TOP_TABLE) */
#define ARC_FEAT_PRECOMP 32u     /* the ray class's step budget, LOD thresholds and -origin/dir computed once per
                                    ray instead of every DDA step (alone, not combined with other bits) */
#define ARC_FEAT_GI_REPACK 64u   /* the GI pass packs its still-running rays into the block's first warps every
                                    refill_threshold DDA steps (with the default traversal or ARC_FEAT_PRECOMP;
                                    also arc_trace_secondary_dev) */

typedef struct arc_stats {
    float last_kernel_ms;      /* device time of the last traversal launch (CUDA events) */
    uint64_t rays_traced;      /* primary + secondary rays of the last launch */
    uint32_t device_status;    /* bit mask of device-side range check failures; bit 31 = a tensor-core
                                  pipeline wait ran out of its time budget */
    uint32_t n_sm;
} arc_stats;

int arc_create(int device, arc_ctx** out);
int arc_destroy(arc_ctx* ctx);
int arc_last_error(const arc_ctx* ctx, char* buf, size_t n);
int arc_synchronize(arc_ctx* ctx);
/* cudaStream_t of the context, for callers that order their own work after it */
int arc_get_stream(arc_ctx* ctx, void** stream);
int arc_set_launch_config(arc_ctx* ctx, const arc_launch_config* cfg);
/* Device frames (arc_trace_frame_dev) with the plain kernel run in n horizontal bands, each band's
 * primary kernel and GI pass on a stream of their own, forked from and joined back to the context's
 * stream, so one band's GI pass runs in another band's primary tail. 0 = automatic (4 bands; default),
 * 1 = one launch over the frame, at most 8. Primary-only frames, the global GI sort, the resident-CTA
 * primary and the persistent kernel always run as one launch. Results are identical. The band streams
 * are created by the first banded call (or host-buffer frame), so make one such call before capturing
 * a banded frame into a CUDA graph. No counterpart in the reference. */
int arc_set_frame_bands(arc_ctx* ctx, uint32_t n);
/* Times candidate launch configurations (variant x block size x register budget x refill threshold x
 * tile shape) on the caller's frame, installs the fastest and returns it with its median frame time.
 * No counterpart in the reference (its dispatch shape is fixed at 8x8). */
int arc_autotune_frame_dev(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat,
                           uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits,
                           arc_hit_record* gi_hits, uint32_t frames, arc_launch_config* best, float* best_ms);
int arc_get_launch_config(const arc_ctx* ctx, arc_launch_config* cfg);
int arc_get_stats(const arc_ctx* ctx, arc_stats* out);

/* Fault-injection hooks for tests of the library's failure detection; no counterpart in the
 * reference, whose renderer has no device-side checks. They make a failure happen without faulting
 * the GPU: the library's own checks must catch it and the context must stay usable.
 *   ARC_DEBUG_TC_WAIT_BUDGET        value = clock cycles each tensor-core pipeline wait of the NRC
 *                                   kernels may take before it gives up (0 restores the default of
 *                                   about one second). A wait that runs out sets bit 31 of the device
 *                                   status word; the kernel waits for its own copies and MMAs in flight,
 *                                   frees its TMEM and returns, and the call that reads the status back
 *                                   (arc_synchronize or a host-buffer entry point) fails with
 *                                   ARC_E_DEVICE_CHECK ("tensor-core pipeline wait timed out").
 *   ARC_DEBUG_TC_STALL              value 1 = the NRC tensor-core kernels arm the barrier of their weight
 *                                   copy but never issue the copy, so that wait can only run out (after
 *                                   the budget above); 0 restores normal operation.
 *   ARC_DEBUG_SKIP_POOL_VALIDATION  value 1 = arc_upload_world uploads the pools without its range
 *                                   validation, so a corrupt pool reaches the kernels; their range
 *                                   checks read an out-of-range node as empty and an out-of-range
 *                                   brick as air, and the status readback fails with
 *                                   ARC_E_DEVICE_CHECK. 0 restores the validation. */
#define ARC_DEBUG_TC_WAIT_BUDGET 1
#define ARC_DEBUG_SKIP_POOL_VALIDATION 2
#define ARC_DEBUG_TC_STALL 3
int arc_debug_set(arc_ctx* ctx, int what, long long value);

/* Pools as WorldMap packs them. The pools are validated (every child pointer, brick index and root
 * in range) before upload; node/brick capacity reserves headroom for patches. */
int arc_upload_world(arc_ctx* ctx, const uint32_t grid[3], const uint32_t* roots, uint32_t n_roots,
                     const arc_node64* nodes, uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks,
                     const arc_material* palette, uint32_t node_headroom, uint32_t brick_headroom);
int arc_apply_patch(arc_ctx* ctx, uint32_t chunk_flat_idx, uint32_t new_root_node_idx, uint32_t node_offset,
                    const arc_node64* nodes, uint32_t n_nodes, uint32_t brick_offset, const arc_brick64* bricks,
                    uint32_t n_bricks);
int arc_set_camera(arc_ctx* ctx, const arc_camera_uniforms* cam);
/* Extra worlds for batched launches (slots 1..7; slot 0 is the arc_upload_world world). No counterpart
 * in the reference, which renders one WorldMap. */
int arc_upload_world_slot(arc_ctx* ctx, uint32_t slot, const uint32_t grid[3], const uint32_t* roots, uint32_t n_roots,
                          const arc_node64* nodes, uint32_t n_nodes, const arc_brick64* bricks, uint32_t n_bricks,
                          const arc_material* palette);

/* One view of a batched launch: world slot, resolution, camera block, device outputs. */
typedef struct arc_view_desc {
    uint32_t world_slot;
    uint32_t width, height;
    uint32_t pad;
    arc_camera_uniforms cam;
    uint32_t* gbuf_depth_mat;
    uint32_t* gbuf_norm_motion;
    uint32_t* gbuf_albedo_ao;
    arc_hit_record* hits;    /* may be NULL */
    arc_hit_record* gi_hits; /* may be NULL */
} arc_view_desc;

/* Primary pass: G-buffer (gbuf_depth_mat and gbuf_norm_motion: 2 u32 per pixel, gbuf_albedo_ao:
 * 1 u32 per pixel, row-major width x height) and optional per-pixel hit records. Width and height
 * must match the camera's world_grid_dims.w. As primary_raymarch (shaders/primary_gbuffer.wgsl:93-312)
 * the G-buffer includes its surface branches: under an underwater camera (point_light_count.y & 0xFFFF)
 * every hit's albedo takes caustics and absorption; above water, a water hit (material 18) traces a
 * refraction ray (ray_distances.x) and, at grazing angles, a reflection ray, and stores the up normal;
 * a mirror hit (material 28) traces a reflection ray (ray_distances.y). Those hits are shaded by a
 * second kernel after the traversal kernel, in the same call. */
int arc_trace_primary(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat,
                      uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits);
int arc_trace_primary_dev(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat,
                          uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits);
/* GI secondary ray per hit pixel from a G-buffer; gi_hits per pixel (face ARC_FACE_NONE and flags 0
 * for pixels without a primary hit). */
int arc_trace_secondary(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                        const uint32_t* gbuf_norm_motion, arc_hit_record* gi_hits);
int arc_trace_secondary_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                            const uint32_t* gbuf_norm_motion, arc_hit_record* gi_hits);
/* Primary rays and GI rays of a frame: writes the G-buffer, primary hits and GI hits (any output may
 * be NULL except the G-buffer). n_gi_out (optional) receives the number of GI rays traced. The
 * host-buffer form traces the frame in horizontal bands on concurrent streams and copies each band's
 * G-buffer and primary hits back while its GI rays trace, and its GI hits once they are done
 * (page-locked host buffers make those copies asynchronous). The device form runs in row bands as
 * arc_set_frame_bands sets. */
int arc_trace_frame(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat, uint32_t* gbuf_norm_motion,
                    uint32_t* gbuf_albedo_ao, arc_hit_record* hits, arc_hit_record* gi_hits, uint64_t* n_gi_out);
int arc_trace_frame_dev(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat,
                        uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits,
                        arc_hit_record* gi_hits, uint64_t* n_gi_dev);
/* arc_trace_frame_dev without any device allocation, for callers that cannot call cudaMalloc while
 * they trace (a renderer whose frame loop runs under a no-allocation rule or its own memory budget).
 * No counterpart in the reference. The kernels' scratch (queue head, GI-ray counter) lives in a
 * 256-byte static device array instead of context memory; frames above 2^26 pixels are rejected with
 * ARC_E_CAPACITY. All calls in one CUDA context share that array, so calls overlapping on the GPU
 * race. The first call in a CUDA context (again after that context is recreated, e.g. after
 * cudaDeviceReset) looks up the array's address with the ctx's device current, then restores the
 * caller's current device; it should come before any stream capture. Under CUDA's lazy module
 * loading the first launch of each kernel instance may load code into device memory: make one
 * warm-up call per launch configuration (and with and without the surface list, if both occur)
 * before the region that must not allocate. */
int arc_trace_frame_noalloc(arc_ctx* ctx, uint32_t width, uint32_t height, uint32_t* gbuf_depth_mat,
                            uint32_t* gbuf_norm_motion, uint32_t* gbuf_albedo_ao, arc_hit_record* hits,
                            arc_hit_record* gi_hits, uint64_t* n_gi_dev);
/* Reserves the surface list (32 B per pixel) of the water / mirror / underwater branches for frames
 * (or view batches) of up to max_pixels pixels. The other entry points allocate it on first need;
 * arc_trace_frame_noalloc requires it when the world holds water or mirror voxels or the camera is
 * under water. No counterpart in the reference. */
int arc_reserve_surface_list(arc_ctx* ctx, uint64_t max_pixels);
/* Primary + GI rays of many views (several worlds, mixed resolutions) in one call: with the default
 * launch configuration (variant 0) the batch's primary kernel and its GI pass over every view; with
 * variant 1 one persistent launch for both (slower in every batch measured; selectable, not tuned).
 * With use_graph the batch is captured once into a CUDA graph and replayed (re-captured when the view
 * count, n_gi_dev or the launch configuration changes). Outputs per view as arc_trace_frame_dev.
 * No counterpart in the reference (one view per frame there). */
int arc_trace_views_dev(arc_ctx* ctx, const arc_view_desc* views, uint32_t n_views, uint64_t* n_gi_dev, int use_graph);
/* Autotuner of the batched launch: variant 0 over block size x register budget x tile shape x tile
 * order (row-major or Morton super-tiles); installs the fastest and returns it with its median time. */
int arc_autotune_views_dev(arc_ctx* ctx, const arc_view_desc* views, uint32_t n_views, uint32_t frames,
                           arc_launch_config* best, float* best_ms);
/* trace_world_64tree on a batch of rays (origin m, unit dir). */
int arc_trace_rays(arc_ctx* ctx, const arc_ray* rays, uint32_t n, float max_dist_m, uint32_t lod_bias,
                   int ignore_water, arc_hit_record* hits);
int arc_trace_rays_dev(arc_ctx* ctx, const arc_ray* rays, uint32_t n, float max_dist_m, uint32_t lod_bias,
                       int ignore_water, arc_hit_record* hits);
/* trace_shadow_vis on a batch (1.0 visible / 0.0 occluded per ray). */
int arc_shadow_rays_dev(arc_ctx* ctx, const arc_ray* rays, uint32_t n, float max_dist_m, float* vis);
/* trace_shadow_vis_di (shaders/common/traversal64.wgsl:781-989, called at
 * shaders/lighting_restir_gi.wgsl:744): the ReSTIR DI any-hit ray towards an emitter at distance
 * max_dist_m[i] (metres). 1.0 when the ray reaches within 2 voxels of the target or strikes an emissive
 * voxel within 16 voxels of it, else 0.0. */
int arc_shadow_rays_di_dev(arc_ctx* ctx, const arc_ray* rays, const float* max_dist_m, uint32_t n, float* vis);

/* SHARC radiance cache, library-owned (keys 512 KB, accumulators 2 MB, resolved slots 2 MB). */
int arc_sharc_reset(arc_ctx* ctx);
int arc_sharc_update_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                         const uint32_t* gbuf_norm_motion);
int arc_sharc_resolve(arc_ctx* ctx);
int arc_sharc_query_dev(arc_ctx* ctx, const float* pos, const float* normal, const float* jitter, uint32_t n,
                        float* out_rgbw);
/* Host-buffer arc_sharc_query_dev: pos/normal 3 floats, jitter 2 floats (may be NULL = no jitter) and
 * out_rgbw 4 floats per query, all in caller memory; returns when out_rgbw is filled. */
int arc_sharc_query(arc_ctx* ctx, const float* pos, const float* normal, const float* jitter, uint32_t n,
                    float* out_rgbw);
int arc_sharc_download(arc_ctx* ctx, uint32_t* keys, uint32_t* accum, arc_sharc_slot* resolved);
int arc_sharc_upload(arc_ctx* ctx, const uint32_t* keys, const uint32_t* accum, const arc_sharc_slot* resolved);
/* Test hook mirroring the reference's SHARC GPU harness (crates/arcadia-render/tests/sharc_gpu.rs:18-29):
 * n_threads device threads each deposit rad at (pos, normal) as seen from cam_pos. */
int arc_sharc_deposit_dev(arc_ctx* ctx, const float pos[3], const float normal[3], const float cam_pos[3],
                          const float rad[3], uint32_t n_threads);

/* Cache comparison (NRC vs SHARC) on identical light transport. Both caches then learn the one-bounce
 * estimator L = albedo * (c_sun max(n.l,0) V(x) + L_sky [cosine ray from x escapes]), c_sun = sun_power *
 * (1, 0.9, 0.75) * 0.55, L_sky = (0.30, 0.42, 0.60). mode 0 = reference sharc_shade_surface (default),
 * mode 1 = that estimator in arc_sharc_update_dev. No counterpart in the reference. */
int arc_sharc_set_mode(arc_ctx* ctx, uint32_t mode);
/* GI hit points of a frame (per pixel: position, normal, albedo, 9 NRC inputs, valid flag). The albedo
 * is the comparison's Lambertian albedo per material id, each channel from U[0.1, 0.9]. */
int arc_gi_points_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                      const uint32_t* gbuf_norm_motion, float* pos, float* normal, float* albedo, float* nrc_in,
                      uint32_t* valid, uint64_t* n_valid, uint32_t* list);
/* list (optional, width*height entries): the pixel indices of the points with valid = 1, compacted to
 * list[0 .. *n_valid) in no particular order. */
/* arc_gi_points_dev from the GI hit records of arc_trace_frame_dev instead of tracing the GI rays again:
 * the point is the centre of the hit cell's entry face, the normal that face's, the view direction
 * from the point to the GI ray's origin (primary hit + 0.10 m along its normal). */
int arc_gi_points_from_hits_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                                const uint32_t* gbuf_norm_motion, const arc_hit_record* gi_hits, float* pos,
                                float* normal, float* albedo, float* nrc_in, uint32_t* valid, uint64_t* n_valid,
                                uint32_t* list);
/* Mean of spp one-bounce samples at points idx[i] (idx may be NULL = identity); accumulate adds. */
int arc_onebounce_dev(arc_ctx* ctx, const uint32_t* idx, uint32_t n, const float* pos, const float* normal,
                      const float* albedo, uint32_t spp, uint32_t seed, int accumulate, float* out);

/* query_sharc at the points list[0 .. min(*n_dev, max_n)) (as from arc_gi_points_dev): out[list[j]]
 * (float4: RGB, 1 if a cached entry was found) from pos/normal[list[j]]. No counterpart in the reference
 * beyond query_sharc itself. */
int arc_sharc_query_list_dev(arc_ctx* ctx, const uint32_t* list, const uint64_t* n_dev, uint32_t max_n,
                             const float* pos, const float* normal, float* out);

/* Rigid voxel bodies (the rigid_bodies buffer, crates/arcadia-render/src/gpu_pools.rs:228-247 and
 * renderer.rs:567-602): up to ARC_MAX_RIGID_BODIES bodies whose trees are already in the node pool
 * (uploaded with the world or patched in). The camera's point_light_count.y >> 16 says how many are
 * traced (the reference's rb_count); frames whose camera names bodies trace them after the world on
 * the primary, surface and GI rays (primary_gbuffer.wgsl:121-136, lighting_restir_gi.wgsl:209-224),
 * and so do SHARC updates and the ReSTIR temporal pass. Batched views do not trace bodies (a view of
 * world slot 0 whose camera names bodies is rejected). n = 0 clears the table. */
int arc_set_rigid_bodies(arc_ctx* ctx, const arc_rigid_body* bodies, uint32_t n);
/* trace_rigid_bodies (traversal64.wgsl:1224-1244) over a ray batch (device pointers): hit records
 * (a body hit has ARC_HIT_FLAG_RIGID, the body index in flags bits 8..12 and the body-local voxel),
 * and, with detail non-NULL, 9 floats per ray: world hit point, previous-frame hit point, normal. */
int arc_trace_rigid_bodies_dev(arc_ctx* ctx, const arc_ray* rays, uint32_t n, float max_dist_m, arc_hit_record* hits,
                               float* detail);

/* ReSTIR GI temporal pass: the GI part of temporal_main (shaders/lighting_restir_gi.wgsl:61-336) for
 * every pixel of a frame traced by arc_trace_frame_dev (its G-buffer and GI hit records, which the
 * pass consumes instead of tracing the GI ray again). reservoir_in holds the previous frame's
 * reservoirs (all empty on the first frame: primary_depth 1e5, the rest 0), reservoir_out receives
 * this frame's; the camera's prev_cam_pos and the G-buffer motion vectors locate the history. The
 * radiance at a secondary hit is query_sharc's (the context's resolved SHARC cache), or, with
 * gi_radiance non-NULL, gi_radiance[3 p .. 3 p + 2] (e.g. arc_nrc_query_list_dev's output). The
 * emissive-light ReSTIR DI half of the reference pass is not part of this call (no emissive light
 * list: its DI reservoirs would be empty). */
int arc_restir_gi_temporal_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                               const uint32_t* gbuf_norm_motion, const arc_hit_record* gi_hits,
                               const arc_gi_reservoir* reservoir_in, arc_gi_reservoir* reservoir_out,
                               const float* gi_radiance);

/* In-place world edits on the device (replaces the CPU edit + GpuPatch round trip:
 * ChunkTree64::carve_sphere_tracked, crates/arcadia-core/src/chunk_tree/edit/carve.rs:39-176,
 * mutate_brick_in_place, edit/set.rs:244-569, then Renderer::apply_world_patches,
 * crates/arcadia-render/src/renderer.rs:147-315). The records (include/arc/layout.h) apply in order to
 * the world of arc_upload_world; the tree afterwards equals the reference's sequential edit node for
 * node (only the pool positions of grown nodes and bricks differ), and the next trace on the context's
 * stream sees it. Growth (uncollapsed nodes, new bricks) comes from the upload headroom. Carve radius
 * in (0, 16] voxels. bricks_rewritten (optional) synchronises and receives the running count of
 * rewritten bricks; an exhausted headroom is reported there as ARC_E_CAPACITY. */
int arc_apply_edits(arc_ctx* ctx, const arc_edit_op* ops, uint32_t n_ops, uint32_t* bricks_rewritten);
/* Copies the device pools back (pool dumps, checks after edits): the roots, and the first
 * min(cap, used) nodes and bricks, where used covers every node and brick the uploads, patches and
 * edits have written; n_nodes / n_bricks receive `used`. Any output pointer may be NULL. No reference
 * counterpart (the reference keeps the CPU copy authoritative). */
int arc_download_world(arc_ctx* ctx, uint32_t* roots, arc_node64* nodes, uint32_t node_cap, arc_brick64* bricks,
                       uint32_t brick_cap, uint32_t* n_nodes, uint32_t* n_bricks);
/* Edit allocator state: next free node and brick, bricks rewritten since the upload, overflow flags. */
int arc_edit_stats(arc_ctx* ctx, uint32_t* next_node, uint32_t* next_brick, uint32_t* bricks_rewritten,
                   uint32_t* overflow);

/* Neural radiance cache (no reference counterpart: it stands in for query_sharc at secondary hits).
 * 9 inputs per query: position normalised to [0,1]^3, normal, view direction; 3 outputs (RGB).
 * 30,400 FP32 master weights: W1[64][216], W2..W5[64][64], W6[3][64], row-major, no biases. */
int arc_nrc_init(arc_ctx* ctx, uint32_t seed);
int arc_nrc_set_weights(arc_ctx* ctx, const float* weights);
int arc_nrc_get_weights(arc_ctx* ctx, float* weights);
/* Inference reads an exponential moving average of the weights, ema = decay * ema + (1 - decay) * w
 * after every Adam step (decay 0.99 by default; 0 = the latest weights). set_weights / init restart
 * it from the given weights. */
int arc_nrc_set_ema_decay(arc_ctx* ctx, float decay);
/* Warm-up of that average: at Adam step k after init / set_weights the decay is
 * min(decay, (1 + k) / (steps + k)), so early in training the average follows the weights closely
 * (default 0 = the fixed decay from the first step: on the cache comparison, the average that starts
 * from the initial weights scores better over the first 30 frames than one that follows the early
 * weights). */
int arc_nrc_set_ema_warmup(arc_ctx* ctx, uint32_t steps);
/* on = 1: queries return max(network output, 0) per channel (radiance is not negative); 0 (default) =
 * the network output as it is. Training is unaffected. */
int arc_nrc_set_output_clamp(arc_ctx* ctx, int on);
/* Training samples in runs of k consecutive hit-list entries (k = 1, 2, 4, 8, 16 or 32; default 1 =
 * every sample from its own stratum); used when n_samples is a multiple of k. */
int arc_nrc_set_sample_cluster(arc_ctx* ctx, uint32_t k);
/* on = 1 (default): the radiance-cache kernels of both caches (NRC tcgen05 training, Adam step and
 * tcgen05 query; SHARC update, resolve and list query) are launched with programmatic dependent launch,
 * so each is scheduled while the kernel ahead of it finishes and waits for it in hardware before it
 * reads that kernel's results; 0 = plain stream order. Results are the same. No counterpart in the
 * reference. */
int arc_set_cache_launch_overlap(arc_ctx* ctx, int on);
/* Adam's moment decays (default beta1 0.9, beta2 0.99; both in [0, 1)). */
int arc_nrc_set_adam_betas(arc_ctx* ctx, float beta1, float beta2);
/* Inference kernel: 1 = tcgen05 tensor cores with TMEM accumulators, one 128-query tile per CTA and
 * two CTAs per SM; 2 = the same with four tile groups in one CTA per SM (7 % faster on a 4K hit list,
 * but its CTA takes a whole SM's shared memory); 3 = automatic (default): four groups for a query on
 * its own, one group for the query that arc_nrc_frame_dev runs beside the training samples;
 * 0 = the warp-level mma.sync kernel (kept as the comparison point). Results are identical for 1-3. */
int arc_nrc_set_infer_path(arc_ctx* ctx, int path);
/* Training kernel (gradients): 1 = tcgen05 (default), 0 = the mma.sync kernel. */
int arc_nrc_set_train_path(arc_ctx* ctx, int path);
int arc_nrc_get_ema_weights(arc_ctx* ctx, float* weights);
/* out_rgb[i] = albedo[i] * network(inputs[i]) per channel; albedo may be NULL (network output only). */
int arc_nrc_query_dev(arc_ctx* ctx, const float* inputs, const float* albedo, uint32_t n, float* out_rgb);
/* Host-buffer arc_nrc_query_dev (9 input floats, 3 albedo floats (albedo may be NULL), 3 output floats
 * per query in caller memory); returns when out_rgb is filled. */
int arc_nrc_query(arc_ctx* ctx, const float* inputs, const float* albedo, uint32_t n, float* out_rgb);
/* arc_nrc_query_dev at the points list[0 .. min(*n_dev, max_n)): out[list[j]] from inputs/albedo[list[j]]. */
int arc_nrc_query_list_dev(arc_ctx* ctx, const uint32_t* list, const uint64_t* n_dev, uint32_t max_n,
                           const float* inputs, const float* albedo, float* out_rgb);
/* One NRC frame with the query beside the training: arc_nrc_query_list_dev at the hit list (as above),
 * on a side stream, with the weights the previous frame's training left, while this frame's training
 * samples are generated; then this frame's Adam steps (as arc_nrc_train_frame_dev). The query's output
 * lags the training by one frame; the frame costs about the training alone. No counterpart in the
 * reference. */
int arc_nrc_frame_dev(arc_ctx* ctx, const uint32_t* list, const uint64_t* n_valid, uint32_t max_n, const float* pos,
                      const float* normal, const float* nrc_in, const float* albedo, float* out_rgb, uint32_t seed,
                      uint32_t n_samples, uint32_t steps, float lr);
/* One SHARC frame with the query beside the update: query_sharc at the hit list (as
 * arc_sharc_query_list_dev) against the previous frame's resolved slots, on a side stream, while
 * arc_sharc_update_dev deposits this frame's radiance; then arc_sharc_resolve. */
int arc_sharc_frame_dev(arc_ctx* ctx, uint32_t width, uint32_t height, const uint32_t* gbuf_depth_mat,
                        const uint32_t* gbuf_norm_motion, const uint32_t* list, const uint64_t* n_dev, uint32_t max_n,
                        const float* pos, const float* normal, float* out);
/* One frame of online training with no host synchronisation (graph-capturable after the first call,
 * which allocates the batch): n_samples points stratified over list[0 .. *n_valid) with a seeded
 * phase, their demodulated 1-spp one-bounce targets, then `steps` Adam steps on interleaved slices of
 * the batch (each slice spans the frame; n_samples must be a multiple of steps). A frame with
 * *n_valid = 0 leaves the weights unchanged. */
int arc_nrc_train_frame_dev(arc_ctx* ctx, const uint32_t* list, const uint64_t* n_valid, const float* pos,
                            const float* normal, const float* nrc_in, uint32_t seed, uint32_t n_samples,
                            uint32_t steps, float lr);
/* The training batch arc_nrc_train_frame_dev draws, into caller device buffers: train_in (9 floats per
 * sample) and train_t (the 1-spp one-bounce target with albedo 1, 3 floats). With sample cluster k
 * (arc_nrc_set_sample_cluster, default 1), sample i is taken from list[min(s + i mod k, n_valid - 1)],
 * s = floor((floor(i / k) * n_valid + phase) / (n_samples / k)), phase = (pcg_hash(seed) * n_valid) >> 32,
 * and stored at slot (i mod steps) * (n_samples / steps) + i / steps. Nothing is stored when
 * *n_valid = 0. */
int arc_nrc_train_samples_dev(arc_ctx* ctx, const uint32_t* list, const uint64_t* n_valid, const float* pos,
                              const float* normal, const float* nrc_in, uint32_t seed, uint32_t n_samples,
                              uint32_t steps, float* train_in, float* train_t);
/* Loss-scaled (x128) weight gradient of the mean relative-L2 loss of one batch (device output). */
int arc_nrc_grad_dev(arc_ctx* ctx, const float* inputs, const float* targets, uint32_t n, float* grad_out);
/* One Adam step (lr; beta 0.9/0.99) on a batch; loss_host (optional) receives the batch loss. */
int arc_nrc_train_step_dev(arc_ctx* ctx, const float* inputs, const float* targets, uint32_t n, float lr,
                           float* loss_host);
/* Host-buffer arc_nrc_train_step_dev (inputs 9 floats, targets 3 floats per sample in caller memory). */
int arc_nrc_train_step(arc_ctx* ctx, const float* inputs, const float* targets, uint32_t n, float lr,
                       float* loss_host);

#ifdef __cplusplus
}
#endif

#endif /* ARC_TRACE_H */
