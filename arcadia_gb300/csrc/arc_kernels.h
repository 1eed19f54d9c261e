// arc_kernels.h — host-visible parameter blocks and launchers of the traversal kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/arc/arc_trace.h"

namespace arc {

struct World;  // arc_traverse.cuh

// Materials with primary-pass surface branches (shaders/common/types.wgsl:15,17).
constexpr uint32_t kMatWaterCrystal = 18u;
constexpr uint32_t kMatMirrorChrome = 28u;

// One hit that takes a surface branch (32 B): output pixel index, pixel coordinates, material,
// face and view, voxel hash, hit distance and hit position of the primary ray (arc_surface.cuh).
struct SurfaceEntry {
    uint32_t k;
    uint32_t xy;             // x | y << 16
    uint32_t mat_face_view;  // mat | face << 8 | view << 16
    uint32_t hash;
    float hit_dist;
    float hp[3];
};
static_assert(sizeof(SurfaceEntry) == 32, "SurfaceEntry is 32 B");

// Per-launch scratch in device memory, cleared before every frame launch.
struct Scratch {
    uint32_t queue_head;          // next queue entry of the persistent kernel
    uint32_t surf_count;          // surface-list entries of a single-band launch
    unsigned long long gi_rays;   // GI rays traced
};

// Where a frame launch traces its GI rays (for a frame with do_gi).
enum GiMode : uint32_t {
    kGiFused = 0u,  // in the frame kernel, after the pixel's primary ray
    kGiRows = 1u,   // after the frame kernel, gi_rows_kernel traces the GI rays of the launch's rows
};

struct FrameParams;

// Scratch of the frame's GI pass with a global sort of its rays (ARC_FEAT_GI_SORT): a counting sort by
// key = direction octant << 12 | Morton code of the origin's cell on a 16 x 16 x 16 grid over the world.
constexpr uint32_t kGiSortBins = 1u << 15;
struct GiSortScratch {
    uint32_t* bins;    // kGiSortBins counters (then the bins' running slots), and the ray total after them
    float4* ray_pix;   // per pixel: GI ray origin xyz, w = key bits (0xFFFFFFFF: no GI ray)
    float4* ray_dir;   // per pixel: GI ray direction xyz
    float4* sorted;    // per sorted slot, two float4: origin xyz + pixel index bits, direction xyz
    uint32_t cell_shift;  // voxel coordinate >> cell_shift = cell (0..15 per axis)
};

}  // namespace arc

#include "arc_traverse.cuh"

namespace arc {

struct FrameParams {
    World world;
    uint32_t width, height;
    uint32_t* gbuf_depth_mat;
    uint32_t* gbuf_norm_motion;
    uint32_t* gbuf_albedo_ao;
    arc_hit_record* hits;
    arc_hit_record* gi_hits;
    uint32_t do_gi;
    Scratch* scratch;
    uint32_t tile_w, tile_h, tiles_x, queue_len, refill_threshold;
    uint32_t row0, row_end;  // rows traced by this launch (a band of the frame; 0, height for all)
    // Surface list of this launch's rows (null when no hit can take a water / mirror / underwater
    // branch): hits that take one are appended here and shaded by launch_surface afterwards.
    SurfaceEntry* surf;
    uint32_t* surf_count;
    uint32_t surf_cap;
    uint32_t gi_mode;  // GiMode of the plain kernel (the persistent kernel always fuses)
    uint32_t order;    // block order of the plain kernel and the GI pass: 0 row-major, 1 Morton (block_coords)
    GiSortScratch gisort;  // bins == nullptr: the GI pass sorts per block (gi_rows_kernel)
    uint4* top;            // ARC_FEAT_TOP_TABLE: table of chunk roots + level-1 nodes (kTopMaxNodes entries)
    uint32_t* top_info;    // its entry count (0: the table did not fit)
};
constexpr uint32_t kTopMaxNodes = 3072;  // 48 KB of 16-byte nodes

// One view of a batched launch: camera block, world slot, resolution, queue offset, outputs.
struct ViewDev {
    arc_camera_uniforms cam;
    uint32_t slot, width, height, tiles_x;
    uint32_t queue_begin, view_id, surf_cap, pad2;
    uint32_t* gbuf_depth_mat;
    uint32_t* gbuf_norm_motion;
    uint32_t* gbuf_albedo_ao;
    arc_hit_record* hits;
    arc_hit_record* gi_hits;
    SurfaceEntry* surf;      // the batch's surface list (shared by all views; null when unused)
    uint32_t* surf_count;
};

struct ViewsParams {
    const ViewDev* views;
    uint32_t n_views;
    const World* worlds;
    Scratch* scratch;
    uint32_t queue_len, tile_w, tile_h, refill_threshold;
    uint32_t surf;      // 1 when the views carry a surface list (the kernels list surface-branch hits)
    uint32_t gi_split;  // 1: views_plain_kernel stops after the primary ray and views_gi_kernel traces the GI rays
    uint32_t order;     // tile order within a view: 0 row-major, 1 Morton super-tiles of 8 x 8 tiles
};

cudaError_t launch_views(const ViewsParams& V, const arc_launch_config& cfg, int n_sm, cudaStream_t st);
// Work between a frame's primary kernel and its GI pass: the surface branches (they rewrite only the
// albedo bytes, and the GI pass reads only depth and normal) and an event that marks the G-buffer and
// the primary hit records final, so their copies can start under the GI pass. The forms without a
// separate GI pass (persistent, fused, rigid bodies) do both after their kernel.
struct FrameHooks {
    bool surface;              // launch_surface here; the caller does not launch it again
    cudaEvent_t primary_done;  // recorded once the G-buffer and primary hit records are final (or null)
};
cudaError_t launch_frame(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg, int n_sm,
                         cudaStream_t st, const FrameHooks* hooks = nullptr);
// Surface branches of the hits a frame launch listed (one thread per entry, grid-stride).
cudaError_t launch_surface(const FrameParams& P, const arc_camera_uniforms& cam, int n_sm, cudaStream_t st);
cudaError_t launch_surface_views(const ViewsParams& V, const SurfaceEntry* surf, const uint32_t* count, uint32_t cap,
                                 int n_sm, cudaStream_t st);
cudaError_t launch_secondary(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg,
                             cudaStream_t st);
cudaError_t launch_rays(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                        uint32_t lod_bias, int ignore_water, arc_hit_record* hits, cudaStream_t st);
cudaError_t launch_rigid_rays(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                              arc_hit_record* hits, float* detail, cudaStream_t st);
cudaError_t launch_shadow_di(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, const float* max_dist_m,
                             uint32_t n, float* vis, cudaStream_t st);
cudaError_t launch_shadow(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                          float* vis, cudaStream_t st);

}  // namespace arc
