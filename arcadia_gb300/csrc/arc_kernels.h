// arc_kernels.h — host-visible parameter blocks and launchers of the traversal kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/arc/arc_trace.h"

namespace arc {

struct World;  // arc_traverse.cuh

// Per-launch scratch in device memory, cleared before every frame launch.
struct Scratch {
    uint32_t queue_head;          // next queue entry of the persistent kernel
    uint32_t pad;
    unsigned long long gi_rays;   // GI rays traced
};

struct FrameParams;

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
};

// One view of a batched launch: camera block, world slot, resolution, queue offset, outputs.
struct ViewDev {
    arc_camera_uniforms cam;
    uint32_t slot, width, height, tiles_x;
    uint32_t queue_begin, pad0, pad1, pad2;
    uint32_t* gbuf_depth_mat;
    uint32_t* gbuf_norm_motion;
    uint32_t* gbuf_albedo_ao;
    arc_hit_record* hits;
    arc_hit_record* gi_hits;
    void* pad3;
};

struct ViewsParams {
    const ViewDev* views;
    uint32_t n_views;
    const World* worlds;
    Scratch* scratch;
    uint32_t queue_len, tile_w, tile_h, refill_threshold;
};

cudaError_t launch_views(const ViewsParams& V, const arc_launch_config& cfg, int n_sm, cudaStream_t st);
cudaError_t launch_frame(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg, int n_sm,
                         cudaStream_t st);
cudaError_t launch_secondary(const FrameParams& P, const arc_camera_uniforms& cam, cudaStream_t st);
cudaError_t launch_rays(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                        uint32_t lod_bias, int ignore_water, arc_hit_record* hits, cudaStream_t st);
cudaError_t launch_shadow_di(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, const float* max_dist_m,
                             uint32_t n, float* vis, cudaStream_t st);
cudaError_t launch_shadow(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                          float* vis, cudaStream_t st);

}  // namespace arc
