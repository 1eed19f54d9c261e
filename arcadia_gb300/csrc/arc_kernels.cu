// arc_kernels.cu — traversal kernels of libarc_trace.so (sm_103a).
//
//   frame_plain_kernel       one thread per pixel: primary ray (primary_raymarch,
//                            shaders/primary_gbuffer.wgsl:93-312); the FUSED instance traces the GI
//                            secondary ray (shaders/lighting_restir_gi.wgsl:195-209) in the same thread,
//                            the primary-only one leaves it to gi_rows_kernel (the frame paths: 1.46x
//                            faster than fused, and without the GI code the primary instance needs 64
//                            instead of 80 registers).
//   frame_persistent_kernel  persistent warps pulling pixels from a global queue; a lane whose ray
//                            finishes is refilled with the next pixel between DDA iterations, a primary
//                            hit turns the lane into its GI ray, so uneven ray lengths do not idle lanes.
//   gi_rows_kernel           the frame's GI rays as their own pass after frame_plain_kernel (octant-
//                            sorted per block); also the GI rays from an existing G-buffer.
//   rays_kernel / shadow_kernel  trace_world_64tree / trace_shadow_vis over a ray batch.
//   sharc_*                  shaders/sharc_update.wgsl, sharc_resolve.wgsl, common/sharc_query.wgsl.
//
// Compiled with --fmad=false --prec-div=true --prec-sqrt=true (canonical arithmetic, arc_math.cuh).
#include <cuda_runtime.h>
#include <stdint.h>

#include <cooperative_groups.h>

#include "arc_kernels.h"
#include "arc_surface.cuh"
#include "arc_traverse.cuh"

namespace arc {

// ------------------------------------------------------------------------------------------------
// Outputs
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void store_hit(arc_hit_record* p, const HitInfo& h, bool hit) {
    uint32_t* q = reinterpret_cast<uint32_t*>(p);
    if (hit) {
        q[0] = h.vx;
        q[1] = h.vy;
        q[2] = h.vz;
        q[3] = face_id(h.normal) | (h.mat << 8) | ((ARC_HIT_FLAG_HIT | ((h.shift >> 1) << 1)) << 16);
    } else {
        q[0] = q[1] = q[2] = 0xFFFFFFFFu;
        q[3] = ARC_FACE_NONE;
    }
    q[4] = __float_as_uint(h.t_voxels * ARC_VOXEL_SIZE);
}

__device__ __forceinline__ void store_no_ray(arc_hit_record* p) {
    uint32_t* q = reinterpret_cast<uint32_t*>(p);
    q[0] = q[1] = q[2] = 0xFFFFFFFFu;
    q[3] = ARC_FACE_NONE;
    q[4] = 0u;
}

__device__ __forceinline__ uint32_t view_of(const FrameParams&) { return 0u; }
__device__ __forceinline__ uint32_t view_of(const ViewDev& v) { return v.view_id; }

// Appends a hit that takes a surface branch to the launch's list; the lanes of a warp that append
// together claim their slots with one atomic.
template <class Out>
__device__ __forceinline__ void surface_append(const Out& P, size_t k, uint32_t x, uint32_t y, const HitInfo& h,
                                               float hit_dist) {
    namespace cg = cooperative_groups;
    cg::coalesced_group g = cg::coalesced_threads();
    uint32_t base = 0u;
    if (g.thread_rank() == 0) base = atomicAdd(P.surf_count, g.size());
    base = g.shfl(base, 0) + g.thread_rank();
    if (base >= P.surf_cap) return;
    uint4* e = reinterpret_cast<uint4*>(&P.surf[base]);
    e[0] = make_uint4((uint32_t)k, x | (y << 16), (h.mat & 0xFFu) | (face_id(h.normal) << 8) | (view_of(P) << 16),
                      h.voxel_hash);
    e[1] = make_uint4(__float_as_uint(hit_dist), __float_as_uint(h.hit_pos_m.x), __float_as_uint(h.hit_pos_m.y),
                      __float_as_uint(h.hit_pos_m.z));
}

// G-buffer words of one pixel (primary_gbuffer.wgsl:138-143 miss, 145-311 hit; no rigid bodies).
// With SURF (the launch has a surface list: the world may hold water or mirror voxels, or the camera
// is under water), a hit on water under an above-water camera stores the up normal
// (primary_gbuffer.wgsl:286) and hits that take the underwater / water / mirror branch are listed
// for surface_kernel, which rewrites their albedo. Without SURF no hit can take a branch and the
// kernels carry none of that code. Returns the packed depth and normal words the GI ray is
// generated from.
template <bool SURF, class Out>
__device__ __forceinline__ void primary_store(const Out& P, const float4* __restrict__ palette,
                                              const arc_camera_uniforms& cam, uint32_t x, uint32_t y, f3 dir, bool hit,
                                              const HitInfo& h, uint32_t* depth_word, uint32_t* normal_word) {
    const size_t k = (size_t)y * P.width + x;
    if (P.hits) store_hit(&P.hits[k], h, hit);
    if (!hit) {
        float ox, oy;
        oct_encode(dir, &ox, &oy);
        const uint32_t n0 = pack2x16snorm(ox, oy);
        reinterpret_cast<uint2*>(P.gbuf_depth_mat)[k] = make_uint2(__float_as_uint(1e5f), 0u);
        reinterpret_cast<uint2*>(P.gbuf_norm_motion)[k] = make_uint2(n0, pack2x16float(0.0f, 0.0f));
        P.gbuf_albedo_ao[k] = pack4x8unorm(0.0f, 0.0f, 0.0f, 1.0f);
        *depth_word = __float_as_uint(1e5f);
        *normal_word = n0;
        return;
    }
    const float hit_dist = h.t_voxels * ARC_VOXEL_SIZE;
    const float4 alb_r = __ldg(&palette[2u * h.mat]);
    const float4 em_m = __ldg(&palette[2u * h.mat + 1u]);
    const float vrw = 1.0f - smoothstepf(18.0f, 48.0f, hit_dist);
    const float vr = (__fdiv_rn((float)(h.voxel_hash & 0xFFu), 255.0f) * 2.0f - 1.0f) * vrw;
    const float k_var = 1.0f + vr * em_m.w;
    const float ar = clampf(alb_r.x * k_var, 0.01f, 1.0f);
    const float ag = clampf(alb_r.y * k_var, 0.01f, 1.0f);
    const float ab = clampf(alb_r.z * k_var, 0.01f, 1.0f);
    // analytic motion vector (primary_gbuffer.wgsl:298-305), column-major prev_view_proj
    const float pu = __fdiv_rn((float)x + 0.5f, (float)P.width);
    const float pv = __fdiv_rn((float)y + 0.5f, (float)P.height);
    const float* M = cam.prev_view_proj;
    const f3 hp = h.hit_pos_m;
    float clip[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) clip[r] = ((M[r] * hp.x + M[4 + r] * hp.y) + M[8 + r] * hp.z) + M[12 + r] * 1.0f;
    float mx = -2.0f, my = -2.0f;
    if (clip[3] > 0.001f) {
        const float ndx = __fdiv_rn(clip[0], clip[3]), ndy = __fdiv_rn(clip[1], clip[3]);
        mx = (ndx * 0.5f + 0.5f) - pu;
        my = (0.5f - ndy * 0.5f) - pv;
    }
    f3 nrm = h.normal;
    if constexpr (SURF) {
        if (h.mat == kMatWaterCrystal && (cam.point_light_count[1] & 0xFFFFu) == 0u) nrm = f3{0.0f, 1.0f, 0.0f};
        if (surface_special(cam, h.mat)) surface_append(P, k, x, y, h, hit_dist);
    }
    float ox, oy;
    oct_encode(nrm, &ox, &oy);
    const uint32_t n0 = pack2x16snorm(ox, oy);
    reinterpret_cast<uint2*>(P.gbuf_depth_mat)[k] = make_uint2(__float_as_uint(hit_dist), h.mat & 0xFFFFu);
    reinterpret_cast<uint2*>(P.gbuf_norm_motion)[k] = make_uint2(n0, pack2x16float(mx, my));
    P.gbuf_albedo_ao[k] = pack4x8unorm(ar, ag, ab, clampf(h.contact_ao, 0.0f, 1.0f));
    *depth_word = __float_as_uint(hit_dist);
    *normal_word = n0;
}

__device__ __forceinline__ void pixel_of(const FrameParams& P, uint32_t q, uint32_t* x, uint32_t* y) {
    const uint32_t tile = q >> 5, within = q & 31u;
    const uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    *x = tx * P.tile_w + within % P.tile_w;
    *y = P.row0 + ty * P.tile_h + within / P.tile_w;
}

// ------------------------------------------------------------------------------------------------
// Frame kernels
// ------------------------------------------------------------------------------------------------

// Block coordinates of block `id` of a 1D launch over an nbx x nby grid of pixel blocks: row-major
// (order 0), or Morton (Z) order inside super-tiles of 8 x 8 blocks that follow each other row-major
// (order 1), so the blocks resident on the GPU at a time cover a compact part of the screen. Returns
// false for the padding blocks of partial super-tiles.
__device__ __forceinline__ bool block_coords(uint32_t id, uint32_t nbx, uint32_t nby, uint32_t order, uint32_t* bx,
                                             uint32_t* by) {
    if (order == 0u) {
        *bx = id % nbx;
        *by = id / nbx;
        return *by < nby;
    }
    const uint32_t nsx = (nbx + 7u) >> 3, st = id >> 6, m = id & 63u;
    *bx = (st % nsx) * 8u + ((m & 1u) | ((m >> 1) & 2u) | ((m >> 2) & 4u));
    *by = (st / nsx) * 8u + (((m >> 1) & 1u) | ((m >> 2) & 2u) | ((m >> 3) & 4u));
    return *bx < nbx && *by < nby;
}

// Tile of a view's queue (32 pixels each): row-major over the view's tiles, or (order 1) Morton order
// within super-tiles of 8 x 8 tiles, so that a block's consecutive tiles form a square patch and the
// blocks resident together cover a compact screen area. Tiles past the view's edge map outside it.
__device__ __forceinline__ void view_tile(uint32_t tile, uint32_t tiles_x, uint32_t order, uint32_t* tx, uint32_t* ty) {
    block_coords(tile, tiles_x, 0xFFFFFFFFu, order, tx, ty);
}

__host__ __device__ __forceinline__ uint32_t blocks_for(uint32_t nbx, uint32_t nby, uint32_t order) {
    return order == 0u ? nbx * nby : ((nbx + 7u) >> 3) * ((nby + 7u) >> 3) * 64u;
}

template <int MINB, bool SURF, bool FUSED, int FEAT = 0>
__global__ void __launch_bounds__(256, MINB) frame_plain_kernel(const FrameParams P,
                                                                   const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t nbx = (P.width + blockDim.x - 1u) / blockDim.x;
    const uint32_t nby = (P.row_end - P.row0 + blockDim.y - 1u) / blockDim.y;
    uint32_t bx, by;
    if (!block_coords(blockIdx.x, nbx, nby, P.order, &bx, &by)) return;
    const uint32_t x = bx * blockDim.x + threadIdx.x;
    const uint32_t y = P.row0 + by * blockDim.y + threadIdx.y;
    if (x >= P.width || y >= P.row_end) return;
    const World& w = P.world;
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const f3 dir = camera_dir(cam, x, y, P.width, P.height);
    const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
    RayState s;
    HitInfo h;
    // One traversal call site for both rays: the primary ray, then (for a hit) the GI ray continues in
    // the same loop, so lanes in either phase run the same instructions together.
    bool active = ray_begin(s, cam, eye, dir, 0.0f, 250.0f, 0u, underwater);
    if constexpr ((FEAT & kFeatPrecomp) != 0) ray_precompute(s, cam);
    bool gi_phase = false;
    const size_t k = (size_t)y * P.width + x;
    f3 go{0.0f, 0.0f, 0.0f}, gd{0.0f, 0.0f, 1.0f};
    const float gmax = cam.ray_distances[2];
    StepResult r;
    for (;;) {
        r = active ? ray_next<FEAT>(s, w, cam, h) : kMiss;
        if (r == kContinue) continue;
        if (gi_phase) break;
        if (r != kHit) hit_init_miss(h, eye, dir, 250.0f);
        uint32_t dw, nw;
        primary_store<SURF>(P, w.palette, cam, x, y, dir, r == kHit, h, &dw, &nw);
        if constexpr (!FUSED) return;  // primary rays only (gi_rows_kernel traces the GI rays, if any)
        if (!P.do_gi) return;
        if (!gi_setup(w, cam, x, y, P.width, P.height, dw, nw, &go, &gd)) {
            if (P.gi_hits) store_no_ray(&P.gi_hits[k]);
            return;
        }
        gi_phase = true;
        active = ray_begin(s, cam, go, gd, 0.0f, gmax, 2u, true);
        if constexpr ((FEAT & kFeatPrecomp) != 0) ray_precompute(s, cam);
    }
    if (r != kHit) hit_init_miss(h, go, gd, gmax);
    if (P.gi_hits) store_hit(&P.gi_hits[k], h, r == kHit);
    // warp-aggregated count of GI rays
    const uint32_t m = __activemask();
    if (((threadIdx.x + threadIdx.y * blockDim.x) & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(&P.scratch->gi_rays, (unsigned long long)__popc(m));
}

// ---- primary rays from resident CTAs (ARC_FEAT_TOP_TABLE, ARC_FEAT_GRID_STRIDE) ---------------
// top_build_kernel (one CTA) writes the table of the top two tree levels from the current pools: entry c
// is chunk c's root, an internal root's child index rebased into the level-1 part that follows the
// roots (each root's child slice in order); *info = number of entries, 0 when they exceed kTopMaxNodes.
__global__ void __launch_bounds__(1024) top_build_kernel(const World w, uint32_t n_chunks, uint4* __restrict__ out,
                                                         uint32_t* __restrict__ info) {
    __shared__ uint32_t s_sum[1024];
    const uint32_t t = threadIdx.x, per = (n_chunks + 1023u) / 1024u;
    uint32_t cnt = 0u;
    for (uint32_t i = 0; i < per; ++i) {
        const uint32_t c = t * per + i;
        if (c >= n_chunks) break;
        const uint32_t r = w.roots[c];
        if (r == ARC_EMPTY_CHUNK || r >= w.n_nodes) continue;
        const uint4 nd = w.nodes[r];
        if (!(nd.z & ARC_IS_LEAF_FLAG)) cnt += __popc(nd.x) + __popc(nd.y);
    }
    s_sum[t] = cnt;
    __syncthreads();
    for (uint32_t o = 1; o < 1024u; o <<= 1) {
        const uint32_t add = t >= o ? s_sum[t - o] : 0u;
        __syncthreads();
        s_sum[t] += add;
        __syncthreads();
    }
    const uint32_t total = s_sum[1023];
    const bool fits = (uint64_t)n_chunks + total <= kTopMaxNodes;
    if (t == 0u) *info = fits ? n_chunks + total : 0u;
    if (!fits) return;
    uint32_t off = s_sum[t] - cnt;
    for (uint32_t i = 0; i < per; ++i) {
        const uint32_t c = t * per + i;
        if (c >= n_chunks) break;
        const uint32_t r = w.roots[c];
        uint4 nd = make_uint4(0u, 0u, 0u, 0u);
        if (r != ARC_EMPTY_CHUNK && r < w.n_nodes) {
            nd = w.nodes[r];
            if (!(nd.z & ARC_IS_LEAF_FLAG)) {
                const uint32_t k = __popc(nd.x) + __popc(nd.y), src = nd.z & ARC_PTR_INDEX_MASK;
                for (uint32_t j = 0; j < k; ++j) out[n_chunks + off + j] = load_node(w, src + j);
                nd.z = off;  // internal node: no flag bits
                off += k;
            }
        }
        out[c] = nd;
    }
}

// Primary rays (no surface list) from resident CTAs that take the pixel blocks of the launch in turn
// (block order as the plain kernel). With TOP each CTA first copies the top-level table into shared
// memory, and restarts from a chunk root read it there.
template <int MINB, bool TOP>
__global__ void __launch_bounds__(256, MINB) frame_grid_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    extern __shared__ uint4 s_top[];
    const World& w = P.world;
    TopView top{nullptr, nullptr};
    if constexpr (TOP) {
        const uint32_t n = *P.top_info;  // the same for every thread
        const uint32_t tid = threadIdx.x + threadIdx.y * blockDim.x, nthr = blockDim.x * blockDim.y;
        for (uint32_t i = tid; i < n; i += nthr) s_top[i] = P.top[i];
        __syncthreads();
        if (n) top = TopView{s_top, s_top + cam.world_grid_dims[0] * cam.world_grid_dims[1] * cam.world_grid_dims[2]};
    }
    const uint32_t nbx = (P.width + blockDim.x - 1u) / blockDim.x;
    const uint32_t nby = (P.row_end - P.row0 + blockDim.y - 1u) / blockDim.y;
    const uint32_t total = blocks_for(nbx, nby, P.order);
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
    for (uint32_t id = blockIdx.x; id < total; id += gridDim.x) {
        uint32_t bx, by;
        if (!block_coords(id, nbx, nby, P.order, &bx, &by)) continue;
        const uint32_t x = bx * blockDim.x + threadIdx.x, y = P.row0 + by * blockDim.y + threadIdx.y;
        if (x >= P.width || y >= P.row_end) continue;
        const f3 dir = camera_dir(cam, x, y, P.width, P.height);
        RayState s;
        HitInfo h;
        StepResult r = kMiss;
        if (ray_begin(s, cam, eye, dir, 0.0f, 250.0f, 0u, underwater)) {
            do {
                r = ray_advance<TOP ? kFeatTopTable : 0>(s, w, cam, h, top);
            } while (r == kContinue);
        }
        if (r != kHit) hit_init_miss(h, eye, dir, 250.0f);
        uint32_t dw, nw;
        primary_store<false>(P, w.palette, cam, x, y, dir, r == kHit, h, &dw, &nw);
    }
}

template <int MINB, bool TOP>
cudaError_t launch_grid_primary(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg, int n_sm,
                                cudaStream_t st) {
    const size_t smem = TOP ? sizeof(uint4) * kTopMaxNodes : 0u;
    if (TOP) {
        const uint32_t n_chunks = cam.world_grid_dims[0] * cam.world_grid_dims[1] * cam.world_grid_dims[2];
        top_build_kernel<<<1, 1024, 0, st>>>(P.world, n_chunks, P.top, P.top_info);
    }
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, frame_grid_kernel<MINB, TOP>, (int)cfg.block_threads, smem);
    if (e != cudaSuccess) return e;
    if (per_sm <= 0) per_sm = 1;
    const dim3 block(8u, cfg.block_threads / 8u);
    frame_grid_kernel<MINB, TOP><<<n_sm * per_sm, block, smem, st>>>(P, cam);
    return cudaGetLastError();
}

enum : uint32_t { kIdle = 0u, kPrimary = 1u, kGi = 2u };

template <int MINB, bool SURF>
__global__ void __launch_bounds__(256, MINB) frame_persistent_kernel(const FrameParams P,
                                                                     const __grid_constant__ arc_camera_uniforms cam) {
    const World& w = P.world;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
    const float gmax = cam.ray_distances[2];
    RayState s;
    HitInfo h;
    uint32_t phase = kIdle;
    uint32_t pxy = 0;  // pixel x | y << 16
    bool exhausted = false;
    uint32_t gi_count = 0;

    for (;;) {
        // Refill idle lanes from the queue (one atomic per warp).
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, phase == kIdle);
        if (!exhausted && (__popc(idle) >= (int)P.refill_threshold || idle == 0xFFFFFFFFu)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&P.scratch->queue_head, (uint32_t)__popc(idle));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + (uint32_t)__popc(idle) >= P.queue_len) exhausted = true;
            if (phase == kIdle) {
                const uint32_t q = base + __popc(idle & lt_mask);
                if (q < P.queue_len) {
                    uint32_t px, py;
                    pixel_of(P, q, &px, &py);
                    pxy = px | (py << 16);
                    if (px < P.width && py < P.row_end) {
                        const f3 dir = camera_dir(cam, px, py, P.width, P.height);
                        if (ray_begin(s, cam, eye, dir, 0.0f, 250.0f, 0u, underwater)) {
                            phase = kPrimary;
                        } else {
                            hit_init_miss(h, eye, dir, 250.0f);
                            uint32_t dw, nw;
                            primary_store<SURF>(P, w.palette, cam, px, py, dir, false, h, &dw, &nw);
                            if (P.do_gi && P.gi_hits) store_no_ray(&P.gi_hits[(size_t)py * P.width + px]);
                        }
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, phase != kIdle) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (phase == kIdle) continue;
        const StepResult r = ray_advance(s, w, cam, h);
        if (r == kContinue) continue;
        const uint32_t px = pxy & 0xFFFFu, py = pxy >> 16;
        if (phase == kPrimary) {
            const f3 dir = s.dir;
            if (r != kHit) hit_init_miss(h, eye, dir, 250.0f);
            uint32_t dw, nw;
            primary_store<SURF>(P, w.palette, cam, px, py, dir, r == kHit, h, &dw, &nw);
            phase = kIdle;
            if (P.do_gi) {
                f3 go, gd;
                if (gi_setup(w, cam, px, py, P.width, P.height, dw, nw, &go, &gd)) {
                    ++gi_count;
                    if (ray_begin(s, cam, go, gd, 0.0f, gmax, 2u, true)) {
                        phase = kGi;
                    } else {
                        hit_init_miss(h, go, gd, gmax);
                        if (P.gi_hits) store_hit(&P.gi_hits[(size_t)py * P.width + px], h, false);
                    }
                } else if (P.gi_hits) {
                    store_no_ray(&P.gi_hits[(size_t)py * P.width + px]);
                }
            }
        } else {
            if (r != kHit) hit_init_miss(h, mul3s(s.vo, ARC_VOXEL_SIZE), s.dir, gmax);
            if (P.gi_hits) store_hit(&P.gi_hits[(size_t)py * P.width + px], h, r == kHit);
            phase = kIdle;
        }
    }
    // warp-reduce the GI ray count
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gi_count += __shfl_down_sync(0xFFFFFFFFu, gi_count, o);
    if (lane == 0 && gi_count) atomicAdd(&P.scratch->gi_rays, (unsigned long long)gi_count);
}

// GI pass over the launch's rows from the G-buffer (lighting_restir_gi.wgsl:195-209). As a pass of its
// own after the primary kernel it runs 1.3x faster than the GI ray traced in the primary kernel's
// thread: there, a warp's lanes whose primary ray missed (the sky) idle through the whole GI phase of
// the others, while here a warp of sky pixels ends at once. A block sets up the GI rays of its 16 x 8
// pixels, sorts them by direction octant in shared memory (a counting sort; the rays without a GI ray
// drop out) and traces them from the sorted slots, so a warp's rays step in the same directions.
// Every ray is computed as before, only by another thread of the block.
//
// With REPACK (ARC_FEAT_GI_REPACK) the block also regroups its rays while they run: every
// P.refill_threshold DDA steps the rays still running are packed into the block's first threads, so
// the warps that keep tracing are full and the others idle. A GI ray's length varies about tenfold
// within a block (7 to 77 steps, 10th to 99th percentile, on the 1024^3 caves frame); without the
// repack a warp runs as long as its longest ray. A ray moves with t, t_limit, its voxel and its step
// count; vo, dir and 1/dir are rebuilt from its sorted slot as ray_begin forms them, and the chunk and
// ancestor caches restart empty. Those caches only save node loads (a descent from the chunk root
// meets the same nodes, and the step is taken at the same level), so every decision and result is
// unchanged. Measured on the 1080p caves frame it is slower than the plain pass at every K (1.45-1.54
// against 1.15 ms per frame): the two block barriers every K steps alone cost about 0.2 ms, more than
// the fuller warps save, so it stays a selectable variant.
template <int MINB, int FEAT = 0, bool REPACK = false>
__global__ void __launch_bounds__(128, MINB) gi_rows_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    __shared__ float s_ray[6][128];
    __shared__ uint32_t s_k[128];
    __shared__ uint32_t s_cnt[9], s_base[10];
    const uint32_t t = threadIdx.x;
    uint32_t bx, by;
    if (!block_coords(blockIdx.x, (P.width + 15u) / 16u, (P.row_end - P.row0 + 7u) / 8u, P.order, &bx, &by)) return;
    const uint32_t x = bx * 16u + (t & 15u);
    const uint32_t y = P.row0 + by * 8u + (t >> 4);
    if (t < 9u) s_cnt[t] = 0u;
    __syncthreads();
    uint32_t key = 8u;
    f3 go{0.0f, 0.0f, 0.0f}, gd{0.0f, 0.0f, 1.0f};
    size_t k = 0;
    if (x < P.width && y < P.row_end) {
        k = (size_t)y * P.width + x;
        if (gi_setup(P.world, cam, x, y, P.width, P.height, P.gbuf_depth_mat[2u * k], P.gbuf_norm_motion[2u * k], &go, &gd))
            key = ((gd.x < 0.0f ? 1u : 0u) | (gd.y < 0.0f ? 2u : 0u) | (gd.z < 0.0f ? 4u : 0u));
        else if (P.gi_hits)
            store_no_ray(&P.gi_hits[k]);
    }
    const uint32_t rank = atomicAdd(&s_cnt[key], 1u);
    __syncthreads();
    if (t == 0u) {
        uint32_t acc = 0u;
        for (int i = 0; i < 9; ++i) {
            s_base[i] = acc;
            acc += s_cnt[i];
        }
        s_base[9] = acc;
    }
    __syncthreads();
    if (key < 8u) {
        const uint32_t slot = s_base[key] + rank;
        s_ray[0][slot] = go.x;
        s_ray[1][slot] = go.y;
        s_ray[2][slot] = go.z;
        s_ray[3][slot] = gd.x;
        s_ray[4][slot] = gd.y;
        s_ray[5][slot] = gd.z;
        s_k[slot] = (uint32_t)k;
    }
    __syncthreads();
    const uint32_t n = s_base[8];
    if constexpr (REPACK) {
        static_assert((FEAT & ~kFeatPrecomp) == 0, "the repacked GI pass moves the descent-loop ray state only");
        __shared__ uint32_t s_st[7][128];  // t, t_limit, vx, vy, vz, step, slot of the running rays
        __shared__ uint32_t s_wc[4];
        const uint32_t lane = t & 31u, warp = t >> 5;
        const float gmax = cam.ray_distances[2];
        const uint32_t K = P.refill_threshold;
        if (t == 0u && n) atomicAdd(&P.scratch->gi_rays, (unsigned long long)n);
        uint32_t slot = t;
        bool live = false;
        RayState s;
        HitInfo h;
        if (t < n) {
            live = ray_begin(s, cam, f3{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, f3{s_ray[3][t], s_ray[4][t], s_ray[5][t]},
                             0.0f, gmax, 2u, true);
            if constexpr ((FEAT & kFeatPrecomp) != 0) {
                if (live) ray_precompute(s, cam);
            }
            if (!live) {
                hit_init_miss(h, f3{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, f3{s_ray[3][t], s_ray[4][t], s_ray[5][t]}, gmax);
                if (P.gi_hits) store_hit(&P.gi_hits[s_k[t]], h, false);
            }
        }
        for (;;) {
            if (live) {
                StepResult g = kContinue;
                for (uint32_t i = 0; i < K && g == kContinue; ++i) g = ray_next<FEAT>(s, P.world, cam, h);
                if (g != kContinue) {
                    live = false;
                    if (g != kHit)
                        hit_init_miss(h, f3{s_ray[0][slot], s_ray[1][slot], s_ray[2][slot]},
                                      f3{s_ray[3][slot], s_ray[4][slot], s_ray[5][slot]}, gmax);
                    if (P.gi_hits) store_hit(&P.gi_hits[s_k[slot]], h, g == kHit);
                }
            }
            const uint32_t ball = __ballot_sync(0xFFFFFFFFu, live);
            if (lane == 0u) s_wc[warp] = (uint32_t)__popc(ball);
            __syncthreads();
            const uint32_t c0 = s_wc[0], c1 = s_wc[1], c2 = s_wc[2], c3 = s_wc[3];
            const uint32_t total = c0 + c1 + c2 + c3;
            if (total == 0u) break;  // the same value in every thread of the block
            if (live) {
                const uint32_t r = (warp > 0u ? c0 : 0u) + (warp > 1u ? c1 : 0u) + (warp > 2u ? c2 : 0u) +
                                   (uint32_t)__popc(ball & ((1u << lane) - 1u));
                s_st[0][r] = __float_as_uint(s.t);
                s_st[1][r] = __float_as_uint(s.t_limit);
                s_st[2][r] = s.vx;
                s_st[3][r] = s.vy;
                s_st[4][r] = s.vz;
                s_st[5][r] = s.step;
                s_st[6][r] = slot;
            }
            __syncthreads();
            live = t < total;
            if (live) {
                slot = s_st[6][t];
                const f3 o{s_ray[0][slot], s_ray[1][slot], s_ray[2][slot]}, d{s_ray[3][slot], s_ray[4][slot], s_ray[5][slot]};
                s.vo = mul3s(o, ARC_VOXELS_PER_METER);
                s.dir = d;
                s.inv = f3{__fdiv_rn(1.0f, safe_component(d.x)), __fdiv_rn(1.0f, safe_component(d.y)),
                           __fdiv_rn(1.0f, safe_component(d.z))};
                s.t = __uint_as_float(s_st[0][t]);
                s.t_limit = __uint_as_float(s_st[1][t]);
                s.vx = s_st[2][t];
                s.vy = s_st[3][t];
                s.vz = s_st[4][t];
                s.step = s_st[5][t];
                s.diff = 0xFFFFFFFFu;  // next step: chunk root from the pool, descent from the root
                s.mtf_c0 = s.mtf_c1 = 0xFFFFFFFFu;
                s.mtf_root0 = s.mtf_root1 = ARC_EMPTY_CHUNK;
                s.cached_shift = 6u;
                s.mode = 2u | 4u;  // lod_bias 2, water ignored (as ray_begin above)
                s.have_node = 0u;
                if constexpr ((FEAT & kFeatPrecomp) != 0) ray_precompute(s, cam);
            }
            __syncthreads();  // s_st and s_wc are written again in the next round
        }
        return;
    }
    if (t >= n) return;
    const f3 o{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, d{s_ray[3][t], s_ray[4][t], s_ray[5][t]};
    const uint32_t kk = s_k[t];
    const float gmax = cam.ray_distances[2];
    RayState s;
    HitInfo h;
    StepResult g = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, gmax, 2u, true)) {
        if constexpr ((FEAT & kFeatPrecomp) != 0) ray_precompute(s, cam);
        do {
            g = ray_next<FEAT>(s, P.world, cam, h);
        } while (g == kContinue);
    }
    if (g != kHit) hit_init_miss(h, o, d, gmax);
    if (P.gi_hits) store_hit(&P.gi_hits[kk], h, g == kHit);
    const uint32_t m = __activemask();
    if ((t & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(&P.scratch->gi_rays, (unsigned long long)__popc(m));
}

// ---- the frame's GI pass with a global sort of its rays (ARC_FEAT_GI_SORT) ----------------------
// 1. gi_sort_keys_kernel: per pixel of the launch's rows, the GI ray (gi_setup, as gi_rows_kernel) and
//    its key = octant << 12 | Morton code of the origin's cell (voxel >> cell_shift, 16 cells per axis);
//    a bin histogram (one atomic per distinct key of a warp).
// 2. gi_sort_scan_kernel: exclusive scan of the bins (one block).
// 3. gi_sort_scatter_kernel: each ray to the next slot of its bin.
// 4. gi_sort_trace_kernel: one thread per sorted slot traces the ray and writes the hit record of its
//    pixel. The rays and their results are gi_rows_kernel's; only the thread that traces each differs.
__device__ __forceinline__ uint32_t spread4(uint32_t v) {  // 4 bits -> bits 0, 3, 6, 9
    return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

__global__ void __launch_bounds__(128) gi_sort_keys_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t t = threadIdx.x;
    uint32_t bx, by;
    if (!block_coords(blockIdx.x, (P.width + 15u) / 16u, (P.row_end - P.row0 + 7u) / 8u, P.order, &bx, &by)) return;
    const uint32_t x = bx * 16u + (t & 15u), y = P.row0 + by * 8u + (t >> 4);
    if (x >= P.width || y >= P.row_end) return;
    const size_t k = (size_t)y * P.width + x;
    f3 go, gd;
    uint32_t key = 0xFFFFFFFFu;
    if (gi_setup(P.world, cam, x, y, P.width, P.height, P.gbuf_depth_mat[2u * k], P.gbuf_norm_motion[2u * k], &go, &gd)) {
        const uint32_t sh = P.gisort.cell_shift;
        const uint32_t cx = umin(f2u(go.x * ARC_VOXELS_PER_METER) >> sh, 15u);
        const uint32_t cy = umin(f2u(go.y * ARC_VOXELS_PER_METER) >> sh, 15u);
        const uint32_t cz = umin(f2u(go.z * ARC_VOXELS_PER_METER) >> sh, 15u);
        const uint32_t oct = (gd.x < 0.0f ? 1u : 0u) | (gd.y < 0.0f ? 2u : 0u) | (gd.z < 0.0f ? 4u : 0u);
        key = (oct << 12) | spread4(cx) | (spread4(cy) << 1) | (spread4(cz) << 2);
        P.gisort.ray_dir[k] = make_float4(gd.x, gd.y, gd.z, 0.0f);
        const uint32_t act = __activemask();
        const uint32_t peers = __match_any_sync(act, key);
        if ((int)lane_id() == __ffs(peers) - 1) atomicAdd(&P.gisort.bins[key], (uint32_t)__popc(peers));
    } else if (P.gi_hits) {
        store_no_ray(&P.gi_hits[k]);
    }
    P.gisort.ray_pix[k] = make_float4(go.x, go.y, go.z, __uint_as_float(key));
}

__global__ void __launch_bounds__(1024) gi_sort_scan_kernel(uint32_t* __restrict__ bins) {
    constexpr uint32_t kPer = kGiSortBins / 1024u;  // 32 bins per thread
    __shared__ uint32_t s_sum[1024];
    const uint32_t t = threadIdx.x;
    uint32_t v[kPer], sum = 0u;
#pragma unroll
    for (uint32_t i = 0; i < kPer; ++i) {
        v[i] = bins[t * kPer + i];
        sum += v[i];
    }
    s_sum[t] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < 1024u; o <<= 1) {  // inclusive scan of the per-thread sums
        const uint32_t add = t >= o ? s_sum[t - o] : 0u;
        __syncthreads();
        s_sum[t] += add;
        __syncthreads();
    }
    uint32_t run = s_sum[t] - sum;
#pragma unroll
    for (uint32_t i = 0; i < kPer; ++i) {
        bins[t * kPer + i] = run;
        run += v[i];
    }
    if (t == 1023u) bins[kGiSortBins] = s_sum[1023];
}

__global__ void __launch_bounds__(256) gi_sort_scatter_kernel(const FrameParams P) {
    const size_t k = (size_t)P.row0 * P.width + (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= (size_t)P.row_end * P.width) return;
    const float4 o = P.gisort.ray_pix[k];
    const uint32_t key = __float_as_uint(o.w);
    if (key == 0xFFFFFFFFu) return;
    const float4 d = P.gisort.ray_dir[k];
    const uint32_t act = __activemask();
    const uint32_t peers = __match_any_sync(act, key);
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0u;
    if ((int)lane_id() == leader) base = atomicAdd(&P.gisort.bins[key], (uint32_t)__popc(peers));
    base = __shfl_sync(act, base, leader);
    const uint32_t slot = base + __popc(peers & ((1u << lane_id()) - 1u));
    P.gisort.sorted[2u * slot] = make_float4(o.x, o.y, o.z, __uint_as_float((uint32_t)k));
    P.gisort.sorted[2u * slot + 1u] = d;
}

template <int MINB>
__global__ void __launch_bounds__(128, MINB) gi_sort_trace_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.gisort.bins[kGiSortBins]) return;
    const float4 a = P.gisort.sorted[2u * i], b = P.gisort.sorted[2u * i + 1u];
    const f3 o{a.x, a.y, a.z}, d{b.x, b.y, b.z};
    const uint32_t kk = __float_as_uint(a.w);
    const float gmax = cam.ray_distances[2];
    RayState s;
    HitInfo h;
    StepResult g = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, gmax, 2u, true)) {
        do {
            g = ray_advance(s, P.world, cam, h);
        } while (g == kContinue);
    }
    if (g != kHit) hit_init_miss(h, o, d, gmax);
    if (P.gi_hits) store_hit(&P.gi_hits[kk], h, g == kHit);
    const uint32_t m = __activemask();
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(m) - 1)) atomicAdd(&P.scratch->gi_rays, (unsigned long long)__popc(m));
}

template <int MINB>
cudaError_t launch_gi_sorted(const FrameParams& P, const arc_camera_uniforms& cam, cudaStream_t st) {
    cudaError_t e = cudaMemsetAsync(P.gisort.bins, 0, sizeof(uint32_t) * (kGiSortBins + 1u), st);
    if (e != cudaSuccess) return e;
    const uint32_t rows = P.row_end - P.row0;
    gi_sort_keys_kernel<<<blocks_for((P.width + 15u) / 16u, (rows + 7u) / 8u, P.order), 128, 0, st>>>(P, cam);
    gi_sort_scan_kernel<<<1, 1024, 0, st>>>(P.gisort.bins);
    const uint32_t npx = P.width * rows;
    gi_sort_scatter_kernel<<<(npx + 255u) / 256u, 256, 0, st>>>(P);
    gi_sort_trace_kernel<MINB><<<(npx + 127u) / 128u, 128, 0, st>>>(P, cam);
    return cudaGetLastError();
}

__global__ void rays_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const arc_ray* __restrict__ rays,
                            uint32_t n, float max_dist_m, uint32_t lod_bias, uint32_t ignore_water,
                            arc_hit_record* __restrict__ hits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* rp = reinterpret_cast<const float*>(&rays[i]);
    const f3 o{rp[0], rp[1], rp[2]}, d{rp[3], rp[4], rp[5]};
    RayState s;
    HitInfo h;
    StepResult r = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, max_dist_m, lod_bias, ignore_water != 0u)) {
        do {
            r = ray_advance(s, w, cam, h);
        } while (r == kContinue);
    }
    if (r != kHit) hit_init_miss(h, o, d, max_dist_m);
    store_hit(&hits[i], h, r == kHit);
}

__global__ void shadow_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const arc_ray* __restrict__ rays,
                              uint32_t n, float max_dist_m, float* __restrict__ vis) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* rp = reinterpret_cast<const float*>(&rays[i]);
    vis[i] = shadow_vis(w, cam, f3{rp[0], rp[1], rp[2]}, f3{rp[3], rp[4], rp[5]}, max_dist_m);
}

// trace_shadow_vis_di over a batch of rays towards emitters, each with its own target distance.
__global__ void shadow_di_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam,
                                 const arc_ray* __restrict__ rays, const float* __restrict__ max_dist_m, uint32_t n,
                                 float* __restrict__ vis) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* rp = reinterpret_cast<const float*>(&rays[i]);
    vis[i] = shadow_vis_di(w, cam, f3{rp[0], rp[1], rp[2]}, f3{rp[3], rp[4], rp[5]}, max_dist_m[i]);
}

// Frame with rigid bodies (the camera's point_light_count.y >> 16 > 0 and a body table uploaded):
// one thread per pixel of the launch's rows. The primary ray is the world trace followed by the
// bodies in front of its hit (primary_gbuffer.wgsl:121-136): a body hit replaces distance, point,
// normal, material, voxel hash and contact AO, puts its previous-frame point into the motion vector
// and sets the G-buffer flag. Surface branches are shaded inline with the bodies in every surface
// ray; the GI ray is the world trace followed by the bodies in front of its hit
// (lighting_restir_gi.wgsl:209-224). Hit records of body hits carry ARC_HIT_FLAG_RIGID, the body
// index and the body-local voxel.
__device__ __forceinline__ void mark_rigid(arc_hit_record* p, uint32_t body) {
    reinterpret_cast<uint32_t*>(p)[3] |= (ARC_HIT_FLAG_RIGID | (body << 8)) << 16;
}

__device__ __forceinline__ void take_rigid(HitInfo& h, const RigidHit& rb) {
    h.t_voxels = rb.t_voxels;
    h.hit_pos_m = rb.pos;
    h.normal = rb.normal;
    h.mat = rb.mat;
    h.voxel_hash = rb.hash;
    h.contact_ao = rb.ao;
    h.vx = rb.vx;
    h.vy = rb.vy;
    h.vz = rb.vz;
    h.shift = rb.shift;
}

__global__ void __launch_bounds__(128) frame_rigid_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t x = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t y = P.row0 + blockIdx.y * 8u + (threadIdx.x >> 4);
    if (x >= P.width || y >= P.row_end) return;
    const World& w = P.world;
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const f3 dir = camera_dir(cam, x, y, P.width, P.height);
    const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
    const size_t k = (size_t)y * P.width + x;
    HitInfo h;
    bool hit = trace_full(w, cam, eye, dir, 250.0f, 0u, underwater, h);
    f3 prev = h.hit_pos_m;
    const RigidHit rb = trace_rigid_bodies(w, cam, eye, dir, hit ? h.t_voxels * ARC_VOXEL_SIZE : 250.0f);
    if (rb.hit) {
        hit = true;
        take_rigid(h, rb);
        prev = rb.prev_pos;
    }
    if (P.hits) {
        store_hit(&P.hits[k], h, hit);
        if (rb.hit) mark_rigid(&P.hits[k], rb.body);
    }
    uint32_t dw, nw;
    if (!hit) {
        float ox, oy;
        oct_encode(dir, &ox, &oy);
        nw = pack2x16snorm(ox, oy);
        dw = __float_as_uint(1e5f);
        reinterpret_cast<uint2*>(P.gbuf_depth_mat)[k] = make_uint2(dw, 0u);
        reinterpret_cast<uint2*>(P.gbuf_norm_motion)[k] = make_uint2(nw, pack2x16float(0.0f, 0.0f));
        P.gbuf_albedo_ao[k] = pack4x8unorm(0.0f, 0.0f, 0.0f, 1.0f);
    } else {
        const float hit_dist = h.t_voxels * ARC_VOXEL_SIZE;
        f3 alb = varied_albedo(w.palette, h.mat, h.voxel_hash, 1.0f - smoothstepf(18.0f, 48.0f, hit_dist));
        const float pu = __fdiv_rn((float)x + 0.5f, (float)P.width), pv = __fdiv_rn((float)y + 0.5f, (float)P.height);
        const float* M = cam.prev_view_proj;
        float clip[4];
#pragma unroll
        for (int r = 0; r < 4; ++r) clip[r] = ((M[r] * prev.x + M[4 + r] * prev.y) + M[8 + r] * prev.z) + M[12 + r] * 1.0f;
        float mx = -2.0f, my = -2.0f;
        if (clip[3] > 0.001f) {
            const float ndx = __fdiv_rn(clip[0], clip[3]), ndy = __fdiv_rn(clip[1], clip[3]);
            mx = (ndx * 0.5f + 0.5f) - pu;
            my = (0.5f - ndy * 0.5f) - pv;
        }
        f3 nrm = h.normal;
        if (surface_special(cam, h.mat)) {
            alb = surface_shade<true>(w, cam, dir, h.mat, h.normal, h.voxel_hash, hit_dist, h.hit_pos_m);
            if (h.mat == kMatWaterCrystal && !underwater) nrm = f3{0.0f, 1.0f, 0.0f};
        }
        float ox, oy;
        oct_encode(nrm, &ox, &oy);
        nw = pack2x16snorm(ox, oy);
        dw = __float_as_uint(hit_dist);
        reinterpret_cast<uint2*>(P.gbuf_depth_mat)[k] = make_uint2(dw, (h.mat & 0xFFFFu) | (rb.hit ? 1u << 16 : 0u));
        reinterpret_cast<uint2*>(P.gbuf_norm_motion)[k] = make_uint2(nw, pack2x16float(mx, my));
        P.gbuf_albedo_ao[k] = pack4x8unorm(alb.x, alb.y, alb.z, clampf(h.contact_ao, 0.0f, 1.0f));
    }
    if (!P.do_gi) return;
    f3 go, gd;
    if (!gi_setup(w, cam, x, y, P.width, P.height, dw, nw, &go, &gd)) {
        if (P.gi_hits) store_no_ray(&P.gi_hits[k]);
        return;
    }
    const float gmax = cam.ray_distances[2];
    HitInfo g;
    bool gh = trace_full(w, cam, go, gd, gmax, 2u, true, g);
    const RigidHit rg = trace_rigid_bodies(w, cam, go, gd, gh ? g.t_voxels * ARC_VOXEL_SIZE : gmax);
    if (rg.hit) {
        gh = true;
        take_rigid(g, rg);
    }
    if (P.gi_hits) {
        store_hit(&P.gi_hits[k], g, gh);
        if (rg.hit) mark_rigid(&P.gi_hits[k], rg.body);
    }
    atomicAdd(&P.scratch->gi_rays, 1ull);
}

// Persistent kernel over many views (several worlds, mixed resolutions) in one launch. The queue is
// the concatenation of every view's 32-pixel tiles; a lane finds its view by binary search over the
// views' queue offsets and reads that view's camera block and world from global memory (L1-cached),
// so the per-ray work is exactly the single-view kernel's.
template <int MINB, bool SURF>
__global__ void __launch_bounds__(256, MINB) views_persistent_kernel(const ViewsParams V) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lt_mask = (1u << lane) - 1u;
    RayState s;
    HitInfo h;
    uint32_t phase = kIdle;
    uint32_t pxy = 0, v = 0;
    bool exhausted = false;
    uint32_t gi_count = 0;
    for (;;) {
        const uint32_t idle = __ballot_sync(0xFFFFFFFFu, phase == kIdle);
        if (!exhausted && (__popc(idle) >= (int)V.refill_threshold || idle == 0xFFFFFFFFu)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&V.scratch->queue_head, (uint32_t)__popc(idle));
            base = __shfl_sync(0xFFFFFFFFu, base, 0);
            if (base + (uint32_t)__popc(idle) >= V.queue_len) exhausted = true;
            if (phase == kIdle) {
                const uint32_t q = base + __popc(idle & lt_mask);
                if (q < V.queue_len) {
                    uint32_t lo = 0, hi = V.n_views;  // last view with queue_begin <= q
                    while (hi - lo > 1u) {
                        const uint32_t mid = (lo + hi) >> 1;
                        if (V.views[mid].queue_begin <= q) lo = mid; else hi = mid;
                    }
                    v = lo;
                    const ViewDev& vd = V.views[v];
                    const uint32_t local = q - vd.queue_begin, tile = local >> 5, within = local & 31u;
                    uint32_t tx, ty;
                    view_tile(tile, vd.tiles_x, V.order, &tx, &ty);
                    const uint32_t px = tx * V.tile_w + within % V.tile_w, py = ty * V.tile_h + within / V.tile_w;
                    pxy = px | (py << 16);
                    if (px < vd.width && py < vd.height) {
                        const arc_camera_uniforms& cam = vd.cam;
                        const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
                        const f3 dir = camera_dir(cam, px, py, vd.width, vd.height);
                        const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
                        if (ray_begin(s, cam, eye, dir, 0.0f, 250.0f, 0u, underwater)) {
                            phase = kPrimary;
                        } else {
                            hit_init_miss(h, eye, dir, 250.0f);
                            uint32_t dw, nw;
                            primary_store<SURF>(vd, V.worlds[vd.slot].palette, cam, px, py, dir, false, h, &dw, &nw);
                            if (vd.gi_hits) store_no_ray(&vd.gi_hits[(size_t)py * vd.width + px]);
                        }
                    }
                }
            }
        }
        if (__ballot_sync(0xFFFFFFFFu, phase != kIdle) == 0u) {
            if (exhausted) break;
            continue;
        }
        if (phase == kIdle) continue;
        const ViewDev& vd = V.views[v];
        const arc_camera_uniforms& cam = vd.cam;
        const World& w = V.worlds[vd.slot];
        const StepResult r = ray_advance(s, w, cam, h);
        if (r == kContinue) continue;
        const uint32_t px = pxy & 0xFFFFu, py = pxy >> 16;
        const size_t k = (size_t)py * vd.width + px;
        if (phase == kPrimary) {
            const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
            const f3 dir = s.dir;
            if (r != kHit) hit_init_miss(h, eye, dir, 250.0f);
            uint32_t dw, nw;
            primary_store<SURF>(vd, w.palette, cam, px, py, dir, r == kHit, h, &dw, &nw);
            phase = kIdle;
            f3 go, gd;
            if (gi_setup(w, cam, px, py, vd.width, vd.height, dw, nw, &go, &gd)) {
                ++gi_count;
                const float gmax = cam.ray_distances[2];
                if (ray_begin(s, cam, go, gd, 0.0f, gmax, 2u, true)) {
                    phase = kGi;
                } else {
                    hit_init_miss(h, go, gd, gmax);
                    if (vd.gi_hits) store_hit(&vd.gi_hits[k], h, false);
                }
            } else if (vd.gi_hits) {
                store_no_ray(&vd.gi_hits[k]);
            }
        } else {
            if (r != kHit) hit_init_miss(h, mul3s(s.vo, ARC_VOXEL_SIZE), s.dir, cam.ray_distances[2]);
            if (vd.gi_hits) store_hit(&vd.gi_hits[k], h, r == kHit);
            phase = kIdle;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gi_count += __shfl_down_sync(0xFFFFFFFFu, gi_count, o);
    if (lane == 0 && gi_count) atomicAdd(&V.scratch->gi_rays, (unsigned long long)gi_count);
}

// One thread per queue slot over many views: the slot's view by binary search, its pixel by the same
// 32-pixel tile mapping as the persistent kernel (a warp traces one tile), then the single-view plain
// kernel's work: the primary ray and, with FUSED (views_gi_kernel does not trace the GI rays), the
// pixel's GI ray through the same traversal call site.
template <int MINB, bool SURF, bool FUSED>
__global__ void __launch_bounds__(256, MINB) views_plain_kernel(const ViewsParams V) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    bool gi_ray = false;
    if (q < V.queue_len) {
        uint32_t lo = 0, hi = V.n_views;  // last view with queue_begin <= q
        while (hi - lo > 1u) {
            const uint32_t mid = (lo + hi) >> 1;
            if (V.views[mid].queue_begin <= q) lo = mid; else hi = mid;
        }
        const ViewDev& vd = V.views[lo];
        const uint32_t local = q - vd.queue_begin, tile = local >> 5, within = local & 31u;
        uint32_t tx, ty;
        view_tile(tile, vd.tiles_x, V.order, &tx, &ty);
        const uint32_t px = tx * V.tile_w + within % V.tile_w, py = ty * V.tile_h + within / V.tile_w;
        if (px < vd.width && py < vd.height) {
            const arc_camera_uniforms& cam = vd.cam;
            const World& w = V.worlds[vd.slot];
            const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
            const f3 dir = camera_dir(cam, px, py, vd.width, vd.height);
            const bool underwater = (cam.point_light_count[1] & 0xFFFFu) != 0u;
            const size_t k = (size_t)py * vd.width + px;
            RayState s;
            HitInfo h;
            bool active = ray_begin(s, cam, eye, dir, 0.0f, 250.0f, 0u, underwater);
            bool gi_phase = false, done = false;
            f3 go{0.0f, 0.0f, 0.0f}, gd{0.0f, 0.0f, 1.0f};
            const float gmax = cam.ray_distances[2];
            StepResult r = kMiss;
            while (!done) {
                r = active ? ray_advance(s, w, cam, h) : kMiss;
                if (r == kContinue) continue;
                if (gi_phase) {
                    if (r != kHit) hit_init_miss(h, go, gd, gmax);
                    if (vd.gi_hits) store_hit(&vd.gi_hits[k], h, r == kHit);
                    done = true;
                    continue;
                }
                if (r != kHit) hit_init_miss(h, eye, dir, 250.0f);
                uint32_t dw, nw;
                primary_store<SURF>(vd, w.palette, cam, px, py, dir, r == kHit, h, &dw, &nw);
                if constexpr (!FUSED) {  // views_gi_kernel traces the GI rays
                    done = true;
                    continue;
                }
                if (!gi_setup(w, cam, px, py, vd.width, vd.height, dw, nw, &go, &gd)) {
                    if (vd.gi_hits) store_no_ray(&vd.gi_hits[k]);
                    done = true;
                    continue;
                }
                gi_ray = true;
                gi_phase = true;
                active = ray_begin(s, cam, go, gd, 0.0f, gmax, 2u, true);
            }
        }
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, gi_ray);
    if ((threadIdx.x & 31u) == 0u && m) atomicAdd(&V.scratch->gi_rays, (unsigned long long)__popc(m));
}

// GI rays of a batch as their own pass after views_plain_kernel (as gi_rows_kernel for a frame). A
// block sets up the GI rays of its queue slots (up to 256; a block may span two views), sorts them by
// direction octant in shared memory (a counting sort; slots without a GI ray, such as sky pixels, drop
// out) and traces them from the sorted slots, so warps are full and step in similar directions. Every
// ray is computed as before, only by another thread of the block.
template <int MINB>
__global__ void __launch_bounds__(256, MINB) views_gi_kernel(const ViewsParams V) {
    __shared__ float s_ray[6][256];
    __shared__ uint32_t s_k[256], s_view[256];
    __shared__ uint32_t s_cnt[9], s_base[10];
    const uint32_t t = threadIdx.x;
    if (t < 9u) s_cnt[t] = 0u;
    __syncthreads();
    const uint32_t q = blockIdx.x * blockDim.x + t;
    uint32_t key = 8u, view = 0u;
    f3 go{0.0f, 0.0f, 0.0f}, gd{0.0f, 0.0f, 1.0f};
    size_t k = 0;
    if (q < V.queue_len) {
        uint32_t lo = 0, hi = V.n_views;  // last view with queue_begin <= q
        while (hi - lo > 1u) {
            const uint32_t mid = (lo + hi) >> 1;
            if (V.views[mid].queue_begin <= q) lo = mid; else hi = mid;
        }
        const ViewDev& vd = V.views[lo];
        const uint32_t local = q - vd.queue_begin, tile = local >> 5, within = local & 31u;
        uint32_t tx, ty;
        view_tile(tile, vd.tiles_x, V.order, &tx, &ty);
        const uint32_t px = tx * V.tile_w + within % V.tile_w, py = ty * V.tile_h + within / V.tile_w;
        if (px < vd.width && py < vd.height) {
            k = (size_t)py * vd.width + px;
            view = lo;
            if (gi_setup(V.worlds[vd.slot], vd.cam, px, py, vd.width, vd.height, vd.gbuf_depth_mat[2u * k],
                         vd.gbuf_norm_motion[2u * k], &go, &gd))
                key = (gd.x < 0.0f ? 1u : 0u) | (gd.y < 0.0f ? 2u : 0u) | (gd.z < 0.0f ? 4u : 0u);
            else if (vd.gi_hits)
                store_no_ray(&vd.gi_hits[k]);
        }
    }
    const uint32_t rank = atomicAdd(&s_cnt[key], 1u);
    __syncthreads();
    if (t == 0u) {
        uint32_t acc = 0u;
        for (int i = 0; i < 9; ++i) {
            s_base[i] = acc;
            acc += s_cnt[i];
        }
        s_base[9] = acc;
        if (s_base[8]) atomicAdd(&V.scratch->gi_rays, (unsigned long long)s_base[8]);
    }
    __syncthreads();
    if (key < 8u) {
        const uint32_t slot = s_base[key] + rank;
        s_ray[0][slot] = go.x;
        s_ray[1][slot] = go.y;
        s_ray[2][slot] = go.z;
        s_ray[3][slot] = gd.x;
        s_ray[4][slot] = gd.y;
        s_ray[5][slot] = gd.z;
        s_k[slot] = (uint32_t)k;
        s_view[slot] = view;
    }
    __syncthreads();
    if (t >= s_base[8]) return;
    const f3 o{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, d{s_ray[3][t], s_ray[4][t], s_ray[5][t]};
    const ViewDev& vd = V.views[s_view[t]];
    const arc_camera_uniforms& cam = vd.cam;
    const World& w = V.worlds[vd.slot];
    const float gmax = cam.ray_distances[2];
    RayState s;
    HitInfo h;
    StepResult g = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, gmax, 2u, true)) {
        do {
            g = ray_advance(s, w, cam, h);
        } while (g == kContinue);
    }
    if (g != kHit) hit_init_miss(h, o, d, gmax);
    if (vd.gi_hits) store_hit(&vd.gi_hits[s_k[t]], h, g == kHit);
}

// ------------------------------------------------------------------------------------------------
// Host launchers (called by the C ABI on the context's stream)
// ------------------------------------------------------------------------------------------------

template <int MINB>
cudaError_t launch_frame_t(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg, int n_sm,
                           cudaStream_t st, const FrameHooks* hooks) {
    auto mid = [&]() -> cudaError_t {  // FrameHooks: after the primary rays, before the GI pass
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess || !hooks) return e;
        if (hooks->surface && (e = launch_surface(P, cam, n_sm, st)) != cudaSuccess) return e;
        return hooks->primary_done ? cudaEventRecord(hooks->primary_done, st) : cudaSuccess;
    };
    if (P.world.n_bodies && ((cam.point_light_count[1] >> 16) & 0xFFFFu)) {
        dim3 grid((P.width + 15u) / 16u, (P.row_end - P.row0 + 7u) / 8u);
        frame_rigid_kernel<<<grid, 128, 0, st>>>(P, cam);
        return mid();
    }
    if (cfg.variant == 0u) {
        const uint32_t bw = 8u, bh = cfg.block_threads / 8u;
        dim3 block(bw, bh);
        const dim3 grid(blocks_for((P.width + bw - 1u) / bw, (P.row_end - P.row0 + bh - 1u) / bh, P.order));
        const bool fused = P.do_gi && P.gi_mode == kGiFused;
        // the traversal variants are built for the primary-only instance and the GI pass (no surface list)
        // the instantiated traversal variants; any other combination of these bits runs the standard kernels
        const int feat0 = (int)(cfg.features & (uint32_t)(kFeatWarpFetch | kFeatNodeVisit | kFeatPrecomp));
        const int feat = (feat0 == kFeatWarpFetch || feat0 == kFeatNodeVisit || feat0 == kFeatPrecomp ||
                          feat0 == (kFeatWarpFetch | kFeatNodeVisit)) ? feat0 : 0;
        const bool variant_kernels = feat != 0 && !P.surf && !fused && (MINB == 2 || MINB == 3);
        const bool grid_primary = (cfg.features & (ARC_FEAT_TOP_TABLE | ARC_FEAT_GRID_STRIDE)) && !P.surf && !fused &&
                                  P.top && (MINB == 2 || MINB == 3);
        if (grid_primary) {
            cudaError_t e = (cfg.features & ARC_FEAT_TOP_TABLE) ? launch_grid_primary<MINB, true>(P, cam, cfg, n_sm, st)
                                                               : launch_grid_primary<MINB, false>(P, cam, cfg, n_sm, st);
            if (e != cudaSuccess) return e;
        } else if (P.surf) {
            if (fused) frame_plain_kernel<MINB, true, true><<<grid, block, 0, st>>>(P, cam);
            else frame_plain_kernel<MINB, true, false><<<grid, block, 0, st>>>(P, cam);
        } else if (variant_kernels) {
            if (feat == kFeatWarpFetch) frame_plain_kernel<MINB, false, false, kFeatWarpFetch><<<grid, block, 0, st>>>(P, cam);
            else if (feat == kFeatNodeVisit) frame_plain_kernel<MINB, false, false, kFeatNodeVisit><<<grid, block, 0, st>>>(P, cam);
            else if (feat == kFeatPrecomp) frame_plain_kernel<MINB, false, false, kFeatPrecomp><<<grid, block, 0, st>>>(P, cam);
            else frame_plain_kernel<MINB, false, false, kFeatWarpFetch | kFeatNodeVisit><<<grid, block, 0, st>>>(P, cam);
        } else {
            if (fused) frame_plain_kernel<MINB, false, true><<<grid, block, 0, st>>>(P, cam);
            else frame_plain_kernel<MINB, false, false><<<grid, block, 0, st>>>(P, cam);
        }
        cudaError_t e = mid();
        if (e != cudaSuccess || !P.do_gi) return e;
        if (P.gi_mode == kGiRows && P.gisort.bins) return launch_gi_sorted<MINB>(P, cam, st);
        if (P.gi_mode == kGiRows) {
            const dim3 g2(blocks_for((P.width + 15u) / 16u, (P.row_end - P.row0 + 7u) / 8u, P.order));
            if ((cfg.features & ARC_FEAT_GI_REPACK) && (feat == 0 || feat == kFeatPrecomp)) {
                if (feat == kFeatPrecomp && (MINB == 2 || MINB == 3))
                    gi_rows_kernel<MINB, kFeatPrecomp, true><<<g2, 128, 0, st>>>(P, cam);
                else
                    gi_rows_kernel<MINB, 0, true><<<g2, 128, 0, st>>>(P, cam);
            } else if (variant_kernels || (feat != 0 && P.surf && (MINB == 2 || MINB == 3))) {
                if (feat == kFeatWarpFetch) gi_rows_kernel<MINB, kFeatWarpFetch><<<g2, 128, 0, st>>>(P, cam);
                else if (feat == kFeatNodeVisit) gi_rows_kernel<MINB, kFeatNodeVisit><<<g2, 128, 0, st>>>(P, cam);
                else if (feat == kFeatPrecomp) gi_rows_kernel<MINB, kFeatPrecomp><<<g2, 128, 0, st>>>(P, cam);
                else gi_rows_kernel<MINB, kFeatWarpFetch | kFeatNodeVisit><<<g2, 128, 0, st>>>(P, cam);
            } else {
                gi_rows_kernel<MINB><<<g2, 128, 0, st>>>(P, cam);
            }
        }
        return cudaGetLastError();
    }
    int per_sm = (int)cfg.blocks_per_sm;
    if (per_sm <= 0) {
        cudaError_t e = P.surf ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, frame_persistent_kernel<MINB, true>,
                                                                               (int)cfg.block_threads, 0)
                               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, frame_persistent_kernel<MINB, false>,
                                                                               (int)cfg.block_threads, 0);
        if (e != cudaSuccess) return e;
        if (per_sm <= 0) per_sm = 1;
    }
    if (P.surf) frame_persistent_kernel<MINB, true><<<n_sm * per_sm, cfg.block_threads, 0, st>>>(P, cam);
    else frame_persistent_kernel<MINB, false><<<n_sm * per_sm, cfg.block_threads, 0, st>>>(P, cam);
    return mid();
}

cudaError_t launch_frame(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg, int n_sm,
                         cudaStream_t st, const FrameHooks* hooks) {
    switch (cfg.reg_blocks) {
        case 2: return launch_frame_t<2>(P, cam, cfg, n_sm, st, hooks);
        case 3: return launch_frame_t<3>(P, cam, cfg, n_sm, st, hooks);
        case 4: return launch_frame_t<4>(P, cam, cfg, n_sm, st, hooks);
        default: return launch_frame_t<1>(P, cam, cfg, n_sm, st, hooks);
    }
}

template <int MINB>
cudaError_t launch_views_t(const ViewsParams& V, const arc_launch_config& cfg, int n_sm, cudaStream_t st) {
    if (cfg.variant == 0u) {
        const uint32_t blocks = (V.queue_len + cfg.block_threads - 1u) / cfg.block_threads;
        if (V.gi_split) {
            if (V.surf) views_plain_kernel<MINB, true, false><<<blocks, cfg.block_threads, 0, st>>>(V);
            else views_plain_kernel<MINB, false, false><<<blocks, cfg.block_threads, 0, st>>>(V);
            views_gi_kernel<MINB><<<blocks, cfg.block_threads, 0, st>>>(V);
        } else {
            if (V.surf) views_plain_kernel<MINB, true, true><<<blocks, cfg.block_threads, 0, st>>>(V);
            else views_plain_kernel<MINB, false, true><<<blocks, cfg.block_threads, 0, st>>>(V);
        }
        return cudaGetLastError();
    }
    int per_sm = (int)cfg.blocks_per_sm;
    if (per_sm <= 0) {
        cudaError_t e = V.surf ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, views_persistent_kernel<MINB, true>,
                                                                               (int)cfg.block_threads, 0)
                               : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, views_persistent_kernel<MINB, false>,
                                                                               (int)cfg.block_threads, 0);
        if (e != cudaSuccess) return e;
        if (per_sm <= 0) per_sm = 1;
    }
    if (V.surf) views_persistent_kernel<MINB, true><<<n_sm * per_sm, cfg.block_threads, 0, st>>>(V);
    else views_persistent_kernel<MINB, false><<<n_sm * per_sm, cfg.block_threads, 0, st>>>(V);
    return cudaGetLastError();
}

cudaError_t launch_views(const ViewsParams& V, const arc_launch_config& cfg, int n_sm, cudaStream_t st) {
    switch (cfg.reg_blocks) {
        case 2: return launch_views_t<2>(V, cfg, n_sm, st);
        case 3: return launch_views_t<3>(V, cfg, n_sm, st);
        case 4: return launch_views_t<4>(V, cfg, n_sm, st);
        default: return launch_views_t<1>(V, cfg, n_sm, st);
    }
}

// ------------------------------------------------------------------------------------------------
// Surface branches (primary_gbuffer.wgsl:163-295) over the listed hits
// ------------------------------------------------------------------------------------------------

__device__ __forceinline__ void surface_store(uint32_t* albedo_ao, uint32_t k, f3 a) {
    // the AO byte stays; the albedo bytes are replaced
    const uint32_t old = albedo_ao[k];
    albedo_ao[k] = (old & 0xFF000000u) | (pack4x8unorm(a.x, a.y, a.z, 0.0f) & 0x00FFFFFFu);
}

__global__ void __launch_bounds__(128) surface_kernel(const FrameParams P, const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t n = umin(*P.surf_count, P.surf_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        SurfaceEntry e;
        const uint4 a = reinterpret_cast<const uint4*>(&P.surf[i])[0];
        const uint4 b = reinterpret_cast<const uint4*>(&P.surf[i])[1];
        e.k = a.x;
        e.xy = a.y;
        e.mat_face_view = a.z;
        e.hash = a.w;
        e.hit_dist = __uint_as_float(b.x);
        e.hp[0] = __uint_as_float(b.y);
        e.hp[1] = __uint_as_float(b.z);
        e.hp[2] = __uint_as_float(b.w);
        const f3 dir = camera_dir(cam, e.xy & 0xFFFFu, e.xy >> 16, P.width, P.height);
        surface_store(P.gbuf_albedo_ao, e.k,
                      surface_shade<false>(P.world, cam, dir, e.mat_face_view & 0xFFu, face_normal((e.mat_face_view >> 8) & 0xFFu),
                                           e.hash, e.hit_dist, f3{e.hp[0], e.hp[1], e.hp[2]}));
    }
}

__global__ void __launch_bounds__(128) surface_views_kernel(const ViewsParams V, const SurfaceEntry* __restrict__ surf,
                                                            const uint32_t* __restrict__ count, uint32_t cap) {
    const uint32_t n = umin(*count, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        SurfaceEntry e;
        const uint4 a = reinterpret_cast<const uint4*>(&surf[i])[0];
        const uint4 b = reinterpret_cast<const uint4*>(&surf[i])[1];
        e.k = a.x;
        e.xy = a.y;
        e.mat_face_view = a.z;
        e.hash = a.w;
        e.hit_dist = __uint_as_float(b.x);
        e.hp[0] = __uint_as_float(b.y);
        e.hp[1] = __uint_as_float(b.z);
        e.hp[2] = __uint_as_float(b.w);
        const uint32_t v = e.mat_face_view >> 16;
        if (v >= V.n_views) continue;
        const ViewDev& vd = V.views[v];
        const f3 dir = camera_dir(vd.cam, e.xy & 0xFFFFu, e.xy >> 16, vd.width, vd.height);
        surface_store(vd.gbuf_albedo_ao, e.k,
                      surface_shade<false>(V.worlds[vd.slot], vd.cam, dir, e.mat_face_view & 0xFFu,
                                           face_normal((e.mat_face_view >> 8) & 0xFFu), e.hash, e.hit_dist,
                                           f3{e.hp[0], e.hp[1], e.hp[2]}));
    }
}

static uint32_t surface_blocks(uint32_t cap, int n_sm) {
    const uint32_t need = (cap + 127u) / 128u, most = (uint32_t)n_sm * 8u;
    return need < 1u ? 1u : (need > most ? most : need);
}

cudaError_t launch_surface(const FrameParams& P, const arc_camera_uniforms& cam, int n_sm, cudaStream_t st) {
    if (!P.surf || !P.surf_count) return cudaSuccess;
    surface_kernel<<<surface_blocks(P.surf_cap, n_sm), 128, 0, st>>>(P, cam);
    return cudaGetLastError();
}

cudaError_t launch_surface_views(const ViewsParams& V, const SurfaceEntry* surf, const uint32_t* count, uint32_t cap,
                                 int n_sm, cudaStream_t st) {
    if (!surf || !count) return cudaSuccess;
    surface_views_kernel<<<surface_blocks(cap, n_sm), 128, 0, st>>>(V, surf, count, cap);
    return cudaGetLastError();
}

cudaError_t launch_secondary(const FrameParams& P, const arc_camera_uniforms& cam, const arc_launch_config& cfg,
                             cudaStream_t st) {
    // the frame's GI pass over the G-buffer's rows (compacted, octant-sorted blocks), at the register
    // budget of the launch configuration as in launch_frame
    const dim3 grid(blocks_for((P.width + 15u) / 16u, (P.row_end - P.row0 + 7u) / 8u, P.order));
    const bool repack = (cfg.features & ARC_FEAT_GI_REPACK) != 0u;
    switch (cfg.reg_blocks) {
        case 2:
            if (repack) gi_rows_kernel<2, 0, true><<<grid, 128, 0, st>>>(P, cam);
            else gi_rows_kernel<2><<<grid, 128, 0, st>>>(P, cam);
            break;
        case 3:
            if (repack) gi_rows_kernel<3, 0, true><<<grid, 128, 0, st>>>(P, cam);
            else gi_rows_kernel<3><<<grid, 128, 0, st>>>(P, cam);
            break;
        case 4:
            if (repack) gi_rows_kernel<4, 0, true><<<grid, 128, 0, st>>>(P, cam);
            else gi_rows_kernel<4><<<grid, 128, 0, st>>>(P, cam);
            break;
        default:
            if (repack) gi_rows_kernel<1, 0, true><<<grid, 128, 0, st>>>(P, cam);
            else gi_rows_kernel<1><<<grid, 128, 0, st>>>(P, cam);
            break;
    }
    return cudaGetLastError();
}

cudaError_t launch_rays(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                        uint32_t lod_bias, int ignore_water, arc_hit_record* hits, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    rays_kernel<<<(n + 127u) / 128u, 128, 0, st>>>(w, cam, rays, n, max_dist_m, lod_bias, ignore_water ? 1u : 0u, hits);
    return cudaGetLastError();
}

// trace_rigid_bodies over a ray batch: hit records (body hits flagged) and optional per-ray detail
// (world hit point, previous-frame hit point, world normal).
__global__ void rigid_rays_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const arc_ray* __restrict__ rays,
                                  uint32_t n, float max_dist_m, arc_hit_record* __restrict__ hits, float* __restrict__ detail) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* rp = reinterpret_cast<const float*>(&rays[i]);
    const f3 o{rp[0], rp[1], rp[2]}, d{rp[3], rp[4], rp[5]};
    const RigidHit rb = trace_rigid_bodies(w, cam, o, d, max_dist_m);
    HitInfo h;
    hit_init_miss(h, o, d, max_dist_m);
    if (rb.hit) take_rigid(h, rb);
    store_hit(&hits[i], h, rb.hit);
    if (rb.hit) mark_rigid(&hits[i], rb.body);
    if (detail) {
        const f3 pp = rb.hit ? rb.prev_pos : h.hit_pos_m;
        float* q = detail + 9u * (size_t)i;
        q[0] = h.hit_pos_m.x;
        q[1] = h.hit_pos_m.y;
        q[2] = h.hit_pos_m.z;
        q[3] = pp.x;
        q[4] = pp.y;
        q[5] = pp.z;
        q[6] = h.normal.x;
        q[7] = h.normal.y;
        q[8] = h.normal.z;
    }
}

cudaError_t launch_rigid_rays(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                              arc_hit_record* hits, float* detail, cudaStream_t st) {
    rigid_rays_kernel<<<(n + 127u) / 128u, 128, 0, st>>>(w, cam, rays, n, max_dist_m, hits, detail);
    return cudaGetLastError();
}

cudaError_t launch_shadow_di(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, const float* max_dist_m,
                             uint32_t n, float* vis, cudaStream_t st) {
    shadow_di_kernel<<<(n + 127u) / 128u, 128, 0, st>>>(w, cam, rays, max_dist_m, n, vis);
    return cudaGetLastError();
}

cudaError_t launch_shadow(const World& w, const arc_camera_uniforms& cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                          float* vis, cudaStream_t st) {
    if (n == 0) return cudaSuccess;
    shadow_kernel<<<(n + 127u) / 128u, 128, 0, st>>>(w, cam, rays, n, max_dist_m, vis);
    return cudaGetLastError();
}

}  // namespace arc
