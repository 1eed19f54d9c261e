// arc_sharc.cu — SHARC voxel-surfel radiance cache on the GPU.
//
//   sharc_update_kernel   sharc_update.wgsl main (shaders/sharc_update.wgsl:148-191): one thread per
//                         screen tile traces x0 -> x1 (GI bounce), a sun shadow ray and one more
//                         bounce at x1, then deposits L_o(x1) with a CAS slot claim and fixed-point adds.
//   sharc_resolve_kernel  sharc_resolve.wgsl main (shaders/sharc_resolve.wgsl:13-70): EMA fold, aging,
//                         eviction, accumulator clear; one thread per slot.
//   sharc_query_kernel    query_sharc (shaders/common/sharc_query.wgsl:21-29) on a batch.
// Compiled with the canonical arithmetic flags (arc_math.cuh).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "arc_ctx.h"
#include "arc_rigid.cuh"
#include "arc_sharc.cuh"

namespace arc {

struct SharcBuffers {
    uint32_t* keys;
    uint32_t* accum;
    uint4* resolved;
};

// sharc_claim_slot + sharc_deposit (shaders/sharc_update.wgsl:108-144). atomicCAS is strong, so the
// WGSL retry after a spurious weak-CAS failure is not needed.
__device__ __forceinline__ void sharc_deposit(const SharcBuffers& S, uint32_t bucket, uint32_t key, f3 rad) {
    const uint32_t base = bucket * ARC_SHARC_WAYS;
    uint32_t slot = ARC_SHARC_NO_SLOT;
    for (uint32_t i = 0; i < ARC_SHARC_WAYS && slot == ARC_SHARC_NO_SLOT; ++i)
        if (reinterpret_cast<volatile uint32_t*>(S.keys)[base + i] == key) slot = base + i;
    for (uint32_t i = 0; i < ARC_SHARC_WAYS && slot == ARC_SHARC_NO_SLOT; ++i) {
        const uint32_t old = atomicCAS(&S.keys[base + i], 0u, key);
        if (old == 0u || old == key) slot = base + i;
    }
    if (slot == ARC_SHARC_NO_SLOT) return;
    const uint32_t a = slot * 4u;
    atomicAdd(&S.accum[a], f2u(clampf(rad.x, 0.0f, ARC_SHARC_MAX_RADIANCE) * ARC_SHARC_FIXED_SCALE));
    atomicAdd(&S.accum[a + 1u], f2u(clampf(rad.y, 0.0f, ARC_SHARC_MAX_RADIANCE) * ARC_SHARC_FIXED_SCALE));
    atomicAdd(&S.accum[a + 2u], f2u(clampf(rad.z, 0.0f, ARC_SHARC_MAX_RADIANCE) * ARC_SHARC_FIXED_SCALE));
    atomicAdd(&S.accum[a + 3u], 1u);
}

struct Surface {
    bool hit;
    uint32_t mat;
    float t_m;
    f3 pos, normal, albedo, emission;
};

// Lambertian albedo of the cache comparison: per material id, each channel drawn from U[0.1, 0.9]
// by a PCG stream (the same value wherever the material appears).
__device__ __forceinline__ f3 cmp_albedo(uint32_t mat) {
    const uint32_t h0 = pcg_hash(mat * 3u + 0x2545F491u), h1 = pcg_hash(h0 ^ 0x9E3779B9u), h2 = pcg_hash(h1 ^ 0x85EBCA6Bu);
    const float s = 0.8f / 16777216.0f;
    return f3{0.1f + (float)(h0 >> 8) * s, 0.1f + (float)(h1 >> 8) * s, 0.1f + (float)(h2 >> 8) * s};
}

// sharc_trace_surface (shaders/sharc_update.wgsl:32-64): the static world, then the rigid bodies in
// front of its hit (a body hit's LOD colour is its material's albedo).
__device__ __forceinline__ Surface trace_surface(const World& w, const arc_camera_uniforms& cam, f3 o, f3 d, float max_dist) {
    Surface out;
    out.hit = false;
    RayState s;
    HitInfo h;
    StepResult r = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, max_dist, 2u, true)) {
        do {
            r = ray_advance(s, w, cam, h);
        } while (r == kContinue);
    }
    if (r != kHit) h.lod_payload = 0u;
    float lr = __fdiv_rn((float)(h.lod_payload & 0xFFu), 255.0f);
    float lg = __fdiv_rn((float)((h.lod_payload >> 8) & 0xFFu), 255.0f);
    float lb = __fdiv_rn((float)((h.lod_payload >> 16) & 0xFFu), 255.0f);
    if (rigid_count(w, cam)) {
        const RigidHit rb = trace_rigid_bodies(w, cam, o, d, r == kHit ? h.t_voxels * ARC_VOXEL_SIZE : max_dist);
        if (rb.hit) {
            r = kHit;
            h.t_voxels = rb.t_voxels;
            h.hit_pos_m = rb.pos;
            h.normal = rb.normal;
            h.mat = rb.mat;
            const float4 ra = __ldg(&w.palette[2u * rb.mat]);
            lr = ra.x;
            lg = ra.y;
            lb = ra.z;
        }
    }
    if (r != kHit) return out;
    const float4 alb = __ldg(&w.palette[2u * h.mat]);
    const float4 em = __ldg(&w.palette[2u * h.mat + 1u]);
    out.hit = true;
    out.mat = h.mat;
    out.t_m = h.t_voxels * ARC_VOXEL_SIZE;
    out.pos = h.hit_pos_m;
    out.normal = h.normal;
    out.albedo = f3{mixf(alb.x, lr, 0.55f), mixf(alb.y, lg, 0.55f), mixf(alb.z, lb, 0.55f)};
    out.emission = f3{em.x, em.y, em.z};
    return out;
}

// One-bounce radiance estimator of the cache comparison (sun directional light + constant sky, Lambertian):
// L = albedo * (c_sun max(n.l, 0) V(x, l) + L_sky [cosine-sampled ray from x escapes within 64 m]),
// c_sun = sun_power * (1, 0.9, 0.75) * 0.55 as in sharc_shade_surface. One sample per call. The two
// terms are independent and traced separately by onebounce_sun / onebounce_sky.
__device__ __forceinline__ f3 onebounce_sun(const World& w, const arc_camera_uniforms& cam, f3 pos, f3 n) {
    const f3 sun{cam.sun_dir_intensity[0], cam.sun_dir_intensity[1], cam.sun_dir_intensity[2]};
    const float sun_power = cam.sun_dir_intensity[3];
    const float ndl = fmaxf(dot3(n, sun), 0.0f);
    if (!(ndl > 0.001f && sun_power > 0.01f)) return f3{0.0f, 0.0f, 0.0f};
    const float k = ((sun_power * ndl) * shadow_vis(w, cam, add3(pos, mul3s(n, 0.10f)), sun, 32.0f)) * 0.55f;
    return f3{1.0f * k, 0.90f * k, 0.75f * k};
}

__device__ __forceinline__ f3 onebounce_sky(const World& w, const arc_camera_uniforms& cam, f3 pos, f3 n, uint32_t seed) {
    const uint32_t h1 = pcg_hash(seed), h2 = pcg_hash(h1 ^ 0x68E31DA4u);
    const float u1 = (float)(h1 >> 8) * (1.0f / 16777216.0f), u2 = (float)(h2 >> 8) * (1.0f / 16777216.0f);
    f3 t, b;
    make_basis(n, &t, &b);
    const f3 d = cosine_sample(u1, u2, n, t, b);
    RayState s;
    HitInfo hh;
    StepResult r = kMiss;
    if (ray_begin(s, cam, add3(pos, mul3s(n, 0.10f)), d, 0.0f, 64.0f, 2u, true)) {
        do {
            r = ray_advance(s, w, cam, hh);
        } while (r == kContinue);
    }
    return r != kHit ? f3{0.30f, 0.42f, 0.60f} : f3{0.0f, 0.0f, 0.0f};
}

__device__ __forceinline__ f3 onebounce(const World& w, const arc_camera_uniforms& cam, f3 pos, f3 n, f3 albedo,
                                        uint32_t seed) {
    const f3 a = onebounce_sun(w, cam, pos, n), c = onebounce_sky(w, cam, pos, n, seed);
    return f3{albedo.x * (a.x + c.x), albedo.y * (a.y + c.y), albedo.z * (a.z + c.z)};
}

__global__ void sharc_update_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const SharcBuffers S,
                                    const uint32_t* __restrict__ gdm, const uint32_t* __restrict__ gnm, uint32_t W,
                                    uint32_t H, uint32_t mode) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the G-buffer / slots of the kernel ahead
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t tile = (cam.quality_flags[3] & 0xFFu) <= 12u ? 16u : 8u;
    const uint32_t tiles_x = (W + tile - 1u) / tile, tiles_y = (H + tile - 1u) / tile;
    const uint32_t gx = blockIdx.x * blockDim.x + threadIdx.x, gy = blockIdx.y * blockDim.y + threadIdx.y;
    if (gx >= tiles_x || gy >= tiles_y) return;
    const uint32_t frame = __float_as_uint(cam.cam_up_frame[3]);
    const uint32_t hsh = pcg_hash(gx * 1973u + gy * 9277u + frame * 26699u + 0x51ED270Bu);
    const uint32_t px = umin(gx * tile + (hsh & (tile - 1u)), W - 1u);
    const uint32_t py = umin(gy * tile + ((hsh >> 8) & (tile - 1u)), H - 1u);
    const size_t p = (size_t)py * W + px;
    const float depth = __uint_as_float(gdm[2 * p]);
    if (depth >= 1e4f) return;
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const f3 x0 = add3(eye, mul3s(camera_dir(cam, px, py, W, H), depth));
    float ox, oy;
    unpack2x16snorm(gnm[2 * p], &ox, &oy);
    const f3 n0 = oct_decode(ox, oy);
    const f3 sun{cam.sun_dir_intensity[0], cam.sun_dir_intensity[1], cam.sun_dir_intensity[2]};
    const float sun_power = cam.sun_dir_intensity[3];
    const float bounce_max = fminf(cam.ray_distances[2], tile == 16u ? 10.0f : 16.0f);
    float a0, a1, b0, b1;
    gradient_noise((float)px, (float)py, frame, &a0, &a1);
    gradient_noise((float)px + 37.0f, (float)py + 91.0f, frame + 4099u, &b0, &b1);
    f3 t, b;
    make_basis(n0, &t, &b);
    const f3 d0 = cosine_sample(a0, a1, n0, t, b);
    const Surface s1 = trace_surface(w, cam, add3(x0, mul3s(n0, 0.10f)), d0, bounce_max);
    if (!s1.hit) return;
    if (mode == 1u) {  // cache-comparison estimator instead of sharc_shade_surface
        const f3 rad = onebounce(w, cam, s1.pos, s1.normal, cmp_albedo(s1.mat), hsh ^ (frame * 0x9E3779B9u));
        uint32_t bk, key;
        sharc_key(s1.pos, s1.normal, eye, 0.0f, 0.0f, &bk, &key);
        sharc_deposit(S, bk, key, rad);
        return;
    }
    // sharc_shade_surface (shaders/sharc_update.wgsl:68-105)
    const f3 n = s1.normal;
    f3 direct{0.0f, 0.0f, 0.0f};
    const float ndl = fmaxf(dot3(n, sun), 0.0f);
    if (ndl > 0.001f && sun_power > 0.01f) {
        const float vis = shadow_vis(w, cam, add3(s1.pos, mul3s(n, 0.10f)), sun, 32.0f);
        direct = f3{(((1.0f * sun_power) * ndl) * vis) * 0.55f, (((0.90f * sun_power) * ndl) * vis) * 0.55f,
                    (((0.75f * sun_power) * ndl) * vis) * 0.55f};
    }
    make_basis(n, &t, &b);
    const f3 bd = cosine_sample(b0, b1, n, t, b);
    const f3 bo = add3(s1.pos, mul3s(n, 0.10f));
    const Surface s2 = trace_surface(w, cam, bo, bd, bounce_max);
    f3 g{0.0f, 0.0f, 0.0f};
    if (s2.hit) {
        const float att = __fdiv_rn(1.0f, (1.0f + s2.t_m * 0.06f) + (s2.t_m * s2.t_m) * 0.025f);
        const float ndl_em = fmaxf(dot3(n, bd), 0.25f);
        g.x += ((s2.emission.x * 1.15f) * att) * ndl_em;
        g.y += ((s2.emission.y * 1.15f) * att) * ndl_em;
        g.z += ((s2.emission.z * 1.15f) * att) * ndl_em;
        const float4 q = sharc_query(S.resolved, s2.pos, s2.normal, eye, 0.0f, 0.0f);
        g.x += q.x;
        g.y += q.y;
        g.z += q.z;
    } else {
        const float end_y = bo.y + bd.y * bounce_max;
        if (bd.y > 0.15f && end_y >= 32.0f) {
            const float esc = clampf(__fdiv_rn(bd.y - 0.15f, 0.35f), 0.0f, 1.0f);
            const f3 sky = sky_radiance(bd, sun);
            g.x += (sky.x * 0.45f) * esc;
            g.y += (sky.y * 0.45f) * esc;
            g.z += (sky.z * 0.45f) * esc;
        }
    }
    const f3 rad{s1.albedo.x * (direct.x + g.x), s1.albedo.y * (direct.y + g.y), s1.albedo.z * (direct.z + g.z)};
    uint32_t bk, key;
    sharc_key(s1.pos, s1.normal, eye, 0.0f, 0.0f, &bk, &key);
    sharc_deposit(S, bk, key, rad);
}

__global__ void sharc_resolve_kernel(SharcBuffers S) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the deposits of the update ahead
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (slot >= ARC_SHARC_SLOTS) return;
    const uint32_t key = S.keys[slot];
    if (key == 0u) {
        S.resolved[slot] = make_uint4(0u, 0u, 0u, 0u);
        return;
    }
    const uint32_t a = slot * 4u;
    const uint32_t count = S.accum[a + 3u];
    const uint4 prev = S.resolved[slot];
    const bool prev_valid = prev.x == key;
    f3 rad{0.0f, 0.0f, 0.0f};
    uint32_t hist = 0u, stale = 0u;
    if (prev_valid) {
        rad = slot_radiance(prev);
        hist = (prev.z >> 16) & 0xFFu;
        stale = (prev.z >> 24) & 0xFFu;
    }
    if (count > 0u) {
        const float inv = __fdiv_rn(1.0f, (float)count * ARC_SHARC_FIXED_SCALE);
        const f3 smp{(float)S.accum[a] * inv, (float)S.accum[a + 1u] * inv, (float)S.accum[a + 2u] * inv};
        hist = umin(hist + 1u, 255u);
        const float alpha = __fdiv_rn(1.0f, fminf((float)hist, ARC_SHARC_HISTORY_CAP));
        rad = f3{mixf(rad.x, smp.x, alpha), mixf(rad.y, smp.y, alpha), mixf(rad.z, smp.z, alpha)};
        stale = 0u;
        reinterpret_cast<uint4*>(S.accum)[slot] = make_uint4(0u, 0u, 0u, 0u);
    } else {
        stale += 1u;
        if (!prev_valid || stale > ARC_SHARC_STALE_EVICT_AGE) {
            S.keys[slot] = 0u;
            S.resolved[slot] = make_uint4(0u, 0u, 0u, 0u);
            return;
        }
    }
    const float cr = clampf(rad.x, 0.0f, ARC_SHARC_MAX_RADIANCE), cg = clampf(rad.y, 0.0f, ARC_SHARC_MAX_RADIANCE),
                cb = clampf(rad.z, 0.0f, ARC_SHARC_MAX_RADIANCE);
    S.resolved[slot] = make_uint4(key, pack2x16float(cr, cg), f16_bits(cb) | ((hist & 0xFFu) << 16) | ((stale & 0xFFu) << 24), 0u);
}

__global__ void sharc_query_kernel(const uint4* __restrict__ res, const float* __restrict__ pos, const float* __restrict__ nrm,
                                   const float* __restrict__ jit, uint32_t n, f3 cam, float4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const f3 p{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, q{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    const float jx = jit ? jit[2 * i] : 0.0f, jy = jit ? jit[2 * i + 1] : 0.0f;
    out[i] = sharc_query(res, p, q, cam, jx, jy);
}

__global__ void sharc_deposit_kernel(SharcBuffers S, f3 pos, f3 n, f3 cam, f3 rad, uint32_t count) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    uint32_t b, k;
    sharc_key(pos, n, cam, 0.0f, 0.0f, &b, &k);
    sharc_deposit(S, b, k, rad);
}

// GI hit points of a frame: per pixel with a primary hit, the Pass-2A GI ray is traced again from the
// G-buffer and its hit recorded as position, normal, material albedo (cmp_albedo) and the 9 NRC inputs
// (position / world extent, normal, view direction = -ray direction). A block of 128 threads sets up
// the GI rays of its 16 x 8 pixels, sorts them by direction octant in shared memory (pixels without a
// GI ray drop out) and traces them from the sorted slots, as gi_rows_kernel does for a frame.
__global__ void __launch_bounds__(128) gi_points_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const uint32_t* __restrict__ gdm,
                                 const uint32_t* __restrict__ gnm, uint32_t W, uint32_t H, float* __restrict__ pos,
                                 float* __restrict__ nrm, float* __restrict__ alb, float* __restrict__ nrc_in,
                                 uint32_t* __restrict__ valid, unsigned long long* __restrict__ n_valid,
                                 uint32_t* __restrict__ list) {
    __shared__ float s_ray[6][128];
    __shared__ uint32_t s_k[128];
    __shared__ uint32_t s_cnt[9], s_base[10];
    const uint32_t t = threadIdx.x;
    if (t < 9u) s_cnt[t] = 0u;
    __syncthreads();
    const uint32_t x = blockIdx.x * 16u + (t & 15u), y = blockIdx.y * 8u + (t >> 4);
    uint32_t key = 8u;
    f3 go{0.0f, 0.0f, 0.0f}, gd{0.0f, 0.0f, 1.0f};
    size_t gk = 0;
    if (x < W && y < H) {
        gk = (size_t)y * W + x;
        if (gi_setup(w, cam, x, y, W, H, gdm[2 * gk], gnm[2 * gk], &go, &gd))
            key = (gd.x < 0.0f ? 1u : 0u) | (gd.y < 0.0f ? 2u : 0u) | (gd.z < 0.0f ? 4u : 0u);
        else
            valid[gk] = 0u;
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
        s_k[slot] = (uint32_t)gk;
    }
    __syncthreads();
    if (t >= s_base[8]) return;
    const size_t k = s_k[t];
    const f3 o{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, d{s_ray[3][t], s_ray[4][t], s_ray[5][t]};
    uint32_t ok = 0u;
    {
        RayState s;
        HitInfo h;
        StepResult r = kMiss;
        if (ray_begin(s, cam, o, d, 0.0f, cam.ray_distances[2], 2u, true)) {
            do {
                r = ray_advance(s, w, cam, h);
            } while (r == kContinue);
        }
        if (r == kHit) {
            ok = 1u;
            const f3 a = cmp_albedo(h.mat);
            pos[3 * k] = h.hit_pos_m.x;
            pos[3 * k + 1] = h.hit_pos_m.y;
            pos[3 * k + 2] = h.hit_pos_m.z;
            nrm[3 * k] = h.normal.x;
            nrm[3 * k + 1] = h.normal.y;
            nrm[3 * k + 2] = h.normal.z;
            alb[3 * k] = a.x;
            alb[3 * k + 1] = a.y;
            alb[3 * k + 2] = a.z;
            const float ex = (float)cam.world_grid_dims[0] * 16.0f, ey = (float)cam.world_grid_dims[1] * 16.0f,
                        ez = (float)cam.world_grid_dims[2] * 16.0f;
            float* q = nrc_in + 9 * k;
            q[0] = __fdiv_rn(h.hit_pos_m.x, ex);
            q[1] = __fdiv_rn(h.hit_pos_m.y, ey);
            q[2] = __fdiv_rn(h.hit_pos_m.z, ez);
            q[3] = h.normal.x;
            q[4] = h.normal.y;
            q[5] = h.normal.z;
            q[6] = -d.x;
            q[7] = -d.y;
            q[8] = -d.z;
        }
    }
    valid[k] = ok;
    // warp-aggregated slot in the compacted list (order across warps is arbitrary)
    const uint32_t act = __activemask();
    const uint32_t m = __ballot_sync(act, ok != 0u);
    const uint32_t lane = t & 31u;
    unsigned long long base = 0ull;
    if (m && lane == (uint32_t)(__ffs(m) - 1)) base = atomicAdd(n_valid, (unsigned long long)__popc(m));
    if (m) base = __shfl_sync(act, base, __ffs(m) - 1);
    if (ok && list) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)k;
}

// GI hit points from the frame kernel's GI hit records, without tracing again: the point is the centre
// of the entry face of the hit cell (LOD cells included), the normal that face's, the albedo the hit
// material's, and the view direction points from the point back to the GI ray's origin (the primary
// hit + 0.10 m along its normal, from the G-buffer). Outputs as gi_points_kernel, list included.
__global__ void gi_points_hits_kernel(const __grid_constant__ arc_camera_uniforms cam, const uint32_t* __restrict__ gdm,
                                      const uint32_t* __restrict__ gnm, const arc_hit_record* __restrict__ gi_hits,
                                      uint32_t W, uint32_t H, float* __restrict__ pos, float* __restrict__ nrm,
                                      float* __restrict__ alb, float* __restrict__ nrc_in, uint32_t* __restrict__ valid,
                                      unsigned long long* __restrict__ n_valid, uint32_t* __restrict__ list) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;
    const size_t k = (size_t)y * W + x;
    const arc_hit_record h = gi_hits[k];
    const float hit_dist = __uint_as_float(gdm[2 * k]);
    uint32_t ok = (h.flags & ARC_HIT_FLAG_HIT) && h.face < 6u && hit_dist < 1e4f ? 1u : 0u;
    if (ok) {
        const int32_t span_i = 1 << (2u * ((h.flags >> 1) & 7u));  // LOD cell of the hit (1 voxel at level 0)
        const float span = (float)span_i;
        const float c0 = (float)(h.voxel[0] & ~(span_i - 1)), c1 = (float)(h.voxel[1] & ~(span_i - 1)),
                    c2 = (float)(h.voxel[2] & ~(span_i - 1));
        const float axis_sign = (h.face & 1u) ? -1.0f : 1.0f;  // +X, -X, +Y, -Y, +Z, -Z
        const uint32_t axis = h.face >> 1;
        f3 n{0.0f, 0.0f, 0.0f};
        f3 p{c0 + 0.5f * span, c1 + 0.5f * span, c2 + 0.5f * span};
        if (axis == 0) {
            n.x = axis_sign;
            p.x = c0 + (axis_sign > 0.0f ? span : 0.0f);
        } else if (axis == 1) {
            n.y = axis_sign;
            p.y = c1 + (axis_sign > 0.0f ? span : 0.0f);
        } else {
            n.z = axis_sign;
            p.z = c2 + (axis_sign > 0.0f ? span : 0.0f);
        }
        p = mul3s(p, ARC_VOXEL_SIZE);
        const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
        const f3 hp = add3(eye, mul3s(camera_dir(cam, x, y, W, H), hit_dist));
        float ox, oy;
        unpack2x16snorm(gnm[2 * k], &ox, &oy);
        const f3 o = add3(hp, mul3s(oct_decode(ox, oy), 0.10f));
        const f3 v = sub3(o, p);
        const float len = length3(v);
        const f3 view = len > 0.0f ? mul3s(v, __fdiv_rn(1.0f, len)) : n;
        const f3 a = cmp_albedo(h.mat);
        pos[3 * k] = p.x;
        pos[3 * k + 1] = p.y;
        pos[3 * k + 2] = p.z;
        nrm[3 * k] = n.x;
        nrm[3 * k + 1] = n.y;
        nrm[3 * k + 2] = n.z;
        alb[3 * k] = a.x;
        alb[3 * k + 1] = a.y;
        alb[3 * k + 2] = a.z;
        const float ex = (float)cam.world_grid_dims[0] * 16.0f, ey = (float)cam.world_grid_dims[1] * 16.0f,
                    ez = (float)cam.world_grid_dims[2] * 16.0f;
        float* q = nrc_in + 9 * k;
        q[0] = __fdiv_rn(p.x, ex);
        q[1] = __fdiv_rn(p.y, ey);
        q[2] = __fdiv_rn(p.z, ez);
        q[3] = n.x;
        q[4] = n.y;
        q[5] = n.z;
        q[6] = view.x;
        q[7] = view.y;
        q[8] = view.z;
    }
    valid[k] = ok;
    const uint32_t act = __activemask();
    const uint32_t m = __ballot_sync(act, ok != 0u);
    const uint32_t lane = (threadIdx.x + threadIdx.y * blockDim.x) & 31u;
    unsigned long long base = 0ull;
    if (m && lane == (uint32_t)(__ffs(m) - 1)) base = atomicAdd(n_valid, (unsigned long long)__popc(m));
    if (m) base = __shfl_sync(act, base, __ffs(m) - 1);
    if (ok && list) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)k;
}

__global__ void onebounce_kernel(const World w, const __grid_constant__ arc_camera_uniforms cam, const uint32_t* __restrict__ idx,
                                 uint32_t n, const float* __restrict__ pos, const float* __restrict__ nrm,
                                 const float* __restrict__ alb, uint32_t spp, uint32_t seed, uint32_t accumulate,
                                 float* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t p = idx ? idx[i] : i;
    const f3 x{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]}, nn{nrm[3 * p], nrm[3 * p + 1], nrm[3 * p + 2]};
    const f3 a{alb[3 * p], alb[3 * p + 1], alb[3 * p + 2]};
    f3 sum{0.0f, 0.0f, 0.0f};
    for (uint32_t k = 0; k < spp; ++k) {
        const f3 l = onebounce(w, cam, x, nn, a, pcg_hash(p * 0x9E3779B9u ^ pcg_hash(seed + k * 0x632BE5ABu)));
        sum.x += l.x;
        sum.y += l.y;
        sum.z += l.z;
    }
    const float inv = __fdiv_rn(1.0f, (float)spp);
    if (accumulate) {
        out[3 * i] += sum.x * inv;
        out[3 * i + 1] += sum.y * inv;
        out[3 * i + 2] += sum.z * inv;
    } else {
        out[3 * i] = sum.x * inv;
        out[3 * i + 1] = sum.y * inv;
        out[3 * i + 2] = sum.z * inv;
    }
}

// NRC training samples from the compacted GI hit list, stratified: with cluster size 1, sample i takes
// list entry floor((i n_valid + phase) / n_samples) (phase in [0, n_valid) from the seed), so every
// point is covered evenly; with cluster size k, samples come in runs of k consecutive list entries
// (a warp's rays then start from neighbouring points: one warp-aggregated append of the GI-points
// pass) whose starts are stratified the same way over n_samples / k runs. A block of
// 4 warps takes 64 samples: warps 0 and 2 trace the sun term of samples 0..31 and 32..63, warps 1 and 3
// the sky term of the same samples (each warp follows one traversal path), and shared memory sums
// them. Sample i is stored at slot (i mod steps) * (n_samples / steps) + i / steps, so each of the
// `steps` training slices spans the whole frame. Target: the 1-spp estimator with albedo 1.
__global__ void __launch_bounds__(128) train_samples_list_kernel(
    const World w, const __grid_constant__ arc_camera_uniforms cam, const uint32_t* __restrict__ list,
    const unsigned long long* __restrict__ n_valid, const float* __restrict__ pos, const float* __restrict__ nrm,
    const float* __restrict__ nrc_in, uint32_t seed, uint32_t n_samples, uint32_t steps, uint32_t cluster,
    float* __restrict__ train_in, float* __restrict__ train_t, uint32_t* __restrict__ gate) {
    __shared__ float s_sun[64][3];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t pair = warp >> 1, part = warp & 1u;  // part 0: sun, 1: sky
    const uint32_t i = blockIdx.x * 64u + pair * 32u + lane;
    const unsigned long long nv = *n_valid;
    if (blockIdx.x == 0 && threadIdx.x == 0) *gate = nv ? n_samples : 0u;
    if (!nv) return;  // uniform over the grid
    const bool valid = i < n_samples;
    f3 l{0.0f, 0.0f, 0.0f};
    uint32_t p = 0;
    if (valid) {
        const unsigned long long phase = ((unsigned long long)pcg_hash(seed) * nv) >> 32;  // < nv
        // clusters of `cluster` consecutive list entries, the clusters stratified over the list
        const uint32_t c = i / cluster, r = i % cluster, n_cl = n_samples / cluster;
        const unsigned long long start = ((unsigned long long)c * nv + phase) / n_cl;  // < nv
        const uint32_t j = (uint32_t)(start + r < nv ? start + r : nv - 1ull);
        p = __ldg(&list[j]);
        const f3 x{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]}, n{nrm[3 * p], nrm[3 * p + 1], nrm[3 * p + 2]};
        l = part ? onebounce_sky(w, cam, x, n, pcg_hash(i ^ pcg_hash(seed ^ 0xB5297A4Du))) : onebounce_sun(w, cam, x, n);
    }
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");  // the training kernel behind may be scheduled
    const uint32_t k = pair * 32u + lane;
    if (part == 0u) {
        s_sun[k][0] = l.x;
        s_sun[k][1] = l.y;
        s_sun[k][2] = l.z;
    }
    __syncthreads();
    if (!valid || part == 0u) return;
    l.x += s_sun[k][0];
    l.y += s_sun[k][1];
    l.z += s_sun[k][2];
    const uint32_t per = n_samples / steps;
    const size_t slot = (size_t)(i % steps) * per + i / steps;
#pragma unroll
    for (int q = 0; q < 9; ++q) train_in[slot * 9 + q] = nrc_in[(size_t)p * 9 + q];
    train_t[3 * slot] = l.x;
    train_t[3 * slot + 1] = l.y;
    train_t[3 * slot + 2] = l.z;
}

__global__ void sharc_query_list_kernel(const uint4* __restrict__ res, const uint32_t* __restrict__ list,
                                        const unsigned long long* __restrict__ n_dev, uint32_t max_n,
                                        const float* __restrict__ pos, const float* __restrict__ nrm, f3 cam,
                                        float4* __restrict__ out) {
    asm volatile("griddepcontrol.wait;" ::: "memory");  // the resolved slots / hit list of the kernel ahead
    const unsigned long long nd = *n_dev;
    const uint32_t n = nd < max_n ? (uint32_t)nd : max_n;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t i = __ldg(&list[j]);
        const f3 p{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]}, q{nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
        out[i] = sharc_query(res, p, q, cam, 0.0f, 0.0f);
    }
}

}  // namespace arc

namespace {

int sharc_err(arc_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

int ensure_sharc(arc_ctx* c) {
    if (c->d_sharc_keys) return ARC_OK;
    cudaError_t e;
    if ((e = cudaMalloc((void**)&c->d_sharc_keys, ARC_SHARC_SLOTS * 4u)) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_sharc_accum, ARC_SHARC_SLOTS * 16u)) != cudaSuccess ||
        (e = cudaMalloc((void**)&c->d_sharc_resolved, ARC_SHARC_SLOTS * 16u)) != cudaSuccess)
        return sharc_err(c, ARC_E_CUDA, std::string("SHARC allocation: ") + cudaGetErrorString(e));
    cudaMemsetAsync(c->d_sharc_keys, 0, ARC_SHARC_SLOTS * 4u, c->stream);
    cudaMemsetAsync(c->d_sharc_accum, 0, ARC_SHARC_SLOTS * 16u, c->stream);
    cudaMemsetAsync(c->d_sharc_resolved, 0, ARC_SHARC_SLOTS * 16u, c->stream);
    return ARC_OK;
}

arc::SharcBuffers bufs(arc_ctx* c) {
    return arc::SharcBuffers{c->d_sharc_keys, c->d_sharc_accum, reinterpret_cast<uint4*>(c->d_sharc_resolved)};
}

int launch_check(arc_ctx* c, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return sharc_err(c, ARC_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return ARC_OK;
}

}  // namespace

extern "C" {

int arc_sharc_reset(arc_ctx* c) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = ensure_sharc(c);
    if (rc) return rc;
    cudaMemsetAsync(c->d_sharc_keys, 0, ARC_SHARC_SLOTS * 4u, c->stream);
    cudaMemsetAsync(c->d_sharc_accum, 0, ARC_SHARC_SLOTS * 16u, c->stream);
    cudaMemsetAsync(c->d_sharc_resolved, 0, ARC_SHARC_SLOTS * 16u, c->stream);
    return launch_check(c, "arc_sharc_reset");
}

int arc_sharc_update_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!gdm || !gnm || width == 0 || height == 0) return sharc_err(c, ARC_E_INVALID_ARG, "bad G-buffer");
    if ((c->cam.world_grid_dims[3] & 0xFFFFu) != width || (c->cam.world_grid_dims[3] >> 16) != height)
        return sharc_err(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    if ((rc = ensure_sharc(c))) return rc;
    const uint32_t tile = (c->cam.quality_flags[3] & 0xFFu) <= 12u ? 16u : 8u;
    const uint32_t tx = (width + tile - 1u) / tile, ty = (height + tile - 1u) / tile;
    dim3 block(8, 8), grid((tx + 7u) / 8u, (ty + 7u) / 8u);
    cudaError_t e = arc_launch_overlapped(c, arc::sharc_update_kernel, grid, block, 0, c->world(), c->cam, bufs(c), gdm, gnm,
                                          width, height, c->sharc_mode);
    if (e != cudaSuccess) return sharc_err(c, ARC_E_CUDA, std::string("sharc_update_kernel: ") + cudaGetErrorString(e));
    return launch_check(c, "sharc_update_kernel");
}

int arc_sharc_set_mode(arc_ctx* c, uint32_t mode) {
    if (!c || mode > 1u) return ARC_E_INVALID_ARG;
    c->sharc_mode = mode;
    return ARC_OK;
}

int arc_gi_points_from_hits_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm,
                                const arc_hit_record* gi_hits, float* pos, float* nrm, float* albedo, float* nrc_in,
                                uint32_t* valid, uint64_t* n_valid, uint32_t* list) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!gdm || !gnm || !gi_hits || !pos || !nrm || !albedo || !nrc_in || !valid || !n_valid)
        return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    if ((c->cam.world_grid_dims[3] & 0xFFFFu) != width || (c->cam.world_grid_dims[3] >> 16) != height)
        return sharc_err(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    cudaMemsetAsync(n_valid, 0, sizeof(uint64_t), c->stream);
    // a warp per 32 consecutive pixels of a row: its 20 B records and the 12 B / 36 B outputs are
    // contiguous runs
    dim3 block(32, 4), grid((width + 31u) / 32u, (height + 3u) / 4u);
    arc::gi_points_hits_kernel<<<grid, block, 0, c->stream>>>(c->cam, gdm, gnm, gi_hits, width, height, pos, nrm, albedo,
                                                              nrc_in, valid, reinterpret_cast<unsigned long long*>(n_valid),
                                                              list);
    return launch_check(c, "gi_points_hits_kernel");
}

int arc_gi_points_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm, float* pos,
                      float* nrm, float* albedo, float* nrc_in, uint32_t* valid, uint64_t* n_valid, uint32_t* list) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!gdm || !gnm || !pos || !nrm || !albedo || !nrc_in || !valid || !n_valid) return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    if ((c->cam.world_grid_dims[3] & 0xFFFFu) != width || (c->cam.world_grid_dims[3] >> 16) != height)
        return sharc_err(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    cudaMemsetAsync(n_valid, 0, sizeof(uint64_t), c->stream);
    dim3 grid((width + 15u) / 16u, (height + 7u) / 8u);
    arc::gi_points_kernel<<<grid, 128, 0, c->stream>>>(c->world(), c->cam, gdm, gnm, width, height, pos, nrm, albedo,
                                                         nrc_in, valid, reinterpret_cast<unsigned long long*>(n_valid), list);
    return launch_check(c, "gi_points_kernel");
}

int arc_launch_train_samples_list(arc_ctx* c, const uint32_t* list, const unsigned long long* n_valid, const float* pos,
                                  const float* nrm, const float* nrc_in, uint32_t seed, uint32_t n_samples, uint32_t steps,
                                  float* train_in, float* train_t, uint32_t* gate) {
    const uint32_t cluster = (n_samples % c->nrc_sample_cluster) ? 1u : c->nrc_sample_cluster;
    arc::train_samples_list_kernel<<<(n_samples + 63u) / 64u, 128, 0, c->stream>>>(
        c->world(), c->cam, list, n_valid, pos, nrm, nrc_in, seed, n_samples, steps, cluster, train_in, train_t, gate);
    return launch_check(c, "train_samples_list_kernel");
}

// One SHARC frame with the query beside the update: the query at the hit list reads the resolved
// slots of the previous frame's resolve, on the side stream, while the update deposits this frame's
// radiance; the resolve waits for both.
int arc_sharc_frame_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm, const uint32_t* gnm,
                        const uint32_t* list, const uint64_t* n_dev, uint32_t max_n, const float* pos, const float* normal,
                        float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = arc_ctx_side_begin(c);
    if (rc) return rc;
    rc = arc_sharc_query_list_dev(c, list, n_dev, max_n, pos, normal, out);
    int rc2 = arc_ctx_side_end(c);
    if (rc || (rc = rc2)) return rc;
    if ((rc = arc_sharc_update_dev(c, width, height, gdm, gnm))) return rc;
    if ((rc = arc_ctx_side_join(c))) return rc;
    return arc_sharc_resolve(c);
}

int arc_sharc_query_list_dev(arc_ctx* c, const uint32_t* list, const uint64_t* n_dev, uint32_t max_n, const float* pos,
                             const float* normal, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (!c->have_cam) return sharc_err(c, ARC_E_NO_CAMERA, "no camera set");
    if (max_n && (!list || !n_dev || !pos || !normal || !out)) return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    int rc = ensure_sharc(c);
    if (rc || max_n == 0) return rc;
    const arc::f3 cam{c->cam.cam_pos_time[0], c->cam.cam_pos_time[1], c->cam.cam_pos_time[2]};
    const uint32_t blocks = std::min<uint32_t>((max_n + 255u) / 256u, (uint32_t)c->n_sm * 8u);
    cudaError_t e = arc_launch_overlapped(c, arc::sharc_query_list_kernel, dim3(blocks), dim3(256), 0, reinterpret_cast<const uint4*>(c->d_sharc_resolved), list,
                                                                reinterpret_cast<const unsigned long long*>(n_dev), max_n,
                                                                pos, normal, cam, reinterpret_cast<float4*>(out));
    if (e != cudaSuccess) return sharc_err(c, ARC_E_CUDA, std::string("sharc_query_list_kernel: ") + cudaGetErrorString(e));
    return launch_check(c, "sharc_query_list_kernel");
}

int arc_onebounce_dev(arc_ctx* c, const uint32_t* idx, uint32_t n, const float* pos, const float* nrm, const float* albedo,
                      uint32_t spp, uint32_t seed, int accumulate, float* out) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (n == 0) return ARC_OK;
    if (!pos || !nrm || !albedo || !out || spp == 0) return sharc_err(c, ARC_E_INVALID_ARG, "null buffer or spp 0");
    arc::onebounce_kernel<<<(n + 127u) / 128u, 128, 0, c->stream>>>(c->world(), c->cam, idx, n, pos, nrm, albedo, spp, seed,
                                                                     accumulate ? 1u : 0u, out);
    return launch_check(c, "onebounce_kernel");
}

int arc_sharc_resolve(arc_ctx* c) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = ensure_sharc(c);
    if (rc) return rc;
    cudaError_t e = arc_launch_overlapped(c, arc::sharc_resolve_kernel, dim3(ARC_SHARC_SLOTS / 256u), dim3(256), 0, bufs(c));
    if (e != cudaSuccess) return sharc_err(c, ARC_E_CUDA, std::string("sharc_resolve_kernel: ") + cudaGetErrorString(e));
    return launch_check(c, "sharc_resolve_kernel");
}

int arc_sharc_query_dev(arc_ctx* c, const float* pos, const float* normal, const float* jitter, uint32_t n, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (!c->have_cam) return sharc_err(c, ARC_E_NO_CAMERA, "no camera set");
    if (n && (!pos || !normal || !out)) return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    int rc = ensure_sharc(c);
    if (rc || n == 0) return rc;
    const arc::f3 cam{c->cam.cam_pos_time[0], c->cam.cam_pos_time[1], c->cam.cam_pos_time[2]};
    arc::sharc_query_kernel<<<(n + 127u) / 128u, 128, 0, c->stream>>>(reinterpret_cast<const uint4*>(c->d_sharc_resolved), pos,
                                                                      normal, jitter, n, cam, reinterpret_cast<float4*>(out));
    return launch_check(c, "sharc_query_kernel");
}

// Host-buffer form: the inputs are staged to the device, the results copied back, and the call returns
// when they are in `out` (the status word is checked as for every host-buffer entry point).
int arc_sharc_query(arc_ctx* c, const float* pos, const float* normal, const float* jitter, uint32_t n, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (n == 0) return ARC_OK;
    if (!pos || !normal || !out) return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    void* stage;
    int rc = arc_ctx_stage(c, (size_t)n * 48u, &stage);
    if (rc) return rc;
    float* d_pos = static_cast<float*>(stage);
    float* d_nrm = d_pos + 3u * (size_t)n;
    float* d_out = d_nrm + 3u * (size_t)n;
    float* d_jit = jitter ? d_out + 4u * (size_t)n : nullptr;
    cudaMemcpyAsync(d_pos, pos, (size_t)n * 12u, cudaMemcpyHostToDevice, c->stream);
    cudaMemcpyAsync(d_nrm, normal, (size_t)n * 12u, cudaMemcpyHostToDevice, c->stream);
    if (jitter) cudaMemcpyAsync(d_jit, jitter, (size_t)n * 8u, cudaMemcpyHostToDevice, c->stream);
    if ((rc = arc_sharc_query_dev(c, d_pos, d_nrm, d_jit, n, d_out))) return rc;
    cudaMemcpyAsync(out, d_out, (size_t)n * 16u, cudaMemcpyDeviceToHost, c->stream);
    if ((rc = launch_check(c, "arc_sharc_query"))) return rc;
    return arc_ctx_finish(c);
}

int arc_nrc_train_samples_dev(arc_ctx* c, const uint32_t* list, const uint64_t* n_valid, const float* pos,
                              const float* normal, const float* nrc_in, uint32_t seed, uint32_t n_samples, uint32_t steps,
                              float* train_in, float* train_t) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!list || !n_valid || !pos || !normal || !nrc_in || !train_in || !train_t)
        return sharc_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (steps == 0 || n_samples < steps || n_samples % steps)
        return sharc_err(c, ARC_E_INVALID_ARG, "n_samples must be a non-zero multiple of steps");
    if (!c->d_nrc_gate && cudaMalloc((void**)&c->d_nrc_gate, sizeof(uint32_t)) != cudaSuccess)
        return sharc_err(c, ARC_E_CUDA, "gate word allocation");
    return arc_launch_train_samples_list(c, list, reinterpret_cast<const unsigned long long*>(n_valid), pos, normal, nrc_in,
                                         seed, n_samples, steps, train_in, train_t, c->d_nrc_gate);
}

int arc_sharc_deposit_dev(arc_ctx* c, const float pos[3], const float normal[3], const float cam_pos[3], const float rad[3],
                          uint32_t n_threads) {
    if (!c || !pos || !normal || !cam_pos || !rad) return ARC_E_INVALID_ARG;
    int rc = ensure_sharc(c);
    if (rc || n_threads == 0) return rc;
    arc::sharc_deposit_kernel<<<(n_threads + 63u) / 64u, 64, 0, c->stream>>>(
        bufs(c), arc::f3{pos[0], pos[1], pos[2]}, arc::f3{normal[0], normal[1], normal[2]},
        arc::f3{cam_pos[0], cam_pos[1], cam_pos[2]}, arc::f3{rad[0], rad[1], rad[2]}, n_threads);
    return launch_check(c, "sharc_deposit_kernel");
}

int arc_sharc_download(arc_ctx* c, uint32_t* keys, uint32_t* accum, arc_sharc_slot* resolved) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = ensure_sharc(c);
    if (rc) return rc;
    if (keys) cudaMemcpyAsync(keys, c->d_sharc_keys, ARC_SHARC_SLOTS * 4u, cudaMemcpyDeviceToHost, c->stream);
    if (accum) cudaMemcpyAsync(accum, c->d_sharc_accum, ARC_SHARC_SLOTS * 16u, cudaMemcpyDeviceToHost, c->stream);
    if (resolved) cudaMemcpyAsync(resolved, c->d_sharc_resolved, ARC_SHARC_SLOTS * 16u, cudaMemcpyDeviceToHost, c->stream);
    if ((rc = launch_check(c, "arc_sharc_download"))) return rc;
    return arc_ctx_finish(c);
}

int arc_sharc_upload(arc_ctx* c, const uint32_t* keys, const uint32_t* accum, const arc_sharc_slot* resolved) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = ensure_sharc(c);
    if (rc) return rc;
    if (keys) cudaMemcpyAsync(c->d_sharc_keys, keys, ARC_SHARC_SLOTS * 4u, cudaMemcpyHostToDevice, c->stream);
    if (accum) cudaMemcpyAsync(c->d_sharc_accum, accum, ARC_SHARC_SLOTS * 16u, cudaMemcpyHostToDevice, c->stream);
    if (resolved) cudaMemcpyAsync(c->d_sharc_resolved, resolved, ARC_SHARC_SLOTS * 16u, cudaMemcpyHostToDevice, c->stream);
    if ((rc = launch_check(c, "arc_sharc_upload"))) return rc;
    return arc_ctx_finish(c);
}

}  // extern "C"
