// arc_restir.cu — ReSTIR GI temporal pass (the GI part of temporal_main,
// shaders/lighting_restir_gi.wgsl:61-336; reservoir helpers shaders/common/types.wgsl:90-190).
//
//   restir_sun_kernel          one thread per pixel: the sun shadow ray of every hit pixel that is
//                              not skipped this frame (checkerboard half rate in low-tap mode), its
//                              visibility parked in the output reservoir's shadow word.
//   restir_gi_temporal_kernel  one thread per pixel: reprojected history validation, the temporal
//                              average of the sun visibility, one GI candidate, temporal RIS, the
//                              32 B reservoir.
//
// The GI candidate is the secondary ray the frame kernel already traced (traced again here only
// when rigid bodies are in the frame, whose hits a record cannot give back): its hit record (hit flag,
// material, face, depth, voxel, cell level) gives back the secondary hit exactly (the hit point is
// (origin * 16 + dir * depth * 16) / 16, the same operations as the traversal's; the node payload
// for the LOD colour is a four-load point query), so the pass traces only the sun shadow ray and,
// on a cache miss, the secondary hit's sun ray. Radiance at the secondary hit comes from the SHARC
// cache (query_sharc with the pass's jitter) or from a per-pixel radiance buffer (a neural cache's
// prediction at the hit). The emissive-light ReSTIR DI half of the reference pass needs the
// emissive light list, which this library does not build; with no emissive lights the reference's
// DI output is the empty reservoir and its GI part is what is computed here.
// Compiled with the canonical arithmetic flags (arc_math.cuh).
#include <cuda_runtime.h>

#include <string>

#include "arc_ctx.h"
#include "arc_sharc.cuh"
#include "arc_surface.cuh"

namespace arc {

struct RestirParams {
    World world;
    uint32_t width, height;
    const uint2* gdm;
    const uint2* gnm;
    const arc_hit_record* gi_hits;
    const arc_gi_reservoir* res_in;
    arc_gi_reservoir* res_out;
    const uint4* sharc;    // resolved SHARC slots (used when radiance is null)
    const float* radiance; // 3 floats per pixel, or null
};

__device__ __forceinline__ float luma3(f3 c) { return (c.x * 0.2126f + c.y * 0.7152f) + c.z * 0.0722f; }

// rand_f32 (types.wgsl:264-267)
__device__ __forceinline__ float rand01(uint32_t& seed) {
    seed = pcg_hash(seed);
    return __fdiv_rn((float)seed, 4294967295.0f);
}

// pack_norm_m_flags (types.wgsl:132-136)
__device__ __forceinline__ uint32_t pack_norm_m_flags(f3 n, uint32_t m, uint32_t age, bool is_sky) {
    const float l1 = (fabsf(n.x) + fabsf(n.y)) + fabsf(n.z);
    const float s = __fdiv_rn(1.0f, fmaxf(l1, 1e-6f));
    float px = n.x * s, py = n.y * s;
    if (n.z < 0.0f) {
        const float wx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        const float wy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = wx;
        py = wy;
    }
    const int ix = max(-128, min(127, (int)rintf(px * 127.0f)));
    const int iy = max(-128, min(127, (int)rintf(py * 127.0f)));
    const uint32_t ux = (uint32_t)(ix + 128), uy = (uint32_t)(iy + 128);
    return (ux & 0xFFu) | ((uy & 0xFFu) << 8) | ((umin(m, 16u) & 0xFFu) << 16) | ((umin(age, 127u) & 0x7Fu) << 24) |
           (is_sky ? 0x80000000u : 0u);
}

// unpack_normal (types.wgsl:138-143)
__device__ __forceinline__ f3 unpack_res_normal(uint32_t nmf) {
    const float ox = __fdiv_rn((float)(nmf & 0xFFu) - 128.0f, 127.0f);
    const float oy = __fdiv_rn((float)((nmf >> 8) & 0xFFu) - 128.0f, 127.0f);
    return oct_decode(ox, oy);
}

__device__ __forceinline__ void store_reservoir(arc_gi_reservoir* r, f3 pos, uint32_t nmf, uint32_t lo_rg, uint32_t lo_b_w,
                                                float depth, uint32_t shadow) {
    uint4* q = reinterpret_cast<uint4*>(r);
    q[0] = make_uint4(__float_as_uint(pos.x), __float_as_uint(pos.y), __float_as_uint(pos.z), nmf);
    q[1] = make_uint4(lo_rg, lo_b_w, __float_as_uint(depth), shadow);
}

// Reprojected history of a hit pixel (lighting_restir_gi.wgsl:95-115): the previous reservoir's two
// halves and whether it is valid here.
__device__ __forceinline__ bool restir_history(const RestirParams& P, const arc_camera_uniforms& cam, uint32_t x, uint32_t y,
                                               uint32_t normal_word, f3 hp, float hit_dist, uint4* pr0, uint4* pr1) {
    const float pu = __fdiv_rn((float)x + 0.5f, (float)P.width), pv = __fdiv_rn((float)y + 0.5f, (float)P.height);
    const float prev_u = pu + f16_value(normal_word & 0xFFFFu), prev_v = pv + f16_value(normal_word >> 16);
    *pr0 = make_uint4(0u, 0u, 0u, 0u);
    *pr1 = make_uint4(0u, 0u, 0u, 0u);
    if (!(prev_u >= 0.0f && prev_u < 1.0f && prev_v >= 0.0f && prev_v < 1.0f)) return false;
    const uint32_t ppx = uclamp(f2u(prev_u * (float)P.width), 0u, P.width - 1u);
    const uint32_t ppy = uclamp(f2u(prev_v * (float)P.height), 0u, P.height - 1u);
    const uint4* q = reinterpret_cast<const uint4*>(&P.res_in[(size_t)ppy * P.width + ppx]);
    *pr0 = q[0];
    *pr1 = q[1];
    const uint32_t pm = (pr0->w >> 16) & 0xFFu, page = (pr0->w >> 24) & 0x7Fu;
    const float pdepth = __uint_as_float(pr1->z);
    if (pm > 0u && page <= 12u && pdepth < 1e4f) {
        const float pcd = length3(sub3(hp, f3{cam.prev_cam_pos[0], cam.prev_cam_pos[1], cam.prev_cam_pos[2]}));
        const float tol = fmaxf(0.12f, hit_dist * 0.05f);
        if (fabsf(pcd - pdepth) < tol) return true;
    }
    return false;
}

// Checkerboard half rate (117-125): a pixel with valid history keeps its previous sample on the
// frames its slot is off.
__device__ __forceinline__ bool restir_skip(const arc_camera_uniforms& cam, uint32_t x, uint32_t y, bool prev_valid) {
    const uint32_t frame = __float_as_uint(cam.cam_up_frame[3]);
    const bool checker = (cam.quality_flags[3] & 0xFFu) <= 12u;
    const uint32_t cslot = (x & 1u) ^ ((y & 1u) << 1);
    return checker && prev_valid && (((cslot ^ (frame & 3u)) & 1u) != 0u);
}

// Sun shadow ray of a hit pixel (127-150): jittered towards the sun, from the hit lifted off the
// surface. False when the pixel traces none (surface facing away from the sun, or no sun).
__device__ __forceinline__ bool restir_sun_ray(const arc_camera_uniforms& cam, f3 hp, f3 n, float u1, float u2, f3* so,
                                               f3* js) {
    const f3 sun{cam.sun_dir_intensity[0], cam.sun_dir_intensity[1], cam.sun_dir_intensity[2]};
    if (!(fmaxf(dot3(n, sun), 0.0f) > 0.001f && cam.sun_dir_intensity[3] > 0.01f)) return false;
    const float j1 = u1 * 2.0f - 1.0f, j2 = u2 * 2.0f - 1.0f;
    const f3 up = fabsf(sun.y) < 0.9f ? f3{0.0f, 1.0f, 0.0f} : f3{1.0f, 0.0f, 0.0f};
    const f3 st = normalize3(cross3(up, sun));
    const f3 sb = cross3(sun, st);
    const float jr = cam.lod_settings[3];
    *js = normalize3(f3{sun.x + (st.x * j1 + sb.x * j2) * jr, sun.y + (st.y * j1 + sb.y * j2) * jr,
                        sun.z + (st.z * j1 + sb.z * j2) * jr});
    *so = add3(hp, mul3s(n, 0.08f));
    return true;
}

// Visibility along a sun ray: shadow_mode 0 traces the full ray (visible when it misses and leaves
// upwards or points down), other modes the any-hit shadow walk.
template <bool kFullRay>
__device__ __forceinline__ float restir_sun_trace(const World& w, const arc_camera_uniforms& cam, f3 so, f3 js) {
    const float smax = cam.ray_distances[3];
    if (kFullRay) {
        RayState s;
        HitInfo h;
        StepResult r = kMiss;
        if (ray_begin(s, cam, so, js, 0.0f, smax, 1u, true)) {
            do {
                r = ray_advance(s, w, cam, h);
            } while (r == kContinue);
        }
        return (r != kHit && (so.y + js.y * smax >= 32.0f || js.y < 0.0f)) ? 1.0f : 0.0f;
    }
    return shadow_vis(w, cam, so, js, smax);
}

// Sun shadow rays of the pass, as a pass of their own so that the kernel holds one traversal: every
// hit pixel that is not skipped this frame parks its visibility in its output reservoir's shadow
// word, which restir_gi_temporal_kernel reads back before it writes the reservoir. A block sets up
// the rays of its 16 x 8 pixels and appends them to shared memory (pixels without a ray, such as
// the sky, drop out), so the warps that trace are full.
template <bool kFullRay>
__global__ void __launch_bounds__(128) restir_sun_kernel(const RestirParams P, const __grid_constant__ arc_camera_uniforms cam) {
    __shared__ float s_ray[6][128];
    __shared__ uint32_t s_p[128];
    __shared__ uint32_t s_n;
    const uint32_t t = threadIdx.x, lane = t & 31u;
    if (t == 0u) s_n = 0u;
    __syncthreads();
    const uint32_t x = blockIdx.x * 16u + (t & 15u);
    const uint32_t y = blockIdx.y * 8u + (t >> 4);
    bool want = false;
    f3 so{0.0f, 0.0f, 0.0f}, js{0.0f, 1.0f, 0.0f};
    size_t p = 0;
    if (x < P.width && y < P.height) {
        p = (size_t)y * P.width + x;
        const uint2 gd = P.gdm[p], gn = P.gnm[p];
        const float hit_dist = __uint_as_float(gd.x);
        if (hit_dist < 1e4f) {
            const f3 rd = camera_dir(cam, x, y, P.width, P.height);
            const f3 hp = add3(f3{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]}, mul3s(rd, hit_dist));
            uint4 pr0, pr1;
            const bool prev_valid = restir_history(P, cam, x, y, gn.y, hp, hit_dist, &pr0, &pr1);
            if (!restir_skip(cam, x, y, prev_valid)) {
                float ox, oy;
                unpack2x16snorm(gn.x, &ox, &oy);
                const f3 n = oct_decode(ox, oy);
                float u1, u2;
                gradient_noise((float)x, (float)y, __float_as_uint(cam.cam_up_frame[3]), &u1, &u2);
                want = restir_sun_ray(cam, hp, n, u1, u2, &so, &js);
                if (!want) reinterpret_cast<float*>(&P.res_out[p])[7] = 0.0f;
            }
        }
    }
    const uint32_t m = __ballot_sync(0xFFFFFFFFu, want);
    uint32_t base = 0u;
    if (lane == 0u && m) base = atomicAdd(&s_n, (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, 0);
    if (want) {
        const uint32_t slot = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
        s_ray[0][slot] = so.x;
        s_ray[1][slot] = so.y;
        s_ray[2][slot] = so.z;
        s_ray[3][slot] = js.x;
        s_ray[4][slot] = js.y;
        s_ray[5][slot] = js.z;
        s_p[slot] = (uint32_t)p;
    }
    __syncthreads();
    if (t >= s_n) return;
    const f3 o{s_ray[0][t], s_ray[1][t], s_ray[2][t]}, d{s_ray[3][t], s_ray[4][t], s_ray[5][t]};
    reinterpret_cast<float*>(&P.res_out[s_p[t]])[7] = restir_sun_trace<kFullRay>(P.world, cam, o, d);
}

// kRigid: rigid bodies are in the frame, so the GI ray is traced again instead of read from its record.
template <bool kRigid>
__global__ void __launch_bounds__(128) restir_gi_temporal_kernel(const RestirParams P,
                                                                 const __grid_constant__ arc_camera_uniforms cam) {
    const uint32_t x = blockIdx.x * 16u + (threadIdx.x & 15u);
    const uint32_t y = blockIdx.y * 8u + (threadIdx.x >> 4);
    if (x >= P.width || y >= P.height) return;
    const World& w = P.world;
    const size_t p = (size_t)y * P.width + x;
    const uint2 gd = P.gdm[p], gn = P.gnm[p];
    f3 gi_o, gi_d;
    GiSetup g;
    if (!gi_setup_full(w, cam, x, y, P.width, P.height, gd.x, gn.x, &gi_o, &gi_d, &g)) {
        store_reservoir(&P.res_out[p], f3{0.0f, 0.0f, 0.0f}, 0u, 0u, 0u, 1e5f, 0u);
        return;
    }
    const f3 hp = g.hit_pos;
    const uint32_t frame = __float_as_uint(cam.cam_up_frame[3]);
    const f3 sun{cam.sun_dir_intensity[0], cam.sun_dir_intensity[1], cam.sun_dir_intensity[2]};
    const float sun_power = cam.sun_dir_intensity[3];

    uint4 pr0, pr1;
    const bool prev_valid = restir_history(P, cam, x, y, gn.y, hp, g.hit_dist, &pr0, &pr1);
    const uint32_t prev_nmf = pr0.w;

    // temporal average of the sun visibility (151-170); skipped pixels keep their previous sample
    float sun_vis, shadow_m = 1.0f, accum;
    const float ps_x = f16_value(pr1.w & 0xFFFFu), ps_y = f16_value(pr1.w >> 16);
    if (restir_skip(cam, x, y, prev_valid)) {
        accum = ps_x;
        shadow_m = fminf(ps_y, 16.0f);
        const f3 pn = unpack_res_normal(prev_nmf);
        const uint32_t nmf = pack_norm_m_flags(pn, (prev_nmf >> 16) & 0xFFu, ((prev_nmf >> 24) & 0x7Fu) + 1u,
                                               (prev_nmf & 0x80000000u) != 0u);
        store_reservoir(&P.res_out[p], f3{__uint_as_float(pr0.x), __uint_as_float(pr0.y), __uint_as_float(pr0.z)}, nmf,
                        pr1.x, pr1.y, g.hit_dist, pack2x16float(accum, shadow_m));
        return;
    }
    sun_vis = reinterpret_cast<const float*>(&P.res_out[p])[7];
    if (prev_valid) {
        const float psm = fminf(ps_y, 16.0f);
        shadow_m = psm + 1.0f;
        accum = __fdiv_rn(ps_x * psm + sun_vis, shadow_m);
    } else {
        accum = sun_vis;
        shadow_m = 1.0f;
    }

    // GI candidate (195-284): the frame's secondary hit from its record, or, with rigid bodies, the GI
    // ray traced again (world, then the bodies in front of its hit)
    bool gi_hit;
    uint32_t mat = 0u;
    float gd_m = 0.0f;
    f3 gpos{0.0f, 0.0f, 0.0f}, gnrm{0.0f, 1.0f, 0.0f}, lod{0.0f, 0.0f, 0.0f};
    if (kRigid) {
        HitInfo gh;
        gi_hit = trace_full(w, cam, gi_o, gi_d, cam.ray_distances[2], 2u, true, gh);
        const RigidHit rb = trace_rigid_bodies(w, cam, gi_o, gi_d, gi_hit ? gh.t_voxels * ARC_VOXEL_SIZE : cam.ray_distances[2]);
        if (rb.hit) {
            gi_hit = true;
            mat = rb.mat;
            gd_m = rb.t_voxels * ARC_VOXEL_SIZE;
            gpos = rb.pos;
            gnrm = rb.normal;
            const float4 ra = __ldg(&w.palette[2u * rb.mat]);
            lod = f3{ra.x, ra.y, ra.z};
        } else if (gi_hit) {
            mat = gh.mat;
            gd_m = gh.t_voxels * ARC_VOXEL_SIZE;
            gpos = gh.hit_pos_m;
            gnrm = gh.normal;
            lod = f3{__fdiv_rn((float)(gh.lod_payload & 0xFFu), 255.0f), __fdiv_rn((float)((gh.lod_payload >> 8) & 0xFFu), 255.0f),
                     __fdiv_rn((float)((gh.lod_payload >> 16) & 0xFFu), 255.0f)};
        }
    } else {
        const uint32_t* hr = reinterpret_cast<const uint32_t*>(&P.gi_hits[p]);
        const uint32_t w3 = hr[3];
        gi_hit = ((w3 >> 16) & ARC_HIT_FLAG_HIT) != 0u;
        if (gi_hit) {
            mat = (w3 >> 8) & 0xFFu;
            const uint32_t face = w3 & 0xFFu;
            const uint32_t shift = ((w3 >> 17) & 7u) << 1;
            gd_m = __uint_as_float(hr[4]);
            const float t = gd_m * ARC_VOXELS_PER_METER;
            const f3 vo = mul3s(gi_o, ARC_VOXELS_PER_METER);
            gpos = mul3s(add3(vo, mul3s(gi_d, t)), ARC_VOXEL_SIZE);
            gnrm = face_normal(face);
            const uint32_t payload = lod_payload_at(w, cam, hr[0], hr[1], hr[2], shift);
            lod = f3{__fdiv_rn((float)(payload & 0xFFu), 255.0f), __fdiv_rn((float)((payload >> 8) & 0xFFu), 255.0f),
                     __fdiv_rn((float)((payload >> 16) & 0xFFu), 255.0f)};
        }
    }
    f3 cand_pos = add3(hp, mul3s(gi_d, 500.0f));
    f3 cand_norm{-gi_d.x, -gi_d.y, -gi_d.z};
    bool cand_sky = true;
    f3 lo{0.0f, 0.0f, 0.0f};
    if (gi_hit) {
        cand_pos = gpos;
        cand_norm = gnrm;
        cand_sky = false;
        const float4 a = __ldg(&w.palette[2u * mat]);
        const float4 em = __ldg(&w.palette[2u * mat + 1u]);
        const f3 alb{mixf(a.x, lod.x, 0.55f), mixf(a.y, lod.y, 0.55f), mixf(a.z, lod.z, 0.55f)};
        const float att = __fdiv_rn(1.0f, (1.0f + gd_m * 0.06f) + (gd_m * gd_m) * 0.025f);
        const float gw = g.guided ? 0.55f : 1.0f;
        lo = f3{((em.x * att) * gw) * 1.0f, ((em.y * att) * gw) * 1.0f, ((em.z * att) * gw) * 1.0f};
        float4 rad;
        if (P.radiance) {
            rad = make_float4(P.radiance[3 * p], P.radiance[3 * p + 1], P.radiance[3 * p + 2], 1.0f);
        } else {
            float jx, jy;
            gradient_noise((float)x + 101.0f, (float)y + 57.0f, frame + 7919u, &jx, &jy);
            const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
            rad = sharc_query(P.sharc, gpos, gnrm, eye, jx * 2.0f - 1.0f, jy * 2.0f - 1.0f);
        }
        if (rad.w > 0.5f) {
            lo = f3{lo.x + rad.x, lo.y + rad.y, lo.z + rad.z};
        } else {
            const float b_ndl = fmaxf(dot3(gnrm, sun), 0.0f);
            f3 bs{0.0f, 0.0f, 0.0f};
            if (b_ndl > 0.001f && sun_power > 0.01f) {
                const float vis = shadow_vis(w, cam, add3(gpos, mul3s(gnrm, 0.10f)), sun, 32.0f);
                if (vis > 0.001f)
                    bs = f3{(((1.0f * sun_power) * b_ndl) * vis) * 0.55f, (((0.90f * sun_power) * b_ndl) * vis) * 0.55f,
                            (((0.75f * sun_power) * b_ndl) * vis) * 0.55f};
            }
            lo = f3{lo.x + alb.x * bs.x, lo.y + alb.y * bs.y, lo.z + alb.z * bs.z};
        }
        const float ao = clampf(__fdiv_rn(gd_m, 0.40f), 0.25f, 1.0f);
        lo = mul3s(lo, ao);
    } else if (gi_d.y > 0.15f && gi_o.y + gi_d.y * cam.ray_distances[2] >= 32.0f) {
        const float esc = clampf(__fdiv_rn(gi_d.y - 0.15f, 0.35f), 0.0f, 1.0f);
        const f3 sky = sky_radiance(gi_d, sun);
        lo = f3{lo.x + (sky.x * 0.45f) * esc, lo.y + (sky.y * 0.45f) * esc, lo.z + (sky.z * 0.45f) * esc};
    }
    const float peak = fmaxf(lo.x, fmaxf(lo.y, lo.z));
    if (peak > 0.001f) {
        const float d = 1.0f + peak * 0.16f;
        lo = f3{__fdiv_rn(lo.x, d), __fdiv_rn(lo.y, d), __fdiv_rn(lo.z, d)};
    }

    // temporal RIS (289-336)
    const f3 sn = g.smooth_n;
    const float cand_p_hat = luma3(lo) * __fdiv_rn(fmaxf(0.0f, dot3(sn, gi_d)), 3.14159265f);
    float w_sum = cand_p_hat > 1e-5f ? luma3(lo) : 0.0f;
    f3 sel_pos = cand_pos, sel_norm = cand_norm, sel_lo = lo;
    float sel_p_hat = cand_p_hat;
    uint32_t sel_age = 0u, m_total = 1u;
    bool sel_sky = cand_sky;
    if (prev_valid) {
        const uint32_t max_m = cam.target_voxel_info[3] > 0.5f ? 8u : 12u;
        const uint32_t pm = umin((prev_nmf >> 16) & 0xFFu, max_m);
        const f3 prev_lo{f16_value(pr1.x & 0xFFFFu), f16_value(pr1.x >> 16), f16_value(pr1.y & 0xFFFFu)};
        const float prev_w = f16_value(pr1.y >> 16);
        const f3 ppos{__uint_as_float(pr0.x), __uint_as_float(pr0.y), __uint_as_float(pr0.z)};
        const f3 tp = sub3(ppos, hp);
        const float d_prev = length3(tp);
        float prev_p_hat = 0.0f;
        if (d_prev > 1e-4f) {
            const f3 dp{__fdiv_rn(tp.x, d_prev), __fdiv_rn(tp.y, d_prev), __fdiv_rn(tp.z, d_prev)};
            prev_p_hat = luma3(prev_lo) * __fdiv_rn(fmaxf(0.0f, dot3(sn, dp)), 3.14159265f);
        }
        const uint32_t eff = umin(pm, max_m - 1u);
        const float prev_weight = prev_p_hat > 1e-5f ? (prev_p_hat * prev_w) * (float)eff : 0.0f;
        w_sum = w_sum + prev_weight;
        m_total = eff + 1u;
        uint32_t seed = pcg_hash(x + pcg_hash(y + pcg_hash(frame + 0x9E3779B9u)));
        if (rand01(seed) * w_sum < prev_weight) {
            sel_pos = ppos;
            sel_norm = unpack_res_normal(prev_nmf);
            sel_lo = prev_lo;
            sel_p_hat = prev_p_hat;
            sel_age = ((prev_nmf >> 24) & 0x7Fu) + 1u;
            sel_sky = (prev_nmf & 0x80000000u) != 0u;
        }
        const float bt = clampf(__fdiv_rn(prev_weight, fmaxf(w_sum, 1e-5f)), 0.0f, 1.0f);
        const f3 mixed{mixf(lo.x, prev_lo.x, bt), mixf(lo.y, prev_lo.y, bt), mixf(lo.z, prev_lo.z, bt)};
        const float wl = luma3(sel_lo), ml = luma3(mixed);
        if (ml > 1e-5f && wl > 1e-5f) sel_lo = mul3s(mixed, __fdiv_rn(wl, ml));
    }
    float final_w = 0.0f;
    if (sel_p_hat > 1e-5f && w_sum > 0.0f) final_w = clampf(__fdiv_rn(w_sum, (float)m_total * sel_p_hat), 0.0f, 12.0f);
    const float cr = clampf(sel_lo.x, 0.0f, 65500.0f), cg = clampf(sel_lo.y, 0.0f, 65500.0f), cb = clampf(sel_lo.z, 0.0f, 65500.0f);
    store_reservoir(&P.res_out[p], sel_pos, pack_norm_m_flags(sel_norm, m_total, sel_age, sel_sky), pack2x16float(cr, cg),
                    pack2x16float(cb, fminf(final_w, 65500.0f)), g.hit_dist, pack2x16float(accum, shadow_m));
}

}  // namespace arc

using arc::RestirParams;

static int restir_err(arc_ctx* c, int code, const char* msg) {
    c->err = msg;
    return code;
}

extern "C" int arc_restir_gi_temporal_dev(arc_ctx* c, uint32_t width, uint32_t height, const uint32_t* gdm,
                                          const uint32_t* gnm, const arc_hit_record* gi_hits,
                                          const arc_gi_reservoir* res_in, arc_gi_reservoir* res_out,
                                          const float* radiance) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    const uint32_t cw = c->cam.world_grid_dims[3] & 0xFFFFu, ch = c->cam.world_grid_dims[3] >> 16;
    if (width == 0 || height == 0 || width != cw || height != ch)
        return restir_err(c, ARC_E_INVALID_ARG, "frame size differs from camera world_grid_dims.w");
    if (!gdm || !gnm || !gi_hits || !res_in || !res_out) return restir_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (res_in == res_out) return restir_err(c, ARC_E_INVALID_ARG, "reservoir_in and reservoir_out must differ");
    if (!radiance && !c->d_sharc_resolved) return restir_err(c, ARC_E_INVALID_ARG, "no SHARC cache (arc_sharc_reset first)");
    RestirParams P;
    P.world = c->world();
    P.width = width;
    P.height = height;
    P.gdm = reinterpret_cast<const uint2*>(gdm);
    P.gnm = reinterpret_cast<const uint2*>(gnm);
    P.gi_hits = gi_hits;
    P.res_in = res_in;
    P.res_out = res_out;
    P.sharc = reinterpret_cast<const uint4*>(c->d_sharc_resolved);
    P.radiance = radiance;
    dim3 grid((width + 15u) / 16u, (height + 7u) / 8u);
    if (c->cam.quality_flags[2] == 0u)
        arc::restir_sun_kernel<true><<<grid, 128, 0, c->stream>>>(P, c->cam);
    else
        arc::restir_sun_kernel<false><<<grid, 128, 0, c->stream>>>(P, c->cam);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        c->err = std::string("restir_sun_kernel: ") + cudaGetErrorString(e);
        return ARC_E_CUDA;
    }
    if (c->n_bodies && ((c->cam.point_light_count[1] >> 16) & 0xFFFFu))
        arc::restir_gi_temporal_kernel<true><<<grid, 128, 0, c->stream>>>(P, c->cam);
    else
        arc::restir_gi_temporal_kernel<false><<<grid, 128, 0, c->stream>>>(P, c->cam);
    e = cudaGetLastError();
    if (e != cudaSuccess) {
        c->err = std::string("restir_gi_temporal_kernel: ") + cudaGetErrorString(e);
        return ARC_E_CUDA;
    }
    return ARC_OK;
}
