// arc_surface.cuh — primary-pass surface shading: underwater camera, translucent water (refraction
// + reflection ray), mirror chrome (reflection ray). shaders/primary_gbuffer.wgsl:163-295, helpers
// primary_gbuffer.wgsl:13-41 (eval_reflection_sky) and shaders/common/types.wgsl:352-468
// (hash22, gerstner_warp, eval_voronoi_caustic_rgb, eval_surface_water_normal, eval_water_caustics).
//
// The frame kernels keep only what the GI ray needs (the water hit's normal becomes (0, 1, 0)) and
// append every hit that takes a branch to a compacted list; surface_kernel shades the list after
// the frame kernel and rewrites the albedo bytes of those pixels. The arithmetic is the canonical
// one of arc_math.cuh (WGSL expressions evaluated left to right, pow with an integer exponent by
// powi, with a non-integer exponent by pow_canon, exp by exp_canon). Frames with rigid bodies shade
// their surface hits inline (frame_rigid_kernel), with the bodies in front of every surface ray.
#pragma once

#include "arc_rigid.cuh"
#include "arc_traverse.cuh"

namespace arc {

__device__ __forceinline__ bool surface_special(const arc_camera_uniforms& cam, uint32_t mat) {
    if ((cam.point_light_count[1] & 0xFFFFu) != 0u) return true;
    return mat == kMatWaterCrystal || mat == kMatMirrorChrome;
}

__device__ __forceinline__ f3 face_normal(uint32_t face) {
    // face_id: 0 +x, 1 -x, 2 +y, 3 -y, 4 +z, 5 -z
    const float s = (face & 1u) ? -1.0f : 1.0f;
    return f3{face < 2u ? s : 0.0f, (face >> 1) == 1u ? s : 0.0f, (face >> 1) == 2u ? s : 0.0f};
}

__device__ __forceinline__ f3 mix3(f3 a, f3 b, float t) { return f3{mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }

// eval_reflection_sky (primary_gbuffer.wgsl:13-41)
__device__ __forceinline__ f3 reflection_sky(f3 dir, f3 sun) {
    const float sun_elev = sun.y;
    const float day_t = clampf(__fdiv_rn(sun_elev + 0.05f, 0.30f), 0.0f, 1.0f);
    const float twilight_t = clampf(1.0f - __fdiv_rn(fabsf(sun_elev - 0.02f), 0.22f), 0.0f, 1.0f);
    const float zenith = clampf(dir.y, 0.0f, 1.0f);
    const float horizon = powi(1.0f - zenith, 3u);
    const f3 sky_z = mix3(f3{0.0015f, 0.0025f, 0.0055f}, f3{0.08f, 0.22f, 0.55f}, day_t);
    f3 sky_h = mix3(f3{0.0035f, 0.0065f, 0.0120f}, f3{0.38f, 0.50f, 0.68f}, day_t);
    sky_h = mix3(sky_h, f3{0.70f, 0.28f, 0.10f}, twilight_t * 0.78f);
    f3 sky = mix3(sky_z, sky_h, horizon);
    if (dir.y < 0.0f) {
        const f3 ground = mix3(f3{0.02f, 0.03f, 0.04f}, f3{0.12f, 0.15f, 0.18f}, day_t);
        sky = mix3(sky_h, ground, clampf(-dir.y * 3.0f, 0.0f, 1.0f));
    }
    const float sun_cos = fmaxf(dot3(dir, sun), 0.0f);
    if (sun_elev > -0.12f) {
        const float p = powi(sun_cos, 16u);
        const float m = fmaxf(day_t, twilight_t);
        sky.x = sky.x + ((0.90f * p) * 0.45f) * m;
        sky.y = sky.y + ((0.55f * p) * 0.45f) * m;
        sky.z = sky.z + ((0.25f * p) * 0.45f) * m;
    }
    return sky;
}

__device__ __forceinline__ float sin_canon(float x) {
    float s, c;
    sincos_canon(x, &s, &c);
    return s;
}
__device__ __forceinline__ float cos_canon(float x) {
    float s, c;
    sincos_canon(x, &s, &c);
    return c;
}

// eval_surface_water_normal (types.wgsl:426-433)
__device__ __forceinline__ f3 surface_water_normal(float x, float z, float t) {
    const float px = x * 1.8f, pz = z * 1.8f;
    const float w1 = t * 1.4f, w2 = t * 2.2f;
    const float wx = (sin_canon(pz * 2.2f + w1) * 0.024f + cos_canon(px * 3.4f - w2) * 0.016f) +
                     sin_canon((px * 5.6f + pz * 4.2f) + t * 3.0f) * 0.008f;
    const float wz = (cos_canon(px * 2.4f - w1 * 0.9f) * 0.024f + sin_canon(pz * 3.1f + w2 * 0.8f) * 0.016f) +
                     cos_canon((px * 4.1f - pz * 5.3f) - t * 2.7f) * 0.008f;
    return normalize3(f3{wx, 1.0f, wz});
}

// hash22 (types.wgsl:352-357)
__device__ __forceinline__ void hash22(float px, float py, float* hx, float* hy) {
    f3 p3{fractf(px * 443.897f), fractf(py * 441.423f), fractf(px * 437.195f)};
    const float d = dot3(p3, f3{p3.y + 19.19f, p3.z + 19.19f, p3.x + 19.19f});
    p3 = f3{p3.x + d, p3.y + d, p3.z + d};
    *hx = fractf(p3.x * p3.y);
    *hy = fractf(p3.y * p3.z);
}

// gerstner_warp (types.wgsl:361-372)
__device__ __forceinline__ void gerstner_warp(float px, float py, float t, float* ox, float* oy) {
    float qx = px, qy = py;
    const float w1 = t * 1.1f;
    qx = qx + (sin_canon(py * 1.6f + w1) * 0.26f + cos_canon(px * 1.2f - w1 * 0.7f) * 0.18f);
    qy = qy + (cos_canon(px * 1.7f - w1 * 0.8f) * 0.26f + sin_canon(py * 1.1f + w1 * 0.6f) * 0.18f);
    const float w2 = t * 1.8f;
    qx = qx + sin_canon((qx * 2.6f + qy * 1.8f) + w2) * 0.10f;
    qy = qy + cos_canon((qx * 1.5f - qy * 2.7f) - w2 * 1.1f) * 0.10f;
    *ox = qx;
    *oy = qy;
}

__device__ __forceinline__ void keep_two_smallest(float d, float& m1, float& m2) {
    if (d < m1) {
        m2 = m1;
        m1 = d;
    } else if (d < m2) {
        m2 = d;
    }
}

// eval_voronoi_caustic_rgb (types.wgsl:375-415)
static __device__ __noinline__ f3 voronoi_caustic_rgb(float u, float v, float dpx, float dpy, float t) {
    const float nx = floorf(u), ny = floorf(v);
    const float fx = u - nx, fy = v - ny;
    float m1_r = 1e4f, m2_r = 1e4f, m1_g = 1e4f, m2_g = 1e4f, m1_b = 1e4f, m2_b = 1e4f;
    for (int dy = -1; dy <= 1; ++dy) {
        for (int dx = -1; dx <= 1; ++dx) {
            const float ox = (float)dx, oy = (float)dy;
            float hx, hy;
            hash22(nx + ox, ny + oy, &hx, &hy);
            const float sx = sin_canon(t * 1.4f + hx * 6.28318f);
            const float sy = sin_canon(t * 1.2f + hy * 6.28318f);
            const float rx = (ox + (0.5f + 0.38f * sx)) - fx;
            const float ry = (oy + (0.5f + 0.38f * sy)) - fy;
            keep_two_smallest(rx * rx + ry * ry, m1_g, m2_g);
            const float ax = rx + dpx, ay = ry + dpy;
            keep_two_smallest(ax * ax + ay * ay, m1_r, m2_r);
            const float bx = rx - dpx, by = ry - dpy;
            keep_two_smallest(bx * bx + by * by, m1_b, m2_b);
        }
    }
    const float del_r = __fsqrt_rn(m2_r) - __fsqrt_rn(m1_r);
    const float del_g = __fsqrt_rn(m2_g) - __fsqrt_rn(m1_g);
    const float del_b = __fsqrt_rn(m2_b) - __fsqrt_rn(m1_b);
    const float fil_r = pow_canon(fmaxf(0.0f, 1.0f - del_r * 4.2f), 2.2f);
    const float fil_g = pow_canon(fmaxf(0.0f, 1.0f - del_g * 4.2f), 2.2f);
    const float fil_b = pow_canon(fmaxf(0.0f, 1.0f - del_b * 4.2f), 2.2f);
    const float glow = pow_canon(fmaxf(0.0f, 1.0f - __fsqrt_rn(m1_g) * 1.4f), 2.5f) * 0.25f;
    return f3{fil_r * 2.2f + glow, fil_g * 2.2f + glow, fil_b * 2.2f + glow};
}

// eval_water_caustics (types.wgsl:437-468)
static __device__ __noinline__ f3 water_caustics(f3 bed, float water_y, f3 water_n, f3 sun, float t) {
    const float day_factor = clampf(sun.y * 3.0f, 0.0f, 1.0f);
    if (day_factor <= 0.001f) return f3{1.0f, 1.0f, 1.0f};
    const f3 sn = normalize3(sun);
    const f3 sd{-sn.x, -sn.y, -sn.z};
    // refract(sun_down, (0, 1, 0), 0.75)
    const float eta = 0.75f;
    const float d = sd.y;
    const float k = 1.0f - (eta * eta) * (1.0f - d * d);
    f3 rd{0.0f, 0.0f, 0.0f};
    if (k >= 0.0f) {
        const float a = eta * d + __fsqrt_rn(k);
        rd = f3{eta * sd.x, eta * sd.y - a, eta * sd.z};
    }
    f3 l{0.0f, 1.0f, 0.0f};
    if (rd.y < -0.1f) {
        const f3 r = normalize3(rd);
        l = f3{-r.x, -r.y, -r.z};
    }
    const float depth = fmaxf(water_y - bed.y, 0.0f);
    const float proj = __fdiv_rn(depth, fmaxf(l.y, 0.1f));
    const float u = (bed.x + l.x * proj) * 2.0f, v = (bed.z + l.z * proj) * 2.0f;
    float u1, v1, u2, v2;
    gerstner_warp(u, v, t, &u1, &v1);
    gerstner_warp(u * 1.8f + 1.7f, v * 1.8f + -2.4f, t * 1.3f, &u2, &v2);
    const float dpx = clampf((u1 - u) * 0.08f, -0.025f, 0.025f);
    const float dpy = clampf((v1 - v) * 0.08f, -0.025f, 0.025f);
    const f3 c1 = voronoi_caustic_rgb(u1, v1, dpx, dpy, t);
    const f3 c2 = voronoi_caustic_rgb(u2, v2, dpx * 1.4f, dpy * 1.4f, t * 1.25f);
    const float focus = smoothstepf(0.05f, 0.6f, depth) * exp_canon(-depth * 0.06f);
    const float plane = clampf(__fdiv_rn(water_n.y - 0.2f, 0.8f), 0.0f, 1.0f);
    const float c1v[3] = {c1.x, c1.y, c1.z}, c2v[3] = {c2.x, c2.y, c2.z};
    float o[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float web = (c1v[i] * 0.65f + c2v[i] * 0.40f) + (c1v[i] * c2v[i]) * 0.45f;
        const float focused = mixf(1.0f, 0.25f + web * 1.4f, focus);
        o[i] = mixf(1.0f, mixf(1.0f, focused, plane), day_factor);
    }
    return f3{o[0], o[1], o[2]};
}

// clamp(albedo * (1 + rand * variation), 0.01, 1), rand from the voxel hash (primary_gbuffer.wgsl:152-162)
__device__ __forceinline__ f3 varied_albedo(const float4* __restrict__ palette, uint32_t mat, uint32_t hash, float weight) {
    const float4 a = __ldg(&palette[2u * mat]);
    const float4 e = __ldg(&palette[2u * mat + 1u]);
    const float r = (__fdiv_rn((float)(hash & 0xFFu), 255.0f) * 2.0f - 1.0f) * weight;
    const float kv = 1.0f + r * e.w;
    return f3{clampf(a.x * kv, 0.01f, 1.0f), clampf(a.y * kv, 0.01f, 1.0f), clampf(a.z * kv, 0.01f, 1.0f)};
}

// Full trace_world_64tree_from for the surface rays (one call site per use, not inlined).
static __device__ __noinline__ bool trace_full(const World& w, const arc_camera_uniforms& cam, f3 o, f3 d, float max_dist_m,
                                        uint32_t lod_bias, bool ignore_water, HitInfo& h) {
    RayState s;
    StepResult r = kMiss;
    if (ray_begin(s, cam, o, d, 0.0f, max_dist_m, lod_bias, ignore_water)) {
        do {
            r = ray_advance(s, w, cam, h);
        } while (r == kContinue);
    }
    if (r != kHit) hit_init_miss(h, o, d, max_dist_m);
    return r == kHit;
}

// Albedo of a primary hit after its branch (primary_gbuffer.wgsl:167-295): material, normal, voxel
// hash, hit distance and point of the hit, primary ray direction. With RB every surface ray is
// followed by the rigid bodies in front of its world hit, as the reference's trace_rigid_bodies calls.
template <bool RB>
__device__ __forceinline__ f3 surface_shade(const World& w, const arc_camera_uniforms& cam, f3 dir, uint32_t mat, f3 n,
                                            uint32_t hash, float hit_dist, f3 hp) {
    const f3 sun{cam.sun_dir_intensity[0], cam.sun_dir_intensity[1], cam.sun_dir_intensity[2]};
    const float sun_power = cam.sun_dir_intensity[3];
    const float t_sec = cam.cam_pos_time[3];
    HitInfo r;
    if ((cam.point_light_count[1] & 0xFFFFu) != 0u) {
        const f3 alb = varied_albedo(w.palette, mat, hash, 1.0f - smoothstepf(18.0f, 48.0f, hit_dist));
        const float water_y = fmaxf(11.25f, cam.cam_pos_time[1] + 0.35f);
        const f3 cau = water_caustics(hp, water_y, n, sun, t_sec);
        const float dd = fminf(hit_dist, 24.0f);
        return f3{mixf(0.02f, alb.x * cau.x, exp_canon(-0.16f * dd)), mixf(0.14f, alb.y * cau.y, exp_canon(-0.045f * dd)),
                  mixf(0.22f, alb.z * cau.z, exp_canon(-0.020f * dd))};
    }
    if (mat == kMatWaterCrystal) {
        const f3 wave = surface_water_normal(hp.x, hp.z, t_sec);
        const f3 refr_dir = normalize3(f3{dir.x - wave.x * 0.38f, dir.y - 0.0f * 0.38f, dir.z - wave.z * 0.38f});
        f3 water_col{0.03f, 0.16f, 0.24f};
        const f3 ro = add3(hp, mul3s(dir, 0.12f));
        bool refr_hit = trace_full(w, cam, ro, refr_dir, cam.ray_distances[0], 1u, true, r);
        if constexpr (RB) {
            const RigidHit rb =
                trace_rigid_bodies(w, cam, ro, refr_dir, refr_hit ? r.t_voxels * ARC_VOXEL_SIZE : cam.ray_distances[0]);
            if (rb.hit) {
                refr_hit = true;
                r.t_voxels = rb.t_voxels;
                r.hit_pos_m = rb.pos;
                r.normal = rb.normal;
                r.mat = rb.mat;
                r.voxel_hash = rb.hash;
            }
        }
        if (refr_hit) {
            const float4 em = __ldg(&w.palette[2u * r.mat + 1u]);
            const f3 bed0 = varied_albedo(w.palette, r.mat, r.voxel_hash, 1.0f);
            const f3 cau = water_caustics(r.hit_pos_m, hp.y, n, sun, t_sec);
            const f3 bed{bed0.x * cau.x + em.x * 0.5f, bed0.y * cau.y + em.y * 0.5f, bed0.z * cau.z + em.z * 0.5f};
            const float wd = length3(sub3(hp, r.hit_pos_m));
            water_col = f3{mixf(0.02f, bed.x, exp_canon(-0.32f * wd)), mixf(0.13f, bed.y, exp_canon(-0.095f * wd)),
                           mixf(0.20f, bed.z, exp_canon(-0.042f * wd))};
        }
        const float dn = dot3(wave, dir);
        const f3 refl_dir{dir.x - (2.0f * dn) * wave.x, dir.y - (2.0f * dn) * wave.y, dir.z - (2.0f * dn) * wave.z};
        const float n_dot_v = fmaxf(dot3(f3{-dir.x, -dir.y, -dir.z}, wave), 0.0f);
        const float fresnel = 0.03f + 0.42f * powi(clampf(1.0f - n_dot_v, 0.0f, 1.0f), 4u);
        const float day_factor = clampf(sun.y * 2.5f + 0.15f, 0.04f, 1.0f);
        f3 refl_col = reflection_sky(refl_dir, sun);
        const bool low = cam.quality_flags[2] != 0u || (cam.quality_flags[3] & 0xFFu) <= 12u;
        if (fresnel > (low ? 0.22f : 0.08f)) {
            const f3 o2{hp.x + 0.0f, hp.y + 0.08f, hp.z + 0.0f};
            bool refl_hit = trace_full(w, cam, o2, refl_dir, 36.0f, 2u, true, r);
            if constexpr (RB) {
                const RigidHit rb = trace_rigid_bodies(w, cam, o2, refl_dir, refl_hit ? r.t_voxels * ARC_VOXEL_SIZE : 36.0f);
                if (rb.hit) {
                    refl_hit = true;
                    r.mat = rb.mat;
                }
            }
            if (refl_hit) {
                const float4 a = __ldg(&w.palette[2u * r.mat]);
                const float4 em = __ldg(&w.palette[2u * r.mat + 1u]);
                refl_col = f3{a.x * day_factor + em.x * 0.35f, a.y * day_factor + em.y * 0.35f, a.z * day_factor + em.z * 0.35f};
            }
        }
        return f3{mixf(water_col.x, clampf(refl_col.x, 0.0f, 1.0f), fresnel),
                  mixf(water_col.y, clampf(refl_col.y, 0.0f, 1.0f), fresnel),
                  mixf(water_col.z, clampf(refl_col.z, 0.0f, 1.0f), fresnel)};
    }
    // mirror chrome
    const float dn = dot3(n, dir);
    const f3 refl_dir{dir.x - (2.0f * dn) * n.x, dir.y - (2.0f * dn) * n.y, dir.z - (2.0f * dn) * n.z};
    const f3 mo = add3(hp, mul3s(n, 0.04f));
    bool hit = trace_full(w, cam, mo, refl_dir, cam.ray_distances[1], 1u, false, r);
    f3 mirror_col = reflection_sky(refl_dir, sun);
    if (hit && r.mat == kMatMirrorChrome && r.t_voxels * ARC_VOXEL_SIZE < 0.12f) {
        HitInfo re;
        if (trace_full(w, cam, add3(r.hit_pos_m, mul3s(refl_dir, 0.08f)), refl_dir, cam.ray_distances[1], 1u, false, re)) r = re;
    }
    const bool self = hit && r.mat == kMatMirrorChrome && r.t_voxels * ARC_VOXEL_SIZE < 0.12f;
    if constexpr (RB) {
        const RigidHit rb = trace_rigid_bodies(w, cam, mo, refl_dir, (hit && !self) ? r.t_voxels * ARC_VOXEL_SIZE : cam.ray_distances[1]);
        if (rb.hit) {
            hit = true;
            r.t_voxels = rb.t_voxels;
            r.hit_pos_m = rb.pos;
            r.normal = rb.normal;
            r.mat = rb.mat;
            r.voxel_hash = rb.hash;
        }
    }
    if (hit && !self) {
        const f3 ra = varied_albedo(w.palette, r.mat, r.voxel_hash, 1.0f);
        const float4 em = __ldg(&w.palette[2u * r.mat + 1u]);
        const float ndl = fmaxf(dot3(r.normal, sun), 0.0f);
        const f3 sky = reflection_sky(r.normal, sun);
        f3 light{((((1.0f * sun_power) * ndl) * 0.75f) + sky.x * 0.45f) + 0.04f,
                 ((((0.92f * sun_power) * ndl) * 0.75f) + sky.y * 0.45f) + 0.04f,
                 ((((0.78f * sun_power) * ndl) * 0.75f) + sky.z * 0.45f) + 0.04f};
        const uint32_t n_pl = umin(cam.point_light_count[0], 8u);
        for (uint32_t l = 0; l < n_pl; ++l) {
            const float* pl = cam.point_light[l];
            const f3 to{pl[0] - r.hit_pos_m.x, pl[1] - r.hit_pos_m.y, pl[2] - r.hit_pos_m.z};
            const float d_pl = length3(to);
            if (d_pl > 0.01f && d_pl < 28.0f) {
                const f3 u{__fdiv_rn(to.x, d_pl), __fdiv_rn(to.y, d_pl), __fdiv_rn(to.z, d_pl)};
                const float pl_ndl = fmaxf(dot3(r.normal, u), 0.0f);
                const float atten = __fdiv_rn(pl[3] * 3.5f, 1.0f + (d_pl * d_pl) * 0.22f);
                light = f3{light.x + (1.0f * pl_ndl) * atten, light.y + (0.92f * pl_ndl) * atten,
                           light.z + (0.78f * pl_ndl) * atten};
            }
        }
        const float rx = ra.x * light.x + em.x * 0.85f, ry = ra.y * light.y + em.y * 0.85f, rz = ra.z * light.z + em.z * 0.85f;
        mirror_col = f3{__fdiv_rn(rx, 1.0f + rx * 0.45f), __fdiv_rn(ry, 1.0f + ry * 0.45f), __fdiv_rn(rz, 1.0f + rz * 0.45f)};
    }
    return f3{clampf(mirror_col.x * 0.93f, 0.01f, 1.0f), clampf(mirror_col.y * 0.96f, 0.01f, 1.0f),
              clampf(mirror_col.z * 1.0f, 0.01f, 1.0f)};
}

}  // namespace arc
