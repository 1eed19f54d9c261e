/*
 * orc_surface.c — primary-pass surface shading branches of the CPU oracle: the underwater camera,
 * translucent water with a refraction and a reflection ray, and mirror chrome with a reflection
 * ray (shaders/primary_gbuffer.wgsl:163-295, helpers shaders/primary_gbuffer.wgsl:13-41 and
 * shaders/common/types.wgsl:352-468).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA product and is never linked
 * into it.
 *
 * Arithmetic is the oracle's canonical one (orc_math.h): expressions are evaluated left to right
 * as written in WGSL, vector operations component by component, pow with an integer exponent by
 * orc_powi and with a non-integer exponent by orc_pow, exp by orc_exp. Every surface ray is followed
 * by the rigid bodies in front of its world hit, as the reference's trace_rigid_bodies calls.
 */
#include <string.h>

#include "orc.h"
#include "orc_math.h"

#define MAT_WATER_CRYSTAL 18u
#define MAT_MIRROR_CHROME 28u

static void mix3(const float a[3], const float b[3], float t, float out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = orc_mix(a[i], b[i], t);
}

/* eval_reflection_sky (primary_gbuffer.wgsl:13-41) */
static void reflection_sky(const float dir[3], const float sun_dir[3], float out[3]) {
    float sun_elev = sun_dir[1];
    float day_t = orc_clamp((sun_elev + 0.05f) / 0.30f, 0.0f, 1.0f);
    float twilight_t = orc_clamp(1.0f - fabsf(sun_elev - 0.02f) / 0.22f, 0.0f, 1.0f);
    float zenith = orc_clamp(dir[1], 0.0f, 1.0f);
    float horizon = orc_powi(1.0f - zenith, 3u);
    static const float day_zenith[3] = {0.08f, 0.22f, 0.55f};
    static const float day_horizon[3] = {0.38f, 0.50f, 0.68f};
    static const float night_zenith[3] = {0.0015f, 0.0025f, 0.0055f};
    static const float night_horizon[3] = {0.0035f, 0.0065f, 0.0120f};
    static const float dusk[3] = {0.70f, 0.28f, 0.10f};
    float sky_z[3], sky_h[3], sky[3];
    mix3(night_zenith, day_zenith, day_t, sky_z);
    mix3(night_horizon, day_horizon, day_t, sky_h);
    mix3(sky_h, dusk, twilight_t * 0.78f, sky_h);
    mix3(sky_z, sky_h, horizon, sky);
    if (dir[1] < 0.0f) {
        static const float g0[3] = {0.02f, 0.03f, 0.04f};
        static const float g1[3] = {0.12f, 0.15f, 0.18f};
        float ground[3];
        mix3(g0, g1, day_t, ground);
        mix3(sky_h, ground, orc_clamp(-dir[1] * 3.0f, 0.0f, 1.0f), sky);
    }
    float sun_cos = orc_max(orc_dot3(dir, sun_dir), 0.0f);
    if (sun_elev > -0.12f) {
        static const float tint[3] = {0.90f, 0.55f, 0.25f};
        float p = orc_powi(sun_cos, 16u);
        float m = orc_max(day_t, twilight_t);
        for (int i = 0; i < 3; ++i) sky[i] = sky[i] + ((tint[i] * p) * 0.45f) * m;
    }
    memcpy(out, sky, sizeof(sky));
}

/* eval_surface_water_normal (types.wgsl:426-433) */
static void surface_water_normal(float x, float z, float t, float out[3]) {
    float px = x * 1.8f, pz = z * 1.8f;
    float w1 = t * 1.4f, w2 = t * 2.2f;
    float s, c, a0, a1, a2, b0, b1, b2;
    orc_sincos(pz * 2.2f + w1, &a0, &c);
    orc_sincos(px * 3.4f - w2, &s, &a1);
    orc_sincos((px * 5.6f + pz * 4.2f) + t * 3.0f, &a2, &c);
    orc_sincos(px * 2.4f - w1 * 0.9f, &s, &b0);
    orc_sincos(pz * 3.1f + w2 * 0.8f, &b1, &c);
    orc_sincos((px * 4.1f - pz * 5.3f) - t * 2.7f, &s, &b2);
    float wx = (a0 * 0.024f + a1 * 0.016f) + a2 * 0.008f;
    float wz = (b0 * 0.024f + b1 * 0.016f) + b2 * 0.008f;
    float v[3] = {wx, 1.0f, wz};
    orc_normalize3(v, out);
}

/* hash22 (types.wgsl:352-357) */
static void hash22(float px, float py, float out[2]) {
    float p3[3] = {orc_fract(px * 443.897f), orc_fract(py * 441.423f), orc_fract(px * 437.195f)};
    float q[3] = {p3[1] + 19.19f, p3[2] + 19.19f, p3[0] + 19.19f};
    float d = orc_dot3(p3, q);
    for (int i = 0; i < 3; ++i) p3[i] = p3[i] + d;
    out[0] = orc_fract(p3[0] * p3[1]);
    out[1] = orc_fract(p3[1] * p3[2]);
}

/* gerstner_warp (types.wgsl:361-372) */
static void gerstner_warp(float px, float py, float t, float out[2]) {
    float qx = px, qy = py;
    float w1 = t * 1.1f;
    float s0, c0, s1, c1;
    orc_sincos(py * 1.6f + w1, &s0, &c0);
    orc_sincos(px * 1.2f - w1 * 0.7f, &s1, &c1);
    qx = qx + (s0 * 0.26f + c1 * 0.18f);
    orc_sincos(px * 1.7f - w1 * 0.8f, &s0, &c0);
    orc_sincos(py * 1.1f + w1 * 0.6f, &s1, &c1);
    qy = qy + (c0 * 0.26f + s1 * 0.18f);
    float w2 = t * 1.8f;
    orc_sincos((qx * 2.6f + qy * 1.8f) + w2, &s0, &c0);
    qx = qx + s0 * 0.10f;
    orc_sincos((qx * 1.5f - qy * 2.7f) - w2 * 1.1f, &s0, &c0);
    qy = qy + c0 * 0.10f;
    out[0] = qx;
    out[1] = qy;
}

static void keep_two_smallest(float d, float* m1, float* m2) {
    if (d < *m1) {
        *m2 = *m1;
        *m1 = d;
    } else if (d < *m2) {
        *m2 = d;
    }
}

/* eval_voronoi_caustic_rgb (types.wgsl:375-415) */
static void voronoi_caustic_rgb(const float uv[2], const float disp[2], float t, float out[3]) {
    float nx = floorf(uv[0]), ny = floorf(uv[1]);
    float fx = uv[0] - nx, fy = uv[1] - ny;
    float m1_r = 1e4f, m2_r = 1e4f, m1_g = 1e4f, m2_g = 1e4f, m1_b = 1e4f, m2_b = 1e4f;
    for (int dy = -1; dy <= 1; ++dy) {
        for (int dx = -1; dx <= 1; ++dx) {
            float ox = (float)dx, oy = (float)dy;
            float h[2];
            hash22(nx + ox, ny + oy, h);
            float sx, sy, c;
            orc_sincos(t * 1.4f + h[0] * 6.28318f, &sx, &c);
            orc_sincos(t * 1.2f + h[1] * 6.28318f, &sy, &c);
            float rx = (ox + (0.5f + 0.38f * sx)) - fx;
            float ry = (oy + (0.5f + 0.38f * sy)) - fy;
            keep_two_smallest(rx * rx + ry * ry, &m1_g, &m2_g);
            float ax = rx + disp[0], ay = ry + disp[1];
            keep_two_smallest(ax * ax + ay * ay, &m1_r, &m2_r);
            float bx = rx - disp[0], by = ry - disp[1];
            keep_two_smallest(bx * bx + by * by, &m1_b, &m2_b);
        }
    }
    float del_r = sqrtf(m2_r) - sqrtf(m1_r);
    float del_g = sqrtf(m2_g) - sqrtf(m1_g);
    float del_b = sqrtf(m2_b) - sqrtf(m1_b);
    float fil_r = orc_pow(orc_max(0.0f, 1.0f - del_r * 4.2f), 2.2f);
    float fil_g = orc_pow(orc_max(0.0f, 1.0f - del_g * 4.2f), 2.2f);
    float fil_b = orc_pow(orc_max(0.0f, 1.0f - del_b * 4.2f), 2.2f);
    float glow = orc_pow(orc_max(0.0f, 1.0f - sqrtf(m1_g) * 1.4f), 2.5f) * 0.25f;
    out[0] = fil_r * 2.2f + glow;
    out[1] = fil_g * 2.2f + glow;
    out[2] = fil_b * 2.2f + glow;
}

/* eval_water_caustics (types.wgsl:437-468) */
static void water_caustics(const float bed[3], float water_y, const float water_n[3], const float sun_dir[3], float t,
                           float out[3]) {
    float day_factor = orc_clamp(sun_dir[1] * 3.0f, 0.0f, 1.0f);
    if (day_factor <= 0.001f) {
        out[0] = out[1] = out[2] = 1.0f;
        return;
    }
    float sn[3], sun_down[3];
    orc_normalize3(sun_dir, sn);
    for (int i = 0; i < 3; ++i) sun_down[i] = -sn[i];
    /* refract(I, N = (0,1,0), eta = 0.75) */
    const float eta = 0.75f;
    float d = sun_down[1];
    float k = 1.0f - (eta * eta) * (1.0f - d * d);
    float refr_down[3] = {0.0f, 0.0f, 0.0f};
    if (k >= 0.0f) {
        float a = eta * d + sqrtf(k);
        refr_down[0] = eta * sun_down[0];
        refr_down[1] = eta * sun_down[1] - a;
        refr_down[2] = eta * sun_down[2];
    }
    float l_refr[3] = {0.0f, 1.0f, 0.0f};
    if (refr_down[1] < -0.1f) {
        float r[3];
        orc_normalize3(refr_down, r);
        for (int i = 0; i < 3; ++i) l_refr[i] = -r[i];
    }
    float depth = orc_max(water_y - bed[1], 0.0f);
    float proj = depth / orc_max(l_refr[1], 0.1f);
    float hx = bed[0] + l_refr[0] * proj, hz = bed[2] + l_refr[2] * proj;
    float uv[2] = {hx * 2.0f, hz * 2.0f};
    float wu1[2], wu2[2];
    gerstner_warp(uv[0], uv[1], t, wu1);
    gerstner_warp(uv[0] * 1.8f + 1.7f, uv[1] * 1.8f + -2.4f, t * 1.3f, wu2);
    float disp[2] = {orc_clamp((wu1[0] - uv[0]) * 0.08f, -0.025f, 0.025f),
                     orc_clamp((wu1[1] - uv[1]) * 0.08f, -0.025f, 0.025f)};
    float disp2[2] = {disp[0] * 1.4f, disp[1] * 1.4f};
    float c1[3], c2[3];
    voronoi_caustic_rgb(wu1, disp, t, c1);
    voronoi_caustic_rgb(wu2, disp2, t * 1.25f, c2);
    float focus = orc_smoothstep(0.05f, 0.6f, depth) * orc_exp(-depth * 0.06f);
    float plane = orc_clamp((water_n[1] - 0.2f) / 0.8f, 0.0f, 1.0f);
    for (int i = 0; i < 3; ++i) {
        float web = (c1[i] * 0.65f + c2[i] * 0.40f) + (c1[i] * c2[i]) * 0.45f;
        float focused = orc_mix(1.0f, 0.25f + web * 1.4f, focus);
        float cp = orc_mix(1.0f, focused, plane);
        out[i] = orc_mix(1.0f, cp, day_factor);
    }
}

/* clamp(albedo * (1 + rand * variation), 0.01, 1) with rand from the voxel hash (primary_gbuffer.wgsl:152-162) */
static void varied_albedo(const arc_material* m, uint32_t hash, float weight, float out[3]) {
    float r = (((float)(hash & 0xFFu) / 255.0f) * 2.0f - 1.0f) * weight;
    for (int i = 0; i < 3; ++i) out[i] = orc_clamp(m->albedo_roughness[i] * (1.0f + r * m->emission_meta[3]), 0.01f, 1.0f);
}

/* trace_rigid_bodies in front of a surface ray's world hit (1 when a body was hit) */
static int rigid_in_front(const orc_world* w, const arc_camera_uniforms* cam, const float o[3], const float d[3],
                          float max_dist_m, orc_rigid_out* rb) {
    if (orc_rigid_count(w, cam) == 0u) return 0;
    orc_trace_rigid_bodies(w, cam, o, d, max_dist_m, rb);
    return rb->hit != 0u;
}

int orc_surface_special(const arc_camera_uniforms* cam, uint32_t mat) {
    if ((cam->point_light_count[1] & 0xFFFFu) != 0u) return 1;
    return mat == MAT_WATER_CRYSTAL || mat == MAT_MIRROR_CHROME;
}

void orc_surface_shade(const orc_world* w, const arc_camera_uniforms* cam, const float ray_dir[3],
                       const orc_trace_out* p, float albedo[3], float normal[3], uint32_t* bytes) {
    const float* sun = cam->sun_dir_intensity;
    const float t_sec = cam->cam_pos_time[3];
    const float sun_power = sun[3];
    const float* hp = p->hit_pos_m;
    float hit_dist = p->t_voxels * ARC_VOXEL_SIZE;
    orc_trace_out r;
    if ((cam->point_light_count[1] & 0xFFFFu) != 0u) {
        /* primary_gbuffer.wgsl:167-173 */
        float water_y = orc_max(11.25f, cam->cam_pos_time[1] + 0.35f);
        float cau[3];
        water_caustics(hp, water_y, normal, sun, t_sec, cau);
        static const float absorb[3] = {-0.16f, -0.045f, -0.020f};
        static const float deep[3] = {0.02f, 0.14f, 0.22f};
        float dd = orc_min(hit_dist, 24.0f);
        for (int i = 0; i < 3; ++i) albedo[i] = orc_mix(deep[i], albedo[i] * cau[i], orc_exp(absorb[i] * dd));
    } else if (p->mat_id == MAT_WATER_CRYSTAL) {
        /* primary_gbuffer.wgsl:174-231 */
        float wave[3];
        surface_water_normal(hp[0], hp[2], t_sec, wave);
        float rv[3] = {ray_dir[0] - wave[0] * 0.38f, ray_dir[1] - 0.0f * 0.38f, ray_dir[2] - wave[2] * 0.38f};
        float refr_dir[3], ro[3];
        orc_normalize3(rv, refr_dir);
        for (int i = 0; i < 3; ++i) ro[i] = hp[i] + ray_dir[i] * 0.12f;
        orc_trace(w, cam, ro, refr_dir, 0.0f, cam->ray_distances[0], 1u, 1, &r);
        *bytes += r.bytes;
        orc_rigid_out rb;
        if (rigid_in_front(w, cam, ro, refr_dir, r.hit ? r.t_voxels * ARC_VOXEL_SIZE : cam->ray_distances[0], &rb)) {
            r.hit = 1;
            r.t_voxels = rb.t_voxels;
            memcpy(r.hit_pos_m, rb.hit_pos_m, sizeof(r.hit_pos_m));
            memcpy(r.normal, rb.normal, sizeof(r.normal));
            r.mat_id = rb.mat_id;
            r.voxel_hash = rb.voxel_hash;
        }
        float water_col[3] = {0.03f, 0.16f, 0.24f};
        if (r.hit) {
            const arc_material* bm = &w->palette[r.mat_id];
            float bed[3], cau[3];
            varied_albedo(bm, r.voxel_hash, 1.0f, bed);
            water_caustics(r.hit_pos_m, hp[1], p->normal, sun, t_sec, cau);
            for (int i = 0; i < 3; ++i) bed[i] = bed[i] * cau[i] + bm->emission_meta[i] * 0.5f;
            float dv[3] = {hp[0] - r.hit_pos_m[0], hp[1] - r.hit_pos_m[1], hp[2] - r.hit_pos_m[2]};
            float wd = orc_length3(dv);
            static const float absorb[3] = {-0.32f, -0.095f, -0.042f};
            static const float scatter[3] = {0.02f, 0.13f, 0.20f};
            for (int i = 0; i < 3; ++i) water_col[i] = orc_mix(scatter[i], bed[i], orc_exp(absorb[i] * wd));
        }
        float dn = orc_dot3(wave, ray_dir);
        float refl_dir[3];
        for (int i = 0; i < 3; ++i) refl_dir[i] = ray_dir[i] - (2.0f * dn) * wave[i];
        float neg[3] = {-ray_dir[0], -ray_dir[1], -ray_dir[2]};
        float n_dot_v = orc_max(orc_dot3(neg, wave), 0.0f);
        float fresnel = 0.03f + 0.42f * orc_powi(orc_clamp(1.0f - n_dot_v, 0.0f, 1.0f), 4u);
        float day_factor = orc_clamp(sun[1] * 2.5f + 0.15f, 0.04f, 1.0f);
        float refl_col[3];
        reflection_sky(refl_dir, sun, refl_col);
        int low = cam->quality_flags[2] != 0u || (cam->quality_flags[3] & 0xFFu) <= 12u;
        float thresh = low ? 0.22f : 0.08f;
        if (fresnel > thresh) {
            float o2[3] = {hp[0] + 0.0f, hp[1] + 0.08f, hp[2] + 0.0f};
            orc_trace(w, cam, o2, refl_dir, 0.0f, 36.0f, 2u, 1, &r);
            *bytes += r.bytes;
            orc_rigid_out rb2;
            if (rigid_in_front(w, cam, o2, refl_dir, r.hit ? r.t_voxels * ARC_VOXEL_SIZE : 36.0f, &rb2)) {
                r.hit = 1;
                r.mat_id = rb2.mat_id;
            }
            if (r.hit) {
                const arc_material* rm = &w->palette[r.mat_id];
                for (int i = 0; i < 3; ++i) refl_col[i] = rm->albedo_roughness[i] * day_factor + rm->emission_meta[i] * 0.35f;
            }
        }
        for (int i = 0; i < 3; ++i) albedo[i] = orc_mix(water_col[i], orc_clamp(refl_col[i], 0.0f, 1.0f), fresnel);
        normal[0] = 0.0f;
        normal[1] = 1.0f;
        normal[2] = 0.0f;
    } else if (p->mat_id == MAT_MIRROR_CHROME) {
        /* primary_gbuffer.wgsl:232-295 */
        const float* n = p->normal;
        float dn = orc_dot3(n, ray_dir);
        float refl_dir[3], ro[3];
        for (int i = 0; i < 3; ++i) refl_dir[i] = ray_dir[i] - (2.0f * dn) * n[i];
        for (int i = 0; i < 3; ++i) ro[i] = hp[i] + n[i] * 0.04f;
        orc_trace(w, cam, ro, refl_dir, 0.0f, cam->ray_distances[1], 1u, 0, &r);
        *bytes += r.bytes;
        float mirror_col[3];
        reflection_sky(refl_dir, sun, mirror_col);
        if (r.hit && r.mat_id == MAT_MIRROR_CHROME && r.t_voxels * ARC_VOXEL_SIZE < 0.12f) {
            float o2[3];
            for (int i = 0; i < 3; ++i) o2[i] = r.hit_pos_m[i] + refl_dir[i] * 0.08f;
            orc_trace_out re;
            orc_trace(w, cam, o2, refl_dir, 0.0f, cam->ray_distances[1], 1u, 0, &re);
            *bytes += re.bytes;
            if (re.hit) r = re;
        }
        int self = r.hit && r.mat_id == MAT_MIRROR_CHROME && r.t_voxels * ARC_VOXEL_SIZE < 0.12f;
        orc_rigid_out rb;
        if (rigid_in_front(w, cam, ro, refl_dir, (r.hit && !self) ? r.t_voxels * ARC_VOXEL_SIZE : cam->ray_distances[1], &rb)) {
            r.hit = 1;
            r.t_voxels = rb.t_voxels;
            memcpy(r.hit_pos_m, rb.hit_pos_m, sizeof(r.hit_pos_m));
            memcpy(r.normal, rb.normal, sizeof(r.normal));
            r.mat_id = rb.mat_id;
            r.voxel_hash = rb.voxel_hash;
        }
        if (r.hit && !self) {
            const arc_material* rm = &w->palette[r.mat_id];
            float ra[3], sky[3], light[3];
            varied_albedo(rm, r.voxel_hash, 1.0f, ra);
            float ndl = orc_max(orc_dot3(r.normal, sun), 0.0f);
            reflection_sky(r.normal, sun, sky);
            static const float warm[3] = {1.0f, 0.92f, 0.78f};
            for (int i = 0; i < 3; ++i) light[i] = ((((warm[i] * sun_power) * ndl) * 0.75f) + sky[i] * 0.45f) + 0.04f;
            uint32_t n_pl = orc_umin(cam->point_light_count[0], 8u);
            for (uint32_t l = 0; l < n_pl; ++l) {
                const float* pl = cam->point_light[l];
                float to[3] = {pl[0] - r.hit_pos_m[0], pl[1] - r.hit_pos_m[1], pl[2] - r.hit_pos_m[2]};
                float d_pl = orc_length3(to);
                if (d_pl > 0.01f && d_pl < 28.0f) {
                    float u[3] = {to[0] / d_pl, to[1] / d_pl, to[2] / d_pl};
                    float pl_ndl = orc_max(orc_dot3(r.normal, u), 0.0f);
                    float atten = (pl[3] * 3.5f) / (1.0f + (d_pl * d_pl) * 0.22f);
                    for (int i = 0; i < 3; ++i) light[i] = light[i] + (warm[i] * pl_ndl) * atten;
                }
            }
            for (int i = 0; i < 3; ++i) {
                float raw = ra[i] * light[i] + rm->emission_meta[i] * 0.85f;
                mirror_col[i] = raw / (1.0f + raw * 0.45f);
            }
        }
        static const float tint[3] = {0.93f, 0.96f, 1.0f};
        for (int i = 0; i < 3; ++i) albedo[i] = orc_clamp(mirror_col[i] * tint[i], 0.01f, 1.0f);
    }
}
