/*
 * orc_restir.c — ReSTIR GI temporal pass of the CPU oracle: the GI part of temporal_main
 * (shaders/lighting_restir_gi.wgsl:61-336) with helpers from shaders/common/types.wgsl:90-190.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA product and is never linked
 * into it.
 *
 * Per pixel, as the reference: reproject the history reservoir through the motion vector and
 * validate it by the distance to the previous camera; sun shadow ray with its temporal average
 * (checkerboard half rate in low-tap mode); one GI candidate (the GI ray is traced here, as the
 * reference does, with orc_trace) whose radiance is emission + the SHARC query at the secondary hit
 * (or the sun bounce with a shadow ray on a cache miss), or sky when the ray escapes; temporal RIS
 * against the history; the 32 B reservoir. The emissive-light ReSTIR DI half of the pass needs the
 * emissive light list, which this library does not build: with no emissive lights (the reference's
 * u_emissive.count = 0) its output is the empty DI reservoir and the GI part is what remains.
 * A radiance buffer may replace the SHARC query (a neural cache's prediction at the secondary hit).
 */
#include <string.h>

#include "orc.h"
#include "orc_math.h"

static float luma3(const float c[3]) { return (c[0] * 0.2126f + c[1] * 0.7152f) + c[2] * 0.0722f; }

/* rand_f32 (types.wgsl:264-267) */
static float rand01(uint32_t* seed) {
    *seed = orc_pcg_hash(*seed);
    return (float)(*seed) / 4294967295.0f;
}

/* pack_norm_m_flags (types.wgsl:132-136) */
static uint32_t pack_norm_m_flags(const float n[3], uint32_t m, uint32_t age, int is_sky) {
    float l1 = (fabsf(n[0]) + fabsf(n[1])) + fabsf(n[2]);
    float s = 1.0f / orc_max(l1, 1e-6f);
    float px = n[0] * s, py = n[1] * s;
    if (n[2] < 0.0f) {
        float wx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float wy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        px = wx;
        py = wy;
    }
    int32_t ix = (int32_t)rintf(px * 127.0f), iy = (int32_t)rintf(py * 127.0f);
    ix = ix < -128 ? -128 : (ix > 127 ? 127 : ix);
    iy = iy < -128 ? -128 : (iy > 127 ? 127 : iy);
    uint32_t ux = (uint32_t)(ix + 128), uy = (uint32_t)(iy + 128);
    return (ux & 0xFFu) | ((uy & 0xFFu) << 8) | ((orc_umin(m, 16u) & 0xFFu) << 16) | ((orc_umin(age, 127u) & 0x7Fu) << 24) |
           (is_sky ? 0x80000000u : 0u);
}

/* unpack_normal (types.wgsl:138-143): oct_decode of the two bytes */
static void unpack_normal(uint32_t nmf, float n[3]) {
    float ox = ((float)(nmf & 0xFFu) - 128.0f) / 127.0f;
    float oy = ((float)((nmf >> 8) & 0xFFu) - 128.0f) / 127.0f;
    float v[3] = {ox, oy, (1.0f - fabsf(ox)) - fabsf(oy)};
    if (v[2] < 0.0f) {
        float sx = ox >= 0.0f ? 1.0f : -1.0f, sy = oy >= 0.0f ? 1.0f : -1.0f;
        float wx = (1.0f - fabsf(oy)) * sx, wy = (1.0f - fabsf(ox)) * sy;
        v[0] = wx;
        v[1] = wy;
    }
    orc_normalize3(v, n);
}

static void unpack_half2(uint32_t p, float out[2]) {
    out[0] = orc_f16_to_f32(p & 0xFFFFu);
    out[1] = orc_f16_to_f32(p >> 16);
}

static void empty_reservoir(arc_gi_reservoir* r) {
    memset(r, 0, sizeof(*r));
    r->primary_depth = 1e5f;
}

static void restir_pixel(const orc_world* w, const arc_camera_uniforms* cam, const arc_sharc_slot* resolved,
                         const float* radiance, uint32_t x, uint32_t y, uint32_t W, uint32_t H, const uint32_t* gdm,
                         const uint32_t* gnm, const arc_gi_reservoir* res_in, arc_gi_reservoir* out) {
    size_t p = (size_t)y * W + x;
    orc_gi_ray g;
    uint32_t bytes = 0;
    if (!orc_gi_setup(w, cam, x, y, W, H, gdm[2 * p], gnm[2 * p], &g, &bytes)) {
        empty_reservoir(out);
        return;
    }
    const float hit_dist = g.hit_dist;
    const float* hit_pos = g.hit_pos;
    const float* normal = g.normal;
    float motion[2];
    unpack_half2(gnm[2 * p + 1], motion);
    float pu = ((float)x + 0.5f) / (float)W, pv = ((float)y + 0.5f) / (float)H;
    float prev_u = pu + motion[0], prev_v = pv + motion[1];
    uint32_t frame = orc_fbits(cam->cam_up_frame[3]);
    const float* sun = cam->sun_dir_intensity;
    const float sun_power = sun[3];
    float n_dot_l = orc_max(orc_dot3(normal, sun), 0.0f);

    /* history validation (lighting_restir_gi.wgsl:95-115) */
    int prev_valid = 0;
    arc_gi_reservoir prev;
    memset(&prev, 0, sizeof(prev));
    if (prev_u >= 0.0f && prev_u < 1.0f && prev_v >= 0.0f && prev_v < 1.0f) {
        uint32_t ppx = orc_uclamp(orc_f2u(prev_u * (float)W), 0u, W - 1u);
        uint32_t ppy = orc_uclamp(orc_f2u(prev_v * (float)H), 0u, H - 1u);
        prev = res_in[(size_t)ppy * W + ppx];
        uint32_t pm = (prev.norm_m_flags >> 16) & 0xFFu, page = (prev.norm_m_flags >> 24) & 0x7Fu;
        if (pm > 0u && page <= 12u && prev.primary_depth < 1e4f) {
            float dv[3] = {hit_pos[0] - cam->prev_cam_pos[0], hit_pos[1] - cam->prev_cam_pos[1], hit_pos[2] - cam->prev_cam_pos[2]};
            float prev_cam_dist = orc_length3(dv);
            float tol = orc_max(0.12f, hit_dist * 0.05f);
            if (fabsf(prev_cam_dist - prev.primary_depth) < tol) prev_valid = 1;
        }
    }

    /* checkerboard half rate (117-125) */
    uint32_t taps = cam->quality_flags[3] & 0xFFu;
    int checker = taps <= 12u;
    uint32_t cslot = (x & 1u) ^ ((y & 1u) << 1);
    int skip = checker && prev_valid && (((cslot ^ (frame & 3u)) & 1u) != 0u);

    /* sun shadow ray and its temporal average (127-170) */
    float sun_vis = 0.0f, shadow_m = 1.0f, accum = 0.0f;
    float ps[2];
    unpack_half2(prev.shadow_vis_m, ps);
    if (skip) {
        accum = ps[0];
        shadow_m = orc_min(ps[1], 16.0f);
    } else {
        if (n_dot_l > 0.001f && sun_power > 0.01f) {
            float j1 = g.xi[0] * 2.0f - 1.0f, j2 = g.xi[1] * 2.0f - 1.0f;
            float up[3] = {1.0f, 0.0f, 0.0f};
            if (fabsf(sun[1]) < 0.9f) {
                up[0] = 0.0f;
                up[1] = 1.0f;
            }
            float c[3], st[3], sb[3];
            orc_cross3(up, sun, c);
            orc_normalize3(c, st);
            orc_cross3(sun, st, sb);
            float jr = cam->lod_settings[3];
            float js_in[3], js[3], so[3];
            for (int i = 0; i < 3; ++i) js_in[i] = sun[i] + (st[i] * j1 + sb[i] * j2) * jr;
            orc_normalize3(js_in, js);
            for (int i = 0; i < 3; ++i) so[i] = hit_pos[i] + normal[i] * 0.08f;
            float smax = cam->ray_distances[3];
            if (cam->quality_flags[2] == 0u) {
                orc_trace_out tr;
                orc_trace(w, cam, so, js, 0.0f, smax, 1u, 1, &tr);
                if (!tr.hit) {
                    float end_y = so[1] + js[1] * smax;
                    if (end_y >= 32.0f || js[1] < 0.0f) sun_vis = 1.0f;
                }
            } else {
                sun_vis = orc_shadow_vis(w, cam, so, js, smax, &bytes);
            }
        }
        if (prev_valid) {
            float psm = orc_min(ps[1], 16.0f);
            shadow_m = psm + 1.0f;
            accum = (ps[0] * psm + sun_vis) / shadow_m;
        } else {
            accum = sun_vis;
            shadow_m = 1.0f;
        }
    }
    if (skip) {
        *out = prev;
        out->primary_depth = hit_dist;
        out->shadow_vis_m = orc_pack2x16float(accum, shadow_m);
        float pn[3];
        unpack_normal(prev.norm_m_flags, pn);
        uint32_t pm = (prev.norm_m_flags >> 16) & 0xFFu, page = (prev.norm_m_flags >> 24) & 0x7Fu;
        out->norm_m_flags = pack_norm_m_flags(pn, pm, page + 1u, (prev.norm_m_flags & 0x80000000u) != 0u);
        return;
    }

    /* GI candidate (195-284) */
    orc_trace_out gi;
    orc_trace_scene(w, cam, g.origin, g.dir, cam->ray_distances[2], 2u, 1, &gi);
    const float* bd = g.dir;
    float cand_pos[3], cand_norm[3], lo[3] = {0.0f, 0.0f, 0.0f};
    int cand_sky = 1;
    for (int i = 0; i < 3; ++i) {
        cand_pos[i] = hit_pos[i] + bd[i] * 500.0f;
        cand_norm[i] = -bd[i];
    }
    if (gi.hit) {
        memcpy(cand_pos, gi.hit_pos_m, sizeof(cand_pos));
        memcpy(cand_norm, gi.normal, sizeof(cand_norm));
        cand_sky = 0;
        const arc_material* m = &w->palette[gi.mat_id];
        float alb[3];
        for (int i = 0; i < 3; ++i) alb[i] = orc_mix(m->albedo_roughness[i], gi.lod_rgb[i], 0.55f);
        float gd = gi.t_voxels * ARC_VOXEL_SIZE;
        float att = 1.0f / ((1.0f + gd * 0.06f) + (gd * gd) * 0.025f);
        float gw = g.guided ? 0.55f : 1.0f;
        for (int i = 0; i < 3; ++i) lo[i] = lo[i] + ((m->emission_meta[i] * att) * gw) * 1.0f;
        float rad[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        if (radiance) {
            rad[0] = radiance[3 * p];
            rad[1] = radiance[3 * p + 1];
            rad[2] = radiance[3 * p + 2];
            rad[3] = 1.0f;
        } else {
            float jn[2];
            orc_ign((float)x + 101.0f, (float)y + 57.0f, frame + 7919u, jn);
            float jit[2] = {jn[0] * 2.0f - 1.0f, jn[1] * 2.0f - 1.0f};
            orc_sharc_query(resolved, gi.hit_pos_m, gi.normal, cam->cam_pos_time, jit, rad);
        }
        if (rad[3] > 0.5f) {
            for (int i = 0; i < 3; ++i) lo[i] = lo[i] + rad[i];
        } else {
            float b_ndl = orc_max(orc_dot3(gi.normal, sun), 0.0f);
            float bs[3] = {0.0f, 0.0f, 0.0f};
            if (b_ndl > 0.001f && sun_power > 0.01f) {
                float o2[3];
                for (int i = 0; i < 3; ++i) o2[i] = gi.hit_pos_m[i] + gi.normal[i] * 0.10f;
                float vis = orc_shadow_vis(w, cam, o2, sun, 32.0f, &bytes);
                if (vis > 0.001f) {
                    static const float warm[3] = {1.0f, 0.90f, 0.75f};
                    for (int i = 0; i < 3; ++i) bs[i] = (((warm[i] * sun_power) * b_ndl) * vis) * 0.55f;
                }
            }
            for (int i = 0; i < 3; ++i) lo[i] = lo[i] + alb[i] * bs[i];
        }
        float ao = orc_clamp(gd / 0.40f, 0.25f, 1.0f);
        for (int i = 0; i < 3; ++i) lo[i] = lo[i] * ao;
    } else {
        float end_y = g.origin[1] + bd[1] * cam->ray_distances[2];
        if (bd[1] > 0.15f && end_y >= 32.0f) {
            float esc = orc_clamp((bd[1] - 0.15f) / 0.35f, 0.0f, 1.0f);
            float sky[3];
            orc_sky_radiance(bd, sun, sky);
            for (int i = 0; i < 3; ++i) lo[i] = lo[i] + (sky[i] * 0.45f) * esc;
        }
    }
    float peak = orc_max(lo[0], orc_max(lo[1], lo[2]));
    if (peak > 0.001f)
        for (int i = 0; i < 3; ++i) lo[i] = lo[i] / (1.0f + peak * 0.16f);

    /* temporal RIS (289-336) */
    const float* sn = g.smooth_n;
    float cand_cos = orc_max(0.0f, orc_dot3(sn, bd));
    float cand_p_hat = luma3(lo) * (cand_cos / 3.14159265f);
    float cand_w = cand_p_hat > 1e-5f ? luma3(lo) : 0.0f;
    float w_sum = cand_w;
    float sel_pos[3], sel_norm[3], sel_lo[3];
    memcpy(sel_pos, cand_pos, sizeof(sel_pos));
    memcpy(sel_norm, cand_norm, sizeof(sel_norm));
    memcpy(sel_lo, lo, sizeof(sel_lo));
    float sel_p_hat = cand_p_hat;
    uint32_t sel_age = 0u, m_total = 1u;
    int sel_sky = cand_sky;
    if (prev_valid) {
        uint32_t max_m = cam->target_voxel_info[3] > 0.5f ? 8u : 12u;
        uint32_t pm = orc_umin((prev.norm_m_flags >> 16) & 0xFFu, max_m);
        float pw[2], prg[2];
        unpack_half2(prev.lo_b_w, pw);
        unpack_half2(prev.lo_rg, prg);
        float prev_lo[3] = {prg[0], prg[1], pw[0]};
        float prev_w = pw[1];
        float pn[3];
        unpack_normal(prev.norm_m_flags, pn);
        uint32_t page = (prev.norm_m_flags >> 24) & 0x7Fu;
        int psky = (prev.norm_m_flags & 0x80000000u) != 0u;
        float tp[3] = {prev.sample_pos[0] - hit_pos[0], prev.sample_pos[1] - hit_pos[1], prev.sample_pos[2] - hit_pos[2]};
        float d_prev = orc_length3(tp);
        float prev_p_hat = 0.0f;
        if (d_prev > 1e-4f) {
            float dp[3] = {tp[0] / d_prev, tp[1] / d_prev, tp[2] / d_prev};
            float pc = orc_max(0.0f, orc_dot3(sn, dp));
            prev_p_hat = luma3(prev_lo) * (pc / 3.14159265f);
        }
        uint32_t eff = orc_umin(pm, max_m - 1u);
        float prev_weight = prev_p_hat > 1e-5f ? (prev_p_hat * prev_w) * (float)eff : 0.0f;
        w_sum = w_sum + prev_weight;
        m_total = eff + 1u;
        uint32_t seed = orc_pcg_hash(x + orc_pcg_hash(y + orc_pcg_hash(frame + 0x9E3779B9u)));
        int pick = rand01(&seed) * w_sum < prev_weight;
        if (pick) {
            memcpy(sel_pos, prev.sample_pos, sizeof(sel_pos));
            memcpy(sel_norm, pn, sizeof(sel_norm));
            memcpy(sel_lo, prev_lo, sizeof(sel_lo));
            sel_p_hat = prev_p_hat;
            sel_age = page + 1u;
            sel_sky = psky;
        }
        float bt = orc_clamp(prev_weight / orc_max(w_sum, 1e-5f), 0.0f, 1.0f);
        float mixed[3];
        for (int i = 0; i < 3; ++i) mixed[i] = orc_mix(lo[i], prev_lo[i], bt);
        float wl = luma3(sel_lo), ml = luma3(mixed);
        if (ml > 1e-5f && wl > 1e-5f)
            for (int i = 0; i < 3; ++i) sel_lo[i] = mixed[i] * (wl / ml);
    }
    float final_w = 0.0f;
    if (sel_p_hat > 1e-5f && w_sum > 0.0f) final_w = orc_clamp(w_sum / ((float)m_total * sel_p_hat), 0.0f, 12.0f);
    float cl[3];
    for (int i = 0; i < 3; ++i) cl[i] = orc_clamp(sel_lo[i], 0.0f, 65500.0f);
    memcpy(out->sample_pos, sel_pos, sizeof(sel_pos));
    out->norm_m_flags = pack_norm_m_flags(sel_norm, m_total, sel_age, sel_sky);
    out->lo_rg = orc_pack2x16float(cl[0], cl[1]);
    out->lo_b_w = orc_pack2x16float(cl[2], orc_min(final_w, 65500.0f));
    out->primary_depth = hit_dist;
    out->shadow_vis_m = orc_pack2x16float(accum, shadow_m);
}

void orc_restir_gi_temporal(const orc_world* w, const arc_camera_uniforms* cam, const arc_sharc_slot* resolved,
                            const float* radiance, const uint32_t* gdm, const uint32_t* gnm, const arc_gi_reservoir* res_in,
                            arc_gi_reservoir* res_out, int threads) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    int64_t n = (int64_t)W * H;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < n; ++i)
        restir_pixel(w, cam, resolved, radiance, (uint32_t)(i % W), (uint32_t)(i / W), W, H, gdm, gnm, res_in, &res_out[i]);
}
