/*
 * orc_sharc.c — oracle restatement of the SHARC voxel-surfel radiance cache:
 *   key hashing / packing        shaders/common/sharc.wgsl:36-116
 *   query_sharc                  shaders/common/sharc_query.wgsl:8-29
 *   claim / deposit / update     shaders/sharc_update.wgsl:32-191
 *   resolve (EMA, aging, evict)  shaders/sharc_resolve.wgsl:13-70
 *   eval_sky_radiance            shaders/common/types.wgsl:500-523
 * Deposits run sequentially in tile order, so slot placement is the single-writer outcome; sums
 * are order-independent integer adds.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h).
 */
#include <math.h>
#include <string.h>
#include "orc.h"
#include "orc_math.h"

static uint32_t norm_id(const float n[3]) { return orc_face_id(n); }

static void tangent_frame(const float n[3], float t[3], float b[3]) {
    float up[3] = {0, 0, 0}, c[3];
    if (fabsf(n[2]) < 0.999f) up[2] = 1.0f; else up[0] = 1.0f;
    orc_cross3(up, n, c);
    orc_normalize3(c, t);
    orc_cross3(n, t, b);
}

void orc_sharc_make_key(const float pos[3], const float normal[3], const float cam_pos[3], const float jitter[2],
                        uint32_t* bucket_out, uint32_t* key_out) {
    float dv[3] = {pos[0] - cam_pos[0], pos[1] - cam_pos[1], pos[2] - cam_pos[2]};
    float d = orc_length3(dv);
    int32_t fl = orc_floor_log2(orc_max(d, 4.0f) * 0.25f);
    uint32_t lod = fl < 0 ? 0u : (fl > 3 ? 3u : (uint32_t)fl);
    float s = 0.25f * (float)(1u << lod);
    float anchor[3];
    for (int i = 0; i < 3; ++i) anchor[i] = pos[i] - normal[i] * 0.02f;
    if (jitter[0] != 0.0f || jitter[1] != 0.0f) {
        float t[3], b[3];
        tangent_frame(normal, t, b);
        float k = 0.42f * s;
        for (int i = 0; i < 3; ++i) anchor[i] += (t[i] * jitter[0] + b[i] * jitter[1]) * k;
    }
    uint32_t cell[3];
    for (int i = 0; i < 3; ++i) cell[i] = (uint32_t)((int32_t)floorf(anchor[i] / s) + 16384);
    uint32_t nid = norm_id(normal);
    uint32_t bucket = orc_pcg_hash((cell[0] * 73856093u) ^ (cell[1] * 19349663u) ^ (cell[2] * 83492791u) ^
                                   (nid * 2654435761u) ^ (lod * 38069u)) &
                      (ARC_SHARC_BUCKETS - 1u);
    uint32_t key = orc_pcg_hash(bucket ^ (cell[0] * 1013904223u) ^ (cell[1] * 1664525u) ^ (cell[2] * 2891336453u) ^
                                (nid << 20) ^ (lod << 24)) |
                   ARC_SHARC_KEY_VALID_BIT;
    *bucket_out = bucket;
    *key_out = key;
}

static uint32_t claim_slot(uint32_t* keys, uint32_t bucket, uint32_t key) {
    uint32_t base = bucket * ARC_SHARC_WAYS;
    for (uint32_t i = 0; i < ARC_SHARC_WAYS; ++i)
        if (keys[base + i] == key) return base + i;
    for (uint32_t i = 0; i < ARC_SHARC_WAYS; ++i) {
        uint32_t idx = base + i;
        if (keys[idx] == 0u) { keys[idx] = key; return idx; }
        if (keys[idx] == key) return idx;
    }
    return ARC_SHARC_NO_SLOT;
}

uint32_t orc_sharc_deposit(uint32_t* keys, uint32_t* accum, uint32_t bucket, uint32_t key, const float rad[3]) {
    uint32_t slot = claim_slot(keys, bucket, key);
    if (slot == ARC_SHARC_NO_SLOT) return slot;
    uint32_t a = slot * 4u;
    for (int i = 0; i < 3; ++i) accum[a + i] += orc_f2u(orc_clamp(rad[i], 0.0f, ARC_SHARC_MAX_RADIANCE) * ARC_SHARC_FIXED_SCALE);
    accum[a + 3] += 1u;
    return slot;
}

static void unpack_rad(const arc_sharc_slot* s, float out[3]) {
    out[0] = orc_f16_to_f32(s->rad_rg & 0xFFFFu);
    out[1] = orc_f16_to_f32(s->rad_rg >> 16);
    out[2] = orc_f16_to_f32(s->rad_b_meta & 0xFFFFu);
}

void orc_sharc_resolve(uint32_t* keys, uint32_t* accum, arc_sharc_slot* resolved) {
    for (uint32_t slot = 0; slot < ARC_SHARC_SLOTS; ++slot) {
        uint32_t key = keys[slot];
        arc_sharc_slot* r = &resolved[slot];
        if (key == 0u) { memset(r, 0, sizeof(*r)); continue; }
        uint32_t a = slot * 4u;
        uint32_t count = accum[a + 3];
        int prev_valid = r->key == key;
        float rad[3] = {0, 0, 0};
        uint32_t hist = 0, stale = 0;
        if (prev_valid) {
            unpack_rad(r, rad);
            hist = (r->rad_b_meta >> 16) & 0xFFu;
            stale = (r->rad_b_meta >> 24) & 0xFFu;
        }
        if (count > 0u) {
            float inv = 1.0f / ((float)count * ARC_SHARC_FIXED_SCALE);
            float smp[3] = {(float)accum[a] * inv, (float)accum[a + 1] * inv, (float)accum[a + 2] * inv};
            hist = orc_umin(hist + 1u, 255u);
            float alpha = 1.0f / orc_min((float)hist, ARC_SHARC_HISTORY_CAP);
            for (int i = 0; i < 3; ++i) rad[i] = orc_mix(rad[i], smp[i], alpha);
            stale = 0u;
            accum[a] = accum[a + 1] = accum[a + 2] = accum[a + 3] = 0u;
        } else {
            stale = stale + 1u;
            if (!prev_valid || stale > ARC_SHARC_STALE_EVICT_AGE) {
                keys[slot] = 0u;
                memset(r, 0, sizeof(*r));
                continue;
            }
        }
        float c[3];
        for (int i = 0; i < 3; ++i) c[i] = orc_clamp(rad[i], 0.0f, ARC_SHARC_MAX_RADIANCE);
        r->key = key;
        r->rad_rg = orc_pack2x16float(c[0], c[1]);
        r->rad_b_meta = (orc_f32_to_f16(c[2]) & 0xFFFFu) | ((hist & 0xFFu) << 16) | ((stale & 0xFFu) << 24);
        r->pad = 0u;
    }
}

static int lookup(const arc_sharc_slot* resolved, uint32_t bucket, uint32_t key, float out[4]) {
    uint32_t base = bucket * ARC_SHARC_WAYS;
    for (uint32_t i = 0; i < ARC_SHARC_WAYS; ++i) {
        const arc_sharc_slot* s = &resolved[base + i];
        if (s->key == key) {
            unpack_rad(s, out);
            out[3] = 1.0f;
            return 1;
        }
    }
    out[0] = out[1] = out[2] = out[3] = 0.0f;
    return 0;
}

void orc_sharc_query(const arc_sharc_slot* resolved, const float pos[3], const float normal[3], const float cam_pos[3],
                     const float jitter[2], float out[4]) {
    uint32_t b, k;
    if (jitter[0] != 0.0f || jitter[1] != 0.0f) {
        orc_sharc_make_key(pos, normal, cam_pos, jitter, &b, &k);
        if (lookup(resolved, b, k, out) && out[3] > 0.5f) return;
    }
    float zero[2] = {0.0f, 0.0f};
    orc_sharc_make_key(pos, normal, cam_pos, zero, &b, &k);
    lookup(resolved, b, k, out);
}

/* ------------------------------------------------------------------------------------------ */
/* sharc_update.wgsl main                                                                      */
/* ------------------------------------------------------------------------------------------ */

static void mix3(const float a[3], const float b[3], float t, float out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = a[i] * (1.0f - t) + b[i] * t;
}

static void eval_sky(const float dir[3], const float sun[3], float out[3]) {
    float sun_elev = sun[1];
    float day_t = orc_clamp((sun_elev + 0.05f) / 0.30f, 0.0f, 1.0f);
    float tw_t = orc_clamp(1.0f - fabsf(sun_elev - 0.02f) / 0.22f, 0.0f, 1.0f);
    float zenith = orc_clamp(dir[1], 0.0f, 1.0f);
    float horizon = orc_powi(1.0f - zenith, 3u);
    const float dz[3] = {0.08f, 0.22f, 0.55f}, dh[3] = {0.38f, 0.50f, 0.68f};
    const float nz[3] = {0.0015f, 0.0025f, 0.0055f}, nh[3] = {0.0035f, 0.0065f, 0.0120f};
    const float tw[3] = {0.65f, 0.25f, 0.10f};
    float sz[3], sh[3], sh2[3], sky[3];
    mix3(nz, dz, day_t, sz);
    mix3(nh, dh, day_t, sh);
    mix3(sh, tw, tw_t * 0.75f, sh2);
    mix3(sz, sh2, horizon, sky);
    float sun_cos = orc_max(orc_dot3(dir, sun), 0.0f);
    if (sun_elev > -0.12f) {
        const float sc[3] = {0.85f, 0.52f, 0.24f};
        float p = orc_powi(sun_cos, 14u);
        float m = orc_max(day_t, tw_t);
        for (int i = 0; i < 3; ++i) sky[i] += ((sc[i] * p) * 0.35f) * m;
    }
    memcpy(out, sky, sizeof(sky));
}

void orc_sky_radiance(const float dir[3], const float sun[3], float out[3]) { eval_sky(dir, sun, out); }

typedef struct surf { int hit; uint32_t mat; float t_m; float pos[3]; float normal[3]; float albedo[3]; float emission[3]; } surf;

static void trace_surface(const orc_world* w, const arc_camera_uniforms* cam, const float o[3], const float d[3],
                          float max_dist, surf* s) {
    memset(s, 0, sizeof(*s));
    orc_trace_out tr;
    orc_trace_scene(w, cam, o, d, max_dist, 2u, 1, &tr);
    if (!tr.hit) return;
    const arc_material* m = &w->palette[tr.mat_id];
    s->hit = 1;
    s->mat = tr.mat_id;
    s->t_m = tr.t_voxels * ARC_VOXEL_SIZE;
    memcpy(s->pos, tr.hit_pos_m, sizeof(s->pos));
    memcpy(s->normal, tr.normal, sizeof(s->normal));
    mix3(m->albedo_roughness, tr.lod_rgb, 0.55f, s->albedo);
    memcpy(s->emission, m->emission_meta, sizeof(s->emission));
}

/* camera ray + ign + basis helpers (same definitions as orc_trace.c) */
static void cam_dir(const arc_camera_uniforms* cam, uint32_t px, uint32_t py, uint32_t W, uint32_t H, float d[3]) {
    float u = (((float)px + 0.5f) + cam->jitter_brush_dt[0]) / (float)W;
    float v = (((float)py + 0.5f) + cam->jitter_brush_dt[1]) / (float)H;
    float nx = u * 2.0f - 1.0f, ny = 1.0f - v * 2.0f;
    float th = cam->cam_forward_fov[3];
    float sx = (nx * cam->cam_right_aspect[3]) * th, sy = ny * th;
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = (cam->cam_forward_fov[i] + cam->cam_right_aspect[i] * sx) + cam->cam_up_frame[i] * sy;
    orc_normalize3(r, d);
}

static void ign2(float px, float py, uint32_t frame, float out[2]) {
    float f = (float)frame;
    uint32_t ux = orc_f2u(px), uy = orc_f2u(py);
    float i1 = orc_fract(52.9829189f * orc_fract(0.06711056f * px + 0.00583715f * py));
    float i2 = orc_fract(52.9829189f * orc_fract((0.00583715f * px - 0.06711056f * py) + 0.5f));
    uint32_t h1 = orc_pcg_hash(ux * 1973u + uy * 9277u + frame * 26699u);
    uint32_t h2 = orc_pcg_hash(h1 ^ 0x9E3779B9u);
    out[0] = orc_fract((i1 + f * 0.754877666f) + (float)(h1 & 0xFFFFu) / 65536.0f);
    out[1] = orc_fract((i2 + f * 0.569840291f) + (float)(h2 & 0xFFFFu) / 65536.0f);
}

static void cos_hemi(float u1, float u2, const float n[3], float out[3]) {
    float t[3], b[3];
    tangent_frame(n, t, b);
    float r = sqrtf(u1), z = sqrtf(orc_max(0.0f, 1.0f - u1)), si, co;
    orc_sincos(6.2831853f * u2, &si, &co);
    float rc = r * co, rs = r * si;
    for (int i = 0; i < 3; ++i) out[i] = (t[i] * rc + b[i] * rs) + n[i] * z;
}

static void oct_decode_packed(uint32_t p, float n[3]) {
    float o[2];
    orc_unpack2x16snorm(p, o);
    float v[3] = {o[0], o[1], (1.0f - fabsf(o[0])) - fabsf(o[1])};
    if (v[2] < 0.0f) {
        float sx = o[0] >= 0.0f ? 1.0f : -1.0f, sy = o[1] >= 0.0f ? 1.0f : -1.0f;
        float wx = (1.0f - fabsf(o[1])) * sx, wy = (1.0f - fabsf(o[0])) * sy;
        v[0] = wx;
        v[1] = wy;
    }
    orc_normalize3(v, n);
}

/* ------------------------------------------------------------------------------------------ */
/* One-bounce estimator of the cache comparison (no reference counterpart: the light transport the */
/* NRC and SHARC are scored on). L(x) = albedo * (c_sun max(n.l, 0) V(x, l) + L_sky [a cosine ray  */
/* from x + 0.10 n escapes within 64 m]); V is trace_shadow_vis (traversal64.wgsl:571-773) from     */
/* x + 0.10 n over 32 m as in sharc_shade_surface (sharc_update.wgsl:68-105), c_sun = sun_power *    */
/* (1, 0.9, 0.75) * 0.55, L_sky = (0.30, 0.42, 0.60); the sky ray is a lod_bias 2, water-ignoring   */
/* trace of the static world with a cosine direction (make_basis + sample_cosine_hemisphere,        */
/* types.wgsl:531-545) from two PCG draws.                                                        */
/* ------------------------------------------------------------------------------------------ */

void orc_cmp_albedo(uint32_t mat, float out[3]) {
    uint32_t h0 = orc_pcg_hash(mat * 3u + 0x2545F491u), h1 = orc_pcg_hash(h0 ^ 0x9E3779B9u), h2 = orc_pcg_hash(h1 ^ 0x85EBCA6Bu);
    const float s = 0.8f / 16777216.0f;
    out[0] = 0.1f + (float)(h0 >> 8) * s;
    out[1] = 0.1f + (float)(h1 >> 8) * s;
    out[2] = 0.1f + (float)(h2 >> 8) * s;
}

void orc_onebounce_sun(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float n[3], float out[3]) {
    const float* sun = cam->sun_dir_intensity;
    float sun_power = cam->sun_dir_intensity[3];
    float ndl = orc_max(orc_dot3(n, sun), 0.0f);
    out[0] = out[1] = out[2] = 0.0f;
    if (!(ndl > 0.001f && sun_power > 0.01f)) return;
    float o[3];
    for (int i = 0; i < 3; ++i) o[i] = pos[i] + n[i] * 0.10f;
    float k = ((sun_power * ndl) * orc_shadow_vis(w, cam, o, sun, 32.0f, NULL)) * 0.55f;
    out[0] = 1.0f * k;
    out[1] = 0.90f * k;
    out[2] = 0.75f * k;
}

void orc_onebounce_sky(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float n[3],
                       uint32_t seed, float out[3]) {
    uint32_t h1 = orc_pcg_hash(seed), h2 = orc_pcg_hash(h1 ^ 0x68E31DA4u);
    float u1 = (float)(h1 >> 8) * (1.0f / 16777216.0f), u2 = (float)(h2 >> 8) * (1.0f / 16777216.0f);
    float d[3], o[3];
    cos_hemi(u1, u2, n, d);
    for (int i = 0; i < 3; ++i) o[i] = pos[i] + n[i] * 0.10f;
    orc_trace_out tr;
    orc_trace(w, cam, o, d, 0.0f, 64.0f, 2u, 1, &tr);
    if (tr.hit) {
        out[0] = out[1] = out[2] = 0.0f;
    } else {
        out[0] = 0.30f;
        out[1] = 0.42f;
        out[2] = 0.60f;
    }
}

static void onebounce(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float n[3],
                      const float albedo[3], uint32_t seed, float out[3]) {
    float a[3], c[3];
    orc_onebounce_sun(w, cam, pos, n, a);
    orc_onebounce_sky(w, cam, pos, n, seed, c);
    for (int i = 0; i < 3; ++i) out[i] = albedo[i] * (a[i] + c[i]);
}

void orc_onebounce(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* idx, uint32_t n, const float* pos,
                   const float* nrm, const float* alb, uint32_t spp, uint32_t seed, int accumulate, float* out, int threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t ii = 0; ii < (int64_t)n; ++ii) {
        uint32_t i = (uint32_t)ii;
        uint32_t p = idx ? idx[i] : i;
        float sum[3] = {0.0f, 0.0f, 0.0f};
        for (uint32_t k = 0; k < spp; ++k) {
            float l[3];
            onebounce(w, cam, &pos[3 * (size_t)p], &nrm[3 * (size_t)p], &alb[3 * (size_t)p],
                      orc_pcg_hash(p * 0x9E3779B9u ^ orc_pcg_hash(seed + k * 0x632BE5ABu)), l);
            for (int c = 0; c < 3; ++c) sum[c] += l[c];
        }
        float inv = 1.0f / (float)spp;
        for (int c = 0; c < 3; ++c) {
            if (accumulate) out[3 * (size_t)i + c] += sum[c] * inv;
            else out[3 * (size_t)i + c] = sum[c] * inv;
        }
    }
}

/* The NRC training batch of a frame: sample i takes list[min(s + i mod k, n_valid - 1)] with
 * s = floor((floor(i / k) * n_valid + phase) / (n_samples / k)), k the cluster size (1: every sample its
 * own stratum), phase = (pcg_hash(seed) * n_valid) >> 32; its target is the 1-spp estimator with albedo
 * 1 (sky ray seeded by pcg_hash(i ^ pcg_hash(seed ^ 0xB5297A4D))), stored with the point's 9 network
 * inputs at slot (i mod steps) * (n_samples / steps) + i / steps. */
void orc_train_samples(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* list, uint64_t n_valid,
                       const float* pos, const float* nrm, const float* nrc_in, uint32_t seed, uint32_t n_samples,
                       uint32_t steps, uint32_t cluster, float* train_in, float* train_t, int threads) {
    if (!n_valid) return;
    const uint64_t phase = ((uint64_t)orc_pcg_hash(seed) * n_valid) >> 32;
    const uint32_t per = n_samples / steps;
    if (cluster == 0u || n_samples % cluster) cluster = 1u;
    const uint32_t n_cl = n_samples / cluster;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t ii = 0; ii < (int64_t)n_samples; ++ii) {
        uint32_t i = (uint32_t)ii;
        /* runs of `cluster` consecutive list entries whose starts are stratified over the list */
        uint64_t start = ((uint64_t)(i / cluster) * n_valid + phase) / n_cl;
        uint64_t jj = start + i % cluster;
        uint32_t j = (uint32_t)(jj < n_valid ? jj : n_valid - 1u);
        uint32_t p = list[j];
        float sun[3], sky[3];
        orc_onebounce_sun(w, cam, &pos[3 * (size_t)p], &nrm[3 * (size_t)p], sun);
        orc_onebounce_sky(w, cam, &pos[3 * (size_t)p], &nrm[3 * (size_t)p], orc_pcg_hash(i ^ orc_pcg_hash(seed ^ 0xB5297A4Du)), sky);
        size_t slot = (size_t)(i % steps) * per + i / steps;
        for (int q = 0; q < 9; ++q) train_in[slot * 9 + q] = nrc_in[(size_t)p * 9 + q];
        for (int c = 0; c < 3; ++c) train_t[3 * slot + c] = sky[c] + sun[c];
    }
}

/* GI hit points of a frame (what both caches are queried at): per pixel with a primary hit, the Pass-2A
 * GI ray from the G-buffer (orc_gi_setup) traced as lod_bias 2, water-ignoring, over ray_distances.z;
 * at its hit the point, normal, comparison albedo and the 9 network inputs (point / world extent,
 * normal, -ray direction). valid = 0 where there is no primary hit or the GI ray misses. */
static void write_point(const arc_camera_uniforms* cam, size_t k, const float p[3], const float n[3], uint32_t mat,
                        const float view[3], float* pos, float* nrm, float* alb, float* nrc_in) {
    float a[3];
    orc_cmp_albedo(mat, a);
    float ex = (float)cam->world_grid_dims[0] * 16.0f, ey = (float)cam->world_grid_dims[1] * 16.0f,
          ez = (float)cam->world_grid_dims[2] * 16.0f;
    for (int i = 0; i < 3; ++i) {
        pos[3 * k + i] = p[i];
        nrm[3 * k + i] = n[i];
        alb[3 * k + i] = a[i];
    }
    float* q = nrc_in + 9 * k;
    q[0] = p[0] / ex;
    q[1] = p[1] / ey;
    q[2] = p[2] / ez;
    q[3] = n[0];
    q[4] = n[1];
    q[5] = n[2];
    q[6] = view[0];
    q[7] = view[1];
    q[8] = view[2];
}

void orc_gi_points(const orc_world* w, const arc_camera_uniforms* cam, uint32_t W, uint32_t H, const uint32_t* gdm,
                   const uint32_t* gnm, float* pos, float* nrm, float* alb, float* nrc_in, uint32_t* valid, int threads) {
#pragma omp parallel for schedule(dynamic, 4) num_threads(threads > 0 ? threads : 1)
    for (int64_t yy = 0; yy < (int64_t)H; ++yy) {
        for (uint32_t x = 0; x < W; ++x) {
            uint32_t y = (uint32_t)yy;
            size_t k = (size_t)y * W + x;
            uint32_t bytes = 0;
            orc_gi_ray g;
            valid[k] = 0u;
            if (!orc_gi_setup(w, cam, x, y, W, H, gdm[2 * k], gnm[2 * k], &g, &bytes)) continue;
            orc_trace_out tr;
            orc_trace(w, cam, g.origin, g.dir, 0.0f, cam->ray_distances[2], 2u, 1, &tr);
            if (!tr.hit) continue;
            valid[k] = 1u;
            float view[3] = {-g.dir[0], -g.dir[1], -g.dir[2]};
            write_point(cam, k, tr.hit_pos_m, tr.normal, tr.mat_id, view, pos, nrm, alb, nrc_in);
        }
    }
}

/* The same points from the frame's GI hit records, without tracing: the centre of the hit cell's entry
 * face (LOD cells included), that face's normal, the view direction from the point back to the GI ray's
 * origin (primary hit + 0.10 m along its G-buffer normal). */
void orc_gi_points_from_hits(const arc_camera_uniforms* cam, uint32_t W, uint32_t H, const uint32_t* gdm, const uint32_t* gnm,
                             const arc_hit_record* gi_hits, float* pos, float* nrm, float* alb, float* nrc_in,
                             uint32_t* valid) {
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            size_t k = (size_t)y * W + x;
            const arc_hit_record* h = &gi_hits[k];
            float hit_dist = orc_bitsf(gdm[2 * k]);
            valid[k] = 0u;
            if (!((h->flags & ARC_HIT_FLAG_HIT) && h->face < 6u && hit_dist < 1e4f)) continue;
            valid[k] = 1u;
            int32_t span_i = 1 << (2u * ((h->flags >> 1) & 7u));
            float span = (float)span_i;
            float c[3] = {(float)(h->voxel[0] & ~(span_i - 1)), (float)(h->voxel[1] & ~(span_i - 1)),
                          (float)(h->voxel[2] & ~(span_i - 1))};
            float axis_sign = (h->face & 1u) ? -1.0f : 1.0f;
            uint32_t axis = h->face >> 1;
            float n[3] = {0.0f, 0.0f, 0.0f}, p[3];
            for (int i = 0; i < 3; ++i) p[i] = c[i] + 0.5f * span;
            n[axis] = axis_sign;
            p[axis] = c[axis] + (axis_sign > 0.0f ? span : 0.0f);
            for (int i = 0; i < 3; ++i) p[i] = p[i] * ARC_VOXEL_SIZE;
            float rd[3], gn[3], o[3], v[3], view[3];
            cam_dir(cam, x, y, W, H, rd);
            oct_decode_packed(gnm[2 * k], gn);
            for (int i = 0; i < 3; ++i) o[i] = (cam->cam_pos_time[i] + rd[i] * hit_dist) + gn[i] * 0.10f;
            for (int i = 0; i < 3; ++i) v[i] = o[i] - p[i];
            float len = orc_length3(v);
            if (len > 0.0f) {
                float inv = 1.0f / len;
                for (int i = 0; i < 3; ++i) view[i] = v[i] * inv;
            } else {
                memcpy(view, n, sizeof(view));
            }
            write_point(cam, k, p, n, h->mat, view, pos, nrm, alb, nrc_in);
        }
}

void orc_sharc_update(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* gdm, const uint32_t* gnm,
                      const arc_sharc_slot* resolved_prev, uint32_t* keys, uint32_t* accum, uint32_t* tile_key,
                      uint32_t* tile_bucket, float* tile_rad, uint32_t* tile_valid) {
    orc_sharc_update_mode(w, cam, gdm, gnm, resolved_prev, keys, accum, tile_key, tile_bucket, tile_rad, tile_valid, 0u);
}

/* mode 0: sharc_shade_surface at the path vertex, as the reference; mode 1: the one-bounce estimator
 * above with the comparison albedo of the vertex's material. */
void orc_sharc_update_mode(const orc_world* w, const arc_camera_uniforms* cam, const uint32_t* gdm, const uint32_t* gnm,
                           const arc_sharc_slot* resolved_prev, uint32_t* keys, uint32_t* accum, uint32_t* tile_key,
                           uint32_t* tile_bucket, float* tile_rad, uint32_t* tile_valid, uint32_t mode) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    uint32_t tile = (cam->quality_flags[3] & 0xFFu) <= 12u ? 16u : 8u;
    uint32_t tx = (W + tile - 1u) / tile, ty = (H + tile - 1u) / tile;
    uint32_t frame = orc_fbits(cam->cam_up_frame[3]);
    const float* sun = cam->sun_dir_intensity;
    float sun_power = cam->sun_dir_intensity[3];
    float bounce_max = orc_min(cam->ray_distances[2], tile == 16u ? 10.0f : 16.0f);
    for (uint32_t gy = 0; gy < ty; ++gy)
        for (uint32_t gx = 0; gx < tx; ++gx) {
            uint32_t ti = gy * tx + gx;
            tile_valid[ti] = 0;
            tile_key[ti] = 0;
            tile_bucket[ti] = 0;
            tile_rad[3 * ti] = tile_rad[3 * ti + 1] = tile_rad[3 * ti + 2] = 0.0f;
            uint32_t h = orc_pcg_hash(gx * 1973u + gy * 9277u + frame * 26699u + 0x51ED270Bu);
            uint32_t px = orc_umin(gx * tile + (h & (tile - 1u)), W - 1u);
            uint32_t py = orc_umin(gy * tile + ((h >> 8) & (tile - 1u)), H - 1u);
            size_t p = (size_t)py * W + px;
            float depth = orc_bitsf(gdm[2 * p]);
            if (depth >= 1e4f) continue;
            float rd[3], x0[3], n0[3];
            cam_dir(cam, px, py, W, H, rd);
            for (int i = 0; i < 3; ++i) x0[i] = cam->cam_pos_time[i] + rd[i] * depth;
            oct_decode_packed(gnm[2 * p], n0);
            float xi0[2], xi1[2];
            ign2((float)px, (float)py, frame, xi0);
            ign2((float)px + 37.0f, (float)py + 91.0f, frame + 4099u, xi1);
            float d0[3], o0[3];
            cos_hemi(xi0[0], xi0[1], n0, d0);
            for (int i = 0; i < 3; ++i) o0[i] = x0[i] + n0[i] * 0.10f;
            surf s1;
            trace_surface(w, cam, o0, d0, bounce_max, &s1);
            if (!s1.hit) continue;
            if (mode == 1u) {
                float a1[3], rad[3], zero[2] = {0.0f, 0.0f};
                orc_cmp_albedo(s1.mat, a1);
                onebounce(w, cam, s1.pos, s1.normal, a1, h ^ (frame * 0x9E3779B9u), rad);
                uint32_t b, k;
                orc_sharc_make_key(s1.pos, s1.normal, cam->cam_pos_time, zero, &b, &k);
                orc_sharc_deposit(keys, accum, b, k, rad);
                tile_valid[ti] = 1;
                tile_key[ti] = k;
                tile_bucket[ti] = b;
                memcpy(&tile_rad[3 * ti], rad, sizeof(rad));
                continue;
            }
            /* sharc_shade_surface */
            const float* n = s1.normal;
            float direct[3] = {0, 0, 0};
            float ndl = orc_max(orc_dot3(n, sun), 0.0f);
            if (ndl > 0.001f && sun_power > 0.01f) {
                float so[3];
                for (int i = 0; i < 3; ++i) so[i] = s1.pos[i] + n[i] * 0.10f;
                float vis = orc_shadow_vis(w, cam, so, sun, 32.0f, NULL);
                const float c[3] = {1.0f, 0.90f, 0.75f};
                for (int i = 0; i < 3; ++i) direct[i] = (((c[i] * sun_power) * ndl) * vis) * 0.55f;
            }
            float bd[3], bo[3];
            cos_hemi(xi1[0], xi1[1], n, bd);
            for (int i = 0; i < 3; ++i) bo[i] = s1.pos[i] + n[i] * 0.10f;
            surf s2;
            trace_surface(w, cam, bo, bd, bounce_max, &s2);
            float gathered[3] = {0, 0, 0};
            if (s2.hit) {
                float em_att = 1.0f / ((1.0f + s2.t_m * 0.06f) + (s2.t_m * s2.t_m) * 0.025f);
                float ndl_em = orc_max(orc_dot3(n, bd), 0.25f);
                for (int i = 0; i < 3; ++i) gathered[i] += ((s2.emission[i] * 1.15f) * em_att) * ndl_em;
                float q[4], zero[2] = {0.0f, 0.0f};
                orc_sharc_query(resolved_prev, s2.pos, s2.normal, cam->cam_pos_time, zero, q);
                for (int i = 0; i < 3; ++i) gathered[i] += q[i];
            } else {
                float end_y = bo[1] + bd[1] * bounce_max;
                if (bd[1] > 0.15f && end_y >= 32.0f) {
                    float esc = orc_clamp((bd[1] - 0.15f) / 0.35f, 0.0f, 1.0f);
                    float sky[3];
                    eval_sky(bd, sun, sky);
                    for (int i = 0; i < 3; ++i) gathered[i] += (sky[i] * 0.45f) * esc;
                }
            }
            float rad[3];
            for (int i = 0; i < 3; ++i) rad[i] = s1.albedo[i] * (direct[i] + gathered[i]);
            float zero[2] = {0.0f, 0.0f};
            uint32_t b, k;
            orc_sharc_make_key(s1.pos, s1.normal, cam->cam_pos_time, zero, &b, &k);
            orc_sharc_deposit(keys, accum, b, k, rad);
            tile_valid[ti] = 1;
            tile_key[ti] = k;
            tile_bucket[ti] = b;
            memcpy(&tile_rad[3 * ti], rad, sizeof(rad));
        }
}
