/*
 * orc_cpu.c — oracle restatement of the reference's CPU ray query:
 *   WorldMap::raycast_meters   crates/arcadia-world/src/world_map.rs:464-545
 *   raycast_chunk_tree         crates/arcadia-core/src/raycast_cpu.rs:28-218
 *   intersect_aabb             crates/arcadia-core/src/raycast_cpu.rs:222-234
 *   step_dda_box               crates/arcadia-core/src/raycast_cpu.rs:245-292
 *   resolve_entry_normal       crates/arcadia-core/src/raycast_cpu.rs:295-327
 * glam 0.29.3 semantics (not vendored in the reference): Vec3 min/max = IEEE minNum/maxNum per
 * component, clamp = max then min, signum(+0) = +1, normalize_or_zero = v * (1 / sqrt(dot)) when
 * that reciprocal is finite and positive.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h). This is the "reference CPU ray query" timed as the
 * host-core baseline; the WGSL transcription (orc_trace.c) is the parity oracle.
 */
#include <math.h>
#include <string.h>
#include "orc.h"
#include "orc_math.h"

static float rs_signum(float x) {
    if (x != x) return x;
    return signbit(x) ? -1.0f : 1.0f;
}

static int cpu_intersect_aabb(const float o[3], const float inv[3], const float bmin[3], const float bmax[3], float* tmin,
                              float* tmax) {
    float lo[3], hi[3];
    for (int i = 0; i < 3; ++i) {
        float t0 = (bmin[i] - o[i]) * inv[i];
        float t1 = (bmax[i] - o[i]) * inv[i];
        lo[i] = fminf(t0, t1);
        hi[i] = fmaxf(t0, t1);
    }
    float a = fmaxf(fmaxf(lo[0], lo[1]), lo[2]);
    float b = fminf(fminf(hi[0], hi[1]), hi[2]);
    if (b >= fmaxf(a, 0.0f)) {
        *tmin = a;
        *tmax = b;
        return 1;
    }
    return 0;
}

static void cpu_step(const float vo[3], const float dir[3], const float inv[3], const float noi[3], const int pos[3],
                     const uint32_t bmin[3], const uint32_t bmax[3], float cur_t, float* t_out, uint32_t vi[3]) {
    uint32_t ex[3];
    float tm[3];
    for (int i = 0; i < 3; ++i) {
        ex[i] = pos[i] ? bmax[i] : bmin[i];
        tm[i] = (float)ex[i] * inv[i] + noi[i];
    }
    float t_exit = fminf(fminf(tm[0], tm[1]), tm[2]);
    float next_t = fmaxf(cur_t, t_exit);
    int is_x = tm[0] <= tm[1] && tm[0] <= tm[2];
    int is_y = !is_x && (tm[1] <= tm[2]);
    int is_z = !is_x && !is_y;
    int is_exit[3] = {is_x, is_y, is_z};
    for (int i = 0; i < 3; ++i) {
        uint32_t outside = ex[i] - (pos[i] ? 0u : 1u);
        float p = fmaxf(vo[i] + dir[i] * next_t, 0.0f);
        uint32_t hi = bmax[i] ? bmax[i] - 1u : 0u;
        uint32_t inside = orc_uclamp(orc_f2u(p), bmin[i], hi);
        vi[i] = is_exit[i] ? outside : inside;
    }
    *t_out = next_t;
}

static void cpu_normal(const float tmv[3], const float dir[3], float n[3]) {
    float max_t = fmaxf(fmaxf(tmv[0], tmv[1]), tmv[2]);
    float eps = 1e-4f * fmaxf(max_t * 0.01f, 1.0f);
    float cx = fabsf(tmv[0] - max_t) <= eps ? fabsf(dir[0]) : 0.0f;
    float cy = fabsf(tmv[1] - max_t) <= eps ? fabsf(dir[1]) : 0.0f;
    float cz = fabsf(tmv[2] - max_t) <= eps ? fabsf(dir[2]) : 0.0f;
    n[0] = n[1] = n[2] = 0.0f;
    if (cx >= cy && cx >= cz && cx > 0.0f) n[0] = -rs_signum(dir[0]);
    else if (cy >= cz && cy > 0.0f) n[1] = -rs_signum(dir[1]);
    else if (cz > 0.0f) n[2] = -rs_signum(dir[2]);
    else if (tmv[0] >= tmv[1] && tmv[0] >= tmv[2]) n[0] = -rs_signum(dir[0]);
    else if (tmv[1] >= tmv[2]) n[1] = -rs_signum(dir[1]);
    else n[2] = -rs_signum(dir[2]);
}

static inline uint32_t child_slot(const arc_node64* n, uint32_t b) {
    uint64_t mask = (uint64_t)n->mask_low | ((uint64_t)n->mask_high << 32);
    uint64_t prefix = (b == 0) ? 0ull : ((1ull << b) - 1ull);
    return (n->child_ptr & ARC_PTR_INDEX_MASK) + (uint32_t)__builtin_popcountll(mask & prefix);
}

static inline int has_child(const arc_node64* n, uint32_t b) {
    uint64_t mask = (uint64_t)n->mask_low | ((uint64_t)n->mask_high << 32);
    return ((mask >> b) & 1ull) != 0;
}

typedef struct cpu_hit { float distance; float normal[3]; uint32_t voxel[3]; uint32_t mat; } cpu_hit;

/* raycast_chunk_tree over the chunk whose root node is nodes[root_idx]; origin in chunk-local voxels. */
static int raycast_chunk(const orc_world* w, uint32_t root_idx, const float o[3], const float ray_dir[3], float max_dist,
                         cpu_hit* hit) {
    const arc_node64* root = &w->nodes[root_idx];
    if (root->mask_low == 0 && root->mask_high == 0) return 0;
    float sd[3], inv[3];
    for (int i = 0; i < 3; ++i) {
        sd[i] = fabsf(ray_dir[i]) > 1e-7f ? ray_dir[i] : copysignf(1e-7f, ray_dir[i]);
        inv[i] = 1.0f / sd[i];
    }
    float zero3[3] = {0, 0, 0}, cmax[3] = {256.0f, 256.0f, 256.0f};
    float te_raw, tx_raw;
    if (!cpu_intersect_aabb(o, inv, zero3, cmax, &te_raw, &tx_raw)) return 0;
    float t_enter = fmaxf(te_raw, 0.0f);
    float t_limit = fminf(tx_raw, max_dist);
    if (tx_raw < t_enter || t_enter >= max_dist) return 0;
    int pos[3] = {inv[0] >= 0.0f, inv[1] >= 0.0f, inv[2] >= 0.0f};
    float noi[3] = {-o[0] * inv[0], -o[1] * inv[1], -o[2] * inv[2]};
    float t = t_enter;
    uint32_t vi[3];
    for (int i = 0; i < 3; ++i) vi[i] = orc_f2u(fminf(fmaxf(o[i] + sd[i] * (t + 1e-4f), 0.0f), 256.0f - 1e-3f));
    uint32_t prev[3] = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t cached_shift = 6u;
    arc_node64 c1, c2, c3;
    memset(&c1, 0, sizeof(c1)); c2 = c1; c3 = c1;
    for (int step = 0; step < 512; ++step) {
        if (t >= t_limit) break;
        if (vi[0] >= 256u || vi[1] >= 256u || vi[2] >= 256u) break;
        uint32_t diff = (prev[0] ^ vi[0]) | (prev[1] ^ vi[1]) | (prev[2] ^ vi[2]);
        memcpy(prev, vi, sizeof(prev));
        arc_node64 node;
        uint32_t shift;
        if (diff < 4u && cached_shift == 0u) { node = c3; shift = 0u; }
        else if (diff < 16u && cached_shift <= 2u) { node = c2; shift = 2u; }
        else if (diff < 64u && cached_shift <= 4u) { node = c1; shift = 4u; }
        else { node = *root; shift = 6u; }
        cached_shift = shift;
        uint32_t l[3] = {vi[0] & 255u, vi[1] & 255u, vi[2] & 255u};
        for (;;) {
            uint32_t b = (((l[2] >> shift) & 3u) << 4) | (((l[1] >> shift) & 3u) << 2) | ((l[0] >> shift) & 3u);
            uint32_t span = 1u << shift;
            uint32_t bmin[3] = {vi[0] & ~(span - 1u), vi[1] & ~(span - 1u), vi[2] & ~(span - 1u)};
            uint32_t bmax[3] = {bmin[0] + span, bmin[1] + span, bmin[2] + span};
            if (!has_child(&node, b)) {
                cpu_step(o, sd, inv, noi, pos, bmin, bmax, t, &t, vi);
                break;
            }
            if (node.child_ptr & ARC_IS_LEAF_FLAG) {
                uint32_t mat;
                if (node.child_ptr & ARC_IS_UNIFORM_FLAG) mat = node.lod_payload >> 24;
                else {
                    uint32_t word = w->bricks[node.child_ptr & ARC_PTR_INDEX_MASK].packed_materials[b >> 2];
                    mat = (word >> ((b & 3u) * 8u)) & 0xFFu;
                }
                if (mat != ARC_MAT_AIR) {
                    float tmv[3];
                    for (int i = 0; i < 3; ++i) {
                        uint32_t e = pos[i] ? bmin[i] : bmax[i];
                        tmv[i] = (float)e * inv[i] + noi[i];
                    }
                    float ce = fmaxf(fmaxf(tmv[0], tmv[1]), tmv[2]);
                    hit->distance = fmaxf(ce, 0.0f);
                    cpu_normal(tmv, ray_dir, hit->normal);
                    memcpy(hit->voxel, vi, sizeof(vi));
                    hit->mat = mat;
                    return 1;
                }
                cpu_step(o, sd, inv, noi, pos, bmin, bmax, t, &t, vi);
                break;
            }
            uint32_t next = child_slot(&node, b);
            node = w->nodes[next];
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) c1 = node;
            else if (shift == 2u) c2 = node;
            else if (shift == 0u) c3 = node;
        }
    }
    return 0;
}

/* raycast_meters; returns 1 on hit and fills the record (depth in meters). */
static int raycast_meters(const orc_world* w, const uint32_t grid[3], const float origin_m[3], const float dir_in[3],
                          float max_dist_m, arc_hit_record* out) {
    out->voxel[0] = out->voxel[1] = out->voxel[2] = -1;
    out->face = ARC_FACE_NONE;
    out->mat = 0;
    out->flags = 0;
    out->depth_m = max_dist_m;
    float len = sqrtf(orc_dot3(dir_in, dir_in));
    float rcp = 1.0f / len;
    if (!(isfinite(rcp) && rcp > 0.0f)) return 0;
    float dir[3] = {dir_in[0] * rcp, dir_in[1] * rcp, dir_in[2] * rcp};
    float vo[3] = {origin_m[0] * 16.0f, origin_m[1] * 16.0f, origin_m[2] * 16.0f};
    float max_v = max_dist_m * 16.0f;
    float inv[3];
    for (int i = 0; i < 3; ++i) inv[i] = fabsf(dir[i]) > 1e-7f ? 1.0f / dir[i] : copysignf(INFINITY, dir[i]);
    float wmax[3] = {(float)grid[0] * 256.0f, (float)grid[1] * 256.0f, (float)grid[2] * 256.0f};
    float zero3[3] = {0, 0, 0};
    float t, t_exit;
    if (!cpu_intersect_aabb(vo, inv, zero3, wmax, &t, &t_exit)) return 0;
    if (t >= max_v || t_exit <= 0.0f) return 0;
    t = fmaxf(t, 0.0f);
    for (int it = 0; it < 128; ++it) {
        if (t >= fminf(t_exit, max_v)) break;
        float p[3];
        for (int i = 0; i < 3; ++i) p[i] = fminf(fmaxf(vo[i] + dir[i] * (t + 1e-2f), 0.0f), wmax[i] - 1e-3f);
        int32_t c[3] = {(int32_t)floorf(p[0] / 256.0f), (int32_t)floorf(p[1] / 256.0f), (int32_t)floorf(p[2] / 256.0f)};
        float cmin[3] = {(float)c[0] * 256.0f, (float)c[1] * 256.0f, (float)c[2] * 256.0f};
        float cmax[3] = {cmin[0] + 256.0f, cmin[1] + 256.0f, cmin[2] + 256.0f};
        if (c[0] >= 0 && c[1] >= 0 && c[2] >= 0 && c[0] < (int32_t)grid[0] && c[1] < (int32_t)grid[1] && c[2] < (int32_t)grid[2]) {
            uint32_t ci = (uint32_t)c[0] + (uint32_t)c[1] * grid[0] + (uint32_t)c[2] * grid[0] * grid[1];
            uint32_t root = w->roots[ci];
            if (root != ARC_EMPTY_CHUNK) {
                float lo[3] = {vo[0] - cmin[0], vo[1] - cmin[1], vo[2] - cmin[2]};
                cpu_hit h;
                if (raycast_chunk(w, root, lo, dir, max_v, &h)) {
                    for (int i = 0; i < 3; ++i) out->voxel[i] = (int32_t)h.voxel[i] + c[i] * 256;
                    out->face = (uint8_t)orc_face_id(h.normal);
                    out->mat = (uint8_t)h.mat;
                    out->flags = ARC_HIT_FLAG_HIT;
                    out->depth_m = h.distance * ARC_VOXEL_SIZE;
                    return 1;
                }
            }
        }
        float a, cexit;
        if (cpu_intersect_aabb(vo, inv, cmin, cmax, &a, &cexit)) t = fmaxf(cexit, t + 0.05f);
        else break;
    }
    return 0;
}

/* raycast_chunk_tree called directly with chunk-local voxel units, as the reference's unit tests do
 * (raycast_cpu.rs:334-446). Returns 1 on hit; out = {distance, nx, ny, nz}, voxel/mat filled. */
int orc_raycast_chunk_local(const orc_world* w, uint32_t root_idx, const float origin_v[3], const float dir[3],
                            float max_dist_v, float out[4], int32_t voxel[3], uint32_t* mat) {
    cpu_hit h;
    if (!raycast_chunk(w, root_idx, origin_v, dir, max_dist_v, &h)) return 0;
    out[0] = h.distance;
    out[1] = h.normal[0];
    out[2] = h.normal[1];
    out[3] = h.normal[2];
    for (int i = 0; i < 3; ++i) voxel[i] = (int32_t)h.voxel[i];
    *mat = h.mat;
    return 1;
}

void orc_cpu_raycast(const orc_world* w, const uint32_t grid[3], const arc_ray* rays, uint32_t n, float max_dist_m,
                     arc_hit_record* hits, int threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < (int64_t)n; ++i) raycast_meters(w, grid, rays[i].origin_m, rays[i].dir, max_dist_m, &hits[i]);
}

/* Camera ray of the pinhole model (primary_gbuffer.wgsl:103-115) for the CPU query's frame sample. */
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

/* Frame sample through the reference CPU query: primary ray per sampled pixel, then one cosine
 * GI ray from its hit (same sampling as the GPU path) through the same query. */
uint64_t orc_cpu_frame_sample(const orc_world* w, const arc_camera_uniforms* cam, uint32_t stride, int threads,
                              uint64_t* n_primary, uint64_t* n_gi, uint64_t* checksum) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    uint32_t grid[3] = {cam->world_grid_dims[0], cam->world_grid_dims[1], cam->world_grid_dims[2]};
    uint64_t total = (uint64_t)W * H, ns = (total + stride - 1) / stride;
    uint64_t np = 0, ng = 0, cs = 0;
    uint32_t frame = orc_fbits(cam->cam_up_frame[3]);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1) reduction(+ : np, ng, cs)
    for (int64_t s = 0; s < (int64_t)ns; ++s) {
        uint64_t k = (uint64_t)s * stride;
        uint32_t x = (uint32_t)(k % W), y = (uint32_t)(k / W);
        float d[3];
        cam_dir(cam, x, y, W, H, d);
        arc_hit_record h;
        np += 1;
        if (!raycast_meters(w, grid, cam->cam_pos_time, d, 250.0f, &h)) continue;
        cs += h.mat + (uint32_t)(h.voxel[0] ^ h.voxel[1] ^ h.voxel[2]);
        static const float axis[6][3] = {{1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1}};
        const float* n = axis[h.face < 6 ? h.face : 2];
        float hp[3], o[3];
        for (int i = 0; i < 3; ++i) hp[i] = cam->cam_pos_time[i] + d[i] * h.depth_m;
        for (int i = 0; i < 3; ++i) o[i] = hp[i] + n[i] * 0.10f;
        /* cosine sample about normalize(n + (0, 0.22, 0)) from the pixel's PCG-seeded gradient noise */
        uint32_t h1 = orc_pcg_hash(x * 1973u + y * 9277u + frame * 26699u);
        uint32_t h2 = orc_pcg_hash(h1 ^ 0x9E3779B9u);
        float u1 = (float)(h1 & 0xFFFFu) / 65536.0f, u2 = (float)(h2 & 0xFFFFu) / 65536.0f;
        float sn_in[3] = {n[0], n[1] + 0.22f, n[2]}, sn[3], t[3], b[3], up[3] = {0, 0, 0}, c[3];
        orc_normalize3(sn_in, sn);
        if (fabsf(sn[2]) < 0.999f) up[2] = 1.0f; else up[0] = 1.0f;
        orc_cross3(up, sn, c);
        orc_normalize3(c, t);
        orc_cross3(sn, t, b);
        float r = sqrtf(u1), z = sqrtf(fmaxf(0.0f, 1.0f - u1)), si, co;
        orc_sincos(6.2831853f * u2, &si, &co);
        float gd[3];
        for (int i = 0; i < 3; ++i) gd[i] = (t[i] * (r * co) + b[i] * (r * si)) + sn[i] * z;
        arc_hit_record g;
        ng += 1;
        if (raycast_meters(w, grid, o, gd, cam->ray_distances[2], &g)) cs += g.mat + (uint32_t)(g.voxel[0] ^ g.voxel[1] ^ g.voxel[2]);
    }
    *n_primary = np;
    *n_gi = ng;
    *checksum = cs;
    return np + ng;
}
