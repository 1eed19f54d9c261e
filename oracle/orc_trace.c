/*
 * orc_trace.c — oracle restatement of the WGSL traversal, the primary G-buffer pass, the Pass-2A
 * GI ray and the FP64 depth check.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h). Canonical arithmetic: orc_math.h.
 *
 * One deliberate deviation from the WGSL, shared with the CUDA kernels: the distance of a hit
 * (t_voxels and everything derived from it) is (enter_coord - origin) / dir on the entry axis,
 * not enter_coord * inv_dir + (-origin * inv_dir) (traversal64.wgsl:468-472). The WGSL form
 * cancels catastrophically for far-from-origin rays with short hits; the DDA decisions and the
 * face choice still use the WGSL form, so hit voxels, faces and materials are unchanged.
 */
#include <math.h>
#include <string.h>
#include <stdlib.h>
#include "orc.h"
#include "orc_math.h"

typedef struct { uint32_t x, y, z; } u3;

static inline int node_has_child(uint32_t lo, uint32_t hi, uint32_t b) {
    uint32_t word = b < 32u ? lo : hi;
    return ((word >> (b & 31u)) & 1u) != 0u;
}

/* traversal64.wgsl:32-40 */
static inline uint32_t node_child_offset(const arc_node64* n, uint32_t b) {
    uint32_t base = n->child_ptr & ARC_PTR_INDEX_MASK;
    int low = b < 32u;
    uint32_t prefix = (1u << (b & 31u)) - 1u;
    uint32_t pl = low ? prefix : 0xFFFFFFFFu;
    uint32_t ph = low ? 0u : prefix;
    return base + orc_popc(n->mask_low & pl) + orc_popc(n->mask_high & ph);
}

/* Pool reads out of range read zero: the reference validates its traversal shaders with naga's
 * ReadZeroSkipWrite bounds-check policy (crates/arcadia-render/tests/shader_validation.rs:39-50), so a
 * corrupt pointer reads an empty node or an air brick word. */
static inline uint32_t brick_get_material(const orc_world* w, uint32_t brick_idx, uint32_t bit, uint32_t* bytes) {
    *bytes += 4;
    if (brick_idx >= w->n_bricks) return 0u;
    uint32_t word = w->bricks[brick_idx].packed_materials[bit >> 2];
    return (word >> ((bit & 3u) * 8u)) & 0xFFu;
}

static inline arc_node64 load_node(const orc_world* w, uint32_t idx, uint32_t* bytes) {
    *bytes += 16;
    if (idx >= w->n_nodes) {
        arc_node64 z = {0u, 0u, 0u, 0u};
        return z;
    }
    return w->nodes[idx];
}

/* step_dda_box: traversal64.wgsl:152-179 */
static void step_dda_box(const float vo[3], const float dir[3], const float inv[3], const float noi[3], const int pos[3],
                         u3 bmin, u3 bmax, float cur_t, float* t_out, u3* vi_out) {
    uint32_t ex[3] = {pos[0] ? bmax.x : bmin.x, pos[1] ? bmax.y : bmin.y, pos[2] ? bmax.z : bmin.z};
    float tm[3];
    for (int i = 0; i < 3; ++i) tm[i] = (float)ex[i] * inv[i] + noi[i];
    float t_exit = orc_min(orc_min(tm[0], tm[1]), tm[2]);
    float next_t = orc_max(cur_t, t_exit);
    int is_x = tm[0] <= tm[1] && tm[0] <= tm[2];
    int is_y = !is_x && (tm[1] <= tm[2]);
    int is_z = !is_x && !is_y;
    uint32_t out_vi[3] = {ex[0] - (pos[0] ? 0u : 1u), ex[1] - (pos[1] ? 0u : 1u), ex[2] - (pos[2] ? 0u : 1u)};
    uint32_t bmn[3] = {bmin.x, bmin.y, bmin.z}, bmx[3] = {bmax.x, bmax.y, bmax.z};
    uint32_t in_vi[3];
    for (int i = 0; i < 3; ++i) {
        float p = orc_max(vo[i] + dir[i] * next_t, 0.0f);
        in_vi[i] = orc_uclamp(orc_f2u(p), bmn[i], bmx[i] - 1u);
    }
    int is_exit[3] = {is_x, is_y, is_z};
    *t_out = next_t;
    vi_out->x = is_exit[0] ? out_vi[0] : in_vi[0];
    vi_out->y = is_exit[1] ? out_vi[1] : in_vi[1];
    vi_out->z = is_exit[2] ? out_vi[2] : in_vi[2];
}

/* intersect_aabb: traversal64.wgsl:134-142 */
static void intersect_aabb(const float o[3], const float inv[3], const float bmin[3], const float bmax[3], float* tmin,
                           float* tmax) {
    float a[3], b[3];
    for (int i = 0; i < 3; ++i) {
        float eb = inv[i] > 0.0f ? bmin[i] : bmax[i];
        float xb = inv[i] > 0.0f ? bmax[i] : bmin[i];
        a[i] = (eb - o[i]) * inv[i];
        b[i] = (xb - o[i]) * inv[i];
    }
    *tmin = orc_max(orc_max(a[0], a[1]), a[2]);
    *tmax = orc_min(orc_min(b[0], b[1]), b[2]);
}

/* eval_leaf_bitwise_ao: traversal64.wgsl:60-131 */
static float eval_leaf_bitwise_ao(uint32_t lo, uint32_t hi, uint32_t cx, uint32_t cy, uint32_t cz, const float n[3],
                                  const float hp[3]) {
    float fx = orc_clamp(orc_fract(hp[0]), 0.0f, 1.0f);
    float fy = orc_clamp(orc_fract(hp[1]), 0.0f, 1.0f);
    float fz = orc_clamp(orc_fract(hp[2]), 0.0f, 1.0f);
    int32_t nx = (int32_t)cx + (int32_t)n[0];
    int32_t ny = (int32_t)cy + (int32_t)n[1];
    int32_t nz = (int32_t)cz + (int32_t)n[2];
    if (nx < 0 || nx > 3 || ny < 0 || ny > 3 || nz < 0 || nz > 3) return 1.0f;
    uint32_t bb = ((uint32_t)nz << 4) | ((uint32_t)ny << 2) | (uint32_t)nx;
    float occ = 0.0f;
    if (fabsf(n[1]) > 0.5f) {
        if (nx > 0 && node_has_child(lo, hi, bb - 1u)) occ += (1.0f - fx) * 0.42f;
        if (nx < 3 && node_has_child(lo, hi, bb + 1u)) occ += fx * 0.42f;
        if (nz > 0 && node_has_child(lo, hi, bb - 16u)) occ += (1.0f - fz) * 0.42f;
        if (nz < 3 && node_has_child(lo, hi, bb + 16u)) occ += fz * 0.42f;
    } else if (fabsf(n[0]) > 0.5f) {
        if (ny > 0 && node_has_child(lo, hi, bb - 4u)) occ += (1.0f - fy) * 0.42f;
        if (ny < 3 && node_has_child(lo, hi, bb + 4u)) occ += fy * 0.42f;
        if (nz > 0 && node_has_child(lo, hi, bb - 16u)) occ += (1.0f - fz) * 0.42f;
        if (nz < 3 && node_has_child(lo, hi, bb + 16u)) occ += fz * 0.42f;
    } else {
        if (nx > 0 && node_has_child(lo, hi, bb - 1u)) occ += (1.0f - fx) * 0.42f;
        if (nx < 3 && node_has_child(lo, hi, bb + 1u)) occ += fx * 0.42f;
        if (ny > 0 && node_has_child(lo, hi, bb - 4u)) occ += (1.0f - fy) * 0.42f;
        if (ny < 3 && node_has_child(lo, hi, bb + 4u)) occ += fy * 0.42f;
    }
    return orc_clamp(1.0f - occ, 0.35f, 1.0f);
}

/* sharc_norm_id order: +X, -X, +Y, -Y, +Z, -Z (sharc.wgsl:48-57). */
uint32_t orc_face_id(const float n[3]) {
    float ax = fabsf(n[0]), ay = fabsf(n[1]), az = fabsf(n[2]);
    if (ax > ay && ax > az) return n[0] > 0.0f ? 0u : 1u;
    if (ay > az) return n[1] > 0.0f ? 2u : 3u;
    return n[2] > 0.0f ? 4u : 5u;
}

/* trace_world_64tree_from: traversal64.wgsl:226-556 */
void orc_trace(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
               float start_t_m, float max_dist_m, uint32_t lod_bias, int ignore_water, orc_trace_out* res) {
    uint32_t bytes = 24;
    memset(res, 0, sizeof(*res));
    res->hit = 0;
    res->t_voxels = max_dist_m * ARC_VOXELS_PER_METER;
    for (int i = 0; i < 3; ++i) res->hit_pos_m[i] = origin_m[i] + dir[i] * max_dist_m;
    res->normal[0] = 0.0f; res->normal[1] = 1.0f; res->normal[2] = 0.0f;
    res->mat_id = ARC_MAT_AIR;
    res->contact_ao = 1.0f;

    float vo[3], safe[3], inv[3];
    for (int i = 0; i < 3; ++i) vo[i] = origin_m[i] * ARC_VOXELS_PER_METER;
    float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    float start_t_v = orc_max(start_t_m * ARC_VOXELS_PER_METER, 0.0f);
    for (int i = 0; i < 3; ++i) {
        safe[i] = fabsf(dir[i]) < 1e-7f ? 1e-7f : dir[i];
        inv[i] = 1.0f / safe[i];
    }
    const uint32_t* g = cam->world_grid_dims;
    float wmax[3] = {(float)g[0] * ARC_CHUNK_DIM_F, (float)g[1] * ARC_CHUNK_DIM_F, (float)g[2] * ARC_CHUNK_DIM_F};
    float zero3[3] = {0.0f, 0.0f, 0.0f};
    float wh_x, wh_y;
    intersect_aabb(vo, inv, zero3, wmax, &wh_x, &wh_y);
    float t_enter = orc_max(wh_x, start_t_v);
    if (wh_y < t_enter || t_enter >= max_t_v) {
        res->bytes = bytes;
        return;
    }
    float t = t_enter;
    float t_limit = orc_min(wh_y, max_t_v);
    uint32_t max_steps = cam->ray_steps[0];
    if (lod_bias == 1u) max_steps = cam->ray_steps[1];
    else if (lod_bias >= 2u) max_steps = cam->ray_steps[2];

    float prim_lod_t = cam->lod_settings[0] * ARC_VOXELS_PER_METER;
    uint32_t prim_lod_step = cam->quality_flags[0];
    float sec_lod_t = cam->lod_settings[1] * ARC_VOXELS_PER_METER;
    uint32_t sec_lod_step = cam->quality_flags[1];
    float gi_lod_t = cam->lod_settings[2] * ARC_VOXELS_PER_METER;
    uint32_t gi_lod_step = (cam->quality_flags[3] >> 16) & 0xFFu;

    int pos[3] = {inv[0] >= 0.0f, inv[1] >= 0.0f, inv[2] >= 0.0f};
    float noi[3] = {-vo[0] * inv[0], -vo[1] * inv[1], -vo[2] * inv[2]};
    uint32_t wmax_vi[3] = {g[0] << 8, g[1] << 8, g[2] << 8};

    u3 vi;
    {
        float sp[3];
        for (int i = 0; i < 3; ++i) sp[i] = orc_clamp(vo[i] + dir[i] * (t + 1e-4f), 0.0f, wmax[i] - 1e-3f);
        vi.x = orc_f2u(sp[0]); vi.y = orc_f2u(sp[1]); vi.z = orc_f2u(sp[2]);
    }

    u3 mtf_c0 = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t mtf_root0 = ARC_EMPTY_CHUNK;
    u3 mtf_c1 = mtf_c0;
    uint32_t mtf_root1 = ARC_EMPTY_CHUNK;
    u3 prev_vi = mtf_c0;
    uint32_t cached_shift = 6u;
    arc_node64 c_l1, c_l2, c_l3;
    memset(&c_l1, 0, sizeof(c_l1)); c_l2 = c_l1; c_l3 = c_l1;

    uint32_t step;
    for (step = 0; step < max_steps; ++step) {
        if (t >= t_limit) break;
        if (vi.x >= wmax_vi[0] || vi.y >= wmax_vi[1] || vi.z >= wmax_vi[2]) {
            t = t_limit;
            break;
        }
        uint32_t diff = (prev_vi.x ^ vi.x) | (prev_vi.y ^ vi.y) | (prev_vi.z ^ vi.z);
        prev_vi = vi;
        uint32_t root_idx = mtf_root0;
        if (diff >= 256u) {
            u3 c = {vi.x >> 8, vi.y >> 8, vi.z >> 8};
            cached_shift = 6u;
            if (c.x == mtf_c1.x && c.y == mtf_c1.y && c.z == mtf_c1.z) {
                root_idx = mtf_root1;
                mtf_c1 = mtf_c0; mtf_root1 = mtf_root0;
                mtf_c0 = c; mtf_root0 = root_idx;
            } else {
                uint32_t c_idx = c.x + c.y * g[0] + c.z * g[0] * g[1];
                bytes += 4;
                root_idx = w->roots[c_idx];
                mtf_c1 = mtf_c0; mtf_root1 = mtf_root0;
                mtf_c0 = c; mtf_root0 = root_idx;
            }
        }
        if (root_idx == ARC_EMPTY_CHUNK) {
            u3 cmin = {vi.x & ~255u, vi.y & ~255u, vi.z & ~255u};
            u3 cmax = {cmin.x + 256u, cmin.y + 256u, cmin.z + 256u};
            step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
            continue;
        }
        uint32_t min_shift = 0u;
        if (lod_bias == 0u) {
            if (t > prim_lod_t || step > prim_lod_step) min_shift = 2u;
        } else if (lod_bias == 1u) {
            if (t > (sec_lod_t * 2.2857f) || step > sec_lod_step) min_shift = 4u;
            else if (t > sec_lod_t) min_shift = 2u;
        } else {
            if (t > gi_lod_t || step > gi_lod_step) min_shift = 2u;
        }
        arc_node64 node;
        uint32_t shift;
        if (diff < 4u && min_shift == 0u && cached_shift == 0u) { node = c_l3; shift = 0u; }
        else if (diff < 16u && min_shift <= 2u && cached_shift <= 2u) { node = c_l2; shift = 2u; }
        else if (diff < 64u && min_shift <= 4u && cached_shift <= 4u) { node = c_l1; shift = 4u; }
        else { node = load_node(w, root_idx, &bytes); shift = 6u; }
        cached_shift = shift;

        u3 l = {vi.x & 255u, vi.y & 255u, vi.z & 255u};
        for (;;) {
            uint32_t cx = (l.x >> shift) & 3u, cy = (l.y >> shift) & 3u, cz = (l.z >> shift) & 3u;
            uint32_t b = (cz << 4) | (cy << 2) | cx;
            if (ignore_water && (node.child_ptr & ARC_IS_UNIFORM_FLAG) != 0u) {
                uint32_t uni = (node.lod_payload >> 24) & 0xFFu;
                if (uni == ARC_MAT_WATER_CRYSTAL) {
                    uint32_t span = 4u << shift;
                    u3 nmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                    u3 nmax = {nmin.x + span, nmin.y + span, nmin.z + span};
                    step_dda_box(vo, dir, inv, noi, pos, nmin, nmax, t, &t, &vi);
                    break;
                }
            }
            if (!node_has_child(node.mask_low, node.mask_high, b)) {
                uint32_t span = 1u << shift;
                u3 cmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                u3 cmax = {cmin.x + span, cmin.y + span, cmin.z + span};
                step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
                break;
            }
            int is_leaf = (node.child_ptr & ARC_IS_LEAF_FLAG) != 0u;
            int stop_for_lod = shift <= min_shift;
            if (is_leaf || stop_for_lod) {
                uint32_t span = 1u << shift;
                u3 cmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                u3 cmax = {cmin.x + span, cmin.y + span, cmin.z + span};
                uint32_t mat = (node.lod_payload >> 24) & 0xFFu;
                if (is_leaf && (node.child_ptr & ARC_IS_UNIFORM_FLAG) == 0u)
                    mat = brick_get_material(w, node.child_ptr & ARC_PTR_INDEX_MASK, b, &bytes);
                if (ignore_water && mat == ARC_MAT_WATER_CRYSTAL) {
                    step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
                    break;
                }
                if (mat != ARC_MAT_AIR) {
                    uint32_t enter[3] = {pos[0] ? cmin.x : cmax.x, pos[1] ? cmin.y : cmax.y, pos[2] ? cmin.z : cmax.z};
                    float tmv[3];
                    for (int i = 0; i < 3; ++i) tmv[i] = (float)enter[i] * inv[i] + noi[i];
                    float cell_enter = orc_max(orc_max(tmv[0], tmv[1]), tmv[2]);
                    (void)cell_enter;
                    /* Entry axis = the one whose plane distance is the largest (ties x, then y). */
                    int ax = (tmv[0] >= tmv[1] && tmv[0] >= tmv[2]) ? 0 : (tmv[1] >= tmv[2] ? 1 : 2);
                    float t_acc = ((float)enter[ax] - vo[ax]) / safe[ax];
                    float exact_t = orc_max(t_acc, 0.0f);
                    float hp[3];
                    for (int i = 0; i < 3; ++i) hp[i] = vo[i] + dir[i] * exact_t;
                    res->hit = 1;
                    res->t_voxels = exact_t;
                    for (int i = 0; i < 3; ++i) res->hit_pos_m[i] = hp[i] * ARC_VOXEL_SIZE;
                    float max_t = orc_max(orc_max(tmv[0], tmv[1]), tmv[2]);
                    float eps = 1e-4f * orc_max(max_t * 0.01f, 1.0f);
                    float cand_x = fabsf(tmv[0] - max_t) <= eps ? fabsf(dir[0]) : 0.0f;
                    float cand_y = fabsf(tmv[1] - max_t) <= eps ? fabsf(dir[1]) : 0.0f;
                    float cand_z = fabsf(tmv[2] - max_t) <= eps ? fabsf(dir[2]) : 0.0f;
                    float nrm[3] = {0.0f, 0.0f, 0.0f};
                    if (cand_x >= cand_y && cand_x >= cand_z && cand_x > 0.0f) nrm[0] = -orc_sign(dir[0]);
                    else if (cand_y >= cand_z && cand_y > 0.0f) nrm[1] = -orc_sign(dir[1]);
                    else if (cand_z > 0.0f) nrm[2] = -orc_sign(dir[2]);
                    else if (tmv[0] >= tmv[1] && tmv[0] >= tmv[2]) nrm[0] = -orc_sign(dir[0]);
                    else if (tmv[1] >= tmv[2]) nrm[1] = -orc_sign(dir[1]);
                    else nrm[2] = -orc_sign(dir[2]);
                    memcpy(res->normal, nrm, sizeof(nrm));
                    res->mat_id = mat;
                    res->lod_rgb[0] = (float)(node.lod_payload & 0xFFu) / 255.0f;
                    res->lod_rgb[1] = (float)((node.lod_payload >> 8) & 0xFFu) / 255.0f;
                    res->lod_rgb[2] = (float)((node.lod_payload >> 16) & 0xFFu) / 255.0f;
                    res->voxel_hash = orc_pcg_hash((vi.x * 73856093u) ^ (vi.y * 19349663u) ^ (vi.z * 83492791u));
                    if (shift == 0u && lod_bias == 0u) {
                        float hit_dist_m = t * ARC_VOXEL_SIZE;
                        float raw = orc_bitsf(cam->point_light_count[3]);
                        float ao_max = raw < 1.0f ? 24.0f : raw;
                        if (hit_dist_m < ao_max) {
                            float raw_ao = eval_leaf_bitwise_ao(node.mask_low, node.mask_high, cx, cy, cz, nrm, hp);
                            float ao_min = ao_max * 0.5f;
                            float wgt = 1.0f - orc_smoothstep(ao_min, ao_max, hit_dist_m);
                            res->contact_ao = orc_mix(1.0f, raw_ao, wgt);
                        } else {
                            res->contact_ao = 1.0f;
                        }
                    }
                    res->vi[0] = vi.x; res->vi[1] = vi.y; res->vi[2] = vi.z;
                    res->shift = shift;
                    res->steps = step + 1;
                    res->bytes = bytes;
                    return;
                }
                step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
                break;
            }
            uint32_t next = node_child_offset(&node, b);
            node = load_node(w, next, &bytes);
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) c_l1 = node;
            else if (shift == 2u) c_l2 = node;
            else if (shift == 0u) c_l3 = node;
        }
    }
    res->steps = step;
    res->bytes = bytes;
}

/* is_emissive_mat: traversal64.wgsl:775-777 */
static void fill_hit_record(const orc_trace_out* r, float t_scale_m, arc_hit_record* h);

/* mat4x4 (column-major) * vec4(v, w): ((c0 x + c1 y) + c2 z) + c3 w per row */
static void xform4(const float* M, const float v[3], float wc, float out[3]) {
    for (int r = 0; r < 3; ++r) out[r] = ((M[r] * v[0] + M[4 + r] * v[1]) + M[8 + r] * v[2]) + M[12 + r] * wc;
}

/* trace_single_rigid_body: traversal64.wgsl:1006-1222 */
static void trace_single_rigid(const orc_world* w, uint32_t body, const float origin_m[3], const float dir[3],
                               float max_dist_m, orc_rigid_out* res) {
    memset(res, 0, sizeof(*res));
    res->t_voxels = max_dist_m * ARC_VOXELS_PER_METER;
    res->normal[1] = 1.0f;
    res->contact_ao = 1.0f;
    res->body = body;
    const arc_rigid_body* rb = &w->bodies[body];
    uint32_t root_idx = orc_fbits(rb->local_bounds_and_root[3]);
    if (root_idx == ARC_EMPTY_CHUNK) return;
    /* bounding-sphere pre-reject */
    float oc[3] = {origin_m[0] - rb->world_sphere[0], origin_m[1] - rb->world_sphere[1], origin_m[2] - rb->world_sphere[2]};
    float bp = orc_dot3(oc, dir);
    float cd = orc_dot3(oc, oc) - rb->world_sphere[3] * rb->world_sphere[3];
    if (cd > 0.0f && bp > 0.0f) return;
    float disc = bp * bp - cd;
    if (disc < 0.0f) return;
    float near = orc_max(-bp - sqrtf(disc), 0.0f);
    if (near >= max_dist_m) return;
    /* body-local voxel space */
    float lo_m[3], ld[3], vo[3], lmax[3], sd[3], inv[3], noi[3];
    xform4(rb->world_to_local, origin_m, 1.0f, lo_m);
    xform4(rb->world_to_local, dir, 0.0f, ld);
    for (int i = 0; i < 3; ++i) {
        vo[i] = lo_m[i] * ARC_VOXELS_PER_METER;
        lmax[i] = rb->local_bounds_and_root[i] * ARC_VOXELS_PER_METER;
        sd[i] = fabsf(ld[i]) < 1e-7f ? 1e-7f : ld[i];
        inv[i] = 1.0f / sd[i];
    }
    float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    const float zero[3] = {0.0f, 0.0f, 0.0f};
    float b0, b1;
    intersect_aabb(vo, inv, zero, lmax, &b0, &b1);
    float t_enter = orc_max(b0, 0.0f);
    if (b1 < t_enter || t_enter >= max_t_v) return;
    float t = t_enter;
    float t_limit = orc_min(b1, max_t_v);
    int pos[3];
    uint32_t maxi[3];
    for (int i = 0; i < 3; ++i) {
        pos[i] = inv[i] >= 0.0f;
        noi[i] = -vo[i] * inv[i];
        maxi[i] = orc_f2u(lmax[i] + 0.5f);
    }
    u3 vi;
    {
        float p[3];
        for (int i = 0; i < 3; ++i) p[i] = orc_clamp(vo[i] + ld[i] * (t + 1e-4f), 0.0f, lmax[i] - 1e-3f);
        vi.x = orc_f2u(p[0]);
        vi.y = orc_f2u(p[1]);
        vi.z = orc_f2u(p[2]);
    }
    u3 prev = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t cached_shift = 6u, bytes = 0;
    arc_node64 c1, c2, c3;
    memset(&c1, 0, sizeof(c1));
    memset(&c2, 0, sizeof(c2));
    memset(&c3, 0, sizeof(c3));
    for (uint32_t step = 0; step < 64u; ++step) {
        if (t >= t_limit) break;
        if (vi.x >= maxi[0] || vi.y >= maxi[1] || vi.z >= maxi[2]) break;
        uint32_t diff = (prev.x ^ vi.x) | (prev.y ^ vi.y) | (prev.z ^ vi.z);
        prev = vi;
        arc_node64 node;
        uint32_t shift;
        if (diff < 4u && cached_shift == 0u) {
            node = c3;
            shift = 0u;
        } else if (diff < 16u && cached_shift <= 2u) {
            node = c2;
            shift = 2u;
        } else if (diff < 64u && cached_shift <= 4u) {
            node = c1;
            shift = 4u;
        } else {
            node = load_node(w, root_idx, &bytes);
            shift = 6u;
        }
        cached_shift = shift;
        uint32_t l[3] = {vi.x & 255u, vi.y & 255u, vi.z & 255u};
        for (;;) {
            uint32_t cx = (l[0] >> shift) & 3u, cy = (l[1] >> shift) & 3u, cz = (l[2] >> shift) & 3u;
            uint32_t b = (cz << 4) | (cy << 2) | cx;
            uint32_t span = 1u << shift;
            u3 cmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
            u3 cmax = {cmin.x + span, cmin.y + span, cmin.z + span};
            if (!node_has_child(node.mask_low, node.mask_high, b)) {
                step_dda_box(vo, ld, inv, noi, pos, cmin, cmax, t, &t, &vi);
                break;
            }
            if (node.child_ptr & ARC_IS_LEAF_FLAG) {
                uint32_t mat = (node.lod_payload >> 24) & 0xFFu;
                if (!(node.child_ptr & ARC_IS_UNIFORM_FLAG)) mat = brick_get_material(w, node.child_ptr & ARC_PTR_INDEX_MASK, b, &bytes);
                if (mat != ARC_MAT_AIR) {
                    uint32_t ec[3] = {pos[0] ? cmin.x : cmax.x, pos[1] ? cmin.y : cmax.y, pos[2] ? cmin.z : cmax.z};
                    float tm[3];
                    for (int i = 0; i < 3; ++i) tm[i] = (float)ec[i] * inv[i] + noi[i];
                    float enter = orc_max(orc_max(tm[0], tm[1]), tm[2]);
                    float et = orc_max(enter, 0.0f);
                    float hpv[3], hpm[3];
                    for (int i = 0; i < 3; ++i) {
                        hpv[i] = vo[i] + ld[i] * et;
                        hpm[i] = hpv[i] * ARC_VOXEL_SIZE;
                    }
                    res->hit = 1;
                    res->t_voxels = et;
                    xform4(rb->local_to_world, hpm, 1.0f, res->hit_pos_m);
                    xform4(rb->prev_local_to_world, hpm, 1.0f, res->prev_hit_pos_m);
                    float ln[3] = {0.0f, 0.0f, 0.0f};
                    if (tm[0] >= tm[1] && tm[0] >= tm[2]) ln[0] = -orc_sign(ld[0]);
                    else if (tm[1] >= tm[2]) ln[1] = -orc_sign(ld[1]);
                    else ln[2] = -orc_sign(ld[2]);
                    float wn[3];
                    xform4(rb->local_to_world, ln, 0.0f, wn);
                    orc_normalize3(wn, res->normal);
                    res->mat_id = mat;
                    res->voxel_hash = orc_pcg_hash((vi.x * 73856093u) ^ (vi.y * 19349663u) ^ (vi.z * 83492791u));
                    res->vi[0] = vi.x;
                    res->vi[1] = vi.y;
                    res->vi[2] = vi.z;
                    res->shift = shift;
                    if (shift == 0u) res->contact_ao = eval_leaf_bitwise_ao(node.mask_low, node.mask_high, cx, cy, cz, ln, hpv);
                    return;
                }
                step_dda_box(vo, ld, inv, noi, pos, cmin, cmax, t, &t, &vi);
                break;
            }
            node = load_node(w, node_child_offset(&node, b), &bytes);
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) c1 = node;
            else if (shift == 2u) c2 = node;
            else if (shift == 0u) c3 = node;
        }
    }
}

/* trace_rigid_bodies: traversal64.wgsl:1224-1244 (bodies min(cam count, table size, 32)) */
void orc_trace_rigid_bodies(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3],
                            const float dir[3], float max_dist_m, orc_rigid_out* best) {
    memset(best, 0, sizeof(*best));
    best->t_voxels = max_dist_m * ARC_VOXELS_PER_METER;
    best->normal[1] = 1.0f;
    best->contact_ao = 1.0f;
    uint32_t n = orc_umin(orc_umin((cam->point_light_count[1] >> 16) & 0xFFFFu, ARC_MAX_RIGID_BODIES), w->n_bodies);
    float cur = max_dist_m;
    for (uint32_t i = 0; i < n; ++i) {
        orc_rigid_out c;
        trace_single_rigid(w, i, origin_m, dir, cur, &c);
        if (c.hit && c.t_voxels < best->t_voxels) {
            *best = c;
            cur = c.t_voxels * ARC_VOXEL_SIZE;
        }
    }
}

/* A secondary-ray trace of the static world followed by the rigid bodies in front of its hit, as
 * the GI ray (lighting_restir_gi.wgsl:209-224) and sharc_trace_surface (sharc_update.wgsl:32-52) do:
 * a rigid hit replaces hit, distance, point, normal and material, and its LOD colour is the
 * material's albedo. Returns the body index of a rigid hit, -1 otherwise. */
int orc_trace_scene(const orc_world* w, const arc_camera_uniforms* cam, const float o[3], const float d[3],
                    float max_dist_m, uint32_t lod_bias, int ignore_water, orc_trace_out* r) {
    orc_trace(w, cam, o, d, 0.0f, max_dist_m, lod_bias, ignore_water, r);
    if (orc_rigid_count(w, cam) == 0u) return -1;
    orc_rigid_out rb;
    orc_trace_rigid_bodies(w, cam, o, d, r->hit ? r->t_voxels * ARC_VOXEL_SIZE : max_dist_m, &rb);
    if (!rb.hit) return -1;
    r->hit = 1;
    r->t_voxels = rb.t_voxels;
    memcpy(r->hit_pos_m, rb.hit_pos_m, sizeof(r->hit_pos_m));
    memcpy(r->normal, rb.normal, sizeof(r->normal));
    r->mat_id = rb.mat_id;
    memcpy(r->lod_rgb, w->palette[rb.mat_id].albedo_roughness, sizeof(r->lod_rgb));
    memcpy(r->vi, rb.vi, sizeof(r->vi));
    r->shift = rb.shift;
    return (int)rb.body;
}

/* trace_rigid_bodies over a ray batch: hit records as the GPU writes them (body hits flagged, the
 * body index in flags bits 8..12) and 9 floats per ray (hit point, previous hit point, normal). */
void orc_trace_rigid_rays(const orc_world* w, const arc_camera_uniforms* cam, const arc_ray* rays, uint32_t n,
                          float max_dist_m, arc_hit_record* hits, float* detail, int threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        orc_rigid_out rb;
        orc_trace_rigid_bodies(w, cam, rays[i].origin_m, rays[i].dir, max_dist_m, &rb);
        orc_trace_out r;
        memset(&r, 0, sizeof(r));
        r.hit = rb.hit;
        r.t_voxels = rb.t_voxels;
        memcpy(r.normal, rb.normal, sizeof(r.normal));
        r.mat_id = rb.mat_id;
        memcpy(r.vi, rb.vi, sizeof(r.vi));
        r.shift = rb.shift;
        fill_hit_record(&r, ARC_VOXEL_SIZE, &hits[i]);
        if (rb.hit) hits[i].flags = (uint16_t)(hits[i].flags | ARC_HIT_FLAG_RIGID | (rb.body << 8));
        if (detail) {
            float* q = detail + 9 * i;
            if (rb.hit) {
                memcpy(q, rb.hit_pos_m, 12);
                memcpy(q + 3, rb.prev_hit_pos_m, 12);
            } else {
                for (int k = 0; k < 3; ++k) q[k] = q[3 + k] = rays[i].origin_m[k] + rays[i].dir[k] * max_dist_m;
            }
            memcpy(q + 6, rb.normal, 12);
        }
    }
}

uint32_t orc_rigid_count(const orc_world* w, const arc_camera_uniforms* cam) {
    return orc_umin(orc_umin((cam->point_light_count[1] >> 16) & 0xFFFFu, ARC_MAX_RIGID_BODIES), w->n_bodies);
}

static int is_emissive_mat(uint32_t m) { return (m >= 19u && m <= 22u) || m == 24u || m == 27u; }

/* trace_shadow_vis: traversal64.wgsl:571-773 (di = 0); trace_shadow_vis_di: traversal64.wgsl:781-989
 * (di = 1): step budget clamped to [32, 48], LOD only with distance left to the target, uniform nodes
 * and brick materials read, an emissive hit within 16 voxels of the target visible, and visible at the
 * end only when within 2 voxels of the target. */
static float shadow_vis_impl(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
                             float max_dist_m, uint32_t* bytes_io, int di) {
    uint32_t bytes = 0;
    float vo[3], inv[3];
    for (int i = 0; i < 3; ++i) {
        vo[i] = origin_m[i] * ARC_VOXELS_PER_METER;
        float s = fabsf(dir[i]) < 1e-7f ? 1e-7f : dir[i];
        inv[i] = 1.0f / s;
    }
    float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    const uint32_t* g = cam->world_grid_dims;
    float wmax[3] = {(float)g[0] * ARC_CHUNK_DIM_F, (float)g[1] * ARC_CHUNK_DIM_F, (float)g[2] * ARC_CHUNK_DIM_F};
    float zero3[3] = {0, 0, 0};
    float wx, wy;
    intersect_aabb(vo, inv, zero3, wmax, &wx, &wy);
    if (wy < orc_max(wx, 0.0f) || wx >= max_t_v) { if (bytes_io) *bytes_io += bytes; return 1.0f; }
    float t = orc_max(wx, 0.0f);
    float t_limit = orc_min(wy, max_t_v);
    uint32_t max_steps = di ? orc_uclamp(cam->ray_steps[3], 32u, 48u) : cam->ray_steps[3];
    int pos[3] = {inv[0] >= 0.0f, inv[1] >= 0.0f, inv[2] >= 0.0f};
    float noi[3] = {-vo[0] * inv[0], -vo[1] * inv[1], -vo[2] * inv[2]};
    uint32_t wmax_vi[3] = {g[0] << 8, g[1] << 8, g[2] << 8};
    u3 vi;
    {
        float sp[3];
        for (int i = 0; i < 3; ++i) sp[i] = orc_clamp(vo[i] + dir[i] * (t + 1e-4f), 0.0f, wmax[i] - 1e-3f);
        vi.x = orc_f2u(sp[0]); vi.y = orc_f2u(sp[1]); vi.z = orc_f2u(sp[2]);
    }
    u3 prev_vi = {0xFFFFFFFFu, 0xFFFFFFFFu, 0xFFFFFFFFu};
    uint32_t cached_shift = 6u;
    arc_node64 c_l1, c_l2, c_l3;
    memset(&c_l1, 0, sizeof(c_l1)); c_l2 = c_l1; c_l3 = c_l1;
    uint32_t cached_root = ARC_EMPTY_CHUNK;
    for (uint32_t step = 0; step < max_steps; ++step) {
        if (t >= t_limit) break;
        if (vi.x >= wmax_vi[0] || vi.y >= wmax_vi[1] || vi.z >= wmax_vi[2]) { t = t_limit; break; }
        uint32_t diff = (prev_vi.x ^ vi.x) | (prev_vi.y ^ vi.y) | (prev_vi.z ^ vi.z);
        prev_vi = vi;
        uint32_t root_idx = cached_root;
        if (diff >= 256u) {
            cached_shift = 6u;
            uint32_t c_idx = (vi.x >> 8) + (vi.y >> 8) * g[0] + (vi.z >> 8) * g[0] * g[1];
            bytes += 4;
            root_idx = w->roots[c_idx];
            cached_root = root_idx;
        }
        if (root_idx == ARC_EMPTY_CHUNK) {
            u3 cmin = {vi.x & ~255u, vi.y & ~255u, vi.z & ~255u};
            u3 cmax = {cmin.x + 256u, cmin.y + 256u, cmin.z + 256u};
            step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
            continue;
        }
        uint32_t min_shift = 0u;
        if (di) {
            float dist_rem = t_limit - t;
            if (t > 48.0f && dist_rem > 32.0f && step > 6u) min_shift = 2u;
            if (t > 160.0f && dist_rem > 64.0f && step > 14u) min_shift = 4u;
        } else {
            if (t > 48.0f || step > 6u) min_shift = 2u;
            if (t > 192.0f || step > 16u) min_shift = 4u;
        }
        arc_node64 node;
        uint32_t shift;
        if (diff < 4u && min_shift == 0u && cached_shift == 0u) { node = c_l3; shift = 0u; }
        else if (diff < 16u && min_shift <= 2u && cached_shift <= 2u) { node = c_l2; shift = 2u; }
        else if (diff < 64u && min_shift <= 4u && cached_shift <= 4u) { node = c_l1; shift = 4u; }
        else { node = load_node(w, root_idx, &bytes); shift = 6u; }
        cached_shift = shift;
        u3 l = {vi.x & 255u, vi.y & 255u, vi.z & 255u};
        for (;;) {
            uint32_t b = (((l.z >> shift) & 3u) << 4) | (((l.y >> shift) & 3u) << 2) | ((l.x >> shift) & 3u);
            if ((node.child_ptr & ARC_IS_UNIFORM_FLAG) != 0u && ((node.lod_payload >> 24) & 0xFFu) == ARC_MAT_WATER_CRYSTAL) {
                uint32_t span = 4u << shift;
                u3 nmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                u3 nmax = {nmin.x + span, nmin.y + span, nmin.z + span};
                step_dda_box(vo, dir, inv, noi, pos, nmin, nmax, t, &t, &vi);
                break;
            }
            if (!node_has_child(node.mask_low, node.mask_high, b)) {
                uint32_t span = 1u << shift;
                u3 cmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                u3 cmax = {cmin.x + span, cmin.y + span, cmin.z + span};
                step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
                break;
            }
            int is_leaf = (node.child_ptr & ARC_IS_LEAF_FLAG) != 0u;
            int is_uniform = (node.child_ptr & ARC_IS_UNIFORM_FLAG) != 0u;
            if (is_leaf || (di && is_uniform) || shift <= min_shift) {
                uint32_t mat = (node.lod_payload >> 24) & 0xFFu;
                if (di && is_leaf && !is_uniform && shift == 0u)
                    mat = brick_get_material(w, node.child_ptr & ARC_PTR_INDEX_MASK, b, &bytes);
                if (mat == ARC_MAT_WATER_CRYSTAL) {
                    uint32_t span = 1u << shift;
                    u3 cmin = {vi.x & ~(span - 1u), vi.y & ~(span - 1u), vi.z & ~(span - 1u)};
                    u3 cmax = {cmin.x + span, cmin.y + span, cmin.z + span};
                    step_dda_box(vo, dir, inv, noi, pos, cmin, cmax, t, &t, &vi);
                    break;
                }
                if (bytes_io) *bytes_io += bytes;
                if (di && is_emissive_mat(mat) && t >= t_limit - 16.0f) return 1.0f;
                return 0.0f;
            }
            uint32_t next = node_child_offset(&node, b);
            node = load_node(w, next, &bytes);
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) c_l1 = node;
            else if (shift == 2u) c_l2 = node;
            else if (shift == 0u) c_l3 = node;
        }
    }
    if (bytes_io) *bytes_io += bytes;
    if (di) return t >= t_limit - 2.0f ? 1.0f : 0.0f;
    if (t < t_limit) {
        float py = vo[1] + dir[1] * t;
        if (py * ARC_VOXEL_SIZE < 32.0f) return 0.0f;
    }
    return 1.0f;
}

float orc_shadow_vis(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
                     float max_dist_m, uint32_t* bytes_io) {
    return shadow_vis_impl(w, cam, origin_m, dir, max_dist_m, bytes_io, 0);
}

float orc_shadow_vis_di(const orc_world* w, const arc_camera_uniforms* cam, const float origin_m[3], const float dir[3],
                        float max_dist_m) {
    return shadow_vis_impl(w, cam, origin_m, dir, max_dist_m, NULL, 1);
}

/* ------------------------------------------------------------------------------------------ */
/* G-buffer helpers: types.wgsl:108-130, 292-345                                              */
/* ------------------------------------------------------------------------------------------ */

static void oct_encode(const float n[3], float p[2]) {
    float l1 = (fabsf(n[0]) + fabsf(n[1])) + fabsf(n[2]);
    float s = 1.0f / orc_max(l1, 1e-6f);
    p[0] = n[0] * s;
    p[1] = n[1] * s;
    if (n[2] < 0.0f) {
        float wx = (1.0f - fabsf(p[1])) * (p[0] >= 0.0f ? 1.0f : -1.0f);
        float wy = (1.0f - fabsf(p[0])) * (p[1] >= 0.0f ? 1.0f : -1.0f);
        p[0] = wx;
        p[1] = wy;
    }
}

/* test hook: the octahedral encoding of n unit normals (3 floats each) into 2 floats each */
void orc_test_oct_encode(const float* nrm, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; ++i) oct_encode(nrm + 3 * i, out + 2 * i);
}

static void oct_decode(const float p[2], float out[3]) {
    float n[3] = {p[0], p[1], (1.0f - fabsf(p[0])) - fabsf(p[1])};
    if (n[2] < 0.0f) {
        float sx = p[0] >= 0.0f ? 1.0f : -1.0f, sy = p[1] >= 0.0f ? 1.0f : -1.0f;
        float wx = (1.0f - fabsf(p[1])) * sx;
        float wy = (1.0f - fabsf(p[0])) * sy;
        n[0] = wx;
        n[1] = wy;
    }
    orc_normalize3(n, out);
}

static void camera_ray_dir(const arc_camera_uniforms* cam, uint32_t px, uint32_t py, uint32_t w, uint32_t h, float d[3]) {
    float u = (((float)px + 0.5f) + cam->jitter_brush_dt[0]) / (float)w;
    float v = (((float)py + 0.5f) + cam->jitter_brush_dt[1]) / (float)h;
    float nx = u * 2.0f - 1.0f;
    float ny = 1.0f - v * 2.0f;
    float th = cam->cam_forward_fov[3];
    float sx = (nx * cam->cam_right_aspect[3]) * th;
    float sy = ny * th;
    float r[3];
    for (int i = 0; i < 3; ++i) r[i] = (cam->cam_forward_fov[i] + cam->cam_right_aspect[i] * sx) + cam->cam_up_frame[i] * sy;
    orc_normalize3(r, d);
}

static void fill_hit_record(const orc_trace_out* r, float t_scale_m, arc_hit_record* h) {
    if (r->hit) {
        h->voxel[0] = (int32_t)r->vi[0];
        h->voxel[1] = (int32_t)r->vi[1];
        h->voxel[2] = (int32_t)r->vi[2];
        h->face = (uint8_t)orc_face_id(r->normal);
        h->mat = (uint8_t)r->mat_id;
        h->flags = (uint16_t)(ARC_HIT_FLAG_HIT | ((r->shift >> 1) << 1));
    } else {
        h->voxel[0] = h->voxel[1] = h->voxel[2] = -1;
        h->face = ARC_FACE_NONE;
        h->mat = 0;
        h->flags = 0;
    }
    h->depth_m = r->t_voxels * t_scale_m;
}

/* primary_raymarch (primary_gbuffer.wgsl:93-312) for pixels [x0,x1) x [y0,y1); no rigid bodies.
 * The underwater / water / mirror shading branches are orc_surface_shade (orc_surface.c). */
static void primary_pixel(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x, uint32_t y, uint32_t W,
                          uint32_t H, uint32_t out[5], arc_hit_record* hit, uint32_t* bytes) {
    float d[3];
    camera_ray_dir(cam, x, y, W, H, d);
    const float* eye = cam->cam_pos_time;
    int underwater = (cam->point_light_count[1] & 0xFFFFu) != 0u;
    orc_trace_out r;
    orc_trace(w, cam, eye, d, 0.0f, 250.0f, 0u, underwater, &r);
    *bytes += r.bytes + 20u + 20u;
    /* rigid bodies in front of the world hit (primary_gbuffer.wgsl:123-136) */
    float prev_pos[3] = {r.hit_pos_m[0], r.hit_pos_m[1], r.hit_pos_m[2]};
    int rigid = 0;
    uint32_t body = 0;
    if (orc_rigid_count(w, cam) > 0u) {
        orc_rigid_out rb;
        orc_trace_rigid_bodies(w, cam, eye, d, r.hit ? r.t_voxels * ARC_VOXEL_SIZE : 250.0f, &rb);
        if (rb.hit) {
            r.hit = 1;
            r.t_voxels = rb.t_voxels;
            memcpy(r.hit_pos_m, rb.hit_pos_m, sizeof(r.hit_pos_m));
            memcpy(r.normal, rb.normal, sizeof(r.normal));
            r.mat_id = rb.mat_id;
            r.voxel_hash = rb.voxel_hash;
            r.contact_ao = rb.contact_ao;
            memcpy(r.vi, rb.vi, sizeof(r.vi));
            r.shift = rb.shift;
            memcpy(prev_pos, rb.prev_hit_pos_m, sizeof(prev_pos));
            rigid = 1;
            body = rb.body;
        }
    }
    if (hit) {
        fill_hit_record(&r, ARC_VOXEL_SIZE, hit);
        if (rigid) hit->flags = (uint16_t)(hit->flags | ARC_HIT_FLAG_RIGID | (body << 8));
    }
    if (!r.hit) {
        float p[2];
        oct_encode(d, p);
        out[0] = orc_fbits(1e5f);
        out[1] = 0u;
        out[2] = orc_pack2x16snorm(p[0], p[1]);
        out[3] = orc_pack2x16float(0.0f, 0.0f);
        out[4] = orc_pack4x8unorm(0.0f, 0.0f, 0.0f, 1.0f);
        return;
    }
    float hit_dist = r.t_voxels * ARC_VOXEL_SIZE;
    const arc_material* m = &w->palette[r.mat_id];
    float vrw = 1.0f - orc_smoothstep(18.0f, 48.0f, hit_dist);
    float vr = (((float)(r.voxel_hash & 0xFFu) / 255.0f) * 2.0f - 1.0f) * vrw;
    float alb[3];
    for (int i = 0; i < 3; ++i) alb[i] = orc_clamp(m->albedo_roughness[i] * (1.0f + vr * m->emission_meta[3]), 0.01f, 1.0f);
    /* motion: primary_gbuffer.wgsl:298-305 */
    float pu = ((float)x + 0.5f) / (float)W, pv = ((float)y + 0.5f) / (float)H;
    const float* M = cam->prev_view_proj;
    float hp[4] = {prev_pos[0], prev_pos[1], prev_pos[2], 1.0f};
    float clip[4];
    for (int row = 0; row < 4; ++row)
        clip[row] = ((M[0 * 4 + row] * hp[0] + M[1 * 4 + row] * hp[1]) + M[2 * 4 + row] * hp[2]) + M[3 * 4 + row] * hp[3];
    float mx = -2.0f, my = -2.0f;
    if (clip[3] > 0.001f) {
        float ndx = clip[0] / clip[3], ndy = clip[1] / clip[3];
        mx = (ndx * 0.5f + 0.5f) - pu;
        my = (0.5f - ndy * 0.5f) - pv;
    }
    float nrm[3] = {r.normal[0], r.normal[1], r.normal[2]};
    if (orc_surface_special(cam, r.mat_id)) orc_surface_shade(w, cam, d, &r, alb, nrm, bytes);
    float p[2];
    oct_encode(nrm, p);
    out[0] = orc_fbits(hit_dist);
    out[1] = (r.mat_id & 0xFFFFu) | ((uint32_t)rigid << 16);
    out[2] = orc_pack2x16snorm(p[0], p[1]);
    out[3] = orc_pack2x16float(mx, my);
    out[4] = orc_pack4x8unorm(alb[0], alb[1], alb[2], orc_clamp(r.contact_ao, 0.0f, 1.0f));
}

void orc_primary(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                 uint32_t* gdm, uint32_t* gnm, uint32_t* gaa, arc_hit_record* hits, uint32_t* bytes_out, int threads) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    uint32_t rw = x1 - x0;
    int64_t n = (int64_t)rw * (y1 - y0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t x = x0 + (uint32_t)(i % rw), y = y0 + (uint32_t)(i / rw);
        uint32_t o[5];
        uint32_t b = 0;
        size_t k = (size_t)y * W + x;
        primary_pixel(w, cam, x, y, W, H, o, hits ? &hits[k] : NULL, &b);
        gdm[2 * k] = o[0]; gdm[2 * k + 1] = o[1];
        gnm[2 * k] = o[2]; gnm[2 * k + 1] = o[3];
        gaa[k] = o[4];
        if (bytes_out) bytes_out[k] = b;
    }
}

/* interleaved_gradient_noise: types.wgsl:483-497 */
static void ign(float px, float py, uint32_t frame, float out[2]) {
    float f = (float)frame;
    uint32_t ux = orc_f2u(px), uy = orc_f2u(py);
    float ign1 = orc_fract(52.9829189f * orc_fract(0.06711056f * px + 0.00583715f * py));
    float ign2 = orc_fract(52.9829189f * orc_fract((0.00583715f * px - 0.06711056f * py) + 0.5f));
    uint32_t h1 = orc_pcg_hash(ux * 1973u + uy * 9277u + frame * 26699u);
    uint32_t h2 = orc_pcg_hash(h1 ^ 0x9E3779B9u);
    float r1 = (float)(h1 & 0xFFFFu) / 65536.0f;
    float r2 = (float)(h2 & 0xFFFFu) / 65536.0f;
    out[0] = orc_fract((ign1 + f * 0.754877666f) + r1);
    out[1] = orc_fract((ign2 + f * 0.569840291f) + r2);
}

/* make_basis + sample_cosine_hemisphere: types.wgsl:531-545 */
static void make_basis(const float n[3], float t[3], float b[3]) {
    float up[3] = {0.0f, 0.0f, 0.0f};
    if (fabsf(n[2]) < 0.999f) up[2] = 1.0f; else up[0] = 1.0f;
    float c[3];
    orc_cross3(up, n, c);
    orc_normalize3(c, t);
    orc_cross3(n, t, b);
}

static void sample_cosine_hemisphere(float u1, float u2, const float n[3], const float t[3], const float b[3], float out[3]) {
    float r = sqrtf(u1);
    float phi = 6.2831853f * u2;
    float z = sqrtf(orc_max(0.0f, 1.0f - u1));
    float s, c;
    orc_sincos(phi, &s, &c);
    float rc = r * c, rs = r * s;
    for (int i = 0; i < 3; ++i) out[i] = (t[i] * rc + b[i] * rs) + n[i] * z;
}

/* probe_emissive_macro_candidate: lighting_restir_gi.wgsl:20-54 */
static float probe_emissive(const orc_world* w, const arc_camera_uniforms* cam, const float pos[3], const float d[3],
                            float dist, uint32_t* bytes) {
    float vp[3];
    for (int i = 0; i < 3; ++i) vp[i] = (pos[i] + d[i] * dist) * ARC_VOXELS_PER_METER;
    const uint32_t* g = cam->world_grid_dims;
    for (int i = 0; i < 3; ++i)
        if (vp[i] < 0.0f || vp[i] >= (float)g[i] * ARC_CHUNK_DIM_F) return 0.0f;
    uint32_t vi[3] = {orc_f2u(vp[0]), orc_f2u(vp[1]), orc_f2u(vp[2])};
    uint32_t c_idx = (vi[0] >> 8) + (vi[1] >> 8) * g[0] + (vi[2] >> 8) * g[0] * g[1];
    *bytes += 4;
    uint32_t root_idx = w->roots[c_idx];
    if (root_idx == ARC_EMPTY_CHUNK) return 0.0f;
    uint32_t l[3] = {vi[0] & 255u, vi[1] & 255u, vi[2] & 255u};
    arc_node64 root = load_node(w, root_idx, bytes);
    uint32_t b0 = (((l[2] >> 6) & 3u) << 4) | (((l[1] >> 6) & 3u) << 2) | ((l[0] >> 6) & 3u);
    if (!node_has_child(root.mask_low, root.mask_high, b0)) return 0.0f;
    const float* em;
    if (root.child_ptr & ARC_IS_LEAF_FLAG) {
        em = w->palette[(root.lod_payload >> 24) & 0xFFu].emission_meta;
        return (em[0] * 0.333f + em[1] * 0.333f) + em[2] * 0.333f;
    }
    arc_node64 l1 = load_node(w, node_child_offset(&root, b0), bytes);
    uint32_t b1 = (((l[2] >> 4) & 3u) << 4) | (((l[1] >> 4) & 3u) << 2) | ((l[0] >> 4) & 3u);
    if (!node_has_child(l1.mask_low, l1.mask_high, b1)) return 0.0f;
    em = w->palette[(l1.lod_payload >> 24) & 0xFFu].emission_meta;
    return (em[0] * 0.333f + em[1] * 0.333f) + em[2] * 0.333f;
}

/* GI secondary ray of pixel (x, y) from the G-buffer (lighting_restir_gi.wgsl:69-87,195-209), with
 * the quantities temporal_main goes on to use. Returns 0 when the pixel has no primary hit. */
int orc_gi_setup(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x, uint32_t y, uint32_t W, uint32_t H,
                 uint32_t gd0, uint32_t gn0, orc_gi_ray* g, uint32_t* bytes) {
    float hit_dist = orc_bitsf(gd0);
    if (hit_dist >= 1e4f) return 0;
    g->hit_dist = hit_dist;
    camera_ray_dir(cam, x, y, W, H, g->ray_dir);
    for (int i = 0; i < 3; ++i) g->hit_pos[i] = cam->cam_pos_time[i] + g->ray_dir[i] * hit_dist;
    float oc[2];
    orc_unpack2x16snorm(gn0, oc);
    oct_decode(oc, g->normal);
    const float* n = g->normal;
    uint32_t frame = orc_fbits(cam->cam_up_frame[3]);
    ign((float)x, (float)y, frame, g->xi);
    float sn_in[3] = {n[0] + 0.0f, n[1] + 0.22f, n[2] + 0.0f};
    float bt[3], bb[3];
    orc_normalize3(sn_in, g->smooth_n);
    make_basis(g->smooth_n, bt, bb);
    float bd[3], cd[3];
    sample_cosine_hemisphere(g->xi[0], g->xi[1], g->smooth_n, bt, bb, bd);
    sample_cosine_hemisphere(orc_fract(g->xi[0] + 0.5f), orc_fract(g->xi[1] + 0.381966f), g->smooth_n, bt, bb, cd);
    float em_near = probe_emissive(w, cam, g->hit_pos, cd, 1.25f, bytes);
    float em_mid = probe_emissive(w, cam, g->hit_pos, cd, 3.0f, bytes);
    g->guided = orc_max(em_near, em_mid) > 0.25f;
    if (g->guided) memcpy(bd, cd, sizeof(bd));
    for (int i = 0; i < 3; ++i) g->origin[i] = g->hit_pos[i] + n[i] * 0.10f;
    memcpy(g->dir, bd, sizeof(bd));
    return 1;
}

static int gi_ray_for_pixel(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x, uint32_t y, uint32_t W,
                            uint32_t H, uint32_t gd0, uint32_t gn0, float origin[3], float dir[3], uint32_t* bytes) {
    orc_gi_ray g;
    if (!orc_gi_setup(w, cam, x, y, W, H, gd0, gn0, &g, bytes)) return 0;
    memcpy(origin, g.origin, sizeof(g.origin));
    memcpy(dir, g.dir, sizeof(g.dir));
    return 1;
}

void orc_ign(float px, float py, uint32_t frame, float out[2]) { ign(px, py, frame, out); }

void orc_oct_decode_packed(uint32_t packed, float n[3]) {
    float oc[2];
    orc_unpack2x16snorm(packed, oc);
    oct_decode(oc, n);
}

void orc_gi_rays(const orc_world* w, const arc_camera_uniforms* cam, uint32_t x0, uint32_t y0, uint32_t x1, uint32_t y1,
                 const uint32_t* gdm, const uint32_t* gnm, arc_ray* gi_rays_out, arc_hit_record* gi_hits,
                 uint32_t* bytes_out, int threads) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    uint32_t rw = x1 - x0;
    int64_t n = (int64_t)rw * (y1 - y0);
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < n; ++i) {
        uint32_t x = x0 + (uint32_t)(i % rw), y = y0 + (uint32_t)(i / rw);
        size_t k = (size_t)y * W + x;
        float o[3], d[3];
        uint32_t b = 0;
        arc_hit_record hr;
        if (gi_ray_for_pixel(w, cam, x, y, W, H, gdm[2 * k], gnm[2 * k], o, d, &b)) {
            orc_trace_out r;
            int body = orc_trace_scene(w, cam, o, d, cam->ray_distances[2], 2u, 1, &r);
            b += r.bytes + 20u;
            fill_hit_record(&r, ARC_VOXEL_SIZE, &hr);
            if (body >= 0) hr.flags = (uint16_t)(hr.flags | ARC_HIT_FLAG_RIGID | ((uint32_t)body << 8));
            if (gi_rays_out) {
                memcpy(gi_rays_out[k].origin_m, o, sizeof(o));
                memcpy(gi_rays_out[k].dir, d, sizeof(d));
            }
        } else {
            memset(&hr, 0, sizeof(hr));
            hr.voxel[0] = hr.voxel[1] = hr.voxel[2] = -1;
            hr.face = ARC_FACE_NONE;
            hr.depth_m = 0.0f;
            if (gi_rays_out) memset(&gi_rays_out[k], 0, sizeof(arc_ray));
        }
        if (gi_hits) gi_hits[k] = hr;
        if (bytes_out) bytes_out[k] = b;
    }
}

void orc_trace_rays(const orc_world* w, const arc_camera_uniforms* cam, const arc_ray* rays, uint32_t n, float max_dist_m,
                    uint32_t lod_bias, int ignore_water, arc_hit_record* hits, uint32_t* bytes_out, int threads) {
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        orc_trace_out r;
        orc_trace(w, cam, rays[i].origin_m, rays[i].dir, 0.0f, max_dist_m, lod_bias, ignore_water, &r);
        fill_hit_record(&r, ARC_VOXEL_SIZE, &hits[i]);
        if (bytes_out) bytes_out[i] = r.bytes + 20u;
    }
}

uint64_t orc_last_sample_bytes = 0;

uint64_t orc_frame_sample(const orc_world* w, const arc_camera_uniforms* cam, uint32_t stride, int threads,
                          uint64_t* n_primary, uint64_t* n_gi, uint64_t* checksum) {
    uint32_t W = cam->world_grid_dims[3] & 0xFFFFu, H = cam->world_grid_dims[3] >> 16;
    uint64_t total = (uint64_t)W * H;
    uint64_t ns = (total + stride - 1) / stride;
    uint64_t np = 0, ng = 0, cs = 0, by = 0;
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1) reduction(+ : np, ng, cs, by)
    for (int64_t s = 0; s < (int64_t)ns; ++s) {
        uint64_t k = (uint64_t)s * stride;
        uint32_t x = (uint32_t)(k % W), y = (uint32_t)(k / W);
        uint32_t o[5];
        uint32_t b = 0;
        arc_hit_record hr;
        primary_pixel(w, cam, x, y, W, H, o, &hr, &b);
        np += 1;
        cs += o[0] ^ (o[1] << 7);
        float go[3], gd[3];
        if (gi_ray_for_pixel(w, cam, x, y, W, H, o[0], o[2], go, gd, &b)) {
            orc_trace_out r;
            orc_trace(w, cam, go, gd, 0.0f, cam->ray_distances[2], 2u, 1, &r);
            ng += 1;
            b += r.bytes + 20u;
            cs += r.mat_id + (r.vi[0] ^ r.vi[1] ^ r.vi[2]);
        }
        by += b;
    }
    *n_primary = np;
    *n_gi = ng;
    *checksum = cs;
    orc_last_sample_bytes = by;
    return np + ng;
}

/* FP64 plane-entry distance of the cell along the ray, in voxels, clamped at 0. */
double orc_depth_fp64(const float origin_m[3], const float dir[3], const int32_t cell_min[3], uint32_t span) {
    double best = -1e300;
    for (int i = 0; i < 3; ++i) {
        double o = (double)origin_m[i] * 16.0;
        double d = fabsf(dir[i]) < 1e-7f ? 1e-7 : (double)dir[i];
        double e = d >= 0.0 ? (double)cell_min[i] : (double)cell_min[i] + (double)span;
        double t = (e - o) / d;
        if (t > best) best = t;
    }
    return best > 0.0 ? best : 0.0;
}
