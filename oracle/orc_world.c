/*
 * orc_world.c — oracle restatement of the world side of the path: the synthetic scene, the
 * recursive 64-tree builder, BFS packing and the Morton-ordered GPU pool flatten.
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h).
 */
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include "orc.h"
#include "orc_math.h"

/* ------------------------------------------------------------------------------------------ */
/* Default palette: crates/arcadia-core/src/material.rs:99-204.                              */
/* ------------------------------------------------------------------------------------------ */

static void set_mat(arc_material* m, float r, float g, float b, float rough, float er, float eg, float eb, float var) {
    m->albedo_roughness[0] = r; m->albedo_roughness[1] = g; m->albedo_roughness[2] = b; m->albedo_roughness[3] = rough;
    m->emission_meta[0] = er; m->emission_meta[1] = eg; m->emission_meta[2] = eb; m->emission_meta[3] = var;
}

void orc_default_palette(arc_material out[256]) {
    memset(out, 0, 256 * sizeof(arc_material));
    set_mat(&out[0], 0.0f, 0.0f, 0.0f, 1.0f, 0, 0, 0, 0.0f);
    set_mat(&out[1], 0.10f, 0.11f, 0.13f, 0.90f, 0, 0, 0, 0.03f);
    set_mat(&out[2], 0.28f, 0.30f, 0.34f, 0.85f, 0, 0, 0, 0.05f);
    set_mat(&out[3], 0.58f, 0.54f, 0.47f, 0.80f, 0, 0, 0, 0.06f);
    set_mat(&out[4], 0.46f, 0.45f, 0.40f, 0.88f, 0, 0, 0, 0.08f);
    set_mat(&out[5], 0.36f, 0.40f, 0.45f, 0.72f, 0, 0, 0, 0.05f);
    set_mat(&out[6], 0.48f, 0.52f, 0.57f, 0.65f, 0, 0, 0, 0.04f);
    set_mat(&out[7], 0.34f, 0.23f, 0.15f, 0.92f, 0, 0, 0, 0.06f);
    set_mat(&out[8], 0.22f, 0.52f, 0.18f, 0.78f, 0, 0, 0, 0.08f);
    set_mat(&out[9], 0.46f, 0.58f, 0.20f, 0.78f, 0, 0, 0, 0.08f);
    set_mat(&out[10], 0.16f, 0.46f, 0.22f, 0.85f, 0, 0, 0, 0.09f);
    set_mat(&out[11], 0.11f, 0.32f, 0.15f, 0.88f, 0, 0, 0, 0.06f);
    set_mat(&out[12], 0.68f, 0.60f, 0.46f, 0.82f, 0, 0, 0, 0.07f);
    set_mat(&out[13], 0.27f, 0.18f, 0.12f, 0.88f, 0, 0, 0, 0.06f);
    set_mat(&out[14], 0.48f, 0.33f, 0.20f, 0.75f, 0, 0, 0, 0.05f);
    set_mat(&out[15], 0.15f, 0.44f, 0.18f, 0.70f, 0, 0, 0, 0.10f);
    set_mat(&out[16], 0.76f, 0.36f, 0.11f, 0.70f, 0, 0, 0, 0.10f);
    set_mat(&out[17], 0.85f, 0.48f, 0.58f, 0.72f, 0, 0, 0, 0.08f);
    set_mat(&out[18], 0.06f, 0.28f, 0.38f, 0.05f, 0, 0, 0, 0.02f);
    set_mat(&out[19], 0.15f, 0.85f, 1.00f, 0.15f, 0.20f, 2.40f, 3.60f, 0.05f);
    set_mat(&out[20], 0.95f, 0.20f, 0.80f, 0.15f, 3.20f, 0.25f, 2.50f, 0.05f);
    set_mat(&out[21], 1.00f, 0.68f, 0.15f, 0.15f, 3.40f, 1.75f, 0.15f, 0.05f);
    set_mat(&out[22], 1.00f, 0.30f, 0.04f, 0.30f, 4.20f, 1.10f, 0.08f, 0.10f);
    set_mat(&out[23], 0.10f, 0.09f, 0.08f, 0.95f, 0, 0, 0, 0.05f);
    set_mat(&out[24], 0.95f, 0.25f, 0.04f, 0.50f, 3.20f, 0.75f, 0.05f, 0.12f);
    set_mat(&out[25], 0.82f, 0.80f, 0.75f, 0.35f, 0, 0, 0, 0.03f);
    set_mat(&out[26], 0.85f, 0.68f, 0.24f, 0.25f, 0, 0, 0, 0.04f);
    set_mat(&out[27], 1.00f, 0.97f, 0.90f, 0.05f, 116.00f, 114.50f, 111.80f, 0.02f);
    set_mat(&out[28], 0.92f, 0.95f, 0.98f, 0.02f, 0, 0, 0, 0.01f);
    for (int i = 29; i < 256; ++i) {
        float t = (float)i / 255.0f;
        set_mat(&out[i], 0.3f + 0.4f * fabsf(sinf(t * 6.28318531f)), 0.3f + 0.4f * fabsf(cosf(t * 3.0f * 3.14159265f)),
                0.3f + 0.3f * t, 0.75f, 0, 0, 0, 0.05f);
    }
}

static int mat_is_emissive(const arc_material* m) {
    return m->emission_meta[0] > 0.01f || m->emission_meta[1] > 0.01f || m->emission_meta[2] > 0.01f;
}

/* Material::pack_lod_payload (material.rs:70-75). */
static uint32_t pack_lod_payload(const arc_material* m, uint32_t mat) {
    uint32_t r = orc_f2u(orc_clamp(m->albedo_roughness[0], 0.0f, 1.0f) * 255.0f);
    uint32_t g = orc_f2u(orc_clamp(m->albedo_roughness[1], 0.0f, 1.0f) * 255.0f);
    uint32_t b = orc_f2u(orc_clamp(m->albedo_roughness[2], 0.0f, 1.0f) * 255.0f);
    return (mat << 24) | (b << 16) | (g << 8) | r;
}

uint32_t orc_pack_lod_payload(const arc_material* m, uint32_t mat) { return pack_lod_payload(m, mat); }
int orc_mat_is_emissive(const arc_material* m) { return mat_is_emissive(m); }

/* pack_rgb_and_mat (builder.rs:72-78). */
static uint32_t pack_rgb_and_mat(float r, float g, float b, uint32_t mat) {
    uint32_t ru = orc_f2u(orc_clamp(r, 0.0f, 1.0f) * 255.0f);
    uint32_t gu = orc_f2u(orc_clamp(g, 0.0f, 1.0f) * 255.0f);
    uint32_t bu = orc_f2u(orc_clamp(b, 0.0f, 1.0f) * 255.0f);
    return (mat << 24) | (bu << 16) | (gu << 8) | ru;
}

uint32_t orc_pack_rgb_and_mat(float r, float g, float b, uint32_t mat) { return pack_rgb_and_mat(r, g, b, mat); }

/* ------------------------------------------------------------------------------------------ */
/* Synthetic scene: seeded 2D value-noise heightfield + 3D value-noise caves.                  */
/* Hash/value-noise/fbm in the style of generator.rs:656-694 with a seed mixed into the hash.  */
/* ------------------------------------------------------------------------------------------ */

/* The reference hash2 shifts an i32 arithmetically, which clears bit 31 of its result and halves
 * its range; the synthetic scene shifts logically so its values cover [0, 1). */
static float hash2s(int32_t x, int32_t z, uint32_t seed) {
    uint32_t n = (uint32_t)x * 374761393u + (uint32_t)z * 668265263u + seed * 0x27D4EB2Du;
    n = (n ^ (n >> 13)) * 1274126177u;
    return (float)(n ^ (n >> 16)) / 4294967296.0f;
}

static uint32_t hash3u(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t n = (uint32_t)x * 374761393u + (uint32_t)y * 1103515245u + (uint32_t)z * 668265263u + seed * 0x27D4EB2Du;
    n = (n ^ (n >> 13)) * 1274126177u;
    return n ^ (n >> 16);
}

static float value_noise2(float x, float z, uint32_t seed) {
    float flx = floorf(x), flz = floorf(z);
    int32_t ix = (int32_t)flx, iz = (int32_t)flz;
    float fx = x - flx, fz = z - flz;
    float ux = fx * fx * (3.0f - 2.0f * fx);
    float uz = fz * fz * (3.0f - 2.0f * fz);
    float v00 = hash2s(ix, iz, seed), v10 = hash2s(ix + 1, iz, seed);
    float v01 = hash2s(ix, iz + 1, seed), v11 = hash2s(ix + 1, iz + 1, seed);
    float a = v00 + ux * (v10 - v00);
    float b = v01 + ux * (v11 - v01);
    return a + uz * (b - a);
}

static float fbm2(float x, float z, uint32_t octaves, uint32_t seed) {
    float sum = 0.0f, amp = 0.5f;
    for (uint32_t i = 0; i < octaves; ++i) {
        sum += (value_noise2(x, z, seed) * 2.0f - 1.0f) * amp;
        x *= 2.03f;
        z *= 2.03f;
        amp *= 0.5f;
    }
    return sum;
}

/* Terrain height (voxels; solid below) of column (x, z). */
static float scene_height(const orc_scene_params* p, uint32_t x, uint32_t z) {
    float wx = (float)(p->grid[0] * 256u);
    float wy = (float)(p->grid[1] * 256u);
    float freq = 2.0f / wx;
    float f = fbm2(((float)x + 0.5f) * freq, ((float)z + 0.5f) * freq, 4u, p->seed);
    float h01 = orc_clamp(0.5f + 1.5f * f, 0.0f, 1.0f);
    float lo = p->height_lo * wy, hi = p->height_hi * wy;
    return floorf(lo + (hi - lo) * h01);
}

void orc_scene_heightmap(const orc_scene_params* p, float* out) {
    uint32_t wx = p->grid[0] * 256u, wz = p->grid[2] * 256u;
    for (uint32_t z = 0; z < wz; ++z)
        for (uint32_t x = 0; x < wx; ++x) out[(size_t)z * wx + x] = scene_height(p, x, z);
}

/* Trilinear value noise on a (1 << lg)-voxel lattice, sampled at voxel centres. */
static float lattice_noise3(uint32_t x, uint32_t y, uint32_t z, uint32_t lg, uint32_t seed) {
    uint32_t m = (1u << lg) - 1u;
    float inv = 1.0f / (float)(1u << lg);
    int32_t ix = (int32_t)(x >> lg), iy = (int32_t)(y >> lg), iz = (int32_t)(z >> lg);
    float fx = ((float)(x & m) + 0.5f) * inv;
    float fy = ((float)(y & m) + 0.5f) * inv;
    float fz = ((float)(z & m) + 0.5f) * inv;
    float ux = fx * fx * (3.0f - 2.0f * fx);
    float uy = fy * fy * (3.0f - 2.0f * fy);
    float uz = fz * fz * (3.0f - 2.0f * fz);
    float c[8];
    for (int k = 0; k < 8; ++k)
        c[k] = (float)hash3u(ix + (k & 1), iy + ((k >> 1) & 1), iz + ((k >> 2) & 1), seed) / 4294967296.0f;
    float x00 = c[0] + ux * (c[1] - c[0]);
    float x10 = c[2] + ux * (c[3] - c[2]);
    float x01 = c[4] + ux * (c[5] - c[4]);
    float x11 = c[6] + ux * (c[7] - c[6]);
    float y0 = x00 + uy * (x10 - x00);
    float y1 = x01 + uy * (x11 - x01);
    return y0 + uz * (y1 - y0);
}

/* Cave noise: mean of a 32-voxel and a 16-voxel lattice octave. */
static float cave_noise(uint32_t x, uint32_t y, uint32_t z, uint32_t seed) {
    float a = lattice_noise3(x, y, z, 5u, seed ^ 0x5BD1E995u);
    float b = lattice_noise3(x, y, z, 4u, seed ^ 0x1B873593u);
    return (a + b) * 0.5f;
}

uint32_t orc_scene_voxel(const orc_scene_params* p, const float* hm, uint32_t x, uint32_t y, uint32_t z) {
    uint32_t wx = p->grid[0] * 256u;
    float h = hm[(size_t)z * wx + x];
    if (!((float)y < h)) return ARC_MAT_AIR;
    int32_t depth = (int32_t)h - 1 - (int32_t)y;
    if (p->caves && (p->cave_depth == 0u || depth < (int32_t)p->cave_depth) &&
        cave_noise(x, y, z, p->seed) > p->cave_threshold)
        return ARC_MAT_AIR;
    if (depth < 3) return 1u + (hash3u((int32_t)x, (int32_t)y, (int32_t)z, p->seed ^ 0xA511E9B3u) & 15u);
    return 1u + (hash3u((int32_t)(x >> 4), (int32_t)(y >> 4), (int32_t)(z >> 4), p->seed ^ 0x63D83595u) & 15u);
}

/* ------------------------------------------------------------------------------------------ */
/* build_recursive / pack_build_tree (builder.rs:106-378)                                      */
/* ------------------------------------------------------------------------------------------ */

enum { BN_EMPTY = 0, BN_UNIFORM = 1, BN_MIXED = 2, BN_INTERNAL = 3 };

typedef struct bnode {
    uint8_t kind;
    uint8_t mat;
    uint8_t fully_solid;
    uint64_t mask;
    uint32_t lod;
    arc_brick64* brick;
    uint32_t n_children;
    struct bnode* children;
} bnode;

typedef struct build_ctx {
    const arc_material* palette;
    /* voxel source */
    const orc_scene_params* scene;
    const float* heightmap;
    const uint8_t* dense; /* 256^3 chunk volume, or NULL */
    uint32_t chunk_org[3];
    uint32_t solid_count;
} build_ctx;

static uint32_t ctx_eval(build_ctx* c, uint32_t x, uint32_t y, uint32_t z) {
    if (c->dense) return c->dense[((size_t)z * 256u + y) * 256u + x];
    return orc_scene_voxel(c->scene, c->heightmap, c->chunk_org[0] + x, c->chunk_org[1] + y, c->chunk_org[2] + z);
}

/* Region hint: all-air when the whole region lies at or above the tallest column of its footprint. */
static int ctx_hint_air(build_ctx* c, uint32_t ox, uint32_t oy, uint32_t oz, uint32_t size) {
    if (c->dense) return 0;
    uint32_t wx = c->scene->grid[0] * 256u;
    float maxh = -1.0f;
    for (uint32_t z = 0; z < size; ++z)
        for (uint32_t x = 0; x < size; ++x) {
            float h = c->heightmap[(size_t)(c->chunk_org[2] + oz + z) * wx + (c->chunk_org[0] + ox + x)];
            if (h > maxh) maxh = h;
        }
    return (float)(c->chunk_org[1] + oy) >= maxh;
}

static void brick_set(arc_brick64* b, uint32_t bit, uint32_t mat) {
    uint32_t w = bit >> 2, sh = (bit & 3u) * 8u;
    b->packed_materials[w] = (b->packed_materials[w] & ~(0xFFu << sh)) | (mat << sh);
}

static uint32_t child_bit(uint32_t x, uint32_t y, uint32_t z) { return (z << 4) | (y << 2) | x; }

static bnode build_recursive(build_ctx* c, uint32_t ox, uint32_t oy, uint32_t oz, uint32_t shift) {
    bnode out;
    memset(&out, 0, sizeof(out));
    uint32_t node_size = 4u << shift;
    if (ctx_hint_air(c, ox, oy, oz, node_size)) return out;

    if (shift == 0) {
        uint64_t mask = 0;
        arc_brick64 brick;
        memset(&brick, 0, sizeof(brick));
        uint32_t first_mat = ARC_MAT_AIR;
        int all_same = 1;
        float r_sum = 0.0f, g_sum = 0.0f, b_sum = 0.0f;
        uint32_t emissive_mat = ARC_MAT_AIR, emissive_voxels = 0;
        for (uint32_t lz = 0; lz < 4; ++lz)
            for (uint32_t ly = 0; ly < 4; ++ly)
                for (uint32_t lx = 0; lx < 4; ++lx) {
                    uint32_t mat = ctx_eval(c, ox + lx, oy + ly, oz + lz);
                    if (mat != ARC_MAT_AIR) {
                        uint32_t b = child_bit(lx, ly, lz);
                        mask |= 1ull << b;
                        brick_set(&brick, b, mat);
                        if (first_mat == ARC_MAT_AIR) first_mat = mat;
                        else if (mat != first_mat) all_same = 0;
                        const arc_material* m = &c->palette[mat];
                        r_sum += orc_min(m->albedo_roughness[0] + m->emission_meta[0] * 0.25f, 1.0f);
                        g_sum += orc_min(m->albedo_roughness[1] + m->emission_meta[1] * 0.25f, 1.0f);
                        b_sum += orc_min(m->albedo_roughness[2] + m->emission_meta[2] * 0.25f, 1.0f);
                        if (mat_is_emissive(m)) { emissive_mat = mat; emissive_voxels++; }
                    }
                }
        if (mask == 0) return out;
        uint32_t count = (uint32_t)__builtin_popcountll(mask);
        c->solid_count += count;
        if (all_same) {
            out.kind = BN_UNIFORM;
            out.mask = mask;
            out.mat = (uint8_t)first_mat;
            out.lod = pack_lod_payload(&c->palette[first_mat], first_mat);
            out.fully_solid = mask == ~0ull;
            return out;
        }
        float inv = 1.0f / (float)count;
        uint32_t rep = (emissive_mat != ARC_MAT_AIR && emissive_voxels * 2u >= count) ? emissive_mat : first_mat;
        out.kind = BN_MIXED;
        out.mask = mask;
        out.lod = pack_rgb_and_mat(r_sum * inv, g_sum * inv, b_sum * inv, rep);
        out.brick = (arc_brick64*)malloc(sizeof(arc_brick64));
        *out.brick = brick;
        return out;
    }

    uint32_t child_size = 1u << shift;
    uint64_t mask = 0;
    bnode kids[64];
    uint32_t nk = 0;
    int all_full = 1;
    uint32_t common_mat = ARC_MAT_AIR;
    uint32_t r_sum = 0, g_sum = 0, b_sum = 0;
    uint32_t solid_mat = ARC_MAT_AIR, emissive_mat = ARC_MAT_AIR, emissive_children = 0;
    for (uint32_t cz = 0; cz < 4; ++cz)
        for (uint32_t cy = 0; cy < 4; ++cy)
            for (uint32_t cx = 0; cx < 4; ++cx) {
                bnode ch = build_recursive(c, ox + cx * child_size, oy + cy * child_size, oz + cz * child_size, shift - 2);
                if (ch.kind == BN_EMPTY) continue;
                uint32_t b = child_bit(cx, cy, cz);
                mask |= 1ull << b;
                r_sum += ch.lod & 0xFFu;
                g_sum += (ch.lod >> 8) & 0xFFu;
                b_sum += (ch.lod >> 16) & 0xFFu;
                uint32_t c_mat = ch.lod >> 24;
                if (mat_is_emissive(&c->palette[c_mat])) { emissive_mat = c_mat; emissive_children++; }
                else if (solid_mat == ARC_MAT_AIR) solid_mat = c_mat;
                if (ch.kind == BN_UNIFORM && ch.fully_solid) {
                    if (common_mat == ARC_MAT_AIR) common_mat = ch.mat;
                    else if (common_mat != ch.mat) all_full = 0;
                } else {
                    all_full = 0;
                }
                kids[nk++] = ch;
            }
    if (mask == 0) return out;
    if (all_full && common_mat != ARC_MAT_AIR) {
        for (uint32_t i = 0; i < nk; ++i) free(kids[i].brick); /* uniform children own nothing */
        out.kind = BN_UNIFORM;
        out.mask = mask;
        out.mat = (uint8_t)common_mat;
        out.lod = pack_lod_payload(&c->palette[common_mat], common_mat);
        out.fully_solid = mask == ~0ull;
        return out;
    }
    uint32_t count = nk;
    uint32_t dominant = (emissive_mat != ARC_MAT_AIR && (emissive_children * 2u >= count || solid_mat == ARC_MAT_AIR))
                            ? emissive_mat
                            : solid_mat;
    out.kind = BN_INTERNAL;
    out.mask = mask;
    out.lod = (dominant << 24) | (((b_sum / count) & 0xFFu) << 16) | (((g_sum / count) & 0xFFu) << 8) | ((r_sum / count) & 0xFFu);
    out.n_children = nk;
    out.children = (bnode*)malloc(sizeof(bnode) * nk);
    memcpy(out.children, kids, sizeof(bnode) * nk);
    return out;
}

static void bnode_free(bnode* b) {
    if (b->kind == BN_INTERNAL) {
        for (uint32_t i = 0; i < b->n_children; ++i) bnode_free(&b->children[i]);
        free(b->children);
    }
    free(b->brick);
}

typedef struct vec_nodes { arc_node64* d; uint32_t n, cap; } vec_nodes;
typedef struct vec_bricks { arc_brick64* d; uint32_t n, cap; } vec_bricks;

static void vn_resize(vec_nodes* v, uint32_t n) {
    if (n > v->cap) {
        uint32_t cap = v->cap ? v->cap : 256;
        while (cap < n) cap *= 2;
        v->d = (arc_node64*)realloc(v->d, sizeof(arc_node64) * cap);
        v->cap = cap;
    }
    for (uint32_t i = v->n; i < n; ++i) memset(&v->d[i], 0, sizeof(arc_node64));
    v->n = n;
}
static void vb_push(vec_bricks* v, const arc_brick64* b) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 128;
        v->d = (arc_brick64*)realloc(v->d, sizeof(arc_brick64) * v->cap);
    }
    v->d[v->n++] = *b;
}

static arc_node64 node_from(uint64_t mask, uint32_t ptr, uint32_t lod) {
    arc_node64 n;
    n.mask_low = (uint32_t)mask;
    n.mask_high = (uint32_t)(mask >> 32);
    n.child_ptr = ptr;
    n.lod_payload = lod;
    return n;
}

/* pack_build_tree: BFS level order, children of a node contiguous. */
static void pack_build_tree(const bnode* root, vec_nodes* nodes, vec_bricks* bricks) {
    nodes->n = 0;
    bricks->n = 0;
    vn_resize(nodes, 1);
    if (root->kind == BN_EMPTY) return;
    uint32_t qcap = 1024, qh = 0, qt = 0;
    struct qe { uint32_t slot; const bnode* b; }* q = (struct qe*)malloc(sizeof(struct qe) * qcap);
    q[qt++] = (struct qe){0, root};
    while (qh < qt) {
        struct qe e = q[qh++];
        const bnode* b = e.b;
        if (b->kind == BN_EMPTY) {
            memset(&nodes->d[e.slot], 0, sizeof(arc_node64));
        } else if (b->kind == BN_UNIFORM) {
            nodes->d[e.slot] = node_from(b->mask, ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG, b->lod);
        } else if (b->kind == BN_MIXED) {
            uint32_t bi = bricks->n;
            vb_push(bricks, b->brick);
            nodes->d[e.slot] = node_from(b->mask, ARC_IS_LEAF_FLAG | bi, b->lod);
        } else {
            uint32_t base = nodes->n;
            vn_resize(nodes, nodes->n + b->n_children);
            nodes->d[e.slot] = node_from(b->mask, base, b->lod);
            if (qt + b->n_children > qcap) {
                while (qt + b->n_children > qcap) qcap *= 2;
                q = (struct qe*)realloc(q, sizeof(struct qe) * qcap);
            }
            for (uint32_t i = 0; i < b->n_children; ++i) q[qt++] = (struct qe){base + i, &b->children[i]};
        }
    }
    free(q);
}

int orc_build_chunk_dense(const uint8_t* vol, const arc_material* palette, arc_node64* nodes_out, uint32_t* n_nodes,
                          arc_brick64* bricks_out, uint32_t* n_bricks) {
    build_ctx c;
    memset(&c, 0, sizeof(c));
    c.palette = palette;
    c.dense = vol;
    bnode root = build_recursive(&c, 0, 0, 0, 6);
    vec_nodes vn = {0};
    vec_bricks vb = {0};
    pack_build_tree(&root, &vn, &vb);
    bnode_free(&root);
    if (nodes_out) memcpy(nodes_out, vn.d, sizeof(arc_node64) * vn.n);
    if (bricks_out && vb.n) memcpy(bricks_out, vb.d, sizeof(arc_brick64) * vb.n);
    *n_nodes = vn.n;
    *n_bricks = vb.n;
    free(vn.d);
    free(vb.d);
    return 0;
}

/* ------------------------------------------------------------------------------------------ */
/* rebuild_all_gpu_pools (world_map.rs:158-205), morton3d (689-702), relocate (705-735)        */
/* ------------------------------------------------------------------------------------------ */

static uint32_t part1by2(uint32_t n) {
    n &= 0x000003FFu;
    n = (n ^ (n << 16)) & 0xFF0000FFu;
    n = (n ^ (n << 8)) & 0x0300F00Fu;
    n = (n ^ (n << 4)) & 0x030C30C3u;
    n = (n ^ (n << 2)) & 0x09249249u;
    return n;
}

uint32_t orc_morton3d(uint32_t x, uint32_t y, uint32_t z) { return part1by2(x) | (part1by2(y) << 1) | (part1by2(z) << 2); }

typedef struct chunk_tree { vec_nodes nodes; vec_bricks bricks; uint32_t solid; } chunk_tree;

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : x > y;
}

int orc_build_world(const orc_scene_params* p, orc_pools* out) {
    memset(out, 0, sizeof(*out));
    arc_material palette[256];
    orc_default_palette(palette);
    uint32_t gx = p->grid[0], gy = p->grid[1], gz = p->grid[2];
    uint32_t nch = gx * gy * gz;
    size_t wx = (size_t)gx * 256u, wz = (size_t)gz * 256u;
    float* hm = (float*)malloc(sizeof(float) * wx * wz);
    orc_scene_heightmap(p, hm);
    chunk_tree* trees = (chunk_tree*)calloc(nch, sizeof(chunk_tree));
    uint64_t solid = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : solid)
    for (int64_t idx = 0; idx < (int64_t)nch; ++idx) {
        uint32_t u = (uint32_t)idx;
        build_ctx c;
        memset(&c, 0, sizeof(c));
        c.palette = palette;
        c.scene = p;
        c.heightmap = hm;
        c.chunk_org[0] = (u % gx) * 256u;
        c.chunk_org[1] = ((u / gx) % gy) * 256u;
        c.chunk_org[2] = (u / (gx * gy)) * 256u;
        bnode root = build_recursive(&c, 0, 0, 0, 6);
        pack_build_tree(&root, &trees[idx].nodes, &trees[idx].bricks);
        bnode_free(&root);
        trees[idx].solid = c.solid_count;
        solid += c.solid_count;
    }
    free(hm);

    uint64_t* order = (uint64_t*)malloc(sizeof(uint64_t) * nch);
    for (uint32_t i = 0; i < nch; ++i)
        order[i] = ((uint64_t)orc_morton3d(i % gx, (i / gx) % gy, i / (gx * gy)) << 32) | i;
    qsort(order, nch, sizeof(uint64_t), cmp_u64);

    uint64_t total_nodes = 1, total_bricks = 1;
    for (uint32_t i = 0; i < nch; ++i) {
        if (trees[i].nodes.d[0].mask_low == 0 && trees[i].nodes.d[0].mask_high == 0) continue;
        total_nodes += trees[i].nodes.n;
        total_bricks += trees[i].bricks.n;
    }
    out->grid[0] = gx; out->grid[1] = gy; out->grid[2] = gz;
    out->n_chunks = nch;
    out->roots = (uint32_t*)malloc(sizeof(uint32_t) * nch);
    out->nodes = (arc_node64*)malloc(sizeof(arc_node64) * total_nodes);
    out->bricks = (arc_brick64*)malloc(sizeof(arc_brick64) * total_bricks);
    memset(&out->nodes[0], 0, sizeof(arc_node64));
    memset(&out->bricks[0], 0, sizeof(arc_brick64));
    uint32_t nn = 1, nb = 1;
    for (uint32_t k = 0; k < nch; ++k) {
        uint32_t idx = (uint32_t)(order[k] & 0xFFFFFFFFu);
        chunk_tree* t = &trees[idx];
        if (t->nodes.d[0].mask_low == 0 && t->nodes.d[0].mask_high == 0) {
            out->roots[idx] = ARC_EMPTY_CHUNK;
            continue;
        }
        uint32_t node_base = nn, brick_base = nb;
        for (uint32_t i = 0; i < t->nodes.n; ++i) {
            arc_node64 n = t->nodes.d[i];
            if (n.mask_low == 0 && n.mask_high == 0) {
                memset(&out->nodes[nn++], 0, sizeof(arc_node64));
                continue;
            }
            uint32_t flags = n.child_ptr & (ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG);
            uint32_t local = n.child_ptr & ARC_PTR_INDEX_MASK;
            uint32_t ptr;
            if (n.child_ptr & ARC_IS_LEAF_FLAG) ptr = (n.child_ptr & ARC_IS_UNIFORM_FLAG) ? flags : (flags | (brick_base + local));
            else ptr = flags | (node_base + local);
            n.child_ptr = ptr;
            out->nodes[nn++] = n;
        }
        if (t->bricks.n) memcpy(&out->bricks[nb], t->bricks.d, sizeof(arc_brick64) * t->bricks.n);
        nb += t->bricks.n;
        out->roots[idx] = node_base;
    }
    out->n_nodes = nn;
    out->n_bricks = nb;
    out->solid_voxels = solid;
    for (uint32_t i = 0; i < nch; ++i) { free(trees[i].nodes.d); free(trees[i].bricks.d); }
    free(trees);
    free(order);
    return 0;
}

void orc_free_pools(orc_pools* p) {
    free(p->roots);
    free(p->nodes);
    free(p->bricks);
    memset(p, 0, sizeof(*p));
}
