/* orc_edit.c — in-place voxel edits on the flattened pools (test infrastructure only).
 *
 * A sequential restatement of the reference's ChunkTree64 edit path:
 *   carve_sphere_tracked             crates/arcadia-core/src/chunk_tree/edit/carve.rs:39-176 (no scorch rim)
 *   mutate_brick_in_place            edit/set.rs:244-319
 *   remove_child / ensure_child      edit/set.rs:322-401
 *   uncollapse_if_needed             edit/set.rs:404-428
 *   apply_voxel_entries_to_leaf      edit/set.rs:431-515
 *   refresh_internal_lod             edit/set.rs:518-569
 *   compute_leaf_lod                 edit/set.rs:573-618
 *   get_brick_solid_mask             crates/arcadia-core/src/chunk_tree/tree.rs:109-166
 * The reference mutates one chunk's node vector and appends grown branches at its end; here the chunk
 * lives inside the flattened pools (child pointers are global), and grown nodes and bricks are appended
 * at the end of the global pools, where the GPU pools keep their upload headroom. An edit of kind
 * ARC_EDIT_RECOLOR is mutate_brick_in_place with one entry (b, material) per solid voxel b of the brick.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "orc.h"
#include "orc_math.h"

uint32_t orc_pack_lod_payload(const arc_material* m, uint32_t mat);
uint32_t orc_pack_rgb_and_mat(float r, float g, float b, uint32_t mat);
int orc_mat_is_emissive(const arc_material* m);

#define MAT_WATER_CRYSTAL 18u

typedef struct ed_pool {
    arc_node64* nodes;
    uint32_t n_nodes, node_cap;
    arc_brick64* bricks;
    uint32_t n_bricks, brick_cap;
    const arc_material* pal;
    int overflow;
} ed_pool;

static uint64_t nmask(const arc_node64* n) { return (uint64_t)n->mask_low | ((uint64_t)n->mask_high << 32); }
static void nset_mask(arc_node64* n, uint64_t m) {
    n->mask_low = (uint32_t)m;
    n->mask_high = (uint32_t)(m >> 32);
}
static int nleaf(const arc_node64* n) { return (n->child_ptr & ARC_IS_LEAF_FLAG) != 0; }
static int nuniform(const arc_node64* n) { return (n->child_ptr & ARC_IS_UNIFORM_FLAG) != 0; }
static uint32_t nbase(const arc_node64* n) { return n->child_ptr & ARC_PTR_INDEX_MASK; }
static uint32_t nprimary(const arc_node64* n) { return n->lod_payload >> 24; }
static uint32_t ncount(const arc_node64* n) { return (uint32_t)__builtin_popcountll(nmask(n)); }
static uint32_t nslot(const arc_node64* n, uint32_t b) {
    return nbase(n) + (uint32_t)__builtin_popcountll(nmask(n) & ((1ull << b) - 1ull));
}
static arc_node64 node_make(uint64_t m, uint32_t ptr, uint32_t lod) {
    arc_node64 n;
    nset_mask(&n, m);
    n.child_ptr = ptr;
    n.lod_payload = lod;
    return n;
}
static uint32_t brick_get(const arc_brick64* b, uint32_t bit) { return (b->packed_materials[bit >> 2] >> ((bit & 3u) * 8u)) & 0xFFu; }
static void brick_set(arc_brick64* b, uint32_t bit, uint32_t mat) {
    const uint32_t s = (bit & 3u) * 8u;
    b->packed_materials[bit >> 2] = (b->packed_materials[bit >> 2] & ~(0xFFu << s)) | (mat << s);
}
static uint32_t cbit(uint32_t x, uint32_t y, uint32_t z) { return (z << 4) | (y << 2) | x; }

/* Appends `count` nodes; returns the first index, or UINT32_MAX when the pool is full. */
static uint32_t grow_nodes(ed_pool* p, uint32_t count) {
    if (p->n_nodes + count > p->node_cap) {
        p->overflow = 1;
        return 0xFFFFFFFFu;
    }
    const uint32_t base = p->n_nodes;
    memset(&p->nodes[base], 0, sizeof(arc_node64) * count);
    p->n_nodes += count;
    return base;
}

/* get_brick_solid_mask (tree.rs:109-166) from node `root` of a chunk. */
static uint64_t brick_solid_mask(const ed_pool* p, uint32_t root, uint32_t bx, uint32_t by, uint32_t bz) {
    const uint32_t x = bx << 2, y = by << 2, z = bz << 2;
    uint32_t idx = root, shift = 6;
    for (;;) {
        const arc_node64* n = &p->nodes[idx];
        if (nleaf(n)) {
            if (shift > 0) {
                const uint32_t mat = nprimary(n);
                return (mat != ARC_MAT_AIR && mat != MAT_WATER_CRYSTAL) ? ~0ull : 0ull;
            }
            const uint64_t mask = nmask(n);
            if (nuniform(n)) {
                const uint32_t mat = nprimary(n);
                return (mat != ARC_MAT_AIR && mat != MAT_WATER_CRYSTAL) ? mask : 0ull;
            }
            const arc_brick64* br = &p->bricks[nbase(n)];
            uint64_t solid = mask, rem = mask;
            while (rem) {
                const uint32_t bit = (uint32_t)__builtin_ctzll(rem);
                const uint32_t mat = brick_get(br, bit);
                if (mat == ARC_MAT_AIR || mat == MAT_WATER_CRYSTAL) solid &= ~(1ull << bit);
                rem &= rem - 1ull;
            }
            return solid;
        }
        const uint32_t b = cbit((x >> shift) & 3u, (y >> shift) & 3u, (z >> shift) & 3u);
        if (!(nmask(n) & (1ull << b))) return 0ull;
        idx = nslot(n, b);
        shift -= 2;
    }
}

static void uncollapse_if_needed(ed_pool* p, uint32_t idx, uint32_t shift) {
    if (shift == 0 || !nleaf(&p->nodes[idx])) return;
    const uint32_t mat = nprimary(&p->nodes[idx]);
    const uint32_t count = ncount(&p->nodes[idx]);
    if (count == 0) {
        p->nodes[idx].child_ptr = 0;
        return;
    }
    const uint32_t base = grow_nodes(p, count);
    if (base == 0xFFFFFFFFu) return;
    const uint32_t lod = orc_pack_lod_payload(&p->pal[mat], mat);
    for (uint32_t i = 0; i < count; ++i) p->nodes[base + i] = node_make(~0ull, ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG, lod);
    p->nodes[idx].child_ptr = base;
}

static uint32_t ensure_child(ed_pool* p, uint32_t parent, uint32_t b, uint32_t shift) {
    uncollapse_if_needed(p, parent, shift);
    if (nmask(&p->nodes[parent]) & (1ull << b)) return nslot(&p->nodes[parent], b);
    const uint32_t old_count = ncount(&p->nodes[parent]);
    const uint32_t old_base = nbase(&p->nodes[parent]);
    const uint32_t base = grow_nodes(p, old_count + 1u);
    if (base == 0xFFFFFFFFu) return 0;
    const uint32_t rank = (uint32_t)__builtin_popcountll(nmask(&p->nodes[parent]) & ((1ull << b) - 1ull));
    for (uint32_t i = 0; i < rank; ++i) p->nodes[base + i] = p->nodes[old_base + i];
    for (uint32_t i = rank; i < old_count; ++i) p->nodes[base + i + 1] = p->nodes[old_base + i];
    const uint32_t child = base + rank;
    p->nodes[child] = shift == 2 ? node_make(0, ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG, 0) : node_make(0, 0, 0);
    p->nodes[parent].child_ptr = (p->nodes[parent].child_ptr & ~ARC_PTR_INDEX_MASK) | base;
    nset_mask(&p->nodes[parent], nmask(&p->nodes[parent]) | (1ull << b));
    return child;
}

static void remove_child(ed_pool* p, uint32_t parent, uint32_t b) {
    arc_node64* n = &p->nodes[parent];
    if (!(nmask(n) & (1ull << b))) return;
    const uint32_t old_count = ncount(n);
    const uint32_t old_base = nbase(n);
    if (old_count <= 1) {
        if (old_count == 1 && old_base > 0 && old_base < p->n_nodes) p->nodes[old_base] = node_make(0, 0, 0);
        nset_mask(n, 0);
        n->child_ptr = 0;
        n->lod_payload = 0;
        return;
    }
    const uint32_t rank = (uint32_t)__builtin_popcountll(nmask(n) & ((1ull << b) - 1ull));
    const uint32_t new_count = old_count - 1u;
    for (uint32_t i = rank; i < new_count; ++i) p->nodes[old_base + i] = p->nodes[old_base + i + 1];
    p->nodes[old_base + new_count] = node_make(0, 0, 0);
    nset_mask(n, nmask(n) & ~(1ull << b));
}

static uint32_t compute_leaf_lod(const ed_pool* p, uint64_t mask, const arc_brick64* br) {
    if (mask == 0) return 0;
    /* check_uniform (node64.rs:142-158) */
    const uint32_t first = brick_get(br, (uint32_t)__builtin_ctzll(mask));
    int uniform = 1;
    for (uint64_t rem = mask & (mask - 1ull); rem; rem &= rem - 1ull)
        if (brick_get(br, (uint32_t)__builtin_ctzll(rem)) != first) {
            uniform = 0;
            break;
        }
    if (uniform) return first == ARC_MAT_AIR ? 0u : orc_pack_lod_payload(&p->pal[first], first);
    float r = 0.0f, g = 0.0f, bl = 0.0f;
    uint32_t solid_mat = ARC_MAT_AIR, emissive_mat = ARC_MAT_AIR, emissive = 0;
    const uint32_t count = (uint32_t)__builtin_popcountll(mask);
    for (uint64_t rem = mask; rem; rem &= rem - 1ull) {
        const uint32_t id = brick_get(br, (uint32_t)__builtin_ctzll(rem));
        const arc_material* m = &p->pal[id];
        r += orc_min(m->albedo_roughness[0] + m->emission_meta[0] * 0.25f, 1.0f);
        g += orc_min(m->albedo_roughness[1] + m->emission_meta[1] * 0.25f, 1.0f);
        bl += orc_min(m->albedo_roughness[2] + m->emission_meta[2] * 0.25f, 1.0f);
        if (orc_mat_is_emissive(m)) {
            emissive_mat = id;
            emissive++;
        } else if (solid_mat == ARC_MAT_AIR) {
            solid_mat = id;
        }
    }
    const uint32_t rep = (emissive_mat != ARC_MAT_AIR && (emissive * 2u >= count || solid_mat == ARC_MAT_AIR)) ? emissive_mat
                                                                                                            : solid_mat;
    const float inv = 1.0f / (float)count;
    return orc_pack_rgb_and_mat(r * inv, g * inv, bl * inv, rep);
}

static void apply_entries(ed_pool* p, uint32_t leaf, const uint32_t* bits, const uint32_t* mats, uint32_t n_entries) {
    for (uint32_t e = 0; e < n_entries; ++e) {
        const uint32_t b = bits[e], mat = mats[e];
        const arc_node64 node = p->nodes[leaf];
        const uint64_t mask = nmask(&node);
        const int was_solid = (mask >> b) & 1ull;
        if (nuniform(&node)) {
            if (mat == ARC_MAT_AIR) {
                if (was_solid) nset_mask(&p->nodes[leaf], mask & ~(1ull << b));
            } else if (mask == 0) {
                nset_mask(&p->nodes[leaf], 1ull << b);
                p->nodes[leaf].lod_payload = mat << 24;
            } else if (mat == nprimary(&node)) {
                if (!was_solid) nset_mask(&p->nodes[leaf], mask | (1ull << b));
            } else if (was_solid && mask == (1ull << b)) {
                p->nodes[leaf].lod_payload = mat << 24;
            } else {
                if (p->n_bricks >= p->brick_cap) {
                    p->overflow = 1;
                    return;
                }
                const uint32_t bi = p->n_bricks++;
                arc_brick64 br;
                memset(&br, 0, sizeof br);
                const uint32_t primary = nprimary(&node);
                for (uint64_t rem = mask; rem; rem &= rem - 1ull) brick_set(&br, (uint32_t)__builtin_ctzll(rem), primary);
                brick_set(&br, b, mat);
                p->bricks[bi] = br;
                p->nodes[leaf].child_ptr = ARC_IS_LEAF_FLAG | (bi & ARC_PTR_INDEX_MASK);
                nset_mask(&p->nodes[leaf], mask | (1ull << b));
            }
        } else {
            brick_set(&p->bricks[nbase(&node)], b, mat);
            if (mat == ARC_MAT_AIR) {
                if (was_solid) nset_mask(&p->nodes[leaf], mask & ~(1ull << b));
            } else if (!was_solid) {
                nset_mask(&p->nodes[leaf], mask | (1ull << b));
            }
        }
    }
    const arc_node64 fin = p->nodes[leaf];
    const uint64_t fm = nmask(&fin);
    if (fm == 0) p->nodes[leaf].lod_payload = 0;
    else if (nuniform(&fin)) p->nodes[leaf].lod_payload = orc_pack_lod_payload(&p->pal[nprimary(&fin)], nprimary(&fin));
    else p->nodes[leaf].lod_payload = compute_leaf_lod(p, fm, &p->bricks[nbase(&fin)]);
}

static void refresh_internal_lod(ed_pool* p, uint32_t idx) {
    const arc_node64 n = p->nodes[idx];
    const uint32_t count = ncount(&n);
    if (count == 0) {
        p->nodes[idx].lod_payload = 0;
        return;
    }
    const uint32_t base = nbase(&n);
    uint32_t r = 0, g = 0, b = 0, solid_mat = ARC_MAT_AIR, emissive_mat = ARC_MAT_AIR, emissive = 0, non_empty = 0;
    for (uint32_t i = 0; i < count; ++i) {
        const arc_node64* c = &p->nodes[base + i];
        if (nmask(c) == 0) continue;
        const uint32_t lod = c->lod_payload;
        r += lod & 0xFFu;
        g += (lod >> 8) & 0xFFu;
        b += (lod >> 16) & 0xFFu;
        const uint32_t cm = lod >> 24;
        if (orc_mat_is_emissive(&p->pal[cm])) {
            emissive_mat = cm;
            emissive++;
        } else if (solid_mat == ARC_MAT_AIR) {
            solid_mat = cm;
        }
        non_empty++;
    }
    if (non_empty == 0) {
        p->nodes[idx].lod_payload = 0;
        return;
    }
    const uint32_t dom = (emissive_mat != ARC_MAT_AIR && (emissive * 2u >= non_empty || solid_mat == ARC_MAT_AIR)) ? emissive_mat
                                                                                                               : solid_mat;
    p->nodes[idx].lod_payload = (dom << 24) | (((b / non_empty) & 0xFFu) << 16) | (((g / non_empty) & 0xFFu) << 8) |
                                ((r / non_empty) & 0xFFu);
}

static void mutate_brick(ed_pool* p, uint32_t root, uint32_t bx, uint32_t by, uint32_t bz, const uint32_t* bits,
                         const uint32_t* mats, uint32_t n_entries) {
    const uint32_t b0 = cbit((bx >> 4) & 3u, (by >> 4) & 3u, (bz >> 4) & 3u);
    const uint32_t b1 = cbit((bx >> 2) & 3u, (by >> 2) & 3u, (bz >> 2) & 3u);
    const uint32_t b2 = cbit(bx & 3u, by & 3u, bz & 3u);
    uint32_t path[4];
    path[0] = root;
    path[1] = ensure_child(p, path[0], b0, 6);
    if (p->overflow) return;
    path[2] = ensure_child(p, path[1], b1, 4);
    if (p->overflow) return;
    path[3] = ensure_child(p, path[2], b2, 2);
    if (p->overflow) return;
    apply_entries(p, path[3], bits, mats, n_entries);
    if (p->overflow) return;
    if (nmask(&p->nodes[path[3]]) == 0) {
        remove_child(p, path[2], b2);
        if (nmask(&p->nodes[path[2]]) == 0) {
            remove_child(p, path[1], b1);
            if (nmask(&p->nodes[path[1]]) == 0) {
                remove_child(p, path[0], b0);
                if (nmask(&p->nodes[path[0]]) == 0) p->nodes[path[0]] = node_make(0, 0, 0);
                else refresh_internal_lod(p, path[0]);
            } else {
                refresh_internal_lod(p, path[1]);
                refresh_internal_lod(p, path[0]);
            }
        } else {
            refresh_internal_lod(p, path[2]);
            refresh_internal_lod(p, path[1]);
            refresh_internal_lod(p, path[0]);
        }
    } else {
        refresh_internal_lod(p, path[2]);
        refresh_internal_lod(p, path[1]);
        refresh_internal_lod(p, path[0]);
    }
}

static float clampf(float x, float lo, float hi) { return orc_min(orc_max(x, lo), hi); }
static float dist2(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = ax - bx, dy = ay - by, dz = az - bz;
    return (dx * dx + dy * dy) + dz * dz;
}

/* carve_sphere_tracked (carve.rs:39-176) on one chunk, chunk-local centre. */
static void carve_chunk(ed_pool* p, uint32_t root, float cx, float cy, float cz, float r) {
    if (nmask(&p->nodes[root]) == 0) return;
    const float outer = r;
    const float kx = clampf(cx, 0.0f, 256.0f), ky = clampf(cy, 0.0f, 256.0f), kz = clampf(cz, 0.0f, 256.0f);
    if (dist2(cx, cy, cz, kx, ky, kz) > outer * outer) return;
    const float sx0 = orc_max(floorf(cx - outer), 0.0f), sy0 = orc_max(floorf(cy - outer), 0.0f),
                sz0 = orc_max(floorf(cz - outer), 0.0f);
    const float sx1 = orc_min(ceilf(cx + outer), 255.0f), sy1 = orc_min(ceilf(cy + outer), 255.0f),
                sz1 = orc_min(ceilf(cz + outer), 255.0f);
    if (sx0 > sx1 || sy0 > sy1 || sz0 > sz1) return;
    const uint32_t x0 = (uint32_t)sx0 >> 2, x1 = (uint32_t)sx1 >> 2, y0 = (uint32_t)sy0 >> 2, y1 = (uint32_t)sy1 >> 2,
                   z0 = (uint32_t)sz0 >> 2, z1 = (uint32_t)sz1 >> 2;
    const float inner2 = r * r, outer2 = outer * outer;
    uint32_t bits[64], mats[64];
    for (uint32_t bz = z0; bz <= z1; ++bz)
        for (uint32_t by = y0; by <= y1; ++by)
            for (uint32_t bx = x0; bx <= x1; ++bx) {
                const float mnx = (float)(bx * 4u), mny = (float)(by * 4u), mnz = (float)(bz * 4u);
                const float qx = clampf(cx, mnx, mnx + 4.0f), qy = clampf(cy, mny, mny + 4.0f), qz = clampf(cz, mnz, mnz + 4.0f);
                if (dist2(cx, cy, cz, qx, qy, qz) > outer2) continue;
                const uint64_t solid = brick_solid_mask(p, root, bx, by, bz);
                if (solid == 0) continue;
                uint32_t n = 0;
                for (uint64_t rem = solid; rem; rem &= rem - 1ull) {
                    const uint32_t b = (uint32_t)__builtin_ctzll(rem);
                    const uint32_t vx = (bx << 2) | (b & 3u), vy = (by << 2) | ((b >> 2) & 3u), vz = (bz << 2) | ((b >> 4) & 3u);
                    if (dist2(cx, cy, cz, (float)vx + 0.5f, (float)vy + 0.5f, (float)vz + 0.5f) <= inner2) {
                        bits[n] = b;
                        mats[n] = ARC_MAT_AIR;
                        n++;
                    }
                }
                if (n) mutate_brick(p, root, bx, by, bz, bits, mats, n);
                if (p->overflow) return;
            }
}

static void recolor_brick(ed_pool* p, uint32_t root, uint32_t bx, uint32_t by, uint32_t bz, uint32_t mat) {
    if (nmask(&p->nodes[root]) == 0) return;
    const uint64_t solid = brick_solid_mask(p, root, bx, by, bz);
    if (solid == 0) return;
    uint32_t bits[64], mats[64], n = 0;
    for (uint64_t rem = solid; rem; rem &= rem - 1ull) {
        bits[n] = (uint32_t)__builtin_ctzll(rem);
        mats[n] = mat;
        n++;
    }
    mutate_brick(p, root, bx, by, bz, bits, mats, n);
}

/* Applies `ops` in order. The pools have room for node_cap nodes and brick_cap bricks; *n_nodes and
 * *n_bricks grow. Returns 0, or -1 when a pool ran out of room (the edits stop there). */
int orc_apply_edits(const uint32_t grid[3], const uint32_t* roots, arc_node64* nodes, uint32_t* n_nodes, uint32_t node_cap,
                    arc_brick64* bricks, uint32_t* n_bricks, uint32_t brick_cap, const arc_material* palette,
                    const arc_edit_op* ops, uint32_t n_ops) {
    ed_pool p = {nodes, *n_nodes, node_cap, bricks, *n_bricks, brick_cap, palette, 0};
    for (uint32_t k = 0; k < n_ops && !p.overflow; ++k) {
        const arc_edit_op* op = &ops[k];
        if (op->kind == ARC_EDIT_RECOLOR) {
            const uint32_t cxi = op->brick[0] >> 6, cyi = op->brick[1] >> 6, czi = op->brick[2] >> 6;
            if (cxi >= grid[0] || cyi >= grid[1] || czi >= grid[2]) continue;
            const uint32_t root = roots[cxi + cyi * grid[0] + czi * grid[0] * grid[1]];
            if (root == ARC_EMPTY_CHUNK) continue;
            recolor_brick(&p, root, op->brick[0] & 63u, op->brick[1] & 63u, op->brick[2] & 63u, op->material);
        } else if (op->kind == ARC_EDIT_CARVE) {
            const float r = op->radius;
            for (int64_t cz = (int64_t)floorf((op->center[2] - r) / 256.0f); cz <= (int64_t)floorf((op->center[2] + r) / 256.0f); ++cz)
                for (int64_t cy = (int64_t)floorf((op->center[1] - r) / 256.0f); cy <= (int64_t)floorf((op->center[1] + r) / 256.0f); ++cy)
                    for (int64_t cx = (int64_t)floorf((op->center[0] - r) / 256.0f); cx <= (int64_t)floorf((op->center[0] + r) / 256.0f);
                         ++cx) {
                        if (cx < 0 || cy < 0 || cz < 0 || cx >= grid[0] || cy >= grid[1] || cz >= grid[2]) continue;
                        const uint32_t root = roots[cx + cy * grid[0] + cz * grid[0] * grid[1]];
                        if (root == ARC_EMPTY_CHUNK) continue;
                        carve_chunk(&p, root, op->center[0] - (float)(cx * 256), op->center[1] - (float)(cy * 256),
                                    op->center[2] - (float)(cz * 256), r);
                    }
        }
    }
    *n_nodes = p.n_nodes;
    *n_bricks = p.n_bricks;
    return p.overflow ? -1 : 0;
}

/* Material of every voxel of chunk (cx, cy, cz) by point descent (tree.rs:58-86), (z, y, x) order. */
void orc_pool_chunk_volume(const uint32_t grid[3], const uint32_t* roots, const arc_node64* nodes, const arc_brick64* bricks,
                           uint32_t cx, uint32_t cy, uint32_t cz, uint8_t* vol) {
    const uint32_t root = roots[cx + cy * grid[0] + cz * grid[0] * grid[1]];
    memset(vol, 0, 256u * 256u * 256u);
    if (root == ARC_EMPTY_CHUNK) return;
#pragma omp parallel for schedule(static)
    for (int z = 0; z < 256; ++z)
        for (uint32_t y = 0; y < 256; ++y)
            for (uint32_t x = 0; x < 256; ++x) {
                uint32_t idx = root, shift = 6, mat = ARC_MAT_AIR;
                for (;;) {
                    const arc_node64* n = &nodes[idx];
                    const uint32_t b = cbit((x >> shift) & 3u, (y >> shift) & 3u, ((uint32_t)z >> shift) & 3u);
                    if (!(nmask(n) & (1ull << b))) break;
                    if (nleaf(n)) {
                        mat = nuniform(n) ? nprimary(n) : brick_get(&bricks[nbase(n)], b);
                        break;
                    }
                    idx = nslot(n, b);
                    shift -= 2;
                }
                vol[((size_t)z * 256u + y) * 256u + x] = (uint8_t)mat;
            }
}

/* Compares two chunk trees node by node in child order: masks, flags, lod payloads and the materials
 * of every voxel under a leaf mask, wherever the nodes sit in their pools. With leaf_form = 0 a
 * brick-level leaf may be uniform in one tree and a brick in the other when their voxels agree (the
 * reference never turns a brick leaf back into a uniform one; a fresh build does). Returns 0 when
 * equal, else the 1-based depth-first position of the first difference. */
static uint32_t leaf_mat(const arc_node64* n, const arc_brick64* bricks, uint32_t bit) {
    return nuniform(n) ? nprimary(n) : brick_get(&bricks[nbase(n)], bit);
}

static uint64_t cmp_rec(const arc_node64* na, const arc_brick64* ba, uint32_t ia, const arc_node64* nb, const arc_brick64* bb,
                        uint32_t ib, uint32_t shift, int leaf_form, uint64_t* pos) {
    const arc_node64* a = &na[ia];
    const arc_node64* b = &nb[ib];
    const uint32_t flags = ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG;
    const uint32_t fmask = (leaf_form || shift > 0) ? flags : ARC_IS_LEAF_FLAG;
    ++*pos;
    if (nmask(a) != nmask(b) || a->lod_payload != b->lod_payload || (a->child_ptr & fmask) != (b->child_ptr & fmask))
        return *pos;
    if (nmask(a) == 0) return 0;
    if (nleaf(a)) {
        if (shift > 0) return 0;
        for (uint64_t rem = nmask(a); rem; rem &= rem - 1ull) {
            const uint32_t bit = (uint32_t)__builtin_ctzll(rem);
            if (leaf_mat(a, ba, bit) != leaf_mat(b, bb, bit)) return *pos;
        }
        return 0;
    }
    const uint32_t n = ncount(a);
    for (uint32_t i = 0; i < n; ++i) {
        const uint64_t r = cmp_rec(na, ba, nbase(a) + i, nb, bb, nbase(b) + i, shift - 2, leaf_form, pos);
        if (r) return r;
    }
    return 0;
}

uint64_t orc_tree_compare(uint32_t root_a, const arc_node64* nodes_a, const arc_brick64* bricks_a, uint32_t root_b,
                          const arc_node64* nodes_b, const arc_brick64* bricks_b, int leaf_form) {
    uint64_t pos = 0;
    if ((root_a == ARC_EMPTY_CHUNK) != (root_b == ARC_EMPTY_CHUNK)) return 1;
    if (root_a == ARC_EMPTY_CHUNK) return 0;
    return cmp_rec(nodes_a, bricks_a, root_a, nodes_b, bricks_b, root_b, 6, leaf_form, &pos);
}
