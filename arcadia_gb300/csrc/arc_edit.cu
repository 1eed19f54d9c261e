// arc_edit.cu — in-place world edits on the device: carved spheres and recoloured bricks.
//
// The reference edits one chunk at a time on the CPU (ChunkTree64::carve_sphere_tracked,
// crates/arcadia-core/src/chunk_tree/edit/carve.rs:39-176; mutate_brick_in_place and its helpers,
// edit/set.rs:244-569) and ships the changed node and brick ranges to the GPU as patches
// (crates/arcadia-world/src/world_map.rs:319-383). Here the tree is updated where it lives.
//
// Three launches per batch:
//   root uncollapse  one thread per touched chunk: a collapsed root (the whole chunk one uniform solid)
//                    expands when an edit rewrites a voxel of it (uncollapse_if_needed, set.rs:404-428)
//   regions          one CTA per (chunk, 64^3 region) with edits: the CTA owns the region's L1 node and
//                    everything below it and applies the region's edits in order. For each edit:
//       candidates   the bricks it changes (sphere-brick test, brick solid mask, voxel-centre distance,
//                    tree.rs:109-166 semantics) with their 64-bit entry masks
//       uncollapse   the L1 node, then the L2 nodes on candidate paths (one thread per node)
//       leaves       one thread per candidate applies the entries in ascending voxel order
//                    (apply_voxel_entries_to_leaf, set.rs:431-515), allocating a brick when a uniform
//                    leaf turns mixed, and refreshes the leaf's LOD (compute_leaf_lod, set.rs:573-618)
//       bottom-up    touched L2 nodes, then the L1 node: drop emptied children, compacting the child
//                    slice as remove_child does (set.rs:322-354), and refresh the LOD payload
//                    (refresh_internal_lod, set.rs:518-569)
//   root refresh     one thread per chunk with rewritten leaves: the same for its root
// Edits in different regions touch disjoint nodes below the root, so regions run in parallel; the
// root's child slice stays put until the root pass.
// The result equals the reference's sequential edit node for node (masks, flags, LOD payloads, brick
// materials); only the pool positions of grown nodes and bricks differ. Growth comes from the pools'
// upload headroom through atomic counters; exhausted headroom skips the growth and raises an overflow
// flag. Compiled with the canonical arithmetic flags: the distance tests are the reference's f32
// ((dx*dx + dy*dy) + dz*dz) without contraction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "arc_ctx.h"

namespace arc {
namespace edit {

constexpr uint32_t kMatWater = 18u;
constexpr int kThreads = 256;
constexpr int kMaxCand = 1024;  // bricks of a radius-16 sphere inside one chunk: at most 10^3

struct Params {
    const arc_edit_op* ops;
    const uint32_t* chunk_list;   // touched chunks (flat index)
    const uint32_t* op_start;     // per touched chunk: first entry in op_idx
    const uint32_t* op_idx;       // op indices, in op order per chunk
    const uint32_t* roots;
    uint4* nodes;
    uint32_t* bricks;             // 16 words per brick
    const float4* palette;        // 2 float4 per material
    uint32_t* counters;           // [0] next node, [1] next brick, [2] bricks rewritten, [3] overflow
    uint32_t node_cap, brick_cap;
};

__device__ __forceinline__ uint64_t nmask(uint4 n) { return (uint64_t)n.x | ((uint64_t)n.y << 32); }
__device__ __forceinline__ uint4 with_mask(uint4 n, uint64_t m) {
    n.x = (uint32_t)m;
    n.y = (uint32_t)(m >> 32);
    return n;
}
__device__ __forceinline__ bool nleaf(uint4 n) { return (n.z & ARC_IS_LEAF_FLAG) != 0u; }
__device__ __forceinline__ bool nuniform(uint4 n) { return (n.z & ARC_IS_UNIFORM_FLAG) != 0u; }
__device__ __forceinline__ uint32_t nbase(uint4 n) { return n.z & ARC_PTR_INDEX_MASK; }
__device__ __forceinline__ uint32_t nprimary(uint4 n) { return n.w >> 24; }
__device__ __forceinline__ uint32_t nslot(uint4 n, uint32_t b) {
    return nbase(n) + (uint32_t)__popcll(nmask(n) & ((1ull << b) - 1ull));
}
__device__ __forceinline__ uint32_t cbit(uint32_t x, uint32_t y, uint32_t z) { return (z << 4) | (y << 2) | x; }
__device__ __forceinline__ uint32_t brick_get(const uint32_t* br, uint32_t bit) { return (br[bit >> 2] >> ((bit & 3u) * 8u)) & 0xFFu; }
__device__ __forceinline__ void brick_set(uint32_t* br, uint32_t bit, uint32_t mat) {
    const uint32_t s = (bit & 3u) * 8u;
    br[bit >> 2] = (br[bit >> 2] & ~(0xFFu << s)) | (mat << s);
}

__device__ __forceinline__ bool emissive(const Params& P, uint32_t m) {
    const float4 e = P.palette[2u * m + 1u];
    return e.x > 0.01f || e.y > 0.01f || e.z > 0.01f;
}
// Material::pack_lod_payload (crates/arcadia-core/src/material.rs:70-75)
__device__ __forceinline__ uint32_t pack_lod(const Params& P, uint32_t m) {
    const float4 a = P.palette[2u * m];
    const uint32_t r = f2u(clampf(a.x, 0.0f, 1.0f) * 255.0f), g = f2u(clampf(a.y, 0.0f, 1.0f) * 255.0f),
                   b = f2u(clampf(a.z, 0.0f, 1.0f) * 255.0f);
    return (m << 24) | (b << 16) | (g << 8) | r;
}
// pack_rgb_and_mat (crates/arcadia-core/src/chunk_tree/builder.rs:72-78)
__device__ __forceinline__ uint32_t pack_rgb_mat(float r, float g, float b, uint32_t m) {
    return (m << 24) | (f2u(clampf(b, 0.0f, 1.0f) * 255.0f) << 16) | (f2u(clampf(g, 0.0f, 1.0f) * 255.0f) << 8) |
           f2u(clampf(r, 0.0f, 1.0f) * 255.0f);
}

__device__ __forceinline__ float dist2(float ax, float ay, float az, float bx, float by, float bz) {
    const float dx = ax - bx, dy = ay - by, dz = az - bz;
    return (dx * dx + dy * dy) + dz * dz;
}

// get_brick_solid_mask (tree.rs:109-166): a collapsed ancestor counts as full when its material is solid.
__device__ uint64_t solid_mask(const Params& P, uint32_t root, uint32_t bx, uint32_t by, uint32_t bz) {
    const uint32_t x = bx << 2, y = by << 2, z = bz << 2;
    uint32_t idx = root, shift = 6;
    for (int guard = 0; guard < 4; ++guard) {
        const uint4 n = P.nodes[idx];
        if (nleaf(n)) {
            if (shift > 0) {
                const uint32_t m = nprimary(n);
                return (m != ARC_MAT_AIR && m != kMatWater) ? ~0ull : 0ull;
            }
            const uint64_t mask = nmask(n);
            if (nuniform(n)) {
                const uint32_t m = nprimary(n);
                return (m != ARC_MAT_AIR && m != kMatWater) ? mask : 0ull;
            }
            const uint32_t* br = P.bricks + 16u * (size_t)nbase(n);
            uint64_t s = mask;
            for (uint64_t rem = mask; rem; rem &= rem - 1ull) {
                const uint32_t bit = (uint32_t)__ffsll((long long)rem) - 1u;
                const uint32_t m = brick_get(br, bit);
                if (m == ARC_MAT_AIR || m == kMatWater) s &= ~(1ull << bit);
            }
            return s;
        }
        const uint32_t b = cbit((x >> shift) & 3u, (y >> shift) & 3u, (z >> shift) & 3u);
        if (!(nmask(n) & (1ull << b))) return 0ull;
        idx = nslot(n, b);
        shift -= 2;
    }
    return 0ull;
}

// uncollapse_if_needed (set.rs:404-428) of node idx whose children sit one level down.
__device__ void uncollapse(const Params& P, uint32_t idx) {
    const uint4 n = P.nodes[idx];
    if (!nleaf(n)) return;
    const uint32_t count = (uint32_t)__popcll(nmask(n));
    if (count == 0) {
        P.nodes[idx].z = 0u;
        return;
    }
    const uint32_t base = atomicAdd(&P.counters[0], count);
    if (base + count > P.node_cap) {
        atomicOr(&P.counters[3], 1u);
        return;
    }
    const uint32_t mat = nprimary(n);
    const uint4 child = make_uint4(0xFFFFFFFFu, 0xFFFFFFFFu, ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG, pack_lod(P, mat));
    for (uint32_t i = 0; i < count; ++i) P.nodes[base + i] = child;
    uint4 m = n;
    m.z = base;  // internal now: flags cleared
    P.nodes[idx] = m;
}

// compute_leaf_lod (set.rs:573-618)
__device__ uint32_t leaf_lod(const Params& P, uint64_t mask, const uint32_t* br) {
    if (mask == 0) return 0u;
    const uint32_t first = brick_get(br, (uint32_t)__ffsll((long long)mask) - 1u);
    bool uniform = true;
    for (uint64_t rem = mask & (mask - 1ull); rem; rem &= rem - 1ull)
        if (brick_get(br, (uint32_t)__ffsll((long long)rem) - 1u) != first) {
            uniform = false;
            break;
        }
    if (uniform) return first == ARC_MAT_AIR ? 0u : pack_lod(P, first);
    float r = 0.0f, g = 0.0f, b = 0.0f;
    uint32_t solid = ARC_MAT_AIR, emis = ARC_MAT_AIR, n_emis = 0;
    const uint32_t count = (uint32_t)__popcll(mask);
    for (uint64_t rem = mask; rem; rem &= rem - 1ull) {
        const uint32_t id = brick_get(br, (uint32_t)__ffsll((long long)rem) - 1u);
        const float4 a = P.palette[2u * id], e = P.palette[2u * id + 1u];
        r += fminf(a.x + e.x * 0.25f, 1.0f);
        g += fminf(a.y + e.y * 0.25f, 1.0f);
        b += fminf(a.z + e.z * 0.25f, 1.0f);
        if (e.x > 0.01f || e.y > 0.01f || e.z > 0.01f) {
            emis = id;
            n_emis++;
        } else if (solid == ARC_MAT_AIR) {
            solid = id;
        }
    }
    const uint32_t rep = (emis != ARC_MAT_AIR && (n_emis * 2u >= count || solid == ARC_MAT_AIR)) ? emis : solid;
    const float inv = __fdiv_rn(1.0f, (float)count);
    return pack_rgb_mat(r * inv, g * inv, b * inv, rep);
}

// apply_voxel_entries_to_leaf (set.rs:431-515): voxels of `entries` (ascending) get material `mat`.
__device__ void apply_leaf(const Params& P, uint32_t leaf, uint64_t entries, uint32_t mat) {
    for (uint64_t rem = entries; rem; rem &= rem - 1ull) {
        const uint32_t b = (uint32_t)__ffsll((long long)rem) - 1u;
        const uint4 node = P.nodes[leaf];
        const uint64_t mask = nmask(node);
        const bool was = (mask >> b) & 1ull;
        if (nuniform(node)) {
            if (mat == ARC_MAT_AIR) {
                if (was) P.nodes[leaf] = with_mask(node, mask & ~(1ull << b));
            } else if (mask == 0) {
                uint4 m = with_mask(node, 1ull << b);
                m.w = mat << 24;
                P.nodes[leaf] = m;
            } else if (mat == nprimary(node)) {
                if (!was) P.nodes[leaf] = with_mask(node, mask | (1ull << b));
            } else if (was && mask == (1ull << b)) {
                uint4 m = node;
                m.w = mat << 24;
                P.nodes[leaf] = m;
            } else {
                const uint32_t bi = atomicAdd(&P.counters[1], 1u);
                if (bi >= P.brick_cap) {
                    atomicOr(&P.counters[3], 1u);
                    return;
                }
                uint32_t* br = P.bricks + 16u * (size_t)bi;
                uint32_t w[16];
#pragma unroll
                for (int k = 0; k < 16; ++k) w[k] = 0u;
                const uint32_t primary = nprimary(node);
                for (uint64_t r2 = mask; r2; r2 &= r2 - 1ull) brick_set(w, (uint32_t)__ffsll((long long)r2) - 1u, primary);
                brick_set(w, b, mat);
#pragma unroll
                for (int k = 0; k < 16; ++k) br[k] = w[k];
                uint4 m = with_mask(node, mask | (1ull << b));
                m.z = ARC_IS_LEAF_FLAG | (bi & ARC_PTR_INDEX_MASK);
                P.nodes[leaf] = m;
            }
        } else {
            brick_set(P.bricks + 16u * (size_t)nbase(node), b, mat);
            if (mat == ARC_MAT_AIR) {
                if (was) P.nodes[leaf] = with_mask(node, mask & ~(1ull << b));
            } else if (!was) {
                P.nodes[leaf] = with_mask(node, mask | (1ull << b));
            }
        }
    }
    uint4 fin = P.nodes[leaf];
    const uint64_t fm = nmask(fin);
    if (fm == 0) fin.w = 0u;
    else if (nuniform(fin)) fin.w = pack_lod(P, nprimary(fin));
    else fin.w = leaf_lod(P, fm, P.bricks + 16u * (size_t)nbase(fin));
    P.nodes[leaf] = fin;
}

// Drops the empty children of internal node idx (compacting its slice like repeated remove_child,
// set.rs:322-354) and refreshes its LOD payload (refresh_internal_lod, set.rs:518-569).
__device__ void compact_refresh(const Params& P, uint32_t idx) {
    uint4 n = P.nodes[idx];
    const uint64_t mask = nmask(n);
    const uint32_t count = (uint32_t)__popcll(mask), base = nbase(n);
    uint64_t kept = 0ull;
    uint32_t k = 0, r = 0, g = 0, b = 0, solid = ARC_MAT_AIR, emis = ARC_MAT_AIR, n_emis = 0;
    uint32_t i = 0;
    for (uint64_t rem = mask; rem; rem &= rem - 1ull, ++i) {
        const uint32_t bit = (uint32_t)__ffsll((long long)rem) - 1u;
        const uint4 c = P.nodes[base + i];
        if (nmask(c) == 0ull) continue;
        kept |= 1ull << bit;
        if (k != i) P.nodes[base + k] = c;
        ++k;
        r += c.w & 0xFFu;
        g += (c.w >> 8) & 0xFFu;
        b += (c.w >> 16) & 0xFFu;
        const uint32_t cm = c.w >> 24;
        if (emissive(P, cm)) {
            emis = cm;
            n_emis++;
        } else if (solid == ARC_MAT_AIR) {
            solid = cm;
        }
    }
    if (base > 0u)
        for (uint32_t j = k; j < count; ++j) P.nodes[base + j] = make_uint4(0u, 0u, 0u, 0u);
    if (k == 0) {
        P.nodes[idx] = make_uint4(0u, 0u, 0u, 0u);
        return;
    }
    const uint32_t dom = (emis != ARC_MAT_AIR && (n_emis * 2u >= k || solid == ARC_MAT_AIR)) ? emis : solid;
    n = with_mask(n, kept);
    n.w = (dom << 24) | (((b / k) & 0xFFu) << 16) | (((g / k) & 0xFFu) << 8) | ((r / k) & 0xFFu);
    P.nodes[idx] = n;
}

// Work item: one 64^3 L1 region of one chunk with the edits touching it (op_idx[op_start[i] ..
// op_start[i + 1]), in edit order). The CTA owns the region's L1 node and everything below it.
__global__ void __launch_bounds__(kThreads) edit_regions_kernel(const Params P, const uint32_t* __restrict__ item_chunk,
                                                               const uint32_t* __restrict__ item_region,
                                                               const uint32_t* __restrict__ item_slot,
                                                               uint32_t* __restrict__ chunk_touched, uint32_t grid_x,
                                                               uint32_t grid_y) {
    __shared__ uint32_t s_cand[kMaxCand];        // bx | by << 6 | bz << 12 (chunk-local bricks)
    __shared__ unsigned long long s_entries[kMaxCand];
    __shared__ uint32_t s_l2[2], s_u2[2];        // touched / claimed L2 nodes of the region (64 bits)
    __shared__ uint32_t s_n_cand, s_touched;
    const uint32_t tid = threadIdx.x;
    const uint32_t chunk = item_chunk[blockIdx.x], b0 = item_region[blockIdx.x];
    const uint32_t root = P.roots[chunk];
    if (root == ARC_EMPTY_CHUNK) return;  // uniform over the CTA
    {
        const uint4 rn = P.nodes[root];
        if (nleaf(rn) || !(nmask(rn) & (1ull << b0))) return;  // empty region (or growth refused): nothing to edit
    }
    const uint32_t l1 = nslot(P.nodes[root], b0);  // the root's slice is stable until the root pass
    const uint32_t r0x = (b0 & 3u) * 16u, r0y = ((b0 >> 2) & 3u) * 16u, r0z = (b0 >> 4) * 16u;  // region bricks
    const float ox = (float)((chunk % grid_x) * 256u), oy = (float)(((chunk / grid_x) % grid_y) * 256u),
                oz = (float)((chunk / (grid_x * grid_y)) * 256u);
    if (tid == 0) s_touched = 0u;
    for (uint32_t e = P.op_start[blockIdx.x]; e < P.op_start[blockIdx.x + 1]; ++e) {
        const arc_edit_op op = P.ops[P.op_idx[e]];
        if (tid == 0) s_n_cand = 0;
        if (tid < 2) s_l2[tid] = s_u2[tid] = 0u;
        __syncthreads();
        if (nmask(P.nodes[l1]) == 0ull) break;  // region emptied by an earlier edit (uniform)
        // ---- candidates inside this region
        const bool carve = op.kind == ARC_EDIT_CARVE;
        const uint32_t mat = carve ? ARC_MAT_AIR : op.material;
        const float cx = op.center[0] - ox, cy = op.center[1] - oy, cz = op.center[2] - oz, rr = op.radius;
        int32_t x0, x1, y0, y1, z0, z1;
        if (carve) {
            const float kx = clampf(cx, 0.0f, 256.0f), ky = clampf(cy, 0.0f, 256.0f), kz = clampf(cz, 0.0f, 256.0f);
            const float sx0 = fmaxf(floorf(cx - rr), 0.0f), sy0 = fmaxf(floorf(cy - rr), 0.0f), sz0 = fmaxf(floorf(cz - rr), 0.0f);
            const float sx1 = fminf(ceilf(cx + rr), 255.0f), sy1 = fminf(ceilf(cy + rr), 255.0f), sz1 = fminf(ceilf(cz + rr), 255.0f);
            const bool any = !(dist2(cx, cy, cz, kx, ky, kz) > rr * rr) && !(sx0 > sx1 || sy0 > sy1 || sz0 > sz1);
            x0 = any ? (int32_t)((uint32_t)sx0 >> 2) : 1;
            x1 = any ? (int32_t)((uint32_t)sx1 >> 2) : 0;
            y0 = any ? (int32_t)((uint32_t)sy0 >> 2) : 1;
            y1 = any ? (int32_t)((uint32_t)sy1 >> 2) : 0;
            z0 = any ? (int32_t)((uint32_t)sz0 >> 2) : 1;
            z1 = any ? (int32_t)((uint32_t)sz1 >> 2) : 0;
        } else {
            x0 = x1 = (int32_t)(op.brick[0] & 63u);
            y0 = y1 = (int32_t)(op.brick[1] & 63u);
            z0 = z1 = (int32_t)(op.brick[2] & 63u);
        }
        x0 = max(x0, (int32_t)r0x);
        x1 = min(x1, (int32_t)r0x + 15);
        y0 = max(y0, (int32_t)r0y);
        y1 = min(y1, (int32_t)r0y + 15);
        z0 = max(z0, (int32_t)r0z);
        z1 = min(z1, (int32_t)r0z + 15);
        const uint32_t nx = x1 >= x0 ? (uint32_t)(x1 - x0 + 1) : 0u, ny = y1 >= y0 ? (uint32_t)(y1 - y0 + 1) : 0u,
                       nz = z1 >= z0 ? (uint32_t)(z1 - z0 + 1) : 0u;
        const float r2 = rr * rr;
        for (uint32_t i = tid; i < nx * ny * nz; i += kThreads) {
            const uint32_t bx = (uint32_t)x0 + i % nx, by = (uint32_t)y0 + (i / nx) % ny, bz = (uint32_t)z0 + i / (nx * ny);
            if (carve) {
                const float mnx = (float)(bx * 4u), mny = (float)(by * 4u), mnz = (float)(bz * 4u);
                if (dist2(cx, cy, cz, clampf(cx, mnx, mnx + 4.0f), clampf(cy, mny, mny + 4.0f), clampf(cz, mnz, mnz + 4.0f)) > r2)
                    continue;
            }
            const uint64_t solid = solid_mask(P, root, bx, by, bz);
            uint64_t ent = 0ull;
            if (carve) {
                for (uint64_t rem = solid; rem; rem &= rem - 1ull) {
                    const uint32_t b = (uint32_t)__ffsll((long long)rem) - 1u;
                    const float vx = (float)((bx << 2) | (b & 3u)) + 0.5f, vy = (float)((by << 2) | ((b >> 2) & 3u)) + 0.5f,
                                vz = (float)((bz << 2) | ((b >> 4) & 3u)) + 0.5f;
                    if (dist2(cx, cy, cz, vx, vy, vz) <= r2) ent |= 1ull << b;
                }
            } else {
                ent = solid;
            }
            if (ent) {
                const uint32_t slot = atomicAdd(&s_n_cand, 1u);
                if (slot < kMaxCand) {
                    s_cand[slot] = bx | (by << 6) | (bz << 12);
                    s_entries[slot] = ent;
                }
            }
        }
        __syncthreads();
        if (tid == 0 && s_n_cand > (uint32_t)kMaxCand) atomicOr(&P.counters[3], 2u);
        const uint32_t n_cand = min(s_n_cand, (uint32_t)kMaxCand);
        if (n_cand == 0) continue;  // uniform over the CTA
        // ---- uncollapse top-down: the region's L1 node, then its L2 nodes
        if (tid == 0) uncollapse(P, l1);
        __syncthreads();
        for (uint32_t c = tid; c < n_cand; c += kThreads) {
            const uint32_t bx = s_cand[c] & 63u, by = (s_cand[c] >> 6) & 63u, bz = s_cand[c] >> 12;
            const uint32_t b1 = cbit((bx >> 2) & 3u, (by >> 2) & 3u, (bz >> 2) & 3u);
            const uint4 n1 = P.nodes[l1];
            if (nleaf(n1) || !(nmask(n1) & (1ull << b1))) continue;
            if (!(atomicOr(&s_u2[b1 >> 5], 1u << (b1 & 31u)) & (1u << (b1 & 31u)))) uncollapse(P, nslot(n1, b1));
        }
        __syncthreads();
        // ---- leaves
        for (uint32_t c = tid; c < n_cand; c += kThreads) {
            const uint32_t bx = s_cand[c] & 63u, by = (s_cand[c] >> 6) & 63u, bz = s_cand[c] >> 12;
            const uint32_t b1 = cbit((bx >> 2) & 3u, (by >> 2) & 3u, (bz >> 2) & 3u);
            const uint32_t b2 = cbit(bx & 3u, by & 3u, bz & 3u);
            const uint4 n1 = P.nodes[l1];
            if (nleaf(n1) || !(nmask(n1) & (1ull << b1))) continue;  // growth was refused
            const uint4 n2 = P.nodes[nslot(n1, b1)];
            if (nleaf(n2) || !(nmask(n2) & (1ull << b2))) continue;
            apply_leaf(P, nslot(n2, b2), s_entries[c], mat);
            atomicOr(&s_l2[b1 >> 5], 1u << (b1 & 31u));
            s_touched = 1u;
            atomicAdd(&P.counters[2], 1u);
        }
        __syncthreads();
        // ---- bottom-up: the touched L2 nodes, then the L1 node (the root waits for the root pass)
        if (tid < 64 && (s_l2[tid >> 5] & (1u << (tid & 31u)))) compact_refresh(P, nslot(P.nodes[l1], tid));
        __syncthreads();
        if (tid == 0 && (s_l2[0] | s_l2[1])) compact_refresh(P, l1);
        __syncthreads();
    }
    if (tid == 0 && s_touched) chunk_touched[item_slot[blockIdx.x]] = 1u;
}

// Before the region pass: a chunk whose root is collapsed (the whole chunk one uniform solid) expands
// when one of its edits rewrites a voxel, as ensure_child does on the first mutated brick. For a full
// chunk that is: any recolour, or a carve whose nearest voxel centre lies within the radius.
__global__ void edit_root_uncollapse_kernel(const Params P, uint32_t grid_x, uint32_t grid_y, uint32_t n_chunks) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_chunks) return;
    const uint32_t chunk = P.chunk_list[i];
    const uint32_t root = P.roots[chunk];
    if (root == ARC_EMPTY_CHUNK || !nleaf(P.nodes[root]) || nmask(P.nodes[root]) == 0ull) return;
    const uint32_t m = nprimary(P.nodes[root]);
    if (m == ARC_MAT_AIR || m == kMatWater) return;  // not solid: no edit rewrites it
    const float ox = (float)((chunk % grid_x) * 256u), oy = (float)(((chunk / grid_x) % grid_y) * 256u),
                oz = (float)((chunk / (grid_x * grid_y)) * 256u);
    for (uint32_t e = P.op_start[i]; e < P.op_start[i + 1]; ++e) {
        const arc_edit_op op = P.ops[P.op_idx[e]];
        bool hit = op.kind == ARC_EDIT_RECOLOR;
        if (!hit) {
            const float cx = op.center[0] - ox, cy = op.center[1] - oy, cz = op.center[2] - oz;
            const float vx = clampf(floorf(cx), 0.0f, 255.0f) + 0.5f, vy = clampf(floorf(cy), 0.0f, 255.0f) + 0.5f,
                        vz = clampf(floorf(cz), 0.0f, 255.0f) + 0.5f;
            hit = dist2(cx, cy, cz, vx, vy, vz) <= op.radius * op.radius;
        }
        if (hit) {
            uncollapse(P, root);
            return;
        }
    }
}

// After the region pass: roots of chunks with rewritten leaves drop emptied L1 nodes and refresh LOD.
__global__ void edit_root_refresh_kernel(const Params P, const uint32_t* __restrict__ chunks,
                                         const uint32_t* __restrict__ touched, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !touched[i]) return;
    const uint32_t root = P.roots[chunks[i]];
    if (root != ARC_EMPTY_CHUNK && !nleaf(P.nodes[root])) compact_refresh(P, root);
}

// Raises the allocator floors to cover host-written patch ranges.
__global__ void floor_kernel(uint32_t* counters, uint32_t node_floor, uint32_t brick_floor) {
    atomicMax(&counters[0], node_floor);
    atomicMax(&counters[1], brick_floor);
}

}  // namespace edit
}  // namespace arc

namespace {

int edit_err(arc_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

}  // namespace

int arc_edit_reset(arc_ctx* c) {
    // allocator state after a world upload: growth starts at the end of the uploaded pools
    if (!c->d_edit) {
        if (cudaMalloc((void**)&c->d_edit, 4 * sizeof(uint32_t)) != cudaSuccess) return edit_err(c, ARC_E_OUT_OF_MEMORY, "edit counters");
    }
    const uint32_t init[4] = {c->n_nodes, c->n_bricks, 0u, 0u};
    if (cudaMemcpyAsync(c->d_edit, init, sizeof init, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
        return edit_err(c, ARC_E_CUDA, "edit counters");
    return ARC_OK;
}

int arc_edit_raise_floor(arc_ctx* c, uint32_t node_floor, uint32_t brick_floor) {
    if (!c->d_edit) return ARC_OK;
    arc::edit::floor_kernel<<<1, 1, 0, c->stream>>>(c->d_edit, node_floor, brick_floor);
    return cudaGetLastError() == cudaSuccess ? ARC_OK : edit_err(c, ARC_E_CUDA, "floor_kernel");
}

extern "C" {

int arc_apply_edits(arc_ctx* c, const arc_edit_op* ops, uint32_t n_ops, uint32_t* bricks_rewritten) {
    int rc = arc_ctx_check_ready(c, false);
    if (rc) return rc;
    if (n_ops && !ops) return edit_err(c, ARC_E_INVALID_ARG, "null edit list");
    const uint32_t gx = c->grid[0], gy = c->grid[1], gz = c->grid[2];
    std::vector<std::pair<uint32_t, uint32_t>> pairs;  // (chunk, op)
    for (uint32_t k = 0; k < n_ops; ++k) {
        const arc_edit_op& op = ops[k];
        if (op.kind == ARC_EDIT_RECOLOR) {
            if (op.material == ARC_MAT_AIR || op.material > 255u) return edit_err(c, ARC_E_INVALID_ARG, "recolour material must be 1..255");
            if (op.brick[0] >= gx * 64u || op.brick[1] >= gy * 64u || op.brick[2] >= gz * 64u)
                return edit_err(c, ARC_E_INVALID_ARG, "recolour brick outside the world");
            pairs.emplace_back((op.brick[0] >> 6) + (op.brick[1] >> 6) * gx + (op.brick[2] >> 6) * gx * gy, k);
            // water and mirror voxels take the primary pass's surface branches from now on
            if (op.material == 18u || op.material == 28u) c->surface_mats[0] = true;
        } else if (op.kind == ARC_EDIT_CARVE) {
            if (!(op.radius > 0.0f && op.radius <= 16.0f)) return edit_err(c, ARC_E_INVALID_ARG, "carve radius must lie in (0, 16]");
            if (!(std::isfinite(op.center[0]) && std::isfinite(op.center[1]) && std::isfinite(op.center[2])))
                return edit_err(c, ARC_E_INVALID_ARG, "carve centre must be finite");
            const float r = op.radius;
            const int64_t lo[3] = {(int64_t)std::floor((op.center[0] - r) / 256.0f), (int64_t)std::floor((op.center[1] - r) / 256.0f),
                                   (int64_t)std::floor((op.center[2] - r) / 256.0f)};
            const int64_t hi[3] = {(int64_t)std::floor((op.center[0] + r) / 256.0f), (int64_t)std::floor((op.center[1] + r) / 256.0f),
                                   (int64_t)std::floor((op.center[2] + r) / 256.0f)};
            for (int64_t z = std::max<int64_t>(lo[2], 0); z <= std::min<int64_t>(hi[2], gz - 1); ++z)
                for (int64_t y = std::max<int64_t>(lo[1], 0); y <= std::min<int64_t>(hi[1], gy - 1); ++y)
                    for (int64_t x = std::max<int64_t>(lo[0], 0); x <= std::min<int64_t>(hi[0], gx - 1); ++x)
                        pairs.emplace_back((uint32_t)(x + y * gx + z * gx * gy), k);
        } else {
            return edit_err(c, ARC_E_INVALID_ARG, "unknown edit kind");
        }
    }
    if (!c->d_edit && (rc = arc_edit_reset(c))) return rc;
    if (!pairs.empty()) {
        std::stable_sort(pairs.begin(), pairs.end(), [](const auto& x, const auto& y) { return x.first < y.first; });
        // per touched chunk: its edits in order (root passes)
        std::vector<uint32_t> chunks, start, idx;
        for (size_t i = 0; i < pairs.size(); ++i) {
            if (i == 0 || pairs[i].first != pairs[i - 1].first) {
                chunks.push_back(pairs[i].first);
                start.push_back((uint32_t)i);
            }
            idx.push_back(pairs[i].second);
        }
        start.push_back((uint32_t)pairs.size());
        // per (chunk, 64^3 region): the edits whose voxel bounds reach the region, in order (region pass)
        std::vector<uint64_t> trip;  // chunk slot << 40 | region << 32 | op
        for (uint32_t ci = 0; ci < (uint32_t)chunks.size(); ++ci) {
            const uint32_t ch = chunks[ci];
            const float ox = (float)((ch % gx) * 256u), oy = (float)(((ch / gx) % gy) * 256u), oz = (float)((ch / (gx * gy)) * 256u);
            for (uint32_t e = start[ci]; e < start[ci + 1]; ++e) {
                const arc_edit_op& op = ops[idx[e]];
                uint32_t lo[3], hi[3];
                if (op.kind == ARC_EDIT_RECOLOR) {
                    for (int a = 0; a < 3; ++a) lo[a] = hi[a] = (op.brick[a] & 63u) >> 4;
                } else {
                    const float l[3] = {op.center[0] - ox, op.center[1] - oy, op.center[2] - oz};
                    bool empty = false;
                    for (int a = 0; a < 3; ++a) {
                        const float s0 = std::max(std::floor(l[a] - op.radius), 0.0f), s1 = std::min(std::ceil(l[a] + op.radius), 255.0f);
                        if (s0 > s1) empty = true;
                        lo[a] = empty ? 1u : (uint32_t)s0 >> 6;
                        hi[a] = empty ? 0u : (uint32_t)s1 >> 6;
                    }
                    if (empty) continue;
                }
                for (uint32_t z = lo[2]; z <= hi[2]; ++z)
                    for (uint32_t y = lo[1]; y <= hi[1]; ++y)
                        for (uint32_t x = lo[0]; x <= hi[0]; ++x)
                            trip.push_back(((uint64_t)ci << 40) | ((uint64_t)(x | (y << 2) | (z << 4)) << 32) | idx[e]);
            }
        }
        // edit order inside a (chunk, region) group: op index order
        std::sort(trip.begin(), trip.end());
        std::vector<uint32_t> it_chunk, it_region, it_slot, it_start, it_idx;
        for (size_t i = 0; i < trip.size(); ++i) {
            const uint64_t key = trip[i] >> 32;
            if (i == 0 || key != (trip[i - 1] >> 32)) {
                it_slot.push_back((uint32_t)(trip[i] >> 40));
                it_chunk.push_back(chunks[trip[i] >> 40]);
                it_region.push_back((uint32_t)(key & 63u));
                it_start.push_back((uint32_t)i);
            }
            it_idx.push_back((uint32_t)trip[i]);
        }
        it_start.push_back((uint32_t)trip.size());
        const uint32_t n_items = (uint32_t)it_chunk.size(), n_ch = (uint32_t)chunks.size();
        // one staged upload
        const size_t parts[11] = {sizeof(arc_edit_op) * n_ops, 4 * chunks.size(), 4 * start.size(), 4 * idx.size(),
                                  4 * it_chunk.size(), 4 * it_region.size(), 4 * it_slot.size(), 4 * it_start.size(),
                                  4 * it_idx.size(), 4 * (size_t)n_ch, 0};
        size_t off[11] = {0};
        for (int k = 1; k < 11; ++k) off[k] = (off[k - 1] + parts[k - 1] + 15) & ~(size_t)15;
        const size_t total = off[10];
        if (c->edit_stage_bytes < total) {
            cudaFree(c->d_edit_stage);
            cudaFreeHost(c->h_edit_stage);
            c->d_edit_stage = nullptr;
            c->h_edit_stage = nullptr;
            c->edit_stage_bytes = 0;
            if (cudaMalloc(&c->d_edit_stage, total) != cudaSuccess || cudaMallocHost(&c->h_edit_stage, total) != cudaSuccess)
                return edit_err(c, ARC_E_OUT_OF_MEMORY, "edit staging");
            c->edit_stage_bytes = total;
        }
        // the pinned block may still feed the previous batch's copy
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) return edit_err(c, ARC_E_CUDA, "edit staging sync");
        uint8_t* h = static_cast<uint8_t*>(c->h_edit_stage);
        const void* src[10] = {ops, chunks.data(), start.data(), idx.data(), it_chunk.data(), it_region.data(),
                               it_slot.data(), it_start.data(), it_idx.data(), nullptr};
        for (int k = 0; k < 9; ++k) std::memcpy(h + off[k], src[k], parts[k]);
        std::memset(h + off[9], 0, parts[9]);
        if (cudaMemcpyAsync(c->d_edit_stage, h, total, cudaMemcpyHostToDevice, c->stream) != cudaSuccess)
            return edit_err(c, ARC_E_CUDA, "edit upload");
        uint8_t* d = static_cast<uint8_t*>(c->d_edit_stage);
        auto dptr = [&](int k) { return reinterpret_cast<uint32_t*>(d + off[k]); };
        arc::edit::Params P;
        P.ops = reinterpret_cast<const arc_edit_op*>(d);
        P.chunk_list = dptr(1);
        P.op_start = dptr(2);
        P.op_idx = dptr(3);
        P.roots = c->d_roots;
        P.nodes = reinterpret_cast<uint4*>(c->d_nodes);
        P.bricks = reinterpret_cast<uint32_t*>(c->d_bricks);
        P.palette = reinterpret_cast<const float4*>(c->d_palette);
        P.counters = c->d_edit;
        P.node_cap = c->cap_nodes;
        P.brick_cap = c->cap_bricks;
        arc::edit::edit_root_uncollapse_kernel<<<(n_ch + 127u) / 128u, 128, 0, c->stream>>>(P, gx, gy, n_ch);
        if (n_items) {
            arc::edit::Params R = P;
            R.op_start = dptr(7);
            R.op_idx = dptr(8);
            arc::edit::edit_regions_kernel<<<n_items, arc::edit::kThreads, 0, c->stream>>>(R, dptr(4), dptr(5), dptr(6),
                                                                                            dptr(9), gx, gy);
        }
        arc::edit::edit_root_refresh_kernel<<<(n_ch + 127u) / 128u, 128, 0, c->stream>>>(P, dptr(1), dptr(9), n_ch);
        if (cudaGetLastError() != cudaSuccess) return edit_err(c, ARC_E_CUDA, "edit kernels launch");
        // traversal range checks now cover the whole pools: grown nodes live in the headroom
        if (c->n_nodes != c->cap_nodes || c->n_bricks != c->cap_bricks) {
            c->n_nodes = c->cap_nodes;
            c->n_bricks = c->cap_bricks;
            if ((rc = arc_ctx_sync_world_table(c))) return rc;
        }
    }
    if (bricks_rewritten) {
        uint32_t cnt[4];
        if (cudaMemcpyAsync(cnt, c->d_edit, sizeof cnt, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess)
            return edit_err(c, ARC_E_CUDA, "edit counters readback");
        *bricks_rewritten = cnt[2];
        if (cnt[3]) return edit_err(c, ARC_E_CAPACITY, "edit growth beyond the pools' headroom (re-upload with more)");
    }
    return ARC_OK;
}

int arc_download_world(arc_ctx* c, uint32_t* roots, arc_node64* nodes, uint32_t node_cap, arc_brick64* bricks,
                       uint32_t brick_cap, uint32_t* n_nodes, uint32_t* n_bricks) {
    int rc = arc_ctx_check_ready(c, false);
    if (rc) return rc;
    uint32_t used[2] = {c->n_nodes, c->n_bricks};
    if (c->d_edit) {
        uint32_t cnt[4];
        if (cudaMemcpyAsync(cnt, c->d_edit, sizeof cnt, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess)
            return edit_err(c, ARC_E_CUDA, "edit counters readback");
        // the allocator starts at the uploaded counts and rises with patches and edits
        used[0] = std::min(cnt[0], c->cap_nodes);
        used[1] = std::min(cnt[1], c->cap_bricks);
    }
    if (n_nodes) *n_nodes = used[0];
    if (n_bricks) *n_bricks = used[1];
    if (roots && cudaMemcpyAsync(roots, c->d_roots, sizeof(uint32_t) * c->n_roots, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
        return edit_err(c, ARC_E_CUDA, "roots readback");
    if (nodes && cudaMemcpyAsync(nodes, c->d_nodes, sizeof(arc_node64) * std::min(node_cap, used[0]), cudaMemcpyDeviceToHost,
                                 c->stream) != cudaSuccess)
        return edit_err(c, ARC_E_CUDA, "nodes readback");
    if (bricks && cudaMemcpyAsync(bricks, c->d_bricks, sizeof(arc_brick64) * std::min(brick_cap, used[1]),
                                  cudaMemcpyDeviceToHost, c->stream) != cudaSuccess)
        return edit_err(c, ARC_E_CUDA, "bricks readback");
    return cudaStreamSynchronize(c->stream) == cudaSuccess ? ARC_OK : edit_err(c, ARC_E_CUDA, "world readback");
}

int arc_edit_stats(arc_ctx* c, uint32_t* next_node, uint32_t* next_brick, uint32_t* bricks_rewritten, uint32_t* overflow) {
    if (!c) return ARC_E_INVALID_ARG;
    uint32_t cnt[4] = {c->n_nodes, c->n_bricks, 0u, 0u};
    if (c->d_edit) {
        if (cudaMemcpyAsync(cnt, c->d_edit, sizeof cnt, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
            cudaStreamSynchronize(c->stream) != cudaSuccess)
            return edit_err(c, ARC_E_CUDA, "edit counters readback");
    }
    if (next_node) *next_node = cnt[0];
    if (next_brick) *next_brick = cnt[1];
    if (bricks_rewritten) *bricks_rewritten = cnt[2];
    if (overflow) *overflow = cnt[3];
    return ARC_OK;
}

}  // extern "C"
