// arc_world.cpp — native builder of the synthetic worlds into Arcadia's GPU pool layout.
//
// Per chunk (OpenMP-parallel over chunks): a depth-first build into a node arena with exact region
// pruning, then level-order emission; then a Morton-ordered flatten of all chunks.
//
// Region pruning is what makes large worlds cheap. A region is
//   air   when it lies at or above the tallest column of its footprint (2D max pyramid), or when
//         it lies below the terrain and its cave noise is bounded above the threshold;
//   solid when it lies below the 3-voxel top-soil band of every column (2D min pyramid), inside one
//         16^3 material cell, and its cave noise is bounded below the threshold.
// Trilinear value noise with smoothstep weights is a convex combination of its lattice corners, so
// the corner min/max bound the noise over a region (a 1e-5 margin covers float rounding). A region
// the bounds cannot decide is subdivided, down to per-voxel evaluation in 4^3 leaves. Pruning only
// skips work whose outcome is certain, so the pools are the same as an unpruned build
// (ChunkTree64::from_generator, crates/arcadia-core/src/chunk_tree/builder.rs:86-313).
//
// Compiled with -ffp-contract=off: heights, noise and lod colours are float results that must not
// depend on the host ISA.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/arc/arc_trace.h"
#include "../../include/arc/arc_world.h"

struct arc_world_pools {
    std::vector<uint32_t> roots;
    std::vector<arc_node64> nodes;
    std::vector<arc_brick64> bricks;
    uint64_t solid = 0;
};

namespace {

// ------------------------------------------------------------------------------------------------
// Scene definition
// ------------------------------------------------------------------------------------------------

inline float hash2f(int32_t x, int32_t z, uint32_t seed) {
    uint32_t n = (uint32_t)x * 374761393u + (uint32_t)z * 668265263u + seed * 0x27D4EB2Du;
    n = (n ^ (n >> 13)) * 1274126177u;
    return (float)(n ^ (n >> 16)) / 4294967296.0f;
}

inline uint32_t hash3(int32_t x, int32_t y, int32_t z, uint32_t seed) {
    uint32_t n = (uint32_t)x * 374761393u + (uint32_t)y * 1103515245u + (uint32_t)z * 668265263u + seed * 0x27D4EB2Du;
    n = (n ^ (n >> 13)) * 1274126177u;
    return n ^ (n >> 16);
}

inline float hash3f(int32_t x, int32_t y, int32_t z, uint32_t seed) { return (float)hash3(x, y, z, seed) / 4294967296.0f; }

inline float smooth_w(float f) { return f * f * (3.0f - 2.0f * f); }

float noise2(float x, float z, uint32_t seed) {
    const float fx0 = std::floor(x), fz0 = std::floor(z);
    const int32_t ix = (int32_t)fx0, iz = (int32_t)fz0;
    const float ux = smooth_w(x - fx0), uz = smooth_w(z - fz0);
    const float v00 = hash2f(ix, iz, seed), v10 = hash2f(ix + 1, iz, seed);
    const float v01 = hash2f(ix, iz + 1, seed), v11 = hash2f(ix + 1, iz + 1, seed);
    const float a = v00 + ux * (v10 - v00);
    const float b = v01 + ux * (v11 - v01);
    return a + uz * (b - a);
}

float terrain_height(const arc_scene_desc& d, uint32_t x, uint32_t z) {
    const float wx = (float)(d.grid[0] * 256u), wy = (float)(d.grid[1] * 256u);
    const float freq = 2.0f / wx;
    float px = ((float)x + 0.5f) * freq, pz = ((float)z + 0.5f) * freq;
    float f = 0.0f, amp = 0.5f;
    for (int o = 0; o < 4; ++o) {
        f += (noise2(px, pz, d.seed) * 2.0f - 1.0f) * amp;
        px *= 2.03f;
        pz *= 2.03f;
        amp *= 0.5f;
    }
    float h01 = std::fmin(std::fmax(0.5f + 1.5f * f, 0.0f), 1.0f);
    const float lo = d.height_lo * wy, hi = d.height_hi * wy;
    return std::floor(lo + (hi - lo) * h01);
}

// Corner values of the lattice cell (cell size 1 << lg) that contains voxel (x, y, z).
inline void lattice_corners(uint32_t x, uint32_t y, uint32_t z, uint32_t lg, uint32_t seed, float c[8]) {
    const int32_t ix = (int32_t)(x >> lg), iy = (int32_t)(y >> lg), iz = (int32_t)(z >> lg);
    for (int k = 0; k < 8; ++k) c[k] = hash3f(ix + (k & 1), iy + ((k >> 1) & 1), iz + ((k >> 2) & 1), seed);
}

inline float lattice_interp(uint32_t x, uint32_t y, uint32_t z, uint32_t lg, const float c[8]) {
    const uint32_t m = (1u << lg) - 1u;
    const float inv = 1.0f / (float)(1u << lg);
    const float ux = smooth_w(((float)(x & m) + 0.5f) * inv);
    const float uy = smooth_w(((float)(y & m) + 0.5f) * inv);
    const float uz = smooth_w(((float)(z & m) + 0.5f) * inv);
    const float x00 = c[0] + ux * (c[1] - c[0]);
    const float x10 = c[2] + ux * (c[3] - c[2]);
    const float x01 = c[4] + ux * (c[5] - c[4]);
    const float x11 = c[6] + ux * (c[7] - c[6]);
    const float y0 = x00 + uy * (x10 - x00);
    const float y1 = x01 + uy * (x11 - x01);
    return y0 + uz * (y1 - y0);
}

constexpr uint32_t kCaveSeedA = 0x5BD1E995u, kCaveSeedB = 0x1B873593u;
constexpr uint32_t kSoilSeed = 0xA511E9B3u, kRockSeed = 0x63D83595u;

struct Scene {
    arc_scene_desc d;
    uint32_t wx, wz;
    std::vector<float> h;                     // heightmap, z-major
    std::vector<float> hmax[4], hmin[4];      // per block size 4, 16, 64, 256

    float cave(uint32_t x, uint32_t y, uint32_t z) const {
        float ca[8], cb[8];
        lattice_corners(x, y, z, 5u, d.seed ^ kCaveSeedA, ca);
        lattice_corners(x, y, z, 4u, d.seed ^ kCaveSeedB, cb);
        return (lattice_interp(x, y, z, 5u, ca) + lattice_interp(x, y, z, 4u, cb)) * 0.5f;
    }

    uint32_t voxel(uint32_t x, uint32_t y, uint32_t z) const {
        const float hh = h[(size_t)z * wx + x];
        if (!((float)y < hh)) return ARC_MAT_AIR;
        const int32_t depth = (int32_t)hh - 1 - (int32_t)y;
        if (d.caves && (d.cave_depth == 0u || depth < (int32_t)d.cave_depth) && cave(x, y, z) > d.cave_threshold)
            return ARC_MAT_AIR;
        if (depth < 3) return 1u + (hash3((int32_t)x, (int32_t)y, (int32_t)z, d.seed ^ kSoilSeed) & 15u);
        return 1u + (hash3((int32_t)(x >> 4), (int32_t)(y >> 4), (int32_t)(z >> 4), d.seed ^ kRockSeed) & 15u);
    }

    enum Hint { kNone, kAir, kSolid };

    // Exact classification of the aligned region [x0, x0+size) x [y0, ...) x [z0, ...), size in {4,16,64,256}.
    Hint classify(uint32_t x0, uint32_t y0, uint32_t z0, uint32_t size, uint32_t* mat) const {
        const int lvl = size == 4u ? 0 : size == 16u ? 1 : size == 64u ? 2 : 3;
        const uint32_t bs = 4u << (2 * lvl);
        const size_t bi = (size_t)(z0 / bs) * (wx / bs) + (x0 / bs);
        const float mx = hmax[lvl][bi], mn = hmin[lvl][bi];
        if ((float)y0 >= mx) return kAir;
        if (!((float)(y0 + size + 3u) <= mn)) return kNone;
        // every voxel of the region deeper than the cave band: no cave can reach it
        const bool below_band = d.cave_depth && (mn - (float)(y0 + size)) >= (float)d.cave_depth;
        if (d.caves && !below_band) {
            if (size > 16u) return kNone;
            float ca[8], cb[8];
            lattice_corners(x0, y0, z0, 5u, d.seed ^ kCaveSeedA, ca);
            lattice_corners(x0, y0, z0, 4u, d.seed ^ kCaveSeedB, cb);
            const float amax = *std::max_element(ca, ca + 8), amin = *std::min_element(ca, ca + 8);
            const float bmax = *std::max_element(cb, cb + 8), bmin = *std::min_element(cb, cb + 8);
            const float hi = (amax + bmax) * 0.5f, lo = (amin + bmin) * 0.5f;
            // all empty only if every voxel also lies inside the band
            const bool in_band = !d.cave_depth || (mx - 1.0f - (float)y0) < (float)d.cave_depth;
            if (lo > d.cave_threshold + 1e-5f && in_band) return kAir;
            if (!(hi <= d.cave_threshold - 1e-5f)) return kNone;
        }
        if (size > 16u) return kNone;
        *mat = 1u + (hash3((int32_t)(x0 >> 4), (int32_t)(y0 >> 4), (int32_t)(z0 >> 4), d.seed ^ kRockSeed) & 15u);
        return kSolid;
    }
};

void build_scene(Scene& S, const arc_scene_desc& d, int threads) {
    S.d = d;
    S.wx = d.grid[0] * 256u;
    S.wz = d.grid[2] * 256u;
    S.h.assign((size_t)S.wx * S.wz, 0.0f);
#pragma omp parallel for schedule(static) num_threads(threads)
    for (int64_t z = 0; z < (int64_t)S.wz; ++z)
        for (uint32_t x = 0; x < S.wx; ++x) S.h[(size_t)z * S.wx + x] = terrain_height(d, x, (uint32_t)z);
    for (int l = 0; l < 4; ++l) {
        const uint32_t bs = 4u << (2 * l);
        const uint32_t nx = S.wx / bs, nz = S.wz / bs;
        S.hmax[l].assign((size_t)nx * nz, -1.0f);
        S.hmin[l].assign((size_t)nx * nz, 3.0e38f);
        const std::vector<float>& sx = l == 0 ? S.h : S.hmax[l - 1];
        const std::vector<float>& sn = l == 0 ? S.h : S.hmin[l - 1];
        const uint32_t f = l == 0 ? 4u : 4u, srcw = l == 0 ? S.wx : S.wx / (bs / 4u);
        for (uint32_t bz = 0; bz < nz; ++bz)
            for (uint32_t bx = 0; bx < nx; ++bx) {
                float a = -1.0f, b = 3.0e38f;
                for (uint32_t j = 0; j < f; ++j)
                    for (uint32_t i = 0; i < f; ++i) {
                        const size_t k = (size_t)(bz * f + j) * srcw + (bx * f + i);
                        a = std::max(a, sx[k]);
                        b = std::min(b, sn[k]);
                    }
                S.hmax[l][(size_t)bz * nx + bx] = a;
                S.hmin[l][(size_t)bz * nx + bx] = b;
            }
    }
}

// ------------------------------------------------------------------------------------------------
// Palette / lod payloads
// ------------------------------------------------------------------------------------------------

inline uint32_t sat_u32(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
inline float clamp01(float v) { return std::fmin(std::fmax(v, 0.0f), 1.0f); }

inline bool emissive(const arc_material& m) {
    return m.emission_meta[0] > 0.01f || m.emission_meta[1] > 0.01f || m.emission_meta[2] > 0.01f;
}

// Material::pack_lod_payload (crates/arcadia-core/src/material.rs:70-75)
inline uint32_t material_lod(const arc_material& m, uint32_t id) {
    return (id << 24) | (sat_u32(clamp01(m.albedo_roughness[2]) * 255.0f) << 16) |
           (sat_u32(clamp01(m.albedo_roughness[1]) * 255.0f) << 8) | sat_u32(clamp01(m.albedo_roughness[0]) * 255.0f);
}

// ------------------------------------------------------------------------------------------------
// Chunk build
// ------------------------------------------------------------------------------------------------

enum Kind : uint8_t { kEmpty = 0, kUniform = 1, kMixed = 2, kInternal = 3 };

struct BNode {
    uint64_t mask;
    uint32_t lod;
    uint32_t link;  // kInternal: first child in the arena; kMixed: brick index in the arena
    uint8_t kind, mat, full, n_children;
};

struct ChunkBuilder {
    const Scene* S;
    const arc_material* pal;
    uint32_t org[3];
    uint32_t solid = 0;
    std::vector<BNode> arena;
    std::vector<arc_brick64> bricks;

    BNode uniform_full(uint32_t mat) {
        return BNode{~0ull, material_lod(pal[mat], mat), 0u, kUniform, (uint8_t)mat, 1u, 0u};
    }

    BNode leaf(uint32_t ox, uint32_t oy, uint32_t oz) {
        uint64_t mask = 0;
        arc_brick64 br;
        std::memset(&br, 0, sizeof br);
        uint32_t first = ARC_MAT_AIR, em_mat = ARC_MAT_AIR, em_n = 0;
        bool same = true;
        float rs = 0.0f, gs = 0.0f, bs = 0.0f;
        for (uint32_t z = 0; z < 4; ++z)
            for (uint32_t y = 0; y < 4; ++y)
                for (uint32_t x = 0; x < 4; ++x) {
                    const uint32_t m = S->voxel(org[0] + ox + x, org[1] + oy + y, org[2] + oz + z);
                    if (m == ARC_MAT_AIR) continue;
                    const uint32_t bit = (z << 4) | (y << 2) | x;
                    mask |= 1ull << bit;
                    br.packed_materials[bit >> 2] |= m << ((bit & 3u) * 8u);
                    if (first == ARC_MAT_AIR) first = m;
                    else if (m != first) same = false;
                    const arc_material& mm = pal[m];
                    rs += std::fmin(mm.albedo_roughness[0] + mm.emission_meta[0] * 0.25f, 1.0f);
                    gs += std::fmin(mm.albedo_roughness[1] + mm.emission_meta[1] * 0.25f, 1.0f);
                    bs += std::fmin(mm.albedo_roughness[2] + mm.emission_meta[2] * 0.25f, 1.0f);
                    if (emissive(mm)) { em_mat = m; ++em_n; }
                }
        if (!mask) return BNode{0, 0, 0, kEmpty, 0, 0, 0};
        const uint32_t cnt = (uint32_t)__builtin_popcountll(mask);
        solid += cnt;
        if (same) return BNode{mask, material_lod(pal[first], first), 0u, kUniform, (uint8_t)first, (uint8_t)(mask == ~0ull), 0u};
        const float inv = 1.0f / (float)cnt;
        const uint32_t rep = (em_mat != ARC_MAT_AIR && em_n * 2u >= cnt) ? em_mat : first;
        const uint32_t lod = (rep << 24) | (sat_u32(clamp01(bs * inv) * 255.0f) << 16) |
                             (sat_u32(clamp01(gs * inv) * 255.0f) << 8) | sat_u32(clamp01(rs * inv) * 255.0f);
        bricks.push_back(br);
        return BNode{mask, lod, (uint32_t)bricks.size() - 1u, kMixed, 0, 0, 0};
    }

    BNode build(uint32_t ox, uint32_t oy, uint32_t oz, uint32_t shift) {
        const uint32_t size = 4u << shift;
        uint32_t hm = 0;
        switch (S->classify(org[0] + ox, org[1] + oy, org[2] + oz, size, &hm)) {
            case Scene::kAir: return BNode{0, 0, 0, kEmpty, 0, 0, 0};
            case Scene::kSolid: solid += size * size * size; return uniform_full(hm);
            default: break;
        }
        if (shift == 0) return leaf(ox, oy, oz);
        const uint32_t cs = 1u << shift;
        BNode kids[64];
        uint32_t nk = 0;
        uint64_t mask = 0;
        uint32_t rs = 0, gs = 0, bs = 0, solid_mat = ARC_MAT_AIR, em_mat = ARC_MAT_AIR, em_n = 0, common = ARC_MAT_AIR;
        bool collapse = true;
        for (uint32_t z = 0; z < 4; ++z)
            for (uint32_t y = 0; y < 4; ++y)
                for (uint32_t x = 0; x < 4; ++x) {
                    const BNode ch = build(ox + x * cs, oy + y * cs, oz + z * cs, shift - 2u);
                    if (ch.kind == kEmpty) continue;
                    mask |= 1ull << ((z << 4) | (y << 2) | x);
                    rs += ch.lod & 0xFFu;
                    gs += (ch.lod >> 8) & 0xFFu;
                    bs += (ch.lod >> 16) & 0xFFu;
                    const uint32_t cm = ch.lod >> 24;
                    if (emissive(pal[cm])) { em_mat = cm; ++em_n; }
                    else if (solid_mat == ARC_MAT_AIR) solid_mat = cm;
                    if (ch.kind == kUniform && ch.full) {
                        if (common == ARC_MAT_AIR) common = ch.mat;
                        else if (common != ch.mat) collapse = false;
                    } else {
                        collapse = false;
                    }
                    kids[nk++] = ch;
                }
        if (!mask) return BNode{0, 0, 0, kEmpty, 0, 0, 0};
        if (collapse && common != ARC_MAT_AIR)
            return BNode{mask, material_lod(pal[common], common), 0u, kUniform, (uint8_t)common, (uint8_t)(mask == ~0ull), 0u};
        const uint32_t dom = (em_mat != ARC_MAT_AIR && (em_n * 2u >= nk || solid_mat == ARC_MAT_AIR)) ? em_mat : solid_mat;
        const uint32_t lod = (dom << 24) | (((bs / nk) & 0xFFu) << 16) | (((gs / nk) & 0xFFu) << 8) | ((rs / nk) & 0xFFu);
        const uint32_t first = (uint32_t)arena.size();
        arena.insert(arena.end(), kids, kids + nk);
        return BNode{mask, lod, first, kInternal, 0, 0, (uint8_t)(nk & 0xFFu)};
    }
};

inline arc_node64 make_node(uint64_t mask, uint32_t ptr, uint32_t lod) {
    return arc_node64{(uint32_t)mask, (uint32_t)(mask >> 32), ptr, lod};
}

// Level-order emission of one chunk (the order pack_build_tree's FIFO produces).
void emit_chunk(const ChunkBuilder& B, const BNode& root, std::vector<arc_node64>& nodes, std::vector<arc_brick64>& bricks) {
    nodes.assign(1, arc_node64{0, 0, 0, 0});
    bricks.clear();
    if (root.kind == kEmpty) return;
    std::vector<std::pair<uint32_t, BNode>> cur{{0u, root}}, next;
    while (!cur.empty()) {
        next.clear();
        for (const auto& e : cur) {
            const BNode& b = e.second;
            if (b.kind == kUniform) {
                nodes[e.first] = make_node(b.mask, ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG, b.lod);
            } else if (b.kind == kMixed) {
                nodes[e.first] = make_node(b.mask, ARC_IS_LEAF_FLAG | (uint32_t)bricks.size(), b.lod);
                bricks.push_back(B.bricks[b.link]);
            } else if (b.kind == kInternal) {
                const uint32_t base = (uint32_t)nodes.size();
                const uint32_t n = b.n_children ? b.n_children : 64u;
                nodes.resize(base + n, arc_node64{0, 0, 0, 0});
                nodes[e.first] = make_node(b.mask, base, b.lod);
                for (uint32_t i = 0; i < n; ++i) next.emplace_back(base + i, B.arena[b.link + i]);
            }
        }
        cur.swap(next);
    }
}

inline uint32_t spread3(uint32_t v) {
    v &= 0x3FFu;
    v = (v | (v << 16)) & 0xFF0000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

void set_mat(arc_material& m, float r, float g, float b, float rough, float er, float eg, float eb, float var) {
    m = arc_material{{r, g, b, rough}, {er, eg, eb, var}};
}

}  // namespace

extern "C" {

int arc_default_palette(arc_material* out) {
    if (!out) return ARC_E_INVALID_ARG;
    std::memset(out, 0, sizeof(arc_material) * 256);
    static const float t[29][8] = {
        {0.00f, 0.00f, 0.00f, 1.00f, 0, 0, 0, 0.00f},       {0.10f, 0.11f, 0.13f, 0.90f, 0, 0, 0, 0.03f},
        {0.28f, 0.30f, 0.34f, 0.85f, 0, 0, 0, 0.05f},       {0.58f, 0.54f, 0.47f, 0.80f, 0, 0, 0, 0.06f},
        {0.46f, 0.45f, 0.40f, 0.88f, 0, 0, 0, 0.08f},       {0.36f, 0.40f, 0.45f, 0.72f, 0, 0, 0, 0.05f},
        {0.48f, 0.52f, 0.57f, 0.65f, 0, 0, 0, 0.04f},       {0.34f, 0.23f, 0.15f, 0.92f, 0, 0, 0, 0.06f},
        {0.22f, 0.52f, 0.18f, 0.78f, 0, 0, 0, 0.08f},       {0.46f, 0.58f, 0.20f, 0.78f, 0, 0, 0, 0.08f},
        {0.16f, 0.46f, 0.22f, 0.85f, 0, 0, 0, 0.09f},       {0.11f, 0.32f, 0.15f, 0.88f, 0, 0, 0, 0.06f},
        {0.68f, 0.60f, 0.46f, 0.82f, 0, 0, 0, 0.07f},       {0.27f, 0.18f, 0.12f, 0.88f, 0, 0, 0, 0.06f},
        {0.48f, 0.33f, 0.20f, 0.75f, 0, 0, 0, 0.05f},       {0.15f, 0.44f, 0.18f, 0.70f, 0, 0, 0, 0.10f},
        {0.76f, 0.36f, 0.11f, 0.70f, 0, 0, 0, 0.10f},       {0.85f, 0.48f, 0.58f, 0.72f, 0, 0, 0, 0.08f},
        {0.06f, 0.28f, 0.38f, 0.05f, 0, 0, 0, 0.02f},       {0.15f, 0.85f, 1.00f, 0.15f, 0.20f, 2.40f, 3.60f, 0.05f},
        {0.95f, 0.20f, 0.80f, 0.15f, 3.20f, 0.25f, 2.50f, 0.05f}, {1.00f, 0.68f, 0.15f, 0.15f, 3.40f, 1.75f, 0.15f, 0.05f},
        {1.00f, 0.30f, 0.04f, 0.30f, 4.20f, 1.10f, 0.08f, 0.10f}, {0.10f, 0.09f, 0.08f, 0.95f, 0, 0, 0, 0.05f},
        {0.95f, 0.25f, 0.04f, 0.50f, 3.20f, 0.75f, 0.05f, 0.12f}, {0.82f, 0.80f, 0.75f, 0.35f, 0, 0, 0, 0.03f},
        {0.85f, 0.68f, 0.24f, 0.25f, 0, 0, 0, 0.04f},       {1.00f, 0.97f, 0.90f, 0.05f, 116.00f, 114.50f, 111.80f, 0.02f},
        {0.92f, 0.95f, 0.98f, 0.02f, 0, 0, 0, 0.01f},
    };
    for (int i = 0; i < 29; ++i) set_mat(out[i], t[i][0], t[i][1], t[i][2], t[i][3], t[i][4], t[i][5], t[i][6], t[i][7]);
    for (int i = 29; i < 256; ++i) {
        const float s = (float)i / 255.0f;
        set_mat(out[i], 0.3f + 0.4f * std::fabs(std::sin(s * 6.28318531f)), 0.3f + 0.4f * std::fabs(std::cos(s * 3.0f * 3.14159265f)),
                0.3f + 0.3f * s, 0.75f, 0, 0, 0, 0.05f);
    }
    return ARC_OK;
}

int arc_world_build(const arc_scene_desc* desc, const arc_material* palette, int threads, arc_world_pools** out) {
    if (!desc || !out) return ARC_E_INVALID_ARG;
    *out = nullptr;
    for (int i = 0; i < 3; ++i)
        if (desc->grid[i] == 0 || desc->grid[i] > 1024u) return ARC_E_INVALID_ARG;
    if (threads <= 0) threads = omp_get_max_threads();
    std::vector<arc_material> pal(256);
    if (palette) std::memcpy(pal.data(), palette, sizeof(arc_material) * 256);
    else arc_default_palette(pal.data());
    arc_world_pools* W = new (std::nothrow) arc_world_pools();
    if (!W) return ARC_E_OUT_OF_MEMORY;
    try {
        Scene S;
        build_scene(S, *desc, threads);
        const uint32_t gx = desc->grid[0], gy = desc->grid[1], gz = desc->grid[2];
        const uint32_t nch = gx * gy * gz;
        std::vector<std::vector<arc_node64>> cn(nch);
        std::vector<std::vector<arc_brick64>> cb(nch);
        std::vector<uint32_t> csolid(nch, 0);
#pragma omp parallel for schedule(dynamic, 1) num_threads(threads)
        for (int64_t i = 0; i < (int64_t)nch; ++i) {
            const uint32_t u = (uint32_t)i;
            ChunkBuilder B;
            B.S = &S;
            B.pal = pal.data();
            B.org[0] = (u % gx) * 256u;
            B.org[1] = ((u / gx) % gy) * 256u;
            B.org[2] = (u / (gx * gy)) * 256u;
            const BNode root = B.build(0, 0, 0, 6);
            emit_chunk(B, root, cn[i], cb[i]);
            csolid[i] = B.solid;
        }
        std::vector<std::pair<uint32_t, uint32_t>> order(nch);
        for (uint32_t i = 0; i < nch; ++i)
            order[i] = {spread3(i % gx) | (spread3((i / gx) % gy) << 1) | (spread3(i / (gx * gy)) << 2), i};
        std::sort(order.begin(), order.end());
        size_t tn = 1, tb = 1;
        for (uint32_t i = 0; i < nch; ++i)
            if (cn[i][0].mask_low | cn[i][0].mask_high) {
                tn += cn[i].size();
                tb += cb[i].size();
            }
        if (tn > ARC_PTR_INDEX_MASK || tb > ARC_PTR_INDEX_MASK) {
            delete W;
            return ARC_E_CAPACITY;
        }
        W->roots.assign(nch, ARC_EMPTY_CHUNK);
        W->nodes.reserve(tn);
        W->bricks.reserve(tb);
        W->nodes.push_back(arc_node64{0, 0, 0, 0});
        arc_brick64 zero;
        std::memset(&zero, 0, sizeof zero);
        W->bricks.push_back(zero);
        for (const auto& oe : order) {
            const uint32_t i = oe.second;
            W->solid += csolid[i];
            const std::vector<arc_node64>& nodes = cn[i];
            if (!(nodes[0].mask_low | nodes[0].mask_high)) continue;
            const uint32_t nb = (uint32_t)W->nodes.size(), bb = (uint32_t)W->bricks.size();
            W->roots[i] = nb;
            for (arc_node64 n : nodes) {
                if (!(n.mask_low | n.mask_high)) {
                    W->nodes.push_back(arc_node64{0, 0, 0, 0});
                    continue;
                }
                const uint32_t flags = n.child_ptr & (ARC_IS_LEAF_FLAG | ARC_IS_UNIFORM_FLAG);
                const uint32_t local = n.child_ptr & ARC_PTR_INDEX_MASK;
                if (!(n.child_ptr & ARC_IS_LEAF_FLAG)) n.child_ptr = flags | (nb + local);
                else if (!(n.child_ptr & ARC_IS_UNIFORM_FLAG)) n.child_ptr = flags | (bb + local);
                else n.child_ptr = flags;
                W->nodes.push_back(n);
            }
            W->bricks.insert(W->bricks.end(), cb[i].begin(), cb[i].end());
        }
    } catch (const std::bad_alloc&) {
        delete W;
        return ARC_E_OUT_OF_MEMORY;
    }
    *out = W;
    return ARC_OK;
}

int arc_world_info(const arc_world_pools* w, uint32_t* n_roots, uint32_t* n_nodes, uint32_t* n_bricks, uint64_t* solid) {
    if (!w) return ARC_E_INVALID_ARG;
    if (n_roots) *n_roots = (uint32_t)w->roots.size();
    if (n_nodes) *n_nodes = (uint32_t)w->nodes.size();
    if (n_bricks) *n_bricks = (uint32_t)w->bricks.size();
    if (solid) *solid = w->solid;
    return ARC_OK;
}

int arc_world_copy(const arc_world_pools* w, uint32_t* roots, arc_node64* nodes, arc_brick64* bricks) {
    if (!w) return ARC_E_INVALID_ARG;
    if (roots) std::memcpy(roots, w->roots.data(), sizeof(uint32_t) * w->roots.size());
    if (nodes) std::memcpy(nodes, w->nodes.data(), sizeof(arc_node64) * w->nodes.size());
    if (bricks) std::memcpy(bricks, w->bricks.data(), sizeof(arc_brick64) * w->bricks.size());
    return ARC_OK;
}

int arc_world_free(arc_world_pools* w) {
    delete w;
    return ARC_OK;
}

}  // extern "C"
