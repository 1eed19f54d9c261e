// arc_traverse.cuh — the hierarchical 64-tree DDA as a resumable per-lane state machine.
//
// trace_world_64tree_from (shaders/common/traversal64.wgsl:226-556) is split into ray_begin
// (lines 234-300: setup, world clip, step budget) and ray_advance (one iteration of the outer loop
// at 302-553: chunk MTF cache, empty-chunk skip, ray-cone LOD, ancestor restart, descent by
// popcount, leaf/LOD hit). A kernel calls ray_advance until it stops returning kContinue, so a
// persistent warp can swap a finished lane for a new ray between iterations without changing any
// DDA decision.
//
// Node fetches are single 16-byte read-only loads (ld.global.nc.v4) of the AoS Node64 pool; brick
// reads fetch the one 32-bit word that holds the voxel. Every pool index is range-checked; an
// out-of-range index records a bit in the context's status word and reads as empty space, so a
// corrupt pool cannot fault the device.
//
// One deliberate deviation from the WGSL, shared with the CPU oracle: the hit distance is
// (enter_coord - origin) / dir on the entry axis, not enter_coord * inv_dir + (-origin * inv_dir)
// (traversal64.wgsl:468-472), whose cancellation breaks 1e-5 relative depth far from the origin.
// The DDA decisions and the face choice keep the WGSL form.
#pragma once

#include "arc_math.cuh"
#include "../../include/arc/layout.h"

namespace arc {

constexpr uint32_t kStatusNodeRange = 1u;
constexpr uint32_t kStatusBrickRange = 2u;
constexpr uint32_t kStatusRootRange = 4u;

struct World {
    const uint32_t* __restrict__ roots;
    const uint4* __restrict__ nodes;
    const uint32_t* __restrict__ bricks;  // 16 words per brick
    const float4* __restrict__ palette;   // 2 float4 per material
    uint32_t n_nodes;
    uint32_t n_bricks;
    uint32_t n_roots;
    uint32_t* status;
    const arc_rigid_body* bodies;  // rigid bodies whose trees live in this node pool (may be null)
    uint32_t n_bodies;
};

__device__ __forceinline__ uint4 load_node(const World& w, uint32_t idx) {
    if (idx >= w.n_nodes) {
        atomicOr(w.status, kStatusNodeRange);
        return make_uint4(0u, 0u, 0u, 0u);
    }
    return __ldg(&w.nodes[idx]);
}

__device__ __forceinline__ uint32_t load_brick_mat(const World& w, uint32_t brick, uint32_t bit) {
    if (brick >= w.n_bricks) {
        atomicOr(w.status, kStatusBrickRange);
        return 0u;
    }
    uint32_t word = __ldg(&w.bricks[brick * 16u + (bit >> 2)]);
    return (word >> ((bit & 3u) * 8u)) & 0xFFu;
}

__device__ __forceinline__ uint32_t load_root(const World& w, uint32_t c_idx) {
    if (c_idx >= w.n_roots) {
        atomicOr(w.status, kStatusRootRange);
        return ARC_EMPTY_CHUNK;
    }
    return __ldg(&w.roots[c_idx]);
}

__device__ __forceinline__ bool has_child(uint32_t lo, uint32_t hi, uint32_t b) {
    return (((b < 32u ? lo : hi) >> (b & 31u)) & 1u) != 0u;
}

// base + popcount of the occupied children below bit b (traversal64.wgsl:32-40).
__device__ __forceinline__ uint32_t child_index(const uint4& n, uint32_t b) {
    uint32_t prefix = (1u << (b & 31u)) - 1u;
    uint32_t rank = b < 32u ? __popc(n.x & prefix) : __popc(n.x) + __popc(n.y & prefix);
    return (n.z & ARC_PTR_INDEX_MASK) + rank;
}

enum StepResult : uint32_t { kContinue = 0u, kHit = 1u, kMiss = 2u };

struct RayState {
    f3 vo;    // origin, voxel units
    f3 dir;   // unit direction as given
    f3 inv;   // 1 / safe_dir (-vo * inv, the reference's neg_orig_inv, is recomputed where used: same bits)
    float t, t_limit;
    uint32_t vx, vy, vz;
    uint32_t diff;            // previous vi ^ vi, per axis or-ed (0xFFFFFFFF before the first step)
    uint32_t mtf_c0, mtf_c1;  // packed chunk coords (x | y << 10 | z << 20), 0xFFFFFFFF = none
    uint32_t mtf_root0, mtf_root1;
    uint4 l1, l2, l3;         // ancestor restart cache (levels shift 4, 2, 0)
    uint32_t cached_shift;
    uint32_t step;
    uint32_t mode;            // lod_bias | ignore_water << 2
    // node-visit loop (ray_visit) only: the node under evaluation, its level, the LOD floor of the
    // current voxel, and whether the head of the outer loop still has to run at this voxel
    uint4 node;
    uint32_t nshift, min_shift, have_node;
    // kFeatPrecomp only: the ray class's step budget and LOD thresholds, and -vo * inv, computed once per ray
    uint32_t max_steps, lod_step, lod_shift;
    float lod_t, lod_t2;
    f3 noi;
};

// Traversal variants (the features field of arc_launch_config); every variant makes the same DDA
// decisions in the same order, so results are identical bit for bit.
constexpr int kFeatWarpFetch = 1;   // lanes that descend into the same node fetch it once per warp
constexpr int kFeatNodeVisit = 2;   // one node evaluation per loop iteration instead of a descent loop
constexpr int kFeatTopTable = 8;    // chunk roots and their level-1 children from a table staged in shared memory
constexpr int kFeatPrecomp = 32;    // step budget, LOD thresholds and -origin/dir of the ray computed once per ray

__device__ __forceinline__ float noi_x(const RayState& s) { return -s.vo.x * s.inv.x; }
__device__ __forceinline__ float noi_y(const RayState& s) { return -s.vo.y * s.inv.y; }
__device__ __forceinline__ float noi_z(const RayState& s) { return -s.vo.z * s.inv.z; }

// Step budget of the ray class (traversal64.wgsl:262-267).
__device__ __forceinline__ uint32_t max_steps_of(const arc_camera_uniforms& cam, uint32_t mode) {
    const uint32_t lod_bias = mode & 3u;
    return lod_bias == 0u ? cam.ray_steps[0] : (lod_bias == 1u ? cam.ray_steps[1] : cam.ray_steps[2]);
}

struct HitInfo {
    float t_voxels;   // accurate plane-entry distance (voxels)
    f3 hit_pos_m;
    f3 normal;
    uint32_t mat;
    uint32_t lod_payload;
    uint32_t vx, vy, vz;
    uint32_t shift;
    uint32_t voxel_hash;
    float contact_ao;
};

// Default (miss) outcome of trace_world_64tree_from (traversal64.wgsl:234-242).
__device__ __forceinline__ void hit_init_miss(HitInfo& h, f3 origin_m, f3 dir, float max_dist_m) {
    h.t_voxels = max_dist_m * ARC_VOXELS_PER_METER;
    h.hit_pos_m = add3(origin_m, mul3s(dir, max_dist_m));
    h.normal = f3{0.0f, 1.0f, 0.0f};
    h.mat = ARC_MAT_AIR;
    h.lod_payload = 0u;
    h.vx = h.vy = h.vz = 0xFFFFFFFFu;
    h.shift = 0u;
    h.voxel_hash = 0u;
    h.contact_ao = 1.0f;
}

__device__ __forceinline__ float safe_component(float d) { return fabsf(d) < 1e-7f ? 1e-7f : d; }

// Setup of trace_world_64tree_from; returns false when the ray misses the world outright.
__device__ __forceinline__ bool ray_begin(RayState& s, const arc_camera_uniforms& cam, f3 origin_m, f3 dir,
                                          float start_t_m, float max_dist_m, uint32_t lod_bias, bool ignore_water) {
    s.vo = mul3s(origin_m, ARC_VOXELS_PER_METER);
    s.dir = dir;
    float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    float start_t_v = fmaxf(start_t_m * ARC_VOXELS_PER_METER, 0.0f);
    s.inv = f3{__fdiv_rn(1.0f, safe_component(dir.x)), __fdiv_rn(1.0f, safe_component(dir.y)),
               __fdiv_rn(1.0f, safe_component(dir.z))};
    const float wx = (float)cam.world_grid_dims[0] * ARC_CHUNK_DIM_F;
    const float wy = (float)cam.world_grid_dims[1] * ARC_CHUNK_DIM_F;
    const float wz = (float)cam.world_grid_dims[2] * ARC_CHUNK_DIM_F;
    // intersect_aabb(vo, inv, 0, world_max) (traversal64.wgsl:134-142)
    float ax0 = ((s.inv.x > 0.0f ? 0.0f : wx) - s.vo.x) * s.inv.x;
    float ay0 = ((s.inv.y > 0.0f ? 0.0f : wy) - s.vo.y) * s.inv.y;
    float az0 = ((s.inv.z > 0.0f ? 0.0f : wz) - s.vo.z) * s.inv.z;
    float ax1 = ((s.inv.x > 0.0f ? wx : 0.0f) - s.vo.x) * s.inv.x;
    float ay1 = ((s.inv.y > 0.0f ? wy : 0.0f) - s.vo.y) * s.inv.y;
    float az1 = ((s.inv.z > 0.0f ? wz : 0.0f) - s.vo.z) * s.inv.z;
    float w_enter = fmaxf(fmaxf(ax0, ay0), az0);
    float w_exit = fminf(fminf(ax1, ay1), az1);
    float t_enter = fmaxf(w_enter, start_t_v);
    if (w_exit < t_enter || t_enter >= max_t_v) return false;
    s.t = t_enter;
    s.t_limit = fminf(w_exit, max_t_v);
    float st = s.t + 1e-4f;
    s.vx = f2u(clampf(s.vo.x + dir.x * st, 0.0f, wx - 1e-3f));
    s.vy = f2u(clampf(s.vo.y + dir.y * st, 0.0f, wy - 1e-3f));
    s.vz = f2u(clampf(s.vo.z + dir.z * st, 0.0f, wz - 1e-3f));
    s.diff = 0xFFFFFFFFu;
    s.mtf_c0 = s.mtf_c1 = 0xFFFFFFFFu;
    s.mtf_root0 = s.mtf_root1 = ARC_EMPTY_CHUNK;
    s.l1 = s.l2 = s.l3 = make_uint4(0u, 0u, 0u, 0u);
    s.cached_shift = 6u;
    s.step = 0u;
    s.mode = lod_bias | (ignore_water ? 4u : 0u);
    s.have_node = 0u;
    return true;
}

// The per-step quantities of the ray class that do not change along the ray (kFeatPrecomp): the step
// budget, the LOD floor's thresholds, min_shift = (t > lod_t || step > lod_step) ? lod_shift
// : (t > lod_t2 ? 2 : 0), and -vo * inv. The products are the ones ray_advance forms every step, so
// the decisions are unchanged.
__device__ __forceinline__ void ray_precompute(RayState& s, const arc_camera_uniforms& cam) {
    const uint32_t lod_bias = s.mode & 3u;
    s.max_steps = max_steps_of(cam, s.mode);
    if (lod_bias == 0u) {
        s.lod_t = cam.lod_settings[0] * ARC_VOXELS_PER_METER;
        s.lod_step = cam.quality_flags[0];
        s.lod_shift = 2u;
        s.lod_t2 = __uint_as_float(0x7F800000u);  // +inf: no second threshold
    } else if (lod_bias == 1u) {
        const float sec_t = cam.lod_settings[1] * ARC_VOXELS_PER_METER;
        s.lod_t = sec_t * 2.2857f;
        s.lod_step = cam.quality_flags[1];
        s.lod_shift = 4u;
        s.lod_t2 = sec_t;
    } else {
        s.lod_t = cam.lod_settings[2] * ARC_VOXELS_PER_METER;
        s.lod_step = (cam.quality_flags[3] >> 16) & 0xFFu;
        s.lod_shift = 2u;
        s.lod_t2 = __uint_as_float(0x7F800000u);
    }
    s.noi = f3{noi_x(s), noi_y(s), noi_z(s)};
}

__device__ __forceinline__ uint32_t lane_id() {
    uint32_t l;
    asm volatile("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}

// A child node fetch. With kFeatWarpFetch the lanes of a warp that need the same node index elect one
// lane to load it and receive it by shuffle (one request per distinct node instead of one per lane).
template <int FEAT>
__device__ __forceinline__ uint4 fetch_node(const World& w, uint32_t idx) {
    if constexpr ((FEAT & kFeatWarpFetch) != 0) {
        const uint32_t act = __activemask();
        const uint32_t peers = __match_any_sync(act, idx);
        const int leader = __ffs(peers) - 1;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if ((int)lane_id() == leader) v = load_node(w, idx);
        v.x = __shfl_sync(act, v.x, leader);
        v.y = __shfl_sync(act, v.y, leader);
        v.z = __shfl_sync(act, v.z, leader);
        v.w = __shfl_sync(act, v.w, leader);
        return v;
    } else {
        return load_node(w, idx);
    }
}

// step_dda_box (traversal64.wgsl:152-179) over the box [bmin, bmin + span)^3. PRE: -vo * inv from the
// ray state (ray_precompute) instead of formed here; the same bits either way.
template <bool PRE = false>
__device__ __forceinline__ void step_box(RayState& s, uint32_t bx, uint32_t by, uint32_t bz, uint32_t span) {
    const bool pxd = s.inv.x >= 0.0f, pyd = s.inv.y >= 0.0f, pzd = s.inv.z >= 0.0f;
    uint32_t ex = pxd ? bx + span : bx, ey = pyd ? by + span : by, ez = pzd ? bz + span : bz;
    float tx = (float)ex * s.inv.x + (PRE ? s.noi.x : noi_x(s));
    float ty = (float)ey * s.inv.y + (PRE ? s.noi.y : noi_y(s));
    float tz = (float)ez * s.inv.z + (PRE ? s.noi.z : noi_z(s));
    float t_exit = fminf(fminf(tx, ty), tz);
    float next_t = fmaxf(s.t, t_exit);
    bool is_x = tx <= ty && tx <= tz;
    bool is_y = !is_x && (ty <= tz);
    bool is_z = !is_x && !is_y;
    uint32_t ox = ex - (pxd ? 0u : 1u), oy = ey - (pyd ? 0u : 1u), oz = ez - (pzd ? 0u : 1u);
    // max(x, 0) before the conversion is implied: cvt.rzi.u32.f32 clamps to [0, 2^32 - 1] and turns NaN into 0
    uint32_t ix = uclamp(f2u(s.vo.x + s.dir.x * next_t), bx, bx + span - 1u);
    uint32_t iy = uclamp(f2u(s.vo.y + s.dir.y * next_t), by, by + span - 1u);
    uint32_t iz = uclamp(f2u(s.vo.z + s.dir.z * next_t), bz, bz + span - 1u);
    const uint32_t nx = is_x ? ox : ix, ny = is_y ? oy : iy, nz = is_z ? oz : iz;
    s.t = next_t;
    s.diff = (s.vx ^ nx) | (s.vy ^ ny) | (s.vz ^ nz);
    s.vx = nx;
    s.vy = ny;
    s.vz = nz;
}

// eval_leaf_bitwise_ao (traversal64.wgsl:60-131).
__device__ __forceinline__ float leaf_ao(uint32_t lo, uint32_t hi, uint32_t cx, uint32_t cy, uint32_t cz, f3 n, f3 hp) {
    float fx = clampf(fractf(hp.x), 0.0f, 1.0f);
    float fy = clampf(fractf(hp.y), 0.0f, 1.0f);
    float fz = clampf(fractf(hp.z), 0.0f, 1.0f);
    int nx = (int)cx + (int)n.x, ny = (int)cy + (int)n.y, nz = (int)cz + (int)n.z;
    if (nx < 0 || nx > 3 || ny < 0 || ny > 3 || nz < 0 || nz > 3) return 1.0f;
    uint32_t bb = ((uint32_t)nz << 4) | ((uint32_t)ny << 2) | (uint32_t)nx;
    float occ = 0.0f;
    if (fabsf(n.y) > 0.5f) {
        if (nx > 0 && has_child(lo, hi, bb - 1u)) occ += (1.0f - fx) * 0.42f;
        if (nx < 3 && has_child(lo, hi, bb + 1u)) occ += fx * 0.42f;
        if (nz > 0 && has_child(lo, hi, bb - 16u)) occ += (1.0f - fz) * 0.42f;
        if (nz < 3 && has_child(lo, hi, bb + 16u)) occ += fz * 0.42f;
    } else if (fabsf(n.x) > 0.5f) {
        if (ny > 0 && has_child(lo, hi, bb - 4u)) occ += (1.0f - fy) * 0.42f;
        if (ny < 3 && has_child(lo, hi, bb + 4u)) occ += fy * 0.42f;
        if (nz > 0 && has_child(lo, hi, bb - 16u)) occ += (1.0f - fz) * 0.42f;
        if (nz < 3 && has_child(lo, hi, bb + 16u)) occ += fz * 0.42f;
    } else {
        if (nx > 0 && has_child(lo, hi, bb - 1u)) occ += (1.0f - fx) * 0.42f;
        if (nx < 3 && has_child(lo, hi, bb + 1u)) occ += fx * 0.42f;
        if (ny > 0 && has_child(lo, hi, bb - 4u)) occ += (1.0f - fy) * 0.42f;
        if (ny < 3 && has_child(lo, hi, bb + 4u)) occ += fy * 0.42f;
    }
    return clampf(1.0f - occ, 0.35f, 1.0f);
}

// Hit resolution of a solid cell (traversal64.wgsl:467-521): accurate entry distance, tie-broken
// face normal, voxel hash and contact AO. It has a single call site in ray_advance.
__device__ __forceinline__ void resolve_hit(const RayState& s, const arc_camera_uniforms& cam, uint4 node, uint32_t mat,
                                         uint32_t bx, uint32_t by, uint32_t bz, uint32_t span, uint32_t shift, uint32_t b,
                                         HitInfo& h) {
    const bool pxd = s.inv.x >= 0.0f, pyd = s.inv.y >= 0.0f, pzd = s.inv.z >= 0.0f;
    const uint32_t ex = pxd ? bx : bx + span, ey = pyd ? by : by + span, ez = pzd ? bz : bz + span;
    const float tx = (float)ex * s.inv.x + noi_x(s);
    const float ty = (float)ey * s.inv.y + noi_y(s);
    const float tz = (float)ez * s.inv.z + noi_z(s);
    const float max_t = fmaxf(fmaxf(tx, ty), tz);
    // accurate entry distance on the entry axis (ties: x, then y)
    float t_acc;
    if (tx >= ty && tx >= tz) t_acc = __fdiv_rn((float)ex - s.vo.x, safe_component(s.dir.x));
    else if (ty >= tz) t_acc = __fdiv_rn((float)ey - s.vo.y, safe_component(s.dir.y));
    else t_acc = __fdiv_rn((float)ez - s.vo.z, safe_component(s.dir.z));
    const float exact_t = fmaxf(t_acc, 0.0f);
    const f3 hp = add3(s.vo, mul3s(s.dir, exact_t));
    h.t_voxels = exact_t;
    h.hit_pos_m = mul3s(hp, ARC_VOXEL_SIZE);
    const float eps = 1e-4f * fmaxf(max_t * 0.01f, 1.0f);
    const float cand_x = fabsf(tx - max_t) <= eps ? fabsf(s.dir.x) : 0.0f;
    const float cand_y = fabsf(ty - max_t) <= eps ? fabsf(s.dir.y) : 0.0f;
    const float cand_z = fabsf(tz - max_t) <= eps ? fabsf(s.dir.z) : 0.0f;
    f3 n{0.0f, 0.0f, 0.0f};
    if (cand_x >= cand_y && cand_x >= cand_z && cand_x > 0.0f) n.x = -signf(s.dir.x);
    else if (cand_y >= cand_z && cand_y > 0.0f) n.y = -signf(s.dir.y);
    else if (cand_z > 0.0f) n.z = -signf(s.dir.z);
    else if (tx >= ty && tx >= tz) n.x = -signf(s.dir.x);
    else if (ty >= tz) n.y = -signf(s.dir.y);
    else n.z = -signf(s.dir.z);
    h.normal = n;
    h.mat = mat;
    h.lod_payload = node.w;
    h.vx = s.vx;
    h.vy = s.vy;
    h.vz = s.vz;
    h.shift = shift;
    h.voxel_hash = pcg_hash((s.vx * 73856093u) ^ (s.vy * 19349663u) ^ (s.vz * 83492791u));
    h.contact_ao = 1.0f;
    if (shift == 0u && (s.mode & 3u) == 0u) {
        const float hit_dist_m = s.t * ARC_VOXEL_SIZE;
        const float raw = __uint_as_float(cam.point_light_count[3]);
        const float ao_max = raw < 1.0f ? 24.0f : raw;
        if (hit_dist_m < ao_max) {
            const float raw_ao = leaf_ao(node.x, node.y, b & 3u, (b >> 2) & 3u, b >> 4, n, hp);
            const float wgt = 1.0f - smoothstepf(ao_max * 0.5f, ao_max, hit_dist_m);
            h.contact_ao = mixf(1.0f, raw_ao, wgt);
        }
    }
}

// One outer-loop iteration of trace_world_64tree_from (traversal64.wgsl:302-553).
//
// Every branch of the reference loop ends in step_dda_box over some box: the whole chunk (empty
// chunk, 337-352), the uniform water node (398-417), the empty child cell (419-436), the water leaf
// cell (451-465) or the air leaf cell (525-537). Here the branches only choose the box's span and one
// convergent step_box runs after them, so lanes that took different branches step together instead
// of executing five inlined copies one after another. Decisions and their order are unchanged.
// The top two tree levels staged in shared memory for kFeatTopTable: roots[c] is chunk c's root node
// with the child index of an internal root rebased into l1[], which holds every root's level-1 children
// (each root's child slice, in order). Null roots: the nodes come from the pool as usual.
struct TopView {
    const uint4* roots;
    const uint4* l1;
};

template <int FEAT = 0>
__device__ __forceinline__ StepResult ray_advance(RayState& s, const World& w, const arc_camera_uniforms& cam,
                                                  HitInfo& h, const TopView top = TopView{nullptr, nullptr}) {
    if constexpr ((FEAT & kFeatPrecomp) != 0) {
        if (s.step >= s.max_steps) return kMiss;
    } else {
        if (s.step >= max_steps_of(cam, s.mode)) return kMiss;
    }
    if (s.t >= s.t_limit) return kMiss;
    const uint32_t gx = cam.world_grid_dims[0], gy = cam.world_grid_dims[1], gz = cam.world_grid_dims[2];
    if (s.vx >= (gx << 8) || s.vy >= (gy << 8) || s.vz >= (gz << 8)) return kMiss;

    const uint32_t diff = s.diff;  // the voxel changes only in step_box, which records how
    uint32_t root_idx = s.mtf_root0;
    if (diff >= 256u) {
        const uint32_t cxk = s.vx >> 8, cyk = s.vy >> 8, czk = s.vz >> 8;
        const uint32_t c = cxk | (cyk << 10) | (czk << 20);
        s.cached_shift = 6u;
        if (c == s.mtf_c1) {
            root_idx = s.mtf_root1;
        } else {
            root_idx = load_root(w, cxk + cyk * gx + czk * gx * gy);
        }
        s.mtf_c1 = s.mtf_c0;
        s.mtf_root1 = s.mtf_root0;
        s.mtf_c0 = c;
        s.mtf_root0 = root_idx;
    }

    uint32_t span = 256u;  // empty chunk: leave the whole chunk
    if (root_idx != ARC_EMPTY_CHUNK) {
        const uint32_t lod_bias = s.mode & 3u;
        const bool ignore_water = (s.mode & 4u) != 0u;
        uint32_t min_shift = 0u;
        if constexpr ((FEAT & kFeatPrecomp) != 0) {
            min_shift = (s.t > s.lod_t || s.step > s.lod_step) ? s.lod_shift : (s.t > s.lod_t2 ? 2u : 0u);
        } else if (lod_bias == 0u) {
            if (s.t > cam.lod_settings[0] * ARC_VOXELS_PER_METER || s.step > cam.quality_flags[0]) min_shift = 2u;
        } else if (lod_bias == 1u) {
            const float sec_t = cam.lod_settings[1] * ARC_VOXELS_PER_METER;
            if (s.t > sec_t * 2.2857f || s.step > cam.quality_flags[1]) min_shift = 4u;
            else if (s.t > sec_t) min_shift = 2u;
        } else {
            if (s.t > cam.lod_settings[2] * ARC_VOXELS_PER_METER || s.step > ((cam.quality_flags[3] >> 16) & 0xFFu))
                min_shift = 2u;
        }

        uint4 node;
        uint32_t shift;
        if (diff < 4u && min_shift == 0u && s.cached_shift == 0u) {
            node = s.l3;
            shift = 0u;
        } else if (diff < 16u && min_shift <= 2u && s.cached_shift <= 2u) {
            node = s.l2;
            shift = 2u;
        } else if (diff < 64u && min_shift <= 4u && s.cached_shift <= 4u) {
            node = s.l1;
            shift = 4u;
        } else {
            if constexpr ((FEAT & kFeatTopTable) != 0) {
                node = top.roots ? top.roots[(s.vx >> 8) + (s.vy >> 8) * gx + (s.vz >> 8) * gx * gy] : load_node(w, root_idx);
            } else {
                node = load_node(w, root_idx);
            }
            shift = 6u;
        }
        s.cached_shift = shift;

        const uint32_t lx = s.vx & 255u, ly = s.vy & 255u, lz = s.vz & 255u;
        for (;;) {
            const uint32_t b = (((lz >> shift) & 3u) << 4) | (((ly >> shift) & 3u) << 2) | ((lx >> shift) & 3u);
            if (ignore_water && (node.z & ARC_IS_UNIFORM_FLAG) != 0u && ((node.w >> 24) & 0xFFu) == ARC_MAT_WATER_CRYSTAL) {
                span = 4u << shift;  // uniform water node
                break;
            }
            span = 1u << shift;
            if (!has_child(node.x, node.y, b)) break;  // empty child cell
            const bool is_leaf = (node.z & ARC_IS_LEAF_FLAG) != 0u;
            if (is_leaf || shift <= min_shift) {
                uint32_t mat = (node.w >> 24) & 0xFFu;
                if (is_leaf && (node.z & ARC_IS_UNIFORM_FLAG) == 0u) mat = load_brick_mat(w, node.z & ARC_PTR_INDEX_MASK, b);
                if (ignore_water && mat == ARC_MAT_WATER_CRYSTAL) break;  // water cell
                if (mat != ARC_MAT_AIR) {
                    resolve_hit(s, cam, node, mat, s.vx & ~(span - 1u), s.vy & ~(span - 1u), s.vz & ~(span - 1u), span,
                                shift, b, h);
                    return kHit;
                }
                break;  // air leaf cell
            }
            if constexpr ((FEAT & kFeatTopTable) != 0) {
                // at level 6 the node is the chunk root, from the table when it is staged
                node = (shift == 6u && top.roots) ? top.l1[child_index(node, b)] : fetch_node<FEAT>(w, child_index(node, b));
            } else {
                node = fetch_node<FEAT>(w, child_index(node, b));
            }
            shift -= 2u;
            s.cached_shift = shift;
            if (shift == 4u) s.l1 = node;
            else if (shift == 2u) s.l2 = node;
            else if (shift == 0u) s.l3 = node;
        }
    }
    step_box<(FEAT & kFeatPrecomp) != 0>(s, s.vx & ~(span - 1u), s.vy & ~(span - 1u), s.vz & ~(span - 1u), span);
    s.step++;
    return kContinue;
}

// ray_advance with the descent loop unrolled across calls (kFeatNodeVisit): every call evaluates one
// node. A call at a new voxel first runs the head of the reference's outer loop (budget and bounds
// checks, chunk MTF cache, LOD floor, ancestor restart: traversal64.wgsl:302-387); a call that
// descends loads the child and returns, and the next call evaluates it; a call that decides the cell
// steps. Lanes of a warp then spend one short, mostly common iteration per node instead of waiting
// in the descent loop for the deepest lane. The state changes, their order and the results are
// those of ray_advance.
template <int FEAT = 0>
__device__ __forceinline__ StepResult ray_visit(RayState& s, const World& w, const arc_camera_uniforms& cam,
                                                HitInfo& h) {
    uint32_t span = 256u;  // empty chunk: leave the whole chunk
    bool eval = true;
    if (!s.have_node) {
        if (s.step >= max_steps_of(cam, s.mode)) return kMiss;
        if (s.t >= s.t_limit) return kMiss;
        const uint32_t gx = cam.world_grid_dims[0], gy = cam.world_grid_dims[1], gz = cam.world_grid_dims[2];
        if (s.vx >= (gx << 8) || s.vy >= (gy << 8) || s.vz >= (gz << 8)) return kMiss;
        const uint32_t diff = s.diff;
        uint32_t root_idx = s.mtf_root0;
        if (diff >= 256u) {
            const uint32_t cxk = s.vx >> 8, cyk = s.vy >> 8, czk = s.vz >> 8;
            const uint32_t c = cxk | (cyk << 10) | (czk << 20);
            s.cached_shift = 6u;
            if (c == s.mtf_c1) root_idx = s.mtf_root1;
            else root_idx = load_root(w, cxk + cyk * gx + czk * gx * gy);
            s.mtf_c1 = s.mtf_c0;
            s.mtf_root1 = s.mtf_root0;
            s.mtf_c0 = c;
            s.mtf_root0 = root_idx;
        }
        if (root_idx == ARC_EMPTY_CHUNK) {
            eval = false;
        } else {
            const uint32_t lod_bias = s.mode & 3u;
            uint32_t min_shift = 0u;
            if (lod_bias == 0u) {
                if (s.t > cam.lod_settings[0] * ARC_VOXELS_PER_METER || s.step > cam.quality_flags[0]) min_shift = 2u;
            } else if (lod_bias == 1u) {
                const float sec_t = cam.lod_settings[1] * ARC_VOXELS_PER_METER;
                if (s.t > sec_t * 2.2857f || s.step > cam.quality_flags[1]) min_shift = 4u;
                else if (s.t > sec_t) min_shift = 2u;
            } else {
                if (s.t > cam.lod_settings[2] * ARC_VOXELS_PER_METER || s.step > ((cam.quality_flags[3] >> 16) & 0xFFu))
                    min_shift = 2u;
            }
            s.min_shift = min_shift;
            if (diff < 4u && min_shift == 0u && s.cached_shift == 0u) {
                s.node = s.l3;
                s.nshift = 0u;
            } else if (diff < 16u && min_shift <= 2u && s.cached_shift <= 2u) {
                s.node = s.l2;
                s.nshift = 2u;
            } else if (diff < 64u && min_shift <= 4u && s.cached_shift <= 4u) {
                s.node = s.l1;
                s.nshift = 4u;
            } else {
                s.node = load_node(w, root_idx);
                s.nshift = 6u;
            }
            s.cached_shift = s.nshift;
            s.have_node = 1u;
        }
    }
    if (eval) {
        const uint32_t shift = s.nshift;
        const uint4 node = s.node;
        const bool ignore_water = (s.mode & 4u) != 0u;
        const uint32_t lx = s.vx & 255u, ly = s.vy & 255u, lz = s.vz & 255u;
        const uint32_t b = (((lz >> shift) & 3u) << 4) | (((ly >> shift) & 3u) << 2) | ((lx >> shift) & 3u);
        if (ignore_water && (node.z & ARC_IS_UNIFORM_FLAG) != 0u && ((node.w >> 24) & 0xFFu) == ARC_MAT_WATER_CRYSTAL) {
            span = 4u << shift;  // uniform water node
        } else {
            span = 1u << shift;
            if (has_child(node.x, node.y, b)) {
                const bool is_leaf = (node.z & ARC_IS_LEAF_FLAG) != 0u;
                if (is_leaf || shift <= s.min_shift) {
                    uint32_t mat = (node.w >> 24) & 0xFFu;
                    if (is_leaf && (node.z & ARC_IS_UNIFORM_FLAG) == 0u)
                        mat = load_brick_mat(w, node.z & ARC_PTR_INDEX_MASK, b);
                    if (!(ignore_water && mat == ARC_MAT_WATER_CRYSTAL) && mat != ARC_MAT_AIR) {
                        resolve_hit(s, cam, node, mat, s.vx & ~(span - 1u), s.vy & ~(span - 1u), s.vz & ~(span - 1u),
                                    span, shift, b, h);
                        return kHit;
                    }
                    // water cell or air leaf cell: step
                } else {
                    const uint4 child = fetch_node<FEAT>(w, child_index(node, b));
                    const uint32_t cs = shift - 2u;
                    s.node = child;
                    s.nshift = cs;
                    s.cached_shift = cs;
                    if (cs == 4u) s.l1 = child;
                    else if (cs == 2u) s.l2 = child;
                    else if (cs == 0u) s.l3 = child;
                    return kContinue;  // the next call evaluates the child
                }
            }
        }
    }
    step_box(s, s.vx & ~(span - 1u), s.vy & ~(span - 1u), s.vz & ~(span - 1u), span);
    s.step++;
    s.have_node = 0u;
    return kContinue;
}

// The traversal loop body of a kernel instantiated with the feature bits FEAT.
template <int FEAT>
__device__ __forceinline__ StepResult ray_next(RayState& s, const World& w, const arc_camera_uniforms& cam, HitInfo& h) {
    if constexpr ((FEAT & kFeatNodeVisit) != 0) return ray_visit<FEAT>(s, w, cam, h);
    else return ray_advance<FEAT>(s, w, cam, h);
}

// is_emissive_mat (traversal64.wgsl:775-777)
__device__ __forceinline__ bool is_emissive_mat(uint32_t m) { return (m >= 19u && m <= 22u) || m == 24u || m == 27u; }

// trace_shadow_vis (traversal64.wgsl:571-773) for kDi = false; trace_shadow_vis_di (781-989), the
// ReSTIR DI any-hit ray towards an emitter, for kDi = true. 1.0 unoccluded, 0.0 occluded. The DI
// variant clamps the step budget to [32, 48], coarsens only with distance left to the target, reads
// brick materials, lets an emissive hit within 16 voxels of the target through, and calls the ray
// visible only when it ended within 2 voxels of the target.
template <bool kDi>
__device__ __forceinline__ float shadow_vis_t(const World& w, const arc_camera_uniforms& cam, f3 origin_m, f3 dir,
                                              float max_dist_m) {
    const f3 vo = mul3s(origin_m, ARC_VOXELS_PER_METER);
    const float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    RayState s;
    s.vo = vo;
    s.dir = dir;
    s.inv = f3{__fdiv_rn(1.0f, safe_component(dir.x)), __fdiv_rn(1.0f, safe_component(dir.y)),
               __fdiv_rn(1.0f, safe_component(dir.z))};
    const uint32_t gx = cam.world_grid_dims[0], gy = cam.world_grid_dims[1], gz = cam.world_grid_dims[2];
    const float wx = (float)gx * ARC_CHUNK_DIM_F, wy = (float)gy * ARC_CHUNK_DIM_F, wz = (float)gz * ARC_CHUNK_DIM_F;
    float ax0 = ((s.inv.x > 0.0f ? 0.0f : wx) - vo.x) * s.inv.x;
    float ay0 = ((s.inv.y > 0.0f ? 0.0f : wy) - vo.y) * s.inv.y;
    float az0 = ((s.inv.z > 0.0f ? 0.0f : wz) - vo.z) * s.inv.z;
    float ax1 = ((s.inv.x > 0.0f ? wx : 0.0f) - vo.x) * s.inv.x;
    float ay1 = ((s.inv.y > 0.0f ? wy : 0.0f) - vo.y) * s.inv.y;
    float az1 = ((s.inv.z > 0.0f ? wz : 0.0f) - vo.z) * s.inv.z;
    float w_enter = fmaxf(fmaxf(ax0, ay0), az0);
    float w_exit = fminf(fminf(ax1, ay1), az1);
    if (w_exit < fmaxf(w_enter, 0.0f) || w_enter >= max_t_v) return 1.0f;
    s.t = fmaxf(w_enter, 0.0f);
    s.t_limit = fminf(w_exit, max_t_v);
    const uint32_t max_steps = kDi ? umin(umax(cam.ray_steps[3], 32u), 48u) : cam.ray_steps[3];
    float st = s.t + 1e-4f;
    s.vx = f2u(clampf(vo.x + dir.x * st, 0.0f, wx - 1e-3f));
    s.vy = f2u(clampf(vo.y + dir.y * st, 0.0f, wy - 1e-3f));
    s.vz = f2u(clampf(vo.z + dir.z * st, 0.0f, wz - 1e-3f));
    uint32_t px = 0xFFFFFFFFu, py = 0xFFFFFFFFu, pz = 0xFFFFFFFFu;
    uint32_t cached_shift = 6u;
    uint4 l1 = make_uint4(0, 0, 0, 0), l2 = l1, l3 = l1;
    uint32_t cached_root = ARC_EMPTY_CHUNK;
    for (uint32_t step = 0; step < max_steps; ++step) {
        if (s.t >= s.t_limit) break;
        if (s.vx >= (gx << 8) || s.vy >= (gy << 8) || s.vz >= (gz << 8)) {
            s.t = s.t_limit;
            break;
        }
        const uint32_t diff = (px ^ s.vx) | (py ^ s.vy) | (pz ^ s.vz);
        px = s.vx;
        py = s.vy;
        pz = s.vz;
        uint32_t root_idx = cached_root;
        if (diff >= 256u) {
            cached_shift = 6u;
            root_idx = load_root(w, (s.vx >> 8) + (s.vy >> 8) * gx + (s.vz >> 8) * gx * gy);
            cached_root = root_idx;
        }
        if (root_idx == ARC_EMPTY_CHUNK) {
            step_box(s, s.vx & ~255u, s.vy & ~255u, s.vz & ~255u, 256u);
            continue;
        }
        uint32_t min_shift = 0u;
        if (kDi) {
            const float dist_rem = s.t_limit - s.t;
            if (s.t > 48.0f && dist_rem > 32.0f && step > 6u) min_shift = 2u;
            if (s.t > 160.0f && dist_rem > 64.0f && step > 14u) min_shift = 4u;
        } else {
            if (s.t > 48.0f || step > 6u) min_shift = 2u;
            if (s.t > 192.0f || step > 16u) min_shift = 4u;
        }
        uint4 node;
        uint32_t shift;
        if (diff < 4u && min_shift == 0u && cached_shift == 0u) { node = l3; shift = 0u; }
        else if (diff < 16u && min_shift <= 2u && cached_shift <= 2u) { node = l2; shift = 2u; }
        else if (diff < 64u && min_shift <= 4u && cached_shift <= 4u) { node = l1; shift = 4u; }
        else { node = load_node(w, root_idx); shift = 6u; }
        cached_shift = shift;
        const uint32_t lx = s.vx & 255u, ly = s.vy & 255u, lz = s.vz & 255u;
        for (;;) {
            const uint32_t b = (((lz >> shift) & 3u) << 4) | (((ly >> shift) & 3u) << 2) | ((lx >> shift) & 3u);
            if ((node.z & ARC_IS_UNIFORM_FLAG) != 0u && ((node.w >> 24) & 0xFFu) == ARC_MAT_WATER_CRYSTAL) {
                const uint32_t span = 4u << shift;
                step_box(s, s.vx & ~(span - 1u), s.vy & ~(span - 1u), s.vz & ~(span - 1u), span);
                break;
            }
            const uint32_t span = 1u << shift;
            const uint32_t bx = s.vx & ~(span - 1u), by = s.vy & ~(span - 1u), bz = s.vz & ~(span - 1u);
            if (!has_child(node.x, node.y, b)) {
                step_box(s, bx, by, bz, span);
                break;
            }
            const bool is_leaf = (node.z & ARC_IS_LEAF_FLAG) != 0u, is_uniform = (node.z & ARC_IS_UNIFORM_FLAG) != 0u;
            if (is_leaf || (kDi && is_uniform) || shift <= min_shift) {
                uint32_t mat = (node.w >> 24) & 0xFFu;
                if (kDi && is_leaf && !is_uniform && shift == 0u) mat = load_brick_mat(w, node.z & ARC_PTR_INDEX_MASK, b);
                if (mat == ARC_MAT_WATER_CRYSTAL) {
                    step_box(s, bx, by, bz, span);
                    break;
                }
                if (kDi && is_emissive_mat(mat) && s.t >= s.t_limit - 16.0f) return 1.0f;
                return 0.0f;
            }
            node = load_node(w, child_index(node, b));
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) l1 = node;
            else if (shift == 2u) l2 = node;
            else if (shift == 0u) l3 = node;
        }
    }
    if (kDi) return s.t >= s.t_limit - 2.0f ? 1.0f : 0.0f;
    if (s.t < s.t_limit) {
        if ((vo.y + dir.y * s.t) * ARC_VOXEL_SIZE < 32.0f) return 0.0f;
    }
    return 1.0f;
}

__device__ __forceinline__ float shadow_vis(const World& w, const arc_camera_uniforms& cam, f3 origin_m, f3 dir,
                                            float max_dist_m) {
    return shadow_vis_t<false>(w, cam, origin_m, dir, max_dist_m);
}
__device__ __forceinline__ float shadow_vis_di(const World& w, const arc_camera_uniforms& cam, f3 origin_m, f3 dir,
                                               float max_dist_m) {
    return shadow_vis_t<true>(w, cam, origin_m, dir, max_dist_m);
}

// Pinhole camera ray (primary_gbuffer.wgsl:103-115, reconstruct_ray_dir types.wgsl:334-345).
__device__ __forceinline__ f3 camera_dir(const arc_camera_uniforms& cam, uint32_t x, uint32_t y, uint32_t W, uint32_t H) {
    const float u = __fdiv_rn(((float)x + 0.5f) + cam.jitter_brush_dt[0], (float)W);
    const float v = __fdiv_rn(((float)y + 0.5f) + cam.jitter_brush_dt[1], (float)H);
    const float nx = u * 2.0f - 1.0f, ny = 1.0f - v * 2.0f;
    const float th = cam.cam_forward_fov[3];
    const float sx = (nx * cam.cam_right_aspect[3]) * th, sy = ny * th;
    f3 r{(cam.cam_forward_fov[0] + cam.cam_right_aspect[0] * sx) + cam.cam_up_frame[0] * sy,
         (cam.cam_forward_fov[1] + cam.cam_right_aspect[1] * sx) + cam.cam_up_frame[1] * sy,
         (cam.cam_forward_fov[2] + cam.cam_right_aspect[2] * sx) + cam.cam_up_frame[2] * sy};
    return normalize3(r);
}

// probe_emissive_macro_candidate (lighting_restir_gi.wgsl:20-54).
__device__ __forceinline__ float probe_emissive(const World& w, const arc_camera_uniforms& cam, f3 pos, f3 d, float dist) {
    const f3 vp = mul3s(add3(pos, mul3s(d, dist)), ARC_VOXELS_PER_METER);
    const uint32_t gx = cam.world_grid_dims[0], gy = cam.world_grid_dims[1], gz = cam.world_grid_dims[2];
    if (vp.x < 0.0f || vp.y < 0.0f || vp.z < 0.0f) return 0.0f;
    if (vp.x >= (float)gx * ARC_CHUNK_DIM_F || vp.y >= (float)gy * ARC_CHUNK_DIM_F || vp.z >= (float)gz * ARC_CHUNK_DIM_F)
        return 0.0f;
    const uint32_t vx = f2u(vp.x), vy = f2u(vp.y), vz = f2u(vp.z);
    const uint32_t root_idx = load_root(w, (vx >> 8) + (vy >> 8) * gx + (vz >> 8) * gx * gy);
    if (root_idx == ARC_EMPTY_CHUNK) return 0.0f;
    const uint32_t lx = vx & 255u, ly = vy & 255u, lz = vz & 255u;
    const uint4 root = load_node(w, root_idx);
    const uint32_t b0 = (((lz >> 6) & 3u) << 4) | (((ly >> 6) & 3u) << 2) | ((lx >> 6) & 3u);
    if (!has_child(root.x, root.y, b0)) return 0.0f;
    uint32_t m_id;
    if (root.z & ARC_IS_LEAF_FLAG) {
        m_id = (root.w >> 24) & 0xFFu;
    } else {
        const uint4 l1 = load_node(w, child_index(root, b0));
        const uint32_t b1 = (((lz >> 4) & 3u) << 4) | (((ly >> 4) & 3u) << 2) | ((lx >> 4) & 3u);
        if (!has_child(l1.x, l1.y, b1)) return 0.0f;
        m_id = (l1.w >> 24) & 0xFFu;
    }
    const float4 em = __ldg(&w.palette[2u * m_id + 1u]);
    return (em.x * 0.333f + em.y * 0.333f) + em.z * 0.333f;
}

// What the GI ray setup of a hit pixel also yields for the temporal pass: primary hit point and
// normal, the smoothed hemisphere normal, the noise pair and whether the emissive probe chose the
// candidate direction.
struct GiSetup {
    float hit_dist;
    f3 hit_pos, normal, smooth_n;
    float u1, u2;
    bool guided;
};

// GI secondary ray of a hit pixel from its G-buffer words (lighting_restir_gi.wgsl:69-87, 195-209).
__device__ __forceinline__ bool gi_setup_full(const World& w, const arc_camera_uniforms& cam, uint32_t x, uint32_t y,
                                              uint32_t W, uint32_t H, uint32_t depth_word, uint32_t normal_word,
                                              f3* origin, f3* dir, GiSetup* g) {
    const float hit_dist = __uint_as_float(depth_word);
    if (hit_dist >= 1e4f) return false;
    const f3 rd = camera_dir(cam, x, y, W, H);
    const f3 eye{cam.cam_pos_time[0], cam.cam_pos_time[1], cam.cam_pos_time[2]};
    const f3 hp = add3(eye, mul3s(rd, hit_dist));
    float ox, oy;
    unpack2x16snorm(normal_word, &ox, &oy);
    const f3 n = oct_decode(ox, oy);
    float u1, u2;
    gradient_noise((float)x, (float)y, __float_as_uint(cam.cam_up_frame[3]), &u1, &u2);
    const f3 sn = normalize3(f3{n.x + 0.0f, n.y + 0.22f, n.z + 0.0f});
    f3 bt, bb;
    make_basis(sn, &bt, &bb);
    f3 bd = cosine_sample(u1, u2, sn, bt, bb);
    const f3 cd = cosine_sample(fractf(u1 + 0.5f), fractf(u2 + 0.381966f), sn, bt, bb);
    const float em_near = probe_emissive(w, cam, hp, cd, 1.25f);
    const float em_mid = probe_emissive(w, cam, hp, cd, 3.0f);
    const bool guided = fmaxf(em_near, em_mid) > 0.25f;
    if (guided) bd = cd;
    *origin = add3(hp, mul3s(n, 0.10f));
    *dir = bd;
    g->hit_dist = hit_dist;
    g->hit_pos = hp;
    g->normal = n;
    g->smooth_n = sn;
    g->u1 = u1;
    g->u2 = u2;
    g->guided = guided;
    return true;
}

__device__ __forceinline__ bool gi_setup(const World& w, const arc_camera_uniforms& cam, uint32_t x, uint32_t y,
                                         uint32_t W, uint32_t H, uint32_t depth_word, uint32_t normal_word, f3* origin,
                                         f3* dir) {
    GiSetup g;
    return gi_setup_full(w, cam, x, y, W, H, depth_word, normal_word, origin, dir, &g);
}

// lod_payload of the node whose child cells have span 1 << shift on the way from the chunk root to
// voxel (vx, vy, vz): the node a traversal hit at that cell read its payload from (leaf, uniform
// leaf or LOD cell). The voxel must lie in a non-empty chunk.
__device__ __forceinline__ uint32_t lod_payload_at(const World& w, const arc_camera_uniforms& cam, uint32_t vx, uint32_t vy,
                                                   uint32_t vz, uint32_t shift) {
    const uint32_t gx = cam.world_grid_dims[0], gy = cam.world_grid_dims[1];
    const uint32_t root_idx = load_root(w, (vx >> 8) + (vy >> 8) * gx + (vz >> 8) * gx * gy);
    if (root_idx == ARC_EMPTY_CHUNK) return 0u;
    uint4 node = load_node(w, root_idx);
    const uint32_t lx = vx & 255u, ly = vy & 255u, lz = vz & 255u;
    for (uint32_t s = 6u; s > shift && !(node.z & ARC_IS_LEAF_FLAG); s -= 2u) {
        const uint32_t b = (((lz >> s) & 3u) << 4) | (((ly >> s) & 3u) << 2) | ((lx >> s) & 3u);
        if (!has_child(node.x, node.y, b)) break;
        node = load_node(w, child_index(node, b));
    }
    return node.w;
}

}  // namespace arc
