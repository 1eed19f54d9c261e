// arc_rigid.cuh — ray march through rigid voxel bodies: trace_single_rigid_body and
// trace_rigid_bodies (shaders/common/traversal64.wgsl:1006-1244).
//
// A body is a 64-tree (one 256^3 chunk tree in the node pool) under a rigid transform. The ray is
// rejected against the body's bounding sphere, moved into body-local voxel space, clipped to the
// local box and marched for at most 64 DDA steps with the reference's per-level node cache; the hit
// comes back to world space through local_to_world (and prev_local_to_world for the motion vector).
// trace_rigid_bodies keeps the nearest hit over min(camera count, table size, 32) bodies, shrinking
// the search distance to each hit found. Canonical arithmetic (arc_math.cuh); matrix-vector
// products sum the columns in order.
#pragma once

#include "arc_traverse.cuh"

namespace arc {

struct RigidHit {
    bool hit;
    float t_voxels;
    f3 pos, prev_pos, normal;
    uint32_t mat, hash;
    float ao;
    uint32_t vx, vy, vz, shift, body;
};

// mat4x4 (column-major) * vec4(v, wc)
__device__ __forceinline__ f3 xform4(const float* M, f3 v, float wc) {
    return f3{((M[0] * v.x + M[4] * v.y) + M[8] * v.z) + M[12] * wc, ((M[1] * v.x + M[5] * v.y) + M[9] * v.z) + M[13] * wc,
              ((M[2] * v.x + M[6] * v.y) + M[10] * v.z) + M[14] * wc};
}

__device__ __forceinline__ uint32_t rigid_count(const World& w, const arc_camera_uniforms& cam) {
    return umin(umin((cam.point_light_count[1] >> 16) & 0xFFFFu, ARC_MAX_RIGID_BODIES), w.n_bodies);
}

// step_dda_box (traversal64.wgsl:152-179) in body-local voxel space
__device__ __forceinline__ void rigid_step(f3 vo, f3 d, f3 inv, f3 noi, bool px, bool py, bool pz, uint32_t bx, uint32_t by,
                                           uint32_t bz, uint32_t span, float& t, uint32_t& vx, uint32_t& vy, uint32_t& vz) {
    const uint32_t ex = px ? bx + span : bx, ey = py ? by + span : by, ez = pz ? bz + span : bz;
    const float tx = (float)ex * inv.x + noi.x, ty = (float)ey * inv.y + noi.y, tz = (float)ez * inv.z + noi.z;
    const float t_exit = fminf(fminf(tx, ty), tz);
    const float nt = fmaxf(t, t_exit);
    const bool is_x = tx <= ty && tx <= tz;
    const bool is_y = !is_x && ty <= tz;
    const bool is_z = !is_x && !is_y;
    // max(x, 0) before the conversion is implied: cvt.rzi.u32.f32 clamps to [0, 2^32 - 1] and turns NaN into 0
    const uint32_t ix = uclamp(f2u(vo.x + d.x * nt), bx, bx + span - 1u);
    const uint32_t iy = uclamp(f2u(vo.y + d.y * nt), by, by + span - 1u);
    const uint32_t iz = uclamp(f2u(vo.z + d.z * nt), bz, bz + span - 1u);
    t = nt;
    vx = is_x ? (px ? ex : ex - 1u) : ix;
    vy = is_y ? (py ? ey : ey - 1u) : iy;
    vz = is_z ? (pz ? ez : ez - 1u) : iz;
}

// trace_single_rigid_body (traversal64.wgsl:1006-1222); res.hit stays false on a miss.
static __device__ __noinline__ void trace_single_rigid(const World& w, uint32_t body, f3 o, f3 dir, float max_dist_m,
                                                       RigidHit& res) {
    res.hit = false;
    const arc_rigid_body& rb = w.bodies[body];
    const uint32_t root_idx = __float_as_uint(rb.local_bounds_and_root[3]);
    if (root_idx == ARC_EMPTY_CHUNK) return;
    const f3 oc{o.x - rb.world_sphere[0], o.y - rb.world_sphere[1], o.z - rb.world_sphere[2]};
    const float bp = dot3(oc, dir);
    const float cd = dot3(oc, oc) - rb.world_sphere[3] * rb.world_sphere[3];
    if (cd > 0.0f && bp > 0.0f) return;
    const float disc = bp * bp - cd;
    if (disc < 0.0f) return;
    if (fmaxf(-bp - __fsqrt_rn(disc), 0.0f) >= max_dist_m) return;
    const f3 ld = xform4(rb.world_to_local, dir, 0.0f);
    const f3 vo = mul3s(xform4(rb.world_to_local, o, 1.0f), ARC_VOXELS_PER_METER);
    const f3 lmax{rb.local_bounds_and_root[0] * ARC_VOXELS_PER_METER, rb.local_bounds_and_root[1] * ARC_VOXELS_PER_METER,
                  rb.local_bounds_and_root[2] * ARC_VOXELS_PER_METER};
    const float max_t_v = max_dist_m * ARC_VOXELS_PER_METER;
    const f3 inv{__fdiv_rn(1.0f, safe_component(ld.x)), __fdiv_rn(1.0f, safe_component(ld.y)), __fdiv_rn(1.0f, safe_component(ld.z))};
    // intersect_aabb(vo, inv, 0, lmax) (traversal64.wgsl:134-142)
    const float a0 = fmaxf(fmaxf(((inv.x > 0.0f ? 0.0f : lmax.x) - vo.x) * inv.x, ((inv.y > 0.0f ? 0.0f : lmax.y) - vo.y) * inv.y),
                           ((inv.z > 0.0f ? 0.0f : lmax.z) - vo.z) * inv.z);
    const float a1 = fminf(fminf(((inv.x > 0.0f ? lmax.x : 0.0f) - vo.x) * inv.x, ((inv.y > 0.0f ? lmax.y : 0.0f) - vo.y) * inv.y),
                           ((inv.z > 0.0f ? lmax.z : 0.0f) - vo.z) * inv.z);
    const float t_enter = fmaxf(a0, 0.0f);
    if (a1 < t_enter || t_enter >= max_t_v) return;
    float t = t_enter;
    const float t_limit = fminf(a1, max_t_v);
    const bool px = inv.x >= 0.0f, py = inv.y >= 0.0f, pz = inv.z >= 0.0f;
    const f3 noi{-vo.x * inv.x, -vo.y * inv.y, -vo.z * inv.z};
    const uint32_t mx = f2u(lmax.x + 0.5f), my = f2u(lmax.y + 0.5f), mz = f2u(lmax.z + 0.5f);
    uint32_t vx = f2u(clampf(vo.x + ld.x * (t + 1e-4f), 0.0f, lmax.x - 1e-3f));
    uint32_t vy = f2u(clampf(vo.y + ld.y * (t + 1e-4f), 0.0f, lmax.y - 1e-3f));
    uint32_t vz = f2u(clampf(vo.z + ld.z * (t + 1e-4f), 0.0f, lmax.z - 1e-3f));
    uint32_t qx = 0xFFFFFFFFu, qy = 0xFFFFFFFFu, qz = 0xFFFFFFFFu;
    uint32_t cached_shift = 6u;
    uint4 c1 = make_uint4(0u, 0u, 0u, 0u), c2 = c1, c3 = c1;
    for (uint32_t step = 0; step < 64u; ++step) {
        if (t >= t_limit) break;
        if (vx >= mx || vy >= my || vz >= mz) break;
        const uint32_t diff = (qx ^ vx) | (qy ^ vy) | (qz ^ vz);
        qx = vx;
        qy = vy;
        qz = vz;
        uint4 node;
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
            node = load_node(w, root_idx);
            shift = 6u;
        }
        cached_shift = shift;
        const uint32_t lx = vx & 255u, ly = vy & 255u, lz = vz & 255u;
        for (;;) {
            const uint32_t cx = (lx >> shift) & 3u, cy = (ly >> shift) & 3u, cz = (lz >> shift) & 3u;
            const uint32_t b = (cz << 4) | (cy << 2) | cx;
            const uint32_t span = 1u << shift;
            const uint32_t bx = vx & ~(span - 1u), by = vy & ~(span - 1u), bz = vz & ~(span - 1u);
            if (!has_child(node.x, node.y, b)) {
                rigid_step(vo, ld, inv, noi, px, py, pz, bx, by, bz, span, t, vx, vy, vz);
                break;
            }
            if (node.z & ARC_IS_LEAF_FLAG) {
                uint32_t mat = (node.w >> 24) & 0xFFu;
                if (!(node.z & ARC_IS_UNIFORM_FLAG)) mat = load_brick_mat(w, node.z & ARC_PTR_INDEX_MASK, b);
                if (mat != ARC_MAT_AIR) {
                    const float tx = (float)(px ? bx : bx + span) * inv.x + noi.x;
                    const float ty = (float)(py ? by : by + span) * inv.y + noi.y;
                    const float tz = (float)(pz ? bz : bz + span) * inv.z + noi.z;
                    const float et = fmaxf(fmaxf(fmaxf(tx, ty), tz), 0.0f);
                    const f3 hpv = add3(vo, mul3s(ld, et));
                    const f3 hpm = mul3s(hpv, ARC_VOXEL_SIZE);
                    f3 ln{0.0f, 0.0f, 0.0f};
                    if (tx >= ty && tx >= tz) ln.x = -signf(ld.x);
                    else if (ty >= tz) ln.y = -signf(ld.y);
                    else ln.z = -signf(ld.z);
                    res.hit = true;
                    res.t_voxels = et;
                    res.pos = xform4(rb.local_to_world, hpm, 1.0f);
                    res.prev_pos = xform4(rb.prev_local_to_world, hpm, 1.0f);
                    res.normal = normalize3(xform4(rb.local_to_world, ln, 0.0f));
                    res.mat = mat;
                    res.hash = pcg_hash((vx * 73856093u) ^ (vy * 19349663u) ^ (vz * 83492791u));
                    res.ao = shift == 0u ? leaf_ao(node.x, node.y, cx, cy, cz, ln, hpv) : 1.0f;
                    res.vx = vx;
                    res.vy = vy;
                    res.vz = vz;
                    res.shift = shift;
                    res.body = body;
                    return;
                }
                rigid_step(vo, ld, inv, noi, px, py, pz, bx, by, bz, span, t, vx, vy, vz);
                break;
            }
            node = load_node(w, child_index(node, b));
            shift -= 2u;
            cached_shift = shift;
            if (shift == 4u) c1 = node;
            else if (shift == 2u) c2 = node;
            else if (shift == 0u) c3 = node;
        }
    }
}

// trace_rigid_bodies (traversal64.wgsl:1224-1244): nearest body hit within max_dist_m.
__device__ __forceinline__ RigidHit trace_rigid_bodies(const World& w, const arc_camera_uniforms& cam, f3 o, f3 dir,
                                                       float max_dist_m) {
    RigidHit best;
    best.hit = false;
    best.t_voxels = max_dist_m * ARC_VOXELS_PER_METER;
    const uint32_t n = rigid_count(w, cam);
    float cur = max_dist_m;
    for (uint32_t i = 0; i < n; ++i) {
        RigidHit c;
        trace_single_rigid(w, i, o, dir, cur, c);
        if (c.hit && c.t_voxels < best.t_voxels) {
            best = c;
            cur = c.t_voxels * ARC_VOXEL_SIZE;
        }
    }
    return best;
}

}  // namespace arc
