// arc_sharc.cuh — read side of the SHARC cache (key, lookup, query) and the sky radiance, shared
// by the SHARC kernels and the ReSTIR GI temporal pass. Canonical arithmetic (arc_math.cuh).
#pragma once

#include "arc_traverse.cuh"

namespace arc {

// sharc_make_key (shaders/common/sharc.wgsl:69-93).
__device__ __forceinline__ void sharc_key(f3 pos, f3 n, f3 cam, float jx, float jy, uint32_t* bucket, uint32_t* key) {
    const float d = length3(sub3(pos, cam));
    const int fl = floor_log2(fmaxf(d, 4.0f) * 0.25f);
    const uint32_t lod = fl < 0 ? 0u : (fl > 3 ? 3u : (uint32_t)fl);
    const float s = 0.25f * (float)(1u << lod);
    f3 a = sub3(pos, mul3s(n, 0.02f));
    if (jx != 0.0f || jy != 0.0f) {
        f3 t, b;
        make_basis(n, &t, &b);
        const float k = 0.42f * s;
        a.x += (t.x * jx + b.x * jy) * k;
        a.y += (t.y * jx + b.y * jy) * k;
        a.z += (t.z * jx + b.z * jy) * k;
    }
    const uint32_t cx = (uint32_t)((int)floorf(__fdiv_rn(a.x, s)) + 16384);
    const uint32_t cy = (uint32_t)((int)floorf(__fdiv_rn(a.y, s)) + 16384);
    const uint32_t cz = (uint32_t)((int)floorf(__fdiv_rn(a.z, s)) + 16384);
    const uint32_t nid = face_id(n);
    const uint32_t bk = pcg_hash((cx * 73856093u) ^ (cy * 19349663u) ^ (cz * 83492791u) ^ (nid * 2654435761u) ^ (lod * 38069u)) &
                        (ARC_SHARC_BUCKETS - 1u);
    *bucket = bk;
    *key = pcg_hash(bk ^ (cx * 1013904223u) ^ (cy * 1664525u) ^ (cz * 2891336453u) ^ (nid << 20) ^ (lod << 24)) |
           ARC_SHARC_KEY_VALID_BIT;
}

__device__ __forceinline__ f3 slot_radiance(uint4 s) {
    return f3{f16_value(s.y & 0xFFFFu), f16_value(s.y >> 16), f16_value(s.z & 0xFFFFu)};
}

// sharc_lookup / query_sharc (shaders/common/sharc_query.wgsl:8-29); w = 1 on hit.
__device__ __forceinline__ float4 sharc_lookup(const uint4* res, uint32_t bucket, uint32_t key) {
    const uint32_t base = bucket * ARC_SHARC_WAYS;
#pragma unroll
    for (uint32_t i = 0; i < ARC_SHARC_WAYS; ++i) {
        const uint4 s = res[base + i];
        if (s.x == key) {
            const f3 r = slot_radiance(s);
            return make_float4(r.x, r.y, r.z, 1.0f);
        }
    }
    return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

__device__ __forceinline__ float4 sharc_query(const uint4* res, f3 pos, f3 n, f3 cam, float jx, float jy) {
    uint32_t b, k;
    if (jx != 0.0f || jy != 0.0f) {
        sharc_key(pos, n, cam, jx, jy, &b, &k);
        const float4 r = sharc_lookup(res, b, k);
        if (r.w > 0.5f) return r;
    }
    sharc_key(pos, n, cam, 0.0f, 0.0f, &b, &k);
    return sharc_lookup(res, b, k);
}

// eval_sky_radiance (shaders/common/types.wgsl:500-523).
__device__ __forceinline__ f3 sky_radiance(f3 dir, f3 sun) {
    const float day_t = clampf(__fdiv_rn(sun.y + 0.05f, 0.30f), 0.0f, 1.0f);
    const float tw_t = clampf(1.0f - __fdiv_rn(fabsf(sun.y - 0.02f), 0.22f), 0.0f, 1.0f);
    const float horizon = powi(1.0f - clampf(dir.y, 0.0f, 1.0f), 3u);
    const f3 sz{mixf(0.0015f, 0.08f, day_t), mixf(0.0025f, 0.22f, day_t), mixf(0.0055f, 0.55f, day_t)};
    f3 sh{mixf(0.0035f, 0.38f, day_t), mixf(0.0065f, 0.50f, day_t), mixf(0.0120f, 0.68f, day_t)};
    const float tw = tw_t * 0.75f;
    sh = f3{mixf(sh.x, 0.65f, tw), mixf(sh.y, 0.25f, tw), mixf(sh.z, 0.10f, tw)};
    f3 sky{mixf(sz.x, sh.x, horizon), mixf(sz.y, sh.y, horizon), mixf(sz.z, sh.z, horizon)};
    if (sun.y > -0.12f) {
        const float p = powi(fmaxf(dot3(dir, sun), 0.0f), 14u);
        const float m = fmaxf(day_t, tw_t);
        sky.x += ((0.85f * p) * 0.35f) * m;
        sky.y += ((0.52f * p) * 0.35f) * m;
        sky.z += ((0.24f * p) * 0.35f) * m;
    }
    return sky;
}

}  // namespace arc
