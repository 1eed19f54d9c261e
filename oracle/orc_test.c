/*
 * orc_test.c — small hooks that expose the oracle's canonical-arithmetic helpers to the tests.
 * TEST INFRASTRUCTURE ONLY (see orc.h).
 */
#include "orc.h"
#include <stdlib.h>
#include "orc_math.h"

void orc_test_sincos(const float* x, uint32_t n, float* s, float* c) {
    for (uint32_t i = 0; i < n; ++i) orc_sincos(x[i], &s[i], &c[i]);
}

void orc_test_f16(const float* x, uint32_t n, uint16_t* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = (uint16_t)orc_f32_to_f16(x[i]);
}

void orc_test_powi(const float* x, uint32_t n, uint32_t e, float* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = orc_powi(x[i], e);
}

void orc_test_exp2_log2(const float* x, uint32_t n, float* e2, float* l2) {
    for (uint32_t i = 0; i < n; ++i) {
        e2[i] = orc_exp2(x[i]);
        l2[i] = x[i] > 0.0f ? orc_log2(x[i]) : 0.0f;
    }
}

void orc_test_pow(const float* x, uint32_t n, float y, float* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = orc_pow(x[i], y);
}

/* Dense (z, y, x) material volume of one chunk of a synthetic scene, by per-voxel evaluation. */
void orc_test_scene_volume(const orc_scene_params* p, uint32_t cx, uint32_t cy, uint32_t cz, uint8_t* vol) {
    uint32_t wx = p->grid[0] * 256u, wz = p->grid[2] * 256u;
    float* hm = (float*)malloc(sizeof(float) * (size_t)wx * wz);
    orc_scene_heightmap(p, hm);
#pragma omp parallel for schedule(dynamic, 4)
    for (int z = 0; z < 256; ++z)
        for (uint32_t y = 0; y < 256; ++y)
            for (uint32_t x = 0; x < 256; ++x)
                vol[((size_t)z * 256u + y) * 256u + x] =
                    (uint8_t)orc_scene_voxel(p, hm, cx * 256u + x, cy * 256u + y, cz * 256u + (uint32_t)z);
    free(hm);
}

/* WGSL pack4x8unorm / pack2x16snorm as the oracle's G-buffer writer applies them (orc_math.h). */
void orc_test_pack4x8unorm(const float* x, uint32_t n, uint32_t* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = orc_pack4x8unorm(x[4 * i], x[4 * i + 1], x[4 * i + 2], x[4 * i + 3]);
}

void orc_test_pack2x16snorm(const float* x, uint32_t n, uint32_t* out) {
    for (uint32_t i = 0; i < n; ++i) out[i] = orc_pack2x16snorm(x[2 * i], x[2 * i + 1]);
}

