/*
 * orc_math.h — canonical arithmetic of the CPU oracle.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA product and is never linked
 * into it.
 *
 * The WGSL reference leaves several float results implementation-defined (SPIR-V allows
 * contraction, 2.5-ulp division, approximate sin/cos/pow). To compare hit voxels, faces and
 * materials bit-for-bit, the oracle fixes one arithmetic and the CUDA kernels implement the same
 * one independently:
 *   - IEEE binary32, round-to-nearest-even, no FMA contraction (-ffp-contract=off);
 *   - correctly rounded division and square root;
 *   - min/max are IEEE minNum/maxNum (fminf/fmaxf);
 *   - float -> u32 conversion saturates (NaN and negatives give 0);
 *   - WGSL sign(0) = 0;
 *   - normalize(v) = v / sqrt((x*x + y*y) + z*z);
 *   - sin/cos: Cody-Waite reduction by pi/2 with a three-term split, then Taylor polynomials
 *     (degree 11 for sin, 12 for cos) in Horner form on [-pi/4, pi/4];
 *   - pow(x, n) for the integer exponents the shaders use: binary exponentiation;
 *   - floor(log2(x)) for x >= 1: the binary exponent of x;
 *   - f32 -> f16 packing: round to nearest even, subnormals kept.
 */
#ifndef ORC_MATH_H
#define ORC_MATH_H

#include <math.h>
#include <stdint.h>
#include <string.h>

static inline uint32_t orc_fbits(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float orc_bitsf(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

static inline float orc_min(float a, float b) { return fminf(a, b); }
static inline float orc_max(float a, float b) { return fmaxf(a, b); }
static inline float orc_clamp(float x, float lo, float hi) { return orc_min(orc_max(x, lo), hi); }
static inline float orc_fract(float x) { return x - floorf(x); }
static inline float orc_sign(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
static inline float orc_mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
static inline float orc_smoothstep(float e0, float e1, float x) {
    float t = orc_clamp((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

/* Saturating float -> u32 (WGSL u32(f)); NaN -> 0. */
static inline uint32_t orc_f2u(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}
static inline uint32_t orc_umin(uint32_t a, uint32_t b) { return a < b ? a : b; }
static inline uint32_t orc_umax(uint32_t a, uint32_t b) { return a > b ? a : b; }
static inline uint32_t orc_uclamp(uint32_t x, uint32_t lo, uint32_t hi) { return orc_umin(orc_umax(x, lo), hi); }

static inline uint32_t orc_popc(uint32_t x) { return (uint32_t)__builtin_popcount(x); }

static inline float orc_dot3(const float a[3], const float b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
static inline float orc_length3(const float v[3]) { return sqrtf(orc_dot3(v, v)); }
static inline void orc_normalize3(const float v[3], float out[3]) {
    float l = sqrtf(orc_dot3(v, v));
    out[0] = v[0] / l;
    out[1] = v[1] / l;
    out[2] = v[2] / l;
}
static inline void orc_cross3(const float a[3], const float b[3], float out[3]) {
    float x = a[1] * b[2] - a[2] * b[1];
    float y = a[2] * b[0] - a[0] * b[2];
    float z = a[0] * b[1] - a[1] * b[0];
    out[0] = x; out[1] = y; out[2] = z;
}

/* sin and cos of x (|x| up to a few thousand) by quadrant reduction and Taylor series. */
static inline void orc_sincos(float x, float* s_out, float* c_out) {
    /* pi/2 = C1 + C2 + C3 with C1 (8 significant bits) and C2 (12 bits) short enough that
     * k*C1 and k*C2 are exact for the |k| < 4096 this library produces. */
    const float two_over_pi = 0.636619772f;
    const float C1 = 1.5703125f;
    const float C2 = 4.837512969970703125e-4f;
    const float C3 = 7.54979013e-8f;
    float kf = rintf(x * two_over_pi);
    int32_t k = (int32_t)kf;
    float r = ((x - kf * C1) - kf * C2) - kf * C3;
    float r2 = r * r;
    /* sin(r) = r (1 - r^2/3! + r^4/5! - r^6/7! + r^8/9! - r^10/11!) */
    float ps = -2.50521084e-8f;
    ps = ps * r2 + 2.75573192e-6f;
    ps = ps * r2 + -1.98412698e-4f;
    ps = ps * r2 + 8.33333333e-3f;
    ps = ps * r2 + -1.66666667e-1f;
    float sr = r + r * (r2 * ps);
    /* cos(r) = 1 - r^2/2! + r^4/4! - r^6/6! + r^8/8! - r^10/10! + r^12/12! */
    float pc = 2.08767570e-9f;
    pc = pc * r2 + -2.75573192e-7f;
    pc = pc * r2 + 2.48015873e-5f;
    pc = pc * r2 + -1.38888889e-3f;
    pc = pc * r2 + 4.16666667e-2f;
    pc = pc * r2 + -0.5f;
    float cr = 1.0f + r2 * pc;
    switch (k & 3) {
        case 0: *s_out = sr; *c_out = cr; break;
        case 1: *s_out = cr; *c_out = -sr; break;
        case 2: *s_out = -sr; *c_out = -cr; break;
        default: *s_out = -cr; *c_out = sr; break;
    }
}

/* x^n for n >= 0 by binary exponentiation (right-to-left). */
static inline float orc_powi(float x, uint32_t n) {
    float result = 1.0f;
    float base = x;
    while (n) {
        if (n & 1u) result = result * base;
        n >>= 1;
        if (n) base = base * base;
    }
    return result;
}

/* 2^x: x = k + r with k = rint(x), |r| <= 1/2; 2^r = e^(r ln 2) by its Taylor series to degree 7
 * in Horner form; k enters through the exponent field. Below -126: 0; above 127: clamped. */
static inline float orc_exp2(float x) {
    if (!(x >= -126.0f)) return 0.0f;
    x = fminf(x, 127.0f);
    float kf = rintf(x);
    float t = (x - kf) * 0.693147181f;
    float p = 1.98412698e-4f;
    p = p * t + 1.38888889e-3f;
    p = p * t + 8.33333333e-3f;
    p = p * t + 4.16666667e-2f;
    p = p * t + 1.66666667e-1f;
    p = p * t + 0.5f;
    p = p * t + 1.0f;
    p = p * t + 1.0f;
    return p * orc_bitsf((uint32_t)((int32_t)kf + 127) << 23);
}

/* log2(x), normal x > 0: x = m 2^e, m in [sqrt(1/2), sqrt(2)); log2 m = (2/ln 2) atanh(s),
 * s = (m-1)/(m+1), atanh(s) = s (1 + s^2/3 + ... + s^10/11). */
static inline float orc_log2(float x) {
    uint32_t b = orc_fbits(x);
    int32_t e = (int32_t)((b >> 23) & 0xFFu) - 127;
    float m = orc_bitsf((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    float s = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float p = 9.09090909e-2f;
    p = p * s2 + 1.11111111e-1f;
    p = p * s2 + 1.42857143e-1f;
    p = p * s2 + 2.0e-1f;
    p = p * s2 + 3.33333333e-1f;
    p = p * s2 + 1.0f;
    return (float)e + (s * p) * 2.88539008f;
}

/* pow(x, y) for the non-integer exponents of the shading code: 2^(y log2 x); x below the normal
 * range (0, negatives) gives 0. */
static inline float orc_pow(float x, float y) {
    if (!(x >= 1.17549435e-38f)) return 0.0f;
    return orc_exp2(y * orc_log2(x));
}

static inline float orc_exp(float x) { return orc_exp2(x * 1.44269504f); }

/* floor(log2(x)) for normal x > 0, as the unbiased binary exponent. */
static inline int32_t orc_floor_log2(float x) {
    uint32_t b = orc_fbits(x);
    return (int32_t)((b >> 23) & 0xFFu) - 127;
}

/* f32 -> f16 bits, round to nearest even. */
static inline uint32_t orc_f32_to_f16(float f) {
    uint32_t x = orc_fbits(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t e = (x >> 23) & 0xFFu;
    uint32_t m = x & 0x7FFFFFu;
    if (e == 0xFFu) return sign | 0x7C00u | (m ? (0x200u | (m >> 13)) : 0u);
    int32_t ee = (int32_t)e - 112;
    if (ee >= 31) return sign | 0x7C00u;
    if (ee <= 0) {
        if (ee < -10) return sign;
        m |= 0x800000u;
        uint32_t shift = (uint32_t)(14 - ee);
        uint32_t r = m >> shift;
        uint32_t rem = m & ((1u << shift) - 1u);
        uint32_t half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (r & 1u))) r++;
        return sign | r;
    }
    uint32_t r = ((uint32_t)ee << 10) | (m >> 13);
    uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (r & 1u))) r++;
    return sign | r;
}

static inline float orc_f16_to_f32(uint32_t h) {
    uint32_t sign = (h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1Fu;
    uint32_t m = h & 0x3FFu;
    if (e == 0) {
        if (m == 0) return orc_bitsf(sign);
        /* subnormal: m * 2^-24 */
        float v = (float)m * 5.96046448e-8f;
        return sign ? -v : v;
    }
    if (e == 31) return orc_bitsf(sign | 0x7F800000u | (m << 13));
    return orc_bitsf(sign | ((e + 112u) << 23) | (m << 13));
}

static inline uint32_t orc_pack2x16float(float a, float b) {
    return orc_f32_to_f16(a) | (orc_f32_to_f16(b) << 16);
}

/* WGSL pack2x16snorm: floor(0.5 + 32767 * clamp(e, -1, 1)) as i16 per half. */
static inline uint32_t orc_pack2x16snorm(float a, float b) {
    int32_t ia = (int32_t)floorf(0.5f + 32767.0f * orc_min(1.0f, orc_max(-1.0f, a)));
    int32_t ib = (int32_t)floorf(0.5f + 32767.0f * orc_min(1.0f, orc_max(-1.0f, b)));
    return ((uint32_t)ia & 0xFFFFu) | (((uint32_t)ib & 0xFFFFu) << 16);
}

static inline void orc_unpack2x16snorm(uint32_t p, float out[2]) {
    int16_t a = (int16_t)(p & 0xFFFFu);
    int16_t b = (int16_t)(p >> 16);
    out[0] = orc_max((float)a / 32767.0f, -1.0f);
    out[1] = orc_max((float)b / 32767.0f, -1.0f);
}

/* WGSL pack4x8unorm: floor(0.5 + 255 * clamp(e, 0, 1)) per byte. */
static inline uint32_t orc_pack4x8unorm(float a, float b, float c, float d) {
    uint32_t ua = (uint32_t)floorf(0.5f + 255.0f * orc_min(1.0f, orc_max(0.0f, a)));
    uint32_t ub = (uint32_t)floorf(0.5f + 255.0f * orc_min(1.0f, orc_max(0.0f, b)));
    uint32_t uc = (uint32_t)floorf(0.5f + 255.0f * orc_min(1.0f, orc_max(0.0f, c)));
    uint32_t ud = (uint32_t)floorf(0.5f + 255.0f * orc_min(1.0f, orc_max(0.0f, d)));
    return ua | (ub << 8) | (uc << 16) | (ud << 24);
}

/* PCG hash: shaders/common/types.wgsl:258-262. */
static inline uint32_t orc_pcg_hash(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

#endif /* ORC_MATH_H */
