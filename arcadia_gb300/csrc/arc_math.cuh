// arc_math.cuh — the canonical float arithmetic of the traversal kernels.
//
// Hit voxels, faces and materials are integer results of float DDA decisions, so the kernels pin
// one arithmetic (the WGSL leaves contraction, division accuracy and sin/cos/pow implementation-
// defined). Translation units that include this header are compiled with --fmad=false
// --prec-div=true --prec-sqrt=true --ftz=false, which makes a*b+c two rounded operations and
// '/' and sqrtf correctly rounded. On top of IEEE binary32 the definition fixes:
//   min/max = IEEE minNum/maxNum (fminf/fmaxf); float -> u32 saturates (NaN -> 0); sign(0) = 0;
//   normalize(v) = v / sqrt((x*x + y*y) + z*z);
//   sin/cos: reduction by pi/2 = C1 + C2 + C3 (C1, C2 short enough that k*C1, k*C2 are exact),
//            then Taylor polynomials of degree 11 (sin) and 12 (cos) in Horner form;
//   pow(x, n) for the shaders' integer exponents: binary exponentiation;
//   floor(log2(x)), x >= 1: the binary exponent;
//   f32 -> f16: round to nearest even (cvt.rn.f16.f32).
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace arc {

struct f3 {
    float x, y, z;
};

__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 mul3s(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot3(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ f3 cross3(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 normalize3(f3 v) {
    float l = __fsqrt_rn(dot3(v, v));
    return f3{__fdiv_rn(v.x, l), __fdiv_rn(v.y, l), __fdiv_rn(v.z, l)};
}
__device__ __forceinline__ float length3(f3 v) { return __fsqrt_rn(dot3(v, v)); }

__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float fractf(float x) { return x - floorf(x); }
__device__ __forceinline__ float signf(float x) { return x > 0.0f ? 1.0f : (x < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ float smoothstepf(float e0, float e1, float x) {
    float t = clampf(__fdiv_rn(x - e0, e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
__device__ __forceinline__ uint32_t f2u(float f) { return __float2uint_rz(f); }
__device__ __forceinline__ uint32_t uclamp(uint32_t x, uint32_t lo, uint32_t hi) { return umin(umax(x, lo), hi); }

__device__ __forceinline__ uint32_t pcg_hash(uint32_t input) {
    uint32_t state = input * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

__device__ __forceinline__ void sincos_canon(float x, float* s, float* c) {
    const float kTwoOverPi = 0.636619772f;
    const float kC1 = 1.5703125f;
    const float kC2 = 4.837512969970703125e-4f;
    const float kC3 = 7.54979013e-8f;
    float kf = rintf(x * kTwoOverPi);
    int k = (int)kf;
    float r = ((x - kf * kC1) - kf * kC2) - kf * kC3;
    float r2 = r * r;
    float ps = -2.50521084e-8f;
    ps = ps * r2 + 2.75573192e-6f;
    ps = ps * r2 + -1.98412698e-4f;
    ps = ps * r2 + 8.33333333e-3f;
    ps = ps * r2 + -1.66666667e-1f;
    float sr = r + r * (r2 * ps);
    float pc = 2.08767570e-9f;
    pc = pc * r2 + -2.75573192e-7f;
    pc = pc * r2 + 2.48015873e-5f;
    pc = pc * r2 + -1.38888889e-3f;
    pc = pc * r2 + 4.16666667e-2f;
    pc = pc * r2 + -0.5f;
    float cr = 1.0f + r2 * pc;
    switch (k & 3) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

__device__ __forceinline__ float powi(float x, uint32_t n) {
    float result = 1.0f, base = x;
    while (n) {
        if (n & 1u) result = result * base;
        n >>= 1;
        if (n) base = base * base;
    }
    return result;
}

// 2^x: x = k + r with k = rint(x), |r| <= 1/2; 2^r = e^(r ln 2) from its Taylor series to degree 7
// (remainder below 6e-9 relative) in Horner form; k enters through the exponent field. Arguments
// below -126 give 0, above 127 are clamped to 127.
__device__ __forceinline__ float exp2_canon(float x) {
    if (!(x >= -126.0f)) return 0.0f;
    x = fminf(x, 127.0f);
    const float kf = rintf(x);
    const float t = (x - kf) * 0.693147181f;
    float p = 1.98412698e-4f;
    p = p * t + 1.38888889e-3f;
    p = p * t + 8.33333333e-3f;
    p = p * t + 4.16666667e-2f;
    p = p * t + 1.66666667e-1f;
    p = p * t + 0.5f;
    p = p * t + 1.0f;
    p = p * t + 1.0f;
    return p * __uint_as_float((uint32_t)((int)kf + 127) << 23);
}

// log2(x) for normal x > 0: x = m 2^e with m in [sqrt(1/2), sqrt(2)); log2 m = (2 / ln 2) atanh(s)
// with s = (m - 1) / (m + 1), |s| <= 0.1716, and atanh(s) = s (1 + s^2/3 + s^4/5 + ... + s^10/11).
__device__ __forceinline__ float log2_canon(float x) {
    const uint32_t b = __float_as_uint(x);
    int e = (int)((b >> 23) & 0xFFu) - 127;
    float m = __uint_as_float((b & 0x7FFFFFu) | 0x3F800000u);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e += 1;
    }
    const float s = __fdiv_rn(m - 1.0f, m + 1.0f);
    const float s2 = s * s;
    float p = 9.09090909e-2f;
    p = p * s2 + 1.11111111e-1f;
    p = p * s2 + 1.42857143e-1f;
    p = p * s2 + 2.0e-1f;
    p = p * s2 + 3.33333333e-1f;
    p = p * s2 + 1.0f;
    return (float)e + (s * p) * 2.88539008f;
}

// pow(x, y) = 2^(y log2 x) for the non-integer exponents of the shading code; x below the normal
// range (including 0 and negatives) gives 0.
__device__ __forceinline__ float pow_canon(float x, float y) {
    if (!(x >= 1.17549435e-38f)) return 0.0f;
    return exp2_canon(y * log2_canon(x));
}

__device__ __forceinline__ float exp_canon(float x) { return exp2_canon(x * 1.44269504f); }

__device__ __forceinline__ int floor_log2(float x) { return (int)((__float_as_uint(x) >> 23) & 0xFFu) - 127; }

__device__ __forceinline__ uint32_t f16_bits(float x) { return (uint32_t)__half_as_ushort(__float2half_rn(x)); }
__device__ __forceinline__ float f16_value(uint32_t h) { return __half2float(__ushort_as_half((unsigned short)(h & 0xFFFFu))); }
__device__ __forceinline__ uint32_t pack2x16float(float a, float b) { return f16_bits(a) | (f16_bits(b) << 16); }
__device__ __forceinline__ uint32_t pack2x16snorm(float a, float b) {
    int ia = (int)floorf(0.5f + 32767.0f * fminf(1.0f, fmaxf(-1.0f, a)));
    int ib = (int)floorf(0.5f + 32767.0f * fminf(1.0f, fmaxf(-1.0f, b)));
    return ((uint32_t)ia & 0xFFFFu) | (((uint32_t)ib & 0xFFFFu) << 16);
}
__device__ __forceinline__ void unpack2x16snorm(uint32_t p, float* a, float* b) {
    *a = fmaxf(__fdiv_rn((float)(int16_t)(p & 0xFFFFu), 32767.0f), -1.0f);
    *b = fmaxf(__fdiv_rn((float)(int16_t)(p >> 16), 32767.0f), -1.0f);
}
__device__ __forceinline__ uint32_t unorm8(float v) { return (uint32_t)floorf(0.5f + 255.0f * fminf(1.0f, fmaxf(0.0f, v))); }
__device__ __forceinline__ uint32_t pack4x8unorm(float a, float b, float c, float d) {
    return unorm8(a) | (unorm8(b) << 8) | (unorm8(c) << 16) | (unorm8(d) << 24);
}

// Octahedral normal encode/decode (shaders/common/types.wgsl:108-130).
__device__ __forceinline__ void oct_encode(f3 n, float* px, float* py) {
    float l1 = (fabsf(n.x) + fabsf(n.y)) + fabsf(n.z);
    float s = __fdiv_rn(1.0f, fmaxf(l1, 1e-6f));
    float x = n.x * s, y = n.y * s;
    if (n.z < 0.0f) {
        float wx = (1.0f - fabsf(y)) * (x >= 0.0f ? 1.0f : -1.0f);
        float wy = (1.0f - fabsf(x)) * (y >= 0.0f ? 1.0f : -1.0f);
        x = wx;
        y = wy;
    }
    *px = x;
    *py = y;
}
__device__ __forceinline__ f3 oct_decode(float px, float py) {
    f3 n{px, py, (1.0f - fabsf(px)) - fabsf(py)};
    if (n.z < 0.0f) {
        float wx = (1.0f - fabsf(py)) * (px >= 0.0f ? 1.0f : -1.0f);
        float wy = (1.0f - fabsf(px)) * (py >= 0.0f ? 1.0f : -1.0f);
        n.x = wx;
        n.y = wy;
    }
    return normalize3(n);
}

// Face id in sharc_norm_id order (+X, -X, +Y, -Y, +Z, -Z; shaders/common/sharc.wgsl:48-57).
__device__ __forceinline__ uint32_t face_id(f3 n) {
    float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
    if (ax > ay && ax > az) return n.x > 0.0f ? 0u : 1u;
    if (ay > az) return n.y > 0.0f ? 2u : 3u;
    return n.z > 0.0f ? 4u : 5u;
}

// Orthonormal frame about a unit normal (make_basis, types.wgsl:531-537; sharc_tangent_frame).
__device__ __forceinline__ void make_basis(f3 n, f3* t, f3* b) {
    f3 up = fabsf(n.z) < 0.999f ? f3{0.0f, 0.0f, 1.0f} : f3{1.0f, 0.0f, 0.0f};
    *t = normalize3(cross3(up, n));
    *b = cross3(n, *t);
}

// sample_cosine_hemisphere (types.wgsl:540-545).
__device__ __forceinline__ f3 cosine_sample(float u1, float u2, f3 n, f3 t, f3 b) {
    float r = __fsqrt_rn(u1);
    float phi = 6.2831853f * u2;
    float z = __fsqrt_rn(fmaxf(0.0f, 1.0f - u1));
    float s, c;
    sincos_canon(phi, &s, &c);
    float rc = r * c, rs = r * s;
    return f3{(t.x * rc + b.x * rs) + n.x * z, (t.y * rc + b.y * rs) + n.y * z, (t.z * rc + b.z * rs) + n.z * z};
}

// interleaved_gradient_noise (types.wgsl:483-497).
__device__ __forceinline__ void gradient_noise(float px, float py, uint32_t frame, float* u1, float* u2) {
    float f = (float)frame;
    uint32_t ux = f2u(px), uy = f2u(py);
    float i1 = fractf(52.9829189f * fractf(0.06711056f * px + 0.00583715f * py));
    float i2 = fractf(52.9829189f * fractf((0.00583715f * px - 0.06711056f * py) + 0.5f));
    uint32_t h1 = pcg_hash(ux * 1973u + uy * 9277u + frame * 26699u);
    uint32_t h2 = pcg_hash(h1 ^ 0x9E3779B9u);
    *u1 = fractf((i1 + f * 0.754877666f) + __fdiv_rn((float)(h1 & 0xFFFFu), 65536.0f));
    *u2 = fractf((i2 + f * 0.569840291f) + __fdiv_rn((float)(h2 & 0xFFFFu), 65536.0f));
}

}  // namespace arc
