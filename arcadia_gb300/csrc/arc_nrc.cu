// arc_nrc.cu — neural radiance cache: fused tensor-core inference and training (sm_103a).
//
// No reference counterpart: the NRC stands in for SHARC's hashed lookup (query_sharc,
// shaders/common/sharc_query.wgsl:21-29) at secondary hits.
//
// Network: 9 inputs (position in [0,1]^3, normal, view direction) -> sin/cos(2^k pi v), k = 0..11
// (216 features, index = input*24 + 2k + {0 sin, 1 cos}) -> 5 x 64 ReLU -> 3 linear outputs, no
// biases. FP32 master weights (compact, W[out][in] per layer) with FP16 copies in padded layouts.
//
// The default path runs on the fifth-generation tensor cores: infer_tc_kernel and train_tc_kernel
// issue tcgen05.mma from one thread into TMEM accumulators, with operands in shared memory (below,
// "tcgen05 inference" / "tcgen05 training"). The warp-level mma.sync.m16n8k16 kernels (infer_kernel,
// train_kernel) stay selectable (arc_nrc_set_infer_path / arc_nrc_set_train_path) as the comparison
// point. In them activations move between layers in registers: the m16n8k16 accumulator fragment of
// two adjacent 8-column tiles is exactly the A fragment of the next layer's 16-wide k step, so ReLU +
// FP16 packing is all the conversion a layer needs.
//
// mma.sync training (one fused kernel per batch): a CTA of 4 warps takes 64 samples at a time; each warp runs
// the forward pass for 16 samples and stores the transposed activations in shared memory; the backward
// pass runs layer by layer (dZ in registers, dZ^T in a double-buffered shared tile), and after each
// layer all warps compute that layer's weight-gradient tiles dW = dZ^T A over the 64 samples on the
// tensor cores and add them to the FP32 gradient with red.global.add.v2.f32. A loss scale of 128 keeps
// the FP16 gradients in range; Adam divides it out.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <utility>
#include <vector>

#include "arc_ctx.h"
#include "arc_tc.cuh"

namespace nrc {

constexpr int kIn = 9, kEnc = 216, kEncPad = 224, kW = 64, kOut = 3;
constexpr int kParams = kEnc * kW + 4 * kW * kW + kOut * kW;  // 30400
// compact FP32 master offsets per layer
__host__ __device__ constexpr int off(int l) { return l == 0 ? 0 : (l == 6 ? kParams : kEnc * kW + (l - 1) * kW * kW); }
// FP16 forward layout W[out][in_pad]
constexpr int kS1 = 232, kS = 72;
constexpr int kF1 = 0, kF2 = 64 * kS1;  // layer 2..5 at kF2 + (l-2)*64*kS
constexpr int kF6 = kF2 + 4 * 64 * kS;
constexpr int kFwdHalves = kF6 + 8 * kS;  // 33856
// FP16 transposed layout WT[in][out_pad] (layers 2..6)
constexpr int kST6 = 24;
constexpr int kT2 = kFwdHalves;
constexpr int kT6 = kT2 + 4 * 64 * kS;
constexpr int kAllHalves = kT6 + 64 * kST6;  // 53824
constexpr float kLossScale = 128.0f;
// training activations (per CTA of 64 samples; sample stride kSS)
constexpr int kSS = 72;
constexpr int kXT = 0;                       // [224][kSS]
constexpr int kHT = kXT + kEncPad * kSS;     // 5 x [64][kSS]
constexpr int kDZ = kHT + 5 * 64 * kSS;      // 2 x [64][kSS]
constexpr int kActHalves = kDZ + 2 * 64 * kSS;

__host__ __device__ constexpr int fwd_off(int l) { return l == 1 ? kF1 : (l <= 5 ? kF2 + (l - 2) * 64 * kS : kF6); }
__host__ __device__ constexpr int fwd_stride(int l) { return l == 1 ? kS1 : kS; }

// FP16 tensor-core operand layout (tcgen05 kernels): per layer an N_l x K_l K-major block in the
// canonical no-swizzle layout, element (n, k) at u_index(l, n, k) (halves): 8 x 8 core matrices of
// 128 B, K-adjacent core matrices 128 B apart, 8-row groups K_l/8 core matrices apart. Layer 1 is
// 64 x 224 (features 216..223 zero), layers 2..5 64 x 64, layer 6 16 x 64 (outputs 3..15 zero).
constexpr int kU2 = 64 * kEncPad;
constexpr int kU6 = kU2 + 4 * 64 * 64;
constexpr int kUHalves = kU6 + 16 * 64;  // 31744 halves = 63,488 B
__host__ __device__ constexpr int u_off(int l) { return l == 1 ? 0 : (l <= 5 ? kU2 + (l - 2) * 4096 : kU6); }
__host__ __device__ constexpr int u_k(int l) { return l == 1 ? kEncPad : kW; }
__host__ __device__ constexpr int u_index(int l, int n, int k) {
    return u_off(l) + (n >> 3) * (u_k(l) >> 3) * 64 + (k >> 3) * 64 + (n & 7) * 8 + (k & 7);
}

__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ uint32_t pack_h2(float lo, float hi) {
    __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
// ReLU of an FP16-rounded pair, one packed max after the conversion: the same values as
// pack_h2(fmaxf(lo, 0), fmaxf(hi, 0)) (rounding keeps the sign), except that an input rounding to -0
// may stay -0, which no product or mask downstream tells from +0.
__device__ __forceinline__ uint32_t relu_pack_h2(float lo, float hi) {
    __half2 h = __hmax2(__floats2half2_rn(lo, hi), __float2half2_rn(0.0f));
    return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t lds32(const __half* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ void red_add2(float* p, float a, float b) {
    asm volatile("red.global.add.v2.f32 [%0], {%1, %2};\n" ::"l"(p), "f"(a), "f"(b) : "memory");
}

// Encoded features (f, f+1) = (sin, cos)(2^k pi v) of the even feature index f.
__device__ __forceinline__ uint32_t enc_pair(const float (&v)[kIn], int f) {
    if (f >= kEnc) return 0u;
    const int i = f / 24, k = (f % 24) >> 1;
    float x = v[0];
#pragma unroll
    for (int q = 1; q < kIn; ++q) x = (i == q) ? v[q] : x;  // register select, no local-memory indexing
    float s, c;
    sincospif(ldexpf(x, k), &s, &c);
    return pack_h2(s, c);
}

// Layer with K = 64 from A fragments held in registers: acc[nt] += A * W_l^T (8 output tiles).
__device__ __forceinline__ void layer64(const __half* sw, int l, const uint32_t (&a)[4][4], float (&acc)[8][4], int gid,
                                        int tig) {
    const __half* W = sw + fwd_off(l);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
        const __half* row = W + (nt * 8 + gid) * kS + 2 * tig;
#pragma unroll
        for (int j = 0; j < 4; ++j) mma16816(acc[nt], a[j], lds32(row + 16 * j), lds32(row + 16 * j + 8));
    }
}

__device__ __forceinline__ void relu_to_a(const float (&acc)[8][4], uint32_t (&a)[4][4]) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        a[j][0] = pack_h2(fmaxf(acc[2 * j][0], 0.0f), fmaxf(acc[2 * j][1], 0.0f));
        a[j][1] = pack_h2(fmaxf(acc[2 * j][2], 0.0f), fmaxf(acc[2 * j][3], 0.0f));
        a[j][2] = pack_h2(fmaxf(acc[2 * j + 1][0], 0.0f), fmaxf(acc[2 * j + 1][1], 0.0f));
        a[j][3] = pack_h2(fmaxf(acc[2 * j + 1][2], 0.0f), fmaxf(acc[2 * j + 1][3], 0.0f));
    }
}

__device__ __forceinline__ void load_inputs(const float* __restrict__ in, uint32_t n, uint32_t row, float (&v)[kIn]) {
    // training batch rows (row < n)
#pragma unroll
    for (int i = 0; i < kIn; ++i) v[i] = row < n ? __ldg(&in[(size_t)row * kIn + i]) : 0.0f;
}

// Forward of one warp's 16 rows up to the output tile (acc6), optionally storing transposed activations.
template <bool kStore>
__device__ __forceinline__ void forward16(const __half* sw, __half* act, const float (&v0)[kIn], const float (&v1)[kIn],
                                          int gid, int tig, int s0, float (&acc6)[4]) {
    float acc[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.0f;
    for (int j = 0; j < kEncPad / 16; ++j) {
        uint32_t a[4];
        const int f = 16 * j + 2 * tig;
        a[0] = enc_pair(v0, f);
        a[1] = enc_pair(v1, f);
        a[2] = enc_pair(v0, f + 8);
        a[3] = enc_pair(v1, f + 8);
        if (kStore) {
            __half* x = act + kXT;
            const __half2 p0 = *reinterpret_cast<__half2*>(&a[0]), p1 = *reinterpret_cast<__half2*>(&a[1]);
            const __half2 p2 = *reinterpret_cast<__half2*>(&a[2]), p3 = *reinterpret_cast<__half2*>(&a[3]);
            x[f * kSS + s0 + gid] = p0.x;
            x[(f + 1) * kSS + s0 + gid] = p0.y;
            x[f * kSS + s0 + gid + 8] = p1.x;
            x[(f + 1) * kSS + s0 + gid + 8] = p1.y;
            x[(f + 8) * kSS + s0 + gid] = p2.x;
            x[(f + 9) * kSS + s0 + gid] = p2.y;
            x[(f + 8) * kSS + s0 + gid + 8] = p3.x;
            x[(f + 9) * kSS + s0 + gid + 8] = p3.y;
        }
#pragma unroll
        for (int nt = 0; nt < 8; ++nt) {
            const __half* row = sw + kF1 + (nt * 8 + gid) * kS1 + 16 * j + 2 * tig;
            mma16816(acc[nt], a, lds32(row), lds32(row + 8));
        }
    }
    uint32_t a[4][4];
    for (int l = 2; l <= 6; ++l) {
        relu_to_a(acc, a);
        if (kStore) {  // A_{l-1}^T
            __half* h = act + kHT + (l - 2) * 64 * kSS;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                const int c = nt * 8 + 2 * tig;
                const uint32_t lo = a[nt >> 1][(nt & 1) * 2], hi = a[nt >> 1][(nt & 1) * 2 + 1];
                const __half2 p = *reinterpret_cast<const __half2*>(&lo), q = *reinterpret_cast<const __half2*>(&hi);
                h[c * kSS + s0 + gid] = p.x;
                h[(c + 1) * kSS + s0 + gid] = p.y;
                h[c * kSS + s0 + gid + 8] = q.x;
                h[(c + 1) * kSS + s0 + gid + 8] = q.y;
            }
        }
        if (l < 6) {
            layer64(sw, l, a, acc, gid, tig);
        } else {
            acc6[0] = acc6[1] = acc6[2] = acc6[3] = 0.0f;
            const __half* row = sw + kF6 + gid * kS + 2 * tig;
#pragma unroll
            for (int j = 0; j < 4; ++j) mma16816(acc6, a[j], lds32(row + 16 * j), lds32(row + 16 * j + 8));
        }
    }
}

__device__ __forceinline__ void load_weights_smem(__half* sw, const __half* __restrict__ w16, int halves) {
    const uint4* src = reinterpret_cast<const uint4*>(w16);
    uint4* dst = reinterpret_cast<uint4*>(sw);
    for (int i = threadIdx.x; i < halves / 8; i += blockDim.x) dst[i] = src[i];
}

// Query rows j < n (n = min(n, *n_dev) when n_dev is given); row j reads and writes point list[j] when a
// list is given, else point j.
// Radiance is not negative: with `clamp` set, the queries return max(network output, 0).
__device__ __forceinline__ float out_clamp(float v, uint32_t clamp) { return clamp ? fmaxf(v, 0.0f) : v; }

__global__ void __launch_bounds__(128) infer_kernel(const __half* __restrict__ w16, const float* __restrict__ in,
                                                    const float* __restrict__ albedo, uint32_t n, float* __restrict__ out,
                                                    const uint32_t* __restrict__ list,
                                                    const unsigned long long* __restrict__ n_dev, uint32_t clamp) {
    extern __shared__ __align__(16) __half smem[];
    if (n_dev) {
        const unsigned long long nd = *n_dev;
        n = nd < n ? (uint32_t)nd : n;
    }
    load_weights_smem(smem, w16, kFwdHalves);
    __syncthreads();
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const uint32_t warps = blockDim.x >> 5, tiles = (n + 15u) / 16u;
    for (uint32_t t = blockIdx.x * warps + (threadIdx.x >> 5); t < tiles; t += gridDim.x * warps) {
        const uint32_t j0 = t * 16u + gid, j1 = j0 + 8u;
        const bool ok0 = j0 < n, ok1 = j1 < n;
        const uint32_t p0 = list ? (ok0 ? __ldg(&list[j0]) : 0u) : j0;
        const uint32_t p1 = list ? (ok1 ? __ldg(&list[j1]) : 0u) : j1;
        float v0[kIn], v1[kIn], y[4];
#pragma unroll
        for (int i = 0; i < kIn; ++i) {
            v0[i] = ok0 ? __ldg(&in[(size_t)p0 * kIn + i]) : 0.0f;
            v1[i] = ok1 ? __ldg(&in[(size_t)p1 * kIn + i]) : 0.0f;
        }
        forward16<false>(smem, nullptr, v0, v1, gid, tig, 0, y);
        // output tile columns 2*tig, 2*tig+1 (valid: 0..2; tig 1 holds column 2 only), times the albedo
        if (tig < 2) {
            const size_t c = 2u * tig;
            if (ok0) {
                const size_t o = (size_t)p0 * 3 + c;
                out[o] = albedo ? out_clamp(y[0], clamp) * __ldg(&albedo[o]) : out_clamp(y[0], clamp);
                if (tig == 0) out[o + 1] = albedo ? out_clamp(y[1], clamp) * __ldg(&albedo[o + 1]) : out_clamp(y[1], clamp);
            }
            if (ok1) {
                const size_t o = (size_t)p1 * 3 + c;
                out[o] = albedo ? out_clamp(y[2], clamp) * __ldg(&albedo[o]) : out_clamp(y[2], clamp);
                if (tig == 0) out[o + 1] = albedo ? out_clamp(y[3], clamp) * __ldg(&albedo[o + 1]) : out_clamp(y[3], clamp);
            }
        }
    }
}

// dW_l tiles over the CTA's 64 samples: D[m][n] = sum_s dZT[m][s] * AT[n][s]; m < mrows, n < ncols.
__device__ __forceinline__ void weight_grad(const __half* dzt, const __half* at, int mtiles, int ntiles, int mrows,
                                            int ncols, float* __restrict__ g, int warp, int gid, int tig) {
    const int tiles = mtiles * ntiles;
    for (int tt = warp; tt < tiles; tt += 4) {
        const int mt = tt / ntiles, nt = tt % ntiles;
        float d[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
            uint32_t a[4];
            const __half* ar = dzt + (mt * 16 + gid) * kSS + ks * 16 + 2 * tig;
            a[0] = lds32(ar);
            a[1] = lds32(ar + 8 * kSS);
            a[2] = lds32(ar + 8);
            a[3] = lds32(ar + 8 * kSS + 8);
            const __half* br = at + (nt * 8 + gid) * kSS + ks * 16 + 2 * tig;
            mma16816(d, a, lds32(br), lds32(br + 8));
        }
        const int m0 = mt * 16 + gid, n0 = nt * 8 + 2 * tig;
        if (n0 < ncols) {
            if (m0 < mrows) red_add2(&g[m0 * ncols + n0], d[0], d[1]);
            if (m0 + 8 < mrows) red_add2(&g[(m0 + 8) * ncols + n0], d[2], d[3]);
        }
    }
}

// Stores a 16x64 tile of dZ (C fragments) transposed into dzt and returns its A fragments.
__device__ __forceinline__ void store_dz(const float (&dz)[8][4], __half* dzt, int s0, int gid, int tig, uint32_t (&a)[4][4]) {
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        const int c = nt * 8 + 2 * tig;
        dzt[c * kSS + s0 + gid] = __float2half_rn(dz[nt][0]);
        dzt[(c + 1) * kSS + s0 + gid] = __float2half_rn(dz[nt][1]);
        dzt[c * kSS + s0 + gid + 8] = __float2half_rn(dz[nt][2]);
        dzt[(c + 1) * kSS + s0 + gid + 8] = __float2half_rn(dz[nt][3]);
    }
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        a[j][0] = pack_h2(dz[2 * j][0], dz[2 * j][1]);
        a[j][1] = pack_h2(dz[2 * j][2], dz[2 * j][3]);
        a[j][2] = pack_h2(dz[2 * j + 1][0], dz[2 * j + 1][1]);
        a[j][3] = pack_h2(dz[2 * j + 1][2], dz[2 * j + 1][3]);
    }
}

// dA_{l-1} = dZ_l W_l (B from WT_l), masked by A_{l-1} > 0 read from its transposed tile.
__device__ __forceinline__ void backward64(const __half* sw, int l, const uint32_t (&a)[4][4], const __half* at_prev,
                                           int s0, int gid, int tig, float (&dz)[8][4]) {
    const __half* WT = sw + kT2 + (l - 2) * 64 * kS;
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
        dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.0f;
        const __half* row = WT + (nt * 8 + gid) * kS + 2 * tig;
#pragma unroll
        for (int j = 0; j < 4; ++j) mma16816(dz[nt], a[j], lds32(row + 16 * j), lds32(row + 16 * j + 8));
        const int c = nt * 8 + 2 * tig;
        if (!(__half2float(at_prev[c * kSS + s0 + gid]) > 0.0f)) dz[nt][0] = 0.0f;
        if (!(__half2float(at_prev[(c + 1) * kSS + s0 + gid]) > 0.0f)) dz[nt][1] = 0.0f;
        if (!(__half2float(at_prev[c * kSS + s0 + gid + 8]) > 0.0f)) dz[nt][2] = 0.0f;
        if (!(__half2float(at_prev[(c + 1) * kSS + s0 + gid + 8]) > 0.0f)) dz[nt][3] = 0.0f;
    }
}

__global__ void __launch_bounds__(128) train_kernel(const __half* __restrict__ w16, const float* __restrict__ in,
                                                    const float* __restrict__ target, uint32_t n, float inv_norm,
                                                    float* __restrict__ grad, float* __restrict__ loss_sum,
                                                    const uint32_t* __restrict__ gate) {
    extern __shared__ __align__(16) __half smem[];
    if (gate && *gate == 0u) return;  // empty frame batch: no gradient (uniform over the grid)
    __half* sw = smem;                      // forward + transposed weights
    __half* act = smem + kAllHalves;        // XT, HT1..5, dZT x2
    load_weights_smem(sw, w16, kAllHalves);
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3, warp = threadIdx.x >> 5;
    const int s0 = warp * 16;
    const uint32_t tiles = (n + 63u) / 64u;
    float my_loss = 0.0f;
    __syncthreads();
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t r0 = tile * 64u + s0 + gid, r1 = r0 + 8u;
        float v0[kIn], v1[kIn], y[4];
        load_inputs(in, n, r0, v0);
        load_inputs(in, n, r1, v1);
        forward16<true>(sw, act, v0, v1, gid, tig, s0, y);
        // relative L2: dL/dy = 2 (y - t) / (y^2 + 0.01) / N, scaled; cols 2*tig, 2*tig+1 of rows r0, r1
        float dy[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int col = 2 * tig + (e & 1);
            const uint32_t r = e < 2 ? r0 : r1;
            if (col < kOut && r < n) {
                const float t = __ldg(&target[(size_t)r * 3 + col]);
                const float den = y[e] * y[e] + 0.01f;
                my_loss += (y[e] - t) * (y[e] - t) / den;
                dy[e] = 2.0f * (y[e] - t) / den * inv_norm * kLossScale;
            }
        }
        // layer 6: dZ6 = dY (16 x 3, K padded to 16) -> dZT6 in buffer 0 (rows 0..15)
        __half* dzt0 = act + kDZ;
        __half* dzt1 = act + kDZ + 64 * kSS;
        {
            const int c = 2 * tig;
            // rows 0..7 of dZT6 hold outputs 0..7 (only 0..2 non-zero); write all 8 so padding is zero
            dzt0[c * kSS + s0 + gid] = __float2half_rn(dy[0]);
            dzt0[(c + 1) * kSS + s0 + gid] = __float2half_rn(dy[1]);
            dzt0[c * kSS + s0 + gid + 8] = __float2half_rn(dy[2]);
            dzt0[(c + 1) * kSS + s0 + gid + 8] = __float2half_rn(dy[3]);
            dzt0[(c + 8) * kSS + s0 + gid] = __float2half_rn(0.0f);
            dzt0[(c + 9) * kSS + s0 + gid] = __float2half_rn(0.0f);
            dzt0[(c + 8) * kSS + s0 + gid + 8] = __float2half_rn(0.0f);
            dzt0[(c + 9) * kSS + s0 + gid + 8] = __float2half_rn(0.0f);
        }
        uint32_t a6[4] = {pack_h2(dy[0], dy[1]), pack_h2(dy[2], dy[3]), 0u, 0u};
        float dz[8][4];
        {
            // dA5 = dZ6 W6 (B = WT6[in][out_pad 16]), masked by A5 > 0
            const __half* at5 = act + kHT + 4 * 64 * kSS;
#pragma unroll
            for (int nt = 0; nt < 8; ++nt) {
                dz[nt][0] = dz[nt][1] = dz[nt][2] = dz[nt][3] = 0.0f;
                const __half* row = sw + kT6 + (nt * 8 + gid) * kST6 + 2 * tig;
                mma16816(dz[nt], a6, lds32(row), lds32(row + 8));
                const int c = nt * 8 + 2 * tig;
                if (!(__half2float(at5[c * kSS + s0 + gid]) > 0.0f)) dz[nt][0] = 0.0f;
                if (!(__half2float(at5[(c + 1) * kSS + s0 + gid]) > 0.0f)) dz[nt][1] = 0.0f;
                if (!(__half2float(at5[c * kSS + s0 + gid + 8]) > 0.0f)) dz[nt][2] = 0.0f;
                if (!(__half2float(at5[(c + 1) * kSS + s0 + gid + 8]) > 0.0f)) dz[nt][3] = 0.0f;
            }
        }
        __syncthreads();
        weight_grad(dzt0, act + kHT + 4 * 64 * kSS, 1, 8, kOut, kW, grad + off(5), warp, gid, tig);
        // layers 5..1
        for (int l = 5; l >= 1; --l) {
            __half* dzt = (l & 1) ? dzt1 : dzt0;
            uint32_t a[4][4];
            store_dz(dz, dzt, s0, gid, tig, a);
            if (l > 1) backward64(sw, l, a, act + kHT + (l - 2) * 64 * kSS, s0, gid, tig, dz);
            __syncthreads();
            if (l > 1) weight_grad(dzt, act + kHT + (l - 2) * 64 * kSS, 4, 8, kW, kW, grad + off(l - 1), warp, gid, tig);
            else weight_grad(dzt, act + kXT, 4, 28, kW, kEnc, grad + off(0), warp, gid, tig);
        }
        __syncthreads();
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_down_sync(0xFFFFFFFFu, my_loss, o);
    if (lane == 0 && loss_sum) atomicAdd(loss_sum, my_loss);
}

// Adam on the FP32 masters, then refresh both FP16 layouts; the weight EMA (and its FP16 forward
// layout, which inference reads) follows: ema = decay * ema + (1 - decay) * w. The consumed gradient
// is cleared here, so the next step accumulates into zeros.
__global__ void adam_kernel(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                            float* __restrict__ g, __half* __restrict__ w16, float* __restrict__ ema,
                            __half* __restrict__ w16_ema, __half* __restrict__ wu, __half* __restrict__ wu_ema, float decay,
                            float lr, float c1, float c2, float inv_scale, const uint32_t* __restrict__ gate, float b1,
                            float b2) {
    tc::pdl_wait();  // the gradient of the training kernel ahead
    tc::pdl_trigger();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams || (gate && *gate == 0u)) return;
    const float eps = 1e-8f;
    const float gi = g[i] * inv_scale;
    g[i] = 0.0f;  // the gradient starts from zero for the next step (no separate clear)
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    w[i] = wi;
    int l = 0;
    while (i >= off(l + 1)) ++l;
    const int din = l == 0 ? kEnc : kW, local = i - off(l), o = local / din, k = local % din;
    const __half h = __float2half_rn(wi);
    w16[fwd_off(l + 1) + o * fwd_stride(l + 1) + k] = h;
    if (l >= 1 && l <= 4) w16[kT2 + (l - 1) * 64 * kS + k * kS + o] = h;
    if (l == 5) w16[kT6 + k * kST6 + o] = h;
    wu[u_index(l + 1, o, k)] = h;
    const float e = decay * ema[i] + (1.0f - decay) * wi;
    ema[i] = e;
    const __half he = __float2half_rn(e);
    w16_ema[fwd_off(l + 1) + o * fwd_stride(l + 1) + k] = he;
    wu_ema[u_index(l + 1, o, k)] = he;
}

// FP16 layouts from the masters (used after init / set_weights; padding stays zero); the EMA restarts
// from the same weights.
__global__ void pack_kernel(const float* __restrict__ w, __half* __restrict__ w16, float* __restrict__ ema,
                            __half* __restrict__ w16_ema, __half* __restrict__ wu, __half* __restrict__ wu_ema) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    int l = 0;
    while (i >= off(l + 1)) ++l;
    const int din = l == 0 ? kEnc : kW, local = i - off(l), o = local / din, k = local % din;
    const __half h = __float2half_rn(w[i]);
    w16[fwd_off(l + 1) + o * fwd_stride(l + 1) + k] = h;
    if (l >= 1 && l <= 4) w16[kT2 + (l - 1) * 64 * kS + k * kS + o] = h;
    if (l == 5) w16[kT6 + k * kST6 + o] = h;
    ema[i] = w[i];
    w16_ema[fwd_off(l + 1) + o * fwd_stride(l + 1) + k] = h;
    wu[u_index(l + 1, o, k)] = h;
    wu_ema[u_index(l + 1, o, k)] = h;
}


// ---- tcgen05 inference --------------------------------------------------------------------------
// A CTA of 128 threads evaluates 128 queries per tile, thread m owning row m. The elected thread 0
// issues tcgen05.mma (M = 128, N = 64 or 16, K = 16 per instruction) from shared-memory operands into
// a TMEM accumulator (128 lanes x 64 + 16 columns); every thread reads its lane back with tcgen05.ld,
// applies ReLU, packs FP16 and writes the next layer's A operand. The weights (63.5 KB) arrive once per
// CTA through one bulk copy. The A buffer (28 KB) holds half of the 224 encoded features or one hidden
// layer, so layer 1 runs as two accumulating passes; two CTAs fit on an SM.
constexpr int kTcA = 128 * 112;  // halves
constexpr uint32_t kTcSmem = kUHalves * 2 + kTcA * 2 + 64;          // one tile group
constexpr int kTcGroups = 4;                                       // tile groups of the default kernel
constexpr uint32_t kTcSmemG = kUHalves * 2 + kTcGroups * kTcA * 2 + 64;
constexpr long long kTcBudget = 2000000000ll;  // cycles (about one second) per wait
// A kernel whose wait ran out sets bit 31 of the status word, stops issuing work, and before it frees
// TMEM and returns waits (with the full budget again) for what it still has in flight: the weight copy
// into shared memory and, if one was committed and not yet seen to complete, the last MMA batch. The
// `budget` kernel argument is the per-wait budget in cycles (kTcBudget unless a test shrinks it). With
// `stall` set (a test's fault injection) the weight barrier is armed but the copy is never issued, so
// the first wait can only run out; nothing is then in flight and the drain waits only `budget`.

// sin/cos(2^k pi x), k = 0..11, as 12 packed (sin, cos) FP16 pairs: sincospif at k = 0 and k = 6 and
// five angle doublings after each (s' = 2 s c, c' = (c - s)(c + s)), which add a few ulp of FP32.
__device__ __forceinline__ void enc_input(float x, uint32_t (&h)[12]) {
    float s, c;
#pragma unroll
    for (int base = 0; base < 12; base += 6) {
        sincospif(base ? x * 64.0f : x, &s, &c);
        h[base] = pack_h2(s, c);
#pragma unroll
        for (int k = 1; k < 6; ++k) {
            const float s2 = 2.0f * s * c, c2 = (c - s) * (c + s);
            s = s2;
            c = c2;
            h[base + k] = pack_h2(s, c);
        }
    }
}

// 16-byte chunk lc (8 halves along K) of row m in an A buffer of kbc chunks per row.
__device__ __forceinline__ void st_chunk(uint8_t* sa, int kbc, int m, int lc, uint4 v) {
    *reinterpret_cast<uint4*>(sa + 2 * ((m >> 3) * kbc * 64 + lc * 64 + (m & 7) * 8)) = v;
}

// OR of `v` over the 128 threads of tile group `id - 1` (named barrier `id`; id 0 is __syncthreads).
__device__ __forceinline__ bool group_sync_or(uint32_t id, bool v) {
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.or.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
        : "=r"(r)
        : "r"((uint32_t)v), "r"(id)
        : "memory");
    return r != 0u;
}

// Tensor-core inference with G tile groups per CTA: the CTA holds the weights once and G groups of
// four warps each run their own 128-query tiles (own A buffer, TMEM columns 128 g .. 128 g + 79,
// mbarrier and named barrier). G = 1 (the default) is the single-tile kernel, two CTAs per SM. G = 4
// keeps four tiles in flight per SM (weights 63.5 KB + 4 x 28 KB of A buffers) but measured 7 %
// slower on a 1080p hit list (0.0547 against 0.0513 ms), and its one CTA per SM no longer shares the
// SMs with the training-sample kernel when the query runs beside it.
template <int G>
__global__ void __launch_bounds__(128 * G, G == 1 ? 2 : 1) infer_tc_kernel(
    const __half* __restrict__ wu, const float* __restrict__ in, const float* __restrict__ albedo, uint32_t n,
    float* __restrict__ out, const uint32_t* __restrict__ list, const unsigned long long* __restrict__ n_dev,
    uint32_t* __restrict__ status, long long budget, uint32_t stall, uint32_t clamp) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    const uint32_t g = threadIdx.x >> 7, tid = threadIdx.x & 127u, warp = tid >> 5;
    uint8_t* sw = smem_raw;
    uint8_t* sa = smem_raw + kUHalves * 2 + (size_t)g * kTcA * 2;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + kUHalves * 2 + (size_t)G * kTcA * 2);  // bar_w, bar_m[G]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 1 + G);
    tc::pdl_wait();  // the weight average of the Adam step ahead, the hit list of the kernel ahead
    if (n_dev) {
        const unsigned long long nd = *n_dev;
        n = nd < n ? (uint32_t)nd : n;
    }
    const uint32_t tiles = (n + 127u) / 128u;
    if (blockIdx.x * G >= tiles) return;  // uniform over the CTA, before any TMEM allocation
    const uint32_t bar_w = tc::smem_u32(&bars[0]), bar_m = tc::smem_u32(&bars[1 + g]);
    const uint32_t sa_u = tc::smem_u32(sa), sw_u = tc::smem_u32(sw);
    if (threadIdx.x == 0) {
        tc::mbar_init(bar_w, 1);
        for (int i = 0; i < G; ++i) tc::mbar_init(tc::smem_u32(&bars[1 + i]), 1);
        tc::fence_mbar_init();
    }
    if (threadIdx.x < 32) {
        tc::tmem_alloc(tc::smem_u32(tslot), G == 1 ? 128u : (G == 2 ? 256u : 512u));
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot;
    const uint32_t d_hid = tmem + 128u * g, d_out = d_hid + 64u, lane_off = (warp * 32u) << 16;
    if (threadIdx.x == 0) {
        tc::mbar_expect_tx(bar_w, kUHalves * 2);
        if (!stall) tc::bulk_g2s(sw_u, wu, kUHalves * 2, bar_w);
    }
    // the weights are waited for after the group's first tile is fetched and half encoded (the operand
    // buffer and the weights are disjoint), so the copy runs under that work
    bool ok = true, weights_pending = true;
    bool fail = false;
    uint32_t phase = 0;
    bool mma_pending = false;  // group leader: a committed MMA batch whose completion it has not seen
    auto gsync = [&](bool v) { return G == 1 ? (__syncthreads_or(v) != 0) : group_sync_or(1u + g, v); };
    constexpr uint32_t kId64 = tc::idesc_f16(128, 64, false, false), kId16 = tc::idesc_f16(128, 16, false, false);
    // one MMA pass: D (+)= A[sa] * W^T, `steps` K-steps; A has a_sbo bytes per 8-row group
    auto issue = [&](uint32_t d, uint32_t w_byte, uint32_t w_sbo, uint32_t a_sbo, int steps, uint32_t idesc, bool acc) {
        if (tid == 0) {
            tc::fence_after();
            for (int st = 0; st < steps; ++st)
                tc::mma_f16(d, tc::sdesc(sa_u + 256u * st, 128u, a_sbo), tc::sdesc(sw_u + w_byte + 256u * st, 128u, w_sbo),
                            idesc, (acc || st) ? 1u : 0u);
            tc::commit(bar_m);
            mma_pending = true;
        }
        ok = tc::mbar_wait(bar_m, phase, budget);
        if (ok) {
            phase ^= 1u;
            mma_pending = false;
        }
        tc::fence_after();
    };
    // inputs (and albedo) of the group's first tile; each iteration then fetches the next tile's before
    // its MMA chain
    float vn[kIn], an[kOut];
    uint32_t pn = 0u;
    bool valid_n = false;
    auto fetch = [&](uint32_t tile) {
        const uint32_t j = tile * 128u + tid;
        valid_n = tile < tiles && j < n;
        pn = valid_n ? (list ? __ldg(&list[j]) : j) : 0u;
#pragma unroll
        for (int i = 0; i < kIn; ++i) vn[i] = valid_n ? __ldg(&in[(size_t)pn * kIn + i]) : 0.0f;
#pragma unroll
        for (int c = 0; c < kOut; ++c) an[c] = valid_n && albedo ? __ldg(&albedo[(size_t)pn * 3 + c]) : 1.0f;
    };
    const uint32_t first = blockIdx.x * G + g, stride = gridDim.x * G;
    fetch(first);
    for (uint32_t tile = first; !fail && tile < tiles; tile += stride) {
        const bool valid = valid_n;
        const uint32_t p = pn;
        float v[kIn], a[kOut];
#pragma unroll
        for (int i = 0; i < kIn; ++i) v[i] = vn[i];
#pragma unroll
        for (int c = 0; c < kOut; ++c) a[c] = an[c];
        fetch(tile + stride);
        // layer 1, first half: features 0..111 = inputs 0..3 and the first 16 features of input 4
        uint32_t h[12];
        uint4 keep;
#pragma unroll
        for (int i = 0; i < 5; ++i) {
            enc_input(v[i], h);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const uint4 ch = make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]);
                if (3 * i + q < 14) st_chunk(sa, 14, tid, 3 * i + q, ch);
                else keep = ch;
            }
        }
        tc::fence_async_smem();
        tc::fence_before();
        if (weights_pending) {
            ok = tc::mbar_wait(bar_w, 0, budget);
            weights_pending = false;
        }
        if ((fail = gsync(!ok))) break;
        issue(d_hid, 2u * u_off(1), 3584u, 1792u, 7, kId64, false);
        // second half: features 112..223 (the rest of input 4, inputs 5..8, 8 zero features)
        if ((fail = gsync(!ok))) break;
        st_chunk(sa, 14, tid, 0, keep);
#pragma unroll
        for (int i = 5; i < kIn; ++i) {
            enc_input(v[i], h);
#pragma unroll
            for (int q = 0; q < 3; ++q)
                st_chunk(sa, 14, tid, 3 * i + q - 14, make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]));
        }
        st_chunk(sa, 14, tid, 13, make_uint4(0u, 0u, 0u, 0u));
        tc::fence_async_smem();
        tc::fence_before();
        if ((fail = gsync(!ok))) break;
        issue(d_hid, 2u * u_off(1) + 14u * 128u, 3584u, 1792u, 7, kId64, true);
        // layers 2..6: ReLU of the accumulator -> FP16 A operand -> next MMA
        for (int l = 2; l <= 6 && !fail; ++l) {
            uint32_t r[4][16];
#pragma unroll
            for (int q = 0; q < 4; ++q) tc::tmem_ld16(d_hid + lane_off + 16u * q, r[q]);
            tc::tmem_wait_ld();
#pragma unroll
            for (int q = 0; q < 4; ++q) {
#pragma unroll
                for (int c2 = 0; c2 < 2; ++c2) {
                    uint32_t pk[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        pk[e] = relu_pack_h2(__uint_as_float(r[q][8 * c2 + 2 * e]), __uint_as_float(r[q][8 * c2 + 2 * e + 1]));
                    st_chunk(sa, 8, tid, 2 * q + c2, make_uint4(pk[0], pk[1], pk[2], pk[3]));
                }
            }
            tc::fence_async_smem();
            tc::fence_before();
            if ((fail = gsync(!ok))) break;
            issue(l < 6 ? d_hid : d_out, 2u * u_off(l), 1024u, 1024u, 4, l < 6 ? kId64 : kId16, false);
        }
        if ((fail = gsync(!ok))) break;
        uint32_t y[16];
        tc::tmem_ld16(d_out + lane_off, y);
        tc::tmem_wait_ld();
        if (valid) {
#pragma unroll
            for (int c = 0; c < kOut; ++c) {
                const float val = out_clamp(__uint_as_float(y[c]), clamp);
                out[(size_t)p * 3 + c] = albedo ? val * a[c] : val;
            }
        }
        tc::fence_before();
    }
    if (fail && tid == 0) {
        atomicOr(status, 0x80000000u);
        // the weight copy and an MMA still in flight finish before shared memory and TMEM are released
        tc::mbar_wait(bar_w, 0, stall ? budget : kTcBudget);
        if (mma_pending) tc::mbar_wait(bar_m, phase, kTcBudget);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (threadIdx.x < 32) tc::tmem_dealloc(tmem, G == 1 ? 128u : (G == 2 ? 256u : 512u));
}

// ---- tcgen05 training -----------------------------------------------------------------------------
// One CTA per SM takes 128-sample tiles of the batch (thread m = sample m of the tile):
//   forward   layers 1..6 as in inference, keeping the FP16 operands: the encoding A0 (128 x 256,
//             features 216..255 zero) in region R, then H1..H4 in R (A0 is dead after layer 1) and H5
//   output    dY = 2 (y - t) / (y^2 + 0.01) / n * 128 (loss scale) -> dZ6 (128 x 16)
//   backward  dA_{l-1} = dZ_l W_l (B = W_l read MN-major from the forward layout), masked by H_{l-1} > 0
//   gradients dW_l^T += H_{l-1}^T dZ_l in TMEM (A and B MN-major views of the activation buffers; M 64
//             rows of H features, or 2 x M 128 over the re-encoded A0 for layer 1), accumulated over all
//             of the CTA's tiles and added to the FP32 gradient once at the end.
// TMEM columns: 0..63 layer accumulator, 64..79 output, 80..95 dW6^T, 128..255 dW1^T (two M-halves),
// 256..511 dW2^T..dW5^T. An M = 64 accumulator keeps row r in lane 32 (r / 16) + r % 16.
constexpr uint32_t kTtR = kUHalves * 2;         // region R: A0, then H1..H4 (64 KB)
constexpr uint32_t kTtH5 = kTtR + 65536;        // H5 (16 KB)
constexpr uint32_t kTtDZ = kTtH5 + 16384;       // dZ (16 KB)
constexpr uint32_t kTtBar = kTtDZ + 16384;
constexpr uint32_t kTtSmem = kTtBar + 64;       // 161,856 B

__device__ __forceinline__ uint32_t tt_h(int l) { return l <= 4 ? kTtR + 16384u * (l - 1) : kTtH5; }  // H_l, l = 1..5

// red.add of one TMEM row (64 FP32 columns, loss-scaled) of a transposed weight gradient: g[o * din + f].
__device__ __forceinline__ void red_row(float* __restrict__ g, int din, int f, int ncols, const uint32_t (&r)[4][16]) {
#pragma unroll
    for (int q = 0; q < 4; ++q)
#pragma unroll
        for (int e = 0; e < 16; ++e)
            if (16 * q + e < ncols) atomicAdd(&g[(16 * q + e) * din + f], __uint_as_float(r[q][e]));
}

__global__ void __launch_bounds__(128, 1) train_tc_kernel(const __half* __restrict__ wu, const float* __restrict__ in,
                                                          const float* __restrict__ target, uint32_t n, float inv_norm,
                                                          float* __restrict__ grad, float* __restrict__ loss_sum,
                                                          const uint32_t* __restrict__ gate, uint32_t* __restrict__ status,
                                                          long long budget, uint32_t stall) {
    extern __shared__ __align__(128) uint8_t smem_raw[];
    tc::pdl_wait();  // the samples (or the weights of the Adam step) of the kernel ahead
    if (gate && *gate == 0u) return;  // empty frame batch (uniform over the grid)
    const uint32_t tiles = (n + 127u) / 128u;
    if (blockIdx.x >= tiles) return;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smem_raw + kTtBar);
    uint32_t* tslot = reinterpret_cast<uint32_t*>(bars + 2);
    const uint32_t tid = threadIdx.x, warp = tid >> 5, lane = tid & 31u;
    const uint32_t bar_w = tc::smem_u32(&bars[0]), bar_m = tc::smem_u32(&bars[1]);
    const uint32_t s0 = tc::smem_u32(smem_raw);
    if (tid == 0) {
        tc::mbar_init(bar_w, 1);
        tc::mbar_init(bar_m, 1);
        tc::fence_mbar_init();
    }
    if (warp == 0) {
        tc::tmem_alloc(tc::smem_u32(tslot), 512);
        tc::tmem_relinquish();
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = *tslot, lane_off = (warp * 32u) << 16;
    const uint32_t d_hid = tmem, d_out = tmem + 64u, d_w6 = tmem + 80u, d_w1 = tmem + 128u;
    auto d_wl = [&](int l) { return tmem + 256u + 64u * (uint32_t)(l - 2); };  // dW_l^T, l = 2..5
    if (tid == 0) {
        tc::mbar_expect_tx(bar_w, kUHalves * 2);
        if (!stall) tc::bulk_g2s(s0, wu, kUHalves * 2, bar_w);
    }
    // the weights are waited for after the first tile's inputs are loaded and encoded (their regions
    // are disjoint), so the copy runs under that work
    bool ok = true, weights_pending = true;
    bool fail = false;
    uint32_t phase = 0;
    bool mma_pending = false;  // thread 0: a committed MMA batch whose completion it has not seen
    float my_loss = 0.0f;
    bool first = true;  // first tile of this CTA: weight-gradient accumulators start from zero
    constexpr uint32_t kF64 = tc::idesc_f16(128, 64, false, false), kF16 = tc::idesc_f16(128, 16, false, false);
    constexpr uint32_t kBwd = tc::idesc_f16(128, 64, false, true);   // dZ (K-major) x W (MN-major)
    constexpr uint32_t kG64 = tc::idesc_f16(64, 64, true, true), kG16 = tc::idesc_f16(64, 16, true, true);
    constexpr uint32_t kG1 = tc::idesc_f16(128, 64, true, true);
    auto wait_mma = [&]() {
        if (tid == 0) {
            tc::commit(bar_m);
            mma_pending = true;
        }
        ok = tc::mbar_wait(bar_m, phase, budget);
        if (ok) {
            phase ^= 1u;
            mma_pending = false;
        }
        tc::fence_after();
    };
    auto fwd_layer = [&](uint32_t d, uint32_t a_off, uint32_t a_sbo, int l, int steps, uint32_t idesc) {
        if (tid == 0) {
            tc::fence_after();
            const uint32_t w_sbo = (uint32_t)(u_k(l) / 8) * 128u;
            for (int st = 0; st < steps; ++st)
                tc::mma_f16(d, tc::sdesc(s0 + a_off + 256u * st, 128u, a_sbo), tc::sdesc(s0 + 2u * u_off(l) + 256u * st, 128u, w_sbo),
                            idesc, st ? 1u : 0u);
        }
        wait_mma();
    };
    // FP16 row of 64 features from the accumulator (ReLU optional) into a K-major buffer
    auto store_row64 = [&](const uint32_t (&r)[4][16], uint32_t buf, bool relu) {
#pragma unroll
        for (int c = 0; c < 8; ++c) {
            uint32_t pk[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const float a = __uint_as_float(r[c >> 1][8 * (c & 1) + 2 * e]), b = __uint_as_float(r[c >> 1][8 * (c & 1) + 2 * e + 1]);
                pk[e] = relu ? relu_pack_h2(a, b) : pack_h2(a, b);
            }
            st_chunk(smem_raw + buf, 8, tid, c, make_uint4(pk[0], pk[1], pk[2], pk[3]));
        }
    };
    auto ld64 = [&](uint32_t d, uint32_t (&r)[4][16]) {
#pragma unroll
        for (int q = 0; q < 4; ++q) tc::tmem_ld16(d + lane_off + 16u * q, r[q]);
        tc::tmem_wait_ld();
    };
    auto encode_a0 = [&](const float (&v)[kIn]) {
        uint32_t h[12];
#pragma unroll
        for (int i = 0; i < kIn; ++i) {
            enc_input(v[i], h);
#pragma unroll
            for (int q = 0; q < 3; ++q)
                st_chunk(smem_raw + kTtR, 32, tid, 3 * i + q, make_uint4(h[4 * q], h[4 * q + 1], h[4 * q + 2], h[4 * q + 3]));
        }
#pragma unroll
        for (int c = 27; c < 32; ++c) st_chunk(smem_raw + kTtR, 32, tid, c, make_uint4(0u, 0u, 0u, 0u));
    };
    for (uint32_t tile = blockIdx.x; !fail && tile < tiles; tile += gridDim.x) {
        const uint32_t j = tile * 128u + tid;
        const bool valid = j < n;
        float v[kIn], t[kOut];
#pragma unroll
        for (int i = 0; i < kIn; ++i) v[i] = valid ? __ldg(&in[(size_t)j * kIn + i]) : 0.0f;
#pragma unroll
        for (int c = 0; c < kOut; ++c) t[c] = valid ? __ldg(&target[(size_t)j * kOut + c]) : 0.0f;
        // ---- forward
        encode_a0(v);
        tc::fence_async_smem();
        tc::fence_before();
        if (weights_pending) {
            ok = tc::mbar_wait(bar_w, 0, budget);
            weights_pending = false;
        }
        if ((fail = __syncthreads_or(!ok))) break;
        fwd_layer(d_hid, kTtR, 4096u, 1, 14, kF64);
        uint32_t r[4][16];
        for (int l = 2; l <= 6 && !fail; ++l) {
            ld64(d_hid, r);
            store_row64(r, tt_h(l - 1), true);
            tc::fence_async_smem();
            tc::fence_before();
            if ((fail = __syncthreads_or(!ok))) break;
            fwd_layer(l < 6 ? d_hid : d_out, tt_h(l - 1), 1024u, l, 4, l < 6 ? kF64 : kF16);
        }
        if ((fail = __syncthreads_or(!ok))) break;
        // ---- output gradient
        uint32_t y[16];
        tc::tmem_ld16(d_out + lane_off, y);
        tc::tmem_wait_ld();
        float dy[kOut];
#pragma unroll
        for (int c = 0; c < kOut; ++c) {
            const float yc = __uint_as_float(y[c]);
            const float den = yc * yc + 0.01f;
            dy[c] = valid ? 2.0f * (yc - t[c]) / den * inv_norm * kLossScale : 0.0f;
            if (valid) my_loss += (yc - t[c]) * (yc - t[c]) / den;
        }
        st_chunk(smem_raw + kTtDZ, 8, tid, 0, make_uint4(pack_h2(dy[0], dy[1]), pack_h2(dy[2], 0.0f), 0u, 0u));
        st_chunk(smem_raw + kTtDZ, 8, tid, 1, make_uint4(0u, 0u, 0u, 0u));
        tc::fence_async_smem();
        tc::fence_before();
        if ((fail = __syncthreads_or(!ok))) break;
        if (tid == 0) {
            tc::fence_after();
            // dA5 = dZ6 W6 (K = 16 outputs)
            tc::mma_f16(d_hid, tc::sdesc(s0 + kTtDZ, 128u, 1024u), tc::sdesc(s0 + 2u * u_off(6), 1024u, 128u), kBwd, 0u);
            // dW6^T += H5^T dZ6 (K = 128 samples)
            for (int st = 0; st < 8; ++st)
                tc::mma_f16(d_w6, tc::sdesc(s0 + kTtH5 + 2048u * st, 1024u, 128u), tc::sdesc(s0 + kTtDZ + 2048u * st, 1024u, 128u),
                            kG16, (!first || st) ? 1u : 0u);
        }
        wait_mma();
        // ---- backward through layers 5..1
        for (int l = 5; l >= 1 && !fail; --l) {
            ld64(d_hid, r);  // dA_l
            const uint8_t* hrow = smem_raw + tt_h(l) + 2 * ((tid >> 3) * 8 * 64 + (tid & 7) * 8);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const uint4 hv = *reinterpret_cast<const uint4*>(hrow + 2 * 64 * c);
                const uint32_t hw[4] = {hv.x, hv.y, hv.z, hv.w};
                uint32_t pk[4];
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const __half2 hh = *reinterpret_cast<const __half2*>(&hw[e]);
                    const float a = __half2float(hh.x) > 0.0f ? __uint_as_float(r[c >> 1][8 * (c & 1) + 2 * e]) : 0.0f;
                    const float b = __half2float(hh.y) > 0.0f ? __uint_as_float(r[c >> 1][8 * (c & 1) + 2 * e + 1]) : 0.0f;
                    pk[e] = pack_h2(a, b);
                }
                st_chunk(smem_raw + kTtDZ, 8, tid, c, make_uint4(pk[0], pk[1], pk[2], pk[3]));
            }
            if (l == 1) {  // H1..H4 are consumed (every thread has read its H1 mask row): A0 again for dW1
                __syncthreads();
                encode_a0(v);
            }
            tc::fence_async_smem();
            tc::fence_before();
            if ((fail = __syncthreads_or(!ok))) break;
            if (tid == 0) {
                tc::fence_after();
                if (l >= 2) {
                    // dA_{l-1} = dZ_l W_l
                    for (int st = 0; st < 4; ++st)
                        tc::mma_f16(d_hid, tc::sdesc(s0 + kTtDZ + 256u * st, 128u, 1024u),
                                    tc::sdesc(s0 + 2u * u_off(l) + 2048u * st, 1024u, 128u), kBwd, st ? 1u : 0u);
                    // dW_l^T += H_{l-1}^T dZ_l
                    for (int st = 0; st < 8; ++st)
                        tc::mma_f16(d_wl(l), tc::sdesc(s0 + tt_h(l - 1) + 2048u * st, 1024u, 128u),
                                    tc::sdesc(s0 + kTtDZ + 2048u * st, 1024u, 128u), kG64, (!first || st) ? 1u : 0u);
                } else {
                    // dW1^T += A0^T dZ1, features 0..127 and 128..255
                    for (int half = 0; half < 2; ++half)
                        for (int st = 0; st < 8; ++st)
                            tc::mma_f16(d_w1 + 64u * half, tc::sdesc(s0 + kTtR + 2048u * half + 8192u * st, 4096u, 128u),
                                        tc::sdesc(s0 + kTtDZ + 2048u * st, 1024u, 128u), kG1, (!first || st) ? 1u : 0u);
                }
            }
            wait_mma();
        }
        first = false;
    }
    tc::pdl_trigger();  // the Adam step behind may be scheduled (it waits for this grid to finish)
    if (!fail) fail = __syncthreads_or(!ok);
    if (!fail) {
        // weight gradients out of TMEM (every warp runs the collective loads; lanes pick their rows)
        uint32_t r[4][16];
        for (int half = 0; half < 2; ++half) {  // layer 1: lane = feature
            ld64(d_w1 + 64u * half, r);
            const int f = (int)tid + 128 * half;
            if (f < kEnc) red_row(grad + off(0), kEnc, f, 64, r);
        }
        const bool row_lane = lane < 16u;  // M = 64 accumulators: rows 16 warp + lane for lanes 0..15
        const int f = (int)(16u * warp + lane);
        for (int l = 2; l <= 5; ++l) {
            ld64(d_wl(l), r);
            if (row_lane) red_row(grad + off(l - 1), kW, f, 64, r);
        }
        uint32_t r6[16];
        tc::tmem_ld16(d_w6 + lane_off, r6);
        tc::tmem_wait_ld();
        if (row_lane) {
#pragma unroll
            for (int o = 0; o < kOut; ++o) atomicAdd(&grad[off(5) + o * kW + f], __uint_as_float(r6[o]));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) my_loss += __shfl_down_sync(0xFFFFFFFFu, my_loss, o);
        if (lane == 0 && loss_sum) atomicAdd(loss_sum, my_loss);
    } else if (tid == 0) {
        atomicOr(status, 0x80000000u);
        // the weight copy and an MMA still in flight finish before shared memory and TMEM are released
        tc::mbar_wait(bar_w, 0, stall ? budget : kTcBudget);
        if (mma_pending) tc::mbar_wait(bar_m, phase, kTcBudget);
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    if (warp == 0) tc::tmem_dealloc(tmem, 512);
}

}  // namespace nrc

// ------------------------------------------------------------------------------------------------
// C ABI
// ------------------------------------------------------------------------------------------------

namespace {

int nrc_err(arc_ctx* c, int code, const std::string& m) {
    c->err = m;
    return code;
}

int nrc_cuda(arc_ctx* c, cudaError_t e, const char* what) {
    return nrc_err(c, ARC_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define NRC_CK(expr)                                        \
    do {                                                    \
        cudaError_t e__ = (expr);                           \
        if (e__ != cudaSuccess) return nrc_cuda(c, e__, #expr); \
    } while (0)

int ensure_nrc(arc_ctx* c) {
    if (c->d_nrc_w32) return ARC_OK;
    NRC_CK(cudaMalloc((void**)&c->d_nrc_w32, sizeof(float) * nrc::kParams * 5));
    c->d_nrc_m = c->d_nrc_w32 + nrc::kParams;
    c->d_nrc_v = c->d_nrc_m + nrc::kParams;
    c->d_nrc_grad = c->d_nrc_v + nrc::kParams;
    c->d_nrc_ema = c->d_nrc_grad + nrc::kParams;
    NRC_CK(cudaMalloc(&c->d_nrc_w16, sizeof(__half) * nrc::kAllHalves));
    NRC_CK(cudaMalloc(&c->d_nrc_w16_ema, sizeof(__half) * nrc::kFwdHalves));
    NRC_CK(cudaMalloc(&c->d_nrc_wu_ema, sizeof(__half) * nrc::kUHalves));
    NRC_CK(cudaMalloc(&c->d_nrc_wu, sizeof(__half) * nrc::kUHalves));
    NRC_CK(cudaMalloc((void**)&c->d_nrc_loss, sizeof(float)));
    NRC_CK(cudaMemsetAsync(c->d_nrc_w32, 0, sizeof(float) * nrc::kParams * 5, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_w16, 0, sizeof(__half) * nrc::kAllHalves, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_w16_ema, 0, sizeof(__half) * nrc::kFwdHalves, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_wu_ema, 0, sizeof(__half) * nrc::kUHalves, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_wu, 0, sizeof(__half) * nrc::kUHalves, c->stream));
    NRC_CK(cudaFuncSetAttribute(nrc::train_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrc::kTtSmem));
    NRC_CK(cudaFuncSetAttribute(nrc::infer_tc_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)nrc::kTcSmem));
    NRC_CK(cudaFuncSetAttribute(nrc::infer_tc_kernel<nrc::kTcGroups>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)nrc::kTcSmemG));
    NRC_CK(cudaFuncSetAttribute(nrc::infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                nrc::kFwdHalves * (int)sizeof(__half)));
    NRC_CK(cudaFuncSetAttribute(nrc::train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (nrc::kAllHalves + nrc::kActHalves) * (int)sizeof(__half)));
    c->nrc_step = 0;
    return ARC_OK;
}

// Uniform(-b, b) weights from a splitmix64 stream.
void init_weights(std::vector<float>& w, uint32_t seed) {
    uint64_t s = 0x9E3779B97F4A7C15ull ^ seed;
    auto next = [&]() {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    for (int l = 0; l < 6; ++l) {
        const int din = l == 0 ? nrc::kEnc : nrc::kW;
        // He-uniform for the ReLU layers; the linear output layer starts 10x smaller so the first
        // predictions sit near zero instead of far above the radiance scale
        const float bound = std::sqrt(6.0f / (float)din) * (l == 5 ? 0.1f : 1.0f);
        for (int i = nrc::off(l); i < nrc::off(l + 1); ++i) {
            const float u = (float)((next() >> 40) * (1.0 / 16777216.0));
            w[i] = (2.0f * u - 1.0f) * bound;
        }
    }
}

long long tc_budget(const arc_ctx* c) { return c->tc_wait_budget > 0 ? c->tc_wait_budget : nrc::kTcBudget; }

int launch_infer(arc_ctx* c, const float* inputs, const float* albedo, uint32_t n, float* out, const uint32_t* list,
                 const unsigned long long* n_dev, bool beside = false) {
    const __half* wu = static_cast<const __half*>(c->d_nrc_wu_ema);
    // path 3 (automatic): four tile groups for a query on its own; one group beside the training
    // samples, whose kernel shares the SMs (a four-group CTA takes a whole SM's shared memory)
    const int path = c->nrc_infer_path == 3 ? (beside ? 1 : 2) : c->nrc_infer_path;
    if (path == 2) {  // four tile groups per CTA, one CTA per SM
        const uint32_t tiles = (n + 127u) / 128u;
        const uint32_t blocks = std::min<uint32_t>((tiles + nrc::kTcGroups - 1u) / nrc::kTcGroups, (uint32_t)c->n_sm);
        NRC_CK(arc_launch_overlapped(c, nrc::infer_tc_kernel<nrc::kTcGroups>, dim3(blocks), dim3(128 * nrc::kTcGroups), nrc::kTcSmemG, wu,
                        inputs, albedo, n, out, list, n_dev, c->d_status, tc_budget(c), c->tc_stall ? 1u : 0u,
                        c->nrc_clamp ? 1u : 0u));
        return ARC_OK;
    }
    if (path == 1) {  // one tile group per CTA, two CTAs per SM
        const uint32_t blocks = std::min<uint32_t>((n + 127u) / 128u, (uint32_t)c->n_sm * 2u);
        NRC_CK(arc_launch_overlapped(c, nrc::infer_tc_kernel<1>, dim3(blocks), dim3(128), nrc::kTcSmem, wu, inputs, albedo, n, out, list,
                        n_dev, c->d_status, tc_budget(c), c->tc_stall ? 1u : 0u, c->nrc_clamp ? 1u : 0u));
        return ARC_OK;
    }
    const uint32_t tiles = (n + 15u) / 16u;
    const uint32_t blocks = std::min<uint32_t>((tiles + 3u) / 4u, (uint32_t)c->n_sm * 3u);
    nrc::infer_kernel<<<blocks, 128, nrc::kFwdHalves * sizeof(__half), c->stream>>>(
        static_cast<const __half*>(c->d_nrc_w16_ema), inputs, albedo, n, out, list, n_dev, c->nrc_clamp ? 1u : 0u);
    NRC_CK(cudaGetLastError());
    return ARC_OK;
}

// Loss-scaled gradient of one batch added to d_nrc_grad (which the previous Adam step, or the
// gradient query, left at zero); with want_loss the batch loss sum goes to d_nrc_loss.
int launch_grad(arc_ctx* c, const float* inputs, const float* targets, uint32_t n, const uint32_t* gate,
                bool want_loss = false) {
    float* loss = want_loss ? c->d_nrc_loss : nullptr;
    if (want_loss) NRC_CK(cudaMemsetAsync(c->d_nrc_loss, 0, sizeof(float), c->stream));
    if (c->nrc_train_path == 1) {
        const uint32_t blocks = std::min<uint32_t>((n + 127u) / 128u, (uint32_t)c->n_sm);
        NRC_CK(arc_launch_overlapped(c, nrc::train_tc_kernel, dim3(blocks), dim3(128), nrc::kTtSmem, static_cast<const __half*>(c->d_nrc_wu),
                        inputs, targets, n, 1.0f / (float)n, c->d_nrc_grad, loss, gate, c->d_status, tc_budget(c),
                        c->tc_stall ? 1u : 0u));
        return ARC_OK;
    }
    const uint32_t tiles = (n + 63u) / 64u;
    const uint32_t blocks = std::min<uint32_t>(tiles, (uint32_t)c->n_sm);
    nrc::train_kernel<<<blocks, 128, (nrc::kAllHalves + nrc::kActHalves) * sizeof(__half), c->stream>>>(
        static_cast<const __half*>(c->d_nrc_w16), inputs, targets, n, 1.0f / (float)n, c->d_nrc_grad, loss, gate);
    NRC_CK(cudaGetLastError());
    return ARC_OK;
}

// Decay of the weight average at Adam step k (counted from the last init / set_weights): the set decay,
// or during a warm-up of w steps min(decay, (1 + k) / (w + k)), so the average follows the early
// training instead of keeping the initial weights' share (at decay 0.99 they still weigh 30 % after
// 120 steps). The warm-up is off by default.
float ema_decay_at(const arc_ctx* c, uint32_t k) {
    if (c->nrc_ema_warmup == 0u) return c->nrc_ema_decay;
    return std::min(c->nrc_ema_decay, (1.0f + (float)k) / ((float)c->nrc_ema_warmup + (float)k));
}

// One Adam step from d_nrc_grad; the host step counter sets the bias correction.
int launch_adam(arc_ctx* c, float lr, const uint32_t* gate) {
    c->nrc_step += 1;
    const float c1 = 1.0f - std::pow(c->nrc_beta1, (float)c->nrc_step), c2 = 1.0f - std::pow(c->nrc_beta2, (float)c->nrc_step);
    NRC_CK(arc_launch_overlapped(c, nrc::adam_kernel, dim3((nrc::kParams + 255) / 256), dim3(256), 0, c->d_nrc_w32, c->d_nrc_m,
                    c->d_nrc_v, c->d_nrc_grad, static_cast<__half*>(c->d_nrc_w16), c->d_nrc_ema,
                    static_cast<__half*>(c->d_nrc_w16_ema), static_cast<__half*>(c->d_nrc_wu),
                    static_cast<__half*>(c->d_nrc_wu_ema), ema_decay_at(c, c->nrc_step), lr, c1, c2,
                    1.0f / nrc::kLossScale, gate, c->nrc_beta1, c->nrc_beta2));
    return ARC_OK;
}

}  // namespace

// One training frame: samples from the hit list, then `steps` Adam steps (join_side: the context's
// stream waits for the side-stream query before the first step).
static int train_frame(arc_ctx* c, const uint32_t* list, const uint64_t* n_valid, const float* pos, const float* normal,
                       const float* nrc_in, uint32_t seed, uint32_t n_samples, uint32_t steps, float lr, bool join_side);

extern "C" {

int arc_nrc_init(arc_ctx* c, uint32_t seed) {
    if (!c) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    std::vector<float> w(nrc::kParams);
    init_weights(w, seed);
    return arc_nrc_set_weights(c, w.data());
}

int arc_nrc_set_weights(arc_ctx* c, const float* w) {
    if (!c || !w) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    NRC_CK(cudaMemcpyAsync(c->d_nrc_w32, w, sizeof(float) * nrc::kParams, cudaMemcpyHostToDevice, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_m, 0, sizeof(float) * nrc::kParams * 2, c->stream));
    nrc::pack_kernel<<<(nrc::kParams + 255) / 256, 256, 0, c->stream>>>(c->d_nrc_w32, static_cast<__half*>(c->d_nrc_w16),
                                                                       c->d_nrc_ema, static_cast<__half*>(c->d_nrc_w16_ema),
                                                                       static_cast<__half*>(c->d_nrc_wu),
                                                                       static_cast<__half*>(c->d_nrc_wu_ema));
    NRC_CK(cudaGetLastError());
    c->nrc_step = 0;
    return arc_ctx_finish(c);
}

int arc_nrc_get_weights(arc_ctx* c, float* w) {
    if (!c || !w) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    NRC_CK(cudaMemcpyAsync(w, c->d_nrc_w32, sizeof(float) * nrc::kParams, cudaMemcpyDeviceToHost, c->stream));
    return arc_ctx_finish(c);
}

int arc_nrc_get_ema_weights(arc_ctx* c, float* w) {
    if (!c || !w) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    NRC_CK(cudaMemcpyAsync(w, c->d_nrc_ema, sizeof(float) * nrc::kParams, cudaMemcpyDeviceToHost, c->stream));
    return arc_ctx_finish(c);
}

int arc_nrc_set_infer_path(arc_ctx* c, int path) {
    if (!c || path < 0 || path > 3) return ARC_E_INVALID_ARG;
    c->nrc_infer_path = path;
    return ARC_OK;
}

int arc_nrc_set_train_path(arc_ctx* c, int path) {
    if (!c || (path != 0 && path != 1)) return ARC_E_INVALID_ARG;
    c->nrc_train_path = path;
    return ARC_OK;
}

int arc_nrc_set_ema_decay(arc_ctx* c, float decay) {
    if (!c) return ARC_E_INVALID_ARG;
    if (!(decay >= 0.0f && decay < 1.0f)) {
        c->err = "EMA decay must lie in [0, 1)";
        return ARC_E_INVALID_ARG;
    }
    c->nrc_ema_decay = decay;
    return ARC_OK;
}

int arc_nrc_set_adam_betas(arc_ctx* c, float beta1, float beta2) {
    if (!c) return ARC_E_INVALID_ARG;
    if (!(beta1 >= 0.0f && beta1 < 1.0f && beta2 >= 0.0f && beta2 < 1.0f)) {
        c->err = "Adam betas must lie in [0, 1)";
        return ARC_E_INVALID_ARG;
    }
    c->nrc_beta1 = beta1;
    c->nrc_beta2 = beta2;
    return ARC_OK;
}

int arc_set_cache_launch_overlap(arc_ctx* c, int on) {
    if (!c) return ARC_E_INVALID_ARG;
    c->cache_pdl = on != 0;
    return ARC_OK;
}

int arc_nrc_set_sample_cluster(arc_ctx* c, uint32_t k) {
    if (!c) return ARC_E_INVALID_ARG;
    if (k == 0u || k > 32u || (k & (k - 1u))) {
        c->err = "sample cluster must be 1, 2, 4, 8, 16 or 32";
        return ARC_E_INVALID_ARG;
    }
    c->nrc_sample_cluster = k;
    return ARC_OK;
}

int arc_nrc_set_output_clamp(arc_ctx* c, int on) {
    if (!c) return ARC_E_INVALID_ARG;
    c->nrc_clamp = on != 0;
    return ARC_OK;
}

int arc_nrc_set_ema_warmup(arc_ctx* c, uint32_t steps) {
    if (!c) return ARC_E_INVALID_ARG;
    c->nrc_ema_warmup = steps;
    return ARC_OK;
}

int arc_nrc_query_dev(arc_ctx* c, const float* inputs, const float* albedo, uint32_t n, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (n && (!inputs || !out)) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    int rc = ensure_nrc(c);
    if (rc || n == 0) return rc;
    return launch_infer(c, inputs, albedo, n, out, nullptr, nullptr);
}

int arc_nrc_query_list_dev(arc_ctx* c, const uint32_t* list, const uint64_t* n_dev, uint32_t max_n, const float* inputs,
                           const float* albedo, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (max_n && (!list || !n_dev || !inputs || !out)) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    int rc = ensure_nrc(c);
    if (rc || max_n == 0) return rc;
    return launch_infer(c, inputs, albedo, max_n, out, list, reinterpret_cast<const unsigned long long*>(n_dev));
}

int arc_nrc_grad_dev(arc_ctx* c, const float* inputs, const float* targets, uint32_t n, float* grad_out) {
    if (!c || !inputs || !targets || n == 0) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    if ((rc = launch_grad(c, inputs, targets, n, nullptr, true))) return rc;
    if (grad_out)
        NRC_CK(cudaMemcpyAsync(grad_out, c->d_nrc_grad, sizeof(float) * nrc::kParams, cudaMemcpyDeviceToDevice, c->stream));
    NRC_CK(cudaMemsetAsync(c->d_nrc_grad, 0, sizeof(float) * nrc::kParams, c->stream));  // no step consumes it
    return ARC_OK;
}

int arc_nrc_train_step_dev(arc_ctx* c, const float* inputs, const float* targets, uint32_t n, float lr, float* loss_host) {
    if (!c || !inputs || !targets || n == 0) return ARC_E_INVALID_ARG;
    int rc = ensure_nrc(c);
    if (rc) return rc;
    if ((rc = launch_grad(c, inputs, targets, n, nullptr, loss_host != nullptr)) || (rc = launch_adam(c, lr, nullptr))) return rc;
    if (loss_host) {
        float l = 0.0f;
        NRC_CK(cudaMemcpyAsync(&l, c->d_nrc_loss, sizeof(float), cudaMemcpyDeviceToHost, c->stream));
        if ((rc = arc_ctx_finish(c))) return rc;
        *loss_host = l / (float)n;
    }
    return ARC_OK;
}

// Host-buffer forms of the query and the training step: inputs staged to the device, results copied
// back before the call returns.
int arc_nrc_query(arc_ctx* c, const float* inputs, const float* albedo, uint32_t n, float* out) {
    if (!c) return ARC_E_INVALID_ARG;
    if (n == 0) return ARC_OK;
    if (!inputs || !out) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    void* stage;
    int rc = arc_ctx_stage(c, (size_t)n * 60u, &stage);
    if (rc) return rc;
    float* d_in = static_cast<float*>(stage);
    float* d_out = d_in + 9u * (size_t)n;
    float* d_alb = albedo ? d_out + 3u * (size_t)n : nullptr;
    NRC_CK(cudaMemcpyAsync(d_in, inputs, (size_t)n * 36u, cudaMemcpyHostToDevice, c->stream));
    if (albedo) NRC_CK(cudaMemcpyAsync(d_alb, albedo, (size_t)n * 12u, cudaMemcpyHostToDevice, c->stream));
    if ((rc = arc_nrc_query_dev(c, d_in, d_alb, n, d_out))) return rc;
    NRC_CK(cudaMemcpyAsync(out, d_out, (size_t)n * 12u, cudaMemcpyDeviceToHost, c->stream));
    return arc_ctx_finish(c);
}

int arc_nrc_train_step(arc_ctx* c, const float* inputs, const float* targets, uint32_t n, float lr, float* loss_host) {
    if (!c) return ARC_E_INVALID_ARG;
    if (n == 0) return ARC_OK;
    if (!inputs || !targets) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    void* stage;
    int rc = arc_ctx_stage(c, (size_t)n * 48u, &stage);
    if (rc) return rc;
    float* d_in = static_cast<float*>(stage);
    float* d_t = d_in + 9u * (size_t)n;
    NRC_CK(cudaMemcpyAsync(d_in, inputs, (size_t)n * 36u, cudaMemcpyHostToDevice, c->stream));
    NRC_CK(cudaMemcpyAsync(d_t, targets, (size_t)n * 12u, cudaMemcpyHostToDevice, c->stream));
    if ((rc = arc_nrc_train_step_dev(c, d_in, d_t, n, lr, loss_host))) return rc;
    return arc_ctx_finish(c);
}

int arc_nrc_frame_dev(arc_ctx* c, const uint32_t* list, const uint64_t* n_valid, uint32_t max_n, const float* pos,
                      const float* normal, const float* nrc_in, const float* albedo, float* out_rgb, uint32_t seed,
                      uint32_t n_samples, uint32_t steps, float lr) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!list || !n_valid || !pos || !normal || !nrc_in || !out_rgb) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (steps == 0 || n_samples < steps || n_samples % steps)
        return nrc_err(c, ARC_E_INVALID_ARG, "n_samples must be a non-zero multiple of steps");
    if ((rc = ensure_nrc(c))) return rc;
    // the query reads the weights the previous frame's last step left; it runs beside the sample
    // generation and ends before this frame's first Adam step rewrites them
    if ((rc = arc_ctx_side_begin(c))) return rc;
    rc = max_n ? launch_infer(c, nrc_in, albedo, max_n, out_rgb, list, reinterpret_cast<const unsigned long long*>(n_valid), true)
               : ARC_OK;
    int rc2 = arc_ctx_side_end(c);
    if (rc || (rc = rc2)) return rc;
    return train_frame(c, list, n_valid, pos, normal, nrc_in, seed, n_samples, steps, lr, true);
}

int arc_nrc_train_frame_dev(arc_ctx* c, const uint32_t* list, const uint64_t* n_valid, const float* pos,
                            const float* normal, const float* nrc_in, uint32_t seed, uint32_t n_samples,
                            uint32_t steps, float lr) {
    return train_frame(c, list, n_valid, pos, normal, nrc_in, seed, n_samples, steps, lr, false);
}

}  // extern "C"

static int train_frame(arc_ctx* c, const uint32_t* list, const uint64_t* n_valid, const float* pos, const float* normal,
                       const float* nrc_in, uint32_t seed, uint32_t n_samples, uint32_t steps, float lr, bool join_side) {
    int rc = arc_ctx_check_ready(c, true);
    if (rc) return rc;
    if (!list || !n_valid || !pos || !normal || !nrc_in) return nrc_err(c, ARC_E_INVALID_ARG, "null buffer");
    if (steps == 0 || n_samples < steps || n_samples % steps)
        return nrc_err(c, ARC_E_INVALID_ARG, "n_samples must be a non-zero multiple of steps");
    if ((rc = ensure_nrc(c))) return rc;
    if (c->nrc_batch_cap < n_samples) {
        cudaFree(c->d_nrc_batch);
        c->d_nrc_batch = nullptr;
        c->nrc_batch_cap = 0;
        NRC_CK(cudaMalloc((void**)&c->d_nrc_batch, sizeof(float) * 12u * (size_t)n_samples));
        c->nrc_batch_cap = n_samples;
    }
    if (!c->d_nrc_gate) NRC_CK(cudaMalloc((void**)&c->d_nrc_gate, sizeof(uint32_t)));
    float* train_in = c->d_nrc_batch;
    float* train_t = c->d_nrc_batch + 9u * (size_t)n_samples;
    if ((rc = arc_launch_train_samples_list(c, list, reinterpret_cast<const unsigned long long*>(n_valid), pos, normal,
                                            nrc_in, seed, n_samples, steps, train_in, train_t, c->d_nrc_gate)))
        return rc;
    if (join_side && (rc = arc_ctx_side_join(c))) return rc;
    const uint32_t per = n_samples / steps;
    for (uint32_t k = 0; k < steps; ++k) {
        if ((rc = launch_grad(c, train_in + 9u * (size_t)k * per, train_t + 3u * (size_t)k * per, per, c->d_nrc_gate)) ||
            (rc = launch_adam(c, lr, c->d_nrc_gate)))
            return rc;
    }
    return ARC_OK;
}
