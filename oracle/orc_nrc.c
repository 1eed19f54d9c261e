/*
 * orc_nrc.c — FP64 reference of the neural radiance cache (no reference counterpart: the NRC is this
 * project's replacement for SHARC's hashed lookup at secondary hits).
 *
 * TEST INFRASTRUCTURE ONLY (see orc.h). The GPU kernels (arcadia_gb300/csrc/arc_nrc.cu) are checked
 * against these functions within stated tolerances.
 *
 * Network: 9 inputs (position normalised to [0,1]^3, normal, view direction) -> frequency encoding
 * sin/cos(2^k pi v), k = 0..11 (216 features, index = input*24 + 2k + {0 sin, 1 cos}) -> 5 hidden
 * layers of 64 with ReLU -> 3 outputs (linear). No biases. Weights are stored row-major per layer as
 * W[out][in]; the GPU keeps FP32 master weights and FP16 copies, activations in FP16 between layers,
 * FP32 accumulation. The reference here quantises weights, encoded features and hidden activations
 * to FP16 at the same points and accumulates in FP64.
 * Loss: relative L2, mean over the batch of sum_c (y_c - t_c)^2 / (sg(y_c)^2 + 0.01).
 * Optimiser: Adam (beta1 0.9, beta2 0.99, eps 1e-8), bias-corrected, on the FP32 master weights.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include "orc.h"
#include "orc_math.h"

#define NRC_IN 9
#define NRC_FREQS 12
#define NRC_ENC 216
#define NRC_W 64
#define NRC_OUT 3
#define NRC_LAYERS 6

static const int k_dims[NRC_LAYERS + 1] = {NRC_ENC, NRC_W, NRC_W, NRC_W, NRC_W, NRC_W, NRC_OUT};

uint32_t orc_nrc_param_count(void) {
    uint32_t n = 0;
    for (int l = 0; l < NRC_LAYERS; ++l) n += (uint32_t)(k_dims[l] * k_dims[l + 1]);
    return n;
}

static double q16(double v) { return (double)orc_f16_to_f32(orc_f32_to_f16((float)v)); }

void orc_nrc_encode(const float in[NRC_IN], double out[NRC_ENC]) {
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < NRC_IN; ++i)
        for (int k = 0; k < NRC_FREQS; ++k) {
            double a = pi * ldexp((double)in[i], k);
            out[i * 24 + 2 * k] = sin(a);
            out[i * 24 + 2 * k + 1] = cos(a);
        }
}

/* Forward pass of n queries; acts (optional) receives per-layer FP16-quantised activations
 * (layer 0 = encoding, n x 216; layers 1..5 = hidden, n x 64) laid out layer after layer. */
void orc_nrc_forward(const float* weights, const float* inputs, uint32_t n, double* outputs, double* acts) {
    double a[NRC_ENC], b[NRC_ENC];
    size_t act_off[NRC_LAYERS];
    size_t off = 0;
    for (int l = 0; l < NRC_LAYERS; ++l) {
        act_off[l] = off;
        off += (size_t)n * k_dims[l];
    }
    for (uint32_t q = 0; q < n; ++q) {
        orc_nrc_encode(&inputs[9 * q], a);
        for (int i = 0; i < NRC_ENC; ++i) a[i] = q16(a[i]);
        const float* W = weights;
        for (int l = 0; l < NRC_LAYERS; ++l) {
            const int din = k_dims[l], dout = k_dims[l + 1];
            if (acts) memcpy(&acts[act_off[l] + (size_t)q * din], a, sizeof(double) * din);
            for (int o = 0; o < dout; ++o) {
                double s = 0.0;
                for (int i = 0; i < din; ++i) s += q16(W[o * din + i]) * a[i];
                b[o] = s;
            }
            W += din * dout;
            if (l < NRC_LAYERS - 1)
                for (int o = 0; o < dout; ++o) b[o] = q16(b[o] > 0.0 ? b[o] : 0.0);
            memcpy(a, b, sizeof(double) * dout);
        }
        for (int c = 0; c < NRC_OUT; ++c) outputs[3 * q + c] = a[c];
    }
}

/* Loss and weight gradient of one batch (mean relative L2). Returns the loss. */
double orc_nrc_grad(const float* weights, const float* inputs, const float* targets, uint32_t n, double* grad) {
    size_t total = 0;
    for (int l = 0; l < NRC_LAYERS; ++l) total += (size_t)n * k_dims[l];
    double* acts = (double*)malloc(sizeof(double) * total);
    double* out = (double*)malloc(sizeof(double) * 3 * n);
    orc_nrc_forward(weights, inputs, n, out, acts);
    uint32_t np = orc_nrc_param_count();
    memset(grad, 0, sizeof(double) * np);
    size_t w_off[NRC_LAYERS], act_off[NRC_LAYERS];
    size_t wo = 0, ao = 0;
    for (int l = 0; l < NRC_LAYERS; ++l) {
        w_off[l] = wo;
        wo += (size_t)k_dims[l] * k_dims[l + 1];
        act_off[l] = ao;
        ao += (size_t)n * k_dims[l];
    }
    double loss = 0.0;
    double d[NRC_ENC], dn[NRC_ENC];
    for (uint32_t q = 0; q < n; ++q) {
        for (int c = 0; c < NRC_OUT; ++c) {
            double y = out[3 * q + c], t = targets[3 * q + c];
            double den = y * y + 0.01;
            loss += (y - t) * (y - t) / den;
            d[c] = 2.0 * (y - t) / den / (double)n;
        }
        for (int l = NRC_LAYERS - 1; l >= 0; --l) {
            const int din = k_dims[l], dout = k_dims[l + 1];
            const double* a_in = &acts[act_off[l] + (size_t)q * din];
            double* g = &grad[w_off[l]];
            const float* W = &weights[w_off[l]];
            for (int o = 0; o < dout; ++o)
                for (int i = 0; i < din; ++i) g[o * din + i] += d[o] * a_in[i];
            if (l == 0) break;
            for (int i = 0; i < din; ++i) {
                double s = 0.0;
                for (int o = 0; o < dout; ++o) s += q16(W[o * din + i]) * d[o];
                dn[i] = a_in[i] > 0.0 ? s : 0.0; /* ReLU' of the layer that produced a_in */
            }
            memcpy(d, dn, sizeof(double) * din);
        }
    }
    free(acts);
    free(out);
    return loss / (double)n;
}

/* One Adam step on FP32 master weights (step t >= 1). */
void orc_nrc_adam(float* weights, float* m, float* v, const float* grad, uint32_t n_params, uint32_t t, float lr) {
    const float b1 = 0.9f, b2 = 0.99f, eps = 1e-8f;
    const float c1 = 1.0f - powf(b1, (float)t), c2 = 1.0f - powf(b2, (float)t);
    for (uint32_t i = 0; i < n_params; ++i) {
        m[i] = b1 * m[i] + (1.0f - b1) * grad[i];
        v[i] = b2 * v[i] + (1.0f - b2) * grad[i] * grad[i];
        const float mh = m[i] / c1, vh = v[i] / c2;
        weights[i] -= lr * mh / (sqrtf(vh) + eps);
    }
}
