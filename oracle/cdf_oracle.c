/*
 * cdf_oracle.c — CPU restatement of the learned CDF model used by the GPU
 * learned partition (no counterpart in the reference crate).
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward kernels
 * (gradients compared within a relative 1e-4) and for the model's
 * predictions.  The product never links or calls it.
 *
 * Model: a 2-layer MLP, 2 inputs -> 64 ReLU units -> 1 output, predicting
 * the rank fraction (CDF) of a suffix from its 64-bit packed prefix.
 * Inputs: f0 = hi32 * 2^-31 - 1 and f1 = lo32 * 2^-31 - 1 (the prefix's
 * high and low 32-bit halves mapped to [-1, 1)), each computed in float with
 * the same IEEE operations as the GPU.  Parameters (257 floats): w1[h*2+d],
 * b1[h], w2[h], b2.  Loss: mean squared error over the batch.
 * Gradients here are accumulated in double.
 */
#include <math.h>
#include <stdint.h>

#include "capssa_oracle.h"

#define H OR_CDF_HIDDEN

void or_cdf_features(uint64_t prefix, float f[2]) {
    const float s = 0x1p-31f;
    float t0 = (float)(uint32_t)(prefix >> 32) * s;
    float t1 = (float)(uint32_t)(prefix & 0xFFFFFFFFu) * s;
    f[0] = t0 - 1.0f;
    f[1] = t1 - 1.0f;
}

double or_cdf_forward(const float *params, uint64_t prefix) {
    const float *w1 = params, *b1 = params + 2 * H, *w2 = params + 3 * H, *b2 = params + 4 * H;
    float f[2];
    or_cdf_features(prefix, f);
    double y = b2[0];
    for (int h = 0; h < H; h++) {
        double z = (double)w1[2 * h] * f[0] + (double)w1[2 * h + 1] * f[1] + b1[h];
        if (z > 0) y += (double)w2[h] * z;
    }
    return y;
}

double or_cdf_loss_grad(const float *params, const uint64_t *prefix, const float *target,
                        uint64_t n, double *grad) {
    const float *w1 = params, *b1 = params + 2 * H, *w2 = params + 3 * H, *b2 = params + 4 * H;
    for (int i = 0; i < OR_CDF_PARAMS; i++) grad[i] = 0;
    double loss = 0;
    for (uint64_t i = 0; i < n; i++) {
        float f[2];
        or_cdf_features(prefix[i], f);
        double z[H], y = b2[0];
        for (int h = 0; h < H; h++) {
            z[h] = (double)w1[2 * h] * f[0] + (double)w1[2 * h + 1] * f[1] + b1[h];
            if (z[h] > 0) y += (double)w2[h] * z[h];
        }
        double e = y - target[i];
        loss += e * e;
        double dy = 2.0 * e / (double)n;
        for (int h = 0; h < H; h++) {
            if (z[h] > 0) {
                double dz = dy * w2[h];
                grad[3 * H + h] += dy * z[h];
                grad[2 * H + h] += dz;
                grad[2 * h] += dz * f[0];
                grad[2 * h + 1] += dz * f[1];
            }
        }
        grad[4 * H] += dy;
    }
    return n ? loss / (double)n : 0.0;
}
