// cdf.cuh — the learned CDF model of the learned partition: a 2-layer MLP
// (2 inputs -> 64 ReLU units -> 1 output) that maps a suffix's 64-bit packed
// prefix to its predicted rank fraction among the splitter sample, trained
// on the GPU by this file's own forward/backward and Adam kernels (FP32) and
// evaluated from BF16 weights.  No counterpart in the reference crate.
//
// Inputs: f0 = hi32 * 2^-31 - 1, f1 = lo32 * 2^-31 - 1 (the prefix's halves
// mapped to [-1, 1)).  Parameters (kCdfParams floats): w1[h*2+d], b1[h],
// w2[h], b2.  Loss: mean squared error against the targets.
#pragma once

#include <cuda_bf16.h>

#include "common.cuh"

namespace capssa {
namespace cdf {

constexpr int kHidden = 64;
constexpr int kParams = 4 * kHidden + 1;

__device__ __forceinline__ void features(uint64_t x, float &f0, float &f1) {
    const float s = 0x1p-31f;
    const float t0 = (float)(uint32_t)(x >> 32) * s;
    const float t1 = (float)(uint32_t)(x & 0xFFFFFFFFu) * s;
    f0 = t0 - 1.0f;
    f1 = t1 - 1.0f;
}

// Model output from BF16 weights (shared memory), FP32 arithmetic.
__device__ __forceinline__ float infer_bf16(const __nv_bfloat16 *w, uint64_t x) {
    float f0, f1;
    features(x, f0, f1);
    const __nv_bfloat16 *w1 = w, *b1 = w + 2 * kHidden, *w2 = w + 3 * kHidden;
    float y = __bfloat162float(w[4 * kHidden]);
#pragma unroll 16
    for (int h = 0; h < kHidden; h++) {
        const __nv_bfloat162 wp = *reinterpret_cast<const __nv_bfloat162 *>(w1 + 2 * h);
        const float z = fmaf(__low2float(wp), f0, fmaf(__high2float(wp), f1, __bfloat162float(b1[h])));
        y = fmaf(__bfloat162float(w2[h]), fmaxf(z, 0.0f), y);
    }
    return y;
}

// Mean-squared-error gradient over n samples, summed into grad (kParams,
// zeroed by the caller) and the loss sum into *loss.
capssa_status grad(Ctx &c, const float *params, const uint64_t *x, const float *t, uint32_t n,
                   float *grad, float *loss);

// Trains params (device, kParams floats; initialised here) on n (prefix,
// target) samples with `steps` full-batch Adam steps, replayed from a CUDA
// graph; writes the BF16 copy to w_bf16 (device, kParams) and returns the
// final mean loss in *final_loss.  knot_start (samples sorted by prefix):
// start from the piecewise-linear interpolant through 64 of the samples
// instead of evenly spread kinks.
capssa_status train(Ctx &c, const uint64_t *x, const float *t, uint32_t n, int steps,
                    float *params, __nv_bfloat16 *w_bf16, float *final_loss,
                    bool knot_start = false);

// Deterministic initial parameters: ReLU kinks evenly spread over f0.
void init_params(float *h_params);

}  // namespace cdf
}  // namespace capssa
