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

// Tensor-core inference for a whole warp: every lane passes its own prefix
// and gets the model's output for it.  Layer 1 is 2 x 8 mma.sync
// m16n8k16 (bf16 operands, fp32 accumulation) over 16-suffix row tiles;
// each input feature is split into a bf16 high part and the bf16 rounding
// of its remainder (two columns sharing the weight), so the inputs keep
// about 16 bits; the bias is a constant-one column.  Layer 2 (ReLU, then
// the dot with the output weights) runs in fp32 on the accumulators.  All
// 32 lanes must call it together.  B1/W2/b2 come from mma_weights.
struct MmaWeights {
    uint32_t b1[8];  // layer-1 B fragments, one per 8-unit tile of hidden units
    float w2[16];    // output weights of this lane's accumulator columns
    float b2;
};

__device__ __forceinline__ uint32_t pack_bf16(float lo_half, float hi_half) {
    // the first argument lands in the low 16 bits (lower column index)
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo_half, hi_half);
    return *reinterpret_cast<const uint32_t *>(&v);
}

// Fragments of this lane from the BF16 weights (shared memory): column k
// of layer 1 is f0 high, f0 low, f1 high, f1 low, one, then zeros.
__device__ __forceinline__ MmaWeights mma_weights(const __nv_bfloat16 *w) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    MmaWeights W;
#pragma unroll
    for (int t = 0; t < 8; t++) {
        const int h = 8 * t + g;
        float x0 = 0.0f, x1 = 0.0f;
        if (tig == 0) x0 = x1 = __bfloat162float(w[2 * h]);
        if (tig == 1) x0 = x1 = __bfloat162float(w[2 * h + 1]);
        if (tig == 2) x0 = __bfloat162float(w[2 * kHidden + h]);
        W.b1[t] = pack_bf16(x0, x1);
        W.w2[2 * t] = __bfloat162float(w[3 * kHidden + 8 * t + 2 * tig]);
        W.w2[2 * t + 1] = __bfloat162float(w[3 * kHidden + 8 * t + 2 * tig + 1]);
    }
    W.b2 = __bfloat162float(w[4 * kHidden]);
    return W;
}

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], uint32_t a0, uint32_t a1,
                                               uint32_t b0) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
        "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%10,%11,%12,%13};\n"
        : "=f"(d[0]), "=f"(d[1]), "=f"(d[2]), "=f"(d[3])
        : "r"(a0), "r"(a1), "r"(0u), "r"(0u), "r"(b0), "r"(0u), "f"(0.0f), "f"(0.0f),
          "f"(0.0f), "f"(0.0f));
}

__device__ __forceinline__ float infer_mma(const MmaWeights &W, uint64_t x) {
    const int lane = threadIdx.x & 31, g = lane >> 2, tig = lane & 3;
    float f0, f1;
    features(x, f0, f1);
    float acc[2][2];
#pragma unroll
    for (int m = 0; m < 2; m++) {
        uint32_t a[2];
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int src = 16 * m + g + 8 * half;
            const float s0 = __shfl_sync(0xffffffffu, f0, src);
            const float s1 = __shfl_sync(0xffffffffu, f1, src);
            const float v = tig == 0 ? s0 : s1;
            const float hi = __bfloat162float(__float2bfloat16_rn(v));
            a[half] = tig < 2 ? pack_bf16(hi, v - hi) : (tig == 2 ? pack_bf16(1.0f, 0.0f) : 0u);
        }
        float r0 = 0.0f, r1 = 0.0f;
#pragma unroll
        for (int t = 0; t < 8; t++) {
            float d[4];
            mma_bf16_16816(d, a[0], a[1], W.b1[t]);
            r0 = fmaf(W.w2[2 * t], fmaxf(d[0], 0.0f), r0);
            r0 = fmaf(W.w2[2 * t + 1], fmaxf(d[1], 0.0f), r0);
            r1 = fmaf(W.w2[2 * t], fmaxf(d[2], 0.0f), r1);
            r1 = fmaf(W.w2[2 * t + 1], fmaxf(d[3], 0.0f), r1);
        }
        r0 += __shfl_xor_sync(0xffffffffu, r0, 1);
        r0 += __shfl_xor_sync(0xffffffffu, r0, 2);
        r1 += __shfl_xor_sync(0xffffffffu, r1, 1);
        r1 += __shfl_xor_sync(0xffffffffu, r1, 2);
        acc[m][0] = r0;
        acc[m][1] = r1;
    }
    // this lane's suffix is row (lane & 15) of tile lane >> 4
    const int r = lane & 15, src = 4 * (r & 7);
    const float v00 = __shfl_sync(0xffffffffu, acc[0][0], src);
    const float v01 = __shfl_sync(0xffffffffu, acc[0][1], src);
    const float v10 = __shfl_sync(0xffffffffu, acc[1][0], src);
    const float v11 = __shfl_sync(0xffffffffu, acc[1][1], src);
    const float v = lane < 16 ? (r < 8 ? v00 : v01) : (r < 8 ? v10 : v11);
    return W.b2 + v;
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

// The model's output for n prefixes as the learned partition evaluates it:
// the FP32 parameters (device) rounded to BF16, then infer_mma.
capssa_status infer(Ctx &c, const float *params, const uint64_t *x, uint32_t n, float *y);

// Deterministic initial parameters: ReLU kinks evenly spread over f0.
void init_params(float *h_params);

}  // namespace cdf
}  // namespace capssa
