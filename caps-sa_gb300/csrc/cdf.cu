// cdf.cu — training kernels of the learned CDF model (see cdf.cuh).
#include <cmath>
#include <vector>

#include "cdf.cuh"

namespace capssa {
namespace cdf {

namespace {

constexpr int kGradThreads = 256;
constexpr int kGradBlocks = 304;  // two per SM

// One warp handles 32 samples at a time (a lane each); for every hidden
// unit the four per-unit gradient terms are summed over the warp with
// butterflies and added to the block's shared accumulator, which the block
// adds to the global gradient once.
__global__ void __launch_bounds__(kGradThreads)
    grad_kernel(const float *__restrict__ params, const uint64_t *__restrict__ x,
                const float *__restrict__ t, uint32_t n, float *__restrict__ grad,
                float *__restrict__ loss) {
    __shared__ float sp[kParams];
    __shared__ float sg[kParams + 1];  // + loss
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        sp[i] = params[i];
        sg[i] = 0.0f;
    }
    if (threadIdx.x == 0) sg[kParams] = 0.0f;
    __syncthreads();
    const float *w1 = sp, *b1 = sp + 2 * kHidden, *w2 = sp + 3 * kHidden;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    const float inv_n = 1.0f / (float)n;
    // lane h & 31 keeps the sums of hidden units h and h + 32 in registers
    float a2[2] = {0.0f, 0.0f}, ab[2] = {0.0f, 0.0f}, a0[2] = {0.0f, 0.0f}, a1[2] = {0.0f, 0.0f};
    float aloss = 0.0f, adsum = 0.0f;
    for (uint32_t base = warp * 32; base < n; base += nwarps * 32) {
        const uint32_t i = base + lane;
        const bool valid = i < n;
        float f0 = 0.0f, f1 = 0.0f, tg = 0.0f;
        if (valid) {
            features(x[i], f0, f1);
            tg = t[i];
        }
        float y = sp[4 * kHidden];
#pragma unroll 4
        for (int h = 0; h < kHidden; h++) {
            const float z = fmaf(w1[2 * h], f0, fmaf(w1[2 * h + 1], f1, b1[h]));
            y = fmaf(w2[h], fmaxf(z, 0.0f), y);
        }
        const float e = valid ? y - tg : 0.0f;
        const float dy = 2.0f * e * inv_n;
        float le = e * e, dsum = dy;
#pragma unroll 2
        for (int h = 0; h < kHidden; h++) {
            const float z = fmaf(w1[2 * h], f0, fmaf(w1[2 * h + 1], f1, b1[h]));
            const bool on = z > 0.0f;
            float gw2 = on ? dy * z : 0.0f;
            float gb1 = on ? dy * w2[h] : 0.0f;
            float gw0 = gb1 * f0, gw1 = gb1 * f1;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                gw2 += __shfl_xor_sync(0xffffffffu, gw2, o);
                gb1 += __shfl_xor_sync(0xffffffffu, gb1, o);
                gw0 += __shfl_xor_sync(0xffffffffu, gw0, o);
                gw1 += __shfl_xor_sync(0xffffffffu, gw1, o);
            }
            if (lane == (h & 31)) {
                if (h < 32) {
                    a2[0] += gw2;
                    ab[0] += gb1;
                    a0[0] += gw0;
                    a1[0] += gw1;
                } else {
                    a2[1] += gw2;
                    ab[1] += gb1;
                    a0[1] += gw0;
                    a1[1] += gw1;
                }
            }
        }
        aloss += le;
        adsum += dsum;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        aloss += __shfl_xor_sync(0xffffffffu, aloss, o);
        adsum += __shfl_xor_sync(0xffffffffu, adsum, o);
    }
#pragma unroll
    for (int q = 0; q < 2; q++) {
        const int h = lane + 32 * q;
        atomicAdd(&sg[3 * kHidden + h], a2[q]);
        atomicAdd(&sg[2 * kHidden + h], ab[q]);
        atomicAdd(&sg[2 * h], a0[q]);
        atomicAdd(&sg[2 * h + 1], a1[q]);
    }
    if (lane == 0) {
        atomicAdd(&sg[4 * kHidden], adsum);
        atomicAdd(&sg[kParams], aloss);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
        if (sg[i] != 0.0f) atomicAdd(&grad[i], sg[i]);
    if (threadIdx.x == 0) atomicAdd(loss, sg[kParams]);
}

// One Adam step (bias-corrected), then the gradient and loss are cleared for
// the next step; the step's mean loss is kept in loss_out.
__global__ void adam_kernel(float *__restrict__ params, float *__restrict__ grad,
                            float *__restrict__ m, float *__restrict__ v, int *__restrict__ step,
                            float lr, float *__restrict__ loss, float *__restrict__ loss_out,
                            uint32_t n) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int tstep = *step + 1;
    const float c1 = 1.0f - powf(b1, (float)tstep), c2 = 1.0f - powf(b2, (float)tstep);
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) {
        const float g = grad[i];
        const float mi = b1 * m[i] + (1.0f - b1) * g;
        const float vi = b2 * v[i] + (1.0f - b2) * g * g;
        m[i] = mi;
        v[i] = vi;
        params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        grad[i] = 0.0f;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        *loss_out = *loss / (float)n;
        *loss = 0.0f;
        *step = tstep;
    }
}

__global__ void to_bf16_kernel(const float *__restrict__ params, __nv_bfloat16 *__restrict__ w) {
    for (int i = threadIdx.x; i < kParams; i += blockDim.x) w[i] = __float2bfloat16(params[i]);
}

// Data-dependent start for n samples sorted by prefix: the ReLU kinks sit on
// f0 at 64 evenly spaced samples, and the output weights make the model the
// piecewise-linear interpolant of the targets through those samples (flat
// before the first and after the last); coinciding kinks get no slope.
// Training then only has to refine it.
__global__ void knot_init_kernel(const uint64_t *__restrict__ x, const float *__restrict__ t,
                                 uint32_t n, float *__restrict__ params) {
    __shared__ float c[kHidden], y[kHidden], m[kHidden];
    const int h = threadIdx.x;
    if (h < kHidden) {
        const uint32_t i = (uint32_t)(((uint64_t)h * (n - 1)) / (kHidden - 1));
        float f0, f1;
        features(x[i], f0, f1);
        c[h] = f0;
        y[h] = t[i];
    }
    __syncthreads();
    if (h < kHidden) {  // slope of the segment after kink h (0 after the last)
        const float dx = h + 1 < kHidden ? c[h + 1] - c[h] : 0.0f;
        m[h] = dx > 1e-6f ? (y[h + 1] - y[h]) / dx : 0.0f;
    }
    __syncthreads();
    if (h < kHidden) {
        params[2 * h] = 1.0f;
        params[2 * h + 1] = 0.0f;
        params[2 * kHidden + h] = -c[h];
        params[3 * kHidden + h] = m[h] - (h > 0 ? m[h - 1] : 0.0f);
        if (h == 0) params[4 * kHidden] = y[0];
    }
}

// Workspace of one training: grad, m, v (kParams each), loss, loss_out, step.
struct TrainState {
    float *grad, *m, *v, *loss, *loss_out;
    int *step;
};

// Tensor-core inference (infer_mma) of n prefixes from BF16 weights:
// whole warps step together, lanes past the end repeat the last prefix.
__global__ void __launch_bounds__(256)
    infer_kernel(const __nv_bfloat16 *__restrict__ w, const uint64_t *__restrict__ x, uint32_t n,
                 float *__restrict__ y) {
    __shared__ __nv_bfloat16 sw[kParams + 1];
    for (int j = threadIdx.x; j < kParams; j += blockDim.x) sw[j] = w[j];
    __syncthreads();
    const MmaWeights W = mma_weights(sw);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        const float v = infer_mma(W, x[i < n ? i : n - 1]);
        if (i < n) y[i] = v;
    }
}

}  // namespace

capssa_status infer(Ctx &c, const float *params, const uint64_t *x, uint32_t n, float *y) {
    if (n == 0) return CAPSSA_OK;
    __nv_bfloat16 *wb = (__nv_bfloat16 *)ws_get(c, WS_CDF, (size_t)(4 * kParams + 16) * 4);
    if (!wb) return set_err(c, CAPSSA_ENOMEM, "model weights");
    to_bf16_kernel<<<1, 320, 0, c.stream>>>(params, wb);
    CAPSSA_LAUNCHED(c);
    infer_kernel<<<std::min<unsigned>((n + 255) / 256, (unsigned)c.sm_count * 8), 256, 0,
                   c.stream>>>(wb, x, n, y);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

void init_params(float *p) {
    for (int h = 0; h < kHidden; h++) {
        const float c = -1.0f + (2.0f * h + 1.0f) / kHidden;  // kink position on f0
        p[2 * h] = 1.0f;
        p[2 * h + 1] = 0.0f;
        p[2 * kHidden + h] = -c;
        p[3 * kHidden + h] = h == 0 ? 0.5f : 0.0f;
    }
    p[4 * kHidden] = 0.0f;
}

capssa_status grad(Ctx &c, const float *params, const uint64_t *x, const float *t, uint32_t n,
                   float *g, float *loss) {
    if (n == 0) return CAPSSA_OK;
    const unsigned blocks = std::min<unsigned>(kGradBlocks, (n + kGradThreads - 1) / kGradThreads);
    grad_kernel<<<blocks, kGradThreads, 0, c.stream>>>(params, x, t, n, g, loss);
    CAPSSA_LAUNCHED(c);
    return CAPSSA_OK;
}

capssa_status train(Ctx &c, const uint64_t *x, const float *t, uint32_t n, int steps,
                    float *params, __nv_bfloat16 *w_bf16, float *final_loss, bool knot_start) {
    std::vector<float> h(kParams);
    init_params(h.data());
    float *st = (float *)ws_get(c, WS_CDF, (size_t)(4 * kParams + 16) * 4);
    if (!st) return set_err(c, CAPSSA_ENOMEM, "model training state");
    TrainState S{st, st + kParams, st + 2 * kParams, st + 3 * kParams, st + 3 * kParams + 1,
                 (int *)(st + 3 * kParams + 2)};
    CAPSSA_CUDA(c, cudaMemcpyAsync(params, h.data(), kParams * 4, cudaMemcpyHostToDevice,
                                   c.stream));
    CAPSSA_CUDA(c, cudaMemsetAsync(st, 0, (size_t)(4 * kParams + 16) * 4, c.stream));
    CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));  // h goes out of scope
    if (n == 0) return CAPSSA_OK;
    if (knot_start && n >= 2) {
        knot_init_kernel<<<1, kHidden, 0, c.stream>>>(x, t, n, params);
        CAPSSA_LAUNCHED(c);
    }
    const unsigned blocks = std::min<unsigned>(kGradBlocks, (n + kGradThreads - 1) / kGradThreads);
    auto step_launch = [&](int s) {
        // from the interpolating start only small steps refine the fit
        const float lr0 = knot_start ? 2e-4f : 1e-2f;
        const float lr = s < steps * 3 / 4 ? lr0 : lr0 * 0.2f;
        grad_kernel<<<blocks, kGradThreads, 0, c.stream>>>(params, x, t, n, S.grad, S.loss);
        adam_kernel<<<1, 320, 0, c.stream>>>(params, S.grad, S.m, S.v, S.step, lr, S.loss,
                                             S.loss_out, n);
    };
    float hl = 0.0f;
    if (c.stream == nullptr) {
        // the legacy default stream cannot be captured: plain launches
        for (int s = 0; s < steps; s++) step_launch(s);
        c.launches += 2ull * (uint64_t)steps;
        to_bf16_kernel<<<1, 320, 0, c.stream>>>(params, w_bf16);
        CAPSSA_LAUNCHED(c);
        CAPSSA_CUDA(c, cudaMemcpyAsync(&hl, S.loss_out, 4, cudaMemcpyDeviceToHost, c.stream));
        CAPSSA_CUDA(c, cudaStreamSynchronize(c.stream));
        *final_loss = hl;
        return CAPSSA_OK;
    }
    // the whole step loop is one graph: captured on the context's stream,
    // replayed once
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    CAPSSA_CUDA(c, cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
    for (int s = 0; s < steps; s++) step_launch(s);
    cudaError_t e = cudaStreamEndCapture(c.stream, &graph);
    if (e != cudaSuccess) return cuda_err(c, e, "capture of the training loop");
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_err(c, e, "instantiating the training graph");
    }
    e = cudaGraphLaunch(exec, c.stream);
    c.launches += 2ull * (uint64_t)steps;
    to_bf16_kernel<<<1, 320, 0, c.stream>>>(params, w_bf16);
    CAPSSA_LAUNCHED(c);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&hl, S.loss_out, 4, cudaMemcpyDeviceToHost, c.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c.stream);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_err(c, e, "training graph");
    *final_loss = hl;
    return CAPSSA_OK;
}

}  // namespace cdf
}  // namespace capssa
