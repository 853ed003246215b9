// Small MLP for the learned aliasing correction: 4 -> 64 -> 64 -> 64 -> 1, tanh
// hidden layers, BF16 weights, FP32 accumulation.  No counterpart in the
// reference.  Kernels: forward (one thread per sample, weights staged in
// shared memory as bf16), backward in two steps (per-sample deltas, then one
// thread per weight summing delta x activation over the batch), and Adam on
// FP32 master weights that re-rounds the BF16 copy.
//
// Parameter layout (row-major [out][in]):
//   W1[64][4] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[1][64] b4[1]
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

constexpr int IN = 4, H = 64;
constexpr int OW1 = 0, OB1 = OW1 + H * IN, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H,
              OB3 = OW3 + H * H, OW4 = OB3 + H, OB4 = OW4 + H, NPARAM = OB4 + 1;
constexpr int ACT = 3 * H;   // stored activations per sample: h1 | h2 | h3

__device__ __forceinline__ float wload(const __nv_bfloat16 *w, int i) { return __bfloat162float(w[i]); }

// Forward pass; h (B x 192, may be null) keeps the hidden activations for backward.
__global__ void __launch_bounds__(128) mlp_forward_kernel(const __nv_bfloat16 *__restrict__ params,
                                                          const float *__restrict__ x, int B,
                                                          float *__restrict__ h, float *__restrict__ y)
{
    __shared__ __nv_bfloat16 w[NPARAM];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = params[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    float a[H], b[H];
    float xin[IN];
#pragma unroll
    for (int i = 0; i < IN; i++) xin[i] = x[(long long)s * IN + i];
#pragma unroll 4
    for (int j = 0; j < H; j++) {
        float acc = wload(w, OB1 + j);
#pragma unroll
        for (int i = 0; i < IN; i++) acc = fmaf(wload(w, OW1 + j * IN + i), xin[i], acc);
        a[j] = tanhf(acc);
    }
    if (h) for (int j = 0; j < H; j++) h[(long long)s * ACT + j] = a[j];
#pragma unroll 2
    for (int j = 0; j < H; j++) {
        float acc = wload(w, OB2 + j);
        for (int i = 0; i < H; i++) acc = fmaf(wload(w, OW2 + j * H + i), a[i], acc);
        b[j] = tanhf(acc);
    }
    if (h) for (int j = 0; j < H; j++) h[(long long)s * ACT + H + j] = b[j];
#pragma unroll 2
    for (int j = 0; j < H; j++) {
        float acc = wload(w, OB3 + j);
        for (int i = 0; i < H; i++) acc = fmaf(wload(w, OW3 + j * H + i), b[i], acc);
        a[j] = tanhf(acc);
    }
    if (h) for (int j = 0; j < H; j++) h[(long long)s * ACT + 2 * H + j] = a[j];
    float out = wload(w, OB4);
    for (int i = 0; i < H; i++) out = fmaf(wload(w, OW4 + i), a[i], out);
    y[s] = out;
}

// Per-sample deltas of the weighted MSE loss sum_s wt_s (y_s - t_s)^2 / sum_s wt_s:
// d (B x 192) receives dL/d(pre-activation) of layers 1..3; dy[s] = dL/dy_s.
__global__ void __launch_bounds__(128) mlp_delta_kernel(const __nv_bfloat16 *__restrict__ params,
                                                        const float *__restrict__ h, const float *__restrict__ y,
                                                        const float *__restrict__ t, const float *__restrict__ wt,
                                                        float inv_wsum, int B, float *__restrict__ d,
                                                        float *__restrict__ dy)
{
    __shared__ __nv_bfloat16 w[NPARAM];
    for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) w[i] = params[i];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= B) return;
    const float g = 2.0f * (wt ? wt[s] : 1.0f) * inv_wsum * (y[s] - t[s]);
    dy[s] = g;
    const float *hs = h + (long long)s * ACT;
    float d3[H], d2[H];
    for (int j = 0; j < H; j++) {
        const float a3 = hs[2 * H + j];
        d3[j] = g * wload(w, OW4 + j) * (1.0f - a3 * a3);
    }
    for (int i = 0; i < H; i++) {
        float acc = 0.0f;
        for (int j = 0; j < H; j++) acc = fmaf(wload(w, OW3 + j * H + i), d3[j], acc);
        const float a2 = hs[H + i];
        d2[i] = acc * (1.0f - a2 * a2);
    }
    float *ds = d + (long long)s * ACT;
    for (int i = 0; i < H; i++) {
        float acc = 0.0f;
        for (int j = 0; j < H; j++) acc = fmaf(wload(w, OW2 + j * H + i), d2[j], acc);
        const float a1 = hs[i];
        ds[i] = acc * (1.0f - a1 * a1);
    }
    for (int j = 0; j < H; j++) {
        ds[H + j] = d2[j];
        ds[2 * H + j] = d3[j];
    }
}

// One thread per parameter: gradient = sum over the batch of delta x input.
__global__ void __launch_bounds__(256) mlp_grad_kernel(const float *__restrict__ x, const float *__restrict__ h,
                                                       const float *__restrict__ d, const float *__restrict__ dy,
                                                       int B, float *__restrict__ grad)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= NPARAM) return;
    float acc = 0.0f;
    if (p < OB1) {                       // W1[j][i]: d1[j] * x[i]
        const int j = p / IN, i = p % IN;
        for (int s = 0; s < B; s++) acc = fmaf(d[(long long)s * ACT + j], x[(long long)s * IN + i], acc);
    } else if (p < OW2) {                // b1
        const int j = p - OB1;
        for (int s = 0; s < B; s++) acc += d[(long long)s * ACT + j];
    } else if (p < OB2) {                // W2[j][i]: d2[j] * h1[i]
        const int q = p - OW2, j = q / H, i = q % H;
        for (int s = 0; s < B; s++) acc = fmaf(d[(long long)s * ACT + H + j], h[(long long)s * ACT + i], acc);
    } else if (p < OW3) {
        const int j = p - OB2;
        for (int s = 0; s < B; s++) acc += d[(long long)s * ACT + H + j];
    } else if (p < OB3) {                // W3[j][i]: d3[j] * h2[i]
        const int q = p - OW3, j = q / H, i = q % H;
        for (int s = 0; s < B; s++) acc = fmaf(d[(long long)s * ACT + 2 * H + j], h[(long long)s * ACT + H + i], acc);
    } else if (p < OW4) {
        const int j = p - OB3;
        for (int s = 0; s < B; s++) acc += d[(long long)s * ACT + 2 * H + j];
    } else if (p < OB4) {                // W4[i]: dy * h3[i]
        const int i = p - OW4;
        for (int s = 0; s < B; s++) acc = fmaf(dy[s], h[(long long)s * ACT + 2 * H + i], acc);
    } else {
        for (int s = 0; s < B; s++) acc += dy[s];
    }
    grad[p] = acc;
}

__global__ void __launch_bounds__(256) mlp_adam_kernel(float *master, __nv_bfloat16 *params, const float *grad,
                                                       float *m, float *v, int n, float lr, float b1, float b2,
                                                       float eps, float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const float g = grad[p];
    const float mm = b1 * m[p] + (1.0f - b1) * g;
    const float vv = b2 * v[p] + (1.0f - b2) * g * g;
    m[p] = mm;
    v[p] = vv;
    const float w = master[p] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    master[p] = w;
    params[p] = __float2bfloat16_rn(w);
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_mlp_param_count(void) { return NPARAM; }

extern "C" int pyl_mlp_forward(const void *params_bf16, const float *x, int batch, float *act, float *y,
                               void *stream)
{
    PYL_CHECK_ARG(params_bf16 && x && y && batch >= 0, "bad arguments");
    if (batch == 0) return PYL_OK;
    mlp_forward_kernel<<<(batch + 127) / 128, 128, 0, (cudaStream_t)stream>>>(
        (const __nv_bfloat16 *)params_bf16, x, batch, act, y);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_mlp_backward(const void *params_bf16, const float *x, const float *act, const float *y,
                                const float *target, const float *weights, float weight_sum, int batch,
                                float *delta, float *dy, float *grad, void *stream)
{
    PYL_CHECK_ARG(params_bf16 && x && act && y && target && delta && dy && grad && batch > 0, "bad arguments");
    PYL_CHECK_ARG(weight_sum > 0.0f, "weight_sum must be positive");
    cudaStream_t st = (cudaStream_t)stream;
    mlp_delta_kernel<<<(batch + 127) / 128, 128, 0, st>>>((const __nv_bfloat16 *)params_bf16, act, y, target,
                                                          weights, 1.0f / weight_sum, batch, delta, dy);
    PYL_LAUNCH_CHECK();
    mlp_grad_kernel<<<(NPARAM + 255) / 256, 256, 0, st>>>(x, act, delta, dy, batch, grad);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_mlp_adam(float *master, void *params_bf16, const float *grad, float *m, float *v, int n,
                            float lr, float beta1, float beta2, float eps, int step, void *stream)
{
    PYL_CHECK_ARG(master && params_bf16 && grad && m && v && n > 0 && step >= 1, "bad arguments");
    const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
    mlp_adam_kernel<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(
        master, (__nv_bfloat16 *)params_bf16, grad, m, v, n, lr, beta1, beta2, eps, c1, c2);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
