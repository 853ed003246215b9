// smoothing_library (smoothing_library.pyx:20-114): the real-space filter of
// FT_filter on the grid and the Fourier-space product of field_smoothing.
//   pyl_filter_grid: Top-Hat (1 where d^2 <= R_grid^2) or Gaussian
//     (exp(-d^2 / (2 R_grid^2)), float64 exp rounded to float), R_grid =
//     R dims / BoxSize in float; *norm = float64 sum; then every value divided by
//     it (float64 division, rounded), as the reference.  The R2C follows.
//   pyl_cmul: a[i] *= b[i] over complex64 arrays.
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

__device__ __forceinline__ float filter_value(long long i, int dims, float R2, int gaussian)
{
    const long long plane = (long long)dims * dims;
    const int x = freq_of((int)(i / plane), dims), y = freq_of((int)((i / dims) % dims), dims),
              z = freq_of((int)(i % dims), dims);
    const int d2 = x * x + y * y + z * z;
    if (!gaussian) return (float)d2 <= R2 ? 1.0f : 0.0f;
    return (float)exp(-(double)d2 / (2.0 * (double)R2));
}

__global__ void __launch_bounds__(256) filter_fill_kernel(float *__restrict__ f, int dims, float R2, int gaussian,
                                                          double *__restrict__ norm)
{
    __shared__ double part[8];
    const long long n = (long long)dims * dims * dims;
    const long long stride = (long long)gridDim.x * blockDim.x;
    double s = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float v = filter_value(i, dims, R2, gaussian);
        f[i] = v;
        s += v;
    }
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += part[w];
        atomicAdd(norm, t);
    }
}

__global__ void __launch_bounds__(256) filter_norm_kernel(float *__restrict__ f, long long n,
                                                          const double *__restrict__ norm)
{
    const double s = *norm;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        f[i] = (float)((double)f[i] / s);
}

__global__ void __launch_bounds__(256) cmul_kernel(float2 *__restrict__ a, const float2 *__restrict__ b, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float2 x = a[i], y = b[i];
        a[i] = make_float2(__fsub_rn(__fmul_rn(x.x, y.x), __fmul_rn(x.y, y.y)),
                           __fadd_rn(__fmul_rn(x.x, y.y), __fmul_rn(x.y, y.x)));
    }
}

inline unsigned blocks_of(long long n)
{
    long long b = (n + 255) / 256;
    const long long cap = (long long)num_sms() * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_filter_grid(float *field, int dims, float box_size, float R, int gaussian, double *norm,
                               void *stream)
{
    PYL_CHECK_ARG(field != nullptr && norm != nullptr && dims >= 2 && dims <= 8192, "bad arguments");
    PYL_CHECK_ARG(box_size > 0.0f && R >= 0.0f, "BoxSize must be positive and R non-negative");
    cudaStream_t st = (cudaStream_t)stream;
    const float r_grid = R * (float)dims / box_size;            // smoothing_library.pyx:32
    const float R2 = r_grid * r_grid;
    const long long n = (long long)dims * dims * dims;
    PYL_CUDA(cudaMemsetAsync(norm, 0, sizeof(double), st));
    filter_fill_kernel<<<blocks_of(n), 256, 0, st>>>(field, dims, R2, gaussian ? 1 : 0, norm);
    PYL_LAUNCH_CHECK();
    filter_norm_kernel<<<blocks_of(n), 256, 0, st>>>(field, n, norm);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_cmul(void *a, const void *b, int64_t n, void *stream)
{
    PYL_CHECK_ARG(a != nullptr && b != nullptr && n >= 0, "bad arguments");
    if (n == 0) return PYL_OK;
    cmul_kernel<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>((float2 *)a, (const float2 *)b, n);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
