// Overdensity normalisation and in-place deconvolution (keep_deltak / bispectrum
// input), plus the sizes of the P(k) sums.  The fused bin kernel and the mode
// geometry live in pkbin.cu.
#include <cuda_runtime.h>

#include <math.h>
#include <vector>

#include "pk_common.cuh"

namespace pyl {

namespace {

// Per-axis float64 tables in shared memory, built once per CTA: the MAS factor
// C(k) = (x / sin x)^p of each frequency and, for the interlaced combine, the
// phase e^{i pi k / N}.  Per mode: the float64 product C(kx) C(ky) C(kz) rounded to
// float32 (Pk_library.pyx:86-87,353-355) and the phase as the product of the three
// axis phases (equal to e^{i pi (kx+ky+kz)/N} to float64 rounding).
__global__ void __launch_bounds__(256) deconvolve_kernel(float2 *dk, const float2 *dk2, PkDims d, int p)
{
    extern __shared__ double dtab[];
    const int dims = d.dims;
    double *corr = dtab;                        // [dims]
    double2 *ph = (double2 *)(dtab + dims);     // [dims] when interlaced
    for (int i = threadIdx.x; i < dims; i += blockDim.x) {
        const int k = freq_of(i, dims);
        corr[i] = mas_corr_d(k, dims, p);
        if (dk2) {
            double s, c;
            sincospi((double)k / dims, &s, &c);
            ph[i] = make_double2(c, s);
        }
    }
    __syncthreads();
    const long long total = (long long)dims * dims * d.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const int kz = (int)(i % d.nz);
        const long long rr = i / d.nz;
        const int kyy = (int)(rr % dims), kxx = (int)(rr / dims);
        float2 v = dk[i];
        if (dk2) {
            const double2 a = ph[kxx], b = ph[kyy], e = ph[kz];
            const double2 ab = make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
            const float pc = (float)(ab.x * e.x - ab.y * e.y), ps = (float)(ab.x * e.y + ab.y * e.x);
            const float2 w = dk2[i];
            v.x = 0.5f * (v.x + (w.x * pc - w.y * ps));
            v.y = 0.5f * (v.y + (w.x * ps + w.y * pc));
        }
        const float mf = (float)(corr[kxx] * corr[kyy] * corr[kz]);
        dk[i] = make_float2(__fmul_rn(v.x, mf), __fmul_rn(v.y, mf));
    }
}

// float64 sum of float32 values: float32 partial sums of 4 values, float64 above.
__global__ void __launch_bounds__(256) grid_sum_kernel(const float *__restrict__ g, long long n, double *out)
{
    double acc = 0.0;
    const long long stride = (long long)gridDim.x * blockDim.x * 4;
    const long long n4 = n / 4;
    const float4 *g4 = (const float4 *)g;
    const bool aligned = (((uintptr_t)g) & 15) == 0;
    if (aligned) {
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
             i += (long long)gridDim.x * blockDim.x) {
            const float4 v = __ldg(g4 + i);
            acc += (double)(v.x + v.y) + (double)(v.z + v.w);
        }
        for (long long i = n4 * 4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (long long)gridDim.x * blockDim.x)
            acc += g[i];
    } else {
        for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n;
             i += (long long)gridDim.x * blockDim.x)
            acc += g[i];
    }
    (void)stride;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    __shared__ double ws[8];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += ws[i];
        atomicAdd(out, t);
    }
}

__global__ void __launch_bounds__(256) overdensity_kernel(float *__restrict__ g, long long n,
                                                          const double *d_sum, double host_mean)
{
    const double mean = d_sum ? *d_sum / (double)n : host_mean;
    const float m = (float)mean;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        g[i] = __fsub_rn(__fdiv_rn(g[i], m), 1.0f);
}

inline int blocks_for(long long n, int threads, int per_sm = 8)
{
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)num_sms() * per_sm;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int64_t pyl_pk_sums_len(int dims, int n_fields)
{
    if (dims <= 0 || n_fields <= 0) return 0;
    const PkDims d = pk_dims(dims);
    const long long C = n_fields + n_fields * (n_fields - 1) / 2;
    return (long long)d.nb3 * (3 * C + n_fields) + (long long)d.nb1 * C + (long long)d.nb2 * C;
}

extern "C" int64_t pyl_pk_geometry_len(int dims)
{
    if (dims <= 0) return 0;
    const PkDims d = pk_dims(dims);
    return 2LL * d.nb1 + d.nb2 + 2LL * d.nb3;
}

extern "C" int pyl_mas_deconvolve(void *dk, const void *dk_interlaced, int dims, int mas_p, void *stream)
{
    PYL_CHECK_ARG(dk != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(mas_p >= 0 && mas_p <= 4, "MAS exponent must be 0..4");
    const PkDims d = pk_dims(dims);
    const long long total = (long long)dims * dims * d.nz;
    const size_t smem = sizeof(double) * (size_t)dims * (dk_interlaced ? 3 : 1);
    PYL_CUDA(ensure_smem(deconvolve_kernel, smem));
    // two CTAs per SM: each builds its tables once and strides over the modes
    deconvolve_kernel<<<blocks_for(total, 256, 2), 256, smem, (cudaStream_t)stream>>>(
        (float2 *)dk, (const float2 *)dk_interlaced, d, mas_p);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_grid_sum(const float *grid, int64_t n, double *d_sum, void *stream)
{
    PYL_CHECK_ARG(grid != nullptr && d_sum != nullptr && n > 0, "bad arguments");
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(d_sum, 0, sizeof(double), st));
    grid_sum_kernel<<<blocks_for(n / 4 + 1, 256), 256, 0, st>>>(grid, n, d_sum);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_overdensity(float *grid, int64_t n, const double *d_sum, double host_mean, void *stream)
{
    PYL_CHECK_ARG(grid != nullptr && n > 0, "bad arguments");
    PYL_CHECK_ARG(d_sum != nullptr || host_mean != 0.0, "mean density is zero");
    overdensity_kernel<<<blocks_for(n, 256), 256, 0, (cudaStream_t)stream>>>(grid, n, d_sum, host_mean);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
