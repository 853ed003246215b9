// Correlation function of a grid (Pk_library.Xi, Pk_library.pyx:2035-2150):
//   pyl_xi_power: every stored mode of the R2C output becomes
//                 (|delta_k * W(k)^-1|^2, 0), the MAS factor rounded to float as
//                 the reference's MAS_factor (:2073-2083);
//   (C2R of that, unnormalised, by the caller)
//   pyl_xi_bin:   over all dims^3 separations r = (rx, ry, rz) (signed like
//                 frequencies): bin int(|r|), sums of xi, xi (3 mu^2 - 1)/2,
//                 xi (35 mu^4 - 30 mu^2 + 3)/8, |r| and counts (:2101-2136).
// One thread per row (rx, ry) walks rz sequentially and adds to shared memory
// only when the bin changes; per-CTA float sums, float64 global sums.
#include <cuda_runtime.h>

#include "pk_common.cuh"

namespace pyl {
namespace {

__global__ void __launch_bounds__(256) xi_power_kernel(float2 *dk, PkDims d, int p)
{
    const int dims = d.dims;
    const long long total = (long long)dims * dims * d.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const int kz = (int)(i % d.nz);
        const long long rr = i / d.nz;
        const int kyy = (int)(rr % dims), kxx = (int)(rr / dims);
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        const float mf = (float)(mas_corr_d(kx, dims, p) * mas_corr_d(ky, dims, p) * mas_corr_d(kz, dims, p));
        const float2 v = dk[i];
        const float re = __fmul_rn(v.x, mf), im = __fmul_rn(v.y, mf);
        dk[i] = make_float2(__fadd_rn(__fmul_rn(re, re), __fmul_rn(im, im)), 0.0f);
    }
}

// sums: X[nb3][3] | R[nb3] | N[nb3] (float64)
__global__ void __launch_bounds__(256) xi_bin_kernel(const float *__restrict__ xi, PkDims d, int axis,
                                                     double *__restrict__ sums)
{
    extern __shared__ float acc[];                      // [nb3][3]
    const int dims = d.dims, nb = d.nb3;
    for (int i = threadIdx.x; i < 3 * nb; i += blockDim.x) acc[i] = 0.0f;
    __syncthreads();
    const long long rows = (long long)dims * dims;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
         row += (long long)gridDim.x * blockDim.x) {
        const int rx = freq_of((int)(row / dims), dims), ry = freq_of((int)(row % dims), dims);
        const float *g = xi + row * dims;
        int cur = -1;
        float s0 = 0.0f, s2 = 0.0f, s4 = 0.0f;
        for (int zz = 0; zz < dims; zz++) {
            const int rz = freq_of(zz, dims);
            const int n2 = rx * rx + ry * ry + rz * rz;
            const int bin = isqrt_exact(n2);
            const int par = axis == 0 ? rx : (axis == 1 ? ry : rz);
            const float mu2 = n2 ? (float)((double)(par * par) / (double)n2) : 0.0f;
            const float v = __ldg(g + zz);
            if (bin != cur) {
                if (cur >= 0) {
                    atomicAdd(acc + 3 * cur, s0);
                    atomicAdd(acc + 3 * cur + 1, s2);
                    atomicAdd(acc + 3 * cur + 2, s4);
                }
                cur = bin;
                s0 = s2 = s4 = 0.0f;
            }
            s0 += v;
            s2 += v * (0.5f * (3.0f * mu2 - 1.0f));
            s4 += v * (0.125f * ((35.0f * mu2 - 30.0f) * mu2 + 3.0f));
        }
        if (cur >= 0) {
            atomicAdd(acc + 3 * cur, s0);
            atomicAdd(acc + 3 * cur + 1, s2);
            atomicAdd(acc + 3 * cur + 2, s4);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 3 * nb; i += blockDim.x)
        if (acc[i] != 0.0f) atomicAdd(sums + i, (double)acc[i]);
}

// Data-independent sums: R[bin] = sum |r|, N[bin] = count, over all dims^3 separations.
__global__ void __launch_bounds__(256) xi_geometry_kernel(PkDims d, double *__restrict__ sums)
{
    const int dims = d.dims, nb = d.nb3;
    double *R = sums + 3 * nb, *N = R + nb;
    const long long rows = (long long)dims * dims;
    for (long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x; row < rows;
         row += (long long)gridDim.x * blockDim.x) {
        const int rx = freq_of((int)(row / dims), dims), ry = freq_of((int)(row % dims), dims);
        int cur = -1;
        double r = 0.0, c = 0.0;
        for (int zz = 0; zz < dims; zz++) {
            const int rz = freq_of(zz, dims);
            const int n2 = rx * rx + ry * ry + rz * rz;
            const int bin = isqrt_exact(n2);
            if (bin != cur) {
                if (cur >= 0) { atomicAdd(R + cur, r); atomicAdd(N + cur, c); }
                cur = bin;
                r = 0.0;
                c = 0.0;
            }
            r += sqrt((double)n2);
            c += 1.0;
        }
        if (cur >= 0) { atomicAdd(R + cur, r); atomicAdd(N + cur, c); }
    }
}

// correct_MAS's mode loop (Pk_library.pyx:1776-1794): every stored mode but the
// redundant half of the kz = 0 and kz = N/2 planes (:1789-1792) is multiplied by
// the float-rounded MAS factor.
__global__ void __launch_bounds__(256) correct_mas_kernel(float2 *dk, PkDims d, int p)
{
    const int dims = d.dims;
    const long long total = (long long)dims * dims * d.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const int kz = (int)(i % d.nz);
        const long long rr = i / d.nz;
        const int kyy = (int)(rr % dims), kxx = (int)(rr / dims);
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        if (hermitian_skip(kx, ky, kz, d)) continue;
        const float mf = (float)(mas_corr_d(kx, dims, p) * mas_corr_d(ky, dims, p) * mas_corr_d(kz, dims, p));
        const float2 v = dk[i];
        dk[i] = make_float2(__fmul_rn(v.x, mf), __fmul_rn(v.y, mf));
    }
}

// The reference's half-corrected kz = 0 and kz = N/2 planes are not Hermitian; its
// C2R (FFTW through pyFFTW, or any C2R that transforms x and y before z) uses
// their Hermitian part (P(k) + conj P(-k)) / 2.  Writing that part explicitly
// makes cuFFT's C2R give the same field whatever its internal order.  One thread
// per (k, -k) pair of a plane (the pair's lower flat index does the work).
__global__ void __launch_bounds__(256) hermitian_planes_kernel(float2 *dk, PkDims d)
{
    const int dims = d.dims;
    const long long plane = (long long)dims * dims;
    const int nplanes = (dims & 1) ? 1 : 2;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < nplanes * plane; t += stride) {
        const int kz = t < plane ? 0 : d.middle;
        const long long j = t % plane;
        const int kxx = (int)(j / dims), kyy = (int)(j % dims);
        const int mxx = kxx ? dims - kxx : 0, myy = kyy ? dims - kyy : 0;
        const long long jm = (long long)mxx * dims + myy;
        if (jm < j) continue;
        float2 *a = dk + j * d.nz + kz, *b = dk + jm * d.nz + kz;
        const float2 va = *a, vb = *b;
        const float re = 0.5f * (va.x + vb.x), im = 0.5f * (va.y - vb.y);
        *a = make_float2(re, im);
        *b = make_float2(re, -im);
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

extern "C" int64_t pyl_xi_sums_len(int dims) { return dims < 2 ? 0 : 5LL * pk_dims(dims).nb3; }

extern "C" int pyl_correct_mas(void *dk, int dims, int mas_p, void *stream)
{
    PYL_CHECK_ARG(dk != nullptr && dims >= 2 && dims <= 8192, "bad arguments");
    PYL_CHECK_ARG(mas_p >= 0 && mas_p <= 4, "MAS exponent must be 0..4");
    const PkDims d = pk_dims(dims);
    cudaStream_t st = (cudaStream_t)stream;
    correct_mas_kernel<<<blocks_of((long long)dims * dims * d.nz), 256, 0, st>>>((float2 *)dk, d, mas_p);
    PYL_LAUNCH_CHECK();
    hermitian_planes_kernel<<<blocks_of(2LL * dims * dims), 256, 0, st>>>((float2 *)dk, d);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_xi_power(void *dk, int dims, int mas_p, void *stream)
{
    PYL_CHECK_ARG(dk != nullptr && dims >= 2 && dims <= 8192, "bad arguments");
    PYL_CHECK_ARG(mas_p >= 0 && mas_p <= 4, "MAS exponent must be 0..4");
    const PkDims d = pk_dims(dims);
    xi_power_kernel<<<blocks_of((long long)dims * dims * d.nz), 256, 0, (cudaStream_t)stream>>>((float2 *)dk, d,
                                                                                             mas_p);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_xi_bin(const float *xi_grid, int dims, int axis, double *sums, void *stream)
{
    PYL_CHECK_ARG(xi_grid != nullptr && sums != nullptr && dims >= 2 && dims <= 8192, "bad arguments");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    const PkDims d = pk_dims(dims);
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * 5 * d.nb3, st));
    const size_t smem = sizeof(float) * 3 * d.nb3;
    PYL_CHECK_ARG(smem <= 48 * 1024, "grid too large for the shared-memory bins");
    const long long rows = (long long)dims * dims;
    xi_bin_kernel<<<blocks_of(rows), 256, smem, st>>>(xi_grid, d, axis, sums);
    PYL_LAUNCH_CHECK();
    xi_geometry_kernel<<<blocks_of(rows), 256, 0, st>>>(d, sums);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
