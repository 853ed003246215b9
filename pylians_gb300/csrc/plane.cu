// P(k) of 2D fields (Pk_library.Pk_plane / XPk_plane, Pk_library.pyx:440-516,
// 814-941) over the 2D R2C output: per independent mode (ky = 0 and, for even
// grids, ky = N/2 keep kx >= 0), MAS factor of each field (the float-rounded
// float64 product of the two axis factors), bin int(|k|), sums of |k|,
// counts, |d1|^2, |d2|^2 and Re(d1 d2*) in float64 per mode, as the reference.
// One thread per row kx walks ky sequentially and adds to shared memory only
// when the bin changes; float64 shared sums, float64 global atomics per CTA.
#include <cuda_runtime.h>

#include "pk_common.cuh"

namespace pyl {
namespace {

__device__ __forceinline__ void plane_flush(double *acc, int nb, int bin, double k, double c, double p1,
                                            double p2, double px)
{
    atomicAdd(acc + bin, k);
    atomicAdd(acc + nb + bin, c);
    atomicAdd(acc + 2 * nb + bin, p1);
    atomicAdd(acc + 3 * nb + bin, p2);
    atomicAdd(acc + 4 * nb + bin, px);
}

// sums: K[nb] | N[nb] | P1[nb] | P2[nb] | PX[nb], nb = int(sqrt(2) N/2) + 1
__global__ void __launch_bounds__(256) plane_bin_kernel(const float2 *__restrict__ d1, const float2 *__restrict__ d2,
                                                        int dims, int p1, int p2, int nb, double *__restrict__ sums)
{
    extern __shared__ double acc[];                    // [5][nb]
    for (int i = threadIdx.x; i < 5 * nb; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int middle = dims / 2, ny = dims / 2 + 1;
    const bool even = (dims & 1) == 0;
    for (int kxx = blockIdx.x * blockDim.x + threadIdx.x; kxx < dims; kxx += gridDim.x * blockDim.x) {
        const int kx = freq_of(kxx, dims);
        const double cx1 = mas_corr_d(kx, dims, p1), cx2 = mas_corr_d(kx, dims, p2);
        int cur = -1;
        double sk = 0.0, sc = 0.0, s1 = 0.0, s2 = 0.0, sx = 0.0;
        for (int ky = 0; ky < ny; ky++) {
            if ((ky == 0 || (ky == middle && even)) && kx < 0) continue;
            const int n2 = kx * kx + ky * ky;
            const int bin = isqrt_exact(n2);
            if (bin != cur) {
                if (cur >= 0) plane_flush(acc, nb, cur, sk, sc, s1, s2, sx);
                cur = bin;
                sk = sc = s1 = s2 = sx = 0.0;
            }
            const float m1 = (float)(cx1 * mas_corr_d(ky, dims, p1));
            float2 a = d1[(long long)kxx * ny + ky];
            a.x = __fmul_rn(a.x, m1);
            a.y = __fmul_rn(a.y, m1);
            sk += sqrt((double)n2);
            sc += 1.0;
            s1 += (double)a.x * a.x + (double)a.y * a.y;
            if (d2) {
                const float m2 = (float)(cx2 * mas_corr_d(ky, dims, p2));
                float2 b = d2[(long long)kxx * ny + ky];
                b.x = __fmul_rn(b.x, m2);
                b.y = __fmul_rn(b.y, m2);
                s2 += (double)b.x * b.x + (double)b.y * b.y;
                sx += (double)a.x * b.x + (double)a.y * b.y;
            }
        }
        if (cur >= 0) plane_flush(acc, nb, cur, sk, sc, s1, s2, sx);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 5 * nb; i += blockDim.x)
        if (acc[i] != 0.0) atomicAdd(sums + i, acc[i]);
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_pk_plane_bins(int dims)
{
    const int middle = dims / 2;
    return dims < 2 ? 0 : (int)sqrt((double)middle * middle * 2.0) + 1;
}

extern "C" int pyl_pk_plane_bin(const void *dk1, const void *dk2, int dims, int mas_p1, int mas_p2, double *sums,
                                void *stream)
{
    PYL_CHECK_ARG(dk1 != nullptr && sums != nullptr && dims >= 2 && dims <= 65536, "bad arguments");
    PYL_CHECK_ARG(mas_p1 >= 0 && mas_p1 <= 4 && mas_p2 >= 0 && mas_p2 <= 4, "MAS exponent must be 0..4");
    const int nb = pyl_pk_plane_bins(dims);
    const size_t smem = sizeof(double) * 5 * nb;
    PYL_CHECK_ARG(smem <= 200 * 1024, "grid too large for the shared-memory bins");
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * 5 * nb, st));
    PYL_CUDA(ensure_smem(plane_bin_kernel, smem));
    int blocks = (dims + 255) / 256;
    plane_bin_kernel<<<blocks, 256, smem, st>>>((const float2 *)dk1, (const float2 *)dk2, dims, mas_p1, mas_p2,
                                                nb, sums);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
