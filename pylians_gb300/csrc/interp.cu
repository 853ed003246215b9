// Neighbours of the mass assignment on the particle side:
//   * CIC interpolation of a grid at particle positions (MAS_library.pyx:558-599),
//     the gather dual of the CIC scatter;
//   * redshift-space positions s = x + v (1+z)/H(z) along one axis with the
//     periodic wrap of redshift_space_library.pyx:29-43.
// One thread per particle, grid-stride loops; positions are read as float32
// [n][3] rows exactly as the reference's typed memoryviews hold them.
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

// den[i] = sum of the eight corner values times d/u weights, added in the
// reference's order: (d,d,d), (d,d,u), (d,u,d), (d,u,u), (u,d,d), (u,d,u),
// (u,u,d), (u,u,u); each term density * w0 * w1 * w2 left to right.
__global__ void __launch_bounds__(256) cic_interp_kernel(const float *__restrict__ g, int dims, float inv,
                                                         const float *__restrict__ pos, long long n,
                                                         float *__restrict__ den)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long D = dims;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float u[3], dd[3];
        long long id[3], iu[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float dist = __fmul_rn(__ldg(pos + 3 * i + a), inv);
            const float t = truncf(dist);
            u[a] = __fsub_rn(dist, t);
            dd[a] = __fsub_rn(1.0f, u[a]);
            const int k = wrap_index(__float2int_rz(t), dims);
            id[a] = k;
            iu[a] = k + 1 == dims ? 0 : k + 1;
        }
        const float w0[2] = {dd[0], u[0]}, w1[2] = {dd[1], u[1]}, w2[2] = {dd[2], u[2]};
        const long long c0[2] = {id[0], iu[0]}, c1[2] = {id[1], iu[1]}, c2[2] = {id[2], iu[2]};
        float acc = 0.0f;
#pragma unroll
        for (int l = 0; l < 2; l++)
#pragma unroll
            for (int m = 0; m < 2; m++)
#pragma unroll
                for (int q = 0; q < 2; q++) {
                    const float v = __ldg(g + (c0[l] * D + c1[m]) * D + c2[q]);
                    const float term = __fmul_rn(__fmul_rn(__fmul_rn(v, w0[l]), w1[m]), w2[q]);
                    acc = (l | m | q) ? __fadd_rn(acc, term) : term;
                }
        den[i] = acc;
    }
}

__global__ void __launch_bounds__(256) rsd_kernel(float *__restrict__ pos, const float *__restrict__ vel,
                                                  long long n, float box, float factor, int axis)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float p = __fadd_rn(pos[3 * i + axis], __fmul_rn(__ldg(vel + 3 * i + axis), factor));
        if (p > box || p < 0.0f) p = fmodf(__fadd_rn(p, box), box);
        pos[3 * i + axis] = p;
    }
}

inline unsigned blocks_of(long long n)
{
    long long b = (n + 255) / 256;
    const long long cap = (long long)num_sms() * 16;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_cic_interp(const float *grid, int dims, float box_size, const float *pos, int64_t n,
                              float *out, void *stream)
{
    PYL_CHECK_ARG(dims > 0 && dims <= 65536, "dims out of range");
    PYL_CHECK_ARG(n >= 0, "negative particle count");
    PYL_CHECK_ARG(n == 0 || (grid != nullptr && pos != nullptr && out != nullptr), "null pointer");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    if (n == 0) return PYL_OK;
    const float inv = (float)dims / box_size;             // MAS_library.pyx:575
    cic_interp_kernel<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(grid, dims, inv, pos, n, out);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_pos_redshift_space(float *pos, const float *vel, int64_t n, float box_size, float hubble,
                                      float redshift, int axis, void *stream)
{
    PYL_CHECK_ARG(n >= 0, "negative particle count");
    PYL_CHECK_ARG(n == 0 || (pos != nullptr && vel != nullptr), "null pointer");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    PYL_CHECK_ARG(hubble != 0.0f, "Hubble must be non-zero");
    if (n == 0) return PYL_OK;
    // factor = (1.0 + redshift) / Hubble in double, kept as float (redshift_space_library.pyx:36)
    const float factor = (float)((1.0 + (double)redshift) / (double)hubble);
    rsd_kernel<<<blocks_of(n), 256, 0, (cudaStream_t)stream>>>(pos, vel, n, box_size, factor, axis);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
