// Bispectrum: shell-mask fill of the deconvolved half-complex field and the
// real-space triple-product reduction.
//
// Restates library/Pk_library/bispectrum_library.pyx:
//   shells [k/kF - 1, k/kF + 1) over ALL stored half-space modes (:73-77,
//   95-118; the Hermitian skip there is commented out), delta_s / I_s fill
//   (:121-127), P(k_s) = sum delta_s^2 / sum I_s^2 (:132-138) and
//   B = sum d1 d2 d3 / sum I1 I2 I3 (:183-189).
// Shell membership is an integer range test on kx^2+ky^2+kz^2; the host turns
// the reference's float64 bounds into exact integer bounds.  sum_x delta_s(x)^2
// and sum_x I_s(x)^2 come from Parseval on the half grid (modes with
// 0 < kz < N/2 stand for two), so only the triple products need real space.
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

struct ShellBounds {
    long long lo[PYL_BK_MAX_SHELLS], hi[PYL_BK_MAX_SHELLS];
    int n;
};

__global__ void __launch_bounds__(256) shell_fill_kernel(const float2 *__restrict__ dk, int dims,
                                                         ShellBounds sb, float2 *__restrict__ od,
                                                         float2 *__restrict__ oi, double *power)
{
    __shared__ double acc[2 * PYL_BK_MAX_SHELLS];
    for (int i = threadIdx.x; i < 2 * sb.n; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int nz = dims / 2 + 1;
    const long long half = (long long)dims * dims * nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const bool even = (dims & 1) == 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < half; i += stride) {
        const int kz = (int)(i % nz);
        const long long rr = i / nz;
        const int ky = freq_of((int)(rr % dims), dims), kx = freq_of((int)(rr / dims), dims);
        const long long n2 = (long long)kx * kx + (long long)ky * ky + (long long)kz * kz;
        // skip quickly when outside every shell
        bool any = false;
        for (int s = 0; s < sb.n; s++) any |= (n2 >= sb.lo[s]) & (n2 < sb.hi[s]);
        if (!any) continue;
        const float2 v = __ldg(dk + i);
        const double w = (kz == 0 || (even && kz == dims / 2)) ? 1.0 : 2.0;
        const double p2 = w * ((double)v.x * v.x + (double)v.y * v.y);
        for (int s = 0; s < sb.n; s++) {
            if (n2 >= sb.lo[s] && n2 < sb.hi[s]) {
                od[s * half + i] = v;
                oi[s * half + i] = make_float2(1.0f, 0.0f);
                atomicAdd(acc + 2 * s, p2);
                atomicAdd(acc + 2 * s + 1, w);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * sb.n; i += blockDim.x)
        if (acc[i] != 0.0) atomicAdd(power + i, acc[i]);
}

struct TriList {
    int a[PYL_BK_MAX_SHELLS], b[PYL_BK_MAX_SHELLS], c[PYL_BK_MAX_SHELLS];
};

// blockIdx.y = triangle within this launch; float32 partial sums over 32 cells,
// float64 above that.
__global__ void __launch_bounds__(256) triangle_kernel(const float *__restrict__ d, const float *__restrict__ I,
                                                       long long cells, long long fs, TriList tl, int tri0,
                                                       double *num, double *den)
{
    const int t = blockIdx.y;
    const float4 *da = (const float4 *)(d + tl.a[t] * fs);
    const float4 *db = (const float4 *)(d + tl.b[t] * fs);
    const float4 *dc = (const float4 *)(d + tl.c[t] * fs);
    const float4 *ia = (const float4 *)(I + tl.a[t] * fs);
    const float4 *ib = (const float4 *)(I + tl.b[t] * fs);
    const float4 *ic = (const float4 *)(I + tl.c[t] * fs);
    const long long n4 = cells / 4;
    double sn = 0.0, sd = 0.0;
    float fn = 0.0f, fd = 0.0f;
    int k = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
         i += (long long)gridDim.x * blockDim.x) {
        const float4 x = __ldg(da + i), y = __ldg(db + i), z = __ldg(dc + i);
        const float4 p = __ldg(ia + i), q = __ldg(ib + i), r = __ldg(ic + i);
        fn += (x.x * y.x) * z.x + (x.y * y.y) * z.y + (x.z * y.z) * z.z + (x.w * y.w) * z.w;
        fd += (p.x * q.x) * r.x + (p.y * q.y) * r.y + (p.z * q.z) * r.z + (p.w * q.w) * r.w;
        if (++k == 8) { sn += fn; sd += fd; fn = fd = 0.0f; k = 0; }
    }
    sn += fn; sd += fd;
    if (blockIdx.x == 0 && threadIdx.x < (cells & 3)) {   // tail cells (cells % 4)
        const long long j = n4 * 4 + threadIdx.x;
        const float *a0 = d + tl.a[t] * fs, *b0 = d + tl.b[t] * fs, *c0 = d + tl.c[t] * fs;
        const float *a1 = I + tl.a[t] * fs, *b1 = I + tl.b[t] * fs, *c1 = I + tl.c[t] * fs;
        sn += (a0[j] * b0[j]) * c0[j];
        sd += (a1[j] * b1[j]) * c1[j];
    }
    for (int o = 16; o > 0; o >>= 1) {
        sn += __shfl_down_sync(0xffffffffu, sn, o);
        sd += __shfl_down_sync(0xffffffffu, sd, o);
    }
    __shared__ double wsn[8], wsd[8];
    if ((threadIdx.x & 31) == 0) { wsn[threadIdx.x >> 5] = sn; wsd[threadIdx.x >> 5] = sd; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a += wsn[w]; b += wsd[w]; }
        atomicAdd(num + tri0 + t, a);
        atomicAdd(den + tri0 + t, b);
    }
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_bk_shell_fill(const void *dk, int dims, const int64_t *host_k2_lo,
                                 const int64_t *host_k2_hi, int n_shells, void *out_delta,
                                 void *out_ind, double *power, void *stream)
{
    PYL_CHECK_ARG(dk && out_delta && out_ind && power && host_k2_lo && host_k2_hi, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 4096, "dims out of range");
    PYL_CHECK_ARG(n_shells >= 1 && n_shells <= PYL_BK_MAX_SHELLS, "1..96 shells per call");
    ShellBounds sb;
    sb.n = n_shells;
    for (int s = 0; s < n_shells; s++) { sb.lo[s] = host_k2_lo[s]; sb.hi[s] = host_k2_hi[s]; }
    const long long half = (long long)dims * dims * (dims / 2 + 1);
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(out_delta, 0, sizeof(float2) * half * n_shells, st));
    PYL_CUDA(cudaMemsetAsync(out_ind, 0, sizeof(float2) * half * n_shells, st));
    PYL_CUDA(cudaMemsetAsync(power, 0, sizeof(double) * 2 * n_shells, st));
    long long blocks = (half + 255) / 256;
    if (blocks > (long long)num_sms() * 8) blocks = (long long)num_sms() * 8;
    shell_fill_kernel<<<(unsigned)blocks, 256, 0, st>>>((const float2 *)dk, dims, sb, (float2 *)out_delta,
                                                        (float2 *)out_ind, power);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_bk_triangles(const float *d_fields, const float *i_fields, int dims,
                                int64_t field_stride, int n_shells, const int *host_tri, int n_tri,
                                double *num, double *den, void *stream)
{
    PYL_CHECK_ARG(d_fields && i_fields && host_tri && num && den, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && n_shells >= 1 && n_tri >= 1, "bad sizes");
    PYL_CHECK_ARG((((uintptr_t)d_fields) & 15) == 0 && (((uintptr_t)i_fields) & 15) == 0,
                  "field buffers must be 16-byte aligned");
    const long long cells = (long long)dims * dims * dims;
    PYL_CHECK_ARG(field_stride >= cells && (field_stride & 3) == 0,
                  "field_stride must be >= dims^3 and a multiple of 4");
    for (int t = 0; t < 3 * n_tri; t++)
        PYL_CHECK_ARG(host_tri[t] >= 0 && host_tri[t] < n_shells, "triangle shell index out of range");
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(num, 0, sizeof(double) * n_tri, st));
    PYL_CUDA(cudaMemsetAsync(den, 0, sizeof(double) * n_tri, st));
    long long bx = (cells / 4 + 255) / 256;
    const long long cap = (long long)num_sms() * 4;
    for (int t0 = 0; t0 < n_tri; t0 += PYL_BK_MAX_SHELLS) {
        const int nt = n_tri - t0 < PYL_BK_MAX_SHELLS ? n_tri - t0 : PYL_BK_MAX_SHELLS;
        TriList tl;
        for (int t = 0; t < nt; t++) {
            tl.a[t] = host_tri[3 * (t0 + t)];
            tl.b[t] = host_tri[3 * (t0 + t) + 1];
            tl.c[t] = host_tri[3 * (t0 + t) + 2];
        }
        long long b = bx;
        const long long per_tri_cap = cap / nt > 8 ? cap / nt : 8;
        if (b > per_tri_cap) b = per_tri_cap;
        if (b < 1) b = 1;
        dim3 grid((unsigned)b, (unsigned)nt);
        triangle_kernel<<<grid, 256, 0, st>>>(d_fields, i_fields, cells, field_stride, tl, t0, num, den);
        PYL_LAUNCH_CHECK();
    }
    return PYL_OK;
}
