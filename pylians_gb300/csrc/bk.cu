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
//
// Band-limited evaluation: every mode of a call's shells has |k_a| <= K < N/2 on
// each axis, so the product of three shell fields has no wave number beyond 3K per
// axis, and sum_x d_a d_b d_c over an M^3 grid with M > 3K equals (M/N)^3 times
// the sum over the N^3 grid (a sum over x keeps the k_a + k_b + k_c = 0 terms, and
// with |k_a + k_b + k_c| <= 3K < M no other sum of three modes aliases to zero).
// B and P are ratios of such sums, so the shells are written into M^3 half grids
// (the caller picks M), transformed there and reduced there: (M/N)^3 of the C2R
// and reduction work.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <utility>
#include <vector>

#include "common.cuh"

namespace pyl {
namespace {

struct ShellBounds {
    long long lo[PYL_BK_MAX_SHELLS], hi[PYL_BK_MAX_SHELLS];
    int slot[PYL_BK_MAX_SHELLS];     // output field of each shell, -1: power only
    int n;
};

// One thread per stored mode of the N grid with |kx|, |ky|, kz <= K (no shell
// reaches past K): kx, ky in [klo, khi] = [-min(K, (N-1)/2), min(K, N/2)], the
// grid's own signed frequencies, each stored mode once.  The mode's value and
// indicator go to slot (kx mod M, ky mod M, kz) of every shell that holds it; the
// Parseval sums use the N grid's weights (1 on the kz = 0 and kz = N/2 planes, 2
// elsewhere).  FD / FI: write the delta / indicator fields (the indicator fields
// only depend on the shells, so a plan writes them once).
template <bool FD, bool FI>
__global__ void __launch_bounds__(256) shell_fill_kernel(const float2 *__restrict__ dk, int dims, int K, int M,
                                                         ShellBounds sb, float2 *__restrict__ od,
                                                         float2 *__restrict__ oi, double *power)
{
    __shared__ double acc[2 * PYL_BK_MAX_SHELLS];
    for (int i = threadIdx.x; i < 2 * sb.n; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int nz = dims / 2 + 1, mz = M / 2 + 1;
    const int klo = -min(K, (dims - 1) / 2), khi = min(K, dims / 2), kzhi = min(K, dims / 2);
    const int side = khi - klo + 1;
    const long long cube = (long long)side * side * (kzhi + 1);
    const long long half_m = (long long)M * M * mz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const bool even = (dims & 1) == 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cube; i += stride) {
        const int kz = (int)(i % (kzhi + 1));
        const long long rr = i / (kzhi + 1);
        const int ky = (int)(rr % side) + klo, kx = (int)(rr / side) + klo;
        const long long n2 = (long long)kx * kx + (long long)ky * ky + (long long)kz * kz;
        bool any = false;
        for (int s = 0; s < sb.n; s++) any |= (n2 >= sb.lo[s]) & (n2 < sb.hi[s]);
        if (!any) continue;
        const long long src = ((long long)(kx < 0 ? kx + dims : kx) * dims + (ky < 0 ? ky + dims : ky)) * nz + kz;
        const long long dst = ((long long)(kx < 0 ? kx + M : kx) * M + (ky < 0 ? ky + M : ky)) * mz + kz;
        const float2 v = FD ? __ldg(dk + src) : make_float2(0.0f, 0.0f);
        const double w = (kz == 0 || (even && kz == dims / 2)) ? 1.0 : 2.0;
        const double p2 = w * ((double)v.x * v.x + (double)v.y * v.y);
        for (int s = 0; s < sb.n; s++) {
            if (n2 >= sb.lo[s] && n2 < sb.hi[s]) {
                const long long f = sb.slot[s];
                if (FD) {
                    if (f >= 0 && od) od[f * half_m + dst] = v;
                    atomicAdd(acc + 2 * s, p2);
                }
                if (FI && f >= 0) oi[f * half_m + dst] = make_float2(1.0f, 0.0f);
                atomicAdd(acc + 2 * s + 1, w);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * sb.n; i += blockDim.x)
        if (acc[i] != 0.0) atomicAdd(power + i, acc[i]);
}

// Triangles grouped by their first two shells: a group reads d_a d_b and I_a I_b
// once per cell and the third shell of each of its (up to GC) triangles.  GC = 4
// keeps a thread within 85 registers (three resident CTAs per SM: with GC = 8 and
// 128 registers the reduction was latency bound at 18% of the warp slots); groups
// sharing (a, b) re-read those two fields, mostly from L2.
constexpr int GC = 4;
constexpr int MAX_GROUPS = 96;

struct TriGroups {
    int a[MAX_GROUPS], b[MAX_GROUPS], n[MAX_GROUPS];
    int c[MAX_GROUPS][GC], t[MAX_GROUPS][GC];
};

// blockIdx.y = group; float32 partial sums over 8 float4 steps, float64 above.
// Products (d_a d_b) d_c, as the reference forms d12 * d3 (:183-186).  WD / WI:
// reduce the delta / indicator fields (num / den).
template <int NC, bool WD, bool WI>
__device__ __forceinline__ void tri_group(const float *__restrict__ d, const float *__restrict__ I, long long cells,
                                          long long fs, const TriGroups &tg, int gi, double *num, double *den)
{
    const float4 *da = (const float4 *)(d + tg.a[gi] * fs), *db = (const float4 *)(d + tg.b[gi] * fs);
    const float4 *ia = (const float4 *)(I + tg.a[gi] * fs), *ib = (const float4 *)(I + tg.b[gi] * fs);
    const float4 *dc[NC], *ic[NC];
#pragma unroll
    for (int j = 0; j < NC; j++) {
        dc[j] = (const float4 *)(d + tg.c[gi][j] * fs);
        ic[j] = (const float4 *)(I + tg.c[gi][j] * fs);
    }
    const long long n4 = cells / 4;
    double sn[NC], sd[NC];
    float fn[NC], fd[NC];
#pragma unroll
    for (int j = 0; j < NC; j++) { sn[j] = sd[j] = 0.0; fn[j] = fd[j] = 0.0f; }
    int k = 0;
#pragma unroll 1    // unrolled, the one-sided forms spill at the 85-register cap
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4;
         i += (long long)gridDim.x * blockDim.x) {
        if (WD) {
            const float4 x = __ldg(da + i), y = __ldg(db + i);
            const float4 xy = make_float4(x.x * y.x, x.y * y.y, x.z * y.z, x.w * y.w);
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const float4 z = __ldg(dc[j] + i);
                fn[j] += xy.x * z.x + xy.y * z.y + xy.z * z.z + xy.w * z.w;
            }
        }
        if (WI) {
            const float4 p = __ldg(ia + i), q = __ldg(ib + i);
            const float4 pq = make_float4(p.x * q.x, p.y * q.y, p.z * q.z, p.w * q.w);
#pragma unroll
            for (int j = 0; j < NC; j++) {
                const float4 r = __ldg(ic[j] + i);
                fd[j] += pq.x * r.x + pq.y * r.y + pq.z * r.z + pq.w * r.w;
            }
        }
        if (++k == 8) {
#pragma unroll
            for (int j = 0; j < NC; j++) { sn[j] += fn[j]; sd[j] += fd[j]; fn[j] = fd[j] = 0.0f; }
            k = 0;
        }
    }
#pragma unroll
    for (int j = 0; j < NC; j++) { sn[j] += fn[j]; sd[j] += fd[j]; }
    if (blockIdx.x == 0 && threadIdx.x < (cells & 3)) {   // tail cells (cells % 4)
        const long long i = n4 * 4 + threadIdx.x;
        const float *a0 = d + tg.a[gi] * fs, *b0 = d + tg.b[gi] * fs;
        const float *a1 = I + tg.a[gi] * fs, *b1 = I + tg.b[gi] * fs;
#pragma unroll
        for (int j = 0; j < NC; j++) {
            if (WD) sn[j] += (a0[i] * b0[i]) * d[tg.c[gi][j] * fs + i];
            if (WI) sd[j] += (a1[i] * b1[i]) * I[tg.c[gi][j] * fs + i];
        }
    }
    __shared__ double wsn[8][GC], wsd[8][GC];
#pragma unroll
    for (int j = 0; j < NC; j++) {
        double a = sn[j], b = sd[j];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if ((threadIdx.x & 31) == 0) { wsn[threadIdx.x >> 5][j] = a; wsd[threadIdx.x >> 5][j] = b; }
    }
    __syncthreads();
    if (threadIdx.x < NC) {
        double a = 0.0, b = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { a += wsn[w][threadIdx.x]; b += wsd[w][threadIdx.x]; }
        if (WD) atomicAdd(num + tg.t[gi][threadIdx.x], a);
        if (WI) atomicAdd(den + tg.t[gi][threadIdx.x], b);
    }
}

template <bool WD, bool WI>
__global__ void __launch_bounds__(256, 3) triangle_group_kernel(const float *__restrict__ d,
                                                                const float *__restrict__ I, long long cells,
                                                                long long fs, TriGroups tg, double *num, double *den)
{
    const int gi = blockIdx.y;
    switch (tg.n[gi]) {     // the third-shell count of a group is uniform over its CTAs
        case 1: tri_group<1, WD, WI>(d, I, cells, fs, tg, gi, num, den); break;
        case 2: tri_group<2, WD, WI>(d, I, cells, fs, tg, gi, num, den); break;
        case 3: tri_group<3, WD, WI>(d, I, cells, fs, tg, gi, num, den); break;
        default: tri_group<4, WD, WI>(d, I, cells, fs, tg, gi, num, den); break;
    }
}

// out = a * b, elementwise over n floats (the float32 product the real-space
// reduction forms first, d_a d_b).
__global__ void __launch_bounds__(256) bk_product_kernel(const float *__restrict__ a, const float *__restrict__ b,
                                                         float *__restrict__ out, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n4 = n / 4;
    const float4 *a4 = (const float4 *)a, *b4 = (const float4 *)b;
    float4 *o4 = (float4 *)out;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
        const float4 x = __ldg(a4 + i), y = __ldg(b4 + i);
        o4[i] = make_float4(x.x * y.x, x.y * y.y, x.z * y.z, x.w * y.w);
    }
    for (long long i = n4 * 4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        out[i] = a[i] * b[i];
}

// Triangle sums in Fourier space: for triangle t with third shell bounds
// [lo[t], hi[t]), out[t] = (1/M^3) sum over the stored modes k of that shell of
// w Re(v(k) conj(P(k))), where P is the R2C of the product field P_ab(x) on the
// M^3 grid, v the deconvolved dims^3 field (or 1 for the indicator) and w = 2 for
// modes standing for a conjugate pair (0 < kz < M/2), 1 otherwise.  By Parseval
// that is sum_x P_ab(x) d_c(x) over the M^3 cells, the real-space triple sum.
// Modes are walked as in shell_fill_kernel (the cube |kx|, |ky|, kz <= K).
struct TriBounds {
    long long lo[PYL_BK_MAX_SHELLS], hi[PYL_BK_MAX_SHELLS];
    int dst[PYL_BK_MAX_SHELLS];      // output index of each triangle
    int n;
};

__global__ void __launch_bounds__(256) shell_dot_kernel(const float2 *__restrict__ dk, int dims, int K, int M,
                                                        TriBounds tb, const float2 *__restrict__ prod_hat,
                                                        double *out)
{
    __shared__ double acc[PYL_BK_MAX_SHELLS];
    for (int i = threadIdx.x; i < tb.n; i += blockDim.x) acc[i] = 0.0;
    __syncthreads();
    const int nz = dims / 2 + 1, mz = M / 2 + 1;
    const int klo = -min(K, (dims - 1) / 2), khi = min(K, dims / 2), kzhi = min(K, dims / 2);
    const int side = khi - klo + 1;
    const long long cube = (long long)side * side * (kzhi + 1);
    const long long stride = (long long)gridDim.x * blockDim.x;
    const bool even_m = (M & 1) == 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < cube; i += stride) {
        const int kz = (int)(i % (kzhi + 1));
        const long long rr = i / (kzhi + 1);
        const int ky = (int)(rr % side) + klo, kx = (int)(rr / side) + klo;
        const long long n2 = (long long)kx * kx + (long long)ky * ky + (long long)kz * kz;
        bool any = false;
        for (int t = 0; t < tb.n; t++) any |= (n2 >= tb.lo[t]) & (n2 < tb.hi[t]);
        if (!any) continue;
        const long long dst = ((long long)(kx < 0 ? kx + M : kx) * M + (ky < 0 ? ky + M : ky)) * mz + kz;
        const float2 q = __ldg(prod_hat + dst);
        float2 v = make_float2(1.0f, 0.0f);
        if (dk) {
            const long long src = ((long long)(kx < 0 ? kx + dims : kx) * dims + (ky < 0 ? ky + dims : ky)) * nz + kz;
            v = __ldg(dk + src);
        }
        const double w = (kz == 0 || (even_m && 2 * kz == M)) ? 1.0 : 2.0;
        const double c = w * ((double)v.x * q.x + (double)v.y * q.y);
        for (int t = 0; t < tb.n; t++)
            if (n2 >= tb.lo[t] && n2 < tb.hi[t]) atomicAdd(acc + t, c);
    }
    __syncthreads();
    const double inv = 1.0 / ((double)M * M * M);
    for (int t = threadIdx.x; t < tb.n; t += blockDim.x)
        if (acc[t] != 0.0) atomicAdd(out + tb.dst[t], acc[t] * inv);
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_bk_shell_fill(const void *dk, int dims, int out_dims, const int64_t *host_k2_lo,
                                 const int64_t *host_k2_hi, const int *host_slot, int n_shells, void *out_delta,
                                 void *out_ind, double *power, void *stream)
{
    PYL_CHECK_ARG(power && host_k2_lo && host_k2_hi, "null pointer");
    PYL_CHECK_ARG(dk || !out_delta, "the delta fields need dk");
    PYL_CHECK_ARG(dk || out_ind, "no output: give dk (delta fields and powers) or out_ind");
    PYL_CHECK_ARG(dims >= 2 && dims <= 4096, "dims out of range");
    PYL_CHECK_ARG(n_shells >= 1 && n_shells <= PYL_BK_MAX_SHELLS, "1..96 shells per call");
    ShellBounds sb;
    sb.n = n_shells;
    long long hi_max = 0;
    for (int s = 0; s < n_shells; s++) {
        PYL_CHECK_ARG(host_k2_lo[s] >= 0 && host_k2_hi[s] >= host_k2_lo[s], "bad shell bounds");
        sb.lo[s] = host_k2_lo[s];
        sb.hi[s] = host_k2_hi[s];
        sb.slot[s] = host_slot ? host_slot[s] : s;
        PYL_CHECK_ARG(sb.slot[s] >= -1 && sb.slot[s] < n_shells, "slot out of range");
        hi_max = std::max(hi_max, (long long)host_k2_hi[s]);
    }
    int n_out = 0;                                   // output fields the slots address
    for (int s = 0; s < n_shells; s++) n_out = std::max(n_out, sb.slot[s] + 1);
    PYL_CHECK_ARG(n_out == 0 || !dk || out_delta, "slots address delta fields: out_delta is NULL");
    // K: the largest |k| component of any shell mode (k^2 < hi_max)
    int K = 0;
    while ((long long)(K + 1) * (K + 1) < hi_max) K++;
    PYL_CHECK_ARG(out_dims == dims || (2 * K < out_dims && 3 * K < out_dims && out_dims <= dims),
                  "out_dims must equal dims, or exceed 3 K (and 2 K) with K the largest shell wave number");
    const long long half_m = (long long)out_dims * out_dims * (out_dims / 2 + 1);
    cudaStream_t st = (cudaStream_t)stream;
    if (out_delta && n_out) PYL_CUDA(cudaMemsetAsync(out_delta, 0, sizeof(float2) * half_m * n_out, st));
    if (out_ind && n_out) PYL_CUDA(cudaMemsetAsync(out_ind, 0, sizeof(float2) * half_m * n_out, st));
    PYL_CUDA(cudaMemsetAsync(power, 0, sizeof(double) * 2 * n_shells, st));
    const long long side = std::min(K, dims / 2) + std::min(K, (dims - 1) / 2) + 1;
    const long long cube = side * side * (std::min(K, dims / 2) + 1);
    long long blocks = (cube + 255) / 256;
    if (blocks > (long long)num_sms() * 8) blocks = (long long)num_sms() * 8;
    const unsigned g = (unsigned)std::max(1LL, blocks);
    const float2 *src = (const float2 *)dk;
    float2 *od = (float2 *)out_delta, *oi = (float2 *)out_ind;
    if (src && oi) shell_fill_kernel<true, true><<<g, 256, 0, st>>>(src, dims, K, out_dims, sb, od, oi, power);
    else if (src) shell_fill_kernel<true, false><<<g, 256, 0, st>>>(src, dims, K, out_dims, sb, od, oi, power);
    else shell_fill_kernel<false, true><<<g, 256, 0, st>>>(src, dims, K, out_dims, sb, od, oi, power);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_bk_triangles(const float *d_fields, const float *i_fields, int dims,
                                int64_t field_stride, int n_shells, const int *host_tri, int n_tri,
                                double *num, double *den, void *stream)
{
    PYL_CHECK_ARG(host_tri, "null pointer");
    PYL_CHECK_ARG(d_fields || i_fields, "no field set");
    PYL_CHECK_ARG((!d_fields || num) && (!i_fields || den), "null sum buffer");
    PYL_CHECK_ARG(dims >= 2 && n_shells >= 1 && n_tri >= 1, "bad sizes");
    PYL_CHECK_ARG((((uintptr_t)d_fields) & 15) == 0 && (((uintptr_t)i_fields) & 15) == 0,
                  "field buffers must be 16-byte aligned");
    const long long cells = (long long)dims * dims * dims;
    PYL_CHECK_ARG(field_stride >= cells && (field_stride & 3) == 0,
                  "field_stride must be >= dims^3 and a multiple of 4");
    for (int t = 0; t < 3 * n_tri; t++)
        PYL_CHECK_ARG(host_tri[t] >= 0 && host_tri[t] < n_shells, "triangle shell index out of range");
    cudaStream_t st = (cudaStream_t)stream;
    if (d_fields) PYL_CUDA(cudaMemsetAsync(num, 0, sizeof(double) * n_tri, st));
    if (i_fields) PYL_CUDA(cudaMemsetAsync(den, 0, sizeof(double) * n_tri, st));
    // groups: triangles of equal (a, b), at most GC each
    std::map<std::pair<int, int>, std::vector<int>> by_ab;
    for (int t = 0; t < n_tri; t++) by_ab[std::make_pair(host_tri[3 * t], host_tri[3 * t + 1])].push_back(t);
    std::vector<std::pair<std::pair<int, int>, std::vector<int>>> groups;
    for (auto &kv : by_ab)
        for (size_t i = 0; i < kv.second.size(); i += GC)
            groups.emplace_back(kv.first, std::vector<int>(kv.second.begin() + i,
                                                           kv.second.begin() + std::min(kv.second.size(), i + GC)));
    const long long bx = (cells / 4 + 255) / 256;
    for (size_t g0 = 0; g0 < groups.size(); g0 += MAX_GROUPS) {
        const int ng = (int)std::min(groups.size() - g0, (size_t)MAX_GROUPS);
        TriGroups tg;
        for (int g = 0; g < ng; g++) {
            const auto &gr = groups[g0 + g];
            tg.a[g] = gr.first.first;
            tg.b[g] = gr.first.second;
            tg.n[g] = (int)gr.second.size();
            for (int j = 0; j < GC; j++) {
                const int t = gr.second[std::min(j, tg.n[g] - 1)];
                tg.c[g][j] = host_tri[3 * t + 2];
                tg.t[g][j] = t;
            }
        }
        // about sixteen CTAs per SM over all groups of the launch (three resident)
        long long b = std::max(8LL, (long long)num_sms() * 16 / ng);
        if (b > bx) b = bx;
        if (b < 1) b = 1;
        const dim3 grid((unsigned)b, (unsigned)ng);
        if (d_fields && i_fields)
            triangle_group_kernel<true, true><<<grid, 256, 0, st>>>(d_fields, i_fields, cells, field_stride, tg, num, den);
        else if (d_fields)
            triangle_group_kernel<true, false><<<grid, 256, 0, st>>>(d_fields, i_fields, cells, field_stride, tg, num, den);
        else
            triangle_group_kernel<false, true><<<grid, 256, 0, st>>>(d_fields, i_fields, cells, field_stride, tg, num, den);
        PYL_LAUNCH_CHECK();
    }
    return PYL_OK;
}

extern "C" int pyl_bk_product(const float *a, const float *b, float *out, int64_t n, void *stream)
{
    PYL_CHECK_ARG(a && b && out, "null pointer");
    PYL_CHECK_ARG(n >= 0, "negative length");
    PYL_CHECK_ARG(((((uintptr_t)a) | ((uintptr_t)b) | ((uintptr_t)out)) & 15) == 0, "buffers must be 16-byte aligned");
    if (n == 0) return PYL_OK;
    long long blocks = (n / 4 + 255) / 256;
    if (blocks > (long long)num_sms() * 8) blocks = (long long)num_sms() * 8;
    bk_product_kernel<<<(unsigned)std::max(1LL, blocks), 256, 0, (cudaStream_t)stream>>>(a, b, out, n);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_bk_shell_dots(const void *dk, int dims, const void *prod_hat, int out_dims,
                                 const int64_t *host_k2_lo, const int64_t *host_k2_hi, const int *host_dst,
                                 int n_tri, double *out, void *stream)
{
    PYL_CHECK_ARG(prod_hat && out && host_k2_lo && host_k2_hi && host_dst, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 4096, "dims out of range");
    PYL_CHECK_ARG(n_tri >= 1 && n_tri <= PYL_BK_MAX_SHELLS, "1..96 triangles per call");
    TriBounds tb;
    tb.n = n_tri;
    long long hi_max = 0;
    for (int t = 0; t < n_tri; t++) {
        PYL_CHECK_ARG(host_k2_lo[t] >= 0 && host_k2_hi[t] >= host_k2_lo[t], "bad shell bounds");
        PYL_CHECK_ARG(host_dst[t] >= 0, "negative output index");
        tb.lo[t] = host_k2_lo[t];
        tb.hi[t] = host_k2_hi[t];
        tb.dst[t] = host_dst[t];
        hi_max = std::max(hi_max, (long long)host_k2_hi[t]);
    }
    int K = 0;
    while ((long long)(K + 1) * (K + 1) < hi_max) K++;
    PYL_CHECK_ARG(out_dims == dims || (2 * K < out_dims && 3 * K < out_dims && out_dims <= dims),
                  "out_dims must equal dims, or exceed 3 K (and 2 K) with K the largest shell wave number");
    const long long side = std::min(K, dims / 2) + std::min(K, (dims - 1) / 2) + 1;
    const long long cube = side * side * (std::min(K, dims / 2) + 1);
    long long blocks = (cube + 255) / 256;
    if (blocks > (long long)num_sms() * 8) blocks = (long long)num_sms() * 8;
    shell_dot_kernel<<<(unsigned)std::max(1LL, blocks), 256, 0, (cudaStream_t)stream>>>(
        (const float2 *)dk, dims, K, out_dims, tb, (const float2 *)prod_hat, out);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

