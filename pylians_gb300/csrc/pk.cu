// Power spectrum: overdensity normalisation, the fused deconvolve + bin +
// Legendre kernel over cuFFT's R2C output, the data-independent mode geometry,
// and in-place deconvolution (keep_deltak / bispectrum input).
//
// Restates the mode loops of library/Pk_library/Pk_library.pyx: Pk 311-381 and
// XPk 625-737 (frequencies 59-64, MAS_correction 86-87, Hermitian-plane skip
// 327-330, 1D bins for |k| <= N/2 364-367, 2D index (kmax_par+1)*k_per+k_par
// 371, 3D l=0,2,4 and phase sums 376-381).  Bin indices come from exact integer
// square roots of kx^2+ky^2+kz^2, so they match the reference's (int)sqrt(double)
// bit for bit.
//
// Mapping: one CTA owns one "plane" of rows that share a coordinate — kx for
// axis 0 and 2, ky for axis 1 — (or a chunk of its rows when the grid is small),
// one warp per row, lanes stride kz.  For axis 0/1 the plane shares k_par, so its
// 1D and 2D bins, like its 3D bins, are accumulated in shared memory; for axis 2
// k_par = kz and the 2D sums go to float64 red.global.add, coalesced along kz.
// Per-CTA partial sums are flushed with float64 atomics into `sums`.
#include <cuda_runtime.h>

#include <math.h>
#include <vector>

#include "common.cuh"

namespace pyl {

struct PkDims {
    int dims, middle, nz, kmax_par, kmax_per, kmax, nb1, nb2, nb3;
};

static PkDims pk_dims(int dims)
{
    PkDims d;
    d.dims = dims;
    d.middle = dims / 2;
    d.nz = dims / 2 + 1;
    d.kmax_par = d.middle;
    d.kmax_per = (int)sqrt((double)d.middle * d.middle * 2.0);
    d.kmax = (int)sqrt((double)d.middle * d.middle * 3.0);
    d.nb1 = d.kmax_par + 1;
    d.nb2 = (d.kmax_par + 1) * (d.kmax_per + 1);
    d.nb3 = d.kmax + 1;
    return d;
}

namespace {

constexpr int MAX_FIELDS = 4;

__device__ __forceinline__ bool hermitian_skip(int kx, int ky, int kz, const PkDims &d)
{
    // kz=0 and kz=middle planes keep one mode of each +-k pair (Pk_library.pyx:327-330)
    const bool even = (d.dims & 1) == 0;
    if (kz == 0 || (kz == d.middle && even)) {
        if (kx < 0) return true;
        if (kx == 0 || (kx == d.middle && even)) return ky < 0;
    }
    return false;
}

// (x / sin x)^p with x = pi k / dims, C(0) = 1, evaluated in float64 (:86-87).
__device__ __forceinline__ double mas_corr_d(int k, int dims, int p)
{
    if (k == 0 || p == 0) return 1.0;
    const double x = (M_PI / dims) * k;
    const double r = x / sin(x);
    double v = 1.0;
    for (int i = 0; i < p; i++) v *= r;
    return v;
}

struct PkArgs {
    const float2 *dk;        // F fields
    const float2 *dk2;       // interlaced partners or null
    long long fstride;       // complex elements between fields
    int F, C, axis, chunks;  // fields, channels, LOS axis, row chunks per plane
    int mas_p[MAX_FIELDS];
    double *sums;
    PkDims d;
};

// smem layout (floats): corr[F][dims] | phase table (2*dims, if interlaced) |
//                       acc3[nb3][3C+F] | acc1[nb1][C] | acc2[kmax_per+1][C] (axis 0/1)
struct PkSmem {
    int corr, ph, acc3, acc1, acc2, total;
};

__host__ __device__ inline PkSmem pk_smem_layout(const PkDims &d, int F, int C, int axis, bool inter)
{
    PkSmem s;
    int o = 0;
    s.corr = o; o += F * d.dims;
    o = (o + 3) & ~3;                 // 16-byte aligned float2 phase table
    s.ph = o; o += inter ? 2 * d.dims : 0;
    s.acc3 = o; o += d.nb3 * (3 * C + F);
    s.acc1 = o; o += d.nb1 * C;
    s.acc2 = o; o += axis == 2 ? 0 : (d.kmax_per + 1) * C;
    s.total = o;
    return s;
}

template <bool INTER>
__global__ void __launch_bounds__(256) pk_bin_kernel(PkArgs a)
{
    extern __shared__ float sm[];
    const PkDims d = a.d;
    const int F = a.F, C = a.C, dims = d.dims;
    const PkSmem L = pk_smem_layout(d, F, C, a.axis, INTER);
    float *corr = sm + L.corr;
    float2 *ph = (float2 *)(sm + L.ph);
    float *acc3 = sm + L.acc3, *acc1 = sm + L.acc1, *acc2 = sm + L.acc2;
    const int slots3 = 3 * C + F;

    for (int i = threadIdx.x; i < F * dims; i += blockDim.x) {
        const int f = i / dims, k = freq_of(i % dims, dims);
        corr[i] = (float)mas_corr_d(k, dims, a.mas_p[f]);
    }
    if (INTER) {
        for (int i = threadIdx.x; i < dims; i += blockDim.x) {
            double s, c;
            sincospi((double)freq_of(i, dims) / dims, &s, &c);
            ph[i] = make_float2((float)c, (float)s);
        }
    }
    for (int i = L.acc3 + threadIdx.x; i < L.total; i += blockDim.x) sm[i] = 0.0f;
    __syncthreads();

    const int plane = blockIdx.x / a.chunks, chunk = blockIdx.x % a.chunks;
    const int rows_per = (dims + a.chunks - 1) / a.chunks;
    const int r0 = chunk * rows_per, r1 = min(dims, r0 + rows_per);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const int middle = d.middle, nz = d.nz;
    const long long m2 = (long long)middle * middle;
    // float64 2D sums for axis 2 (P2 block of `sums`, see the flush below)
    double *gP2 = a.sums + (long long)d.nb3 * (3 * C + F) + (long long)d.nb1 * C;

    for (int r = r0 + warp; r < r1; r += nwarps) {
        const int kxx = a.axis == 1 ? r : plane;
        const int kyy = a.axis == 1 ? plane : r;
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        const long long row = ((long long)kxx * dims + kyy) * nz;
        float cxy[MAX_FIELDS];
#pragma unroll
        for (int f = 0; f < MAX_FIELDS; f++)
            if (f < F) cxy[f] = __fmul_rn(corr[f * dims + kxx], corr[f * dims + kyy]);
        float2 pxy = make_float2(1.0f, 0.0f);
        if (INTER) {
            const float2 px = ph[kxx], py = ph[kyy];
            pxy = make_float2(px.x * py.x - px.y * py.y, px.x * py.y + px.y * py.x);
        }
        const int kperp_row = a.axis == 2 ? isqrt_exact(kx * kx + ky * ky) : 0;
        for (int kz = lane; kz < nz; kz += 32) {
            if (hermitian_skip(kx, ky, kz, d)) continue;
            const int n2 = kx * kx + ky * ky + kz * kz;
            const int ki = isqrt_exact(n2);
            int kpar, kper;
            if (a.axis == 0)      { kpar = kx; kper = isqrt_exact(ky * ky + kz * kz); }
            else if (a.axis == 1) { kpar = ky; kper = isqrt_exact(kx * kx + kz * kz); }
            else                  { kpar = kz; kper = kperp_row; }
            const float mu2 = n2 ? __fdiv_rn((float)(kpar * kpar), (float)n2) : 0.0f;
            const float l2 = 0.5f * (3.0f * mu2 - 1.0f);
            const float l4 = 0.125f * ((35.0f * mu2 - 30.0f) * mu2 + 3.0f);
            if (kpar < 0) kpar = -kpar;
            const bool in1d = (long long)n2 <= m2;
            float re[MAX_FIELDS], im[MAX_FIELDS];
            float2 pz;
            if (INTER) {
                const float2 q = ph[kz];
                pz = make_float2(pxy.x * q.x - pxy.y * q.y, pxy.x * q.y + pxy.y * q.x);
            }
#pragma unroll
            for (int f = 0; f < MAX_FIELDS; f++) {
                if (f >= F) break;
                float2 v = __ldg(a.dk + f * a.fstride + row + kz);
                if (INTER) {
                    const float2 w = __ldg(a.dk2 + f * a.fstride + row + kz);
                    v.x = 0.5f * (v.x + (w.x * pz.x - w.y * pz.y));
                    v.y = 0.5f * (v.y + (w.x * pz.y + w.y * pz.x));
                }
                const float mf = __fmul_rn(cxy[f], corr[f * dims + kz]);
                re[f] = __fmul_rn(v.x, mf);
                im[f] = __fmul_rn(v.y, mf);
            }
            float *b3 = acc3 + ki * slots3;
            int c = 0;
#pragma unroll
            for (int f = 0; f < MAX_FIELDS; f++) {
                if (f >= F) break;
                const float p2 = re[f] * re[f] + im[f] * im[f];
                const float phase = p2 > 0.0f ? atanf(re[f] * rsqrtf(p2)) : 0.0f;
                atomicAdd(b3 + 3 * f, p2);
                atomicAdd(b3 + 3 * f + 1, p2 * l2);
                atomicAdd(b3 + 3 * f + 2, p2 * l4);
                atomicAdd(b3 + 3 * C + f, phase * phase);
                if (in1d) atomicAdd(acc1 + kpar * C + f, p2);
                if (a.axis == 2)
                    atomicAdd(gP2 + ((long long)(d.kmax_par + 1) * kper + kpar) * C + f, (double)p2);
                else
                    atomicAdd(acc2 + kper * C + f, p2);
            }
            c = F;
            for (int i = 0; i < F; i++)
                for (int j = i + 1; j < F; j++, c++) {
                    const float x = re[i] * re[j] + im[i] * im[j];
                    atomicAdd(b3 + 3 * c, x);
                    atomicAdd(b3 + 3 * c + 1, x * l2);
                    atomicAdd(b3 + 3 * c + 2, x * l4);
                    if (in1d) atomicAdd(acc1 + kpar * C + c, x);
                    if (a.axis == 2)
                        atomicAdd(gP2 + ((long long)(d.kmax_par + 1) * kper + kpar) * C + c, (double)x);
                    else
                        atomicAdd(acc2 + kper * C + c, x);
                }
        }
    }
    __syncthreads();

    // flush: sums = P3[nb3][3][C] | PH[nb3][F] | P1[nb1][C] | P2[nb2][C]
    double *P3 = a.sums;
    double *PH = P3 + (long long)d.nb3 * 3 * C;
    double *P1 = PH + (long long)d.nb3 * F;
    double *P2 = P1 + (long long)d.nb1 * C;
    for (int i = threadIdx.x; i < d.nb3 * slots3; i += blockDim.x) {
        const float v = acc3[i];
        if (v == 0.0f) continue;
        const int bin = i / slots3, s = i % slots3;
        if (s < 3 * C) {
            const int ch = s / 3, l = s % 3;
            atomicAdd(P3 + ((long long)bin * 3 + l) * C + ch, (double)v);
        } else {
            atomicAdd(PH + (long long)bin * F + (s - 3 * C), (double)v);
        }
    }
    for (int i = threadIdx.x; i < d.nb1 * C; i += blockDim.x) {
        const float v = acc1[i];
        if (v != 0.0f) atomicAdd(P1 + i, (double)v);
    }
    if (a.axis != 2) {
        const int kpar = abs(freq_of(plane, dims));
        for (int i = threadIdx.x; i < (d.kmax_per + 1) * C; i += blockDim.x) {
            const float v = acc2[i];
            if (v == 0.0f) continue;
            const int kper = i / C, ch = i % C;
            atomicAdd(P2 + ((long long)(d.kmax_par + 1) * kper + kpar) * C + ch, (double)v);
        }
    }
}

// Data-independent per-bin quantities: K1 sum|k_par| and N1 for |k| <= N/2,
// N2, K3 sum|k| and N3 (Pk_library.pyx:364-381).  One CTA per (plane, chunk).
__global__ void __launch_bounds__(256) pk_geometry_kernel(PkDims d, int axis, double *geom)
{
    extern __shared__ double gsm[];
    double *K1 = gsm, *N1 = K1 + d.nb1, *K3 = N1 + d.nb1, *N3 = K3 + d.nb3;
    unsigned *N2 = (unsigned *)(N3 + d.nb3);   // kmax_per+1 (axis 0/1)
    const int nsm = 2 * d.nb1 + 2 * d.nb3;
    for (int i = threadIdx.x; i < nsm; i += blockDim.x) gsm[i] = 0.0;
    for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x) N2[i] = 0;
    __syncthreads();
    const int dims = d.dims, plane = blockIdx.x;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    const long long m2 = (long long)d.middle * d.middle;
    double *gK1 = geom, *gN1 = gK1 + d.nb1, *gN2 = gN1 + d.nb1, *gK3 = gN2 + d.nb2, *gN3 = gK3 + d.nb3;
    for (int r = warp; r < dims; r += nwarps) {
        const int kxx = axis == 1 ? r : plane, kyy = axis == 1 ? plane : r;
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        for (int kz = lane; kz < d.nz; kz += 32) {
            if (hermitian_skip(kx, ky, kz, d)) continue;
            const int n2 = kx * kx + ky * ky + kz * kz;
            const int ki = isqrt_exact(n2);
            int kpar, kper;
            if (axis == 0)      { kpar = kx; kper = isqrt_exact(ky * ky + kz * kz); }
            else if (axis == 1) { kpar = ky; kper = isqrt_exact(kx * kx + kz * kz); }
            else                { kpar = kz; kper = isqrt_exact(kx * kx + ky * ky); }
            if (kpar < 0) kpar = -kpar;
            if ((long long)n2 <= m2) {
                atomicAdd(K1 + kpar, (double)kpar);
                atomicAdd(N1 + kpar, 1.0);
            }
            atomicAdd(K3 + ki, sqrt((double)n2));
            atomicAdd(N3 + ki, 1.0);
            if (axis == 2) atomicAdd(gN2 + (long long)(d.kmax_par + 1) * kper + kpar, 1.0);
            else atomicAdd(N2 + kper, 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < d.nb1; i += blockDim.x) {
        if (N1[i] != 0.0) { atomicAdd(gK1 + i, K1[i]); atomicAdd(gN1 + i, N1[i]); }
    }
    for (int i = threadIdx.x; i < d.nb3; i += blockDim.x) {
        if (N3[i] != 0.0) { atomicAdd(gK3 + i, K3[i]); atomicAdd(gN3 + i, N3[i]); }
    }
    if (axis != 2) {
        const int kpar = abs(freq_of(plane, dims));
        for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x)
            if (N2[i]) atomicAdd(gN2 + (long long)(d.kmax_par + 1) * i + kpar, (double)N2[i]);
    }
}

__global__ void __launch_bounds__(256) deconvolve_kernel(float2 *dk, const float2 *dk2, PkDims d, int p)
{
    const int dims = d.dims;
    const long long total = (long long)dims * dims * d.nz;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const int kz = (int)(i % d.nz);
        const long long rr = i / d.nz;
        const int kyy = (int)(rr % dims), kxx = (int)(rr / dims);
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        float2 v = dk[i];
        if (dk2) {
            double s, c;
            sincospi((double)(kx + ky + kz) / dims, &s, &c);
            const float2 w = dk2[i];
            const float pc = (float)c, ps = (float)s;
            v.x = 0.5f * (v.x + (w.x * pc - w.y * ps));
            v.y = 0.5f * (v.y + (w.x * ps + w.y * pc));
        }
        const float mf = (float)(mas_corr_d(kx, dims, p) * mas_corr_d(ky, dims, p) * mas_corr_d(kz, dims, p));
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

extern "C" size_t pyl_pk_workspace_size(int dims, int n_fields, int axis)
{
    (void)dims; (void)n_fields; (void)axis;
    return 0;
}

extern "C" int pyl_pk_bin(const void *dk, const void *dk_interlaced, int n_fields, int64_t field_stride,
                          int dims, int axis, const int *host_mas_p, double *sums, void *workspace,
                          size_t workspace_bytes, void *stream)
{
    (void)workspace; (void)workspace_bytes;
    PYL_CHECK_ARG(dk != nullptr && sums != nullptr && host_mas_p != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    PYL_CHECK_ARG(n_fields >= 1, "need at least one field");
    if (n_fields > MAX_FIELDS) {
        set_error("pyl_pk_bin: at most 4 fields per call; bin larger sets pairwise");
        return PYL_ERR_UNSUPPORTED;
    }
    const PkDims d = pk_dims(dims);
    const long long half = (long long)dims * dims * d.nz;
    PYL_CHECK_ARG(n_fields == 1 || field_stride >= half, "field_stride smaller than one field");
    PkArgs a;
    a.dk = (const float2 *)dk;
    a.dk2 = (const float2 *)dk_interlaced;
    a.fstride = field_stride;
    a.F = n_fields;
    a.C = n_fields + n_fields * (n_fields - 1) / 2;
    a.axis = axis;
    a.sums = sums;
    a.d = d;
    for (int f = 0; f < MAX_FIELDS; f++) {
        a.mas_p[f] = f < n_fields ? host_mas_p[f] : 0;
        PYL_CHECK_ARG(a.mas_p[f] >= 0 && a.mas_p[f] <= 4, "MAS exponent must be 0..4");
    }
    const bool inter = dk_interlaced != nullptr;
    const PkSmem L = pk_smem_layout(d, a.F, a.C, axis, inter);
    const size_t smem = sizeof(float) * (size_t)L.total;
    if (smem > 220 * 1024) {
        set_error("pyl_pk_bin: bins for this grid and field count exceed shared memory");
        return PYL_ERR_UNSUPPORTED;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * pyl_pk_sums_len(dims, n_fields), st));
    a.chunks = 1;
    while ((long long)dims * a.chunks < 2LL * num_sms() && a.chunks * 8 < dims) a.chunks *= 2;
    const unsigned blocks = (unsigned)(dims * a.chunks);
    static size_t done_t = 0, done_f = 0;
    if (inter) {
        PYL_CUDA(ensure_smem(pk_bin_kernel<true>, smem, &done_t));
        pk_bin_kernel<true><<<blocks, 256, smem, st>>>(a);
    } else {
        PYL_CUDA(ensure_smem(pk_bin_kernel<false>, smem, &done_f));
        pk_bin_kernel<false><<<blocks, 256, smem, st>>>(a);
    }
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_pk_geometry(int dims, int axis, double *geom, void *stream)
{
    PYL_CHECK_ARG(geom != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    const PkDims d = pk_dims(dims);
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(geom, 0, sizeof(double) * pyl_pk_geometry_len(dims), st));
    const size_t smem = sizeof(double) * (2 * d.nb1 + 2 * d.nb3) + sizeof(unsigned) * (d.kmax_per + 1);
    static size_t done = 0;
    PYL_CUDA(ensure_smem(pk_geometry_kernel, smem, &done));
    pk_geometry_kernel<<<dims, 256, smem, st>>>(d, axis, geom);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_mas_deconvolve(void *dk, const void *dk_interlaced, int dims, int mas_p, void *stream)
{
    PYL_CHECK_ARG(dk != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(mas_p >= 0 && mas_p <= 4, "MAS exponent must be 0..4");
    const PkDims d = pk_dims(dims);
    const long long total = (long long)dims * dims * d.nz;
    deconvolve_kernel<<<blocks_for(total, 256), 256, 0, (cudaStream_t)stream>>>(
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
