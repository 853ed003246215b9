// Fused P(k) / XPk binning over cuFFT's R2C output, and the mode geometry.
//
// Restates the mode loops of library/Pk_library/Pk_library.pyx: Pk 311-381 and
// XPk 625-737 (frequencies 59-64, MAS_correction 86-87, Hermitian-plane skip
// 327-330, 1D bins for |k| <= N/2 364-367, 2D index (kmax_par+1)*k_per+k_par
// 371, 3D l=0,2,4 and phase sums 376-381).  Bin indices are exact integer
// square roots of kx^2+ky^2+kz^2, equal to the reference's (int)sqrt(double).
//
// Mapping: a warp walks a row (fixed kx, ky) 32 consecutive kz at a time, so
// its loads are coalesced.  Along kz the 3D bin, and for axis 0/1 the 2D bin
// k_per, never decrease, so a warp-level segmented sum (shuffles) collapses
// each run of equal bins and only the run's last lane adds to shared memory.
//   axis 0/1: a CTA owns rows of one plane (fixed kx for axis 0, ky for axis 1),
//             which share k_par: 1D sums stay in registers, 2D sums (by k_per)
//             in shared memory.
//   axis 2:   k_par = kz.  Rows are visited in order of their k_per ring
//             (a counting sort of the rows, done on the device each call), and
//             each warp keeps private kz-indexed 2D and 1D sums in shared
//             memory, flushed to float64 global sums when its ring changes.
// Per-CTA float32 partial sums are flushed into the float64 `sums` with
// float64 atomics.
#include <cuda_runtime.h>

#include "pk_common.cuh"

namespace pyl {
namespace {

constexpr int MAX_FIELDS = 4;
constexpr int NW = 8;                    // warps per CTA (256 threads)
constexpr unsigned FULL = 0xffffffffu;
constexpr int KEY_NONE = 0x7fffffff;

struct Seg {
    int start;
    bool tail;
};

// Segments of equal keys across the lanes of a warp (keys non-decreasing).
__device__ __forceinline__ Seg seg_of(int key)
{
    const int lane = threadIdx.x & 31;
    const int prev = __shfl_up_sync(FULL, key, 1);
    const bool head = lane == 0 || key != prev;
    const unsigned hm = __ballot_sync(FULL, head);
    Seg s;
    s.start = 31 - __clz(hm & (FULL >> (31 - lane)));
    s.tail = lane == 31 || ((hm >> (lane + 1)) & 1u);
    return s;
}

// Inclusive segmented sum; a segment's total sits on its tail lane.
template <typename T>
__device__ __forceinline__ T seg_sum(T v, int start)
{
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const T y = __shfl_up_sync(FULL, v, o);
        if (lane - o >= start) v += y;
    }
    return v;
}

struct BinArgs {
    const float2 *dk, *dk2;
    long long fstride;
    int F, C, axis;
    int mas_p[MAX_FIELDS];
    double *sums;        // P3 | PH | P1 | P2 (float64)
    double *geom;        // K1 | N1 | N2 | K3 | N3 (geometry kernel)
    PkDims d;
    const unsigned *rows;  // axis 2: row ids (kxx*dims + kyy) sorted by k_per ring
    int chunks;            // axis 0/1: CTAs per plane
    int rows_per_cta;      // axis 2: table entries per CTA
    int warp_arrays;       // axis 2: per-warp kz arrays in shared memory
    float *part;           // one field: per-CTA partial sums in global memory (null: shared memory)
    int part_stride;       // floats per CTA: 3D bins x 4, then k_per bins (axes 0/1)
    const pyl_pk_item *items;  // batched one-field spectra: item blockIdx.y (dk, dk2, sums, MAS)
};

struct BinSmem {
    int corr, ph, acc3, acc1, acc2, w, total;
};

__host__ __device__ inline BinSmem bin_smem(const PkDims &d, int F, int C, int axis, bool inter,
                                            int warp_arrays)
{
    BinSmem s;
    int o = 0;
    s.corr = o; o += F * d.dims;
    o = (o + 3) & ~3;                   // 16-byte aligned float2 phase table
    s.ph = o; o += inter ? 2 * d.dims : 0;
    s.acc3 = o; o += d.nb3 * (3 * C + F);
    s.acc1 = o; o += d.nb1 * C;
    s.acc2 = o; o += axis == 2 ? 0 : (d.kmax_per + 1) * C;
    s.w = o; o += (axis == 2 && warp_arrays) ? NW * 2 * d.nz * C : 0;
    s.total = o;
    return s;
}

// Row sequence of CTA blockIdx.x: axis 0/1 interleave the rows of one plane
// among the warps; axis 2 gives each warp a contiguous run of the ring table.
struct RowIter {
    int first, step, count;    // positions: first, first+step, ... (count of them)
    int plane;
};

__device__ __forceinline__ RowIter row_iter(const BinArgs &a, int warp)
{
    RowIter it;
    const int dims = a.d.dims;
    if (a.axis != 2) {
        it.plane = blockIdx.x / a.chunks;
        const int chunk = blockIdx.x % a.chunks;
        const int per = (dims + a.chunks - 1) / a.chunks;
        const int r0 = chunk * per, r1 = min(dims, r0 + per);
        it.first = r0 + warp;
        it.step = NW;
        it.count = it.first < r1 ? (r1 - it.first + NW - 1) / NW : 0;
    } else {
        it.plane = 0;
        const long long total = (long long)dims * dims;
        const long long b = (long long)blockIdx.x * a.rows_per_cta;
        const long long e = min(total, b + a.rows_per_cta);
        const int L = (a.rows_per_cta + NW - 1) / NW;
        const long long wb = b + (long long)warp * L;
        it.first = (int)wb;
        it.step = 1;
        it.count = wb < e ? (int)min((long long)L, e - wb) : 0;
    }
    return it;
}

__device__ __forceinline__ void row_coords(const BinArgs &a, const RowIter &it, int pos, int &kxx, int &kyy)
{
    const int dims = a.d.dims;
    if (a.axis == 0)      { kxx = it.plane; kyy = pos; }
    else if (a.axis == 1) { kxx = pos; kyy = it.plane; }
    else {
        const unsigned r = a.rows[pos];
        kxx = (int)(r / (unsigned)dims);
        kyy = (int)(r % (unsigned)dims);
    }
}

template <bool INTER, int AXIS, int F>
__global__ void __launch_bounds__(256) pk_bin_kernel(BinArgs a)
{
    constexpr int C = F + F * (F - 1) / 2;          // autos, then cross pairs
    extern __shared__ float sm[];
    const PkDims d = a.d;
    const int dims = d.dims, nz = d.nz;
    const BinSmem L = bin_smem(d, F, C, AXIS, INTER, a.warp_arrays);
    float *corr = sm + L.corr;
    float2 *ph = (float2 *)(sm + L.ph);
    float *acc3 = sm + L.acc3, *acc1 = sm + L.acc1, *acc2 = sm + L.acc2;
    const int slots3 = 3 * C + F;
    // Per-axis tables in float32 (fp64 is slow on this part; each factor is within
    // an ulp of the reference's float64 value before the float32 product).
    for (int i = threadIdx.x; i < F * dims; i += blockDim.x) {
        const int f = i / dims;
        const int p = f == 0 ? a.mas_p[0] : f == 1 ? a.mas_p[1] : f == 2 ? a.mas_p[2] : a.mas_p[3];
        corr[i] = mas_corr_f(freq_of(i % dims, dims), dims, p);
    }
    if (INTER) {
        for (int i = threadIdx.x; i < dims; i += blockDim.x) {
            float s, c;
            sincospif((float)freq_of(i, dims) / (float)dims, &s, &c);
            ph[i] = make_float2(c, s);
        }
    }
    for (int i = L.acc3 + threadIdx.x; i < L.total; i += blockDim.x) sm[i] = 0.0f;
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long m2 = (long long)d.middle * d.middle;
    double *P3 = a.sums;
    double *PH = P3 + (long long)d.nb3 * 3 * C;
    double *P1 = PH + (long long)d.nb3 * F;
    double *P2 = P1 + (long long)d.nb1 * C;
    float *w2 = sm + L.w + warp * 2 * nz * C;      // axis 2 with warp arrays
    float *w1 = w2 + nz * C;
    float r1[C];
#pragma unroll
    for (int c = 0; c < C; c++) r1[c] = 0.0f;
    int cur_ring = -1;

    const RowIter it = row_iter(a, warp);
    for (int q = 0; q < it.count; q++) {
        int kxx, kyy;
        row_coords(a, it, it.first + q * it.step, kxx, kyy);
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        const long long row = ((long long)kxx * dims + kyy) * nz;
        float cxy[F];
#pragma unroll
        for (int f = 0; f < F; f++) cxy[f] = __fmul_rn(corr[f * dims + kxx], corr[f * dims + kyy]);
        float2 pxy = make_float2(1.0f, 0.0f);
        if (INTER) {
            const float2 px = ph[kxx], py = ph[kyy];
            pxy = make_float2(px.x * py.x - px.y * py.y, px.x * py.y + px.y * py.x);
        }
        const int ring = AXIS == 2 ? isqrt_exact(kx * kx + ky * ky) : 0;
        if (AXIS == 2 && a.warp_arrays && ring != cur_ring) {
            if (cur_ring >= 0) {
                for (int kz = lane; kz < nz; kz += 32)
                    for (int c = 0; c < C; c++) {
                        const float v = w2[kz * C + c];
                        if (v != 0.0f) {
                            atomicAdd(P2 + ((long long)(d.kmax_par + 1) * cur_ring + kz) * C + c, (double)v);
                            w2[kz * C + c] = 0.0f;
                        }
                    }
            }
            cur_ring = ring;
        }
        for (int kz0 = 0; kz0 < nz; kz0 += 32) {
            const int kz = kz0 + lane;
            const bool valid = kz < nz;
            const bool live = valid && !hermitian_skip(kx, ky, kz, d);
            const int n2 = kx * kx + ky * ky + kz * kz;
            const int ki = valid ? isqrt_fast(n2) : KEY_NONE;
            int kpar, kper;
            if (AXIS == 0)      { kpar = kx; kper = isqrt_fast(ky * ky + kz * kz); }
            else if (AXIS == 1) { kpar = ky; kper = isqrt_fast(kx * kx + kz * kz); }
            else                { kpar = kz; kper = ring; }
            const float mu2 = n2 ? __fdividef((float)(kpar * kpar), (float)n2) : 0.0f;
            const float l2 = 0.5f * (3.0f * mu2 - 1.0f);
            const float l4 = 0.125f * ((35.0f * mu2 - 30.0f) * mu2 + 3.0f);
            if (kpar < 0) kpar = -kpar;
            const bool in1d = (long long)n2 <= m2;
            float re[F], im[F];
            float2 pz = make_float2(1.0f, 0.0f);
            if (INTER && valid) {
                const float2 t = ph[kz];
                pz = make_float2(pxy.x * t.x - pxy.y * t.y, pxy.x * t.y + pxy.y * t.x);
            }
#pragma unroll
            for (int f = 0; f < F; f++) {
                re[f] = 0.0f;
                im[f] = 0.0f;
                if (live) {
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
            }
            // channel values: autos then cross pairs (i<j)
            float val[C];
#pragma unroll
            for (int f = 0; f < F; f++) val[f] = re[f] * re[f] + im[f] * im[f];
#pragma unroll
            for (int i = 0, c = F; i < F; i++)
#pragma unroll
                for (int j = i + 1; j < F; j++, c++) val[c] = re[i] * re[j] + im[i] * im[j];
            // 3D: segmented sums by |k| bin
            const Seg s3 = seg_of(ki);
            float *b3 = acc3 + (ki == KEY_NONE ? 0 : ki) * slots3;
            const bool t3 = s3.tail && ki != KEY_NONE;
#pragma unroll
            for (int c = 0; c < C; c++) {
                const float v0 = seg_sum(val[c], s3.start);
                const float v2 = seg_sum(val[c] * l2, s3.start);
                const float v4 = seg_sum(val[c] * l4, s3.start);
                if (t3) {
                    atomicAdd(b3 + 3 * c, v0);
                    atomicAdd(b3 + 3 * c + 1, v2);
                    atomicAdd(b3 + 3 * c + 2, v4);
                }
            }
#pragma unroll
            for (int f = 0; f < F; f++) {
                const float p2 = val[f];
                // phase = atan2(Re d, |d|) = atan(Re d / |d|), |Re d / |d|| <= 1
                const float phase = p2 > 0.0f ? atan_unit(re[f] * rsqrtf(p2)) : 0.0f;
                const float vph = seg_sum(phase * phase, s3.start);
                if (t3) atomicAdd(b3 + 3 * C + f, vph);
            }
            if (AXIS != 2) {
                // 2D by k_per (shared memory), 1D by the plane's k_par (registers)
                const Seg s2 = seg_of(valid ? kper : KEY_NONE);
                const bool t2 = s2.tail && valid;
#pragma unroll
                for (int c = 0; c < C; c++) {
                    const float v = seg_sum(val[c], s2.start);
                    if (t2) atomicAdd(acc2 + kper * C + c, v);
                    if (in1d) r1[c] += val[c];
                }
            } else if (a.warp_arrays) {
                if (valid) {
#pragma unroll
                    for (int c = 0; c < C; c++) {
                        w2[kz * C + c] += val[c];
                        if (in1d) w1[kz * C + c] += val[c];
                    }
                }
            } else if (live) {
#pragma unroll
                for (int c = 0; c < C; c++) {
                    atomicAdd(P2 + ((long long)(d.kmax_par + 1) * ring + kz) * C + c, (double)val[c]);
                    if (in1d) atomicAdd(P1 + (long long)kz * C + c, (double)val[c]);
                }
            }
        }
    }
    // per-warp flushes
    if (AXIS != 2) {
#pragma unroll
        for (int c = 0; c < C; c++) {
            float v = r1[c];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
            if (lane == 0 && v != 0.0f) atomicAdd(acc1 + abs(freq_of(it.plane, dims)) * C + c, v);
        }
    } else if (a.warp_arrays) {
        for (int kz = lane; kz < nz; kz += 32)
            for (int c = 0; c < C; c++) {
                const float v2 = w2[kz * C + c];
                if (cur_ring >= 0 && v2 != 0.0f)
                    atomicAdd(P2 + ((long long)(d.kmax_par + 1) * cur_ring + kz) * C + c, (double)v2);
                const float v1 = w1[kz * C + c];
                if (v1 != 0.0f) atomicAdd(P1 + (long long)kz * C + c, (double)v1);
            }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < d.nb3 * slots3; i += blockDim.x) {
        const float v = acc3[i];
        if (v == 0.0f) continue;
        const int bin = i / slots3, s = i % slots3;
        if (s < 3 * C) atomicAdd(P3 + ((long long)bin * 3 + s % 3) * C + s / 3, (double)v);
        else atomicAdd(PH + (long long)bin * F + (s - 3 * C), (double)v);
    }
    if (AXIS != 2) {
        for (int i = threadIdx.x; i < d.nb1 * C; i += blockDim.x) {
            const float v = acc1[i];
            if (v != 0.0f) atomicAdd(P1 + i, (double)v);
        }
        const int kpar = abs(freq_of(it.plane, dims));
        for (int i = threadIdx.x; i < (d.kmax_per + 1) * C; i += blockDim.x) {
            const float v = acc2[i];
            if (v == 0.0f) continue;
            atomicAdd(P2 + ((long long)(d.kmax_par + 1) * (i / C) + kpar) * C + i % C, (double)v);
        }
    }
}

// Single-field P(k) (F = 1), sequential per lane.  For each row a warp first
// computes, with coalesced loads along kz, every mode's power |d|^2 and phase^2
// (interlacing and the MAS deconvolution included) into a per-warp staging
// array; then each lane walks its own run of `chunk` consecutive kz, updating
// the |k| bin and the k_per bin incrementally (along kz each grows by at most
// one per step) and adding to shared memory only when a bin changes.  Staging:
// mode kz at kz + kz / chunk (one pad slot per run; chunk even, so lane runs are
// an odd number of 8-byte slots apart and the sequential reads do not conflict).
struct SeqSmem {
    int corr, ph, acc3, acc1, acc2, w, stage, total;
};

// part: the 3D and k_per flushes go to global partial sums, so their shared
// arrays are left out (more resident CTAs).
__host__ __device__ inline SeqSmem seq_smem(const PkDims &d, int axis, bool inter, int chunk, bool part)
{
    SeqSmem s;
    int o = 0;
    s.corr = o; o += d.dims;
    o = (o + 3) & ~3;
    s.ph = o; o += inter ? 2 * d.dims : 0;
    s.acc3 = o; o += part ? 0 : d.nb3 * 4;
    s.acc1 = o; o += d.nb1;
    s.acc2 = o; o += (axis == 2 || part) ? 0 : d.kmax_per + 1;
    s.w = o; o += axis == 2 ? NW * 2 * d.nz : 0;
    o = (o + 3) & ~3;
    s.stage = o; o += NW * 2 * 32 * (chunk + 1);
    s.total = o;
    return s;
}

inline int seq_chunk(int nz)
{
    int c = (nz + 31) / 32;
    return c + (c & 1);
}

// umulhi(kz, magic) = kz / chunk for the kz < 2^13 of any grid here
inline unsigned seq_chunk_magic(int chunk) { return (unsigned)((0x100000000ull + chunk - 1) / chunk); }


// ---- the four sign rows of a representative (|kx|, |ky|) ----------------------------
// Every bin index (|k|^2 = kx^2 + ky^2 + kz^2, k_per^2, k_par^2 for any line of
// sight) and every Legendre weight depends on kx^2 and ky^2 only, so the rows
// (+-kx, +-ky) share their bins at every kz: the one-field kernels sum the (up to
// four) modes' |d|^2 and phase^2 at each kz and walk the bins once for all of
// them (a quarter of the bin walk, its flushes and the staging of one row at a
// time; the loads and per-mode arithmetic are the same).  The representatives are
// 0..dims/2 on each axis; 0 and dims/2 have no partner.  Each mode's power is
// |v|^2 mf^2 with mf the deconvolution factor, shared by the four modes; its phase
// atan(Re v / |v|) does not depend on mf > 0.
__host__ __device__ inline int sym_groups(int dims) { return dims / 2 + 1; }

struct SignRows {
    long long off[4];       // row r = (y sign << 1) | x sign
    float2 pxy[4];          // interlacing phase exp(i pi (kx + ky) / dims) of each row
    unsigned skip0, skipm;  // rows whose kz = 0 / kz = dims/2 modes the Hermitian skip drops
    unsigned used;          // rows that exist (a representative without partner repeats row 0)
};

template <bool INTER>
__device__ __forceinline__ SignRows sign_rows(int xr, int yr, const PkDims &d, const float2 *ph)
{
    const int dims = d.dims;
    const bool even = (dims & 1) == 0;
    const int nx = (xr == 0 || 2 * xr == dims) ? 1 : 2, ny = (yr == 0 || 2 * yr == dims) ? 1 : 2;
    SignRows R;
    R.skip0 = R.skipm = 0u;
    R.used = 1u | (nx == 2 ? 2u : 0u) | (ny == 2 ? 4u : 0u) | (nx == 2 && ny == 2 ? 8u : 0u);
#pragma unroll
    for (int r = 0; r < 4; r++) {
        const int kxx = ((r & 1) && nx == 2) ? dims - xr : xr;     // in range for every r
        const int kyy = ((r & 2) && ny == 2) ? dims - yr : yr;
        R.off[r] = ((long long)kxx * dims + kyy) * d.nz;
        const int kx = freq_of(kxx, dims), ky = freq_of(kyy, dims);
        R.pxy[r] = make_float2(1.0f, 0.0f);
        if (INTER) {
            const float2 px = ph[kxx], py = ph[kyy];
            R.pxy[r] = make_float2(px.x * py.x - px.y * py.y, px.x * py.y + px.y * py.x);
        }
        if (hermitian_skip(kx, ky, 0, d)) R.skip0 |= 1u << r;
        if (even && hermitian_skip(kx, ky, d.middle, d)) R.skipm |= 1u << r;
    }
    return R;
}

// Pass 1 for one representative: the summed power and phase^2 of its rows at each
// kz (lanes along kz, coalesced), into the warp's staging array at kz + kz / chunk.
// All four rows are loaded (in range for every r), so an iteration's loads issue
// together.
template <bool INTER>
__device__ __forceinline__ void stage_sign_rows(const SignRows &R, const float2 *__restrict__ dk,
                                                const float2 *__restrict__ dk2, const float *corr,
                                                const float2 *ph, float cxy, const PkDims &d, float2 *stage,
                                                unsigned chunk_magic, int lane)
{
    const bool even = (d.dims & 1) == 0;
#pragma unroll 2
    for (int kz = lane; kz < d.nz; kz += 32) {
        float2 t = make_float2(1.0f, 0.0f);
        if (INTER) t = ph[kz];
        const unsigned skip = kz == 0 ? R.skip0 : ((even && kz == d.middle) ? R.skipm : 0u);
        const unsigned take = R.used & ~skip;
        float2 v[4], w[4];
#pragma unroll
        for (int r = 0; r < 4; r++) {
            v[r] = __ldg(dk + R.off[r] + kz);
            if (INTER) w[r] = __ldg(dk2 + R.off[r] + kz);
        }
        float a2s = 0.0f, p2s = 0.0f;
#pragma unroll
        for (int r = 0; r < 4; r++) {
            float2 u = v[r];
            if (INTER) {
                const float2 pz = make_float2(R.pxy[r].x * t.x - R.pxy[r].y * t.y, R.pxy[r].x * t.y + R.pxy[r].y * t.x);
                u.x = 0.5f * (u.x + (w[r].x * pz.x - w[r].y * pz.y));
                u.y = 0.5f * (u.y + (w[r].x * pz.y + w[r].y * pz.x));
            }
            const float a2 = u.x * u.x + u.y * u.y;
            const float phase = a2 > 0.0f ? atan_unit(u.x * rsqrtf(a2)) : 0.0f;
            if ((take >> r) & 1u) {
                a2s += a2;
                p2s += phase * phase;
            }
        }
        const float mf = __fmul_rn(cxy, corr[kz]);
        stage[kz + __umulhi((unsigned)kz, chunk_magic)] = make_float2(a2s * (mf * mf), p2s);
    }
}

// One field, axis 2 (axes 0/1: pk_bin_sym_kernel below): the representatives
// (|kx|, |ky|) in the order of their k_per ring (a.rows), each the four sign rows of
// sign_rows; per-warp kz-indexed 2D and 1D sums, flushed when the ring changes.
// BATCH: blockIdx.y picks an item of a.items (its field, partner, sums, MAS and
// its slice of the partial sums); the CTA partition along blockIdx.x is a
// one-field call's.
template <bool INTER, int AXIS, bool BATCH>
__global__ void __launch_bounds__(256) pk_bin_seq_kernel(BinArgs a, int chunk, unsigned chunk_magic)
{
    static_assert(AXIS == 2, "axis 2 (rows in k_per ring order)");
    extern __shared__ float sm[];
    const PkDims d = a.d;
    const int dims = d.dims, nz = d.nz;
    const SeqSmem L = seq_smem(d, AXIS, INTER, chunk, a.part != nullptr);
    // one field: the kernel parameters themselves (read from the constant bank,
    // no registers held); batched: the item's record
    const float2 *bdk = nullptr, *bdk2 = nullptr;
    double *bsums = nullptr;
    int bmas = 0;
    if (BATCH) {
        const pyl_pk_item it = a.items[blockIdx.y];
        bdk = (const float2 *)it.dk;
        bdk2 = (const float2 *)it.dk_interlaced;
        bsums = it.sums;
        bmas = it.mas_p;
    }
    const float2 *dk = BATCH ? bdk : a.dk;
    const float2 *dk2 = BATCH ? bdk2 : a.dk2;
    double *sums = BATCH ? bsums : a.sums;
    const int mas = BATCH ? bmas : a.mas_p[0];
    float *part_base = (BATCH && a.part) ? a.part + (long long)blockIdx.y * gridDim.x * a.part_stride : a.part;
    float *corr = sm + L.corr;
    float2 *ph = (float2 *)(sm + L.ph);
    float *acc3 = sm + L.acc3;
    for (int i = threadIdx.x; i < dims; i += blockDim.x) corr[i] = mas_corr_f(freq_of(i, dims), dims, mas);
    if (INTER) {
        for (int i = threadIdx.x; i < dims; i += blockDim.x) {
            float s, c;
            sincospif((float)freq_of(i, dims) / (float)dims, &s, &c);
            ph[i] = make_float2(c, s);
        }
    }
    for (int i = L.acc3 + threadIdx.x; i < L.stage; i += blockDim.x) sm[i] = 0.0f;
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m2 = d.middle * d.middle;
    double *P3 = sums;
    double *PH = P3 + (long long)d.nb3 * 3;
    double *P1 = PH + d.nb3;
    double *P2 = P1 + d.nb1;
    float2 *stage = (float2 *)(sm + L.stage) + warp * 32 * (chunk + 1);
    float *w2 = sm + L.w + warp * 2 * nz;             // axis 2: per-warp kz arrays
    float *w1 = w2 + nz;
    const int kz_begin = lane * chunk;
    const int kz_end = min(nz, kz_begin + chunk);
    float *part = part_base ? part_base + (long long)blockIdx.x * a.part_stride : nullptr;
    int cur_ring = -1;

    // the CTA's run of the representatives' table (ring order), split among the warps
    const int G = sym_groups(dims);
    const long long total = (long long)G * G;
    const long long b = (long long)blockIdx.x * a.rows_per_cta;
    const long long e = min(total, b + a.rows_per_cta);
    const int per_warp = (a.rows_per_cta + NW - 1) / NW;
    const long long wb = b + (long long)warp * per_warp;
    const int count = wb < e ? (int)min((long long)per_warp, e - wb) : 0;
    for (int j = 0; j < count; j++) {
        const unsigned rid = a.rows[wb + j];
        const int kx = (int)(rid / (unsigned)G), ky = (int)(rid % (unsigned)G);    // representatives
        const int ring = isqrt_exact(kx * kx + ky * ky);
        if (ring != cur_ring) {
            __syncwarp();
            if (cur_ring >= 0) {
                for (int kz = lane; kz < nz; kz += 32) {
                    const float v = w2[kz];
                    if (v != 0.0f) {
                        atomicAdd(P2 + (long long)(d.kmax_par + 1) * cur_ring + kz, (double)v);
                        w2[kz] = 0.0f;
                    }
                }
            }
            cur_ring = ring;
            __syncwarp();
        }
        const SignRows R = sign_rows<INTER>(kx, ky, d, ph);
        stage_sign_rows<INTER>(R, dk, dk2, corr, ph, __fmul_rn(corr[kx], corr[ky]), d, stage, chunk_magic, lane);
        __syncwarp();
        // pass 2: this lane's run of kz, sums kept while the bins stay the same
        if (kz_begin < kz_end) {
            const int kxy2 = kx * kx + ky * ky;
            int kz = kz_begin;
            int n2 = kxy2 + kz * kz;
            int ki = isqrt_exact(n2);
            float s0 = 0.0f, s2 = 0.0f, s4 = 0.0f, sp = 0.0f;
            const float2 *run = stage + lane * (chunk + 1);
            for (; kz < kz_end; kz++) {
                const float2 e = run[kz - kz_begin];
                const float val = e.x;
                const float mu2 = n2 ? __fdividef((float)(kz * kz), (float)n2) : 0.0f;
                const float l2 = 0.5f * (3.0f * mu2 - 1.0f);
                const float l4 = 0.125f * ((35.0f * mu2 - 30.0f) * mu2 + 3.0f);
                s0 += val;
                s2 += val * l2;
                s4 += val * l4;
                sp += e.y;
                w2[kz] += val;
                if (n2 <= m2) w1[kz] += val;
                // step to kz + 1
                n2 += 2 * kz + 1;
                const bool new3 = (ki + 1) * (ki + 1) <= n2;
                if (new3 || kz + 1 == kz_end) {
                    if (part) {                         // one vector reduction in L2
                        atomicAdd(reinterpret_cast<float4 *>(part + ki * 4), make_float4(s0, s2, s4, sp));
                    } else {                            // float shared atomics: compare-and-swap loops
                        float *b3 = acc3 + ki * 4;
                        if (s0 != 0.0f) atomicAdd(b3, s0);
                        if (s2 != 0.0f) atomicAdd(b3 + 1, s2);
                        if (s4 != 0.0f) atomicAdd(b3 + 2, s4);
                        if (sp != 0.0f) atomicAdd(b3 + 3, sp);
                    }
                    s0 = s2 = s4 = sp = 0.0f;
                    ki += new3 ? 1 : 0;
                }
            }
        }
        __syncwarp();
    }
    // per-warp flushes
    __syncwarp();
    for (int kz = lane; kz < nz; kz += 32) {
        const float v2 = w2[kz];
        if (cur_ring >= 0 && v2 != 0.0f)
            atomicAdd(P2 + (long long)(d.kmax_par + 1) * cur_ring + kz, (double)v2);
        const float v1 = w1[kz];
        if (v1 != 0.0f) atomicAdd(P1 + kz, (double)v1);
    }
    __syncthreads();
    if (!part) {
        for (int i = threadIdx.x; i < d.nb3 * 4; i += blockDim.x) {
            const float v = acc3[i];
            if (v == 0.0f) continue;
            const int bin = i >> 2, s = i & 3;
            if (s < 3) atomicAdd(P3 + (long long)bin * 3 + s, (double)v);
            else atomicAdd(PH + bin, (double)v);
        }
    }
}

// ---- axes 0/1 ---------------------------------------------------------------------
// CTA blockIdx.x / chunks takes plane representative p (|k_par| with the line of
// sight along x for axis 0, y for axis 1), its warps the row representatives q
// of the CTA's chunk; each (p, q) is the four sign rows of sign_rows.
template <bool INTER, int AXIS, bool BATCH>
__global__ void __launch_bounds__(256, INTER ? 3 : 4) pk_bin_sym_kernel(BinArgs a, int chunk, unsigned chunk_magic)
{
    static_assert(AXIS == 0 || AXIS == 1, "axes 0 and 1");
    extern __shared__ float sm[];
    const PkDims d = a.d;
    const int dims = d.dims, nz = d.nz;
    const SeqSmem L = seq_smem(d, AXIS, INTER, chunk, a.part != nullptr);
    const float2 *bdk = nullptr, *bdk2 = nullptr;
    double *bsums = nullptr;
    int bmas = 0;
    if (BATCH) {
        const pyl_pk_item it = a.items[blockIdx.y];
        bdk = (const float2 *)it.dk;
        bdk2 = (const float2 *)it.dk_interlaced;
        bsums = it.sums;
        bmas = it.mas_p;
    }
    const float2 *dk = BATCH ? bdk : a.dk;
    const float2 *dk2 = BATCH ? bdk2 : a.dk2;
    double *sums = BATCH ? bsums : a.sums;
    const int mas = BATCH ? bmas : a.mas_p[0];
    float *part_base = (BATCH && a.part) ? a.part + (long long)blockIdx.y * gridDim.x * a.part_stride : a.part;
    float *corr = sm + L.corr;
    float2 *ph = (float2 *)(sm + L.ph);
    float *acc3 = sm + L.acc3, *acc1 = sm + L.acc1, *acc2 = sm + L.acc2;
    for (int i = threadIdx.x; i < dims; i += blockDim.x) corr[i] = mas_corr_f(freq_of(i, dims), dims, mas);
    if (INTER) {
        for (int i = threadIdx.x; i < dims; i += blockDim.x) {
            float sn, cs;
            sincospif((float)freq_of(i, dims) / (float)dims, &sn, &cs);
            ph[i] = make_float2(cs, sn);
        }
    }
    for (int i = L.acc3 + threadIdx.x; i < L.stage; i += blockDim.x) sm[i] = 0.0f;
    __syncthreads();

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m2 = d.middle * d.middle;
    double *P3 = sums;
    double *PH = P3 + (long long)d.nb3 * 3;
    double *P1 = PH + d.nb3;
    double *P2 = P1 + d.nb1;
    float2 *stage = (float2 *)(sm + L.stage) + warp * 32 * (chunk + 1);
    const int kz_begin = lane * chunk;
    const int kz_end = min(nz, kz_begin + chunk);
    float *part = part_base ? part_base + (long long)blockIdx.x * a.part_stride : nullptr;
    float r1 = 0.0f;

    const int G = sym_groups(dims);
    const int p = blockIdx.x / a.chunks;                 // |k_par|
    const int cid = blockIdx.x % a.chunks;
    const int per = (G + a.chunks - 1) / a.chunks;
    const int q0 = cid * per, q1 = min(G, q0 + per);
    for (int q = q0 + warp; q < q1; q += NW) {
        const SignRows R = sign_rows<INTER>(AXIS == 0 ? p : q, AXIS == 0 ? q : p, d, ph);
        stage_sign_rows<INTER>(R, dk, dk2, corr, ph, __fmul_rn(corr[p], corr[q]), d, stage, chunk_magic, lane);
        __syncwarp();
        // pass 2: this lane's run of kz, sums kept while the bins stay the same
        if (kz_begin < kz_end) {
            const int kperp2 = q * q;               // k_per^2 - kz^2
            const int kxy2 = p * p + q * q;
            int kz = kz_begin;
            int n2 = kxy2 + kz * kz;
            int ki = isqrt_exact(n2);
            int kp2 = kperp2 + kz * kz;
            int kper = isqrt_exact(kp2);
            const float kpar2f = (float)(p * p);
            float s0 = 0.0f, s2 = 0.0f, s4 = 0.0f, sp = 0.0f, sd = 0.0f;
            const float2 *run = stage + lane * (chunk + 1);
            for (; kz < kz_end; kz++) {
                const float2 e = run[kz - kz_begin];
                const float val = e.x;
                const float mu2 = n2 ? __fdividef(kpar2f, (float)n2) : 0.0f;
                const float l2 = 0.5f * (3.0f * mu2 - 1.0f);
                const float l4 = 0.125f * ((35.0f * mu2 - 30.0f) * mu2 + 3.0f);
                s0 += val;
                s2 += val * l2;
                s4 += val * l4;
                sp += e.y;
                sd += val;
                if (n2 <= m2) r1 += val;
                const int dn = 2 * kz + 1;
                n2 += dn;
                const bool new3 = (ki + 1) * (ki + 1) <= n2;
                kp2 += dn;
                const bool new2 = (kper + 1) * (kper + 1) <= kp2;
                if (new3 || kz + 1 == kz_end) {
                    if (part) {
                        atomicAdd(reinterpret_cast<float4 *>(part + ki * 4), make_float4(s0, s2, s4, sp));
                    } else {
                        float *b3 = acc3 + ki * 4;
                        if (s0 != 0.0f) atomicAdd(b3, s0);
                        if (s2 != 0.0f) atomicAdd(b3 + 1, s2);
                        if (s4 != 0.0f) atomicAdd(b3 + 2, s4);
                        if (sp != 0.0f) atomicAdd(b3 + 3, sp);
                    }
                    s0 = s2 = s4 = sp = 0.0f;
                    ki += new3 ? 1 : 0;
                }
                if (new2 || kz + 1 == kz_end) {
                    if (part) atomicAdd(part + d.nb3 * 4 + kper, sd);
                    else if (sd != 0.0f) atomicAdd(acc2 + kper, sd);
                    sd = 0.0f;
                    kper += new2 ? 1 : 0;
                }
            }
        }
        __syncwarp();
    }
    {
        float v = r1;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
        if (lane == 0 && v != 0.0f) atomicAdd(acc1 + p, v);
    }
    __syncthreads();
    if (!part) {
        for (int i = threadIdx.x; i < d.nb3 * 4; i += blockDim.x) {
            const float v = acc3[i];
            if (v == 0.0f) continue;
            const int bin = i >> 2, s = i & 3;
            if (s < 3) atomicAdd(P3 + (long long)bin * 3 + s, (double)v);
            else atomicAdd(PH + bin, (double)v);
        }
    }
    for (int i = threadIdx.x; i < d.nb1; i += blockDim.x) {
        const float v = acc1[i];
        if (v != 0.0f) atomicAdd(P1 + i, (double)v);
    }
    if (!part) {
        for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x) {
            const float v = acc2[i];
            if (v == 0.0f) continue;
            atomicAdd(P2 + (long long)(d.kmax_par + 1) * i + p, (double)v);
        }
    }
}

// Per-CTA partial sums of pk_bin_seq_kernel into the float64 sums.  3D slots:
// blockIdx.y splits the CTAs into groups, each thread sums one slot over its
// group in float64.  k_per slots (axes 0/1): each CTA's plane fixes k_par, so a
// thread per (CTA, k_per) adds its value where it belongs.
// With items, blockIdx.z is the item: its sums, and its n_cta x stride slice of part.
__global__ void __launch_bounds__(256) pk_part_reduce_kernel(const float *__restrict__ part, int n_cta,
                                                             int stride, int per_group, int chunks, int axis,
                                                             PkDims d, double *__restrict__ sums,
                                                             const pyl_pk_item *__restrict__ items)
{
    if (items) {
        sums = items[blockIdx.z].sums;
        part += (long long)blockIdx.z * n_cta * stride;
    }
    double *P3 = sums, *PH = P3 + (long long)d.nb3 * 3;
    double *P2 = PH + d.nb3 + d.nb1;
    const int n3 = d.nb3 * 4;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const int c0 = blockIdx.y * per_group, c1 = min(n_cta, c0 + per_group);
    if (s < n3) {
        double acc = 0.0;
        for (int c = c0; c < c1; c++) acc += (double)part[(long long)c * stride + s];
        if (acc != 0.0) {
            const int bin = s >> 2, k = s & 3;
            if (k < 3) atomicAdd(P3 + (long long)bin * 3 + k, acc);
            else atomicAdd(PH + bin, acc);
        }
    } else if (axis != 2 && s < n3 + d.kmax_per + 1) {
        const int kper = s - n3;
        for (int c = c0; c < c1; c++) {
            const float v = part[(long long)c * stride + s];
            if (v == 0.0f) continue;
            const int kpar = c / chunks;        // pk_bin_sym_kernel: CTA c holds plane |k_par| = c / chunks
            atomicAdd(P2 + (long long)(d.kmax_par + 1) * kper + kpar, (double)v);
        }
    }
}

// Zeroes every item's sums (blockIdx.x = item).
__global__ void __launch_bounds__(256) pk_items_zero_kernel(const pyl_pk_item *__restrict__ items, long long len)
{
    double *s = items[blockIdx.x].sums;
    for (long long i = threadIdx.x; i < len; i += blockDim.x) s[i] = 0.0;
}

// Data-independent per-bin sums: N3 and K3 = sum |k| by 3D bin, N1 by |k_par| for
// |k| <= N/2 (K1 = |k_par| N1), N2 by 2D bin.  The modes are walked by sign-row
// representatives like the one-field bin kernels (axes 0/1: CTA = plane
// representative p, warps = row representatives q; axis 2: the representatives'
// ring table): each (p, q, kz) stands for its m = 1..4 sign rows not dropped by
// the Hermitian skip, counted m times, with |k| = sqrt(p^2 + q^2 + kz^2) in
// float64 (one square root per representative instead of per mode).
// shared memory (doubles): N3[nb3] K3[nb3] N1[nb1] N2[kmax_per+1] (axis 0/1) or
// per-warp kz arrays c2[NW][nz] c1[NW][nz] (axis 2).
template <int AXIS>
__global__ void __launch_bounds__(256) pk_geometry_kernel(BinArgs a)
{
    extern __shared__ double gs[];
    const PkDims d = a.d;
    const int dims = d.dims, nz = d.nz;
    double *N3 = gs, *K3 = N3 + d.nb3, *N1 = K3 + d.nb3, *N2 = N1 + d.nb1;
    const int nsm = 2 * d.nb3 + d.nb1 + (AXIS == 2 ? 2 * NW * nz : d.kmax_per + 1);
    for (int i = threadIdx.x; i < nsm; i += blockDim.x) gs[i] = 0.0;
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long m2 = (long long)d.middle * d.middle;
    const bool even = (dims & 1) == 0;
    double *gK1 = a.geom, *gN1 = gK1 + d.nb1, *gN2 = gN1 + d.nb1, *gK3 = gN2 + d.nb2, *gN3 = gK3 + d.nb3;
    double *c2 = N2 + warp * 2 * nz, *c1 = c2 + nz;   // axis 2
    float n1reg = 0.0f;
    int cur_ring = -1;
    const int G = sym_groups(dims);
    // this warp's representatives: (p, q) of a plane (axes 0/1) or a run of the ring table
    int p = 0, q_first = 0, q_step = 1, count = 0;
    long long wb = 0;
    if (AXIS != 2) {
        p = blockIdx.x / a.chunks;
        const int cid = blockIdx.x % a.chunks, per = (G + a.chunks - 1) / a.chunks;
        const int q0 = cid * per, q1 = min(G, q0 + per);
        q_first = q0 + warp;
        q_step = NW;
        count = q_first < q1 ? (q1 - q_first + NW - 1) / NW : 0;
    } else {
        const long long total = (long long)G * G;
        const long long b = (long long)blockIdx.x * a.rows_per_cta, e = min(total, b + a.rows_per_cta);
        const int per_warp = (a.rows_per_cta + NW - 1) / NW;
        wb = b + (long long)warp * per_warp;
        count = wb < e ? (int)min((long long)per_warp, e - wb) : 0;
    }
    for (int j = 0; j < count; j++) {
        int xr, yr;                                  // |kx|, |ky| representatives
        if (AXIS == 2) {
            const unsigned rid = a.rows[wb + j];
            xr = (int)(rid / (unsigned)G);
            yr = (int)(rid % (unsigned)G);
        } else {
            const int q = q_first + j * q_step;
            xr = AXIS == 0 ? p : q;
            yr = AXIS == 0 ? q : p;
        }
        const SignRows R = sign_rows<false>(xr, yr, d, nullptr);
        const int mall = __popc(R.used), m0 = __popc(R.used & ~R.skip0), mm = __popc(R.used & ~R.skipm);
        const int kxy2 = xr * xr + yr * yr;
        const int ring = AXIS == 2 ? isqrt_exact(kxy2) : 0;
        if (AXIS == 2 && ring != cur_ring) {
            if (cur_ring >= 0)
                for (int kz = lane; kz < nz; kz += 32)
                    if (c2[kz] != 0.0) {
                        atomicAdd(gN2 + (long long)(d.kmax_par + 1) * cur_ring + kz, c2[kz]);
                        c2[kz] = 0.0;
                    }
            cur_ring = ring;
        }
        const int kper2 = AXIS == 0 ? yr * yr : xr * xr;      // axes 0/1: k_per^2 - kz^2
        for (int kz0 = 0; kz0 < nz; kz0 += 32) {
            const int kz = kz0 + lane;
            const bool valid = kz < nz;
            const int m = !valid ? 0 : (kz == 0 ? m0 : ((even && kz == d.middle) ? mm : mall));
            const int n2 = kxy2 + kz * kz;
            const int ki = valid ? isqrt_exact(n2) : KEY_NONE;
            const Seg s3 = seg_of(ki);
            const float cnt = seg_sum((float)m, s3.start);
            const double ks = seg_sum(m ? (double)m * sqrt((double)n2) : 0.0, s3.start);
            if (s3.tail && ki != KEY_NONE && cnt != 0.0f) {
                atomicAdd(N3 + ki, (double)cnt);
                atomicAdd(K3 + ki, ks);
            }
            const bool in1d = m && (long long)n2 <= m2;
            if (AXIS != 2) {
                const int kper = isqrt_exact(kper2 + kz * kz);
                const Seg s2 = seg_of(valid ? kper : KEY_NONE);
                const float c = seg_sum((float)m, s2.start);
                if (s2.tail && valid && c != 0.0f) atomicAdd(N2 + kper, (double)c);
                if (in1d) n1reg += (float)m;
            } else if (m) {
                c2[kz] += (double)m;
                if (in1d) c1[kz] += (double)m;
            }
        }
    }
    if (AXIS != 2) {
        float v = n1reg;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(FULL, v, o);
        if (lane == 0 && v != 0.0f) atomicAdd(N1 + p, (double)v);
    } else {
        for (int kz = lane; kz < nz; kz += 32) {
            if (cur_ring >= 0 && c2[kz] != 0.0)
                atomicAdd(gN2 + (long long)(d.kmax_par + 1) * cur_ring + kz, c2[kz]);
            if (c1[kz] != 0.0) {
                atomicAdd(gN1 + kz, c1[kz]);
                atomicAdd(gK1 + kz, c1[kz] * kz);
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < d.nb3; i += blockDim.x)
        if (N3[i] != 0.0) { atomicAdd(gN3 + i, N3[i]); atomicAdd(gK3 + i, K3[i]); }
    if (AXIS != 2) {
        for (int i = threadIdx.x; i < d.nb1; i += blockDim.x)
            if (N1[i] != 0.0) { atomicAdd(gN1 + i, N1[i]); atomicAdd(gK1 + i, N1[i] * i); }
        for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x)
            if (N2[i] != 0.0) atomicAdd(gN2 + (long long)(d.kmax_par + 1) * i + p, N2[i]);
    }
}

// ---- ring table for axis 2: rows (kxx*dims + kyy) sorted by k_per = isqrt(kx^2+ky^2)
// Row tables: every row (kxx, kyy), id kxx * dims + kyy, or with sym only the
// representatives (p, q) of the four sign rows, p, q in [0, dims/2], id p * G + q.
__device__ __forceinline__ int ring_of(long long r, const PkDims &d, bool sym)
{
    if (sym) {
        const int G = d.dims / 2 + 1;
        const int p = (int)(r / G), q = (int)(r % G);
        return isqrt_exact(p * p + q * q);
    }
    const int kx = freq_of((int)(r / d.dims), d.dims), ky = freq_of((int)(r % d.dims), d.dims);
    return isqrt_exact(kx * kx + ky * ky);
}

__host__ __device__ inline long long ring_rows(const PkDims &d, bool sym)
{
    const long long side = sym ? d.dims / 2 + 1 : d.dims;
    return side * side;
}

__global__ void __launch_bounds__(256) ring_count_kernel(PkDims d, bool sym, unsigned *cnt)
{
    extern __shared__ unsigned h[];
    for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const long long total = ring_rows(d, sym);
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < total;
         r += (long long)gridDim.x * blockDim.x)
        atomicAdd(h + ring_of(r, d, sym), 1u);
    __syncthreads();
    for (int i = threadIdx.x; i <= d.kmax_per; i += blockDim.x)
        if (h[i]) atomicAdd(cnt + i, h[i]);
}

__global__ void __launch_bounds__(1024) ring_scan_kernel(const unsigned *cnt, int n, unsigned *cursor)
{
    __shared__ unsigned part[1024];
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int b = threadIdx.x * per, e = min(n, b + per);
    unsigned s = 0;
    for (int i = b; i < e; i++) s += cnt[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const unsigned v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned run = part[threadIdx.x] - s;
    for (int i = b; i < e; i++) { cursor[i] = run; run += cnt[i]; }
}

__global__ void __launch_bounds__(256) ring_fill_kernel(PkDims d, bool sym, unsigned *cursor, unsigned *rows)
{
    const long long total = ring_rows(d, sym);
    for (long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x; r < total;
         r += (long long)gridDim.x * blockDim.x)
        rows[atomicAdd(cursor + ring_of(r, d, sym), 1u)] = (unsigned)r;
}

inline size_t align256(size_t v) { return (v + 255) / 256 * 256; }

struct RingWs {
    unsigned *rows, *cnt, *cursor;
    size_t bytes;
};

RingWs ring_layout(void *base, const PkDims &d)
{
    RingWs w;
    char *b = (char *)base;
    size_t off = 0;
    w.rows = (unsigned *)(b + off); off = align256(off + sizeof(unsigned) * (size_t)d.dims * d.dims);
    w.cnt = (unsigned *)(b + off); off = align256(off + sizeof(unsigned) * (d.kmax_per + 1));
    w.cursor = (unsigned *)(b + off); off = align256(off + sizeof(unsigned) * (d.kmax_per + 1));
    w.bytes = off;
    return w;
}

int build_rings(const PkDims &d, const RingWs &w, bool sym, cudaStream_t st)
{
    const int n = d.kmax_per + 1;
    PYL_CUDA(cudaMemsetAsync(w.cnt, 0, sizeof(unsigned) * n, st));
    const long long total = ring_rows(d, sym);
    int blocks = (int)min((total + 255) / 256, (long long)num_sms() * 4);
    if (blocks < 1) blocks = 1;
    ring_count_kernel<<<blocks, 256, sizeof(unsigned) * n, st>>>(d, sym, w.cnt);
    PYL_LAUNCH_CHECK();
    ring_scan_kernel<<<1, 1024, 0, st>>>(w.cnt, n, w.cursor);
    PYL_LAUNCH_CHECK();
    ring_fill_kernel<<<blocks, 256, 0, st>>>(d, sym, w.cursor, w.rows);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

inline int plane_chunks(int dims)
{
    int chunks = 1;
    while ((long long)dims * chunks < 2LL * num_sms() && chunks * 8 < dims) chunks *= 2;
    return chunks;
}

constexpr int RING_ROWS_PER_CTA = 256;
constexpr size_t SMEM_LIMIT = 200 * 1024;

struct SeqPart {
    unsigned blocks;
    int stride;           // floats per CTA (a multiple of 4: float4 slots stay aligned)
    size_t bytes;
};

// Axes 0/1 (pk_bin_sym_kernel): CTAs per plane representative, several waves at
// 2-3 resident CTAs per SM and at least two row representatives per warp.
inline int sym_chunks(int dims)
{
    const int G = sym_groups(dims);
    int c = 1;
    while ((long long)G * c < 8LL * num_sms() && c * NW * 2 <= G) c *= 2;
    return c;
}

inline SeqPart seq_part(const PkDims &d, int axis)
{
    SeqPart p;
    p.blocks = axis == 2 ? (unsigned)((ring_rows(d, true) + RING_ROWS_PER_CTA - 1) / RING_ROWS_PER_CTA)
                         : (unsigned)(sym_groups(d.dims) * sym_chunks(d.dims));
    p.stride = (d.nb3 * 4 + (axis == 2 ? 0 : d.kmax_per + 1) + 3) & ~3;
    p.bytes = align256(sizeof(float) * (size_t)p.blocks * p.stride);
    return p;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

// axis 2: the ring table; one field: the per-CTA partial sums of the bin flushes
// (without them, the flushes fall back to float shared-memory atomics).
extern "C" size_t pyl_pk_workspace_size(int dims, int n_fields, int axis)
{
    if (dims < 2) return 0;
    const PkDims d = pk_dims(dims);
    size_t bytes = axis == 2 ? ring_layout(nullptr, d).bytes : 0;
    if (n_fields == 1) bytes += seq_part(d, axis).bytes;
    return bytes;
}

extern "C" int pyl_pk_bin(const void *dk, const void *dk_interlaced, int n_fields, int64_t field_stride,
                          int dims, int axis, const int *host_mas_p, double *sums, void *workspace,
                          size_t workspace_bytes, void *stream)
{
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
    BinArgs a;
    a.dk = (const float2 *)dk;
    a.dk2 = (const float2 *)dk_interlaced;
    a.fstride = field_stride;
    a.F = n_fields;
    a.C = n_fields + n_fields * (n_fields - 1) / 2;
    a.axis = axis;
    a.sums = sums;
    a.geom = nullptr;
    a.d = d;
    a.rows = nullptr;
    a.part = nullptr;
    a.part_stride = 0;
    a.items = nullptr;
    for (int f = 0; f < MAX_FIELDS; f++) {
        a.mas_p[f] = f < n_fields ? host_mas_p[f] : 0;
        PYL_CHECK_ARG(a.mas_p[f] >= 0 && a.mas_p[f] <= 4, "MAS exponent must be 0..4");
    }
    const bool inter = dk_interlaced != nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    // one field: the four-sign-row kernels when their shared memory fits (with the
    // per-CTA partial sums when the workspace holds them); else pk_bin_kernel
    const int chunk = seq_chunk(d.nz);
    const bool warp_arrays = axis == 2 && sizeof(float) * bin_smem(d, a.F, a.C, axis, inter, 1).total <= SMEM_LIMIT;
    const size_t ring_bytes = axis == 2 ? ring_layout(nullptr, d).bytes : 0;
    const SeqPart sp = seq_part(d, axis);
    const bool use_part = n_fields == 1 && workspace != nullptr && workspace_bytes >= ring_bytes + sp.bytes;
    const size_t sms = sizeof(float) * (size_t)seq_smem(d, axis, inter, chunk, use_part).total;
    const bool seq = n_fields == 1 && (axis != 2 || warp_arrays) && sms <= SMEM_LIMIT;
    unsigned blocks;
    if (axis == 2) {
        const RingWs w = ring_layout(workspace, d);
        if (workspace == nullptr || workspace_bytes < w.bytes) {
            set_error("pyl_pk_bin: axis 2 needs " + std::to_string(w.bytes) + " workspace bytes");
            return PYL_ERR_WORKSPACE;
        }
        int rc = build_rings(d, w, seq, st);
        if (rc) return rc;
        a.rows = w.rows;
        a.rows_per_cta = RING_ROWS_PER_CTA;
        a.chunks = 1;
        a.warp_arrays = warp_arrays;
        blocks = (unsigned)((ring_rows(d, seq) + RING_ROWS_PER_CTA - 1) / RING_ROWS_PER_CTA);
    } else {
        a.rows_per_cta = 0;
        a.warp_arrays = 0;
        a.chunks = seq ? sym_chunks(dims) : plane_chunks(dims);
        blocks = (unsigned)((seq ? sym_groups(dims) : dims) * a.chunks);
    }
    if (seq) {
        PYL_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * pyl_pk_sums_len(dims, 1), st));
        a.part_stride = sp.stride;
        if (use_part) {
            a.part = (float *)((char *)workspace + ring_bytes);
            PYL_CUDA(cudaMemsetAsync(a.part, 0, sizeof(float) * (size_t)sp.blocks * sp.stride, st));
        }
#define PYL_SEQ(K, I, A)                                                           \
    do {                                                                           \
        PYL_CUDA(ensure_smem(K<I, A, false>, sms));                         \
        K<I, A, false><<<blocks, 256, sms, st>>>(a, chunk, seq_chunk_magic(chunk)); \
    } while (0)
        if (inter) {
            if (axis == 0) PYL_SEQ(pk_bin_sym_kernel, true, 0);
            else if (axis == 1) PYL_SEQ(pk_bin_sym_kernel, true, 1);
            else PYL_SEQ(pk_bin_seq_kernel, true, 2);
        } else {
            if (axis == 0) PYL_SEQ(pk_bin_sym_kernel, false, 0);
            else if (axis == 1) PYL_SEQ(pk_bin_sym_kernel, false, 1);
            else PYL_SEQ(pk_bin_seq_kernel, false, 2);
        }
#undef PYL_SEQ
        PYL_LAUNCH_CHECK();
        if (a.part) {
            const int slots = d.nb3 * 4 + (axis == 2 ? 0 : d.kmax_per + 1);
            const int groups = 16, per_group = (int)((blocks + groups - 1) / groups);
            pk_part_reduce_kernel<<<dim3((slots + 255) / 256, groups), 256, 0, st>>>(
                a.part, (int)blocks, sp.stride, per_group, a.chunks, axis, d, sums, nullptr);
            PYL_LAUNCH_CHECK();
        }
        return PYL_OK;
    }
    const size_t smem = sizeof(float) * (size_t)bin_smem(d, a.F, a.C, axis, inter, a.warp_arrays).total;
    if (smem > SMEM_LIMIT) {
        set_error("pyl_pk_bin: bins for this grid and field count exceed shared memory");
        return PYL_ERR_UNSUPPORTED;
    }
    PYL_CUDA(cudaMemsetAsync(sums, 0, sizeof(double) * pyl_pk_sums_len(dims, n_fields), st));
#define PYL_BIN(I, A, FF)                                                          \
    do {                                                                           \
        PYL_CUDA(ensure_smem(pk_bin_kernel<I, A, FF>, smem));               \
        pk_bin_kernel<I, A, FF><<<blocks, 256, smem, st>>>(a);                     \
    } while (0)
#define PYL_BIN_F(I, A)                                                            \
    do {                                                                           \
        switch (n_fields) {                                                        \
            case 1: PYL_BIN(I, A, 1); break;                                       \
            case 2: PYL_BIN(I, A, 2); break;                                       \
            case 3: PYL_BIN(I, A, 3); break;                                       \
            default: PYL_BIN(I, A, 4); break;                                      \
        }                                                                          \
    } while (0)
    if (inter) {
        if (axis == 0) PYL_BIN_F(true, 0); else if (axis == 1) PYL_BIN_F(true, 1); else PYL_BIN_F(true, 2);
    } else {
        if (axis == 0) PYL_BIN_F(false, 0); else if (axis == 1) PYL_BIN_F(false, 1); else PYL_BIN_F(false, 2);
    }
#undef PYL_BIN_F
#undef PYL_BIN
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

// Whether the one-field kernel's shared memory holds this grid's bins.
bool batch_fits(const PkDims &d, int axis, bool inter)
{
    if (axis == 2 && sizeof(float) * bin_smem(d, 1, 1, axis, inter, 1).total > SMEM_LIMIT) return false;
    return sizeof(float) * (size_t)seq_smem(d, axis, inter, seq_chunk(d.nz), true).total <= SMEM_LIMIT;
}

// CTA partition of a batched launch: the one-field call's one, coarsened while
// the items together still give several waves (8 CTAs per SM) -- fewer CTAs per
// item amortise each CTA's tables, zeroing and flushes over more rows, which
// small grids need.  Axes 0/1: row chunks per plane representative; axis 2:
// representatives per CTA.
struct BatchPart {
    int chunks, rows_per_cta;
    unsigned blocks;      // CTAs per item
    int stride;           // partial-sum floats per CTA
};

inline BatchPart batch_part(const PkDims &d, int axis, int n_items)
{
    BatchPart b;
    const long long target = 8LL * num_sms();
    b.stride = seq_part(d, axis).stride;
    if (axis != 2) {
        const int G = sym_groups(d.dims);
        const int cmax = sym_chunks(d.dims);
        int c = 1;
        while (c < cmax && (long long)G * c * n_items < target) c *= 2;
        b.chunks = c;
        b.rows_per_cta = 0;
        b.blocks = (unsigned)(G * c);
    } else {
        const long long rows = ring_rows(d, true);
        int rpc = RING_ROWS_PER_CTA;
        while (rpc < 16 * RING_ROWS_PER_CTA && ((rows + 2 * rpc - 1) / (2 * rpc)) * n_items >= target) rpc *= 2;
        b.chunks = 1;
        b.rows_per_cta = rpc;
        b.blocks = (unsigned)((rows + rpc - 1) / rpc);
    }
    return b;
}

// Batched one-field spectra: the axis-2 row table, then each item's per-CTA
// partial sums.  0: not batchable.
extern "C" size_t pyl_pk_bin_batch_workspace_size(int dims, int n_items, int axis, int interlaced)
{
    if (dims < 2 || dims > 8192 || n_items < 1 || axis < 0 || axis > 2) return 0;
    const PkDims d = pk_dims(dims);
    if (!batch_fits(d, axis, interlaced != 0)) return 0;
    const BatchPart bp = batch_part(d, axis, n_items);
    return (axis == 2 ? ring_layout(nullptr, d).bytes : 0) +
           align256(sizeof(float) * (size_t)bp.blocks * bp.stride * (size_t)n_items);
}

extern "C" int pyl_pk_bin_batch(const pyl_pk_item *items, int n_items, int dims, int axis, int interlaced,
                                void *workspace, size_t workspace_bytes, void *stream)
{
    PYL_CHECK_ARG(items != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    PYL_CHECK_ARG(n_items >= 1 && n_items <= 65535, "1..65535 items per call");
    const PkDims d = pk_dims(dims);
    const bool inter = interlaced != 0;
    if (!batch_fits(d, axis, inter)) {
        set_error("pyl_pk_bin_batch: this grid's bins exceed the one-field kernel's shared memory");
        return PYL_ERR_UNSUPPORTED;
    }
    const size_t need = pyl_pk_bin_batch_workspace_size(dims, n_items, axis, interlaced);
    if (workspace == nullptr || workspace_bytes < need) {
        set_error("pyl_pk_bin_batch: needs " + std::to_string(need) + " workspace bytes");
        return PYL_ERR_WORKSPACE;
    }
    const int chunk = seq_chunk(d.nz);
    const size_t sms = sizeof(float) * (size_t)seq_smem(d, axis, inter, chunk, true).total;
    BinArgs a;
    a.dk = a.dk2 = nullptr;
    a.fstride = 0;
    a.F = a.C = 1;
    a.axis = axis;
    a.sums = nullptr;
    a.geom = nullptr;
    a.d = d;
    a.rows = nullptr;
    a.items = items;
    for (int f = 0; f < MAX_FIELDS; f++) a.mas_p[f] = 0;
    cudaStream_t st = (cudaStream_t)stream;
    const BatchPart bp = batch_part(d, axis, n_items);
    size_t ring_bytes = 0;
    if (axis == 2) {
        const RingWs w = ring_layout(workspace, d);
        ring_bytes = w.bytes;
        int rc = build_rings(d, w, true, st);
        if (rc) return rc;
        a.rows = w.rows;
        a.warp_arrays = 1;
    } else {
        a.warp_arrays = 0;
    }
    a.chunks = bp.chunks;
    a.rows_per_cta = bp.rows_per_cta;
    a.part = (float *)((char *)workspace + ring_bytes);
    a.part_stride = bp.stride;
    pk_items_zero_kernel<<<n_items, 256, 0, st>>>(items, pyl_pk_sums_len(dims, 1));
    PYL_LAUNCH_CHECK();
    PYL_CUDA(cudaMemsetAsync(a.part, 0, sizeof(float) * (size_t)bp.blocks * bp.stride * n_items, st));
    const dim3 grid(bp.blocks, (unsigned)n_items);
#define PYL_SEQB(K, I, A)                                                          \
    do {                                                                           \
        PYL_CUDA(ensure_smem(K<I, A, true>, sms));                          \
        K<I, A, true><<<grid, 256, sms, st>>>(a, chunk, seq_chunk_magic(chunk)); \
    } while (0)
    if (inter) {
        if (axis == 0) PYL_SEQB(pk_bin_sym_kernel, true, 0);
        else if (axis == 1) PYL_SEQB(pk_bin_sym_kernel, true, 1);
        else PYL_SEQB(pk_bin_seq_kernel, true, 2);
    } else {
        if (axis == 0) PYL_SEQB(pk_bin_sym_kernel, false, 0);
        else if (axis == 1) PYL_SEQB(pk_bin_sym_kernel, false, 1);
        else PYL_SEQB(pk_bin_seq_kernel, false, 2);
    }
#undef PYL_SEQB
    PYL_LAUNCH_CHECK();
    const int slots = d.nb3 * 4 + (axis == 2 ? 0 : d.kmax_per + 1);
    const int groups = 16, per_group = (int)((bp.blocks + groups - 1) / groups);
    pk_part_reduce_kernel<<<dim3((slots + 255) / 256, groups, (unsigned)n_items), 256, 0, st>>>(
        a.part, (int)bp.blocks, bp.stride, per_group, a.chunks, axis, d, nullptr, items);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_pk_geometry(int dims, int axis, double *geom, void *workspace, size_t workspace_bytes,
                               void *stream)
{
    PYL_CHECK_ARG(geom != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && dims <= 8192, "dims out of range");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    const PkDims d = pk_dims(dims);
    cudaStream_t st = (cudaStream_t)stream;
    BinArgs a;
    a.dk = a.dk2 = nullptr;
    a.fstride = 0;
    a.F = a.C = 1;
    a.axis = axis;
    a.sums = nullptr;
    a.geom = geom;
    a.d = d;
    a.rows = nullptr;
    a.part = nullptr;
    a.part_stride = 0;
    a.items = nullptr;
    for (int f = 0; f < MAX_FIELDS; f++) a.mas_p[f] = 0;
    unsigned blocks;
    if (axis == 2) {
        const RingWs w = ring_layout(workspace, d);
        if (workspace == nullptr || workspace_bytes < w.bytes) {
            set_error("pyl_pk_geometry: axis 2 needs " + std::to_string(w.bytes) + " workspace bytes");
            return PYL_ERR_WORKSPACE;
        }
        int rc = build_rings(d, w, true, st);
        if (rc) return rc;
        a.rows = w.rows;
        a.rows_per_cta = RING_ROWS_PER_CTA;
        a.chunks = 1;
        a.warp_arrays = 1;
        blocks = (unsigned)((ring_rows(d, true) + RING_ROWS_PER_CTA - 1) / RING_ROWS_PER_CTA);
    } else {
        a.chunks = sym_chunks(dims);
        a.rows_per_cta = 0;
        a.warp_arrays = 0;
        blocks = (unsigned)(sym_groups(dims) * a.chunks);
    }
    const size_t smem = sizeof(double) * (2 * d.nb3 + d.nb1 + (axis == 2 ? 2 * NW * d.nz : d.kmax_per + 1));
    if (smem > SMEM_LIMIT) {
        set_error("pyl_pk_geometry: grid too large for the shared-memory bins");
        return PYL_ERR_UNSUPPORTED;
    }
    PYL_CUDA(cudaMemsetAsync(geom, 0, sizeof(double) * pyl_pk_geometry_len(dims), st));
#define PYL_GEOM(A)                                                                \
    do {                                                                           \
        PYL_CUDA(ensure_smem(pk_geometry_kernel<A>, smem));                 \
        pk_geometry_kernel<A><<<blocks, 256, smem, st>>>(a);                       \
    } while (0)
    if (axis == 0) PYL_GEOM(0); else if (axis == 1) PYL_GEOM(1); else PYL_GEOM(2);
#undef PYL_GEOM
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
