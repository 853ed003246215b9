// Batched realizations: one persistent launch deposits a whole batch of
// particle sets with uneven particle counts, grid sizes, MAS and interlacing.
//
// Work is a device list of items (realization, first particle, count); the
// CTAs of the persistent kernel take items from a device counter until the
// list is exhausted, so long and short realizations balance across SMs.  Each
// item deposits its particles with red.global.add into its realization's
// grid(s) (grids of <= 256^3 cells stay resident in L2 while their items run),
// scaled by dims^3 / N so that grids pre-filled with -1 end as the overdensity
// delta = n/mean - 1 (library/Pk_library/Pk_snapshot.py:70-88).  The per-particle
// arithmetic is the one of mas.cu (MAS_library.pyx:123-545).
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"
#include "deposit.cuh"

namespace pyl {
namespace {

__device__ __forceinline__ float ba_dist(float p, float inv) { return __fmul_rn(p, inv); }

// Support of one coordinate (same arithmetic as mas.cu axis_weights).
template <int MAS>
__device__ __forceinline__ int ba_weights(float p, float inv, float *C)
{
    const float dist = ba_dist(p, inv);
    if (MAS == PYL_MAS_NGP) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        int k = __float2int_rz(fl) + (frac >= 0.5f ? 1 : 0);
        if (dist < -0.5f && frac != 0.5f) k += 1;
        C[0] = 1.0f;
        return k;
    } else if (MAS == PYL_MAS_CIC) {
        const float t = truncf(dist);
        const float u = __fsub_rn(dist, t);
        C[0] = __fsub_rn(1.0f, u);
        C[1] = u;
        return __float2int_rz(t);
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        const float fmn = __fsub_rn(__fadd_rn(fl, frac >= 0.5f ? 1.0f : 0.0f), 2.0f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float diff = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
            float c;
            if (diff < 0.5f) c = __fsub_rn(0.75f, __fmul_rn(diff, diff));
            else if (diff < 1.5f) { const float t = __fsub_rn(1.5f, diff); c = __fmul_rn(__fmul_rn(0.5f, t), t); }
            else c = 0.0f;
            C[j] = c;
        }
        return __float2int_rz(fl) - 1 + (frac >= 0.5f ? 1 : 0);
    } else {
        const float fl = floorf(dist);
        const float fmn = __fsub_rn(fl, 2.0f);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float d = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
            float c;
            if (d < 1.0f) {
                const float a = __fmul_rn(__fmul_rn(6.0f, d), d);
                const float b = __fmul_rn(__fmul_rn(__fmul_rn(3.0f, d), d), d);
                c = __fdiv_rn(__fadd_rn(__fsub_rn(4.0f, a), b), 6.0f);
            } else if (d < 2.0f) {
                const float t = __fsub_rn(2.0f, d);
                c = __fdiv_rn(__fmul_rn(__fmul_rn(t, t), t), 6.0f);
            } else c = 0.0f;
            C[j] = c;
        }
        return __float2int_rz(fl) - 1;
    }
}

template <int MAS>
__device__ __forceinline__ void ba_deposit(const float *p, const pyl_batch_real &r, float shift, float *out)
{
    constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS;
    const int dims = r.dims;
    const long long d = dims;
    float C[3][S];
    int idx[3][S];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int f = ba_weights<MAS>(__fadd_rn(p[a], shift), r.inv, C[a]);
#pragma unroll
        for (int j = 0; j < S; j++) idx[a][j] = wrap_index((long long)f + j, dims);
    }
#pragma unroll
    for (int l = 0; l < S; l++)
#pragma unroll
        for (int m = 0; m < S; m++) {
            const float c01 = __fmul_rn(C[0][l], C[1][m]);
            const long long row = ((long long)idx[0][l] * d + idx[1][m]) * d;
#pragma unroll
            for (int q = 0; q < S; q++)
                atomicAdd(out + row + idx[2][q], __fmul_rn(__fmul_rn(c01, C[2][q]), r.scale));
        }
}

__global__ void __launch_bounds__(256) batch_deposit_kernel(const pyl_batch_real *__restrict__ reals,
                                                            const pyl_batch_item *__restrict__ items,
                                                            int n_items, unsigned *counter)
{
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= n_items) break;
        const pyl_batch_item item = items[it];
        const pyl_batch_real r = reals[item.real];
        for (long long i = item.first + threadIdx.x; i < item.first + item.count; i += blockDim.x) {
            const float p[3] = {__ldg(r.pos + 3 * i), __ldg(r.pos + 3 * i + 1), __ldg(r.pos + 3 * i + 2)};
            for (int g = 0; g < (r.grid_interlaced ? 2 : 1); g++) {
                float *out = g ? r.grid_interlaced : r.grid;
                const float sh = g ? r.halfcell : 0.0f;
                switch (r.mas) {
                    case PYL_MAS_NGP: ba_deposit<PYL_MAS_NGP>(p, r, sh, out); break;
                    case PYL_MAS_CIC: ba_deposit<PYL_MAS_CIC>(p, r, sh, out); break;
                    case PYL_MAS_TSC: ba_deposit<PYL_MAS_TSC>(p, r, sh, out); break;
                    default:          ba_deposit<PYL_MAS_PCS>(p, r, sh, out); break;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) fill_value_kernel(float *g, long long n, float v)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) g[i] = v;
}

__global__ void __launch_bounds__(256) scale_value_kernel(float *g, long long n, float f)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) g[i] = __fmul_rn(g[i], f);
}

// ---- batched tiled path ------------------------------------------------------
// The same binning as pyl_ma's TILED strategy, over all realizations of a batch
// at once: every realization's grid is cut into 32^3-cell bins, numbered
// tile_base[r] + (tx*nt + ty)*nt + tz in one global list.
//   bt_count:   persistent over the items: per-item shared-memory histogram of
//               its realization's bins, flushed into the global bin counts;
//   bt_scan:    exclusive scan of the counts (bin offsets and cursors);
//   bt_place:   persistent over the items: per 4096-particle batch, shared-memory
//               ranks per bin, one global atomic per bin to reserve a range,
//               records (x, y, z, 1) written into their bins' ranges;
//   bt_deposit: persistent over the bins: 10.22 fixed-point shared-memory
//               accumulation of the bin (+ halo) for its realization's MAS, both
//               grids when interlaced, red.global into the realization's grid(s)
//               scaled to the overdensity.
constexpr int BT_MAX_TILES = 4096;        // bins per realization (dims <= 512)
constexpr int BT_BATCH = 4096;            // placement batch (particles)

__device__ __forceinline__ int bt_nt(int dims) { return (dims + TB - 1) / TB; }

template <int MAS>
__device__ __forceinline__ int bt_key(const float *p, float inv, int dims, int nt)
{
    const int cx = wrap_index(axis_first<MAS>(p[0], inv), dims) / TB;
    const int cy = wrap_index(axis_first<MAS>(p[1], inv), dims) / TB;
    const int cz = wrap_index(axis_first<MAS>(p[2], inv), dims) / TB;
    return (cx * nt + cy) * nt + cz;
}

__device__ __forceinline__ int bt_key_rt(int mas, const float *p, float inv, int dims, int nt)
{
    switch (mas) {
        case PYL_MAS_NGP: return bt_key<PYL_MAS_NGP>(p, inv, dims, nt);
        case PYL_MAS_CIC: return bt_key<PYL_MAS_CIC>(p, inv, dims, nt);
        case PYL_MAS_TSC: return bt_key<PYL_MAS_TSC>(p, inv, dims, nt);
        default:          return bt_key<PYL_MAS_PCS>(p, inv, dims, nt);
    }
}

// Positions of particles q .. q+3 (q a multiple of 4, so 48 bytes from a 16-byte
// aligned base): three 16-byte loads instead of twelve 4-byte ones; lanes of a
// warp read consecutive 48-byte groups.  Particles at or past `end` are not read.
__device__ __forceinline__ void load_quad(const float *pos, long long q, long long end, bool vec, float p[4][3])
{
    if (vec && q + 4 <= end) {
        const float4 *g = reinterpret_cast<const float4 *>(pos + 3 * q);
        const float4 a = __ldg(g), b = __ldg(g + 1), c = __ldg(g + 2);
        p[0][0] = a.x; p[0][1] = a.y; p[0][2] = a.z;
        p[1][0] = a.w; p[1][1] = b.x; p[1][2] = b.y;
        p[2][0] = b.z; p[2][1] = b.w; p[2][2] = c.x;
        p[3][0] = c.y; p[3][1] = c.z; p[3][2] = c.w;
    } else {
#pragma unroll
        for (int u = 0; u < 4; u++)
            if (q + u < end) {
                p[u][0] = __ldg(pos + 3 * (q + u));
                p[u][1] = __ldg(pos + 3 * (q + u) + 1);
                p[u][2] = __ldg(pos + 3 * (q + u) + 2);
            }
    }
}

__global__ void __launch_bounds__(1024) bt_count_kernel(const pyl_batch_real *__restrict__ reals,
                                                        const pyl_batch_item *__restrict__ items, int n_items,
                                                        const unsigned *__restrict__ tile_base,
                                                        unsigned *__restrict__ counts, unsigned *counter)
{
    __shared__ unsigned h[BT_MAX_TILES];
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = cur;
        if (it >= n_items) break;
        const pyl_batch_item item = items[it];
        const pyl_batch_real r = reals[item.real];
        const int nt = bt_nt(r.dims), ntiles = nt * nt * nt;
        if (ntiles > BT_MAX_TILES) {                   // dims > 512: not binned here
            __syncthreads();
            continue;
        }
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x) h[t] = 0u;
        __syncthreads();
        const long long end = item.first + item.count;
        const bool vec = (item.first & 3) == 0 && (((uintptr_t)r.pos) & 15) == 0;
        for (long long q = item.first + 4 * (long long)threadIdx.x; q < end; q += 4 * (long long)blockDim.x) {
            float p[4][3];
            load_quad(r.pos, q, end, vec, p);
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (q + u < end) atomicAdd(h + bt_key_rt(r.mas, p[u], r.inv, r.dims, nt), 1u);
        }
        __syncthreads();
        const unsigned base = tile_base[item.real];
        for (int t = threadIdx.x; t < ntiles; t += blockDim.x)
            if (h[t]) atomicAdd(counts + base + t, h[t]);
        __syncthreads();
    }
}

// Exclusive scan of n counts into offsets[0..n] and cursor[0..n), one CTA.
__global__ void __launch_bounds__(1024) bt_scan_kernel(const unsigned *__restrict__ counts, unsigned n,
                                                       unsigned *__restrict__ offsets, unsigned *__restrict__ cursor)
{
    __shared__ unsigned long long part[1024];
    const unsigned per = (n + blockDim.x - 1) / blockDim.x;
    const unsigned b = threadIdx.x * per, e = min(n, b + per);
    unsigned long long sum = 0;
    for (unsigned i = b; i < e; i++) sum += counts[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        const unsigned long long v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0ull;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - sum;
    for (unsigned i = b; i < e; i++) {
        offsets[i] = (unsigned)run;
        cursor[i] = (unsigned)run;
        run += counts[i];
    }
    if (threadIdx.x == blockDim.x - 1) offsets[n] = (unsigned)part[threadIdx.x];
}

// Exclusive scan of v[0..n) in place, n <= 4 * blockDim.x (each thread four
// consecutive entries); warp_tot: 32 entries of scratch.  All threads call it.
__device__ __forceinline__ void bt_block_scan4(unsigned *v, int n, unsigned *warp_tot)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = (blockDim.x + 31) >> 5;
    unsigned x[4], tot = 0;
#pragma unroll
    for (int k = 0; k < 4; k++) {
        x[k] = 4 * t + k < n ? v[4 * t + k] : 0u;
        tot += x[k];
    }
    unsigned inc = tot;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        const unsigned wt = lane < nw ? warp_tot[lane] : 0u;
        unsigned wi = wt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < nw) warp_tot[lane] = wi - wt;
    }
    __syncthreads();
    unsigned run = inc - tot + warp_tot[w];
#pragma unroll
    for (int k = 0; k < 4; k++)
        if (4 * t + k < n) {
            v[4 * t + k] = run;
            run += x[k];
        }
    __syncthreads();
}

// Per 4096-particle batch of an item: ranks per bin from shared-memory counters,
// one global atomic per bin touched reserves its run in the bin's range, the batch
// is sorted by bin in shared memory, and the runs are written out coalesced
// (consecutive threads, consecutive slots of a run).
constexpr size_t BT_PLACE_SMEM = sizeof(unsigned) * 2 * BT_MAX_TILES + sizeof(float4) * BT_BATCH +
                                 sizeof(unsigned short) * BT_BATCH;

__global__ void __launch_bounds__(1024) bt_place_kernel(const pyl_batch_real *__restrict__ reals,
                                                        const pyl_batch_item *__restrict__ items, int n_items,
                                                        const unsigned *__restrict__ tile_base,
                                                        unsigned *__restrict__ cursor, unsigned n_total,
                                                        float4 *__restrict__ rec, unsigned *counter)
{
    extern __shared__ __align__(16) unsigned char praw[];
    unsigned *bcnt = (unsigned *)praw, *gbase = bcnt + BT_MAX_TILES;
    float4 *stage = (float4 *)(gbase + BT_MAX_TILES);
    unsigned short *skey = (unsigned short *)(stage + BT_BATCH);
    __shared__ unsigned wt[32];
    __shared__ int cur;
    constexpr int U = BT_BATCH / 1024;
    static_assert(U == 4, "four particles per thread and batch");
    static_assert(BT_MAX_TILES <= 65536, "bin keys held as 16 bits");
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = cur;
        if (it >= n_items) break;
        const pyl_batch_item item = items[it];
        const pyl_batch_real r = reals[item.real];
        const int nt = bt_nt(r.dims), ntiles = nt * nt * nt;
        const unsigned base = tile_base[item.real];
        const long long end = item.first + item.count;
        if (ntiles > BT_MAX_TILES) {
            __syncthreads();
            continue;
        }
        const bool vec = (item.first & 3) == 0 && (((uintptr_t)r.pos) & 15) == 0;
        for (long long s0 = item.first; s0 < end; s0 += BT_BATCH) {
            const int c = (int)min((long long)BT_BATCH, end - s0);
            for (int t = threadIdx.x; t < ntiles; t += blockDim.x) bcnt[t] = 0u;
            __syncthreads();
            float4 v[U];
            int key[U];
            unsigned rank[U];
            // thread t takes particles s0 + 4t .. s0 + 4t + 3 (BT_BATCH = 4 x 1024)
            float p[U][3];
            load_quad(r.pos, s0 + 4 * threadIdx.x, end, vec, p);
#pragma unroll
            for (int u = 0; u < U; u++) {
                const long long i = s0 + 4 * threadIdx.x + u;
                key[u] = -1;
                if (i < end) {
                    v[u] = make_float4(p[u][0], p[u][1], p[u][2], 1.0f);
                    key[u] = bt_key_rt(r.mas, p[u], r.inv, r.dims, nt);
                    rank[u] = atomicAdd(bcnt + key[u], 1u);
                }
            }
            __syncthreads();
            for (int t = threadIdx.x; t < ntiles; t += blockDim.x)
                if (bcnt[t]) gbase[t] = atomicAdd(cursor + base + t, bcnt[t]);
            __syncthreads();
            bt_block_scan4(bcnt, ntiles, wt);                  // bcnt: the batch's run starts
#pragma unroll
            for (int u = 0; u < U; u++)
                if (key[u] >= 0) {
                    const unsigned slot = bcnt[key[u]] + rank[u];
                    stage[slot] = v[u];
                    skey[slot] = (unsigned short)key[u];
                }
            __syncthreads();
            for (int sidx = threadIdx.x; sidx < c; sidx += blockDim.x) {
                const unsigned k = skey[sidx];
                const unsigned dst = gbase[k] + ((unsigned)sidx - bcnt[k]);
                if (dst < n_total) rec[dst] = stage[sidx];
            }
            __syncthreads();
        }
        __syncthreads();
    }
}

// Deposit of one bin of realization r (MAS, interlacing as template
// parameters), fixed point with the float32 redo of mode 1.
template <int MAS, bool INTER>
__device__ __forceinline__ void bt_deposit_bin(unsigned *smw, const float4 *__restrict__ rec, unsigned begin,
                                               unsigned end, const pyl_batch_real &r, const int *o)
{
    using FS = FxShape<MAS, INTER>;
    constexpr int S = Support<MAS>::S, E = FS::E, CELLS = FS::CELLS;
    float *facc = (float *)smw;
    const long long d = r.dims;
    for (int pass = 0; pass < (INTER ? 2 : 1); pass++) {
        for (int mode = 0; mode < 2; mode++) {
            uint4 *z4 = (uint4 *)smw;
            for (int c = threadIdx.x; c < FS::SMEM / 16; c += blockDim.x) z4[c] = make_uint4(0u, 0u, 0u, 0u);
            __syncthreads();
            unsigned bad = 0u, seen = 0u;
            for (unsigned i = begin + threadIdx.x; i < end; i += blockDim.x) {
                const float4 p = rec[i];
                float C[3][S];
                const int b0 = pass ? fx_support<MAS, 1, E>(p, r.inv, r.halfcell, r.dims, o, C)
                                    : fx_support<MAS, 0, E>(p, r.inv, r.halfcell, r.dims, o, C);
                if (mode == 0) {
                    if (MAS == PYL_MAS_CIC) bad |= (unsigned)!(C[0][1] >= 0.0f && C[1][1] >= 0.0f && C[2][1] >= 0.0f);
                    // z weights times 2^22 (exact): each corner one FFMA into the fixed-point format
#pragma unroll
                    for (int q = 0; q < S; q++) C[2][q] = __fmul_rn(C[2][q], FX_SCALE);
                    seen |= fx_scatter_or<MAS, E, (MAS == PYL_MAS_NGP), true>(smw, b0, C);
                } else {
                    float_scatter<MAS, E>(facc, b0, C);
                }
            }
            if (__syncthreads_or((int)(bad | (seen >> 31))) && mode == 0) {
                __syncthreads();
                continue;
            }
            float *out = pass == 0 ? r.grid : r.grid_interlaced;
            for (int c = threadIdx.x; c < CELLS; c += blockDim.x) {
                const unsigned w = smw[c];
                if (w == 0u) continue;
                const float v = mode == 1 ? __uint_as_float(w)
                                          : (MAS == PYL_MAS_NGP ? __uint2float_rn(w)
                                                                : __fmul_rn(__uint2float_rn(w), FX_INV));
                const int lz = c % E, ly = (c / E) % E, lx = c / (E * E);
                const long long gx = add_wrap(o[0], lx, d), gy = add_wrap(o[1], ly, d), gz = add_wrap(o[2], lz, d);
                atomicAdd(out + (gx * d + gy) * d + gz, __fmul_rn(v, r.scale));
            }
            __syncthreads();
            break;
        }
    }
}

constexpr size_t BT_DEPOSIT_SMEM = FxShape<PYL_MAS_PCS, true>::SMEM;

__global__ void __launch_bounds__(1024) bt_deposit_kernel(const pyl_batch_real *__restrict__ reals, int n_reals,
                                                          const unsigned *__restrict__ tile_base,
                                                          unsigned total_tiles, const unsigned *__restrict__ offsets,
                                                          unsigned n_total, const float4 *__restrict__ rec,
                                                          unsigned *counter)
{
    extern __shared__ __align__(16) unsigned bsm[];
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const unsigned t = (unsigned)cur;
        if (t >= total_tiles) break;
        const unsigned end = min(offsets[t + 1], n_total), begin = min(offsets[t], end);
        if (begin == end) {
            __syncthreads();
            continue;
        }
        int lo = 0, hi = n_reals;                       // last realization with tile_base <= t
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (tile_base[mid] <= t) lo = mid; else hi = mid;
        }
        const pyl_batch_real r = reals[lo];
        const int nt = bt_nt(r.dims);
        const int local = (int)(t - tile_base[lo]);
        const int o[3] = {(local / (nt * nt)) * TB, ((local / nt) % nt) * TB, (local % nt) * TB};
        const bool inter = r.grid_interlaced != nullptr;
        switch (r.mas * 2 + (inter ? 1 : 0)) {
            case 2 * PYL_MAS_NGP:     bt_deposit_bin<PYL_MAS_NGP, false>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_NGP + 1: bt_deposit_bin<PYL_MAS_NGP, true>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_CIC:     bt_deposit_bin<PYL_MAS_CIC, false>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_CIC + 1: bt_deposit_bin<PYL_MAS_CIC, true>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_TSC:     bt_deposit_bin<PYL_MAS_TSC, false>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_TSC + 1: bt_deposit_bin<PYL_MAS_TSC, true>(bsm, rec, begin, end, r, o); break;
            case 2 * PYL_MAS_PCS:     bt_deposit_bin<PYL_MAS_PCS, false>(bsm, rec, begin, end, r, o); break;
            default:                  bt_deposit_bin<PYL_MAS_PCS, true>(bsm, rec, begin, end, r, o); break;
        }
    }
}

struct BtWs {
    unsigned *counts, *offsets, *cursor, *counters;
    float4 *rec;
    size_t bytes;
};

inline size_t bt_align(size_t v) { return (v + 255) / 256 * 256; }

BtWs bt_layout(void *base, unsigned total_tiles, long long total_particles)
{
    BtWs w;
    char *b = (char *)base;
    size_t o = 0;
    w.counts = (unsigned *)(b + o); o = bt_align(o + 4 * ((size_t)total_tiles + 1));
    w.offsets = (unsigned *)(b + o); o = bt_align(o + 4 * ((size_t)total_tiles + 1));
    w.cursor = (unsigned *)(b + o); o = bt_align(o + 4 * ((size_t)total_tiles + 1));
    w.counters = (unsigned *)(b + o); o = bt_align(o + 4 * 4);
    w.rec = (float4 *)(b + o); o = bt_align(o + 16 * (size_t)total_particles);
    w.bytes = o;
    return w;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_ma_batch(const pyl_batch_real *reals, int n_reals, const pyl_batch_item *items,
                            int n_items, unsigned *counter, int ctas_per_sm, void *stream)
{
    PYL_CHECK_ARG(reals != nullptr && items != nullptr && counter != nullptr, "null pointer");
    PYL_CHECK_ARG(n_reals >= 1 && n_items >= 0, "bad sizes");
    PYL_CHECK_ARG(ctas_per_sm >= 1 && ctas_per_sm <= 8, "ctas_per_sm must be 1..8");
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    if (n_items == 0) return PYL_OK;
    batch_deposit_kernel<<<num_sms() * ctas_per_sm, 256, 0, st>>>(reals, items, n_items, counter);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_fill(float *p, int64_t n, float value, void *stream)
{
    PYL_CHECK_ARG(p != nullptr && n >= 0, "bad arguments");
    if (n == 0) return PYL_OK;
    long long b = (n + 255) / 256;
    if (b > (long long)num_sms() * 8) b = (long long)num_sms() * 8;
    fill_value_kernel<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(p, n, value);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_scale(float *p, int64_t n, float factor, void *stream)
{
    PYL_CHECK_ARG(p != nullptr && n >= 0, "bad arguments");
    if (n == 0) return PYL_OK;
    long long b = (n + 255) / 256;
    if (b > (long long)num_sms() * 8) b = (long long)num_sms() * 8;
    scale_value_kernel<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(p, n, factor);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" size_t pyl_ma_batch_tiled_workspace_size(uint32_t total_tiles, int64_t total_particles)
{
    if (total_particles < 0) return 0;
    return bt_layout(nullptr, total_tiles, total_particles).bytes;
}

extern "C" int pyl_ma_batch_tiled(const pyl_batch_real *reals, int n_reals, const pyl_batch_item *items,
                                  int n_items, const uint32_t *tile_base, uint32_t total_tiles,
                                  int64_t total_particles, void *workspace, size_t workspace_bytes,
                                  int ctas_per_sm, void *stream)
{
    PYL_CHECK_ARG(reals != nullptr && items != nullptr && tile_base != nullptr, "null pointer");
    PYL_CHECK_ARG(n_reals >= 1 && n_items >= 0 && total_tiles >= 1, "bad sizes");
    PYL_CHECK_ARG(total_particles >= 0 && total_particles < 0xFFFFFFFFLL, "particle total out of range");
    PYL_CHECK_ARG(ctas_per_sm >= 1 && ctas_per_sm <= 8, "ctas_per_sm must be 1..8");
    const BtWs ws = bt_layout(workspace, total_tiles, total_particles);
    if (workspace == nullptr || workspace_bytes < ws.bytes) {
        set_error("pyl_ma_batch_tiled: needs " + std::to_string(ws.bytes) + " workspace bytes");
        return PYL_ERR_WORKSPACE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(ws.counts, 0, 4 * ((size_t)total_tiles + 1), st));
    PYL_CUDA(cudaMemsetAsync(ws.counters, 0, 16, st));
    if (n_items == 0) return PYL_OK;
    const unsigned grid = (unsigned)(num_sms() * ctas_per_sm);
    bt_count_kernel<<<grid, 1024, 0, st>>>(reals, items, n_items, tile_base, ws.counts, ws.counters);
    PYL_LAUNCH_CHECK();
    bt_scan_kernel<<<1, 1024, 0, st>>>(ws.counts, total_tiles, ws.offsets, ws.cursor);
    PYL_LAUNCH_CHECK();
    PYL_CUDA(ensure_smem(bt_place_kernel, BT_PLACE_SMEM));
    bt_place_kernel<<<grid, 1024, BT_PLACE_SMEM, st>>>(reals, items, n_items, tile_base, ws.cursor,
                                                       (unsigned)total_particles, ws.rec, ws.counters + 1);
    PYL_LAUNCH_CHECK();
    PYL_CUDA(ensure_smem(bt_deposit_kernel, BT_DEPOSIT_SMEM));
    bt_deposit_kernel<<<(unsigned)num_sms(), 1024, BT_DEPOSIT_SMEM, st>>>(
        reals, n_reals, tile_base, total_tiles, ws.offsets, (unsigned)total_particles, ws.rec, ws.counters + 2);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
