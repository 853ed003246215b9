// SORTED strategy of pyl_ma / pyl_ma_overdensity: a deterministic mass
// assignment built from a sort by cell key and a per-cell segmented reduction.
//
//   1. key kernel: every particle's base cell (the first cell of its support on
//      each axis, wrapped; MAS_library.pyx:123-545 index arithmetic) as a 32-bit
//      key (ix*dims + iy)*dims + iz, value = particle index.
//   2. stable LSD radix sort of (key, index), 8-bit digits: per-tile digit
//      histograms, one exclusive scan over [digit][tile], and a scatter that
//      ranks each tile's keys stably (warp match + per-warp digit counts) and
//      stages them in shared memory so global writes are coalesced.  Equal keys
//      keep increasing particle index.
//   3. run table: for every cell the [start, end) range of its particles in the
//      sorted order (empty cells keep the all-ones marker).
//   4. the particles' positions (and weights) gathered into sorted order.
//   5. gather deposit: one thread per output cell walks the S^3 neighbouring
//      base cells in a fixed order and, within each run, the particles in index
//      order, adding the weight of its corner; the CTA stages the particles of
//      its base cells in shared memory with their weights computed once per x
//      offset (sd_deposit_kernel).  The interlaced grid runs
//      steps 1-5 again on the shifted positions (its own sort), so its cells
//      also visit S^3 base cells (a gather over the plain grid's sort visited
//      (S+1)^3 and checked each corner: 4x the work for TSC).
//      No atomics: every cell's sum has one fixed order, so the grid is
//      bit-reproducible whatever the launch configuration; NGP sums each cell's
//      particles in index order, exactly the serial reference loop.
// Limits: dims^3 <= 2^32 (dims <= 1625) and fewer than 2^32 particles.
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "common.cuh"
#include "deposit.cuh"
#include "sorted.cuh"

namespace pyl {
namespace {

constexpr int RS_THREADS = 256;
constexpr int RS_ITEMS = 16;
constexpr int RS_TILE = RS_THREADS * RS_ITEMS;       // 4096 keys per tile
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_BLOCK = SCAN_THREADS * SCAN_ITEMS;  // 4096 entries per scan block
constexpr unsigned EMPTY = 0xffffffffu;

template <int MAS>
__device__ __forceinline__ int sd_first(float p, float inv)
{
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_CIC) return __float2int_rz(dist);
    const float fl = floorf(dist);
    const float frac = __fsub_rn(dist, fl);
    const int fi = __float2int_rz(fl);
    if (MAS == PYL_MAS_NGP) {
        int k = fi + (frac >= 0.5f ? 1 : 0);
        if (dist < -0.5f && frac != 0.5f) k += 1;
        return k;
    }
    if (MAS == PYL_MAS_TSC) return fi - 1 + (frac >= 0.5f ? 1 : 0);
    return fi - 1;
}

// Weight of support cell j (0 <= j < S) of one coordinate and the first cell;
// the same float arithmetic as the scatter kernels (mas.cu axis_weights).
template <int MAS>
__device__ __forceinline__ float sd_weight(float p, float inv, int j, int *first)
{
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_NGP) {
        *first = sd_first<MAS>(p, inv);
        return 1.0f;
    } else if (MAS == PYL_MAS_CIC) {
        const float t = truncf(dist);
        const float u = __fsub_rn(dist, t);
        *first = __float2int_rz(t);
        return j == 0 ? __fsub_rn(1.0f, u) : u;
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        *first = __float2int_rz(fl) - 1 + (frac >= 0.5f ? 1 : 0);
        const float fmn = __fsub_rn(__fadd_rn(fl, frac >= 0.5f ? 1.0f : 0.0f), 2.0f);
        const float diff = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
        if (diff < 0.5f) return __fsub_rn(0.75f, __fmul_rn(diff, diff));
        if (diff < 1.5f) {
            const float t = __fsub_rn(1.5f, diff);
            return __fmul_rn(__fmul_rn(0.5f, t), t);
        }
        return 0.0f;
    } else {
        const float fl = floorf(dist);
        *first = __float2int_rz(fl) - 1;
        const float fmn = __fsub_rn(fl, 2.0f);
        const float d = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
        if (d < 1.0f) {
            const float a = __fmul_rn(__fmul_rn(6.0f, d), d);
            const float b = __fmul_rn(__fmul_rn(__fmul_rn(3.0f, d), d), d);
            return __fdiv_rn(__fadd_rn(__fsub_rn(4.0f, a), b), 6.0f);
        }
        if (d < 2.0f) {
            const float t = __fsub_rn(2.0f, d);
            return __fdiv_rn(__fmul_rn(__fmul_rn(t, t), t), 6.0f);
        }
        return 0.0f;
    }
}

// ---- 1. keys --------------------------------------------------------------
// SHIFT: the half-cell-shifted grid's pass, on positions p + halfcell (the
// float32 sum the other strategies form for the interlaced grid).
template <int MAS, bool SHIFT>
__global__ void __launch_bounds__(256) sd_key_kernel(const float *__restrict__ pos, long long n, float inv,
                                                     float halfcell, int dims, unsigned *__restrict__ keys,
                                                     unsigned *__restrict__ vals)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const unsigned d = (unsigned)dims;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float p[3] = {__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2)};
        if (SHIFT)
            for (int a = 0; a < 3; a++) p[a] = __fadd_rn(p[a], halfcell);
        const unsigned cx = (unsigned)wrap_index(sd_first<MAS>(p[0], inv), dims);
        const unsigned cy = (unsigned)wrap_index(sd_first<MAS>(p[1], inv), dims);
        const unsigned cz = (unsigned)wrap_index(sd_first<MAS>(p[2], inv), dims);
        keys[i] = (cx * d + cy) * d + cz;
        vals[i] = (unsigned)i;
    }
}

// ---- 2. radix sort ----------------------------------------------------------
// Per-tile histogram of one digit, stored digit-major: hist[digit * tiles + tile].
__global__ void __launch_bounds__(RS_THREADS) rs_hist_kernel(const unsigned *__restrict__ keys, long long n,
                                                             int shift, unsigned tiles,
                                                             unsigned *__restrict__ hist)
{
    __shared__ unsigned h[256];
    h[threadIdx.x] = 0u;
    __syncthreads();
    const long long base = (long long)blockIdx.x * RS_TILE;
#pragma unroll 4
    for (int r = 0; r < RS_ITEMS; r++) {
        const long long i = base + r * RS_THREADS + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
    }
    __syncthreads();
    hist[(long long)threadIdx.x * tiles + blockIdx.x] = h[threadIdx.x];
}

// Exclusive scan of a block of SCAN_THREADS values (one per thread); returns the
// block total through *total.
__device__ __forceinline__ unsigned block_excl_scan(unsigned v, unsigned *warp_sums, unsigned *total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned s = lane < nw ? warp_sums[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    const unsigned prefix = (warp ? warp_sums[warp - 1] : 0u) + x - v;
    if (total) *total = warp_sums[nw - 1];
    __syncthreads();
    return prefix;
}

// Scan phase 1: sum of each SCAN_BLOCK slice.
__global__ void __launch_bounds__(SCAN_THREADS) scan_reduce_kernel(const unsigned *__restrict__ a, long long n,
                                                                   unsigned *__restrict__ partial)
{
    __shared__ unsigned ws[32];
    const long long base = (long long)blockIdx.x * SCAN_BLOCK;
    unsigned s = 0u;
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
        const long long i = base + r * SCAN_THREADS + threadIdx.x;
        if (i < n) s += a[i];
    }
    unsigned tot;
    block_excl_scan(s, ws, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Scan phase 2: exclusive scan of the partial sums by one block.
__global__ void __launch_bounds__(SCAN_THREADS) scan_partials_kernel(unsigned *__restrict__ partial, long long m)
{
    __shared__ unsigned ws[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0u;
    __syncthreads();
    for (long long b = 0; b < m; b += SCAN_THREADS) {
        const long long i = b + threadIdx.x;
        const unsigned v = i < m ? partial[i] : 0u;
        unsigned tot;
        const unsigned ex = block_excl_scan(v, ws, &tot);
        if (i < m) partial[i] = carry + ex;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
}

// Scan phase 3: exclusive scan of each slice in place, offset by its partial.
__global__ void __launch_bounds__(SCAN_THREADS) scan_apply_kernel(unsigned *__restrict__ a, long long n,
                                                                  const unsigned *__restrict__ partial)
{
    __shared__ unsigned ws[32];
    const long long base = (long long)blockIdx.x * SCAN_BLOCK + (long long)threadIdx.x * SCAN_ITEMS;
    unsigned v[SCAN_ITEMS];
    unsigned s = 0u;
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
        v[r] = base + r < n ? a[base + r] : 0u;
        s += v[r];
    }
    unsigned run = partial[blockIdx.x] + block_excl_scan(s, ws, nullptr);
#pragma unroll
    for (int r = 0; r < SCAN_ITEMS; r++) {
        if (base + r < n) a[base + r] = run;
        run += v[r];
    }
}

// Stable scatter of one tile by one digit.  Warp w holds the tile's elements
// w*512 .. w*512+511 (round r, lane l: element w*512 + r*32 + l), so the order
// (warp, round, lane) is the tile's order.  Each warp ranks its elements with
// its own digit counters (a match_any per round, no block barrier), one block
// scan turns the tile's digit counts into each digit's first staging slot and
// each warp's first slot within it, and the tile is staged in digit order in
// shared memory before the coalesced write.
__global__ void __launch_bounds__(RS_THREADS) rs_scatter_kernel(
    const unsigned *__restrict__ kin, const unsigned *__restrict__ vin, long long n, int shift, unsigned tiles,
    const unsigned *__restrict__ goff, unsigned *__restrict__ kout, unsigned *__restrict__ vout)
{
    constexpr int PER_WARP = RS_ITEMS * 32;
    __shared__ unsigned sk[RS_TILE], sv[RS_TILE];
    __shared__ unsigned wc[RS_WARPS][256];   // a warp's count of each digit, then its first slot
    __shared__ unsigned start[256];          // first staging slot of each digit
    __shared__ unsigned gbase[256];          // global position of the digit's first element
    __shared__ unsigned ws[32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const long long tile0 = (long long)blockIdx.x * RS_TILE;
    const long long base = tile0 + (long long)warp * PER_WARP;
    for (int i = lane; i < 256; i += 32) wc[warp][i] = 0u;
    unsigned dg[RS_ITEMS], key[RS_ITEMS], val[RS_ITEMS], rk[RS_ITEMS];
#pragma unroll
    for (int r = 0; r < RS_ITEMS; r++) {
        const long long i = base + r * 32 + lane;
        key[r] = i < n ? kin[i] : 0u;
        val[r] = i < n ? vin[i] : 0u;
        dg[r] = i < n ? ((key[r] >> shift) & 255u) : 256u;
    }
    __syncwarp();
    const unsigned lt = (1u << lane) - 1u;
#pragma unroll
    for (int r = 0; r < RS_ITEMS; r++) {
        const unsigned d = dg[r];
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const unsigned lrank = __popc(peers & lt);
        const unsigned before = d < 256u ? wc[warp][d] : 0u;
        __syncwarp();
        if (lrank == 0u && d < 256u) wc[warp][d] = before + (unsigned)__popc(peers);
        __syncwarp();
        rk[r] = before + lrank;
    }
    __syncthreads();
    // thread t = digit t: the tile's count, its first slot, each warp's first slot
    unsigned c = 0u;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) c += wc[w][t];
    const unsigned s0 = block_excl_scan(c, ws, nullptr);
    start[t] = s0;
    gbase[t] = goff[(long long)t * tiles + blockIdx.x];
    unsigned run = s0;
#pragma unroll
    for (int w = 0; w < RS_WARPS; w++) {
        const unsigned v = wc[w][t];
        wc[w][t] = run;
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < RS_ITEMS; r++) {
        if (dg[r] < 256u) {
            const unsigned slot = wc[warp][dg[r]] + rk[r];
            sk[slot] = key[r];
            sv[slot] = val[r];
        }
    }
    __syncthreads();
    const unsigned cnt = (unsigned)min((long long)RS_TILE, n - tile0);
    for (unsigned p = t; p < cnt; p += RS_THREADS) {
        const unsigned k = sk[p];
        const unsigned d = (k >> shift) & 255u;
        const unsigned g = gbase[d] + (p - start[d]);
        kout[g] = k;
        vout[g] = sv[p];
    }
}

// ---- 3. run table -------------------------------------------------------------
__global__ void __launch_bounds__(256) sd_runs_kernel(const unsigned *__restrict__ keys, long long n,
                                                      uint2 *__restrict__ runs)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const unsigned k = keys[j];
        if (j == 0 || keys[j - 1] != k) runs[k].x = (unsigned)j;
        if (j == n - 1 || keys[j + 1] != k) runs[k].y = (unsigned)(j + 1);
    }
}

__global__ void __launch_bounds__(256) sd_fill2_kernel(uint2 *__restrict__ p, long long n)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        p[i] = make_uint2(EMPTY, EMPTY);
}

// ---- 4. positions in sorted order -------------------------------------------
template <bool SHIFT>
__global__ void __launch_bounds__(256) sd_gather_kernel(const float *__restrict__ pos, const float *__restrict__ w,
                                                        const unsigned *__restrict__ vals, long long n,
                                                        float halfcell, float4 *__restrict__ spos)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long j = (long long)blockIdx.x * blockDim.x + threadIdx.x; j < n; j += stride) {
        const long long i = vals[j];
        float4 p = make_float4(__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2),
                               w ? __ldg(w + i) : 1.0f);
        if (SHIFT) {
            p.x = __fadd_rn(p.x, halfcell);
            p.y = __fadd_rn(p.y, halfcell);
            p.z = __fadd_rn(p.z, halfcell);
        }
        spos[j] = p;
    }
}

// ---- 5. gather deposit ----------------------------------------------------------
// Cell (x, y, z) sums, over base cells c - (l, m, q) with offsets 0..S-1 per axis
// in that order and each run's particles in index order, the weight of its corner
// ((c0 c1) c2, times the weight), in float32 adds: a fixed order, so the grid is
// the same bits on every run.  The half-cell-shifted grid runs the same gather on
// its own sort of the shifted positions (sorted_pass<MAS, true>).
// scale/base: out = (fold ? out : 0) + sum in fixed order, then
//   (fold ? sum : out_old + sum * scale).

// One (l, m) of one cell straight from the runs and the sorted positions.
template <int MAS, bool WEIGHTED>
__device__ __forceinline__ float sd_direct_lm(const float4 *__restrict__ spos, const uint2 *__restrict__ runs,
                                              long long row, int z, int dims, float inv, int l, int m, float acc)
{
    constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS;
#pragma unroll
    for (int q = 0; q < S; q++) {
        const uint2 rr = runs[row + wrap_index(z - q, dims)];
        if (rr.x == EMPTY) continue;
        for (unsigned j = rr.x; j < rr.y; j++) {
            const float4 p = spos[j];
            int f;
            const float c0 = sd_weight<MAS>(p.x, inv, l, &f);
            const float c1 = sd_weight<MAS>(p.y, inv, m, &f);
            const float c2 = sd_weight<MAS>(p.z, inv, q, &f);
            float v = MAS == PYL_MAS_NGP ? 1.0f : __fmul_rn(__fmul_rn(c0, c1), c2);
            if (WEIGHTED) v = MAS == PYL_MAS_NGP ? p.w : __fmul_rn(v, p.w);
            acc = __fadd_rn(acc, v);
        }
    }
    return acc;
}

constexpr int SDT_CAP = 1024;      // particles a CTA stages per x offset l (shared-memory capacity)
std::atomic<int> g_sd_stage_cap{SDT_CAP};   // pyl_sorted_set_stage_limit

// Of one staged particle: the products (x weight at offset l) (y weight at offset
// m) for m = 0..S-1, the z weights at offsets 0..S-1 (and the weight).
template <int MAS, bool WEIGHTED>
struct SdStage {
    static constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS;
    static constexpr int NV = 2 * S + (WEIGHTED ? 1 : 0);
    static constexpr int RY = 8 + S - 1, W = 32 + S - 1;   // base rows along y, base cells along z
    static constexpr int NC = RY * W;                       // window cells of one l
};

// A CTA takes the 32 x 8 cells (z, y) of one x plane; block (32, 8), grid
// (ceil(dims / 32), ceil(dims / 8), dims).  For each x offset l the CTA reads the
// runs of the (8 + S - 1) x (32 + S - 1) base cells its cells reach in plane
// x - l, places their particles in shared memory by a block scan, and computes
// each staged particle's S (x, y) weight products and S z weights once (all S
// weights of an axis from one axis_weights, the arithmetic of sd_weight),
// instead of once for each of the S^2 cells of the plane that it reaches.
// Every cell then sums its base cells' staged particles in the order above, with
// the same products and adds as sd_direct_lm, which takes over for an l whose
// window holds more than cap (at most SDT_CAP) particles.
template <int MAS, bool WEIGHTED>
__global__ void __launch_bounds__(256) sd_deposit_kernel(const float4 *__restrict__ spos,
                                                         const uint2 *__restrict__ runs, int dims, float inv,
                                                         float *__restrict__ out, float scale_h,
                                                         const float *__restrict__ scale_d, int fold,
                                                         unsigned cap)
{
    using ST = SdStage<MAS, WEIGHTED>;
    constexpr int S = ST::S, NV = ST::NV, W = ST::W, NC = ST::NC;
    constexpr int CPT = (NC + 255) / 256;                   // window cells a thread reads
    __shared__ unsigned s_off[NC + 1];                      // staged start of each window cell
    __shared__ unsigned s_rx[NC];                           // its first particle in sorted order
    __shared__ float s_e[SDT_CAP * NV];
    __shared__ unsigned s_wsum[8];
    const int tid = threadIdx.y * 32 + threadIdx.x, lane = threadIdx.x, warp = threadIdx.y;
    const int z0 = blockIdx.x * 32, y0 = blockIdx.y * 8;
    const int z = z0 + threadIdx.x, y = y0 + threadIdx.y, x = blockIdx.z;
    const bool live = z < dims && y < dims;
    const long long d = dims;
    const long long cell = ((long long)x * d + y) * d + z;
    float acc = (fold && live) ? out[cell] : 0.0f;
#pragma unroll 1
    for (int l = 0; l < S; l++) {
        const long long plane = (long long)wrap_index(x - l, dims) * d;
        // 1. runs of this thread's window cells tid * CPT + k (row r = c / W, cell
        //    i = c % W: base cell (y0 - (S - 1) + r, z0 - (S - 1) + i)); cells past
        //    the grid's end serve no live cell and stay empty
        unsigned cnt[CPT], sum = 0;
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            const int c = tid * CPT + k;
            cnt[k] = 0;
            if (c < NC) {
                const int yb = y0 - (S - 1) + c / W, zb = z0 - (S - 1) + c % W;
                unsigned rx = 0;
                if (yb < dims && zb < dims) {
                    const uint2 rr = runs[(plane + wrap_index(yb, dims)) * d + wrap_index(zb, dims)];
                    if (rr.x != EMPTY) { cnt[k] = rr.y - rr.x; rx = rr.x; }
                }
                s_rx[c] = rx;
            }
            sum += cnt[k];
        }
        // 2. block exclusive scan of the thread sums
        unsigned inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += t;
        }
        if (lane == 31) s_wsum[warp] = inc;
        __syncthreads();
        unsigned before = 0, total = 0;
#pragma unroll
        for (int w2 = 0; w2 < 8; w2++) {
            const unsigned v = s_wsum[w2];
            before += w2 < warp ? v : 0u;
            total += v;
        }
        unsigned run = before + inc - sum;
#pragma unroll
        for (int k = 0; k < CPT; k++) {
            const int c = tid * CPT + k;
            if (c < NC) s_off[c] = run;
            run += cnt[k];
        }
        if (tid == 0) s_off[NC] = total;
        __syncthreads();                                    // s_wsum reads done, s_off / s_rx written
        if (total > cap) {                                  // the same for the whole CTA (cap <= SDT_CAP)
            if (live)
#pragma unroll 1
                for (int m = 0; m < S; m++)
                    acc = sd_direct_lm<MAS, WEIGHTED>(spos, runs, (plane + wrap_index(y - m, dims)) * d, z, dims,
                                                      inv, l, m, acc);
            __syncthreads();
            continue;
        }
        // 3. stage: particle t of the window is particle t - s_off[c] of window cell c
        for (unsigned t = tid; t < total; t += 256) {
            int lo = 0, hi = NC;                            // s_off[lo] <= t < s_off[hi]
            while (hi - lo > 1) {
                const int mid = (lo + hi) >> 1;
                if (s_off[mid] <= t) lo = mid; else hi = mid;
            }
            const float4 p = spos[s_rx[lo] + (t - s_off[lo])];
            float *e = s_e + t * NV;
            if (MAS == PYL_MAS_NGP) {
                e[0] = e[1] = 1.0f;
            } else {
                float cx[S], cy[S], cz[S];
                axis_weights<MAS>(p.x, inv, cx);
                axis_weights<MAS>(p.y, inv, cy);
                axis_weights<MAS>(p.z, inv, cz);
                float c0 = cx[0];
#pragma unroll
                for (int j = 1; j < S; j++) c0 = l == j ? cx[j] : c0;
#pragma unroll
                for (int m = 0; m < S; m++) e[m] = __fmul_rn(c0, cy[m]);
#pragma unroll
                for (int q = 0; q < S; q++) e[S + q] = cz[q];
            }
            if (WEIGHTED) e[2 * S] = p.w;
        }
        __syncthreads();
        // 4. each cell: base rows y - m, base cells z - q, particles in index order
        if (live) {
#pragma unroll 1
            for (int m = 0; m < S; m++) {
#pragma unroll
                for (int q = 0; q < S; q++) {
                    const int c = (warp + (S - 1) - m) * W + lane + (S - 1) - q;
                    const unsigned a = s_off[c], b = s_off[c + 1];
                    for (unsigned t = a; t < b; t++) {
                        const float *e = s_e + t * NV;
                        float v = MAS == PYL_MAS_NGP ? 1.0f : __fmul_rn(e[m], e[S + q]);
                        if (WEIGHTED) v = MAS == PYL_MAS_NGP ? e[2 * S] : __fmul_rn(v, e[2 * S]);
                        acc = __fadd_rn(acc, v);
                    }
                }
            }
        }
        __syncthreads();                                    // before the next l restages
    }
    if (!live) return;
    if (fold) {
        out[cell] = acc;
    } else if (acc != 0.0f) {
        const float s = scale_d ? *scale_d : scale_h;
        out[cell] = __fadd_rn(out[cell], __fmul_rn(acc, s));
    }
}

inline size_t al(size_t v) { return (v + 255) / 256 * 256; }

struct SortedWs {
    unsigned *k0, *v0, *k1, *v1, *hist, *partial;
    uint2 *runs;
    float4 *spos;
    unsigned tiles;
    long long hist_len, parts;
    size_t bytes;
};

SortedWs sorted_layout(void *base, long long n, int dims)
{
    SortedWs w;
    const long long cells = (long long)dims * dims * dims;
    w.tiles = (unsigned)((n + RS_TILE - 1) / RS_TILE);
    w.hist_len = 256LL * w.tiles;
    w.parts = (w.hist_len + SCAN_BLOCK - 1) / SCAN_BLOCK;
    char *b = (char *)base;
    size_t o = 0;
    w.k0 = (unsigned *)(b + o); o = al(o + 4 * (size_t)n);
    w.v0 = (unsigned *)(b + o); o = al(o + 4 * (size_t)n);
    w.k1 = (unsigned *)(b + o); o = al(o + 4 * (size_t)n);
    w.v1 = (unsigned *)(b + o); o = al(o + 4 * (size_t)n);
    w.hist = (unsigned *)(b + o); o = al(o + 4 * (size_t)w.hist_len);
    w.partial = (unsigned *)(b + o); o = al(o + 4 * (size_t)w.parts);
    w.runs = (uint2 *)(b + o); o = al(o + 8 * (size_t)cells);
    w.spos = (float4 *)(b + o); o = al(o + 16 * (size_t)n);
    w.bytes = o;
    return w;
}

inline unsigned blocks_for(long long n, int threads, int per_sm)
{
    long long b = (n + threads - 1) / threads;
    const long long cap = (long long)num_sms() * per_sm;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

// One grid: keys of the (shifted, for SHIFT) positions, stable radix sort, runs,
// positions gathered into sorted order, gather deposit.
template <int MAS, bool SHIFT>
int sorted_pass(const float *pos, const float *w, long long n, float *out, int dims, float inv, float halfcell,
                const SortedWs &ws, float scale_h, const float *scale_d, bool fold, cudaStream_t st)
{
    const long long cells = (long long)dims * dims * dims;
    stage_mark(PYL_STAGE_SORT, true, st);
    sd_key_kernel<MAS, SHIFT><<<blocks_for(n, 256, 16), 256, 0, st>>>(pos, n, inv, halfcell, dims, ws.k0, ws.v0);
    PYL_LAUNCH_CHECK();
    int bits = 1;
    while (bits < 32 && (1ull << bits) < (unsigned long long)cells) bits++;
    unsigned *kin = ws.k0, *vin = ws.v0, *kout = ws.k1, *vout = ws.v1;
    for (int shift = 0; shift < bits; shift += 8) {
        rs_hist_kernel<<<ws.tiles, RS_THREADS, 0, st>>>(kin, n, shift, ws.tiles, ws.hist);
        PYL_LAUNCH_CHECK();
        scan_reduce_kernel<<<(unsigned)ws.parts, SCAN_THREADS, 0, st>>>(ws.hist, ws.hist_len, ws.partial);
        PYL_LAUNCH_CHECK();
        scan_partials_kernel<<<1, SCAN_THREADS, 0, st>>>(ws.partial, ws.parts);
        PYL_LAUNCH_CHECK();
        scan_apply_kernel<<<(unsigned)ws.parts, SCAN_THREADS, 0, st>>>(ws.hist, ws.hist_len, ws.partial);
        PYL_LAUNCH_CHECK();
        rs_scatter_kernel<<<ws.tiles, RS_THREADS, 0, st>>>(kin, vin, n, shift, ws.tiles, ws.hist, kout, vout);
        PYL_LAUNCH_CHECK();
        unsigned *t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
    sd_fill2_kernel<<<blocks_for(cells, 256, 16), 256, 0, st>>>(ws.runs, cells);
    PYL_LAUNCH_CHECK();
    sd_runs_kernel<<<blocks_for(n, 256, 16), 256, 0, st>>>(kin, n, ws.runs);
    PYL_LAUNCH_CHECK();
    sd_gather_kernel<SHIFT><<<blocks_for(n, 256, 16), 256, 0, st>>>(pos, w, vin, n, halfcell, ws.spos);
    PYL_LAUNCH_CHECK();
    stage_mark(PYL_STAGE_SORT, false, st);
    stage_mark(PYL_STAGE_DEPOSIT, true, st);
    const dim3 blk(32, 8), grd((unsigned)((dims + 31) / 32), (unsigned)((dims + 7) / 8), (unsigned)dims);
    const int f = fold ? 1 : 0;
    const unsigned cap = (unsigned)g_sd_stage_cap.load();
    if (w) sd_deposit_kernel<MAS, true><<<grd, blk, 0, st>>>(ws.spos, ws.runs, dims, inv, out, scale_h, scale_d, f, cap);
    else sd_deposit_kernel<MAS, false><<<grd, blk, 0, st>>>(ws.spos, ws.runs, dims, inv, out, scale_h, scale_d, f, cap);
    PYL_LAUNCH_CHECK();
    stage_mark(PYL_STAGE_DEPOSIT, false, st);
    return PYL_OK;
}

template <int MAS>
int sorted_run(const float *pos, const float *w, long long n, float *grid, float *grid2, int dims, float inv,
               float halfcell, void *workspace, float scale_h, const float *scale_d, bool fold, cudaStream_t st)
{
    const SortedWs ws = sorted_layout(workspace, n, dims);
    int rc = sorted_pass<MAS, false>(pos, w, n, grid, dims, inv, halfcell, ws, scale_h, scale_d, fold, st);
    if (rc || !grid2) return rc;
    return sorted_pass<MAS, true>(pos, w, n, grid2, dims, inv, halfcell, ws, scale_h, scale_d, fold, st);
}

}  // namespace

bool sorted_supported(long long n, int dims)
{
    return n >= 0 && n < 0xFFFFFFFFLL && dims >= 1 && (long long)dims * dims * dims <= 0xFFFFFFFFLL;
}

size_t sorted_workspace_bytes(long long n, int dims)
{
    return sorted_layout(nullptr, n, dims).bytes;
}

int launch_sorted(int mas, const float *pos, const float *w, long long n, float *grid, float *grid2, int dims,
                  float inv, float halfcell, void *workspace, float scale_h, const float *scale_d, bool fold,
                  cudaStream_t st)
{
    if (!sorted_supported(n, dims)) {
        set_error("sorted strategy: needs dims^3 <= 2^32 and fewer than 2^32 particles");
        return PYL_ERR_UNSUPPORTED;
    }
    if (n == 0) return PYL_OK;
    switch (mas) {
        case PYL_MAS_NGP: return sorted_run<PYL_MAS_NGP>(pos, w, n, grid, grid2, dims, inv, halfcell, workspace,
                                                         scale_h, scale_d, fold, st);
        case PYL_MAS_CIC: return sorted_run<PYL_MAS_CIC>(pos, w, n, grid, grid2, dims, inv, halfcell, workspace,
                                                         scale_h, scale_d, fold, st);
        case PYL_MAS_TSC: return sorted_run<PYL_MAS_TSC>(pos, w, n, grid, grid2, dims, inv, halfcell, workspace,
                                                         scale_h, scale_d, fold, st);
        case PYL_MAS_PCS: return sorted_run<PYL_MAS_PCS>(pos, w, n, grid, grid2, dims, inv, halfcell, workspace,
                                                         scale_h, scale_d, fold, st);
    }
    set_error("sorted strategy: bad MAS");
    return PYL_ERR_INVALID;
}

}  // namespace pyl

extern "C" int pyl_sorted_set_stage_limit(int max_particles)
{
    PYL_CHECK_ARG(max_particles <= pyl::SDT_CAP, "max_particles above the stage capacity (1024)");
    pyl::g_sd_stage_cap.store(max_particles < 0 ? pyl::SDT_CAP : max_particles);
    return PYL_OK;
}
