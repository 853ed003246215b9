// The tiled mass-assignment pipeline: per-chunk bin histograms, scans, placement of
// the particles into bin order (one or two levels), the per-bin shared-memory
// deposit and the halo kernel of the owned-cell write-out.  Included once per MAS by
// tiled_ngp.cu .. tiled_pcs.cu, which instantiate launch_tiled; the kernels have
// internal linkage in each of those units.
#pragma once
#include <cuda_runtime.h>

#include "tiled.cuh"
#include "tma.cuh"

namespace pyl {
namespace {

// ------------------------------------------------------------------- TILED path
// Tiles are TB^3 cells.  Binning (per-CTA shared-memory histograms, no
// per-particle global atomics):
//   1. chunk_hist:  CTA c counts its contiguous chunk of particles per tile in
//                   shared memory and writes the row hist[c][*];
//   2. colscan:     hist[c][t] <- sum_{c'<c} hist[c'][t], total[t] = column sum;
//   3. tile_scan:   offsets[t] = exclusive scan of total;
//   4. chunk_scatter: CTA c starts shared-memory cursors at offsets[t] + hist[c][t]
//                   and writes each particle to its tile's range.
// Grids with more than HIST_MAX_TILES tiles count and place particles with
// global atomics instead (the same tile layout).  Then one CTA per tile deposits
// into a (TB+H)^3 shared-memory block (H = kernel support - 1, +1 for the
// interlaced shift) and adds it to the grid with coalesced red.global.add.


__device__ __forceinline__ void tile_coords(long long key, const TileGeom &g, int &tx, int &ty, int &tz)
{
    const int local = (int)(key & 63);
    const long long coarse = key >> 6;
    const int cz = (int)(coarse % g.nc), cy = (int)((coarse / g.nc) % g.nc), cx = (int)(coarse / ((long long)g.nc * g.nc));
    tx = cx * 4 + (local >> 4);
    ty = cy * 4 + ((local >> 2) & 3);
    tz = cz * 4 + (local & 3);
}

template <int MAS>
__device__ __forceinline__ unsigned tile_key(const float *p, float inv, const TileGeom &g)
{
    unsigned c[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int f = axis_first<MAS>(p[a], inv);
        if (g.mask) c[a] = (unsigned)f & g.mask;                 // a uniform branch: the same for all threads
        else c[a] = (unsigned)f < (unsigned)g.dims ? (unsigned)f : (unsigned)wrap_index(f, g.dims);   // rare: past the edge
    }
    return tile_key_of(c[0] / TB, c[1] / TB, c[2] / TB, g);
}

template <int MAS>
__global__ void __launch_bounds__(1024) chunk_hist_kernel(const float *__restrict__ pos, long long n,
                                                          long long chunk, float inv, TileGeom g,
                                                          unsigned *__restrict__ hist)
{
    extern __shared__ unsigned cnt[];
    const int T = (int)g.ntiles;
    for (int t = threadIdx.x; t < T; t += blockDim.x) cnt[t] = 0;
    __syncthreads();
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    for (long long i = b + threadIdx.x; i < e; i += blockDim.x) {
        const float p[3] = {__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2)};
        atomicAdd(cnt + tile_key<MAS>(p, inv, g), 1u);
    }
    __syncthreads();
    unsigned *row = hist + (long long)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) row[t] = cnt[t];
}

// hist[c][t] <- exclusive prefix over c; total[t] <- column sum.  Thread per tile.
__global__ void __launch_bounds__(256) colscan_kernel(unsigned *__restrict__ hist, int C, int T,
                                                      unsigned *__restrict__ total)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= T) return;
    unsigned run = 0;
    int c = 0;
    for (; c + 8 <= C; c += 8) {
        unsigned v[8];
#pragma unroll
        for (int j = 0; j < 8; j++) v[j] = hist[(long long)(c + j) * T + t];
#pragma unroll
        for (int j = 0; j < 8; j++) { hist[(long long)(c + j) * T + t] = run; run += v[j]; }
    }
    for (; c < C; c++) {
        const unsigned v = hist[(long long)c * T + t];
        hist[(long long)c * T + t] = run;
        run += v;
    }
    total[t] = run;
}

// Placement chosen on the device from the input's coherence.  The histogram pass
// counts particles that fall in the same bin as the particle before them; input in
// spatial order (lattices, cell-ordered catalogues) scores near 1, random order
// near 1/bins.  Coherent input is placed in one pass straight into the final
// layout (its writes already form long runs), the rest through the two-level
// shared-memory sorts.  Every candidate launch sits in the stream (and a captured
// graph); a launch whose gate does not match the count returns at once.
struct Gate {
    const unsigned long long *same;    // null: the launch always runs
    unsigned long long thresh;         // coherent when *same >= thresh
    int want;                          // 1: run on coherent input only, 0: on incoherent only
};

__device__ __forceinline__ bool gate_closed(const Gate &gt)
{
    if (!gt.same) return false;
    return (*gt.same >= gt.thresh ? 1 : 0) != gt.want;
}

template <int MAS, bool WEIGHTED>
__global__ void __launch_bounds__(1024) chunk_scatter_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n, long long chunk,
    float inv, TileGeom g, const unsigned *__restrict__ colpre, const unsigned *__restrict__ offsets,
    float4 *__restrict__ rec, Gate gate = Gate{nullptr, 0ull, 0})
{
    extern __shared__ unsigned cur[];
    if (gate_closed(gate)) return;
    const int T = (int)g.ntiles;
    const unsigned *row = colpre + (long long)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) cur[t] = offsets[t] + row[t];
    __syncthreads();
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    constexpr int U = 4;            // particles in flight per thread
    const long long step = (long long)blockDim.x * U;
    for (long long base = b; base < e; base += step) {     // uniform over the block
        const long long i0 = base + threadIdx.x;
        float4 r[U];
        unsigned key[U];
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long i = i0 + (long long)u * blockDim.x;
            if (i < e) {
                r[u] = make_float4(__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2),
                                   WEIGHTED ? __ldg(w + i) : 1.0f);
                const float p[3] = {r[u].x, r[u].y, r[u].z};
                key[u] = tile_key<MAS>(p, inv, g);
            }
        }
        // lanes hold consecutive particles: lanes with equal bins take one
        // reservation of consecutive slots (spatially ordered input has whole
        // warps in one bin)
        const unsigned lane = threadIdx.x & 31u;
#pragma unroll
        for (int u = 0; u < U; u++) {
            const long long i = i0 + (long long)u * blockDim.x;
            const unsigned act = __ballot_sync(0xffffffffu, i < e);
            if (i < e) {
                const unsigned peers = __match_any_sync(act, key[u]);
                const unsigned leader = (unsigned)__ffs(peers) - 1u;
                unsigned slot = 0u;
                if (lane == leader) slot = atomicAdd(cur + key[u], (unsigned)__popc(peers));
                slot = __shfl_sync(peers, slot, leader) + (unsigned)__popc(peers & ((1u << lane) - 1u));
                if (slot < (unsigned long long)n) rec[slot] = r[u];
            }
        }
    }
}

// ---- two-level placement for grids with more than TWO_LEVEL_TILES tiles -----
// Writing each particle straight to its tile leaves one partly filled L2 line
// per (CTA, tile) open; past a few thousand tiles they no longer fit L2 and
// every 16-byte record costs a DRAM read-modify-write.  So: level A sorts each
// 4096-particle batch of a chunk by coarse block (4^3 tiles) in shared memory
// and writes coalesced runs into a temporary buffer laid out [coarse][chunk];
// level B splits each (chunk, coarse) segment into its 64 tiles, again through
// a shared-memory sort, into the final [tile][chunk] layout.  Both levels place
// exactly where the single-level scatter would (same per-(chunk, tile) ranges).
// (Level B is the TMA-staged level_b_tma_kernel below.)
constexpr int LA_THREADS = 1024, LA_U = 4, LA_BATCH = LA_THREADS * LA_U;

// Exclusive scan of n <= blockDim.x values in place; returns nothing, needs a
// 32-entry scratch.  All threads of the block must call it.
__device__ __forceinline__ void block_exclusive_scan(unsigned *v, int n, unsigned *warp_tot)
{
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = (blockDim.x + 31) >> 5;
    unsigned x = t < n ? v[t] : 0u;
    unsigned inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[w] = inc;
    __syncthreads();
    if (w == 0) {
        unsigned wt = lane < nw ? warp_tot[lane] : 0u;
        unsigned wi = wt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        if (lane < nw) warp_tot[lane] = wi - wt;
    }
    __syncthreads();
    if (t < n) v[t] = inc - x + warp_tot[w];
    __syncthreads();
}

template <int MAS, bool WEIGHTED>
__global__ void __launch_bounds__(LA_THREADS) level_a_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n, long long chunk, float inv,
    TileGeom g, const unsigned *__restrict__ colpre, const unsigned *__restrict__ offsets,
    float4 *__restrict__ tmp)
{
    extern __shared__ unsigned la[];
    const int NCO = g.nc * g.nc * g.nc;
    const int T = (int)g.ntiles;
    unsigned *cur = la, *bcnt = cur + NCO, *gst = bcnt + NCO, *wt = gst + NCO;
    float4 *stage = (float4 *)(la + ((3 * NCO + 32 + 3) & ~3));
    unsigned short *sco = (unsigned short *)(stage + LA_BATCH);
    const unsigned *row = colpre + (long long)blockIdx.x * T;
    for (int co = threadIdx.x; co < NCO; co += blockDim.x) {
        unsigned sacc = 0;
        for (int l = 0; l < 64; l++) sacc += row[co * 64 + l];
        cur[co] = offsets[co * 64] + sacc;            // this chunk's slot in the coarse block
    }
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    for (long long s0 = b; s0 < e; s0 += LA_BATCH) {
        for (int co = threadIdx.x; co < NCO; co += blockDim.x) bcnt[co] = 0u;
        __syncthreads();
        float4 r[LA_U];
        unsigned co_u[LA_U], rank[LA_U];
#pragma unroll
        for (int u = 0; u < LA_U; u++) {
            const long long i = s0 + threadIdx.x + (long long)u * LA_THREADS;
            co_u[u] = 0xffffffffu;
            if (i < e) {
                r[u] = make_float4(__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2),
                                   WEIGHTED ? __ldg(w + i) : 1.0f);
                const float p[3] = {r[u].x, r[u].y, r[u].z};
                co_u[u] = tile_key<MAS>(p, inv, g) >> 6;
                rank[u] = atomicAdd(bcnt + co_u[u], 1u);
            }
        }
        __syncthreads();
        for (int co = threadIdx.x; co < NCO; co += blockDim.x) {   // global start of this batch's runs
            gst[co] = cur[co];
            cur[co] += bcnt[co];
        }
        __syncthreads();
        block_exclusive_scan(bcnt, NCO, wt);                         // NCO <= 768 < blockDim.x
#pragma unroll
        for (int u = 0; u < LA_U; u++) {
            if (co_u[u] != 0xffffffffu) {
                const unsigned slot = bcnt[co_u[u]] + rank[u];
                stage[slot] = r[u];
                sco[slot] = (unsigned short)co_u[u];
            }
        }
        __syncthreads();
        const int nb = (int)min((long long)LA_BATCH, e - s0);
        for (int sidx = threadIdx.x; sidx < nb; sidx += blockDim.x) {
            const unsigned co = sco[sidx];
            tmp[gst[co] + (sidx - bcnt[co])] = stage[sidx];
        }
        __syncthreads();
    }
}


// ---- TMA-staged variants ---------------------------------------------------
// The histogram and level-A kernels stream each chunk's positions, and level B
// each (chunk, coarse block) segment's records, through two shared-memory
// buffers filled by bulk copies (cp.async.bulk + mbarrier): the copy of batch
// j+2 runs while batch j is processed, so the loads no longer wait on DRAM
// latency between the batches' barriers.  Positions need a 16-byte aligned base
// and chunks that start on multiples of 4 particles (48 bytes); the last
// partial 16 bytes of a batch are read directly.  A wait that runs out sets
// the error word `err` (pyl_device_error) and the CTA leaves after a bounded wait for its
// other copy.


// Particles of batch j wholly inside its bulk copy.
__device__ __forceinline__ int staged_full(int cnt) { return (int)(((long long)cnt * 12 & ~15LL) / 12); }

__device__ __forceinline__ unsigned staged_bytes(long long cnt) { return (unsigned)((cnt * 12) & ~15LL); }

// One CTA per chunk: tile histogram of the chunk's particles (shared-memory counters).

__device__ __forceinline__ float rsd_shift(float p, float v, float factor, float box)
{
    float s = __fadd_rn(p, __fmul_rn(v, factor));
    if (s > box || s < 0.0f) s = fmodf(__fadd_rn(s, box), box);
    return s;
}

// One CTA per SM (grids binned by as many chunks as SMs).  No block barrier per
// batch: lane 0 of each warp waits on the buffer's mbarrier, the warp copies its
// four particles of the batch to registers (44 registers a thread) and counts
// itself out of the buffer, and the last of the 32 warps issues the copy HT_NBUF
// batches ahead into it (1024^3 particles on a 1024^3 grid: 3.13 -> 2.92 ms).  A
// failed wait marks the CTA: no further copies, and the copies in flight are
// drained (bounded) before it leaves without a row.
template <int MAS, bool RSD>
__global__ void __launch_bounds__(1024) chunk_hist_tma_kernel(const float *pos, long long n,
                                                              long long chunk, float inv, TileGeom g,
                                                              unsigned *__restrict__ hist, unsigned *err,
                                                              RsdArgs rsd = RsdArgs{}, unsigned long long *coh = nullptr)
{
    constexpr int HB = HT_BATCH;
    constexpr int PER = HB / 1024;          // particles per thread and batch
    __shared__ unsigned s_same;             // particles in the same bin as their predecessor
    extern __shared__ __align__(16) unsigned char hraw[];
    __shared__ __align__(8) unsigned long long bar[HT_NBUF];
    __shared__ unsigned s_rel[HT_NBUF];     // warps done reading each buffer, counted up forever
    __shared__ long long s_last[HT_NBUF];   // batch of the last copy into each buffer (-1: none)
    __shared__ int s_fail;
    const int T = (int)g.ntiles;
    const int lane = threadIdx.x & 31;
    float *inb = (float *)hraw;                                  // [HT_NBUF][HB * 3]
    unsigned *cnt = (unsigned *)(hraw + HT_NBUF * HB * 12);
    for (int t = threadIdx.x; t < T; t += blockDim.x) cnt[t] = 0;
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    const long long nbat = e > b ? (e - b + HB - 1) / HB : 0;
    unsigned my_same = 0u;                  // lane 0 of each warp: its warp's count
    if (threadIdx.x == 0) {
        s_same = 0u;
        s_fail = 0;
        for (int k = 0; k < HT_NBUF; k++) {
            mbar_init(&bar[k], 1);
            s_rel[k] = 0u;
            s_last[k] = -1;
        }
        mbar_fence_init();
        for (long long j = 0; j < HT_NBUF && j < nbat; j++) {
            const long long s0 = b + j * HB;
            stage_copy(inb + (j % HT_NBUF) * HB * 3, pos + 3 * s0,
                       staged_bytes(min((long long)HB, e - s0)), &bar[j % HT_NBUF]);
            s_last[j % HT_NBUF] = j;
        }
    }
    __syncthreads();
    for (long long j = 0; j < nbat; j++) {
        const long long s0 = b + j * HB;
        const int c = (int)min((long long)HB, e - s0);
        const int full = staged_full(c);
        const int buf = (int)(j % HT_NBUF);
        const float *in = inb + buf * HB * 3;
        int got = 0;
        if (lane == 0) got = mbar_wait_bounded(&bar[buf], (unsigned)((j / HT_NBUF) & 1), err);
        got = __shfl_sync(0xffffffffu, got, 0);             // lane 0's wait orders the copy for the warp
        __syncwarp();
        // every batch but a chunk's last is fully staged: no per-particle fallback test
        const bool all_staged = full == HB;
        float p[PER][3];
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int i = threadIdx.x + u * 1024;
            const long long q = s0 + i;
            if (all_staged || i < full) {
                p[u][0] = in[3 * i]; p[u][1] = in[3 * i + 1]; p[u][2] = in[3 * i + 2];
            } else if (i < c) {
                p[u][0] = pos[3 * q]; p[u][1] = pos[3 * q + 1]; p[u][2] = pos[3 * q + 2];
            }
        }
        __syncwarp();
        if (lane == 0) {
            if (!got) atomicOr(&s_fail, 1);
            __threadfence_block();                          // this warp's reads before its count
            const unsigned done = atomicAdd(&s_rel[buf], 1u);
            if ((done & 31u) == 31u && j + HT_NBUF < nbat && !*(volatile int *)&s_fail) {
                const long long s2 = b + (j + HT_NBUF) * HB;
                fence_proxy_async_smem();
                stage_copy(inb + buf * HB * 3, pos + 3 * s2, staged_bytes(min((long long)HB, e - s2)),
                           &bar[buf]);
                s_last[buf] = j + HT_NBUF;
            }
        }
        if (!got) continue;
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int i = threadIdx.x + u * 1024;
            if (!all_staged && i >= c) break;               // past the chunk's end
            const long long q = s0 + i;
            if (RSD) {                              // selects, not a dynamic index (no local array)
                const int ax = rsd.axis;
                const float pa = ax == 0 ? p[u][0] : (ax == 1 ? p[u][1] : p[u][2]);
                const float sh = rsd_shift(pa, __ldg(rsd.vel + 3 * q + ax), rsd.factor, rsd.box);
                p[u][0] = ax == 0 ? sh : p[u][0];
                p[u][1] = ax == 1 ? sh : p[u][1];
                p[u][2] = ax == 2 ? sh : p[u][2];
                rsd.pos[3 * q + ax] = sh;
            }
            const unsigned key = tile_key<MAS>(p[u], inv, g);
            atomicAdd(cnt + key, 1u);
            if (coh) {                              // the warp's lanes hold consecutive particles
                const unsigned prev = __shfl_up_sync(__activemask(), key, 1);
                const unsigned same = __ballot_sync(__activemask(), (threadIdx.x & 31) && prev == key);
                my_same += (unsigned)__popc(same);
            }
        }
    }
    if (coh && lane == 0 && my_same) atomicAdd(&s_same, my_same);
    __syncthreads();
    if (s_fail) {
        if (threadIdx.x == 0)
            for (int k = 0; k < HT_NBUF; k++)
                if (s_last[k] >= 0) mbar_drain_bounded(&bar[k], (unsigned)((s_last[k] / HT_NBUF) & 1));
        return;
    }
    unsigned *row = hist + (long long)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) row[t] = cnt[t];
    if (coh && threadIdx.x == 0 && s_same) atomicAdd(coh, (unsigned long long)s_same);
}

// chunk_scatter_kernel with its positions streamed through shared memory as in
// chunk_hist_tma_kernel (bulk copies of HT_BATCH particles, HT_NBUF in flight, no
// block barrier per batch: lane 0 of each warp waits, the warp copies its
// particles to registers and counts itself out, the last warp issues the next
// copy into the buffer).  NT threads: 1024 with one chunk per SM, 512 with two
// chunks per SM (two CTAs per SM, 64 registers a thread).  Lanes hold
// consecutive particles, so equal bins still take one reservation per warp.
template <int MAS, bool WEIGHTED, int NT>
__global__ void __launch_bounds__(NT) chunk_scatter_tma_kernel(
    const float *pos, const float *__restrict__ w, long long n, long long chunk, float inv, TileGeom g,
    const unsigned *__restrict__ colpre, const unsigned *__restrict__ offsets, float4 *__restrict__ rec,
    unsigned *err, Gate gate)
{
    if (gate_closed(gate)) return;
    constexpr int HB = HT_BATCH, PER = HB / NT, NW = NT / 32;
    static_assert(PER * NT == HB && (NW & (NW - 1)) == 0, "whole batches, a power-of-two warp count");
    extern __shared__ __align__(16) unsigned char sraw[];
    __shared__ __align__(8) unsigned long long bar[HT_NBUF];
    __shared__ unsigned s_rel[HT_NBUF];     // warps done reading each buffer, counted up forever
    __shared__ long long s_last[HT_NBUF];   // batch of the last copy into each buffer (-1: none)
    __shared__ int s_fail;
    const int T = (int)g.ntiles;
    const unsigned lane = threadIdx.x & 31u;
    float *inb = (float *)sraw;                                  // [HT_NBUF][HB * 3]
    unsigned *cur = (unsigned *)(sraw + HT_NBUF * HB * 12);
    const unsigned *row = colpre + (long long)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += NT) cur[t] = offsets[t] + row[t];
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    const long long nbat = e > b ? (e - b + HB - 1) / HB : 0;
    if (threadIdx.x == 0) {
        s_fail = 0;
        for (int k = 0; k < HT_NBUF; k++) {
            mbar_init(&bar[k], 1);
            s_rel[k] = 0u;
            s_last[k] = -1;
        }
        mbar_fence_init();
        for (long long j = 0; j < HT_NBUF && j < nbat; j++) {
            const long long s0 = b + j * HB;
            stage_copy(inb + (j % HT_NBUF) * HB * 3, pos + 3 * s0, staged_bytes(min((long long)HB, e - s0)),
                       &bar[j % HT_NBUF]);
            s_last[j % HT_NBUF] = j;
        }
    }
    __syncthreads();
    for (long long j = 0; j < nbat; j++) {
        const long long s0 = b + j * HB;
        const int c = (int)min((long long)HB, e - s0);
        const int full = staged_full(c);
        const int buf = (int)(j % HT_NBUF);
        const float *in = inb + buf * HB * 3;
        int got = 0;
        if (lane == 0) got = mbar_wait_bounded(&bar[buf], (unsigned)((j / HT_NBUF) & 1), err);
        got = __shfl_sync(0xffffffffu, got, 0);
        __syncwarp();
        const bool all_staged = full == HB;
        float p[PER][3];
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int i = threadIdx.x + u * NT;
            const long long q = s0 + i;
            if (all_staged || i < full) {
                p[u][0] = in[3 * i]; p[u][1] = in[3 * i + 1]; p[u][2] = in[3 * i + 2];
            } else if (i < c) {
                p[u][0] = pos[3 * q]; p[u][1] = pos[3 * q + 1]; p[u][2] = pos[3 * q + 2];
            }
        }
        __syncwarp();
        if (lane == 0) {
            if (!got) atomicOr(&s_fail, 1);
            __threadfence_block();                          // this warp's reads before its count
            const unsigned done = atomicAdd(&s_rel[buf], 1u);
            if ((done & (NW - 1u)) == NW - 1u && j + HT_NBUF < nbat && !*(volatile int *)&s_fail) {
                const long long s2 = b + (j + HT_NBUF) * HB;
                fence_proxy_async_smem();
                stage_copy(inb + buf * HB * 3, pos + 3 * s2, staged_bytes(min((long long)HB, e - s2)), &bar[buf]);
                s_last[buf] = j + HT_NBUF;
            }
        }
        if (!got) continue;
#pragma unroll
        for (int u = 0; u < PER; u++) {
            const int i = threadIdx.x + u * NT;
            const unsigned act = __ballot_sync(0xffffffffu, i < c);
            if (i < c) {
                const unsigned key = tile_key<MAS>(p[u], inv, g);
                const unsigned peers = __match_any_sync(act, key);
                const unsigned leader = (unsigned)__ffs(peers) - 1u;
                unsigned slot = 0u;
                if (lane == leader) slot = atomicAdd(cur + key, (unsigned)__popc(peers));
                slot = __shfl_sync(peers, slot, leader) + (unsigned)__popc(peers & ((1u << lane) - 1u));
                const float4 r = make_float4(p[u][0], p[u][1], p[u][2], WEIGHTED ? __ldg(w + s0 + i) : 1.0f);
                if (slot < (unsigned long long)n) rec[slot] = r;
            }
        }
    }
    __syncthreads();
    if (s_fail && threadIdx.x == 0)
        for (int k = 0; k < HT_NBUF; k++)
            if (s_last[k] >= 0) mbar_drain_bounded(&bar[k], (unsigned)((s_last[k] / HT_NBUF) & 1));
}

// Two CTAs per SM (grids binned by twice as many chunks as SMs): thread 0 waits
// and the CTA meets at two barriers per batch, with 30 registers a thread.  (The
// barrier-free loop above needs 44 registers; held to 32 it spills, and on
// 2048-particle batches it took 3.8 ms against 2.6 ms for 1024^3 particles on a
// 512^3 grid.)
template <int MAS, bool RSD>
__global__ void __launch_bounds__(1024) chunk_hist_tma_sync_kernel(const float *pos, long long n,
                                                              long long chunk, float inv, TileGeom g,
                                                              unsigned *__restrict__ hist, unsigned *err,
                                                              RsdArgs rsd = RsdArgs{}, unsigned long long *coh = nullptr)
{
    __shared__ unsigned s_same;             // particles in the same bin as their predecessor
    extern __shared__ __align__(16) unsigned char hraw[];
    __shared__ __align__(8) unsigned long long bar[HT_NBUF];
    __shared__ int s_ok;
    const int T = (int)g.ntiles;
    float *inb = (float *)hraw;                                  // [HT_NBUF][HT_BATCH * 3]
    unsigned *cnt = (unsigned *)(hraw + HT_NBUF * HT_BATCH * 12);
    for (int t = threadIdx.x; t < T; t += blockDim.x) cnt[t] = 0;
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    const long long nbat = e > b ? (e - b + HT_BATCH - 1) / HT_BATCH : 0;
    unsigned my_same = 0u;                  // lane 0 of each warp: its warp's count
    if (threadIdx.x == 0) {
        s_same = 0u;
        for (int k = 0; k < HT_NBUF; k++) mbar_init(&bar[k], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (long long j = 0; j < HT_NBUF && j < nbat; j++) {
            const long long s0 = b + j * HT_BATCH;
            stage_copy(inb + (j % HT_NBUF) * HT_BATCH * 3, pos + 3 * s0,
                       staged_bytes(min((long long)HT_BATCH, e - s0)), &bar[j % HT_NBUF]);
        }
    for (long long j = 0; j < nbat; j++) {
        const long long s0 = b + j * HT_BATCH;
        const int c = (int)min((long long)HT_BATCH, e - s0);
        const int full = staged_full(c);
        const int buf = (int)(j % HT_NBUF);
        const float *in = inb + buf * HT_BATCH * 3;
        if (threadIdx.x == 0)
            s_ok = mbar_wait_bounded(&bar[buf], (unsigned)((j / HT_NBUF) & 1), err);
        __syncthreads();
        if (!s_ok) {
            if (threadIdx.x == 0)
                for (long long k = j + 1; k < nbat && k < j + HT_NBUF; k++)
                    mbar_wait_bounded(&bar[k % HT_NBUF], (unsigned)((k / HT_NBUF) & 1), err);
            return;
        }
        // every batch but a chunk's last is fully staged: no per-particle fallback test
        const bool all_staged = full == HT_BATCH;
        for (int i = threadIdx.x; i < c; i += blockDim.x) {
            float p[3];
            const long long q = s0 + i;
            if (all_staged || i < full) { p[0] = in[3 * i]; p[1] = in[3 * i + 1]; p[2] = in[3 * i + 2]; }
            else { p[0] = pos[3 * q]; p[1] = pos[3 * q + 1]; p[2] = pos[3 * q + 2]; }
            if (RSD) {
                const float sh = rsd_shift(p[rsd.axis], __ldg(rsd.vel + 3 * q + rsd.axis), rsd.factor, rsd.box);
                p[rsd.axis] = sh;
                rsd.pos[3 * q + rsd.axis] = sh;
            }
            const unsigned key = tile_key<MAS>(p, inv, g);
            atomicAdd(cnt + key, 1u);
            if (coh) {                              // the warp's lanes hold consecutive particles
                const unsigned prev = __shfl_up_sync(__activemask(), key, 1);
                const unsigned same = __ballot_sync(__activemask(), (threadIdx.x & 31) && prev == key);
                my_same += (unsigned)__popc(same);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && j + HT_NBUF < nbat) {
            const long long s2 = b + (j + HT_NBUF) * HT_BATCH;
            stage_copy(inb + buf * HT_BATCH * 3, pos + 3 * s2, staged_bytes(min((long long)HT_BATCH, e - s2)),
                       &bar[buf]);
        }
    }
    if (coh && (threadIdx.x & 31) == 0 && my_same) atomicAdd(&s_same, my_same);
    __syncthreads();
    unsigned *row = hist + (long long)blockIdx.x * T;
    for (int t = threadIdx.x; t < T; t += blockDim.x) row[t] = cnt[t];
    if (coh && threadIdx.x == 0 && s_same) atomicAdd(coh, (unsigned long long)s_same);
}


constexpr int LAT_U = 4;                                    // particles per thread and batch
constexpr int LA_NBUF = 2;                                  // batches in flight

// NT threads per CTA: 1024 for the one-pass placement by bin (up to 1024 bins,
// scanned by one block scan), 512 for level A of two (two CTAs per SM, so one
// CTA's shared-memory sort overlaps the other's memory traffic).
template <int MAS, bool WEIGHTED, int NT>
__global__ void __launch_bounds__(NT) level_a_tma_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n, long long chunk, float inv,
    TileGeom g, const unsigned *__restrict__ colpre, const unsigned *__restrict__ offsets,
    float4 *__restrict__ tmp, int by_tile, unsigned *err, Gate gate = Gate{nullptr, 0ull, 0})
{
    constexpr int BATCH = NT * LAT_U;
    extern __shared__ __align__(16) unsigned char araw[];
    __shared__ __align__(8) unsigned long long bar[LA_NBUF];
    __shared__ int s_ok;
    if (gate_closed(gate)) return;
    // buckets: coarse blocks of 4^3 bins (level A of two), or the bins themselves
    // (one pass into the final layout, for grids of at most TWO_LEVEL_TILES bins)
    const int T = (int)g.ntiles;
    const int NCO = by_tile ? T : g.nc * g.nc * g.nc;
    float *inb = (float *)araw;                                            // [LA_NBUF][BATCH * 3]
    float4 *stage = (float4 *)(araw + LA_NBUF * BATCH * 12);
    unsigned short *sco = (unsigned short *)(stage + BATCH);
    unsigned *cur = (unsigned *)(sco + BATCH), *bcnt = cur + NCO, *gst = bcnt + NCO, *wt = gst + NCO;
    const unsigned *row = colpre + (long long)blockIdx.x * T;
    for (int co = threadIdx.x; co < NCO; co += blockDim.x) {
        if (by_tile) {
            cur[co] = offsets[co] + row[co];
        } else {
            unsigned sacc = 0;
            for (int l = 0; l < 64; l++) sacc += row[co * 64 + l];
            cur[co] = offsets[co * 64] + sacc;
        }
    }
    const long long b = blockIdx.x * chunk, e = min(n, b + chunk);
    const long long nbat = e > b ? (e - b + BATCH - 1) / BATCH : 0;
    if (threadIdx.x == 0) {
        for (int q = 0; q < LA_NBUF; q++) mbar_init(&bar[q], 1);
        mbar_fence_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (long long j = 0; j < LA_NBUF && j < nbat; j++) {
            const long long s0 = b + j * BATCH;
            stage_copy(inb + (j % LA_NBUF) * BATCH * 3, pos + 3 * s0,
                       staged_bytes(min((long long)BATCH, e - s0)), &bar[j % LA_NBUF]);
        }
    for (long long j = 0; j < nbat; j++) {
        const long long s0 = b + j * BATCH;
        const int c = (int)min((long long)BATCH, e - s0);
        const int full = staged_full(c);
        const int buf = (int)(j % LA_NBUF);
        const float *in = inb + buf * BATCH * 3;
        if (threadIdx.x == 0) s_ok = mbar_wait_bounded(&bar[buf], (unsigned)((j / LA_NBUF) & 1), err);
        for (int co = threadIdx.x; co < NCO; co += blockDim.x) bcnt[co] = 0u;
        __syncthreads();
        if (!s_ok) {
            if (threadIdx.x == 0)
                for (long long q = j + 1; q < nbat && q < j + LA_NBUF; q++)
                    mbar_wait_bounded(&bar[q % LA_NBUF], (unsigned)((q / LA_NBUF) & 1), err);
            return;
        }
        const bool all_staged = full == BATCH;              // every batch but a chunk's last
        float4 r[LAT_U];
        unsigned co_u[LAT_U], rank[LAT_U];
#pragma unroll
        for (int u = 0; u < LAT_U; u++) {
            const int i = threadIdx.x + u * NT;
            co_u[u] = 0xffffffffu;
            if (all_staged || i < c) {
                if (all_staged || i < full) r[u] = make_float4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 1.0f);
                else {
                    const long long q = s0 + i;
                    r[u] = make_float4(__ldg(pos + 3 * q), __ldg(pos + 3 * q + 1), __ldg(pos + 3 * q + 2), 1.0f);
                }
                if (WEIGHTED) r[u].w = __ldg(w + s0 + i);
                const float p[3] = {r[u].x, r[u].y, r[u].z};
                const unsigned key = tile_key<MAS>(p, inv, g);
                co_u[u] = by_tile ? key : key >> 6;
                rank[u] = atomicAdd(bcnt + co_u[u], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && j + LA_NBUF < nbat) {            // this buffer is consumed
            const long long s2 = b + (j + LA_NBUF) * BATCH;
            stage_copy(inb + buf * BATCH * 3, pos + 3 * s2, staged_bytes(min((long long)BATCH, e - s2)),
                       &bar[buf]);
        }
        for (int co = threadIdx.x; co < NCO; co += blockDim.x) {
            gst[co] = cur[co];
            cur[co] += bcnt[co];
        }
        __syncthreads();
        block_exclusive_scan(bcnt, NCO, wt);
#pragma unroll
        for (int u = 0; u < LAT_U; u++) {
            if (co_u[u] != 0xffffffffu) {
                const unsigned slot = bcnt[co_u[u]] + rank[u];
                stage[slot] = r[u];
                sco[slot] = (unsigned short)co_u[u];
            }
        }
        __syncthreads();
        for (int sidx = threadIdx.x; sidx < c; sidx += NT) {
            const unsigned co = sco[sidx];
            const unsigned dst = gst[co] + ((unsigned)sidx - bcnt[co]);      // n < 2^32
            if (dst < (unsigned)n) tmp[dst] = stage[sidx];
        }
        __syncthreads();
    }
}

inline size_t level_a_tma_smem(int nco, int nt)
{
    const size_t batch = (size_t)nt * LAT_U;
    return (size_t)LA_NBUF * batch * 12 + sizeof(float4) * batch + sizeof(unsigned short) * batch +
           sizeof(unsigned) * (3 * nco + 32);
}

constexpr int LBT_THREADS = 512, LBT_U = 4, LBT_BATCH = LBT_THREADS * LBT_U;   // 2048 records

// One CTA per (group of G consecutive chunks, coarse block): the group's records of
// a coarse block are contiguous in tmp, and each bin's records of the group are
// contiguous in the final layout, so a group sorts as one segment.
template <int MAS>
__global__ void __launch_bounds__(LBT_THREADS) level_b_tma_kernel(
    const float4 *__restrict__ tmp, int C, int G, float inv, TileGeom g, const unsigned *__restrict__ colpre,
    const unsigned *__restrict__ total, const unsigned *__restrict__ offsets, float4 *__restrict__ rec,
    unsigned n, unsigned *err, Gate gate = Gate{nullptr, 0ull, 0})
{
    __shared__ unsigned fcur[64], bcnt[64], gst[64], wt[32];
    __shared__ unsigned seg_start, seg_len;
    __shared__ __align__(8) unsigned long long bar[2];
    __shared__ int s_ok;
    if (gate_closed(gate) || *(volatile unsigned *)err) return;   // set: a wait upstream gave up
    extern __shared__ __align__(16) float4 braw[];
    float4 *inb = braw;                                     // [2][LBT_BATCH]
    float4 *stage = braw + 2 * LBT_BATCH;
    unsigned char *slo = (unsigned char *)(stage + LBT_BATCH);
    const int NCO = g.nc * g.nc * g.nc;
    const int T = (int)g.ntiles;
    const int c = (blockIdx.x / NCO) * G, co = blockIdx.x % NCO;
    const int c_end = min(c + G, C);
    if (threadIdx.x < 32) {
        unsigned pre = 0, len = 0;
        for (int l = threadIdx.x; l < 64; l += 32) {
            const int t = co * 64 + l;
            const unsigned cp = colpre[(long long)c * T + t];
            const unsigned nx = c_end < C ? colpre[(long long)c_end * T + t] : total[t];
            fcur[l] = offsets[t] + cp;
            pre += cp;
            len += nx - cp;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            pre += __shfl_down_sync(0xffffffffu, pre, o);
            len += __shfl_down_sync(0xffffffffu, len, o);
        }
        if (threadIdx.x == 0) {
            seg_start = offsets[co * 64] + pre;
            seg_len = len;
            mbar_init(&bar[0], 1);
            mbar_init(&bar[1], 1);
            mbar_fence_init();
        }
    }
    __syncthreads();
    const unsigned start = min(seg_start, n), len = min(seg_len, n - start);
    const unsigned nbat = (len + LBT_BATCH - 1) / LBT_BATCH;
    if (threadIdx.x == 0)
        for (unsigned j = 0; j < 2 && j < nbat; j++) {
            const unsigned s0 = j * LBT_BATCH;
            stage_copy(inb + (j & 1) * LBT_BATCH, tmp + start + s0, 16u * min((unsigned)LBT_BATCH, len - s0),
                       &bar[j & 1]);
        }
    for (unsigned j = 0; j < nbat; j++) {
        const unsigned s0 = j * LBT_BATCH;
        const int cnt = (int)min((unsigned)LBT_BATCH, len - s0);
        const float4 *in = inb + (j & 1) * LBT_BATCH;
        if (threadIdx.x == 0) s_ok = mbar_wait_bounded(&bar[j & 1], (j >> 1) & 1u, err);
        if (threadIdx.x < 64) bcnt[threadIdx.x] = 0u;
        __syncthreads();
        if (!s_ok) {
            if (threadIdx.x == 0 && j + 1 < nbat) mbar_wait_bounded(&bar[(j + 1) & 1], ((j + 1) >> 1) & 1u, err);
            return;
        }
        float4 r[LBT_U];
        int lo_u[LBT_U];
        unsigned rank[LBT_U];
#pragma unroll
        for (int u = 0; u < LBT_U; u++) {
            const int i = threadIdx.x + u * LBT_THREADS;
            lo_u[u] = -1;
            if (i < cnt) {
                r[u] = in[i];
                const float p[3] = {r[u].x, r[u].y, r[u].z};
                lo_u[u] = (int)(tile_key<MAS>(p, inv, g) & 63u);
                rank[u] = atomicAdd(bcnt + lo_u[u], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x == 0 && j + 2 < nbat) {
            const unsigned s2 = (j + 2) * LBT_BATCH;
            stage_copy(inb + (j & 1) * LBT_BATCH, tmp + start + s2, 16u * min((unsigned)LBT_BATCH, len - s2),
                       &bar[j & 1]);
        }
        if (threadIdx.x < 64) {
            gst[threadIdx.x] = fcur[threadIdx.x];
            fcur[threadIdx.x] += bcnt[threadIdx.x];
        }
        __syncthreads();
        block_exclusive_scan(bcnt, 64, wt);
#pragma unroll
        for (int u = 0; u < LBT_U; u++) {
            if (lo_u[u] >= 0) {
                const unsigned slot = bcnt[lo_u[u]] + rank[u];
                stage[slot] = r[u];
                slo[slot] = (unsigned char)lo_u[u];
            }
        }
        __syncthreads();
        for (int sidx = threadIdx.x; sidx < cnt; sidx += LBT_THREADS) {
            const int l = slo[sidx];
            const unsigned dst = gst[l] + ((unsigned)sidx - bcnt[l]);
            if (dst < n) rec[dst] = stage[sidx];
        }
        __syncthreads();
    }
}

inline size_t level_b_tma_smem() { return sizeof(float4) * 3 * LBT_BATCH + LBT_BATCH; }

// Fallback binning for grids with more tiles than one CTA's shared memory can count.
template <int MAS>
__global__ void __launch_bounds__(256) tile_count_kernel(const float *__restrict__ pos, long long n,
                                                         float inv, TileGeom g,
                                                         unsigned *__restrict__ counts)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float p[3] = {__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2)};
        atomicAdd(counts + tile_key<MAS>(p, inv, g), 1u);
    }
}

template <int MAS, bool WEIGHTED>
__global__ void __launch_bounds__(256) tile_scatter_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n, float inv, TileGeom g,
    unsigned *__restrict__ cursor, float4 *__restrict__ rec)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float p[3] = {__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2)};
        const unsigned slot = atomicAdd(cursor + tile_key<MAS>(p, inv, g), 1u);
        rec[slot] = make_float4(p[0], p[1], p[2], WEIGHTED ? __ldg(w + i) : 1.0f);
    }
}

// Exclusive scan of `n` counts into offsets[0..n] (and a copy into cursor when
// non-null), by one CTA of 1024 threads.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const unsigned *__restrict__ counts,
                                                         long long n, unsigned *__restrict__ offsets,
                                                         unsigned *__restrict__ cursor)
{
    __shared__ unsigned long long part[1024];
    const long long per = (n + blockDim.x - 1) / blockDim.x;
    const long long b = threadIdx.x * per, e = min(n, b + per);
    unsigned long long s = 0;
    for (long long i = b; i < e; i++) s += counts[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int off = 1; off < (int)blockDim.x; off <<= 1) {
        unsigned long long v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - s;
    for (long long i = b; i < e; i++) {
        offsets[i] = (unsigned)run;
        if (cursor) cursor[i] = (unsigned)run;
        run += counts[i];
    }
    if (threadIdx.x == blockDim.x - 1) offsets[n] = (unsigned)part[threadIdx.x];
}

// Weighted deposits accumulate weight / max|weight| in the fixed-point sums when the
// weights span at most a factor W_FX_RANGE (contributions are exact to 2^-23 of
// the largest weight, about the float rounding of the reference's sums); wider
// ranges, all-zero or non-finite weights take the float32 shared-memory sums.
// abs_range_kernel: max and min of the non-zero |w| (NaN skipped) as float bits,
// which order like unsigned integers for non-negative floats.
constexpr float W_FX_RANGE = 16.0f;

__global__ void __launch_bounds__(256) abs_range_kernel(const float *__restrict__ w, long long n,
                                                        unsigned *__restrict__ bits)
{
    float hi = 0.0f, lo = __int_as_float(0x7f800000);       // +inf
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float a = fabsf(__ldg(w + i));
        if (a > hi) hi = a;                                 // comparisons are false for NaN
        if (a > 0.0f && a < lo) lo = a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0) {
        if (hi > 0.0f) atomicMax(bits, __float_as_uint(hi));
        atomicMin(bits + 1, __float_as_uint(lo));
    }
}

// wsc: [0] max bits, [1] min bits (from abs_range_kernel), [2] 1 / max|w| (1 on
// the float path), [3] output scale (x max|w| on the fixed-point path; x 2^-22
// for NGP, whose fixed-point sums are read as counts), [4] 1: float path.
__global__ void w_scale_kernel(float *wsc, float host_scale, const float *dev_scale, int ngp)
{
    const unsigned *bits = (const unsigned *)wsc;
    const float wmax = __uint_as_float(bits[0]), wmin = __uint_as_float(bits[1]);
    const bool fx = wmax > 0.0f && isfinite(wmax) && wmax <= W_FX_RANGE * wmin;
    const float base = dev_scale ? *dev_scale : host_scale;
    wsc[2] = fx ? __frcp_rn(wmax) : 1.0f;
    const float s = fx ? __fmul_rn(base, wmax) : base;
    wsc[3] = ngp ? __fmul_rn(s, FX_INV) : s;
    reinterpret_cast<int *>(wsc)[4] = fx ? 0 : 1;
}






// ---- full-bin fixed-point deposit (unweighted) ------------------------------
// One 32-bit word per shared-memory cell, so a whole TB^3 bin plus its + side
// halo fits one CTA for every MAS with and without interlacing.  CIC/TSC/PCS
// accumulate 10.22 fixed point (2^-22 units, cell sums below 1024); each
// contribution v in [0, 1] is converted by one FFMA against 1.5 * 2^23 (exact
// round-to-nearest of v * 2^22, error <= 2^-23) and one integer add.  NGP
// accumulates integer counts.  Integer sums do not depend on the order of the
// adds, so the bin values are reproducible.  A negative or NaN weight (CIC
// positions below 0, non-finite positions) or a cell sum that wraps sets a
// flag, and the pass is redone with float32 shared atomics.  The grids (plain,
// then interlaced) are deposited one after the other; the second pass reads the
// bin's particles again (partly from L2).
// The deposit:
//   * each pass streams the bin's records through two shared-memory buffers of
//     R records filled by bulk copies (batch q+2 loads while batch q deposits);
//   * the overflow test ORs the old values returned by the atomics and checks
//     bit 31 (512.0) once per pass: a cell can only wrap past 1024 through an
//     add whose old value is >= 1023, so a clear bit 31 proves no cell wrapped
//     (a set one, from cells >= 512, conservatively redoes the pass in float32);
//   * the grid (plain or shifted) and the arithmetic (fixed point or float) of a
//     pass are compile-time, and bin-local cells come from tile_key's first cell
//     without the general wrap (taken only by cells past the grid edge);
//   * the write-out walks the cells with incremental (x, y, z) indices, and
//     interior bins (halo inside the grid) use 32-bit cell offsets.
// Only CIC can produce negative or NaN weights (positions below 0, non-finite
// positions); TSC and PCS weights are in [0, 1] for any input.

// Bin-local cell of a particle along one axis (0 <= loc < TB for the first cell
// of the plain grid, loc <= TB for the shifted one) and the axis weights.  The
// particle's bin came from the wrapped first cell, so loc = (f - o) mod dims: for
// power-of-two grids (P2) a mask, otherwise the in-range test with the general
// wrap for cells past the grid edge.
template <int MAS, int G, bool P2>
__device__ __forceinline__ int axis_local(float p, float inv, float halfcell, int dims, int o, float *C)
{
    if (G == 0) {
        const int f = axis_weights<MAS>(p, inv, C);
        const int loc = f - o;
        if (P2) return loc & (dims - 1);
        return (unsigned)loc < (unsigned)TB ? loc : wrap_index(f, dims) - o;
    }
    const int f0 = axis_first<MAS>(p, inv);
    const int f = axis_weights<MAS>(__fadd_rn(p, halfcell), inv, C);
    const int loc0 = f0 - o;
    const int w0 = P2 ? (loc0 & (dims - 1)) : ((unsigned)loc0 < (unsigned)TB ? loc0 : wrap_index(f0, dims) - o);
    return w0 + (f > f0 ? 1 : 0);
}

// Staging state of a deposit CTA (at namespace scope: addressed as constants,
// no registers).
__shared__ __align__(8) unsigned long long fx_bar[2];   // one mbarrier per buffer
__shared__ unsigned fx_rel[2];     // per buffer: warps done reading it, counted up forever
__shared__ unsigned fx_last[2];    // per buffer: batch number of the last copy into it (~0u: none)
__shared__ int fx_fail;            // a wait of this CTA gave up

struct FxStage {
    const float4 *rec;
    unsigned begin, cnt, nb;           // the bin's records and their batches
    float4 *inb;                       // [2][R] staging buffers
    const float *inv_w;                // weighted: 1 / max |w| (weights scaled into [-1, 1]); null: unweighted
    const int *use_float;              // weighted: 1 -> float32 sums from the start
    unsigned *err;                     // device error word of the bounded waits
};

// One pass over the bin's records into shared memory.  Returns 1 when the pass
// must be redone in float32, 0 when done, -1 after a failed staging wait.
// q0: batches staged on the two barriers before this pass.
//
// FREE (owned-cell launches, four bins per CTA): no block-wide barrier per
// batch.  Lane 0 of every warp waits on the buffer's mbarrier, the warp reads its
// records into registers and counts itself out of the buffer; the last of the 32
// warps issues the copy of the batch two ahead into it.  Warps drift up to a
// batch apart instead of meeting twice per 2048 records (1024^3 interlaced
// deposit 13.4 -> 12.5 ms).  One bin per CTA (the red.global write-out) measured
// faster with thread 0 waiting and two barriers per batch (512^3 particles on a
// 512^3 grid, interlaced: 1.83 against 2.03 ms), so those launches keep them;
// both loops in one kernel (a runtime switch) made both slower.
// A failed wait marks the CTA; no new copies are issued, and after the pass
// thread 0 drains the copies in flight (bounded) before the CTA leaves.
template <int MAS, bool INTER, int R, int G, bool FLOAT, bool P2, bool TOT, bool FREE>
__device__ __forceinline__ int fx_accumulate(const FxStage &sg, unsigned q0, float inv, float halfcell, int dims,
                                             const int *o, unsigned *smw)
{
    using FS = FxShape<MAS, INTER>;
    constexpr int S = Support<MAS>::S, E = FS::E;
    constexpr int PER = R / 1024;                       // records per thread and batch
    // record of this thread in each 1024-record block: lanes take records 32 apart
    // (rotated by the warp so the 16-byte reads spread over the banks), so input in
    // spatial order does not put a warp's atomics on the same cells
    const unsigned slot = (threadIdx.x & 31u) * 32u + (((threadIdx.x >> 5) + threadIdx.x) & 31u);
    uint4 *z4 = (uint4 *)smw;
    for (int c = threadIdx.x; c < FS::SMEM / 16; c += 1024) z4[c] = make_uint4(0u, 0u, 0u, 0u);
    if (threadIdx.x == 0) {
        fence_proxy_async_smem();                       // earlier generic use of the buffers (carried blocks)
        for (unsigned j = 0; j < 2 && j < sg.nb; j++) {
            const unsigned q = q0 + j;
            stage_copy(sg.inb + (q & 1) * R, sg.rec + sg.begin + j * R, 16u * min((unsigned)R, sg.cnt - j * R),
                       &fx_bar[q & 1]);
            fx_last[q & 1] = q;
        }
    }
    __syncthreads();
    const bool weighted = sg.inv_w != nullptr;
    const float inv_w = weighted ? *sg.inv_w : 1.0f;
    // Unweighted CIC/TSC/PCS find wrapped cells from the bin's total instead of
    // the atomics' old values: a particle's S^3 rounded corners add up to 2^22
    // within S^3 + 8 units, so the cells of a bin sum to cnt * 2^22 within
    // cnt (S^3 + 8), and every wrap of a cell takes 2^32 off that sum.  That tells
    // wraps apart while 2 cnt (S^3 + 8) < 2^32.  Summing the bin's cells costs
    // about what the old-value ORs save at one particle per cell, and the second
    // path inside one kernel slowed the 1024^3 grid of 1024^3 particles, so TOT
    // (a separate kernel) is launched from two particles per bin cell on average
    // (512^3 grids of 1024^3 particles: deposit 11.4 -> 10.8 ms).
    constexpr unsigned long long PER_P = (unsigned long long)S * S * S + 8;
    const bool by_total = TOT && !FLOAT && MAS != PYL_MAS_NGP && !weighted &&
                          (unsigned long long)sg.cnt * PER_P < (1ull << 31);
    unsigned bad = 0u, seen = 0u;
    for (unsigned j = 0; j < sg.nb; j++) {
        const unsigned q = q0 + j;
        const float4 *in = sg.inb + (q & 1) * R;
        const unsigned c = min((unsigned)R, sg.cnt - j * R);
        float4 r[PER];                                      // (unused after a failed wait)
        int got = 1;
        if constexpr (FREE) {
            if ((threadIdx.x & 31) == 0) got = mbar_wait_bounded(&fx_bar[q & 1], (q >> 1) & 1u, sg.err);
            got = __shfl_sync(0xffffffffu, got, 0);         // lane 0's wait orders the copy for the warp
            __syncwarp();
#pragma unroll
            for (int u = 0; u < PER; u++) r[u] = in[slot + u * 1024];
            __syncwarp();
            if ((threadIdx.x & 31) == 0) {
                if (!got) atomicOr(&fx_fail, 1);
                __threadfence_block();                      // this warp's reads before its count
                const unsigned done = atomicAdd(&fx_rel[q & 1], 1u);
                if ((done & 31u) == 31u && j + 2 < sg.nb && !*(volatile int *)&fx_fail) {
                    fence_proxy_async_smem();
                    stage_copy(sg.inb + (q & 1) * R, sg.rec + sg.begin + (j + 2) * R,
                               16u * min((unsigned)R, sg.cnt - (j + 2) * R), &fx_bar[q & 1]);
                    fx_last[q & 1] = q + 2;
                }
            }
        } else {                                            // thread 0 waits, the CTA meets twice
            if (threadIdx.x == 0 && !mbar_wait_bounded(&fx_bar[q & 1], (q >> 1) & 1u, sg.err))
                fx_fail = 1;
            __syncthreads();
            if (*(volatile int *)&fx_fail) break;
#pragma unroll
            for (int u = 0; u < PER; u++) r[u] = in[slot + u * 1024];
            __syncthreads();                                // buffer consumed
            if (threadIdx.x == 0 && j + 2 < sg.nb) {
                stage_copy(sg.inb + (q & 1) * R, sg.rec + sg.begin + (j + 2) * R,
                           16u * min((unsigned)R, sg.cnt - (j + 2) * R), &fx_bar[q & 1]);
                fx_last[q & 1] = q + 2;
            }
        }
        if (!got) continue;
#pragma unroll
        for (int u = 0; u < PER; u++) {
            if (slot + u * 1024 >= c) continue;
            float C[3][S];
            const int base = (axis_local<MAS, G, P2>(r[u].x, inv, halfcell, dims, o[0], C[0]) * E +
                              axis_local<MAS, G, P2>(r[u].y, inv, halfcell, dims, o[1], C[1])) * E +
                             axis_local<MAS, G, P2>(r[u].z, inv, halfcell, dims, o[2], C[2]);
            float wq = 1.0f;
            if (weighted) {                                 // the scaled weight joins the x weights
                wq = __fmul_rn(r[u].w, inv_w);
#pragma unroll
                for (int l = 0; l < S; l++) C[0][l] = __fmul_rn(C[0][l], wq);
            }
            if (FLOAT) {
                float_scatter<MAS, E>((float *)smw, base, C);
            } else {
                if (MAS == PYL_MAS_CIC) bad |= (unsigned)!(C[0][1] >= 0.0f && C[1][1] >= 0.0f && C[2][1] >= 0.0f);
                // z weights times 2^22 (exact): each corner is then one FFMA into the
                // fixed-point format, rounded once from the exact product
#pragma unroll
                for (int q = 0; q < S; q++) C[2][q] = __fmul_rn(C[2][q], FX_SCALE);
                if (weighted) {
                    bad |= (unsigned)!(wq >= 0.0f);            // negative or NaN weight
                    seen |= fx_scatter_or<MAS, E, false, true>(smw, base, C);
                } else if (by_total) {
                    fx_scatter_add<MAS, E, true>(smw, base, C);
                } else {
                    seen |= fx_scatter_or<MAS, E, (MAS == PYL_MAS_NGP), true>(smw, base, C);
                }
            }
        }
    }
    if (TOT && by_total) {
        __shared__ unsigned long long s_tot[32];
        __syncthreads();                                    // every atomic of the pass done
        unsigned long long t = 0;
        for (int c = threadIdx.x; c < FS::CELLS; c += 1024) t += smw[c];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if ((threadIdx.x & 31) == 0) s_tot[threadIdx.x >> 5] = t;
        __syncthreads();
        if (threadIdx.x == 0) {
            unsigned long long tot = 0;
            for (int w = 0; w < 32; w++) tot += s_tot[w];
            const long long diff = (long long)tot - (long long)((unsigned long long)sg.cnt << 22);
            const long long bound = (long long)((unsigned long long)sg.cnt * PER_P);
            if (diff > bound || diff < -bound) bad = 1u;
        }
    }
    const int redo = __syncthreads_or((int)(bad | (seen >> 31)));
    if (*(volatile int *)&fx_fail) {
        if (threadIdx.x == 0)
            for (int b = 0; b < 2; b++)
                if (fx_last[b] != ~0u) mbar_drain_bounded(&fx_bar[b], (fx_last[b] >> 1) & 1u);
        __syncthreads();
        return -1;
    }
    return (!FLOAT && redo) ? 1 : 0;
}

template <int MAS, bool FLOAT>
__device__ __forceinline__ float fx_value(unsigned w)
{
    if (FLOAT) return __uint_as_float(w);
    if (MAS == PYL_MAS_NGP) return __uint2float_rn(w);
    return __fmul_rn(__uint2float_rn(w), FX_INV);
}

// Adds the bin's cells (with halo) into the grid; threads walk the flattened
// cells 1024 apart with incremental (x, y, z) bin-local indices.
template <int MAS, bool INTER, bool FLOAT>
__device__ __forceinline__ void fx_write_out(const unsigned *smw, float *out, const int *o, int dims,
                                             bool interior, float scale)
{
    using FS = FxShape<MAS, INTER>;
    constexpr int E = FS::E, CELLS = FS::CELLS;
    constexpr int DZ = 1024 % E, DY = (1024 / E) % E, DX = 1024 / (E * E);
    int lz = threadIdx.x % E, ly = (threadIdx.x / E) % E, lx = threadIdx.x / (E * E);
    if (interior) {
        const unsigned gbase = ((unsigned)o[0] * dims + o[1]) * dims + o[2];
        for (int c = threadIdx.x; c < CELLS; c += 1024) {
            const unsigned w = smw[c];
            if (w != 0u)
                atomicAdd(out + (gbase + ((unsigned)lx * dims + ly) * dims + lz), __fmul_rn(fx_value<MAS, FLOAT>(w), scale));
            lz += DZ;
            ly += DY;
            lx += DX;
            if (lz >= E) { lz -= E; ly++; }
            if (ly >= E) { ly -= E; lx++; }
        }
    } else {
        const long long d = dims;
        for (int c = threadIdx.x; c < CELLS; c += 1024) {
            const unsigned w = smw[c];
            if (w != 0u) {
                const long long gx = add_wrap(o[0], lx, d), gy = add_wrap(o[1], ly, d), gz = add_wrap(o[2], lz, d);
                atomicAdd(out + (gx * d + gy) * d + gz, __fmul_rn(fx_value<MAS, FLOAT>(w), scale));
            }
            lz += DZ;
            ly += DY;
            lx += DX;
            if (lz >= E) { lz -= E; ly++; }
            if (ly >= E) { ly -= E; lx++; }
        }
    }
}

// ---- owned-cell write-out --------------------------------------------------------
// With dims a multiple of TB the bins tile the grid exactly, and every cell is the
// core cell of one bin.  A bin stores its TB^3 core cells with plain coalesced
// stores (fill + value for a fresh grid, old + value to accumulate) and its halo
// cells (the + side layers that belong to the next bins) into a per-bin buffer;
// halo_add_kernel then adds each bin's incoming halos into its core cells, in a
// fixed order.  No global atomics, no separate fill pass, and every cell's sum is
// formed in the same order on every run.
// The halo of a bin is seven blocks, h = 1..7 with bits (x, y, z) = (4, 2, 1):
// block h spans H layers along each axis whose bit is set and TB cells along the
// others; bin-local cell (x + TB*hx, y + TB*hy, z + TB*hz) of block h is core cell
// (x, y, z) of the bin offset by (hx, hy, hz).
constexpr int OWN_Z = 4;   // bins along z per CTA of the owned-cell deposit (one coarse block)



// The + z layers of a bin (its halo blocks 1, 3, 5, 7) land on the z < H layers of
// the next bin along z (core cells, and blocks 2, 4, 6).  carry: those four blocks
// of the bin run just before by this CTA, copied into shared memory in this order
// (offsets carry_off), or null.
__host__ __device__ constexpr int carry_off(int H, int h)
{
    return h == 1 ? 0 : h == 3 ? TB * TB * H : h == 5 ? TB * TB * H + TB * H * H : TB * TB * H + 2 * TB * H * H;
}
__host__ __device__ constexpr int carry_floats(int H) { return carry_off(H, 7) + H * H * H; }

template <int MAS, bool INTER, bool FLOAT, int h>
__device__ __forceinline__ void fx_store_halo_block(const unsigned *smw, float *halo_bin, float scale,
                                                    const float *carry)
{
    constexpr int E = FxShape<MAS, INTER>::E, H = E - TB;
    constexpr int EX = halo_ext(H, h & 4), EY = halo_ext(H, h & 2), EZ = halo_ext(H, h & 1);
    constexpr int OX = (h & 4) ? TB : 0, OY = (h & 2) ? TB : 0, OZ = (h & 1) ? TB : 0;
    constexpr int N = EX * EY * EZ, OFF = halo_block_off(H, h);
    for (int i = threadIdx.x; i < N; i += 1024) {
        const int z = i % EZ, y = (i / EZ) % EY, x = i / (EZ * EY);
        const unsigned w = smw[((x + OX) * E + (y + OY)) * E + (z + OZ)];
        float v = __fmul_rn(fx_value<MAS, FLOAT>(w), scale);
        if constexpr (!(h & 1)) {
            if (carry && z < H) v = __fadd_rn(v, carry[carry_off(H, h | 1) + (x * EY + y) * H + z]);
        }
        halo_bin[OFF + i] = v;
    }
}

// cs: the idle staging buffers (no bulk copy in flight during a write-out), where
// the carried blocks of prev are gathered before use.
template <int MAS, bool INTER, bool FLOAT>
__device__ __forceinline__ void fx_store_owned(const unsigned *smw, float *out, float *halo_bin, const int *o,
                                               int dims, float scale, const Owned &ow, const float *prev,
                                               float *cs)
{
    constexpr int E = FxShape<MAS, INTER>::E, H = E - TB;
    const float *carry = nullptr;
    if constexpr (H > 0) {
        if (prev) {
            for (int i = threadIdx.x; i < carry_floats(H); i += 1024) {
                const int h = i < carry_off(H, 3) ? 1 : i < carry_off(H, 5) ? 3 : i < carry_off(H, 7) ? 5 : 7;
                cs[i] = prev[halo_block_off(H, h) + (i - carry_off(H, h))];
            }
            __syncthreads();
            carry = cs;
        }
    }
    // core: thread t holds (y, z) = (t / 32, t % 32) and walks x; z < H adds the
    // carried block 1
    const int ly = threadIdx.x >> 5, lz = threadIdx.x & 31;
    const size_t plane = (size_t)dims * dims;
    float *dst = out + ((size_t)o[0] * dims + (size_t)(o[1] + ly)) * dims + (o[2] + lz);
    const unsigned *src = smw + ly * E + lz;
    const float *cz = (carry && lz < H) ? carry + ly * H + lz : nullptr;
    if (ow.fill_mode) {
#pragma unroll 4
        for (int lx = 0; lx < TB; lx++) {
            float v = __fmul_rn(fx_value<MAS, FLOAT>(src[lx * E * E]), scale);
            if (cz) v = __fadd_rn(v, cz[lx * TB * H]);
            dst[lx * plane] = __fadd_rn(ow.fill, v);
        }
    } else {
#pragma unroll 4
        for (int lx = 0; lx < TB; lx++) {
            float v = __fmul_rn(fx_value<MAS, FLOAT>(src[lx * E * E]), scale);
            if (cz) v = __fadd_rn(v, cz[lx * TB * H]);
            dst[lx * plane] = __fadd_rn(dst[lx * plane], v);
        }
    }
    if constexpr (H > 0) {
        fx_store_halo_block<MAS, INTER, FLOAT, 1>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 2>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 3>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 4>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 5>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 6>(smw, halo_bin, scale, carry);
        fx_store_halo_block<MAS, INTER, FLOAT, 7>(smw, halo_bin, scale, carry);
    }
}

// Adds the halo blocks of the - side neighbours into each bin's core cells.  The
// deposit already carried the + z layers of a bin into the next bin of its CTA,
// so only the first bin of each OWN_Z group along z takes the blocks with the z
// bit set (1, 3, 5, 7); every bin takes blocks 2, 4, 6.  One CTA per bin and
// grid; every receiving cell is read, summed with its incoming halo values in
// block order, and written by one thread, so no atomics and a fixed order.  Rows
// with x < H or y < H receive along their whole length (a warp per row); the
// first H cells of the other rows receive only from the z block.
template <int H>
__global__ void __launch_bounds__(256) halo_add_kernel(float *__restrict__ grid, float *__restrict__ grid2,
                                                       const float *__restrict__ halo, long long stride, TileGeom g)
{
    constexpr int HC = halo_cells(H);
    constexpr int ROWS_A = 2 * H * TB - H * H;          // rows (x, y) with x < H or y < H
    constexpr int CELLS_B = (TB - H) * (TB - H) * H;    // first H cells of the other rows
    __shared__ const float *src[8];
    const int nt = g.nt;
    const int gi = blockIdx.y;                          // 0: plain grid, 1: shifted grid
    int tx, ty, tz;
    tile_coords(blockIdx.x, g, tx, ty, tz);
    if (tx >= nt || ty >= nt || tz >= nt) return;
    float *out = gi ? grid2 : grid;
    if (threadIdx.x < 8) {
        const int h = threadIdx.x, hx = (h >> 2) & 1, hy = (h >> 1) & 1, hz = h & 1;
        const unsigned key = tile_key_of((unsigned)((tx - hx + nt) % nt), (unsigned)((ty - hy + nt) % nt),
                                         (unsigned)((tz - hz + nt) % nt), g);
        src[h] = halo + gi * stride + (size_t)key * HC + halo_block_off(H, h);
    }
    __syncthreads();
    const size_t dims = (size_t)g.dims;
    float *bin = out + ((size_t)tx * TB * dims + (size_t)ty * TB) * dims + (size_t)tz * TB;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int zmask = tz % OWN_Z == 0 ? 7 : 6;          // blocks taken: all, or those without the z bit
    for (int r = warp; r < ROWS_A; r += 8) {
        int x, y;
        if (r < H * TB) { x = r / TB; y = r % TB; }
        else { x = H + (r - H * TB) / H; y = (r - H * TB) % H; }
        const int z = lane;
        const int low = ((x < H ? 4 : 0) | (y < H ? 2 : 0) | (z < H ? 1 : 0)) & zmask;
        float *c = bin + ((size_t)x * dims + y) * dims + z;
        float v = *c;
#pragma unroll
        for (int h = 1; h < 8; h++) {
            if (h & ~low) continue;
            const int EY = (h & 2) ? H : TB, EZ = (h & 1) ? H : TB;
            v = __fadd_rn(v, src[h][(x * EY + y) * EZ + z]);
        }
        *c = v;
    }
    for (int i = threadIdx.x; i < (zmask == 7 ? CELLS_B : 0); i += 256) {
        const int z = i % H, row = i / H;
        const int x = H + row / (TB - H), y = H + row % (TB - H);
        float *c = bin + ((size_t)x * dims + y) * dims + z;
        *c = __fadd_rn(*c, src[1][(x * TB + y) * H + z]);
    }
}

// Both arithmetic modes of one grid: fixed point, float32 if that overflowed.
// Returns false after a failed staging wait.
template <int MAS, bool INTER, int R, int G, bool P2, bool TOT, bool FREE>
__device__ __forceinline__ bool fx_grid(const FxStage &sg, unsigned &q0, float inv, float halfcell, int dims,
                                        const int *o, unsigned *smw, float *out, bool interior, float scale,
                                        const Owned &ow, float *halo_bin, const float *prev)
{
    int st = 1;                                             // float32 from the start
    if (!(sg.use_float && *sg.use_float)) {
        st = fx_accumulate<MAS, INTER, R, G, false, P2, TOT, FREE>(sg, q0, inv, halfcell, dims, o, smw);
        if (st < 0) return false;
        q0 += sg.nb;
    }
    if (st == 0) {
        if (ow.on) fx_store_owned<MAS, INTER, false>(smw, out, halo_bin, o, dims, scale, ow, prev, (float *)sg.inb);
        else fx_write_out<MAS, INTER, false>(smw, out, o, dims, interior, scale);
    } else {
        if (fx_accumulate<MAS, INTER, R, G, true, P2, false, FREE>(sg, q0, inv, halfcell, dims, o, smw) < 0) return false;
        q0 += sg.nb;
        // weighted NGP: `scale` carries the 2^-22 of the fixed-point sums, which
        // float sums do not need
        const float fs = (MAS == PYL_MAS_NGP && sg.inv_w) ? __fmul_rn(scale, FX_SCALE) : scale;
        if (ow.on) fx_store_owned<MAS, INTER, true>(smw, out, halo_bin, o, dims, fs, ow, prev, (float *)sg.inb);
        else fx_write_out<MAS, INTER, true>(smw, out, o, dims, interior, fs);
    }
    __syncthreads();                                        // cells read before the next pass zeroes them
    return true;
}

template <int MAS, bool INTER, int R, bool P2, bool TOT, bool FREE>
__global__ void __launch_bounds__(1024) bin_deposit_fx_tma_kernel(
    const float4 *__restrict__ rec, const unsigned *__restrict__ offsets, TileGeom g, float inv,
    float halfcell, float *__restrict__ grid, float *__restrict__ grid2, OutScale sc, unsigned n_rec,
    Owned ow, const float *inv_w, unsigned *err)
{
    // a bounded wait of the placement gave up (its records may be incomplete, and
    // stale records may lie outside the bin): deposit nothing, the error stands
    if (*(volatile unsigned *)err) return;
    using FS = FxShape<MAS, INTER>;
    constexpr int E = FS::E;
    extern __shared__ __align__(16) unsigned smw[];
    const float scale = out_scale(sc);
    const int dims = g.dims;
    constexpr int HC = halo_cells(FS::H);
    if (threadIdx.x == 0) {
        mbar_init(&fx_bar[0], 1);
        mbar_init(&fx_bar[1], 1);
        mbar_fence_init();
        fx_rel[0] = fx_rel[1] = 0u;
        fx_last[0] = fx_last[1] = ~0u;
        fx_fail = 0;
    }
    __syncthreads();
    unsigned q0 = 0;                                    // batches staged by this CTA so far
    // owned-cell write-out: the OWN_Z bins of a coarse block along z (consecutive
    // keys) one after the other, each taking the + z layers of the one before
    const int nbins = ow.on ? OWN_Z : 1;
    bool have_prev = false;
    for (int k = 0; k < nbins; k++) {
        const long long tile = (long long)blockIdx.x * nbins + k;
        const unsigned end = min(offsets[tile + 1], n_rec), begin = min(offsets[tile], end);
        int tx, ty, tz;
        tile_coords(tile, g, tx, ty, tz);
        if (tx >= g.nt || ty >= g.nt || tz >= g.nt) break;     // keys past the grid: no cells
        if (begin == end && !ow.on) return;                     // owned cells are stored even when empty
        const int o[3] = {tx * TB, ty * TB, tz * TB};
        const bool interior = o[0] + E <= dims && o[1] + E <= dims && o[2] + E <= dims &&
                              (long long)dims * dims * dims < (1LL << 32);
        FxStage sg;
        sg.rec = rec;
        sg.begin = begin;
        sg.cnt = end - begin;
        sg.nb = (sg.cnt + R - 1) / R;
        sg.inb = (float4 *)(smw + FS::SMEM / 4);
        sg.inv_w = inv_w;
        sg.use_float = inv_w ? reinterpret_cast<const int *>(inv_w + 2) : nullptr;
        sg.err = err;
        float *hb = ow.on && HC > 0 ? ow.halo + tile * HC : nullptr;
        const float *prev = have_prev && hb ? hb - HC : nullptr;
        if (!fx_grid<MAS, INTER, R, 0, P2, TOT, FREE>(sg, q0, inv, halfcell, dims, o, smw, grid, interior, scale, ow, hb, prev))
            return;
        if (INTER &&
            !fx_grid<MAS, INTER, R, 1, P2, TOT, FREE>(sg, q0, inv, halfcell, dims, o, smw, grid2, interior, scale, ow,
                                       hb ? hb + ow.stride : nullptr, prev ? prev + ow.stride : nullptr))
            return;
        have_prev = true;
    }
}

// Records per staging buffer that fit beside the bin (0: no staging).
template <int MAS, bool I>
constexpr int fx_tma_batch()
{
    return FxShape<MAS, I>::SMEM + 2 * 2048 * 16 <= 227 * 1024 ? 2048
         : FxShape<MAS, I>::SMEM + 2 * 1024 * 16 <= 227 * 1024 ? 1024 : 0;
}

template <int MAS, bool I>
int launch_deposit_fx(const TiledWs &ws, TileGeom g, float inv, float halfcell, float *grid,
                      float *grid2, OutScale sc, cudaStream_t st, const Owned &ow, const float *inv_w, unsigned *err)
{
    using FS = FxShape<MAS, I>;
    constexpr int R = fx_tma_batch<MAS, I>();
    static_assert(R == 0 || carry_floats(FS::H) * 4 <= 2 * R * 16, "carried blocks fit the staging buffers");
    if (R > 0) {
        constexpr int RR = R > 0 ? R : 1024;
        const bool p2 = (g.dims & (g.dims - 1)) == 0;
        // bin-total wrap detection: unweighted non-NGP deposits of two or more
        // particles per bin cell on average
        const bool tot = MAS != PYL_MAS_NGP && !inv_w &&
                         (double)ws.n >= g_tot_min_per_cell.load() * (double)g.nt * g.nt * g.nt * (double)FS::CELLS;
        // owned-cell launches: no block barriers per batch
        auto kern = ow.on ? (p2 ? (tot ? bin_deposit_fx_tma_kernel<MAS, I, RR, true, true, true>
                                       : bin_deposit_fx_tma_kernel<MAS, I, RR, true, false, true>)
                                : (tot ? bin_deposit_fx_tma_kernel<MAS, I, RR, false, true, true>
                                       : bin_deposit_fx_tma_kernel<MAS, I, RR, false, false, true>))
                          : (p2 ? (tot ? bin_deposit_fx_tma_kernel<MAS, I, RR, true, true, false>
                                       : bin_deposit_fx_tma_kernel<MAS, I, RR, true, false, false>)
                                : (tot ? bin_deposit_fx_tma_kernel<MAS, I, RR, false, true, false>
                                       : bin_deposit_fx_tma_kernel<MAS, I, RR, false, false, false>));
        const size_t smem = FS::SMEM + 2 * (size_t)R * 16;
        PYL_CUDA(ensure_smem(kern, smem));
        const unsigned ctas = (unsigned)(ow.on ? g.ntiles / OWN_Z : g.ntiles);
        kern<<<ctas, 1024, smem, st>>>(ws.rec, ws.offsets, g, inv, halfcell, grid, grid2, sc, ws.n, ow, inv_w, err);
        PYL_LAUNCH_CHECK();
        if constexpr (FS::H > 0) {
            if (ow.on) {
                stage_mark(PYL_STAGE_DEPOSIT, false, st);
                stage_mark(PYL_STAGE_HALO, true, st);
                halo_add_kernel<FS::H><<<dim3((unsigned)g.ntiles, I ? 2 : 1), 256, 0, st>>>(grid, grid2, ow.halo,
                                                                                          ow.stride, g);
                PYL_LAUNCH_CHECK();
                stage_mark(PYL_STAGE_HALO, false, st);
                stage_mark(PYL_STAGE_DEPOSIT, true, st);
            }
        }
        return PYL_OK;
    }
    set_error("no staging buffers fit beside this bin");
    return PYL_ERR_UNSUPPORTED;
}



}  // namespace

template <int MAS>
int launch_tiled(const float *pos, const float *w, long long n, float *grid, float *grid2,
                 int dims, float inv, float halfcell, void *workspace, OutScale sc, cudaStream_t st,
                 unsigned *err, const RsdArgs *rsd, Owned ow)
{
    TileGeom g = tile_geom(dims);
    TiledWs ws = tiled_layout(workspace, n, dims);
    const int T = (int)g.ntiles;
    if (ow.on) {
        if (!owned_applies(dims)) {
            set_error("owned-cell write-out needs dims a multiple of 32");
            return PYL_ERR_INVALID;
        }
        ow.halo = ws.halo;
        ow.stride = (long long)g.ntiles * halo_cells(Support<MAS>::S - 1 + (grid2 ? 1 : 0));
    }
    if (ws.smem_hist) {
        const int C = ws.chunks;
        // chunks start on multiples of 4 particles (48 bytes) for the bulk copies
        const long long chunk = ((n + C - 1) / C + 3) / 4 * 4;
        const bool tma = (((uintptr_t)pos) & 15) == 0;
        const size_t sm = sizeof(unsigned) * T;
        // grids past TWO_LEVEL_TILES bins choose their placement by input coherence
        const bool counted = rsd || (tma && hist_tma_smem(T) <= 227 * 1024);
        const bool gated = counted && tma && ws.tmp;
        unsigned long long *same = gated ? ws.same : nullptr;
        stage_mark(PYL_STAGE_HIST, true, st);
        if (gated) PYL_CUDA(cudaMemsetAsync(ws.same, 0, sizeof(unsigned long long), st));
        const bool two = two_level_small(g);       // two chunks (CTAs) per SM
        const size_t hsm = hist_tma_smem(T);
        if (rsd) {                                 // callers check tiled_rsd_fusable first
            auto k = two ? chunk_hist_tma_sync_kernel<MAS, true> : chunk_hist_tma_kernel<MAS, true>;
            PYL_CUDA(ensure_smem(k, hsm));
            k<<<C, 1024, hsm, st>>>(pos, n, chunk, inv, g, ws.hist, err, *rsd, same);
        } else if (counted) {
            auto k = two ? chunk_hist_tma_sync_kernel<MAS, false> : chunk_hist_tma_kernel<MAS, false>;
            PYL_CUDA(ensure_smem(k, hsm));
            k<<<C, 1024, hsm, st>>>(pos, n, chunk, inv, g, ws.hist, err, RsdArgs{}, same);
        } else {
            PYL_CUDA(ensure_smem(chunk_hist_kernel<MAS>, sm));
            chunk_hist_kernel<MAS><<<C, 1024, sm, st>>>(pos, n, chunk, inv, g, ws.hist);
        }
        PYL_LAUNCH_CHECK();
        colscan_kernel<<<(T + 255) / 256, 256, 0, st>>>(ws.hist, C, T, ws.total);
        PYL_LAUNCH_CHECK();
        tile_scan_kernel<<<1, 1024, 0, st>>>(ws.total, T, ws.offsets, nullptr);
        PYL_LAUNCH_CHECK();
        stage_mark(PYL_STAGE_HIST, false, st);
        stage_mark(PYL_STAGE_PLACE, true, st);
        if (!ws.tmp && tma && level_a_tma_smem(T, 1024) <= 227 * 1024) {
            // at most TWO_LEVEL_TILES bins: level A with one bucket per bin writes the
            // final [bin][chunk] layout in one pass
            const size_t sat = level_a_tma_smem(T, 1024);
            if (w) {
                PYL_CUDA(ensure_smem(level_a_tma_kernel<MAS, true, 1024>, sat));
                level_a_tma_kernel<MAS, true, 1024><<<C, 1024, sat, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                         ws.offsets, ws.rec, 1, err);
            } else {
                PYL_CUDA(ensure_smem(level_a_tma_kernel<MAS, false, 1024>, sat));
                level_a_tma_kernel<MAS, false, 1024><<<C, 1024, sat, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                          ws.offsets, ws.rec, 1, err);
            }
        } else if (ws.tmp) {
            const int NCO = g.nc * g.nc * g.nc;
            const size_t sa = sizeof(unsigned) * ((3 * NCO + 32 + 3) & ~3) + sizeof(float4) * LA_BATCH +
                              sizeof(unsigned short) * LA_BATCH;
            const int lat = two_level_small(g) ? 512 : 1024;
            const size_t sat = level_a_tma_smem(NCO, lat);
            // coherent when at least 3/4 of the particles share their predecessor's bin
            const unsigned long long thresh = (unsigned long long)n - (unsigned long long)n / 4;
            const Gate coherent{same, thresh, 1}, incoherent{same, thresh, 0};
            if (gated && hsm <= 227 * 1024) {      // positions staged by bulk copies
#define PYL_SCATTER_TMA(WW, NT)                                                                               \
    do {                                                                                                     \
        PYL_CUDA(ensure_smem(chunk_scatter_tma_kernel<MAS, WW, NT>, hsm));                                   \
        chunk_scatter_tma_kernel<MAS, WW, NT><<<C, NT, hsm, st>>>(pos, w, n, chunk, inv, g, ws.hist, ws.offsets, \
                                                                 ws.rec, err, coherent);                     \
    } while (0)
                if (w) { if (two) PYL_SCATTER_TMA(true, 512); else PYL_SCATTER_TMA(true, 1024); }
                else   { if (two) PYL_SCATTER_TMA(false, 512); else PYL_SCATTER_TMA(false, 1024); }
#undef PYL_SCATTER_TMA
                PYL_LAUNCH_CHECK();
            } else if (gated) {
                if (w) {
                    PYL_CUDA(ensure_smem(chunk_scatter_kernel<MAS, true>, sm));
                    chunk_scatter_kernel<MAS, true><<<C, 1024, sm, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                         ws.offsets, ws.rec, coherent);
                } else {
                    PYL_CUDA(ensure_smem(chunk_scatter_kernel<MAS, false>, sm));
                    chunk_scatter_kernel<MAS, false><<<C, 1024, sm, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                          ws.offsets, ws.rec, coherent);
                }
                PYL_LAUNCH_CHECK();
            }
            if (tma && sat <= 227 * 1024) {
#define PYL_LEVEL_A(WW, NT)                                                                                   \
    do {                                                                                                     \
        PYL_CUDA(ensure_smem(level_a_tma_kernel<MAS, WW, NT>, sat));                                         \
        level_a_tma_kernel<MAS, WW, NT><<<C, NT, sat, st>>>(pos, w, n, chunk, inv, g, ws.hist, ws.offsets,   \
                                                           ws.tmp, 0, err, incoherent);                      \
    } while (0)
                if (w) { if (lat == 512) PYL_LEVEL_A(true, 512); else PYL_LEVEL_A(true, 1024); }
                else   { if (lat == 512) PYL_LEVEL_A(false, 512); else PYL_LEVEL_A(false, 1024); }
#undef PYL_LEVEL_A
            } else if (w) {
                PYL_CUDA(ensure_smem(level_a_kernel<MAS, true>, sa));
                level_a_kernel<MAS, true><<<C, LA_THREADS, sa, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                    ws.offsets, ws.tmp);
            } else {
                PYL_CUDA(ensure_smem(level_a_kernel<MAS, false>, sa));
                level_a_kernel<MAS, false><<<C, LA_THREADS, sa, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                     ws.offsets, ws.tmp);
            }
            PYL_LAUNCH_CHECK();
            stage_mark(PYL_STAGE_PLACE, false, st);
            stage_mark(PYL_STAGE_PLACE_B, true, st);
            PYL_CUDA(ensure_smem(level_b_tma_kernel<MAS>, level_b_tma_smem()));
            const int G = (C + num_sms() - 1) / num_sms();           // chunks per level-B segment
            level_b_tma_kernel<MAS><<<(unsigned)(((C + G - 1) / G) * NCO), LBT_THREADS, level_b_tma_smem(), st>>>(
                ws.tmp, C, G, inv, g, ws.hist, ws.total, ws.offsets, ws.rec, (unsigned)n, err, incoherent);
            PYL_LAUNCH_CHECK();
            stage_mark(PYL_STAGE_PLACE_B, false, st);
        } else if (w) {
            PYL_CUDA(ensure_smem(chunk_scatter_kernel<MAS, true>, sm));
            chunk_scatter_kernel<MAS, true><<<C, 1024, sm, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                 ws.offsets, ws.rec);
        } else {
            PYL_CUDA(ensure_smem(chunk_scatter_kernel<MAS, false>, sm));
            chunk_scatter_kernel<MAS, false><<<C, 1024, sm, st>>>(pos, w, n, chunk, inv, g, ws.hist,
                                                                  ws.offsets, ws.rec);
        }
        PYL_LAUNCH_CHECK();
        stage_mark(PYL_STAGE_PLACE, false, st);
    } else {
        PYL_CUDA(cudaMemsetAsync(ws.hist, 0, sizeof(unsigned) * g.ntiles, st));
        const int blocks = grid_blocks(n, 256, 16);
        tile_count_kernel<MAS><<<blocks, 256, 0, st>>>(pos, n, inv, g, ws.hist);
        PYL_LAUNCH_CHECK();
        tile_scan_kernel<<<1, 1024, 0, st>>>(ws.hist, g.ntiles, ws.offsets, ws.total);
        PYL_LAUNCH_CHECK();
        if (w) tile_scatter_kernel<MAS, true><<<blocks, 256, 0, st>>>(pos, w, n, inv, g, ws.total, ws.rec);
        else   tile_scatter_kernel<MAS, false><<<blocks, 256, 0, st>>>(pos, w, n, inv, g, ws.total, ws.rec);
        PYL_LAUNCH_CHECK();
    }
    stage_mark(PYL_STAGE_DEPOSIT, true, st);
    static_assert(FxShape<MAS, true>::FITS, "a bin with its halo fits shared memory");
    const float *inv_w = nullptr;
    if (w) {
        PYL_CUDA(cudaMemsetAsync(ws.wsc, 0, sizeof(unsigned), st));
        PYL_CUDA(cudaMemsetAsync(ws.wsc + 1, 0x7f, sizeof(unsigned), st));      // 0x7f7f7f7f: finite, large
        abs_range_kernel<<<grid_blocks(n, 256, 4), 256, 0, st>>>(w, n, (unsigned *)ws.wsc);
        PYL_LAUNCH_CHECK();
        w_scale_kernel<<<1, 1, 0, st>>>(ws.wsc, sc.host, sc.dev, MAS == PYL_MAS_NGP ? 1 : 0);
        PYL_LAUNCH_CHECK();
        inv_w = ws.wsc + 2;
        sc = OutScale{0.0f, ws.wsc + 3};
    }
    const int rc = grid2 ? launch_deposit_fx<MAS, true>(ws, g, inv, halfcell, grid, grid2, sc, st, ow, inv_w, err)
                         : launch_deposit_fx<MAS, false>(ws, g, inv, halfcell, grid, grid2, sc, st, ow, inv_w, err);
    stage_mark(PYL_STAGE_DEPOSIT, false, st);
    return rc;
}


}  // namespace pyl
