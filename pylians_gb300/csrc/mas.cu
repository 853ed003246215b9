// Mass assignment (particles -> grid) for NGP / CIC / TSC / PCS, with weights,
// 2D / 3D grids and interlacing.
//
// Restates the per-particle arithmetic of library/MAS_library/MAS_library.pyx
// (NGP 273-292, CIC 123-166, TSC 369-404, PCS 463-497 and their W variants) in
// float32 exactly as the reference evaluates it:
//   * inv_cell = (float)dims / BoxSize (float division, :282);
//   * NGP: <int>(x*inv + 0.5) with a float product and a DOUBLE +0.5 — done
//     here exactly in float (floor / fraction test), no fp64 arithmetic;
//   * CIC: u = dist - <int>dist, d = 1 - u;  TSC: floor(dist-1.5) taken exactly
//     from floor(dist) and its fraction; TSC weights in float are bit-identical
//     to the reference's double-then-round evaluation (every intermediate is
//     exact); PCS weights are float (within 1 ulp of the reference);
//   * products (C0*C1)*C2 (*W), left to right, never fused into an FMA.
// Cell indices wrap with a non-negative modulo, so no input can write outside
// the grid.
//
// Strategies:
//   ATOMIC  one thread per particle, red.global.add per touched cell.  Best when
//           the grid lives in L2 (<= ~64 MB) or the particles are spatially sorted.
//   TILED   count -> scan -> bin particles by 16x32x32 tile -> one CTA per tile
//           deposits into shared memory (tile + halo for the kernel support and
//           the interlaced shift) and adds the tile into the grid with coalesced
//           red.global.add.  Each HBM grid line is read-modified-written once
//           per tile instead of once per particle.
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

template <int MAS>
struct Support { static constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS; };

// Per-axis support of one particle coordinate: first cell f (unwrapped) and the
// S weights of cells f, f+1, ..., f+S-1.
template <int MAS>
__device__ __forceinline__ long long axis_weights(float p, float inv, float *C)
{
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_NGP) {
        // <int>(dist + 0.5) with the sum in double (exact), truncation toward 0.
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        long long k = (long long)fl + (frac >= 0.5f ? 1 : 0);       // floor(dist + 0.5)
        if (dist < -0.5f && frac != 0.5f) k += 1;                  // trunc for negative sums
        C[0] = 1.0f;
        return k;
    } else if (MAS == PYL_MAS_CIC) {
        const long long k = (long long)truncf(dist);
        const float u = __fsub_rn(dist, truncf(dist));
        C[0] = __fsub_rn(1.0f, u);
        C[1] = u;
        return k;
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        const long long mn = (long long)fl - 2 + (frac >= 0.5f ? 1 : 0);  // floor(dist - 1.5)
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float diff = fabsf(__fsub_rn((float)(mn + j + 1), dist));
            float c;
            if (diff < 0.5f) {
                c = __fsub_rn(0.75f, __fmul_rn(diff, diff));
            } else if (diff < 1.5f) {
                const float t = __fsub_rn(1.5f, diff);
                c = __fmul_rn(__fmul_rn(0.5f, t), t);
            } else {
                c = 0.0f;
            }
            C[j] = c;
        }
        return mn + 1;
    } else {  // PCS
        const long long mn = (long long)floorf(dist) - 2;  // floor(dist - 2)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const float d = fabsf(__fsub_rn((float)(mn + j + 1), dist));
            float c;
            if (d < 1.0f) {
                const float a = __fmul_rn(__fmul_rn(6.0f, d), d);
                const float b = __fmul_rn(__fmul_rn(__fmul_rn(3.0f, d), d), d);
                c = __fdiv_rn(__fadd_rn(__fsub_rn(4.0f, a), b), 6.0f);
            } else if (d < 2.0f) {
                const float t = __fsub_rn(2.0f, d);
                c = __fdiv_rn(__fmul_rn(__fmul_rn(t, t), t), 6.0f);
            } else {
                c = 0.0f;
            }
            C[j] = c;
        }
        return mn + 1;
    }
}

// ------------------------------------------------------------------ ATOMIC path
template <int MAS, int NDIM, bool WEIGHTED, bool INTERLACED>
__global__ void __launch_bounds__(256) ma_atomic_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n,
    float *__restrict__ grid, float *__restrict__ grid2, int dims, float inv, float halfcell)
{
    constexpr int S = Support<MAS>::S;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long sa = NDIM == 3 ? (long long)dims * dims : dims;
    const long long sb = NDIM == 3 ? dims : 1;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float p[NDIM];
#pragma unroll
        for (int a = 0; a < NDIM; a++) p[a] = __ldg(pos + i * NDIM + a);
        const float wi = WEIGHTED ? __ldg(w + i) : 1.0f;
#pragma unroll
        for (int g = 0; g < (INTERLACED ? 2 : 1); g++) {
            float *out = g == 0 ? grid : grid2;
            float C[NDIM][S];
            int idx[NDIM][S];
#pragma unroll
            for (int a = 0; a < NDIM; a++) {
                const float q = g == 0 ? p[a] : __fadd_rn(p[a], halfcell);
                const long long f = axis_weights<MAS>(q, inv, C[a]);
#pragma unroll
                for (int j = 0; j < S; j++) idx[a][j] = wrap_index(f + j, dims);
            }
            if (NDIM == 3) {
#pragma unroll
                for (int l = 0; l < S; l++)
#pragma unroll
                    for (int m = 0; m < S; m++) {
                        const float c01 = __fmul_rn(C[0][l], C[1][m]);
                        const long long row = idx[0][l] * sa + idx[1][m] * sb;
#pragma unroll
                        for (int q = 0; q < S; q++) {
                            float v = __fmul_rn(c01, C[NDIM - 1][q]);
                            if (WEIGHTED) v = __fmul_rn(v, wi);
                            atomicAdd(out + row + idx[NDIM - 1][q], v);
                        }
                    }
            } else {
                // MA() runs 2D grids through the 3D kernels with the third index
                // fixed at 0 and weight 1, so each (l,m) lands S times (:84-110).
#pragma unroll
                for (int l = 0; l < S; l++)
#pragma unroll
                    for (int m = 0; m < S; m++) {
                        float v = __fmul_rn(C[0][l], C[1][m]);
                        if (WEIGHTED) v = __fmul_rn(v, wi);
                        float *cell = out + idx[0][l] * sa + idx[1][m];
                        for (int q = 0; q < S; q++) atomicAdd(cell, v);
                    }
            }
        }
    }
}

// ------------------------------------------------------------------- TILED path
constexpr int TX = 16, TY = 32, TZ = 32;   // tile extent in cells (x slowest)

struct TileGeom {
    int dims, ntx, nty, ntz;               // grid side, tiles per axis
    long long ntiles;
};

__host__ __device__ inline TileGeom tile_geom(int dims)
{
    TileGeom g;
    g.dims = dims;
    g.ntx = (dims + TX - 1) / TX;
    g.nty = (dims + TY - 1) / TY;
    g.ntz = (dims + TZ - 1) / TZ;
    g.ntiles = (long long)g.ntx * g.nty * g.ntz;
    return g;
}

template <int MAS>
__device__ __forceinline__ unsigned tile_key(const float *p, float inv, const TileGeom &g)
{
    float C[4];
    const int cx = wrap_index(axis_weights<MAS>(p[0], inv, C), g.dims);
    const int cy = wrap_index(axis_weights<MAS>(p[1], inv, C), g.dims);
    const int cz = wrap_index(axis_weights<MAS>(p[2], inv, C), g.dims);
    return (unsigned)(((long long)(cx / TX) * g.nty + cy / TY) * g.ntz + cz / TZ);
}

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

// Exclusive scan of `n` counts into offsets[0..n] and a copy into cursor[0..n-1],
// by one CTA of 1024 threads (n up to a few million tiles).
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
        cursor[i] = (unsigned)run;
        run += counts[i];
    }
    if (threadIdx.x == blockDim.x - 1) offsets[n] = (unsigned)part[threadIdx.x];
}

template <int MAS, bool WEIGHTED>
__global__ void __launch_bounds__(256) tile_scatter_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n, float inv, TileGeom g,
    unsigned *__restrict__ cursor, float *__restrict__ bpos, float *__restrict__ bw)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float p[3] = {__ldg(pos + 3 * i), __ldg(pos + 3 * i + 1), __ldg(pos + 3 * i + 2)};
        const unsigned slot = atomicAdd(cursor + tile_key<MAS>(p, inv, g), 1u);
        bpos[3ull * slot] = p[0];
        bpos[3ull * slot + 1] = p[1];
        bpos[3ull * slot + 2] = p[2];
        if (WEIGHTED) bw[slot] = __ldg(w + i);
    }
}

template <int MAS, bool INTERLACED>
struct TileShape {
    static constexpr int H = Support<MAS>::S - 1 + (INTERLACED ? 1 : 0);   // halo on the + side
    static constexpr int EX = TX + H, EY = TY + H, EZ = TZ + H;
    static constexpr int CELLS = EX * EY * EZ;
    static constexpr size_t SMEM = sizeof(float) * CELLS * (INTERLACED ? 2 : 1);
};

template <int MAS, bool WEIGHTED, bool INTERLACED>
__global__ void __launch_bounds__(512) tile_deposit_kernel(
    const float *__restrict__ bpos, const float *__restrict__ bw,
    const unsigned *__restrict__ offsets, TileGeom g, float inv, float halfcell,
    float *__restrict__ grid, float *__restrict__ grid2)
{
    using TS = TileShape<MAS, INTERLACED>;
    constexpr int S = Support<MAS>::S;
    extern __shared__ float smem[];
    const long long tile = blockIdx.x;
    const unsigned begin = offsets[tile], end = offsets[tile + 1];
    if (begin == end) return;
    const int tz = (int)(tile % g.ntz);
    const int ty = (int)((tile / g.ntz) % g.nty);
    const int tx = (int)(tile / ((long long)g.ntz * g.nty));
    const int ox = tx * TX, oy = ty * TY, oz = tz * TZ;
    for (int c = threadIdx.x; c < TS::CELLS * (INTERLACED ? 2 : 1); c += blockDim.x) smem[c] = 0.0f;
    __syncthreads();

    for (unsigned i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const float p[3] = {bpos[3ull * i], bpos[3ull * i + 1], bpos[3ull * i + 2]};
        const float wi = WEIGHTED ? bw[i] : 1.0f;
        int base[3];
        long long f0[3];
#pragma unroll
        for (int g2 = 0; g2 < (INTERLACED ? 2 : 1); g2++) {
            float C[3][S];
            int loc[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float q = g2 == 0 ? p[a] : __fadd_rn(p[a], halfcell);
                const long long f = axis_weights<MAS>(q, inv, C[a]);
                if (g2 == 0) {
                    // local coordinate of the first cell inside the tile
                    const int o = a == 0 ? ox : (a == 1 ? oy : oz);
                    f0[a] = f;
                    base[a] = wrap_index(f, g.dims) - o;
                    loc[a] = base[a];
                } else {
                    // the half-cell shift moves the first cell by 0 or +1; the clamp
                    // only matters for non-finite or astronomically large positions
                    const long long df = f - f0[a];
                    loc[a] = base[a] + (df <= 0 ? 0 : 1);
                }
            }
            float *t = smem + (g2 ? TS::CELLS : 0);
#pragma unroll
            for (int l = 0; l < S; l++)
#pragma unroll
                for (int m = 0; m < S; m++) {
                    const float c01 = __fmul_rn(C[0][l], C[1][m]);
                    float *row = t + ((loc[0] + l) * TS::EY + (loc[1] + m)) * TS::EZ + loc[2];
#pragma unroll
                    for (int q = 0; q < S; q++) {
                        float v = __fmul_rn(c01, C[2][q]);
                        if (WEIGHTED) v = __fmul_rn(v, wi);
                        atomicAdd(row + q, v);
                    }
                }
        }
    }
    __syncthreads();
    const long long d = g.dims;
    for (int gi = 0; gi < (INTERLACED ? 2 : 1); gi++) {
        const float *t = smem + (gi ? TS::CELLS : 0);
        float *out = gi ? grid2 : grid;
        for (int c = threadIdx.x; c < TS::CELLS; c += blockDim.x) {
            const float v = t[c];
            if (v == 0.0f) continue;
            const int lz = c % TS::EZ;
            const int ly = (c / TS::EZ) % TS::EY;
            const int lx = c / (TS::EZ * TS::EY);
            const long long gx = (ox + lx) % d, gy = (oy + ly) % d, gz = (oz + lz) % d;
            atomicAdd(out + (gx * d + gy) * d + gz, v);
        }
    }
}

__global__ void scale_kernel(float *g, long long n, float div)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        g[i] = __fdiv_rn(g[i], div);
}

inline int grid_blocks(long long n, int threads, int per_sm = 8)
{
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)num_sms() * per_sm;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

template <int MAS, int NDIM>
int launch_atomic(const float *pos, const float *w, long long n, float *grid, float *grid2,
                  int dims, float inv, float halfcell, cudaStream_t st)
{
    const int blocks = grid_blocks(n, 256, 16);
#define PYL_ATOMIC(WW, II) \
    ma_atomic_kernel<MAS, NDIM, WW, II><<<blocks, 256, 0, st>>>(pos, w, n, grid, grid2, dims, inv, halfcell)
    if (w) { if (grid2) PYL_ATOMIC(true, true); else PYL_ATOMIC(true, false); }
    else   { if (grid2) PYL_ATOMIC(false, true); else PYL_ATOMIC(false, false); }
#undef PYL_ATOMIC
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

struct TiledWs {
    unsigned *counts, *offsets, *cursor;
    float *bpos, *bw;
    size_t bytes;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

TiledWs tiled_layout(void *base, long long n, int dims, bool weighted)
{
    TileGeom g = tile_geom(dims);
    TiledWs ws;
    size_t off = 0;
    char *b = (char *)base;
    ws.counts = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * g.ntiles, 256);
    ws.offsets = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * (g.ntiles + 1), 256);
    ws.cursor = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * g.ntiles, 256);
    ws.bpos = (float *)(b + off); off = align_up(off + sizeof(float) * 3 * (size_t)n, 256);
    ws.bw = weighted ? (float *)(b + off) : nullptr;
    if (weighted) off = align_up(off + sizeof(float) * (size_t)n, 256);
    ws.bytes = off;
    return ws;
}

template <int MAS, bool W, bool I>
int launch_deposit(const TiledWs &ws, TileGeom g, float inv, float halfcell, float *grid,
                   float *grid2, cudaStream_t st)
{
    using TS = TileShape<MAS, I>;
    auto kern = tile_deposit_kernel<MAS, W, I>;
    static size_t done = 0;
    PYL_CUDA(ensure_smem(kern, TS::SMEM, &done));
    kern<<<(unsigned)g.ntiles, 512, TS::SMEM, st>>>(ws.bpos, ws.bw, ws.offsets, g, inv, halfcell,
                                                     grid, grid2);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

template <int MAS>
int launch_tiled(const float *pos, const float *w, long long n, float *grid, float *grid2,
                 int dims, float inv, float halfcell, void *workspace, cudaStream_t st)
{
    TileGeom g = tile_geom(dims);
    TiledWs ws = tiled_layout(workspace, n, dims, w != nullptr);
    PYL_CUDA(cudaMemsetAsync(ws.counts, 0, sizeof(unsigned) * g.ntiles, st));
    const int blocks = grid_blocks(n, 256, 16);
    tile_count_kernel<MAS><<<blocks, 256, 0, st>>>(pos, n, inv, g, ws.counts);
    PYL_LAUNCH_CHECK();
    tile_scan_kernel<<<1, 1024, 0, st>>>(ws.counts, g.ntiles, ws.offsets, ws.cursor);
    PYL_LAUNCH_CHECK();
    if (w) tile_scatter_kernel<MAS, true><<<blocks, 256, 0, st>>>(pos, w, n, inv, g, ws.cursor, ws.bpos, ws.bw);
    else   tile_scatter_kernel<MAS, false><<<blocks, 256, 0, st>>>(pos, w, n, inv, g, ws.cursor, ws.bpos, ws.bw);
    PYL_LAUNCH_CHECK();
    if (w) return grid2 ? launch_deposit<MAS, true, true>(ws, g, inv, halfcell, grid, grid2, st)
                        : launch_deposit<MAS, true, false>(ws, g, inv, halfcell, grid, grid2, st);
    return grid2 ? launch_deposit<MAS, false, true>(ws, g, inv, halfcell, grid, grid2, st)
                 : launch_deposit<MAS, false, false>(ws, g, inv, halfcell, grid, grid2, st);
}

inline int pick_strategy(int strategy, int ndim, int dims, long long n)
{
    if (strategy != PYL_STRATEGY_AUTO) return strategy;
    if (ndim != 3) return PYL_STRATEGY_ATOMIC;
    const double grid_bytes = 4.0 * dims * (double)dims * dims;
    if (grid_bytes <= 64.0 * 1024 * 1024 || n < 4 * (long long)tile_geom(dims).ntiles)
        return PYL_STRATEGY_ATOMIC;
    return PYL_STRATEGY_TILED;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" size_t pyl_ma_workspace_size(int64_t n_particles, int ndim, int dims, int mas,
                                        int strategy, int interlaced)
{
    (void)mas; (void)interlaced;
    if (n_particles < 0 || dims <= 0) return 0;
    const int s = pick_strategy(strategy, ndim, dims, n_particles);
    if (s == PYL_STRATEGY_TILED && ndim == 3)
        return tiled_layout(nullptr, n_particles, dims, true).bytes;
    return 0;
}

extern "C" int pyl_ma(const float *pos, const float *weights, int64_t n, int ndim, float *grid,
                      float *grid_interlaced, int dims, float box_size, int mas, int strategy,
                      int renormalize_2d, void *workspace, size_t workspace_bytes, void *stream)
{
    PYL_CHECK_ARG(ndim == 2 || ndim == 3, "ndim must be 2 or 3");
    PYL_CHECK_ARG(mas >= PYL_MAS_NGP && mas <= PYL_MAS_PCS, "MAS must be NGP, CIC, TSC or PCS");
    PYL_CHECK_ARG(dims > 0 && dims <= 65536, "dims out of range");
    PYL_CHECK_ARG(n >= 0, "negative particle count");
    PYL_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYL_CHECK_ARG(n == 0 || pos != nullptr, "pos is NULL");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    PYL_CHECK_ARG(strategy >= PYL_STRATEGY_AUTO && strategy <= PYL_STRATEGY_SORTED, "bad strategy");
    cudaStream_t st = (cudaStream_t)stream;
    const float inv = (float)dims / box_size;                 // MAS_library.pyx:282
    const float halfcell = (float)(0.5 * (double)box_size / dims);
    int s = pick_strategy(strategy, ndim, dims, n);
    if (s == PYL_STRATEGY_SORTED) s = PYL_STRATEGY_TILED;
    if (s == PYL_STRATEGY_TILED && (ndim != 3 || n > 0xFFFFFFF0ll)) s = PYL_STRATEGY_ATOMIC;
    if (s == PYL_STRATEGY_TILED) {
        const size_t need = tiled_layout(nullptr, n, dims, weights != nullptr).bytes;
        if (workspace_bytes < need || workspace == nullptr) {
            set_error("pyl_ma: tiled strategy needs " + std::to_string(need) + " workspace bytes");
            return PYL_ERR_WORKSPACE;
        }
    }
    int rc = PYL_OK;
    if (n > 0) {
#define PYL_DISPATCH(M)                                                                              \
    case M:                                                                                          \
        if (s == PYL_STRATEGY_TILED)                                                                 \
            rc = launch_tiled<M>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell,        \
                                 workspace, st);                                                     \
        else if (ndim == 3)                                                                          \
            rc = launch_atomic<M, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, st); \
        else                                                                                         \
            rc = launch_atomic<M, 2>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, st); \
        break;
        switch (mas) {
            PYL_DISPATCH(PYL_MAS_NGP)
            PYL_DISPATCH(PYL_MAS_CIC)
            PYL_DISPATCH(PYL_MAS_TSC)
            PYL_DISPATCH(PYL_MAS_PCS)
        }
#undef PYL_DISPATCH
    }
    if (rc) return rc;
    if (ndim == 2 && renormalize_2d && mas != PYL_MAS_NGP) {
        const long long cells = (long long)dims * dims;
        const float div = mas == PYL_MAS_CIC ? 2.0f : (mas == PYL_MAS_TSC ? 3.0f : 4.0f);
        scale_kernel<<<grid_blocks(cells, 256), 256, 0, st>>>(grid, cells, div);
        PYL_LAUNCH_CHECK();
        if (grid_interlaced) {
            scale_kernel<<<grid_blocks(cells, 256), 256, 0, st>>>(grid_interlaced, cells, div);
            PYL_LAUNCH_CHECK();
        }
    }
    return PYL_OK;
}
