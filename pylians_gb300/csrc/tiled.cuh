// Tiled mass assignment: what the C-ABI (mas.cu) and the units that instantiate the
// pipeline per MAS (tiled_ngp.cu, tiled_cic.cu, tiled_tsc.cu, tiled_pcs.cu) share —
// bin geometry, the workspace layout, the code-path thresholds and launch_tiled.
// The pipeline itself is tiled_impl.cuh.
#pragma once
#include <atomic>

#include <cuda_runtime.h>
#include <stdint.h>

#include "common.cuh"
#include "deposit.cuh"

namespace pyl {

// Factor applied to every deposited value: 1 for MA(), dims^3 / sum(mass) when
// the deposit writes the overdensity directly (read from device memory when the
// mass sum is computed on the device).
struct OutScale {
    float host;
    const float *dev;
};

__device__ __forceinline__ float out_scale(const OutScale &s) { return s.dev ? *s.dev : s.host; }


// Redshift-space shift fused into the histogram pass (pyl_ma_overdensity_rsd):
// the line-of-sight coordinate becomes x + v (1+z)/H, wrapped like
// redshift_space_library.pyx:38-42, and is written back before it is binned.
struct RsdArgs {
    float *pos;          // the same array as the kernel's input, written in place
    const float *vel;
    float factor, box;   // factor = (1 + redshift) / hubble, rounded to float
    float hubble, redshift;
    int axis;
};

constexpr int HIST_MAX_TILES = 49152;
constexpr int MAX_CHUNKS = 512;

struct TileGeom {
    int dims, nt, nc;      // grid side, tiles per axis, coarse blocks (4^3 tiles) per axis
    long long ntiles;      // number of tile keys: nc^3 * 64 (keys of tiles past the grid stay empty)
    unsigned mask;         // dims - 1 for power-of-two grids (cells wrap by a mask), else 0
};

__host__ __device__ inline TileGeom tile_geom(int dims)
{
    TileGeom g;
    g.dims = dims;
    g.nt = (dims + TB - 1) / TB;
    g.nc = (g.nt + 3) / 4;
    g.ntiles = (long long)g.nc * g.nc * g.nc * 64;
    g.mask = (dims & (dims - 1)) == 0 ? (unsigned)dims - 1u : 0u;
    return g;
}

// Tile keys are coarse-major: key = coarse * 64 + local, coarse = (tx/4, ty/4, tz/4),
// local = (tx%4, ty%4, tz%4), so the 64 tiles of a coarse block are contiguous.
__host__ __device__ inline unsigned tile_key_of(unsigned tx, unsigned ty, unsigned tz, const TileGeom &g)
{
    const unsigned coarse = ((tx >> 2) * (unsigned)g.nc + (ty >> 2)) * (unsigned)g.nc + (tz >> 2);
    return coarse * 64u + (((tx & 3u) << 4) | ((ty & 3u) << 2) | (tz & 3u));
}

constexpr int HT_BATCH = 4096;                  // histogram batch (particles)
constexpr int HT_NBUF = 2;                      // batches in flight
inline size_t hist_tma_smem(long long ntiles) { return (size_t)HT_NBUF * HT_BATCH * 12 + sizeof(unsigned) * ntiles; }

constexpr int TWO_LEVEL_TILES = 1024;   // up to here level A sorts by bin in one pass, whatever the input order

inline int grid_blocks(long long n, int threads, int per_sm = 8)
{
    long long b = (n + threads - 1) / threads;
    long long cap = (long long)num_sms() * per_sm;
    return (int)(b < 1 ? 1 : (b > cap ? cap : b));
}

// Halo blocks of the owned-cell write-out (see Owned below): block h = 1..7, bits
// (x, y, z) = (4, 2, 1), spans H layers along the axes whose bit is set and TB
// cells along the others.
__host__ __device__ constexpr int halo_ext(int H, int bit) { return bit ? H : TB; }
__host__ __device__ constexpr int halo_block_size(int H, int h)
{
    return halo_ext(H, h & 4) * halo_ext(H, h & 2) * halo_ext(H, h & 1);
}
__host__ __device__ constexpr int halo_block_off(int H, int h)
{
    return h <= 1 ? 0 : halo_block_off(H, h - 1) + halo_block_size(H, h - 1);
}
__host__ __device__ constexpr int halo_cells(int H) { return halo_block_off(H, 8); }   // (TB + H)^3 - TB^3
static_assert(halo_cells(2) == 34 * 34 * 34 - TB * TB * TB, "halo blocks cover the + side layers");

// Two-level placement over at most 128 coarse blocks (grids up to 512^3): level A
// runs two 512-thread CTAs per SM over twice as many chunks (2048-particle batches
// still give each coarse block runs of about 16 records).  Larger grids keep one
// 1024-thread CTA per SM with 4096-particle batches (512 coarse blocks: 8 records
// per run; halving the batch measured 1 ms slower at 1024^3).
inline bool two_level_small(const TileGeom &g)
{
    return g.ntiles > TWO_LEVEL_TILES && g.ntiles <= HIST_MAX_TILES && (long long)g.nc * g.nc * g.nc <= 128;
}

struct TiledWs {
    unsigned n;                  // particles binned
    unsigned *hist, *total, *offsets;
    float4 *rec;                 // binned particles: x, y, z, weight
    float4 *tmp;                 // two-level placement: the coarse-block layout
    float *halo;                 // owned-cell write-out: per-bin halo blocks
    unsigned long long *same;    // coherence count of the histogram pass
    float *wsc;                  // weighted deposits: w_scale_kernel's 5 words
    int chunks;
    bool smem_hist;
    size_t bytes;
};

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

inline TiledWs tiled_layout(void *base, long long n, int dims, size_t halo_floats = 0)
{
    TileGeom g = tile_geom(dims);
    TiledWs ws;
    ws.n = (unsigned)n;
    ws.smem_hist = g.ntiles <= HIST_MAX_TILES;
    ws.chunks = min(two_level_small(g) ? 2 * num_sms() : num_sms(), MAX_CHUNKS);
    const size_t hist_len = ws.smem_hist ? (size_t)ws.chunks * g.ntiles : (size_t)g.ntiles;
    size_t off = 0;
    char *b = (char *)base;
    ws.hist = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * hist_len, 256);
    ws.total = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * g.ntiles, 256);
    ws.offsets = (unsigned *)(b + off); off = align_up(off + sizeof(unsigned) * (g.ntiles + 1), 256);
    ws.same = (unsigned long long *)(b + off); off = align_up(off + sizeof(unsigned long long), 256);
    ws.wsc = (float *)(b + off); off = align_up(off + sizeof(float) * 8, 256);
    ws.rec = (float4 *)(b + off); off = align_up(off + sizeof(float4) * (size_t)n, 256);
    ws.tmp = nullptr;
    if (ws.smem_hist && g.ntiles > TWO_LEVEL_TILES) {
        ws.tmp = (float4 *)(b + off);
        off = align_up(off + sizeof(float4) * (size_t)n, 256);
    }
    ws.halo = (float *)(b + off);
    off = align_up(off + sizeof(float) * halo_floats, 256);
    ws.bytes = off;
    return ws;
}

// Grids whose bins tile them exactly take the owned-cell write-out from 1024^3 up;
// below that the fill pass plus atomic write-out measures as fast or faster (the
// four-bin CTAs of the owned deposit leave too few CTAs to balance 152 SMs).
constexpr int OWNED_MIN_DIMS = 1024;
// Unweighted CIC/TSC/PCS deposits with at least this many particles per bin cell on
// average find fixed-point wraps from each bin's total (see fx_accumulate).
constexpr double TOT_MIN_PER_CELL = 2.0;
// Both thresholds can be moved process-wide by pyl_ma_set_thresholds (tests reach
// the large-grid code paths on small grids with it).
extern std::atomic<int> g_owned_min_dims;
extern std::atomic<double> g_tot_min_per_cell;

// Particles per tiled pass: records, bin counts and offsets are 32-bit, so calls
// with more particles run the tiled deposit over consecutive passes of at most
// this many (a multiple of 1024, so every pass's positions stay 16-byte aligned).
constexpr long long TILED_PASS_MAX = 0xFFFFF000ll;
extern std::atomic<long long> g_tiled_pass_max;
inline long long tiled_pass_len(long long n) { return n < g_tiled_pass_max.load() ? n : g_tiled_pass_max.load(); }
inline bool owned_applies(int dims) { return dims % TB == 0 && dims >= g_owned_min_dims.load(); }

// Floats of the owned-cell halo buffers of both grids (0 when the grid does not
// take the owned-cell write-out, or a non-interlaced NGP deposit has no halo).
inline size_t owned_halo_floats(int mas, int dims, bool inter)
{
    if (!owned_applies(dims)) return 0;
    const int S = mas == PYL_MAS_NGP ? 1 : mas;
    const int H = S - 1 + (inter ? 1 : 0);
    return (size_t)(inter ? 2 : 1) * (size_t)tile_geom(dims).ntiles * (size_t)halo_cells(H);
}

struct Owned {
    bool on;             // false: atomic write-out of each bin with its halo
    float *halo;         // per-bin halo blocks (plain grid, then shifted grid)
    int fill_mode;       // 1: core = fill + value; 0: core = old + value
    float fill;
    long long stride;    // floats between the plain and the shifted grid's buffers
};

// The whole tiled deposit of one MAS (histogram, scans, placement, per-bin deposit,
// halo), stream-ordered on st.  err: device address of the error word that the
// staged kernels' bounded waits set (pyl_device_error).
template <int MAS>
int launch_tiled(const float *pos, const float *w, long long n, float *grid, float *grid2, int dims, float inv,
                 float halfcell, void *workspace, OutScale sc, cudaStream_t st, unsigned *err,
                 const RsdArgs *rsd = nullptr, Owned ow = Owned{false, nullptr, 0, 0.0f, 0});

extern template int launch_tiled<PYL_MAS_NGP>(const float *, const float *, long long, float *, float *, int, float, float, void *, OutScale,
                                  cudaStream_t, unsigned *, const RsdArgs *, Owned);
extern template int launch_tiled<PYL_MAS_CIC>(const float *, const float *, long long, float *, float *, int, float, float, void *, OutScale,
                                  cudaStream_t, unsigned *, const RsdArgs *, Owned);
extern template int launch_tiled<PYL_MAS_TSC>(const float *, const float *, long long, float *, float *, int, float, float, void *, OutScale,
                                  cudaStream_t, unsigned *, const RsdArgs *, Owned);
extern template int launch_tiled<PYL_MAS_PCS>(const float *, const float *, long long, float *, float *, int, float, float, void *, OutScale,
                                  cudaStream_t, unsigned *, const RsdArgs *, Owned);

}  // namespace pyl
