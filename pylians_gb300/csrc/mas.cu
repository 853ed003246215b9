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

#include <stdlib.h>

#include <atomic>
#include <map>
#include <mutex>

#include "common.cuh"
#include "sorted.cuh"
#include "tiled.cuh"
#include "tma.cuh"

namespace pyl {

// Set by a staged kernel whose bounded wait for its own bulk copies ran out
// (read and cleared by pyl_device_error); kernels get its device address.
__device__ unsigned g_tma_error;

std::atomic<int> g_owned_min_dims{OWNED_MIN_DIMS};
std::atomic<double> g_tot_min_per_cell{TOT_MIN_PER_CELL};
std::atomic<long long> g_tiled_pass_max{TILED_PASS_MAX};

namespace {
std::mutex g_err_mu;
std::map<int, unsigned *> g_err_addr;
}  // namespace

// Device address of g_tma_error on the current device (looked up once per device).
unsigned *tma_error_word()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
    std::lock_guard<std::mutex> lk(g_err_mu);
    auto it = g_err_addr.find(dev);
    if (it != g_err_addr.end()) return it->second;
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_tma_error) != cudaSuccess) return nullptr;
    g_err_addr[dev] = (unsigned *)p;
    return (unsigned *)p;
}

namespace {

// ------------------------------------------------------------------ ATOMIC path
template <int MAS, int NDIM, bool WEIGHTED, bool INTERLACED>
__global__ void __launch_bounds__(256) ma_atomic_kernel(
    const float *__restrict__ pos, const float *__restrict__ w, long long n,
    float *__restrict__ grid, float *__restrict__ grid2, int dims, float inv, float halfcell, OutScale sc)
{
    constexpr int S = Support<MAS>::S;
    const float scale = out_scale(sc);
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
                const int f = axis_weights<MAS>(q, inv, C[a]);
#pragma unroll
                for (int j = 0; j < S; j++) idx[a][j] = wrap_index((long long)f + j, dims);
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
                            atomicAdd(out + row + idx[NDIM - 1][q], __fmul_rn(v, scale));
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
                        v = __fmul_rn(v, scale);
                        float *cell = out + idx[0][l] * sa + idx[1][m];
                        for (int q = 0; q < S; q++) atomicAdd(cell, v);
                    }
            }
        }
    }
}


__global__ void scale_kernel(float *g, long long n, float div)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        g[i] = __fdiv_rn(g[i], div);
}

template <int MAS, int NDIM>
int launch_atomic(const float *pos, const float *w, long long n, float *grid, float *grid2,
                  int dims, float inv, float halfcell, OutScale sc, cudaStream_t st)
{
    const int blocks = grid_blocks(n, 256, 16);
#define PYL_ATOMIC(WW, II) \
    ma_atomic_kernel<MAS, NDIM, WW, II><<<blocks, 256, 0, st>>>(pos, w, n, grid, grid2, dims, inv, halfcell, sc)
    if (w) { if (grid2) PYL_ATOMIC(true, true); else PYL_ATOMIC(true, false); }
    else   { if (grid2) PYL_ATOMIC(false, true); else PYL_ATOMIC(false, false); }
#undef PYL_ATOMIC
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

// AUTO: binning pays once a deposit has about a million particles and several per
// bin; below that, red.global into an L2-resident grid wins.
inline int pick_strategy(int strategy, int ndim, int dims, long long n)
{
    if (strategy != PYL_STRATEGY_AUTO) return strategy;
    if (ndim != 3) return PYL_STRATEGY_ATOMIC;
    if (n < (1LL << 20) || n < 4 * (long long)tile_geom(dims).ntiles) return PYL_STRATEGY_ATOMIC;
    return PYL_STRATEGY_TILED;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" size_t pyl_ma_workspace_size(int64_t n_particles, int ndim, int dims, int mas,
                                        int strategy, int interlaced)
{
    if (n_particles < 0 || dims <= 0) return 0;
    const int s = pick_strategy(strategy, ndim, dims, n_particles);
    // + 256 bytes at the end: the mass sum and scale of pyl_ma_overdensity
    if (s == PYL_STRATEGY_SORTED && ndim == 3 && sorted_supported(n_particles, dims))
        return sorted_workspace_bytes(n_particles, dims) + 256;
    if (s == PYL_STRATEGY_TILED && ndim == 3)
        return tiled_layout(nullptr, tiled_pass_len(n_particles), dims,
                            owned_halo_floats(mas, dims, interlaced != 0)).bytes + 256;
    return 256;
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
    unsigned *err = tma_error_word();
    if (!err) {
        set_error("the device error word has no device address");
        return PYL_ERR_CUDA;
    }
    const float inv = (float)dims / box_size;                 // MAS_library.pyx:282
    const float halfcell = (float)(0.5 * (double)box_size / dims);
    const OutScale sc{1.0f, nullptr};
    int s = pick_strategy(strategy, ndim, dims, n);
    if (s == PYL_STRATEGY_SORTED) {
        if (ndim != 3 || !sorted_supported(n, dims)) {
            set_error("pyl_ma: the sorted strategy needs a 3D grid with dims^3 <= 2^32 and < 2^32 particles");
            return PYL_ERR_UNSUPPORTED;
        }
        const size_t need = sorted_workspace_bytes(n, dims);
        if (workspace_bytes < need || workspace == nullptr) {
            set_error("pyl_ma: sorted strategy needs " + std::to_string(need) + " workspace bytes");
            return PYL_ERR_WORKSPACE;
        }
        return launch_sorted(mas, pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, workspace, 1.0f,
                             nullptr, true, st);
    }
    if (s == PYL_STRATEGY_TILED && ndim != 3) s = PYL_STRATEGY_ATOMIC;
    Owned ow{false, nullptr, 0, 0.0f, 0};
    const long long pass = tiled_pass_len(n);
    if (s == PYL_STRATEGY_TILED) {
        const size_t need = tiled_layout(nullptr, pass, dims).bytes;
        if (workspace_bytes < need || workspace == nullptr) {
            set_error("pyl_ma: tiled strategy needs " + std::to_string(need) + " workspace bytes");
            return PYL_ERR_WORKSPACE;
        }
        // owned-cell write-out when the workspace also holds the halo blocks
        const size_t need_owned =
            tiled_layout(nullptr, pass, dims, owned_halo_floats(mas, dims, grid_interlaced != nullptr)).bytes;
        ow.on = owned_applies(dims) && workspace_bytes >= need_owned;
    }
    int rc = PYL_OK;
    if (n > 0) {
        // tiled: consecutive passes of at most `pass` particles, each accumulating
#define PYL_DISPATCH(M)                                                                              \
    case M:                                                                                          \
        if (s == PYL_STRATEGY_TILED)                                                                 \
            for (long long o = 0; o < n && rc == PYL_OK; o += pass)                                  \
                rc = launch_tiled<M>(pos + 3 * o, weights ? weights + o : nullptr, std::min(pass, n - o), \
                                     grid, grid_interlaced, dims, inv, halfcell, workspace, sc, st, err,  \
                                     nullptr, ow);                                                   \
        else if (ndim == 3)                                                                          \
            rc = launch_atomic<M, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st); \
        else                                                                                         \
            rc = launch_atomic<M, 2>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st); \
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

// ------------------------------------------------------------ overdensity
namespace pyl {
namespace {
__global__ void __launch_bounds__(256) fill_kernel(float *g, long long n, float v)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long n4 = ((((uintptr_t)g) & 15) == 0) ? n / 4 : 0;
    float4 *g4 = (float4 *)g;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride)
        g4[i] = make_float4(v, v, v, v);
    for (long long i = n4 * 4 + (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        g[i] = v;
}

// scale = cells / sum(mass), float64 then rounded once
__global__ void mass_scale_kernel(const double *sum, double cells, float *scale)
{
    *scale = (float)(cells / *sum);
}
}  // namespace
}  // namespace pyl

extern "C" int pyl_grid_sum(const float *grid, int64_t n, double *d_sum, void *stream);

extern "C" int pyl_pos_redshift_space(float *pos, const float *vel, int64_t n, float box_size, float hubble,
                                      float redshift, int axis, void *stream);

namespace {
// The redshift shift can ride on the staged histogram pass of the tiled deposit.
bool tiled_rsd_fusable(const float *pos, int dims)
{
    const TileGeom g = tile_geom(dims);
    return (((uintptr_t)pos) & 15) == 0 && g.ntiles <= HIST_MAX_TILES && hist_tma_smem(g.ntiles) <= 227 * 1024;
}

int ma_overdensity_impl(const float *pos, const float *weights, int64_t n, float *grid, float *grid_interlaced,
                        int dims, float box_size, int mas, int strategy, void *workspace, size_t workspace_bytes,
                        void *stream, const RsdArgs *rsd)
{
    PYL_CHECK_ARG(mas >= PYL_MAS_NGP && mas <= PYL_MAS_PCS, "MAS must be NGP, CIC, TSC or PCS");
    PYL_CHECK_ARG(dims > 0 && dims <= 65536, "dims out of range");
    PYL_CHECK_ARG(n > 0, "need at least one particle (the mean density is zero)");
    PYL_CHECK_ARG(grid != nullptr && pos != nullptr, "null pointer");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    PYL_CHECK_ARG(strategy >= PYL_STRATEGY_AUTO && strategy <= PYL_STRATEGY_SORTED, "bad strategy");
    const size_t need = pyl_ma_workspace_size(n, 3, dims, mas, strategy, grid_interlaced != nullptr);
    if (workspace == nullptr || workspace_bytes < need) {
        set_error("pyl_ma_overdensity: needs " + std::to_string(need) + " workspace bytes");
        return PYL_ERR_WORKSPACE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    unsigned *err = tma_error_word();
    if (!err) {
        set_error("the device error word has no device address");
        return PYL_ERR_CUDA;
    }
    const long long cells = (long long)dims * dims * dims;
    char *tail = (char *)workspace + need - 256;
    double *d_sum = (double *)tail;
    float *d_scale = (float *)(tail + 64);
    OutScale sc{(float)((double)cells / (double)n), nullptr};    // Pk_snapshot.py:85 (mean = N/dims^3)
    if (weights) {                                                // Pk_snapshot.py:80 (mean = sum(M)/dims^3)
        int rc = pyl_grid_sum(weights, n, d_sum, stream);
        if (rc) return rc;
        mass_scale_kernel<<<1, 1, 0, st>>>(d_sum, (double)cells, d_scale);
        PYL_LAUNCH_CHECK();
        sc = OutScale{0.0f, d_scale};
    }
    const float inv = (float)dims / box_size;
    const float halfcell = (float)(0.5 * (double)box_size / dims);
    int s = pick_strategy(strategy, 3, dims, n);
    // the owned-cell write-out stores -1 + value into every cell: no fill pass
    // (with several tiled passes, the first stores and the others accumulate)
    const Owned ow{s == PYL_STRATEGY_TILED && owned_applies(dims), nullptr, 1, -1.0f, 0};
    if (!ow.on) {
        const int blocks = grid_blocks(cells / 4 + 1, 256, 8);
        stage_mark(PYL_STAGE_FILL, true, st);
        fill_kernel<<<blocks, 256, 0, st>>>(grid, cells, -1.0f);
        PYL_LAUNCH_CHECK();
        if (grid_interlaced) {
            fill_kernel<<<blocks, 256, 0, st>>>(grid_interlaced, cells, -1.0f);
            PYL_LAUNCH_CHECK();
        }
        stage_mark(PYL_STAGE_FILL, false, st);
    }
    const RsdArgs *fused = nullptr;
    if (rsd) {
        if (s == PYL_STRATEGY_TILED && tiled_rsd_fusable(pos, dims)) {
            fused = rsd;
        } else {
            const int rc = pyl_pos_redshift_space(rsd->pos, rsd->vel, n, rsd->box, rsd->hubble, rsd->redshift,
                                                  rsd->axis, stream);
            if (rc) return rc;
        }
    }
    if (s == PYL_STRATEGY_SORTED)
        return launch_sorted(mas, pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, workspace, sc.host,
                             sc.dev, false, st);
    if (s != PYL_STRATEGY_TILED) {
        switch (mas) {
            case PYL_MAS_NGP: return launch_atomic<PYL_MAS_NGP, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st);
            case PYL_MAS_CIC: return launch_atomic<PYL_MAS_CIC, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st);
            case PYL_MAS_TSC: return launch_atomic<PYL_MAS_TSC, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st);
            default: return launch_atomic<PYL_MAS_PCS, 3>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, sc, st);
        }
    }
    // tiled: consecutive passes of at most `pass` particles; the scale is the whole
    // call's, and with the owned-cell write-out only the first pass stores
    const long long pass = tiled_pass_len(n);
    int rc = PYL_OK;
    for (long long o = 0; o < n && rc == PYL_OK; o += pass) {
        const long long cnt = std::min(pass, n - o);
        const float *p = pos + 3 * o;
        const float *w = weights ? weights + o : nullptr;
        Owned owp = ow;
        if (o > 0) owp.fill_mode = 0;
        RsdArgs rp;
        const RsdArgs *fp = nullptr;
        if (fused) {
            rp = *fused;
            rp.pos = fused->pos + 3 * o;
            rp.vel = fused->vel + 3 * o;
            fp = &rp;
        }
        switch (mas) {
            case PYL_MAS_NGP: rc = launch_tiled<PYL_MAS_NGP>(p, w, cnt, grid, grid_interlaced, dims, inv, halfcell, workspace, sc, st, err, fp, owp); break;
            case PYL_MAS_CIC: rc = launch_tiled<PYL_MAS_CIC>(p, w, cnt, grid, grid_interlaced, dims, inv, halfcell, workspace, sc, st, err, fp, owp); break;
            case PYL_MAS_TSC: rc = launch_tiled<PYL_MAS_TSC>(p, w, cnt, grid, grid_interlaced, dims, inv, halfcell, workspace, sc, st, err, fp, owp); break;
            default: rc = launch_tiled<PYL_MAS_PCS>(p, w, cnt, grid, grid_interlaced, dims, inv, halfcell, workspace, sc, st, err, fp, owp); break;
        }
    }
    return rc;
}

}  // namespace

extern "C" int pyl_ma_overdensity(const float *pos, const float *weights, int64_t n, float *grid,
                                  float *grid_interlaced, int dims, float box_size, int mas,
                                  int strategy, void *workspace, size_t workspace_bytes, void *stream)
{
    return ma_overdensity_impl(pos, weights, n, grid, grid_interlaced, dims, box_size, mas, strategy, workspace,
                               workspace_bytes, stream, nullptr);
}

extern "C" int pyl_ma_overdensity_rsd(float *pos, const float *vel, const float *weights, int64_t n, float *grid,
                                      float *grid_interlaced, int dims, float box_size, int mas, int strategy,
                                      float hubble, float redshift, int axis, void *workspace,
                                      size_t workspace_bytes, void *stream)
{
    PYL_CHECK_ARG(pos != nullptr && vel != nullptr, "null pointer");
    PYL_CHECK_ARG(axis >= 0 && axis <= 2, "axis must be 0, 1 or 2");
    PYL_CHECK_ARG(hubble != 0.0f, "Hubble must be non-zero");
    RsdArgs r;
    r.pos = pos;
    r.vel = vel;
    r.factor = (float)((1.0 + (double)redshift) / (double)hubble);   // redshift_space_library.pyx:36
    r.box = box_size;
    r.hubble = hubble;
    r.redshift = redshift;
    r.axis = axis;
    return ma_overdensity_impl(pos, weights, n, grid, grid_interlaced, dims, box_size, mas, strategy, workspace,
                               workspace_bytes, stream, &r);
}

// ------------------------------------------------------------- float64 grids
// MAS_library.CICW_d (MAS_library.pyx:229-266) and NGPW_d (:338-358): float32
// positions, weights and per-cell products exactly as the float32 kernels
// ((C0*C1)*C2)*W, no FMA), each product added to a float64 cell.  The grid is
// [dims][dims][depth]; with 2D positions the third index stays 0 and the third
// axis weight 1, so CIC adds each (x, y) term twice into plane 0, as the
// reference's loop over index_d[2] = index_u[2] = 0 does.
namespace pyl {
namespace {
template <int MAS>
__global__ void __launch_bounds__(256) ma_f64_kernel(const float *__restrict__ pos, const float *__restrict__ w,
                                                     long long n, int ndim, double *__restrict__ grid, int dims,
                                                     long long depth, float inv)
{
    constexpr int S = Support<MAS>::S;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        float C[3][S];
        int idx[3][S];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            if (a < ndim) {
                const int f = axis_weights<MAS>(__ldg(pos + i * ndim + a), inv, C[a]);
#pragma unroll
                for (int j = 0; j < S; j++) idx[a][j] = wrap_index((long long)f + j, dims);
            } else {
#pragma unroll
                for (int j = 0; j < S; j++) { C[a][j] = 1.0f; idx[a][j] = 0; }
            }
        }
        const float wi = w ? __ldg(w + i) : 1.0f;
#pragma unroll
        for (int l = 0; l < S; l++)
#pragma unroll
            for (int m = 0; m < S; m++) {
                const float c01 = __fmul_rn(C[0][l], C[1][m]);
                double *row = grid + ((long long)idx[0][l] * dims + idx[1][m]) * depth;
#pragma unroll
                for (int q = 0; q < S; q++)
                    atomicAdd(row + idx[2][q], (double)__fmul_rn(__fmul_rn(c01, C[2][q]), wi));
            }
    }
}
}  // namespace
}  // namespace pyl

extern "C" int pyl_ma_f64(const float *pos, const float *weights, int64_t n, int ndim, double *grid, int dims,
                          int depth, float box_size, int mas, void *stream)
{
    PYL_CHECK_ARG(ndim == 2 || ndim == 3, "ndim must be 2 or 3");
    PYL_CHECK_ARG(mas >= PYL_MAS_NGP && mas <= PYL_MAS_PCS, "MAS must be NGP, CIC, TSC or PCS");
    PYL_CHECK_ARG(dims > 0 && dims <= 65536, "dims out of range");
    PYL_CHECK_ARG(depth > 0 && (ndim == 2 || depth == dims), "depth must equal dims for 3D positions");
    PYL_CHECK_ARG(n >= 0, "negative particle count");
    PYL_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYL_CHECK_ARG(n == 0 || pos != nullptr, "pos is NULL");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    if (n == 0) return PYL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const float inv = (float)dims / box_size;                 // MAS_library.pyx:245,352
    const int blocks = grid_blocks(n, 256, 16);
    switch (mas) {
        case PYL_MAS_NGP: ma_f64_kernel<PYL_MAS_NGP><<<blocks, 256, 0, st>>>(pos, weights, n, ndim, grid, dims, depth, inv); break;
        case PYL_MAS_CIC: ma_f64_kernel<PYL_MAS_CIC><<<blocks, 256, 0, st>>>(pos, weights, n, ndim, grid, dims, depth, inv); break;
        case PYL_MAS_TSC: ma_f64_kernel<PYL_MAS_TSC><<<blocks, 256, 0, st>>>(pos, weights, n, ndim, grid, dims, depth, inv); break;
        default:          ma_f64_kernel<PYL_MAS_PCS><<<blocks, 256, 0, st>>>(pos, weights, n, ndim, grid, dims, depth, inv); break;
    }
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

// ------------------------------------------------------- allocation-free variant
// Some callers cannot allocate device memory around a call: plugins hosted by
// a framework whose allocator owns all device memory, and real-time loops that
// forbid allocation after start-up.  For them,
// pyl_ma_noalloc deposits through the same tiled kernels as pyl_ma but keeps
// the binning scratch in a fixed array compiled into this library.
namespace pyl {
namespace {
constexpr long long NOALLOC_MAX_PARTICLES = 1LL << 19;   // 524,288 particles
constexpr int NOALLOC_MAX_DIMS = 512;                    // <= (512/32)^3 = 4096 bins
// 524288 particles on a 512^3 grid: two record buffers (two-level placement) of
// 8 MiB + 4.8 MiB of chunk histograms (two chunks per SM)
constexpr size_t NOALLOC_SCRATCH_BYTES = 24u << 20;      // 24 MiB per device

// Held by every GPU that loads the library until the process exits.
__device__ __align__(256) unsigned char g_ma_scratch[NOALLOC_SCRATCH_BYTES];

std::mutex g_scratch_mu;
void *g_scratch_addr[64] = {};

// Device address of g_ma_scratch on the current device (looked up once per device).
int scratch_address(void **out)
{
    int dev = 0;
    PYL_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) {
        set_error("pyl_ma_noalloc: device index out of range");
        return PYL_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        PYL_CUDA(cudaGetSymbolAddress(&p, g_ma_scratch));
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return PYL_OK;
}
}  // namespace
}  // namespace pyl

extern "C" int pyl_ma_noalloc(const float *pos, const float *weights, int64_t n, float *grid,
                              float *grid_interlaced, int dims, float box_size, int mas, void *stream)
{
    PYL_CHECK_ARG(mas >= PYL_MAS_NGP && mas <= PYL_MAS_PCS, "MAS must be NGP, CIC, TSC or PCS");
    PYL_CHECK_ARG(grid != nullptr, "grid is NULL");
    PYL_CHECK_ARG(n >= 0, "negative particle count");
    PYL_CHECK_ARG(n == 0 || pos != nullptr, "pos is NULL");
    PYL_CHECK_ARG(box_size > 0.0f && isfinite(box_size), "BoxSize must be positive and finite");
    if (n > NOALLOC_MAX_PARTICLES || dims < 1 || dims > NOALLOC_MAX_DIMS) {
        set_error("pyl_ma_noalloc: at most " + std::to_string(NOALLOC_MAX_PARTICLES) +
                  " particles and dims <= " + std::to_string(NOALLOC_MAX_DIMS) +
                  " (got " + std::to_string(n) + " particles, dims " + std::to_string(dims) +
                  "); use pyl_ma with a workspace for larger inputs");
        return PYL_ERR_INVALID;
    }
    const size_t need = tiled_layout(nullptr, n, dims).bytes;
    if (need > NOALLOC_SCRATCH_BYTES) {
        set_error("pyl_ma_noalloc: request needs " + std::to_string(need) + " scratch bytes");
        return PYL_ERR_INVALID;
    }
    void *scratch = nullptr;
    int rc = scratch_address(&scratch);
    if (rc) return rc;
    if (n == 0) return PYL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    unsigned *err = tma_error_word();
    if (!err) {
        set_error("the device error word has no device address");
        return PYL_ERR_CUDA;
    }
    const float inv = (float)dims / box_size;
    const float halfcell = (float)(0.5 * (double)box_size / dims);
    switch (mas) {
        case PYL_MAS_NGP: return launch_tiled<PYL_MAS_NGP>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, scratch, OutScale{1.0f, nullptr}, st, err);
        case PYL_MAS_CIC: return launch_tiled<PYL_MAS_CIC>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, scratch, OutScale{1.0f, nullptr}, st, err);
        case PYL_MAS_TSC: return launch_tiled<PYL_MAS_TSC>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, scratch, OutScale{1.0f, nullptr}, st, err);
        default:          return launch_tiled<PYL_MAS_PCS>(pos, weights, n, grid, grid_interlaced, dims, inv, halfcell, scratch, OutScale{1.0f, nullptr}, st, err);
    }
}

// ------------------------------------------------------- bounded-wait probe
// One thread arms an mbarrier for arm_bytes of bulk-copy data and issues no copy,
// then waits on it with the staged kernels' bounded wait and the given cycle
// limit: with arm_bytes > 0 the phase never completes, the wait runs out, sets
// the device error word (pyl_device_error) and the kernel returns; with 0 the
// phase completes at the arrive and the word is left alone.  Nothing is in
// flight when the CTA leaves.
namespace pyl {
namespace {
__global__ void wait_probe_kernel(unsigned arm_bytes, long long cycles, unsigned *out)
{
    __shared__ __align__(8) unsigned long long bar;
    if (threadIdx.x != 0) return;
    mbar_init(&bar, 1);
    mbar_fence_init();
    mbar_arrive_expect_tx(&bar, arm_bytes);
    *out = mbar_wait_bounded(&bar, 0u, &g_tma_error, cycles) ? 1u : 0u;
}
}  // namespace
}  // namespace pyl

extern "C" int pyl_wait_probe(unsigned arm_bytes, long long cycles, unsigned *completed, void *stream)
{
    PYL_CHECK_ARG(completed != nullptr, "completed is NULL");
    PYL_CHECK_ARG(cycles > 0 && cycles <= pyl::MBAR_WAIT_CYCLES, "cycles must be in (0, 2e8]");
    PYL_CHECK_ARG(arm_bytes % 16 == 0 && arm_bytes < (1u << 20), "arm_bytes must be a multiple of 16 below 2^20");
    pyl::wait_probe_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(arm_bytes, cycles, completed);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_ma_set_thresholds(int owned_min_dims, double tot_min_per_cell)
{
    PYL_CHECK_ARG(owned_min_dims != 0, "owned_min_dims must be positive (or negative for the default)");
    PYL_CHECK_ARG(!(tot_min_per_cell != tot_min_per_cell), "tot_min_per_cell is NaN");
    pyl::g_owned_min_dims.store(owned_min_dims < 0 ? pyl::OWNED_MIN_DIMS : owned_min_dims);
    pyl::g_tot_min_per_cell.store(tot_min_per_cell < 0.0 ? pyl::TOT_MIN_PER_CELL : tot_min_per_cell);
    return PYL_OK;
}

extern "C" int pyl_ma_set_pass_limit(int64_t max_particles)
{
    PYL_CHECK_ARG(max_particles != 0, "max_particles must be positive (or negative for the default)");
    long long v = max_particles < 0 ? pyl::TILED_PASS_MAX : std::min((long long)max_particles, pyl::TILED_PASS_MAX);
    v = v / 1024 * 1024;
    PYL_CHECK_ARG(v >= 1024, "max_particles must be at least 1024");
    pyl::g_tiled_pass_max.store(v);
    return PYL_OK;
}

extern "C" int pyl_device_error(int reset, unsigned *out)
{
    PYL_CHECK_ARG(out != nullptr, "null pointer");
    PYL_CUDA(cudaMemcpyFromSymbol(out, pyl::g_tma_error, sizeof(unsigned)));
    if (reset) {
        const unsigned zero = 0;
        PYL_CUDA(cudaMemcpyToSymbol(pyl::g_tma_error, &zero, sizeof(unsigned)));
    }
    return PYL_OK;
}
