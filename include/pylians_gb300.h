/*
 * pylians_gb300 — C-ABI of the GB300 (sm_103a) density-field and clustering path.
 *
 * Every entry point is `extern "C"`, takes plain pointers and sizes, returns a
 * status code (0 = success) and never exits the process or traps the GPU.  All
 * buffers are owned by the caller and live on the device unless the parameter
 * name says `host_`.  `stream` is a cudaStream_t (NULL = legacy default stream);
 * every call is stream-ordered and asynchronous unless documented otherwise.
 * The library itself owns only its cached cuFFT plans (and their workspaces),
 * released by pyl_fft_cache_clear().
 *
 * Each entry point names the reference interface it replaces
 * (franciscovillaescusa/Pylians, path:line).
 */
#ifndef PYLIANS_GB300_H
#define PYLIANS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------------- */
#define PYL_OK 0
#define PYL_ERR_INVALID 1     /* bad argument (shape, size, enum, null pointer) */
#define PYL_ERR_CUDA 2        /* a CUDA runtime call failed */
#define PYL_ERR_CUFFT 3       /* a cuFFT call failed */
#define PYL_ERR_WORKSPACE 4   /* workspace smaller than *_workspace_size() */
#define PYL_ERR_UNSUPPORTED 5 /* valid request the library does not implement */

/* mass-assignment schemes: the reference's MAS_function indices (Pk_library.pyx:75-81) */
#define PYL_MAS_NONE 0
#define PYL_MAS_NGP 1
#define PYL_MAS_CIC 2
#define PYL_MAS_TSC 3
#define PYL_MAS_PCS 4

/* scatter strategies for pyl_ma */
#define PYL_STRATEGY_AUTO 0   /* library picks by grid size and particle count */
#define PYL_STRATEGY_ATOMIC 1 /* one thread per particle, atomics into the grid */
#define PYL_STRATEGY_TILED 2  /* bin particles by tile, deposit tiles in shared memory;
                                 3D; calls of 2^32 - 4096 particles and more run as
                                 consecutive passes (pyl_ma_set_pass_limit) */
#define PYL_STRATEGY_SORTED 3 /* radix sort by cell + fixed-order per-cell gather: bit-reproducible */

const char *pyl_strerror(int status);
/* Detail of the last failure on the calling host thread ("" if none). */
const char *pyl_last_error(void);
int pyl_version(void);

/* ---- mass assignment --------------------------------------------------------
 * Replaces MAS_library.MA (library/MAS_library/MAS_library.pyx:57-112) and the
 * kernels it dispatches to: NGP/NGPW (:273-325), CIC/CICW (:123-216),
 * TSC/TSCW (:369-452), PCS/PCSW (:463-545); also MAS_c.c NGP/CIC/TSC/PCS
 * (library/MAS_library/MAS_c.c:8-266) behind NGPc3D..PCSWc2D (:1136-1221).
 *
 * pos      float32 [n_particles][ndim], C-contiguous, ndim = 2 or 3
 * weights  float32 [n_particles] or NULL (W=None)
 * grid     float32 [dims]^ndim, row-major; ACCUMULATED into (+=), as MA does
 * grid_interlaced  NULL, or a second grid that receives the same particles
 *          shifted by +half a cell on every axis (float32 x + 0.5*BoxSize/dims);
 *          no counterpart in the reference (interlacing).
 * renormalize_2d   for ndim == 2: divide the whole grid by 2/3/4 after a
 *          CIC/TSC/PCS deposit, as MA's renormalize_2D=True does (:84-110).
 * Cell indices wrap periodically; positions outside [0, BoxSize) are wrapped,
 * never written out of bounds.  NGP counts (W=NULL) are bit-exact.
 */
size_t pyl_ma_workspace_size(int64_t n_particles, int ndim, int dims, int mas, int strategy,
                             int interlaced);
int pyl_ma(const float *pos, const float *weights, int64_t n_particles, int ndim,
           float *grid, float *grid_interlaced, int dims, float box_size, int mas,
           int strategy, int renormalize_2d, void *workspace, size_t workspace_bytes,
           void *stream);

/* Particles straight to the overdensity: grid (and grid_interlaced) are
 * OVERWRITTEN with delta = n/mean - 1, where n is the deposit and mean =
 * n_particles/dims^3, or sum(weights)/dims^3 (float64) with weights — the
 * callers' convention in library/Pk_library/Pk_snapshot.py:70-88.  One pass:
 * the grids are filled with -1 and every deposit is scaled by 1/mean.  3D only;
 * workspace as for pyl_ma (pyl_ma_workspace_size). */
int pyl_ma_overdensity(const float *pos, const float *weights, int64_t n_particles, float *grid,
                       float *grid_interlaced, int dims, float box_size, int mas, int strategy,
                       void *workspace, size_t workspace_bytes, void *stream);

/* pyl_ma_overdensity with redshift_space_library.pos_redshift_space
 * (library/redshift_space_library.pyx:29-43) in front: pos[:,axis] becomes
 * pos + vel (1+redshift)/hubble, wrapped into the box, IN PLACE (as the reference
 * mutates pos), then the overdensity deposit runs on the shifted positions.  On
 * the tiled path with a 16-byte aligned pos the shift is fused into the
 * histogram pass; otherwise it runs as its own pass first. */
int pyl_ma_overdensity_rsd(float *pos, const float *vel, const float *weights, int64_t n, float *grid,
                           float *grid_interlaced, int dims, float box_size, int mas, int strategy, float hubble,
                           float redshift, int axis, void *workspace, size_t workspace_bytes, void *stream);

/* Float64 grids: replaces MAS_library.CICW_d (library/MAS_library/MAS_library.pyx:229-266)
 * and NGPW_d (:338-358); TSC and PCS run the same way.
 * grid     float64 [dims][dims][depth], ACCUMULATED into (+=); depth == dims for
 *          ndim 3.  With ndim 2 the third index is 0 and the third-axis weight
 *          1, as in the reference's 2D use of these kernels (CIC adds each
 *          (x, y) term twice into plane 0).
 * weights  float32 [n_particles], or NULL for unit weights.
 * Each contribution is the reference's float32 product ((C0 C1) C2) W, added
 * to its float64 cell with a float64 atomic: the sums differ from the
 * reference's serial loop by float64 rounding at most (NGP sums of float32
 * weights are exact while they fit 53 bits). */
int pyl_ma_f64(const float *pos, const float *weights, int64_t n_particles, int ndim, double *grid, int dims,
               int depth, float box_size, int mas, void *stream);

/* Allocation-free mass assignment.  No counterpart in the reference: it exists
 * for callers that cannot allocate device memory around the call, such as
 * plugins inside a host framework whose own allocator owns all device memory,
 * and real-time loops that allocate nothing after start-up.
 * Same deposit as pyl_ma with the tiled strategy (3D grids only, grid +=,
 * optional interlaced grid), but the binning scratch lives in a fixed 24 MiB
 * array compiled into the library, held by every GPU that loads it until the
 * process exits.  Limits: n_particles <= 524288 and dims <= 512; larger
 * requests return PYL_ERR_INVALID.  The first call on a device looks up the
 * array's device address, and the first call with each combination of MAS,
 * weights and interlacing raises the shared-memory limits of its kernels
 * (cudaFuncSetAttribute).  All calls share the one array
 * and each keeps the previous call's contents (the call clears what must start
 * at zero), so calls that overlap on the GPU (different streams, or different
 * host threads) race and must be serialised by the caller.  Calls no
 * cudaMalloc/cudaFree. */
int pyl_ma_noalloc(const float *pos, const float *weights, int64_t n_particles, float *grid,
                   float *grid_interlaced, int dims, float box_size, int mas, void *stream);

/* ---- batched realizations --------------------------------------------------------
 * Many particle sets with uneven sizes, grids, MAS and interlacing in ONE
 * persistent launch (no counterpart in the reference, whose drivers loop over
 * MA() calls, e.g. library/MAS_library/MAS_gadget.py:35-76).  `reals` and
 * `items` live in device memory; each item deposits particles
 * [first, first+count) of realization `real`.  Grids must be pre-filled with -1
 * (pyl_fill); with scale = dims^3 / n_particles they end as the overdensity.
 * `counter` is one device unsigned (the work-queue head, zeroed by the call);
 * the grid size is num_SMs * ctas_per_sm CTAs of 256 threads. */
typedef struct pyl_batch_real {
    const float *pos;          /* float32 [n][3] */
    float *grid;               /* float32 [dims]^3 */
    float *grid_interlaced;    /* NULL or float32 [dims]^3 (positions + half a cell) */
    float inv;                 /* (float)dims / BoxSize */
    float halfcell;            /* (float)(0.5 * BoxSize / dims) */
    float scale;               /* factor on every deposit */
    int dims;
    int mas;                   /* PYL_MAS_NGP..PYL_MAS_PCS */
    int reserved;
} pyl_batch_real;

typedef struct pyl_batch_item {
    int64_t first;             /* first particle (index into the realization's pos) */
    uint32_t count;            /* particles in this item */
    uint32_t real;             /* index into reals */
} pyl_batch_item;

int pyl_ma_batch(const pyl_batch_real *reals, int n_reals, const pyl_batch_item *items, int n_items,
                 unsigned *counter, int ctas_per_sm, void *stream);

/* float32 fill of n values (grids to -1 before an overdensity deposit). */
int pyl_fill(float *p, int64_t n, float value, void *stream);
/* p[i] *= factor (the 1/N normalisation of inverse transforms, Pk_library.IFFT3Dr_f). */
int pyl_scale(float *p, int64_t n, float factor, void *stream);

/* Batched realizations through the tiled binning (no counterpart in the
 * reference): every realization's grid is cut into 32^3-cell bins numbered
 * tile_base[r] + (tx*nt + ty)*nt + tz (nt = ceil(dims/32), dims <= 512;
 * realizations with larger grids are skipped), total_tiles bins in all.  Four
 * stream-ordered launches: per-item bin histograms, a scan, per-item placement,
 * and one persistent deposit over all bins (10.22 fixed point per bin, the
 * realization's MAS and interlacing), adding scale * deposit into the grids
 * (pre-filled by the caller, e.g. with -1 for the overdensity).  reals, items
 * and tile_base live in device memory; total_particles = sum of item counts. */
size_t pyl_ma_batch_tiled_workspace_size(uint32_t total_tiles, int64_t total_particles);
int pyl_ma_batch_tiled(const pyl_batch_real *reals, int n_reals, const pyl_batch_item *items, int n_items,
                       const uint32_t *tile_base, uint32_t total_tiles, int64_t total_particles, void *workspace,
                       size_t workspace_bytes, int ctas_per_sm, void *stream);

/* ---- overdensity --------------------------------------------------------------
 * Replaces the callers' normalisation `delta /= mean; delta -= 1.0`
 * (library/Pk_library/Pk_snapshot.py:80-88, documentation/Documentation.md:93).
 * pyl_grid_sum writes the float64 sum of n float32 values into *d_sum (device).
 * pyl_overdensity applies delta = x / mean - 1 in float32, with mean = *d_sum / n
 * (d_sum != NULL) or mean = host_mean (d_sum == NULL).
 */
int pyl_grid_sum(const float *grid, int64_t n, double *d_sum, void *stream);
int pyl_overdensity(float *grid, int64_t n, const double *d_sum, double host_mean,
                    void *stream);

/* ---- FFT ---------------------------------------------------------------------
 * Replaces FFT3Dr_f / IFFT3Dr_f (library/Pk_library/Pk_library.pyx:120-133,152-165):
 * unnormalised single-precision R2C (forward) and C2R (backward) of `batch`
 * contiguous dims^3 grids.  Complex layout: complex64 [dims][dims][dims/2+1].
 * pyl_fft_c2r overwrites its input (cuFFT multi-dimensional C2R does).
 */
int pyl_fft_r2c(const float *in, void *out_c64, int dims, int batch, void *stream);
int pyl_fft_c2r(void *in_c64, float *out, int dims, int batch, void *stream);
int pyl_fft_cache_clear(void);

/* ---- power spectrum -----------------------------------------------------------
 * Replaces the mode loops of Pk (library/Pk_library/Pk_library.pyx:311-381) and
 * XPk (:625-737).  One read of F half-complex fields; MAS deconvolution
 * (x/sin x)^p per axis, optional interlacing combine, |k| / k_par / k_per
 * binning and Legendre l=0,2,4 sums, all without writing a k-grid.
 *
 * Channels: C = F + F(F-1)/2 — the F autos, then the cross pairs (i<j) in the
 * reference's order.  Bin counts: nb1 = dims/2+1, nb2 = (dims/2+1)*(kmax_per+1),
 * nb3 = kmax+1 (frequencies(), :59-64).  `sums` (device, float64, zeroed by
 * the call) receives, in order:
 *   P3   [nb3][3][C]   sum |d|^2 * L_l(mu), l = 0,2,4
 *   PH   [nb3][F]      sum phase^2, phase = atan2(Re d, |d|)
 *   P1   [nb1][C]      sum |d|^2 over |k| <= dims/2, by |k_par|
 *   P2   [nb2][C]      sum |d|^2 by (kmax_par+1)*k_per + |k_par|
 * pyl_pk_sums_len() returns that length.  `dk_interlaced` is NULL or the
 * half-cell-shifted partners of the F fields; then each field is
 * 1/2 [d1 + d2 exp(i pi (kx+ky+kz)/dims)] before deconvolution.
 * `field_stride` is the distance between consecutive fields in complex elements.
 *
 * pyl_pk_geometry fills the data-independent part (device, float64, zeroed):
 *   K1 [nb1] sum |k_par|, N1 [nb1], N2 [nb2], K3 [nb3] sum |k|, N3 [nb3]
 * (mode counts are exact integers stored as float64).
 * Both take a workspace of pyl_pk_workspace_size() bytes: for axis 2 the table
 * that visits rows in k_per order (required), and for one field the per-CTA
 * partial sums of the bin flushes (optional: with a smaller workspace the
 * flushes go to shared memory, slower; same sums up to float32 rounding order).
 */
int64_t pyl_pk_sums_len(int dims, int n_fields);
int64_t pyl_pk_geometry_len(int dims);
size_t pyl_pk_workspace_size(int dims, int n_fields, int axis);
int pyl_pk_bin(const void *dk, const void *dk_interlaced, int n_fields, int64_t field_stride,
               int dims, int axis, const int *host_mas_p, double *sums, void *workspace,
               size_t workspace_bytes, void *stream);
int pyl_pk_geometry(int dims, int axis, double *geom, void *workspace, size_t workspace_bytes,
                    void *stream);

/* Many one-field spectra of one grid side in one launch (the batched-realization
 * path; no counterpart in the reference, which bins one field per Pk call).  `items`
 * is a DEVICE array of n_items records, each one pyl_pk_bin call with n_fields = 1:
 * its field, its interlaced partner (non-NULL in every record when `interlaced`,
 * ignored otherwise), its own zeroed-by-the-call `sums` (pyl_pk_sums_len(dims, 1)
 * doubles) and MAS exponent.  The sums agree with pyl_pk_bin's item by item to
 * float32 rounding (the same kernels; with many items each CTA takes more rows
 * than in a one-field call, so the float32 partial sums group differently).  The
 * workspace (pyl_pk_bin_batch_workspace_size bytes) holds the axis-2 row table and
 * every item's per-CTA partial sums.  A workspace size of 0, and
 * PYL_ERR_UNSUPPORTED from the call, mean that one field's bins do not fit the
 * one-field kernel's shared memory: bin such items one by one with pyl_pk_bin. */
typedef struct pyl_pk_item {
    const void *dk;
    const void *dk_interlaced;
    double *sums;
    int mas_p;
    int reserved;
} pyl_pk_item;
size_t pyl_pk_bin_batch_workspace_size(int dims, int n_items, int axis, int interlaced);
int pyl_pk_bin_batch(const pyl_pk_item *items, int n_items, int dims, int axis, int interlaced,
                     void *workspace, size_t workspace_bytes, void *stream);

/* In place: d <- (interlace-combined d) * W(k)^-1 as float32, on every stored
 * mode (Pk_library.pyx:353-355; bispectrum_library.pyx:107-109).  This is the
 * delta_k the reference keeps with keep_deltak=True. */
int pyl_mas_deconvolve(void *dk, const void *dk_interlaced, int dims, int mas_p, void *stream);

/* ---- bispectrum ---------------------------------------------------------------
 * Replaces Bk (library/Pk_library/bispectrum_library.pyx:32-196).
 * Shell s holds the modes with host_k2_lo[s] <= kx^2+ky^2+kz^2 < host_k2_hi[s]
 * (the integer form of  k_min <= |k| < k_max  in units of kF, :73-77,116-118).
 * pyl_bk_shell_fill reads the deconvolved half-complex dims^3 field and writes,
 * for each shell, delta_s (complex64) and the indicator I_s (1+0i) as half grids
 * of side out_dims at out_delta + f*half, out_ind + f*half with f = host_slot[s]
 * (host_slot NULL: f = s; f = -1: the shell's power only, no field) (half =
 * out_dims*out_dims*(out_dims/2+1), mode (kx, ky, kz) at (kx mod out_dims,
 * ky mod out_dims, kz)), and power[2*s] = sum_x delta_s(x)^2 / dims^3,
 * power[2*s+1] = sum_x I_s(x)^2 / dims^3 on the dims^3 grid (float64, via
 * Parseval on the Hermitian half grid; zeroed by the call).  out_dims is dims,
 * or any side above 3 K with K the largest wave number of the call's shells:
 * the shell fields are band-limited, so the triple-product sums over out_dims^3
 * cells are (out_dims/dims)^3 times those over dims^3 cells and B, a ratio of
 * two such sums, is the same.  At most PYL_BK_MAX_SHELLS shells per call.
 * Either field set may be left out: the indicator fields and their sums depend
 * only on the shells, so a plan fills them once (dk and out_delta NULL; power[2*s]
 * is then 0) and every later call fills the delta fields alone (out_ind NULL);
 * with every slot -1 and dk given, the call computes the powers alone
 * (power[2*s+1] is written in every call).
 *
 * pyl_bk_triangles reduces the C2R'd real fields: for triangle t with shells
 * (a,b,c) = host_tri[3t..3t+2], num[t] = sum_x d_a d_b d_c and
 * den[t] = sum_x I_a I_b I_c (float64, zeroed by the call) over dims^3 cells
 * (the grid the fields live on); triangles sharing (a, b) are reduced together,
 * reading d_a d_b and I_a I_b once.  d_fields / i_fields are float32, shell s at
 * offset s*field_stride elements (field_stride >= dims^3, a multiple of 4;
 * buffers 16-byte aligned).  With i_fields NULL only num is computed (den may be
 * NULL and is not touched); with d_fields NULL only den.
 */
#define PYL_BK_MAX_SHELLS 96
int pyl_bk_shell_fill(const void *dk, int dims, int out_dims, const int64_t *host_k2_lo,
                      const int64_t *host_k2_hi, const int *host_slot, int n_shells, void *out_delta,
                      void *out_ind, double *power, void *stream);
int pyl_bk_triangles(const float *d_fields, const float *i_fields, int dims, int64_t field_stride,
                     int n_shells, const int *host_tri, int n_tri, double *num, double *den,
                     void *stream);

/* Triangle sums in Fourier space (no counterpart in the reference, which reduces
 * every triangle in real space, bispectrum_library.pyx:162-190).  For triangles
 * sharing their first two shells (a, b): pyl_bk_product forms P_ab = d_a d_b on the
 * out_dims^3 grid (float32, 16-byte aligned buffers), the caller transforms it
 * (pyl_fft_r2c) into prod_hat, and pyl_bk_shell_dots adds to out[host_dst[t]]
 *   (1/out_dims^3) sum over the stored modes k of triangle t's third shell
 *   (host_k2_lo[t] <= k^2 < host_k2_hi[t]) of w Re(v(k) conj(prod_hat(k))),
 * w = 2 for modes standing for a conjugate pair (0 < kz < out_dims/2), else 1,
 * v the deconvolved dims^3 field dk, or 1 (the indicator) when dk is NULL.  By
 * Parseval that is sum_x d_a d_b d_c over the out_dims^3 cells, what
 * pyl_bk_triangles reduces, so a group of triangles needs the real-space fields
 * of its first two shells only.  out is not zeroed (accumulates).  At most
 * PYL_BK_MAX_SHELLS triangles per call; out_dims as for pyl_bk_shell_fill. */
int pyl_bk_product(const float *a, const float *b, float *out, int64_t n, void *stream);
int pyl_bk_shell_dots(const void *dk, int dims, const void *prod_hat, int out_dims, const int64_t *host_k2_lo,
                      const int64_t *host_k2_hi, const int *host_dst, int n_tri, double *out, void *stream);

/* ---- learned aliasing correction (no counterpart in the reference) ----------------
 * MLP 4 -> 64 -> 64 -> 64 -> 1 with tanh hidden layers, BF16 weights and FP32
 * accumulation.  Parameters (pyl_mlp_param_count() of them, row-major [out][in]):
 *   W1[64][4] b1[64] W2[64][64] b2[64] W3[64][64] b3[64] W4[1][64] b4[1].
 * x: float32 [batch][4]; act: float32 [batch][192] hidden activations (forward
 * writes them when non-NULL; backward reads them); y: float32 [batch].
 * pyl_mlp_backward: gradient of sum_s w_s (y_s - t_s)^2 / weight_sum into grad
 * [param_count] (weights NULL = all 1); delta [batch][192] and dy [batch] are
 * scratch.  pyl_mlp_adam: Adam step on FP32 master weights, re-rounding the
 * BF16 copy (step counts from 1). */
int pyl_mlp_param_count(void);
int pyl_mlp_forward(const void *params_bf16, const float *x, int batch, float *act, float *y, void *stream);
int pyl_mlp_backward(const void *params_bf16, const float *x, const float *act, const float *y,
                     const float *target, const float *weights, float weight_sum, int batch, float *delta,
                     float *dy, float *grad, void *stream);
int pyl_mlp_adam(float *master, void *params_bf16, const float *grad, float *m, float *v, int n, float lr,
                 float beta1, float beta2, float eps, int step, void *stream);

/* ---- 2D fields (Pk_library.Pk_plane / XPk_plane, Pk_library.pyx:440-516, 814-941) ----
 * pyl_fft2_r2c: unnormalised R2C of `batch` contiguous dims^2 float32 maps into
 * [dims][dims/2+1] complex64 each (FFT2Dr_f).  pyl_pk_plane_bin: float64 sums
 * over the independent modes of one or two transformed maps (dk2 NULL for one):
 * K[nb] (sum |k|) | N[nb] | P1[nb] | P2[nb] | PX[nb] (Re d1 d2*), each field
 * multiplied by its MAS factor (exponent mas_p1 / mas_p2), nb =
 * pyl_pk_plane_bins(dims) = int(sqrt(2) dims/2) + 1. */
int pyl_fft2_r2c(const float *in, void *out_c64, int dims, int batch, void *stream);
int pyl_pk_plane_bins(int dims);
int pyl_pk_plane_bin(const void *dk1, const void *dk2, int dims, int mas_p1, int mas_p2, double *sums,
                     void *stream);

/* ---- smoothing (smoothing_library.pyx:20-114) ---------------------------------
 * pyl_filter_grid replaces the real-space part of FT_filter: field [dims]^3 gets
 * the Top-Hat (gaussian = 0: 1 where d^2 <= (R dims/BoxSize)^2) or Gaussian
 * (exp(-d^2 / (2 R_grid^2))) filter divided by its float64 sum (written to *norm);
 * pyl_fft_r2c follows.  pyl_cmul: a[i] *= b[i] for n complex64 values (the
 * Fourier-space product of field_smoothing). */
int pyl_filter_grid(float *field, int dims, float box_size, float R, int gaussian, double *norm, void *stream);
int pyl_cmul(void *a, const void *b, int64_t n, void *stream);

/* ---- correlation function (Pk_library.Xi, library/Pk_library/Pk_library.pyx:2035-2150) ----
 * pyl_xi_power: in place over an R2C output, every stored mode becomes
 * (|delta_k * W^-1|^2, 0) with the MAS factor of exponent mas_p rounded to float
 * (:2073-2083).  The caller then runs pyl_fft_c2r (unnormalised).  pyl_xi_bin:
 * sums over all dims^3 separations of that real grid by bin int(|r|): layout
 * X[nb3][3] (xi, xi L2(mu), xi L4(mu)) | R[nb3] (sum |r|) | N[nb3] (counts),
 * float64, pyl_xi_sums_len(dims) = 5 nb3 doubles; mu = r_axis / |r|. */
/* pyl_correct_mas replaces the mode loop of Pk_library.correct_MAS
 * (Pk_library.pyx:1776-1794) on an R2C output, in place: all stored modes but the
 * redundant half of the kz = 0 and kz = N/2 planes times the MAS factor, then
 * those two planes replaced by their Hermitian part, which is what the
 * reference's C2R makes of them; pyl_fft_c2r and a 1/dims^3 scale follow. */
int pyl_correct_mas(void *dk, int dims, int mas_p, void *stream);
int64_t pyl_xi_sums_len(int dims);
int pyl_xi_power(void *dk, int dims, int mas_p, void *stream);
int pyl_xi_bin(const float *xi_grid, int dims, int axis, double *sums, void *stream);

/* ---- optional per-phase timing (no counterpart in the reference; off by default) --
 * pyl_stage_timing(1) makes pyl_ma / pyl_ma_overdensity bracket their internal
 * phases with CUDA events on the launching stream; pyl_stage_times writes the
 * milliseconds summed per phase since the last call into ms_out[0..n) (phases
 * past PYL_STAGE_COUNT read 0).  Phases: */
#define PYL_STAGE_FILL 0      /* grids filled with -1 (overdensity) */
#define PYL_STAGE_HIST 1      /* per-chunk tile histograms and scans */
#define PYL_STAGE_PLACE 2     /* particles to tiles (single level, or level A) */
#define PYL_STAGE_PLACE_B 3   /* two-level placement, level B */
#define PYL_STAGE_DEPOSIT 4   /* per-bin shared-memory deposit and write-out */
#define PYL_STAGE_SORT 5      /* sorted strategy: keys, radix sort, runs, gather */
#define PYL_STAGE_HALO 6      /* owned-cell write-out: halo blocks added into the next bins */
#define PYL_STAGE_COUNT 8
int pyl_stage_timing(int enable);
int pyl_stage_times(double *ms_out, int n);

/* Thresholds of the tiled deposit's code paths (no counterpart in the reference),
 * process-wide, for tests and tuning: grids from owned_min_dims per side up
 * (multiples of 32) take the owned-cell write-out (default 1024), and unweighted
 * CIC/TSC/PCS deposits of at least tot_min_per_cell particles per bin cell on
 * average find fixed-point wraps from each bin's total (default 2.0).  A negative
 * value restores that default.  Change them only between calls (the workspace
 * size depends on the first). */
int pyl_ma_set_thresholds(int owned_min_dims, double tot_min_per_cell);

/* Particles per pass of the tiled deposit (no counterpart in the reference, whose
 * loop counter is a 64-bit long, MAS_library.pyx:123-166): its records and bin
 * offsets are 32-bit, so a call with more particles than the limit (default
 * 2^32 - 4096) deposits consecutive slices of at most that many, each pass
 * accumulating (pyl_ma) or, for the overdensity, the first storing -1 + value
 * and the others accumulating, with the mean density of the whole call; the
 * workspace is one pass's.  Process-wide, rounded down to a multiple of 1024
 * (at least 1024; negative restores the default), for tests and for callers
 * that want smaller workspaces.  Change it only between calls. */
int pyl_ma_set_pass_limit(int64_t max_particles);

/* Particles a CTA of the sorted strategy's gather stages in shared memory per x
 * offset of its cells' support (no counterpart in the reference), process-wide,
 * for tests: default and maximum 1024; a window holding more is summed straight
 * from the sorted runs, in the same order and with the same products, so the
 * grid does not depend on it.  0 sums every window straight from the runs; a
 * negative value restores the default; above 1024 returns PYL_ERR_INVALID.
 * Change it only between calls. */
int pyl_sorted_set_stage_limit(int max_particles);

/* Device-side error word (no counterpart in the reference): nonzero when a kernel's
 * bounded wait for its own bulk copies ran out and the kernel left early (its
 * output is then incomplete).  While it is set, the tiled strategy's second
 * placement level and deposit return at once (their input may be incomplete),
 * so grids are left as they were.  Synchronous; reset = 1 clears it.  The Python
 * package reads and clears it after every call that returns host results, and
 * raises if it was set. */
int pyl_device_error(int reset, unsigned *out);

/* Exercises that bounded wait (no counterpart in the reference; for tests): one
 * thread arms a shared-memory mbarrier for arm_bytes (a multiple of 16) of
 * bulk-copy data, issues no copy and waits at most `cycles` SM clock cycles
 * (0 < cycles <= 2e8).  *completed (device) becomes 1 if the phase completed
 * (arm_bytes == 0) and 0 if the wait ran out, which also sets the device error
 * word read by pyl_device_error.  Nothing is left in flight. */
int pyl_wait_probe(unsigned arm_bytes, long long cycles, unsigned *completed, void *stream);

/* ---- particle-side neighbours of the mass assignment --------------------------
 * pyl_cic_interp replaces MAS_library.CIC_interp (library/MAS_library/MAS_library.pyx:558-599):
 * out[i] = CIC interpolation of grid [dims]^3 at pos[i] (float32 [n][3]), the
 * eight terms added in the reference's order; indices wrap non-negatively.
 * pyl_pos_redshift_space replaces redshift_space_library.pos_redshift_space
 * (library/redshift_space_library.pyx:29-43): pos[:,axis] += vel[:,axis] *
 * (1+redshift)/Hubble in place, then positions above box_size or below 0 become
 * fmod(pos + box_size, box_size). */
int pyl_cic_interp(const float *grid, int dims, float box_size, const float *pos, int64_t n, float *out,
                   void *stream);
int pyl_pos_redshift_space(float *pos, const float *vel, int64_t n, float box_size, float hubble,
                           float redshift, int axis, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PYLIANS_GB300_H */
