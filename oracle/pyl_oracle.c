/*
 * CPU restatement of Pylians' mass-assignment kernels and P(k)/XPk mode loop.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle that the CUDA path is
 * checked against (tests/, __graft_entry__.smoke) and the CPU baseline that
 * bench.py times beside it.  No product code links or calls it.
 *
 * It restates, in plain C, the arithmetic of
 *   library/MAS_library/MAS_library.pyx  NGP 273-292, NGPW 305-325, CIC 123-166,
 *                                        CICW 179-216, TSC 369-404, TSCW 417-452,
 *                                        PCS 463-497, PCSW 510-545
 *   library/MAS_library/MAS_c.c          NGP 74-120, CIC 8-69, TSC 125-193, PCS 198-266
 *   library/Pk_library/Pk_library.pyx    Pk mode loop 311-381, XPk mode loop 625-737,
 *                                        MAS_correction 86-87
 * keeping the reference's precision choices (float32 positions and weights,
 * float32 inverse cell size, double "+0.5" in NGP, double MAS factors rounded
 * to float, double per-bin sums).  It is compiled with -ffp-contract=off so
 * that no multiply-add is fused behind the reader's back.
 *
 * Two deviations from the reference, both outside its defined domain:
 *   - cell indices are wrapped with a non-negative modulo; the reference's C
 *     '%' yields a negative index (an out-of-bounds write) for positions below
 *     -BoxSize (Cython) or below 0 (MAS_c.c);
 *   - threads>1 runs the particle loop with OpenMP atomics exactly like
 *     MAS_c.c, and the mode loop with per-thread bins summed in thread order
 *     (the reference's mode loop is serial).  threads==1 reproduces the
 *     reference's serial summation order.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline int wrap(int i, int n) { int r = i % n; return r < 0 ? r + n : r; }

static inline void add_cell(float *grid, double *grid64, int64_t idx, float v, int atomic)
{
    if (grid64) {
        if (atomic) {
#pragma omp atomic
            grid64[idx] += (double)v;
        } else {
            grid64[idx] += (double)v;
        }
    } else if (atomic) {
#pragma omp atomic
        grid[idx] += v;
    } else {
        grid[idx] += v;
    }
}

/*
 * flavor 0: MAS_library.pyx (the MA() path): inv = (float)dims / BoxSize in
 *           float; 2D grids take the third-axis loop with index 0 and weight 1,
 *           so CIC/TSC/PCS deposit 2/3/4 times (MA() later divides).
 * flavor 1: MAS_c.c: inv = (float)(dims*1.0/BoxSize) via double; 2D grids get
 *           one deposit per (l,m).
 * mas: 1 NGP, 2 CIC, 3 TSC, 4 PCS.   ndim: 2 or 3.   w may be NULL.
 */
static int ma_any(const float *pos, int64_t n, int ndim, float *grid, double *grid64, int dims,
                  float box, int mas, const float *w, int threads, int flavor)
{
    if (ndim != 2 && ndim != 3) return 1;
    if (mas < 1 || mas > 4) return 2;
    float inv = flavor == 0 ? (float)dims / box : (float)(dims * 1.0 / box);
    int64_t sa, sb, sc;                 /* strides of the three index slots */
    int nthird;                         /* deposits along the third slot */
    if (ndim == 3) { sa = (int64_t)dims * dims; sb = dims; sc = 1; }
    else           { sa = dims; sb = 1; sc = 0; }
    const int support = mas == 1 ? 1 : mas;      /* 1,2,3,4 cells per axis */
    if (ndim == 3) nthird = support;
    else           nthird = flavor == 0 ? support : 1;
    int atomic = threads > 1;
#ifdef _OPENMP
    if (threads < 1) threads = 1;
#pragma omp parallel for num_threads(threads) schedule(static) if (threads > 1)
#endif
    for (int64_t i = 0; i < n; i++) {
        int idx[3][4] = {{0}};
        float C[3][4] = {{1, 1, 1, 1}, {1, 1, 1, 1}, {1, 1, 1, 1}};
        for (int a = 0; a < ndim; a++) {
            float p = pos[i * ndim + a];
            if (mas == 1) {
                /* <int>(pos*inv + 0.5): float product, double sum, truncation */
                float prod = p * inv;
                int k = (int)((double)prod + 0.5);
                idx[a][0] = wrap(k, dims);
            } else if (mas == 2) {
                float dist = p * inv;
                int k = (int)dist;
                float u = dist - (float)k;
                float d = (float)(1.0 - (double)u);
                idx[a][0] = wrap(k, dims);
                idx[a][1] = wrap(idx[a][0] + 1, dims);
                C[a][0] = d; C[a][1] = u;
            } else if (mas == 3) {
                float dist = p * inv;
                int mn = (int)floor((double)dist - 1.5);
                for (int j = 0; j < 3; j++) {
                    idx[a][j] = wrap(mn + j + 1, dims);
                    float diff = (float)fabs((double)((float)(mn + j + 1) - dist));
                    float c;
                    if (diff < 0.5)      c = (float)(0.75 - (double)(diff * diff));
                    else if (diff < 1.5) c = (float)(0.5 * (1.5 - (double)diff) * (1.5 - (double)diff));
                    else                 c = 0.0f;
                    C[a][j] = c;
                }
            } else {
                float dist = p * inv;
                int mn = (int)floor((double)dist - 2.0);
                for (int j = 0; j < 4; j++) {
                    idx[a][j] = wrap(mn + j + 1, dims);
                    float diff = (float)fabs((double)((float)(mn + j + 1) - dist));
                    double dd = diff;
                    float c;
                    if (diff < 1.0)      c = (float)((4.0 - 6.0 * dd * dd + 3.0 * dd * dd * dd) / 6.0);
                    else if (diff < 2.0) c = (float)((2.0 - dd) * (2.0 - dd) * (2.0 - dd) / 6.0);
                    else                 c = 0.0f;
                    C[a][j] = c;
                }
            }
        }
        if (mas == 1) {
            int64_t cell = idx[0][0] * sa + idx[1][0] * sb + idx[2][0] * sc;
            add_cell(grid, grid64, cell, w ? w[i] : 1.0f, atomic);
            continue;
        }
        for (int l = 0; l < support; l++)
            for (int m = 0; m < support; m++)
                for (int q = 0; q < nthird; q++) {
                    int64_t cell = idx[0][l] * sa + idx[1][m] * sb + idx[2][q] * sc;
                    float v = C[0][l] * C[1][m];
                    v = v * C[2][q];
                    if (w) v = v * w[i];
                    add_cell(grid, grid64, cell, v, atomic);
                }
    }
    return 0;
}

int oracle_ma(const float *pos, int64_t n, int ndim, float *grid, int dims,
              float box, int mas, const float *w, int threads, int flavor)
{
    return ma_any(pos, n, ndim, grid, NULL, dims, box, mas, w, threads, flavor);
}

/*
 * oracle_ma with the same float32 weights and products added to a float64 grid:
 * the reference's arithmetic without its float32 accumulation rounding (one ulp
 * of the cell value per add, which the MAS deconvolution amplifies near the
 * Nyquist corner).  For comparisons whose error budget is the tested path's own.
 */
int oracle_ma_acc64(const float *pos, int64_t n, int ndim, double *grid, int dims,
                    float box, int mas, const float *w, int threads, int flavor)
{
    return ma_any(pos, n, ndim, NULL, grid, dims, box, mas, w, threads, flavor);
}

/*
 * MAS_library.CIC_interp (MAS_library.pyx:558-599): den[i] = sum over the 8
 * cells around pos[i] of density * d/u weights, terms added left to right in
 * the reference's order (d,d,d), (d,d,u), (d,u,d), (d,u,u), (u,d,d), ...
 * Indices wrap non-negatively (the reference reads out of bounds for
 * positions below 0).
 */
void oracle_cic_interp(const float *density, int dims, float box, const float *pos, int64_t n, float *den)
{
    const float inv = (float)dims / box;
    for (int64_t i = 0; i < n; i++) {
        float u[3], d[3];
        int id[3], iu[3];
        for (int a = 0; a < 3; a++) {
            float dist = pos[i * 3 + a] * inv;
            int k = (int)dist;
            u[a] = dist - (float)k;
            d[a] = (float)(1.0 - (double)u[a]);
            id[a] = wrap(k, dims);
            iu[a] = wrap(id[a] + 1, dims);
        }
        const int64_t D = dims;
#define G(x, y, z) density[((int64_t)(x) * D + (y)) * D + (z)]
        float t = G(id[0], id[1], id[2]) * d[0] * d[1] * d[2];
        t = t + G(id[0], id[1], iu[2]) * d[0] * d[1] * u[2];
        t = t + G(id[0], iu[1], id[2]) * d[0] * u[1] * d[2];
        t = t + G(id[0], iu[1], iu[2]) * d[0] * u[1] * u[2];
        t = t + G(iu[0], id[1], id[2]) * u[0] * d[1] * d[2];
        t = t + G(iu[0], id[1], iu[2]) * u[0] * d[1] * u[2];
        t = t + G(iu[0], iu[1], id[2]) * u[0] * u[1] * d[2];
        t = t + G(iu[0], iu[1], iu[2]) * u[0] * u[1] * u[2];
#undef G
        den[i] = t;
    }
}

/*
 * redshift_space_library.pos_redshift_space (redshift_space_library.pyx:29-43):
 * pos[:,axis] += vel[:,axis] * (1+z)/H, then positions above BoxSize or below 0
 * become fmod(pos + BoxSize, BoxSize) (C remainder, as cdivision(True)).
 */
void oracle_rsd(float *pos, const float *vel, int64_t n, float box, float hubble, float redshift, int axis)
{
    const float factor = (float)((1.0 + (double)redshift) / (double)hubble);
    for (int64_t i = 0; i < n; i++) {
        float p = pos[i * 3 + axis] + vel[i * 3 + axis] * factor;
        if (p > box || p < 0.0f) p = fmodf(p + box, box);
        pos[i * 3 + axis] = p;
    }
}

/* (x/sin x)^p with C(0)=1: Pk_library.pyx:86-87 */
static inline double mas_correction(double x, int p)
{
    return x == 0.0 ? 1.0 : pow(x / sin(x), p);
}

/*
 * Mode loop of Pk / XPk over the half-complex R2C output of F fields.
 *   dk       complex64 interleaved, field-major: F x [dims][dims][dims/2+1];
 *            multiplied in place by the MAS factor (as the reference does).
 *   mas_p    per-field window exponent (0 none, 1 NGP, 2 CIC, 3 TSC, 4 PCS).
 * Output sums are raw (before the reference's finalisation); the caller zeroes
 * them.  Layouts: nb1 = dims/2+1, nb2 = (kmax_par+1)*(kmax_per+1), nb3 = kmax+1,
 * X = F(F-1)/2:
 *   k1D[nb1], Nmodes1D[nb1], Pk1D[nb1][F], PkX1D[nb1][X]
 *   Nmodes2D[nb2], Pk2D[nb2][F], PkX2D[nb2][X]
 *   k3D[nb3], Nmodes3D[nb3], Pk3D[nb3][3][F], PkX3D[nb3][3][X], Pkphase[nb3][F]
 */
int oracle_pk_modes(float *dk, int F, int dims, int axis, const int *mas_p, int threads,
                    double *k1D, double *Nmodes1D, double *Pk1D, double *PkX1D,
                    double *Nmodes2D, double *Pk2D, double *PkX2D,
                    double *k3D, double *Nmodes3D, double *Pk3D, double *PkX3D,
                    double *Pkphase)
{
    const int middle = dims / 2;
    const int kmax_par = middle;
    const int kmax_per = (int)sqrt((double)middle * middle + (double)middle * middle);
    const int kmax = (int)sqrt(3.0 * (double)middle * middle);
    const int nb1 = kmax_par + 1, nb2 = (kmax_par + 1) * (kmax_per + 1), nb3 = kmax + 1;
    const int X = F * (F - 1) / 2;
    const int64_t nz = middle + 1;
    const int64_t fstride = (int64_t)dims * dims * nz;
    const double prefact = M_PI / dims;
    if (threads < 1) threads = 1;

    /* per-thread private bins */
    const int64_t per_thread = 2 * nb1 + nb1 * (F + X) + nb2 + nb2 * (F + X) +
                               2 * nb3 + nb3 * 3 * (F + X) + nb3 * F;
    double *priv = (double *)calloc((size_t)per_thread * threads, sizeof(double));
    if (!priv) return 3;

#ifdef _OPENMP
#pragma omp parallel num_threads(threads) if (threads > 1)
#endif
    {
        int tid = 0;
#ifdef _OPENMP
        tid = omp_get_thread_num();
#endif
        double *b = priv + per_thread * tid;
        double *tk1 = b;              double *tn1 = tk1 + nb1;
        double *tp1 = tn1 + nb1;      double *tx1 = tp1 + (int64_t)nb1 * F;
        double *tn2 = tx1 + (int64_t)nb1 * X;
        double *tp2 = tn2 + nb2;      double *tx2 = tp2 + (int64_t)nb2 * F;
        double *tk3 = tx2 + (int64_t)nb2 * X;
        double *tn3 = tk3 + nb3;      double *tp3 = tn3 + nb3;
        double *tx3 = tp3 + (int64_t)nb3 * 3 * F;
        double *tph = tx3 + (int64_t)nb3 * 3 * X;
        double re[64], im[64];
        double corr[64][3];

#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
        for (int kxx = 0; kxx < dims; kxx++) {
            int kx = kxx > middle ? kxx - dims : kxx;
            for (int f = 0; f < F; f++) corr[f][0] = mas_correction(prefact * kx, mas_p[f]);
            for (int kyy = 0; kyy < dims; kyy++) {
                int ky = kyy > middle ? kyy - dims : kyy;
                for (int f = 0; f < F; f++) corr[f][1] = mas_correction(prefact * ky, mas_p[f]);
                for (int kzz = 0; kzz <= middle; kzz++) {
                    int kz = kzz;
                    for (int f = 0; f < F; f++) corr[f][2] = mas_correction(prefact * kz, mas_p[f]);
                    /* kz=0 and kz=middle planes: keep one of each +-k pair */
                    if (kz == 0 || (kz == middle && dims % 2 == 0)) {
                        if (kx < 0) continue;
                        else if (kx == 0 || (kx == middle && dims % 2 == 0)) {
                            if (ky < 0) continue;
                        }
                    }
                    double k = sqrt((double)(kx * kx + ky * ky + kz * kz));
                    int k_index = (int)k;
                    int k_par, k_per;
                    if (axis == 0)      { k_par = kx; k_per = (int)sqrt((double)(ky * ky + kz * kz)); }
                    else if (axis == 1) { k_par = ky; k_per = (int)sqrt((double)(kx * kx + kz * kz)); }
                    else                { k_par = kz; k_per = (int)sqrt((double)(kx * kx + ky * ky)); }
                    double mu = k == 0 ? 0.0 : k_par / k;
                    double mu2 = mu * mu;
                    double val1 = (3.0 * mu2 - 1.0) / 2.0;
                    double val2 = (35.0 * mu2 * mu2 - 30.0 * mu2 + 3.0) / 8.0;
                    if (k_par < 0) k_par = -k_par;
                    int index_2D = (kmax_par + 1) * k_per + k_par;

                    if (k <= middle) { tk1[k_par] += k_par; tn1[k_par] += 1.0; }
                    tn2[index_2D] += 1.0;
                    tk3[k_index] += k;
                    tn3[k_index] += 1.0;

                    int64_t off = ((int64_t)kxx * dims + kyy) * nz + kzz;
                    for (int f = 0; f < F; f++) {
                        float mf = (float)(corr[f][0] * corr[f][1] * corr[f][2]);
                        float *c = dk + 2 * (f * fstride + off);
                        c[0] = c[0] * mf;
                        c[1] = c[1] * mf;
                        re[f] = c[0];
                        im[f] = c[1];
                        double delta2 = re[f] * re[f] + im[f] * im[f];
                        double phase = atan2(re[f], sqrt(delta2));
                        if (k <= middle) tp1[(int64_t)k_par * F + f] += delta2;
                        tp2[(int64_t)index_2D * F + f] += delta2;
                        tp3[((int64_t)k_index * 3 + 0) * F + f] += delta2;
                        tp3[((int64_t)k_index * 3 + 1) * F + f] += delta2 * val1;
                        tp3[((int64_t)k_index * 3 + 2) * F + f] += delta2 * val2;
                        tph[(int64_t)k_index * F + f] += phase * phase;
                    }
                    int ix = 0;
                    for (int i = 0; i < F; i++)
                        for (int j = i + 1; j < F; j++, ix++) {
                            double d2x = re[i] * re[j] + im[i] * im[j];
                            if (k <= middle) tx1[(int64_t)k_par * X + ix] += d2x;
                            tx2[(int64_t)index_2D * X + ix] += d2x;
                            tx3[((int64_t)k_index * 3 + 0) * X + ix] += d2x;
                            tx3[((int64_t)k_index * 3 + 1) * X + ix] += d2x * val1;
                            tx3[((int64_t)k_index * 3 + 2) * X + ix] += d2x * val2;
                        }
                }
            }
        }
    }
    /* sum the per-thread bins in thread order */
    for (int t = 0; t < threads; t++) {
        double *b = priv + per_thread * t;
        int64_t o = 0;
#define ACC(dst, len) do { for (int64_t q = 0; q < (int64_t)(len); q++) (dst)[q] += b[o + q]; o += (len); } while (0)
        ACC(k1D, nb1); ACC(Nmodes1D, nb1);
        ACC(Pk1D, (int64_t)nb1 * F); if (X) ACC(PkX1D, (int64_t)nb1 * X); else o += 0;
        ACC(Nmodes2D, nb2);
        ACC(Pk2D, (int64_t)nb2 * F); if (X) ACC(PkX2D, (int64_t)nb2 * X);
        ACC(k3D, nb3); ACC(Nmodes3D, nb3);
        ACC(Pk3D, (int64_t)nb3 * 3 * F); if (X) ACC(PkX3D, (int64_t)nb3 * 3 * X);
        ACC(Pkphase, (int64_t)nb3 * F);
#undef ACC
    }
    free(priv);
    return 0;
}

int oracle_max_fields(void) { return 64; }
