// Per-particle mass-assignment arithmetic shared by the deposit kernels
// (mas.cu, batch.cu): first cells and weights of NGP/CIC/TSC/PCS along one axis
// (MAS_library.pyx:123-545), and the per-bin 10.22 fixed-point shared-memory
// accumulation of the tiled and batched deposits.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

// Bin side of the tiled deposits (cells).
constexpr int TB = 32;

template <int MAS>
struct Support { static constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS; };

// First cell (unwrapped) of the support of one particle coordinate.  Cell
// arithmetic is 32-bit (float->int64 conversions run on the slow fp64 pipe):
// coordinates must satisfy |x * dims / BoxSize| < 2^31; beyond that the
// conversion saturates and the cell still wraps into the grid.
template <int MAS>
__device__ __forceinline__ int axis_first(float p, float inv)
{
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_CIC) return __float2int_rz(dist);
    const float fl = floorf(dist);
    const float frac = __fsub_rn(dist, fl);
    const int fi = __float2int_rz(fl);
    if (MAS == PYL_MAS_NGP) {
        int k = fi + (frac >= 0.5f ? 1 : 0);              // floor(dist + 0.5)
        if (dist < -0.5f && frac != 0.5f) k += 1;         // trunc for negative sums
        return k;
    }
    if (MAS == PYL_MAS_TSC) return fi - 1 + (frac >= 0.5f ? 1 : 0);
    return fi - 1;                                        // PCS
}

// Per-axis support of one particle coordinate: first cell f (unwrapped) and the
// S weights of cells f, f+1, ..., f+S-1.  f equals axis_first<MAS>(p, inv).
template <int MAS>
__device__ __forceinline__ int axis_weights(float p, float inv, float *C)
{
    const float dist = __fmul_rn(p, inv);
    if (MAS == PYL_MAS_NGP) {
        C[0] = 1.0f;
        return axis_first<MAS>(p, inv);
    } else if (MAS == PYL_MAS_CIC) {
        // <int>dist truncates toward zero; u = dist - <int>dist, d = 1 - u
        const float t = truncf(dist);
        const float u = __fsub_rn(dist, t);
        C[0] = __fsub_rn(1.0f, u);
        C[1] = u;
        return __float2int_rz(t);
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        const int mn = __float2int_rz(fl) - 2 + (frac >= 0.5f ? 1 : 0);  // floor(dist - 1.5)
        const float fmn = __fsub_rn(__fadd_rn(fl, frac >= 0.5f ? 1.0f : 0.0f), 2.0f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float diff = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
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
        const float fl = floorf(dist);
        const int mn = __float2int_rz(fl) - 2;            // floor(dist - 2)
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
            } else {
                c = 0.0f;
            }
            C[j] = c;
        }
        return mn + 1;
    }
}

// ---- per-bin fixed-point accumulation -------------------------------------------
template <int MAS, bool INTER>
struct FxShape {
    static constexpr int H = Support<MAS>::S - 1 + (INTER ? 1 : 0);
    static constexpr int E = TB + H;
    static constexpr int CELLS = E * E * E;
    static constexpr size_t SMEM = sizeof(unsigned) * ((CELLS + 3) / 4 * 4);
    static constexpr bool FITS = SMEM <= 227 * 1024;
};

constexpr float FX_MAGIC = 12582912.0f;        // 1.5 * 2^23
constexpr unsigned FX_MAGIC_BITS = 0x4B400000u;
constexpr float FX_SCALE = 4194304.0f;         // 2^22
constexpr float FX_INV = 2.384185791015625e-07f;

// Weights and bin-local first cell (base, row-major over E^3) of one particle
// for the plain (G=0) or the half-cell-shifted (G=1) grid.
template <int MAS, int G, int E>
__device__ __forceinline__ int fx_support(const float4 &r, float inv, float halfcell, int dims, const int *o,
                                          float (*C)[Support<MAS>::S])
{
    const float p[3] = {r.x, r.y, r.z};
    int base = 0;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        int loc;
        if (G == 1) {
            const int f0 = axis_first<MAS>(p[a], inv);
            const int f = axis_weights<MAS>(__fadd_rn(p[a], halfcell), inv, C[a]);
            loc = wrap_index(f0, dims) - o[a] + (f > f0 ? 1 : 0);
        } else {
            loc = wrap_index(axis_weights<MAS>(p[a], inv, C[a]), dims) - o[a];
        }
        base = base * E + loc;
    }
    return base;
}

template <int MAS, int E>
__device__ __forceinline__ void float_scatter(float *acc, int base, const float (*C)[Support<MAS>::S])
{
    constexpr int S = Support<MAS>::S;
#pragma unroll
    for (int l = 0; l < S; l++)
#pragma unroll
        for (int m = 0; m < S; m++) {
            const float c01 = __fmul_rn(C[0][l], C[1][m]);
            const int row = base + (l * E + m) * E;
#pragma unroll
            for (int q = 0; q < S; q++) atomicAdd(acc + row + q, __fmul_rn(c01, C[2][q]));
        }
}

// Fixed-point value of one corner: the product c01 * c2 as a 10.22 number.  PRE:
// c2 already carries the factor 2^22 (one FFMA, one rounding of the exact
// product); otherwise the float product is rounded first, then scaled.
template <bool PRE>
__device__ __forceinline__ unsigned fx_corner(float c01, float c2)
{
    const float x = PRE ? __fmaf_rn(c01, c2, FX_MAGIC) : __fmaf_rn(__fmul_rn(c01, c2), FX_SCALE, FX_MAGIC);
    return __float_as_uint(x) - FX_MAGIC_BITS;
}

// Adds the S^3 fixed-point corner weights without reading the old values back
// (wraps are then found from the bin's total, see fx_accumulate).
template <int MAS, int E, bool PRE = false>
__device__ __forceinline__ void fx_scatter_add(unsigned *acc, int base, const float (*C)[Support<MAS>::S])
{
    constexpr int S = Support<MAS>::S;
#pragma unroll
    for (int l = 0; l < S; l++)
#pragma unroll
        for (int m = 0; m < S; m++) {
            const float c01 = __fmul_rn(C[0][l], C[1][m]);
            const int row = base + (l * E + m) * E;
#pragma unroll
            for (int q = 0; q < S; q++) atomicAdd(acc + row + q, fx_corner<PRE>(c01, C[2][q]));
        }
}

// COUNT: unweighted NGP adds one integer count per particle; otherwise every
// corner adds its fixed-point weight (weighted NGP: C holds the scaled weight).
// PRE: C[2] carries the factor 2^22 (see fx_corner).
template <int MAS, int E, bool COUNT = (MAS == PYL_MAS_NGP), bool PRE = false>
__device__ __forceinline__ unsigned fx_scatter_or(unsigned *acc, int base, const float (*C)[Support<MAS>::S])
{
    constexpr int S = Support<MAS>::S;
    if (COUNT) {
        atomicAdd(acc + base, 1u);
        return 0u;
    }
    unsigned seen = 0u;
#pragma unroll
    for (int l = 0; l < S; l++)
#pragma unroll
        for (int m = 0; m < S; m++) {
            const float c01 = __fmul_rn(C[0][l], C[1][m]);
            const int row = base + (l * E + m) * E;
#pragma unroll
            for (int q = 0; q < S; q++) seen |= atomicAdd(acc + row + q, fx_corner<PRE>(c01, C[2][q]));
        }
    return seen;
}

}  // namespace
}  // namespace pyl
