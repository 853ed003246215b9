// Mode-grid helpers shared by the P(k) kernels (Pk_library.pyx:59-102,311-381).
#pragma once
#include "common.cuh"

namespace pyl {

struct PkDims {
    int dims, middle, nz, kmax_par, kmax_per, kmax, nb1, nb2, nb3;
};

// frequencies() (Pk_library.pyx:59-64) in bins: kmax_par = N/2,
// kmax_per = int(sqrt(2) N/2), kmax = int(sqrt(3) N/2).
static inline PkDims pk_dims(int dims)
{
    PkDims d;
    d.dims = dims;
    d.middle = dims / 2;
    d.nz = dims / 2 + 1;
    d.kmax_par = d.middle;
    d.kmax_per = (int)sqrt((double)d.middle * d.middle * 2.0);
    d.kmax = (int)sqrt((double)d.middle * d.middle * 3.0);
    d.nb1 = d.kmax_par + 1;
    d.nb2 = (d.kmax_par + 1) * (d.kmax_per + 1);
    d.nb3 = d.kmax + 1;
    return d;
}

// kz=0 and kz=middle planes keep one mode of each +-k pair (Pk_library.pyx:327-330).
__device__ __forceinline__ bool hermitian_skip(int kx, int ky, int kz, const PkDims &d)
{
    const bool even = (d.dims & 1) == 0;
    if (kz == 0 || (kz == d.middle && even)) {
        if (kx < 0) return true;
        if (kx == 0 || (kx == d.middle && even)) return ky < 0;
    }
    return false;
}

// (x / sin x)^p with x = pi k / dims, C(0) = 1, in float64 (Pk_library.pyx:86-87).
__device__ __forceinline__ double mas_corr_d(int k, int dims, int p)
{
    if (k == 0 || p == 0) return 1.0;
    const double x = (M_PI / dims) * k;
    const double r = x / sin(x);
    double v = 1.0;
    for (int i = 0; i < p; i++) v *= r;
    return v;
}

// Same in float32: (x / sin x)^p, x = pi t, t = k / dims (sinpif needs no
// large-argument reduction, so no local-memory path).
__device__ __forceinline__ float mas_corr_f(int k, int dims, int p)
{
    if (k == 0 || p == 0) return 1.0f;
    const float t = (float)k / (float)dims;
    const float r = ((float)M_PI * t) / sinpif(t);
    float v = 1.0f;
    for (int i = 0; i < p; i++) v *= r;
    return v;
}

}  // namespace pyl
