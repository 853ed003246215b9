// Shared helpers for the sm_103a kernels of the density-field / clustering path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "../../include/pylians_gb300.h"

namespace pyl {

// Thread-local detail message behind the status codes returned by the C-ABI.
void set_error(const std::string &msg);
// Records a CUDA event opening (begin) or closing a timed phase (PYL_STAGE_*)
// when pyl_stage_timing is on; a no-op otherwise.
void stage_mark(int phase, bool begin, cudaStream_t st);

#define PYL_CHECK_ARG(cond, msg)                                 \
    do {                                                         \
        if (!(cond)) {                                           \
            ::pyl::set_error(std::string(__func__) + ": " + msg); \
            return PYL_ERR_INVALID;                              \
        }                                                        \
    } while (0)

#define PYL_CUDA(call)                                                               \
    do {                                                                             \
        cudaError_t e_ = (call);                                                     \
        if (e_ != cudaSuccess) {                                                     \
            ::pyl::set_error(std::string(__func__) + ": " + cudaGetErrorString(e_)); \
            return PYL_ERR_CUDA;                                                     \
        }                                                                            \
    } while (0)

#define PYL_LAUNCH_CHECK() PYL_CUDA(cudaGetLastError())

// Multiprocessor count of the current device, looked up once per device under a
// lock (workspace layouts and grid sizes follow the device a call runs on).
int num_sms();

// Non-negative modulo: the cell index of any integer on a periodic axis.  The
// 64-bit division only runs for indices more than one period outside [0, n).
__device__ __forceinline__ int wrap_index(long long i, int n)
{
    if ((unsigned long long)i < (unsigned long long)n) return (int)i;
    if (i >= n && i < 2LL * n) return (int)(i - n);
    if (i < 0 && i >= -(long long)n) return (int)(i + n);
    long long r = i % n;
    return (int)(r < 0 ? r + n : r);
}

// (a + b) mod n for 0 <= a < n and 0 <= b (b usually < n).
__device__ __forceinline__ long long add_wrap(long long a, long long b, long long n)
{
    long long s = a + b;
    if (s >= n) s -= n;
    if (s >= n) s %= n;
    return s;
}

// Signed frequency of FFT index i on an axis of n points (Pk_library.pyx:315).
__device__ __host__ __forceinline__ int freq_of(int i, int n)
{
    return i > n / 2 ? i - n : i;
}

// Exact floor(sqrt(v)) for 0 <= v < 2^31.
__device__ __forceinline__ int isqrt_exact(int v)
{
    int r = (int)sqrtf((float)v);
    while (r * r > v) --r;
    while ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

// Exact floor(sqrt(v)) for 0 <= v < 2^26 from the hardware reciprocal square
// root (one correction step: its error is far below one unit).
__device__ __forceinline__ int isqrt_fast(int v)
{
    if (v <= 0) return 0;
    const float f = (float)v;
    int r = __float2int_rz(f * rsqrtf(f));
    if (r * r > v) --r;
    else if ((r + 1) * (r + 1) <= v) ++r;
    return r;
}

// atan(x) for |x| <= 1: x * P(x^2) with P of degree 7, a least-squares fit of
// atan(x)/x on [0, 1] made for this library (max error 1.3e-7 in float32).
__device__ __forceinline__ float atan_unit(float x)
{
    const float t = x * x;
    float p = -0.004072933151371148f;
    p = fmaf(p, t, 0.021945309816161062f);
    p = fmaf(p, t, -0.05606139167571965f);
    p = fmaf(p, t, 0.09656133056527133f);
    p = fmaf(p, t, -0.13915757198865716f);
    p = fmaf(p, t, 0.1994850070866807f);
    p = fmaf(p, t, -0.33330106029508433f);
    p = fmaf(p, t, 0.9999994367069165f);
    return x * p;
}

// Raise a kernel's dynamic shared-memory limit once per size (kept out of the
// steady state so that launches can be captured in a CUDA graph).
// Raises a kernel's dynamic shared-memory limit to at least `bytes`.  The limit
// is a per-kernel attribute, so it only ever grows: one record per kernel and
// device (several launch sites of one kernel may ask for different sizes, and
// each device of a process keeps its own attribute).
size_t smem_limit_raise(const void *kernel, size_t bytes, cudaError_t *err);

template <typename K>
static inline cudaError_t ensure_smem(K kernel, size_t bytes)
{
    cudaError_t e = cudaSuccess;
    smem_limit_raise((const void *)kernel, bytes, &e);
    return e;
}

__device__ __forceinline__ void red_add(float *p, float v) { atomicAdd(p, v); }
__device__ __forceinline__ void red_add(double *p, double v) { atomicAdd(p, v); }

}  // namespace pyl
