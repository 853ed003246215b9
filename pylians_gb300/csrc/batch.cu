// Batched realizations: one persistent launch deposits a whole batch of
// particle sets with uneven particle counts, grid sizes, MAS and interlacing.
//
// Work is a device list of items (realization, first particle, count); the
// CTAs of the persistent kernel take items from a device counter until the
// list is exhausted, so long and short realizations balance across SMs.  Each
// item deposits its particles with red.global.add into its realization's
// grid(s) (grids of <= 256^3 cells stay resident in L2 while their items run),
// scaled by dims^3 / N so that grids pre-filled with -1 end as the overdensity
// delta = n/mean - 1 (library/Pk_library/Pk_snapshot.py:70-88).  The per-particle
// arithmetic is the one of mas.cu (MAS_library.pyx:123-545).
#include <cuda_runtime.h>

#include "common.cuh"

namespace pyl {
namespace {

__device__ __forceinline__ float ba_dist(float p, float inv) { return __fmul_rn(p, inv); }

// Support of one coordinate (same arithmetic as mas.cu axis_weights).
template <int MAS>
__device__ __forceinline__ int ba_weights(float p, float inv, float *C)
{
    const float dist = ba_dist(p, inv);
    if (MAS == PYL_MAS_NGP) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        int k = __float2int_rz(fl) + (frac >= 0.5f ? 1 : 0);
        if (dist < -0.5f && frac != 0.5f) k += 1;
        C[0] = 1.0f;
        return k;
    } else if (MAS == PYL_MAS_CIC) {
        const float t = truncf(dist);
        const float u = __fsub_rn(dist, t);
        C[0] = __fsub_rn(1.0f, u);
        C[1] = u;
        return __float2int_rz(t);
    } else if (MAS == PYL_MAS_TSC) {
        const float fl = floorf(dist);
        const float frac = __fsub_rn(dist, fl);
        const float fmn = __fsub_rn(__fadd_rn(fl, frac >= 0.5f ? 1.0f : 0.0f), 2.0f);
#pragma unroll
        for (int j = 0; j < 3; j++) {
            const float diff = fabsf(__fsub_rn(__fadd_rn(fmn, (float)(j + 1)), dist));
            float c;
            if (diff < 0.5f) c = __fsub_rn(0.75f, __fmul_rn(diff, diff));
            else if (diff < 1.5f) { const float t = __fsub_rn(1.5f, diff); c = __fmul_rn(__fmul_rn(0.5f, t), t); }
            else c = 0.0f;
            C[j] = c;
        }
        return __float2int_rz(fl) - 1 + (frac >= 0.5f ? 1 : 0);
    } else {
        const float fl = floorf(dist);
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
            } else c = 0.0f;
            C[j] = c;
        }
        return __float2int_rz(fl) - 1;
    }
}

template <int MAS>
__device__ __forceinline__ void ba_deposit(const float *p, const pyl_batch_real &r, float shift, float *out)
{
    constexpr int S = MAS == PYL_MAS_NGP ? 1 : MAS;
    const int dims = r.dims;
    const long long d = dims;
    float C[3][S];
    int idx[3][S];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const int f = ba_weights<MAS>(__fadd_rn(p[a], shift), r.inv, C[a]);
#pragma unroll
        for (int j = 0; j < S; j++) idx[a][j] = wrap_index((long long)f + j, dims);
    }
#pragma unroll
    for (int l = 0; l < S; l++)
#pragma unroll
        for (int m = 0; m < S; m++) {
            const float c01 = __fmul_rn(C[0][l], C[1][m]);
            const long long row = ((long long)idx[0][l] * d + idx[1][m]) * d;
#pragma unroll
            for (int q = 0; q < S; q++)
                atomicAdd(out + row + idx[2][q], __fmul_rn(__fmul_rn(c01, C[2][q]), r.scale));
        }
}

__global__ void __launch_bounds__(256) batch_deposit_kernel(const pyl_batch_real *__restrict__ reals,
                                                            const pyl_batch_item *__restrict__ items,
                                                            int n_items, unsigned *counter)
{
    __shared__ int cur;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int it = cur;
        __syncthreads();
        if (it >= n_items) break;
        const pyl_batch_item item = items[it];
        const pyl_batch_real r = reals[item.real];
        for (long long i = item.first + threadIdx.x; i < item.first + item.count; i += blockDim.x) {
            const float p[3] = {__ldg(r.pos + 3 * i), __ldg(r.pos + 3 * i + 1), __ldg(r.pos + 3 * i + 2)};
            for (int g = 0; g < (r.grid_interlaced ? 2 : 1); g++) {
                float *out = g ? r.grid_interlaced : r.grid;
                const float sh = g ? r.halfcell : 0.0f;
                switch (r.mas) {
                    case PYL_MAS_NGP: ba_deposit<PYL_MAS_NGP>(p, r, sh, out); break;
                    case PYL_MAS_CIC: ba_deposit<PYL_MAS_CIC>(p, r, sh, out); break;
                    case PYL_MAS_TSC: ba_deposit<PYL_MAS_TSC>(p, r, sh, out); break;
                    default:          ba_deposit<PYL_MAS_PCS>(p, r, sh, out); break;
                }
            }
        }
    }
}

__global__ void __launch_bounds__(256) fill_value_kernel(float *g, long long n, float v)
{
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) g[i] = v;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

extern "C" int pyl_ma_batch(const pyl_batch_real *reals, int n_reals, const pyl_batch_item *items,
                            int n_items, unsigned *counter, int ctas_per_sm, void *stream)
{
    PYL_CHECK_ARG(reals != nullptr && items != nullptr && counter != nullptr, "null pointer");
    PYL_CHECK_ARG(n_reals >= 1 && n_items >= 0, "bad sizes");
    PYL_CHECK_ARG(ctas_per_sm >= 1 && ctas_per_sm <= 8, "ctas_per_sm must be 1..8");
    cudaStream_t st = (cudaStream_t)stream;
    PYL_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    if (n_items == 0) return PYL_OK;
    batch_deposit_kernel<<<num_sms() * ctas_per_sm, 256, 0, st>>>(reals, items, n_items, counter);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}

extern "C" int pyl_fill(float *p, int64_t n, float value, void *stream)
{
    PYL_CHECK_ARG(p != nullptr && n >= 0, "bad arguments");
    if (n == 0) return PYL_OK;
    long long b = (n + 255) / 256;
    if (b > (long long)num_sms() * 8) b = (long long)num_sms() * 8;
    fill_value_kernel<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(p, n, value);
    PYL_LAUNCH_CHECK();
    return PYL_OK;
}
