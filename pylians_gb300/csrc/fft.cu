// cuFFT plan cache: the single-precision 3D R2C / C2R transforms that replace
// pyFFTW's FFT3Dr_f / IFFT3Dr_f (library/Pk_library/Pk_library.pyx:120-133,
// 152-165).  Both are unnormalised, like FFTW's.  cuFFT is the only library
// call on the path.  Plans (and the workspaces cuFFT allocates for them) are
// cached per (device, dims, batch, direction) and live until pyl_fft_cache_clear.
#include <cufft.h>

#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"

namespace pyl {
namespace {

struct PlanKey {
    int device, dims, batch, dir, rank;
    bool operator<(const PlanKey &o) const
    {
        return std::tie(device, dims, batch, dir, rank) < std::tie(o.device, o.dims, o.batch, o.dir, o.rank);
    }
};

std::mutex g_mu;
std::map<PlanKey, cufftHandle> g_plans;

const char *cufft_name(cufftResult r)
{
    switch (r) {
        case CUFFT_SUCCESS: return "CUFFT_SUCCESS";
        case CUFFT_INVALID_PLAN: return "CUFFT_INVALID_PLAN";
        case CUFFT_ALLOC_FAILED: return "CUFFT_ALLOC_FAILED";
        case CUFFT_INVALID_VALUE: return "CUFFT_INVALID_VALUE";
        case CUFFT_INTERNAL_ERROR: return "CUFFT_INTERNAL_ERROR";
        case CUFFT_EXEC_FAILED: return "CUFFT_EXEC_FAILED";
        case CUFFT_SETUP_FAILED: return "CUFFT_SETUP_FAILED";
        case CUFFT_INVALID_SIZE: return "CUFFT_INVALID_SIZE";
        default: return "cuFFT error";
    }
}

#define PYL_CUFFT(call)                                                                 \
    do {                                                                                \
        cufftResult r_ = (call);                                                        \
        if (r_ != CUFFT_SUCCESS) {                                                      \
            ::pyl::set_error(std::string(__func__) + ": " + #call + " -> " + cufft_name(r_)); \
            return PYL_ERR_CUFFT;                                                       \
        }                                                                               \
    } while (0)

// Returns a plan for `batch` contiguous dims^rank transforms, rank 2 or 3
// (caller holds g_mu).
int get_plan(int dims, int batch, int dir, cufftHandle *out, int rank = 3)
{
    int dev = 0;
    PYL_CUDA(cudaGetDevice(&dev));
    PlanKey k{dev, dims, batch, dir, rank};
    auto it = g_plans.find(k);
    if (it != g_plans.end()) { *out = it->second; return PYL_OK; }
    cufftHandle h;
    PYL_CUFFT(cufftCreate(&h));
    long long n[3] = {dims, dims, dims};
    const long long real_dist = rank == 3 ? (long long)dims * dims * dims : (long long)dims * dims;
    const long long cplx_dist = (rank == 3 ? (long long)dims * dims : (long long)dims) * (dims / 2 + 1);
    size_t ws = 0;
    cufftResult r;
    if (dir == CUFFT_R2C)
        r = cufftMakePlanMany64(h, rank, n, nullptr, 1, real_dist, nullptr, 1, cplx_dist, CUFFT_R2C, batch, &ws);
    else
        r = cufftMakePlanMany64(h, rank, n, nullptr, 1, cplx_dist, nullptr, 1, real_dist, CUFFT_C2R, batch, &ws);
    if (r != CUFFT_SUCCESS) {
        cufftDestroy(h);
        set_error(std::string("cufftMakePlanMany64 -> ") + cufft_name(r));
        return PYL_ERR_CUFFT;
    }
    g_plans[k] = h;
    *out = h;
    return PYL_OK;
}

}  // namespace
}  // namespace pyl

using namespace pyl;

// At 1024^3 and above, cuFFT runs a batch of R2C transforms as one batch-1
// transform after another faster than as one batched plan (10.8 ms vs 13.3 ms for
// two 1024^3 grids on GB300), so large batches are split.
constexpr int SPLIT_BATCH_DIMS = 1024;

extern "C" int pyl_fft_r2c(const float *in, void *out_c64, int dims, int batch, void *stream)
{
    PYL_CHECK_ARG(in != nullptr && out_c64 != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && batch >= 1, "bad size");
    std::lock_guard<std::mutex> lk(g_mu);
    cufftHandle h;
    const bool split = batch > 1 && dims >= SPLIT_BATCH_DIMS;
    int rc = get_plan(dims, split ? 1 : batch, CUFFT_R2C, &h);
    if (rc) return rc;
    PYL_CUFFT(cufftSetStream(h, (cudaStream_t)stream));
    if (!split) {
        PYL_CUFFT(cufftExecR2C(h, (cufftReal *)in, (cufftComplex *)out_c64));
        return PYL_OK;
    }
    const long long real_dist = (long long)dims * dims * dims;
    const long long cplx_dist = (long long)dims * dims * (dims / 2 + 1);
    for (int b = 0; b < batch; b++)
        PYL_CUFFT(cufftExecR2C(h, (cufftReal *)(in + b * real_dist), (cufftComplex *)out_c64 + b * cplx_dist));
    return PYL_OK;
}

extern "C" int pyl_fft_c2r(void *in_c64, float *out, int dims, int batch, void *stream)
{
    PYL_CHECK_ARG(in_c64 != nullptr && out != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && batch >= 1, "bad size");
    std::lock_guard<std::mutex> lk(g_mu);
    cufftHandle h;
    int rc = get_plan(dims, batch, CUFFT_C2R, &h);
    if (rc) return rc;
    PYL_CUFFT(cufftSetStream(h, (cudaStream_t)stream));
    PYL_CUFFT(cufftExecC2R(h, (cufftComplex *)in_c64, (cufftReal *)out));
    return PYL_OK;
}

extern "C" int pyl_fft2_r2c(const float *in, void *out_c64, int dims, int batch, void *stream)
{
    PYL_CHECK_ARG(in != nullptr && out_c64 != nullptr, "null pointer");
    PYL_CHECK_ARG(dims >= 2 && batch >= 1, "bad size");
    std::lock_guard<std::mutex> lk(g_mu);
    cufftHandle h;
    int rc = get_plan(dims, batch, CUFFT_R2C, &h, 2);
    if (rc) return rc;
    PYL_CUFFT(cufftSetStream(h, (cudaStream_t)stream));
    PYL_CUFFT(cufftExecR2C(h, (cufftReal *)in, (cufftComplex *)out_c64));
    return PYL_OK;
}

extern "C" int pyl_fft_cache_clear(void)
{
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto &kv : g_plans) cufftDestroy(kv.second);
    g_plans.clear();
    return PYL_OK;
}
