// Status strings, last-error detail and version of the C-ABI.
#include <string>

#include "common.cuh"

namespace pyl {
namespace {
thread_local std::string g_last_error;
}
void set_error(const std::string &msg) { g_last_error = msg; }
}  // namespace pyl

extern "C" const char *pyl_strerror(int status)
{
    switch (status) {
        case PYL_OK: return "success";
        case PYL_ERR_INVALID: return "invalid argument";
        case PYL_ERR_CUDA: return "CUDA error";
        case PYL_ERR_CUFFT: return "cuFFT error";
        case PYL_ERR_WORKSPACE: return "workspace too small";
        case PYL_ERR_UNSUPPORTED: return "unsupported request";
        default: return "unknown status";
    }
}

extern "C" const char *pyl_last_error(void) { return pyl::g_last_error.c_str(); }

extern "C" int pyl_version(void) { return 100; }

// ---- optional per-phase timing of the mass-assignment launches ----------------
// Off by default.  When enabled, the deposit paths bracket each phase with CUDA
// events on the launching stream; pyl_stage_times sums the elapsed times per
// phase since the last read (after synchronizing those events) and clears them.
#include <mutex>
#include <vector>

namespace pyl {
namespace {
struct StageRec {
    int phase;
    cudaEvent_t a, b;
};
std::mutex g_stage_mu;
bool g_stage_on = false;
std::vector<StageRec> g_stage_recs;
std::vector<cudaEvent_t> g_event_pool;
thread_local cudaEvent_t g_open[PYL_STAGE_COUNT] = {};

cudaEvent_t take_event()
{
    if (!g_event_pool.empty()) {
        cudaEvent_t e = g_event_pool.back();
        g_event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
}
}  // namespace

void stage_mark(int phase, bool begin, cudaStream_t st)
{
    if (phase < 0 || phase >= PYL_STAGE_COUNT) return;
    std::lock_guard<std::mutex> lk(g_stage_mu);
    if (!g_stage_on) return;
    cudaEvent_t e = take_event();
    if (!e) return;
    cudaEventRecord(e, st);
    if (begin) {
        if (g_open[phase]) g_event_pool.push_back(g_open[phase]);
        g_open[phase] = e;
    } else if (g_open[phase]) {
        g_stage_recs.push_back(StageRec{phase, g_open[phase], e});
        g_open[phase] = nullptr;
    } else {
        g_event_pool.push_back(e);
    }
}
}  // namespace pyl

#include <map>
#include <utility>

namespace pyl {
namespace {
std::mutex g_smem_mu;
std::map<std::pair<int, const void *>, size_t> g_smem_limits;
std::mutex g_sm_mu;
std::map<int, int> g_sm_count;
}  // namespace

int num_sms()
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_sm_mu);
    auto it = g_sm_count.find(dev);
    if (it != g_sm_count.end()) return it->second;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
        cudaGetLastError();     // no device (host-side size queries): the GB300's count
        n = 152;
    }
    g_sm_count[dev] = n;
    return n;
}

size_t smem_limit_raise(const void *kernel, size_t bytes, cudaError_t *err)
{
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_smem_mu);
    size_t &cur = g_smem_limits[std::make_pair(dev, kernel)];
    if (bytes > cur) {
        *err = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
        if (*err != cudaSuccess) return cur;
        cur = bytes;
    }
    return cur;
}
}  // namespace pyl

extern "C" int pyl_stage_timing(int enable)
{
    std::lock_guard<std::mutex> lk(pyl::g_stage_mu);
    pyl::g_stage_on = enable != 0;
    return PYL_OK;
}

extern "C" int pyl_stage_times(double *ms_out, int n)
{
    PYL_CHECK_ARG(ms_out != nullptr && n >= 0, "bad arguments");
    std::lock_guard<std::mutex> lk(pyl::g_stage_mu);
    for (int i = 0; i < n; i++) ms_out[i] = 0.0;
    for (const auto &r : pyl::g_stage_recs) {
        PYL_CUDA(cudaEventSynchronize(r.b));
        float ms = 0.0f;
        PYL_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
        if (r.phase < n) ms_out[r.phase] += ms;
        pyl::g_event_pool.push_back(r.a);
        pyl::g_event_pool.push_back(r.b);
    }
    pyl::g_stage_recs.clear();
    return PYL_OK;
}
