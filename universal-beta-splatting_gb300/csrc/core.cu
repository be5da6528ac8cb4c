// core.cu -- error state and version of the C ABI.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "ubs_common.cuh"

namespace ubs {

static thread_local char g_last_error[512] = "";
static std::atomic<unsigned long long> g_launches{0};

void note_launch(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }

// FP32 issue-rate probe: 8 independent FMA chains per thread, `iters` rounds.
__global__ void fp32_probe_kernel(int iters, float *out) {
    float a0 = threadIdx.x * 1e-7f, a1 = a0 + 1e-7f, a2 = a0 + 2e-7f, a3 = a0 + 3e-7f;
    float a4 = a0 + 4e-7f, a5 = a0 + 5e-7f, a6 = a0 + 6e-7f, a7 = a0 + 7e-7f;
    const float m = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = fmaf(a0, m, c); a1 = fmaf(a1, m, c); a2 = fmaf(a2, m, c); a3 = fmaf(a3, m, c);
            a4 = fmaf(a4, m, c); a5 = fmaf(a5, m, c); a6 = fmaf(a6, m, c); a7 = fmaf(a7, m, c);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

// XU (MUFU) issue-rate probe: 8 independent chains of base-2 exponentials per
// thread (exp2f is one MUFU.EX2 under fast math); the chain values stay in
// (0, 1] so no special-case path runs.
__global__ void mufu_probe_kernel(int iters, float *out) {
    float a0 = -1e-3f * (threadIdx.x & 7), a1 = a0 - 0.01f, a2 = a0 - 0.02f, a3 = a0 - 0.03f;
    float a4 = a0 - 0.04f, a5 = a0 - 0.05f, a6 = a0 - 0.06f, a7 = a0 - 0.07f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 16; ++u) {
            a0 = -exp2f(a0); a1 = -exp2f(a1); a2 = -exp2f(a2); a3 = -exp2f(a3);
            a4 = -exp2f(a4); a5 = -exp2f(a5); a6 = -exp2f(a6); a7 = -exp2f(a7);
        }
    }
    out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

int set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

// Reports a failed launch or runtime call (sticky or not) as UBS_ERR_CUDA.
int check_launch(const char *what) {
    const cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) return UBS_OK;
    return set_error(UBS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

// ------------------------------------------------------------ kernel timing
namespace {
struct ProfSlot {
    const char *name;
    cudaEvent_t e0, e1;
    double acc_ms;   // accumulated by samples
    long long n;     // samples taken
};
struct ProfEntry {
    const char *name;
    long long launches;
    double ms;
};
std::mutex g_prof_mu;
std::vector<ProfSlot> g_prof_slots;
std::vector<ProfEntry> g_prof_result;
std::atomic<bool> g_prof_on{false};
std::atomic<int> g_prof_next{0};
} // namespace

// Inside stream capture the events become external event-record nodes of
// the graph, so every replay records them again (read with ubs_profile_sample).
static cudaError_t prof_record(cudaEvent_t e, cudaStream_t st) {
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) return cudaErrorUnknown;
    return cudaEventRecordWithFlags(
        e, st, cs == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault);
}

KernelTimer::KernelTimer(const char *name, cudaStream_t s) : slot(-1), st(s) {
    if (!g_prof_on.load(std::memory_order_acquire)) return;
    const int i = g_prof_next.fetch_add(1, std::memory_order_relaxed);
    if (i >= (int)g_prof_slots.size()) return; // pool exhausted: launch is not timed
    g_prof_slots[i].name = name;
    if (prof_record(g_prof_slots[i].e0, st) == cudaSuccess) slot = i;
}

KernelTimer::~KernelTimer() {
    if (slot >= 0 && prof_record(g_prof_slots[slot].e1, st) != cudaSuccess)
        g_prof_slots[slot].name = nullptr;
}

// Adds the current duration of every recorded event pair to its slot.
static int prof_sample_locked() {
    const int n = std::min<int>(g_prof_next.load(), (int)g_prof_slots.size());
    for (int i = 0; i < n; ++i) {
        ProfSlot &p = g_prof_slots[i];
        if (!p.name) continue;
        float ms = 0.f;
        if (cudaEventSynchronize(p.e1) != cudaSuccess) return check_launch("profile sample");
        const cudaError_t et = cudaEventElapsedTime(&ms, p.e0, p.e1);
        if (et == cudaErrorInvalidResourceHandle) {
            // a pair captured into a graph that has not been replayed yet:
            // never recorded, nothing to add
            cudaGetLastError();
            continue;
        }
        if (et != cudaSuccess) return check_launch("profile sample");
        p.acc_ms += ms;
        p.n += 1;
    }
    return UBS_OK;
}

static void prof_release() {
    for (auto &p : g_prof_slots) {
        cudaEventDestroy(p.e0);
        cudaEventDestroy(p.e1);
    }
    g_prof_slots.clear();
}

} // namespace ubs

extern "C" {

const char *ubs_last_error(void) { return ubs::g_last_error; }

int ubs_abi_version(void) { return 2; }

unsigned long long ubs_launch_count(void) { return ubs::g_launches.load(); }

size_t ubs_fp32_probe_workspace_bytes(void) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return 0;
    return (size_t)sms * 8 * 256 * sizeof(float);
}

int ubs_fp32_probe(int32_t iters, void *workspace, size_t workspace_bytes, double *flops,
                   void *stream) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ubs::check_launch("fp32_probe device query");
    const size_t need = (size_t)sms * 8 * 256 * sizeof(float);
    if (iters <= 0 || !workspace || workspace_bytes < need)
        return ubs::set_error(UBS_ERR_INVALID, "fp32_probe: need iters > 0 and %zu B", need);
    ubs::fp32_probe_kernel<<<sms * 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        iters, static_cast<float *>(workspace));
    ubs::note_launch();
    if (flops) *flops = 2.0 * 8 * 16 * (double)iters * sms * 8 * 256;
    return ubs::check_launch("fp32_probe");
}

int ubs_mufu_probe(int32_t iters, void *workspace, size_t workspace_bytes, double *ops,
                   void *stream) {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return ubs::check_launch("mufu_probe device query");
    const size_t need = (size_t)sms * 8 * 256 * sizeof(float);
    if (iters <= 0 || !workspace || workspace_bytes < need)
        return ubs::set_error(UBS_ERR_INVALID, "mufu_probe: need iters > 0 and %zu B", need);
    ubs::mufu_probe_kernel<<<sms * 8, 256, 0, static_cast<cudaStream_t>(stream)>>>(
        iters, static_cast<float *>(workspace));
    ubs::note_launch();
    if (ops) *ops = 8.0 * 16 * (double)iters * sms * 8 * 256;
    return ubs::check_launch("mufu_probe");
}

int ubs_profile_start(int32_t max_launches) {
    using namespace ubs;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (g_prof_on.load()) return set_error(UBS_ERR_INVALID, "profile_start: already running");
    if (max_launches < 1 || max_launches > (1 << 20))
        return set_error(UBS_ERR_INVALID, "profile_start: max_launches %d not in [1, 2^20]",
                         max_launches);
    if ((int)g_prof_slots.size() != max_launches) {
        prof_release();
        g_prof_slots.resize(max_launches);
        for (auto &p : g_prof_slots) {
            p.name = nullptr;
            p.acc_ms = 0.0;
            p.n = 0;
            if (cudaEventCreate(&p.e0) != cudaSuccess || cudaEventCreate(&p.e1) != cudaSuccess) {
                g_prof_slots.clear();
                return check_launch("profile_start event pool");
            }
        }
    }
    for (auto &p : g_prof_slots) {
        p.name = nullptr;
        p.acc_ms = 0.0;
        p.n = 0;
    }
    g_prof_result.clear();
    g_prof_next.store(0);
    g_prof_on.store(true, std::memory_order_release);
    return UBS_OK;
}

int ubs_profile_sample(void) {
    using namespace ubs;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    return prof_sample_locked();
}

int ubs_profile_stop(int32_t *n_kernels) {
    using namespace ubs;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (!g_prof_on.load()) return set_error(UBS_ERR_INVALID, "profile_stop: not running");
    g_prof_on.store(false, std::memory_order_release);
    const int n = std::min<int>(g_prof_next.load(), (int)g_prof_slots.size());
    bool sampled = false;
    for (int i = 0; i < n; ++i) sampled = sampled || g_prof_slots[i].n > 0;
    if (!sampled)
        if (int e = prof_sample_locked()) return e;
    for (int i = 0; i < n; ++i) {
        const ProfSlot &p = g_prof_slots[i];
        if (!p.name || p.n == 0) continue;
        ProfEntry *e = nullptr;
        for (auto &r : g_prof_result)
            if (std::strcmp(r.name, p.name) == 0) e = &r;
        if (!e) {
            g_prof_result.push_back({p.name, 0, 0.0});
            e = &g_prof_result.back();
        }
        e->launches += p.n;
        e->ms += p.acc_ms;
    }
    if (n_kernels) *n_kernels = (int32_t)g_prof_result.size();
    return UBS_OK;
}

int ubs_profile_result(int32_t i, const char **name, int64_t *launches, double *total_ms) {
    using namespace ubs;
    std::lock_guard<std::mutex> lk(g_prof_mu);
    if (i < 0 || i >= (int)g_prof_result.size())
        return set_error(UBS_ERR_INVALID, "profile_result: index %d out of range", i);
    if (name) *name = g_prof_result[i].name;
    if (launches) *launches = g_prof_result[i].launches;
    if (total_ms) *total_ms = g_prof_result[i].ms;
    return UBS_OK;
}

} // extern "C"
