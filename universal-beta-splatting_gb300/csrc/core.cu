// core.cu -- error state and version of the C ABI.
#include <atomic>
#include <cstdarg>
#include <cstdio>

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

} // extern "C"
