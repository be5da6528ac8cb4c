// ubs_common.cuh -- shared device/host helpers of the GB300 rasteriser library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/ubs.h"

namespace ubs {

// ------------------------------------------------------------- error state
// The last error message of the calling host thread (read by ubs_last_error).
int set_error(int code, const char *fmt, ...);
int check_launch(const char *what);
// Counts kernel launches made by this library (read with ubs_launch_count).
void note_launch(int n = 1);

// Opt-in kernel timing (ubs_profile_start / _stop): while enabled, a
// KernelTimer records a CUDA event before its launch and one after it, on the
// launching stream; otherwise it does nothing.
struct KernelTimer {
    int slot;
    cudaStream_t st;
    KernelTimer(const char *name, cudaStream_t s);
    ~KernelTimer();
};

// Launch statement(s) timed as one kernel under `name` when timing is enabled.
#define UBS_TIMED(name, st, ...)                                                \
    do {                                                                        \
        ::ubs::KernelTimer ubs_kt_(name, st);                                   \
        __VA_ARGS__;                                                            \
    } while (0)

#define UBS_REQUIRE(cond, ...)                                                  \
    do {                                                                        \
        if (!(cond)) return ::ubs::set_error(UBS_ERR_INVALID, __VA_ARGS__);     \
    } while (0)

inline unsigned grid_for(int64_t n, int block) {
    return (unsigned)((n + block - 1) / block);
}

// Device-side status word: kernels OR error bits into it instead of trapping.
enum DeviceError : uint32_t {
    DEV_ERR_WAIT_TIMEOUT = 1u,   // an mbarrier wait ran out of iterations
    DEV_ERR_NEG_DEPTH = 2u,      // a visible primitive had a negative depth key
    DEV_ERR_OVERFLOW = 4u,       // an intersection buffer was too small
};

// ------------------------------------------------------- small device math
__device__ __forceinline__ float clamp01_eps(float x) {
    const float maxv = 1.0f - 1.1920928955078125e-07f; // 1 - FLT_EPSILON
    x = x < 0.0f ? 0.0f : x;
    return x > maxv ? maxv : x;
}

// ------------------------------------------ scene activation sections
// Float offsets of the activated-parameter sections of the fused scene
// workspace: scales [N, D] at 0, betas [N, D - 2] and opacities [N] each on a
// 16-byte boundary, so that the activation pass writes every section with
// 16-byte stores whatever N is.
__host__ __device__ inline int64_t act_beta_off(int64_t N, int D) {
    return (N * D + 3) & ~int64_t(3);
}
__host__ __device__ inline int64_t act_opac_off(int64_t N, int D) {
    return act_beta_off(N, D) + ((N * (D - 2) + 3) & ~int64_t(3));
}

// ------------------------------------------ mbarrier + bulk async copy (TMA)
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}
// Bulk (non-tensor) async copy global -> shared, completion on the mbarrier.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes,
                                         uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: gives up after max_iters polls and reports false.  try_wait
// itself suspends for a hardware-defined interval, so the bound is generous.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint32_t max_iters = (1u << 22)) {
    for (uint32_t i = 0; i < max_iters; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// -------------------------------------------------- warp transpose-reduce
// Generalised transpose reduction of S = 2^m values (1 <= S <= 32) over the 32
// lanes: m halving steps (each lane keeps half of its slots and adds its
// partner's other half) then 5 - m plain butterfly steps.  Lane L returns the
// warp total of value tr_index<S>(L): the 32 / S lanes that differ from L only
// in their low 5 - m bits hold the same total, and lanes with L % (32 / S) == 0
// hold each value exactly once.
template <int S> __device__ __forceinline__ int tr_index(int lane) {
    return (int)((unsigned)lane / (32u / S)); // lane bits 4 .. 5 - log2 S
}
// Lane-bit masks of the transpose reductions: m[j] is all ones when bit
// 4 - j of the lane index is set.  Each exchange of tr_reduce picks the value
// to send and the one to keep with bitwise selects on these masks, which
// needs no predicate registers.
struct LaneMasks {
    uint32_t m[5];
};
__device__ __forceinline__ LaneMasks lane_masks(int lane) {
    LaneMasks l;
#pragma unroll
    for (int j = 0; j < 5; ++j) l.m[j] = (lane & (16 >> j)) ? ~0u : 0u;
    return l;
}
template <int S> __device__ __forceinline__ float tr_reduce(float (&v)[S], const LaneMasks &lm) {
    const unsigned full = 0xffffffffu;
    int n = S, h = 16;
#pragma unroll
    for (int step = 0; step < 5; ++step) {
        if (n > 1) {
            const uint32_t m = lm.m[step];
#pragma unroll
            for (int i = 0; i < S / 2; ++i) {
                if (i < n / 2) {
                    const uint32_t a = __float_as_uint(v[i]), b = __float_as_uint(v[i + n / 2]);
                    const float send = __uint_as_float((a & m) | (b & ~m));
                    const float keep = __uint_as_float((b & m) | (a & ~m));
                    v[i] = keep + __shfl_xor_sync(full, send, h);
                }
            }
            n >>= 1;
        } else {
            v[0] += __shfl_xor_sync(full, v[0], h);
        }
        h >>= 1;
    }
    return v[0];
}

} // namespace ubs
