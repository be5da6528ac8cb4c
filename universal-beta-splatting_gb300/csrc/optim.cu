// optim.cu -- one-launch Adam step over all parameter tensors of a scene.
//
// The reference trains with torch.optim.Adam(param groups, eps=1e-15)
// (scene/beta_model.py:239-276, train.py:170-171), whose multi-tensor CUDA
// path runs about seven element-wise passes per step.  This kernel performs
// the same update in one pass over (param, grad, exp_avg, exp_avg_sq) with
// the same sequence of roundings (IEEE round-to-nearest intrinsics, so that
// fast-math compilation changes nothing):
//   exp_avg    <- lerp(exp_avg, grad, 1 - beta1)   = m + (1 - b1) (g - m)
//   exp_avg_sq <- exp_avg_sq * beta2 + (1 - beta2) (g g)
//   param      <- param + step_size * exp_avg / (sqrt(exp_avg_sq) / bc2 + eps)
// with step_size = -lr / (1 - beta1^t) and bc2 = sqrt(1 - beta2^t) of the
// tensor's group, read from a small device array so the launch can be
// captured in a CUDA graph while the host updates the array between replays.
#include "ubs_common.cuh"

namespace ubs {
namespace {

struct AdamTensor {
    float *p;
    const float *g;
    float *m;
    float *v;
    int64_t n;
    int32_t group;
    int32_t pad;
};

__device__ __forceinline__ void adam_one(float &p, float g, float &m, float &v, float c1,
                                         float b2, float c2, float step_size, float bc2,
                                         float eps) {
    m = __fmaf_rn(c1, __fsub_rn(g, m), m);
    v = __fmaf_rn(c2, __fmul_rn(g, g), __fmul_rn(v, b2));
    const float denom = __fadd_rn(__fdiv_rn(__fsqrt_rn(v), bc2), eps);
    p = __fmaf_rn(step_size, __fdiv_rn(m, denom), p);
}

// Flattened form (up to ADAM_FLAT_MAX tensors): the elements of all tensors
// are cut into chunks of ADAM_CHUNK quads (four elements), one block per
// chunk, so large and small tensors are spread evenly over the GPU; a block
// finds its tensor from the running chunk counts of the table.  16-byte
// accesses where all four arrays of a tensor are 16-byte aligned.
constexpr int ADAM_THREADS = 256;
constexpr int ADAM_QPT = 4;                         // quads per thread
constexpr int ADAM_CHUNK = ADAM_THREADS * ADAM_QPT; // quads per block
constexpr int ADAM_FLAT_MAX = 64;

__device__ __forceinline__ void adam_quad(const AdamTensor &t, int64_t q, bool vec, float c1,
                                          float b2, float c2, float ss, float bc2, float eps) {
    const int64_t e = q * 4;
    if (e >= t.n) return;
    if (vec && e + 3 < t.n) {
        float4 p = reinterpret_cast<const float4 *>(t.p)[q];
        const float4 g = reinterpret_cast<const float4 *>(t.g)[q];
        float4 m = reinterpret_cast<const float4 *>(t.m)[q];
        float4 v = reinterpret_cast<const float4 *>(t.v)[q];
        adam_one(p.x, g.x, m.x, v.x, c1, b2, c2, ss, bc2, eps);
        adam_one(p.y, g.y, m.y, v.y, c1, b2, c2, ss, bc2, eps);
        adam_one(p.z, g.z, m.z, v.z, c1, b2, c2, ss, bc2, eps);
        adam_one(p.w, g.w, m.w, v.w, c1, b2, c2, ss, bc2, eps);
        reinterpret_cast<float4 *>(t.p)[q] = p;
        reinterpret_cast<float4 *>(t.m)[q] = m;
        reinterpret_cast<float4 *>(t.v)[q] = v;
        return;
    }
    for (int64_t i = e; i < e + 4 && i < t.n; ++i) {
        float p = t.p[i], m = t.m[i], v = t.v[i];
        adam_one(p, t.g[i], m, v, c1, b2, c2, ss, bc2, eps);
        t.p[i] = p;
        t.m[i] = m;
        t.v[i] = v;
    }
}

__global__ void __launch_bounds__(ADAM_THREADS) adam_flat_kernel(const AdamTensor *__restrict__ tab,
                                                                 int n_tensors,
                                                                 const float *__restrict__ hyper,
                                                                 float c1, float beta2, float c2,
                                                                 float eps) {
    __shared__ int s_t;
    __shared__ long long s_chunk0;
    if (threadIdx.x == 0) {
        long long acc = 0;
        int t = 0;
        for (; t < n_tensors; ++t) {
            const long long ch = (tab[t].n + 4LL * ADAM_CHUNK - 1) / (4LL * ADAM_CHUNK);
            if ((long long)blockIdx.x < acc + ch) break;
            acc += ch;
        }
        s_t = t;
        s_chunk0 = acc;
    }
    __syncthreads();
    if (s_t >= n_tensors) return;
    const AdamTensor t = tab[s_t];
    const float ss = hyper[2 * t.group], bc2 = hyper[2 * t.group + 1];
    const bool vec = ((reinterpret_cast<uintptr_t>(t.p) | reinterpret_cast<uintptr_t>(t.g) |
                       reinterpret_cast<uintptr_t>(t.m) | reinterpret_cast<uintptr_t>(t.v)) &
                      15) == 0;
    const int64_t q0 = ((int64_t)blockIdx.x - s_chunk0) * ADAM_CHUNK;
#pragma unroll
    for (int k = 0; k < ADAM_QPT; ++k)
        adam_quad(t, q0 + threadIdx.x + k * ADAM_THREADS, vec, c1, beta2, c2, ss, bc2, eps);
}

// Many tensors: blockIdx.y = tensor; blocks stride over the tensor's elements
// four at a time (16-byte accesses when aligned), tail scalar.
__global__ void __launch_bounds__(256) adam_kernel(const AdamTensor *__restrict__ tab,
                                                   const float *__restrict__ hyper, float c1,
                                                   float beta2, float c2, float eps) {
    const AdamTensor t = tab[blockIdx.y];
    const float step_size = hyper[2 * t.group], bc2 = hyper[2 * t.group + 1];
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const bool vec = ((reinterpret_cast<uintptr_t>(t.p) | reinterpret_cast<uintptr_t>(t.g) |
                       reinterpret_cast<uintptr_t>(t.m) | reinterpret_cast<uintptr_t>(t.v)) &
                      15) == 0;
    int64_t done = 0;
    if (vec) {
        const int64_t n4 = t.n >> 2;
        for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n4; i += stride) {
            float4 p = reinterpret_cast<const float4 *>(t.p)[i];
            const float4 g = reinterpret_cast<const float4 *>(t.g)[i];
            float4 m = reinterpret_cast<const float4 *>(t.m)[i];
            float4 v = reinterpret_cast<const float4 *>(t.v)[i];
            adam_one(p.x, g.x, m.x, v.x, c1, beta2, c2, step_size, bc2, eps);
            adam_one(p.y, g.y, m.y, v.y, c1, beta2, c2, step_size, bc2, eps);
            adam_one(p.z, g.z, m.z, v.z, c1, beta2, c2, step_size, bc2, eps);
            adam_one(p.w, g.w, m.w, v.w, c1, beta2, c2, step_size, bc2, eps);
            reinterpret_cast<float4 *>(t.p)[i] = p;
            reinterpret_cast<float4 *>(t.m)[i] = m;
            reinterpret_cast<float4 *>(t.v)[i] = v;
        }
        done = n4 << 2;
    }
    for (int64_t i = done + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < t.n; i += stride) {
        float p = t.p[i], m = t.m[i], v = t.v[i];
        adam_one(p, t.g[i], m, v, c1, beta2, c2, step_size, bc2, eps);
        t.p[i] = p;
        t.m[i] = m;
        t.v[i] = v;
    }
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_adam_table_bytes(int32_t n_tensors) {
    return (size_t)(n_tensors < 0 ? 0 : n_tensors) * sizeof(AdamTensor);
}

int ubs_adam_table_entry(void *host_table, int32_t index, float *param, const float *grad,
                         float *exp_avg, float *exp_avg_sq, int64_t numel, int32_t group) {
    UBS_REQUIRE(host_table && index >= 0 && numel >= 0 && group >= 0,
                "adam_table_entry: bad arguments");
    UBS_REQUIRE(numel == 0 || (param && grad && exp_avg && exp_avg_sq),
                "adam_table_entry: null tensor pointer");
    AdamTensor *t = static_cast<AdamTensor *>(host_table) + index;
    t->p = param;
    t->g = grad;
    t->m = exp_avg;
    t->v = exp_avg_sq;
    t->n = numel;
    t->group = group;
    t->pad = 0;
    return UBS_OK;
}

int ubs_adam_step(int32_t n_tensors, const void *device_table, const float *device_hyper,
                  int64_t max_numel, int64_t total_numel, float one_minus_beta1, float beta2,
                  float one_minus_beta2, float eps, void *stream) {
    UBS_REQUIRE(n_tensors >= 0 && n_tensors <= 65535 && max_numel >= 0 && total_numel >= 0,
                "adam_step: bad sizes");
    if (n_tensors == 0 || max_numel == 0) return UBS_OK;
    UBS_REQUIRE(device_table && device_hyper, "adam_step: null table");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (n_tensors <= ADAM_FLAT_MAX && total_numel > 0) {
        // one block per chunk of every tensor (each tensor rounds up to whole chunks)
        const int64_t chunks = (total_numel + 4LL * ADAM_CHUNK - 1) / (4LL * ADAM_CHUNK) + n_tensors;
        UBS_TIMED("adam", st,
                  adam_flat_kernel<<<(unsigned)chunks, ADAM_THREADS, 0, st>>>(
                      static_cast<const AdamTensor *>(device_table), n_tensors, device_hyper,
                      one_minus_beta1, beta2, one_minus_beta2, eps));
        note_launch();
        return check_launch("adam_step");
    }
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (max_numel / 4 + 255) / 256;
    const int64_t cap = (int64_t)sms * 8;
    const dim3 grid((unsigned)(want < 1 ? 1 : (want < cap ? want : cap)), (unsigned)n_tensors);
    UBS_TIMED("adam", st,
              adam_kernel<<<grid, 256, 0, st>>>(static_cast<const AdamTensor *>(device_table),
                                                 device_hyper, one_minus_beta1, beta2,
                                                 one_minus_beta2, eps));
    note_launch();
    return check_launch("adam_step");
}

} // extern "C"
