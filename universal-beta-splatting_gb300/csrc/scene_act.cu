// scene_act.cu -- activations of the raw Universal Beta Splatting parameters
// for the fused scene render, rounded exactly as the reference computes them.
//
// The reference model activates its parameters with PyTorch elementwise
// kernels (scene/beta_model.py:36-52, 103-121): scale = softplus(raw) (beta 1,
// threshold 20), beta = 4 exp(raw), opacity = sigmoid(raw).  PyTorch builds
// those kernels with IEEE single-precision math.  The rest of the library is
// compiled with fast math (as the reference's own CUDA operators are), under
// which expf and division are approximations that differ from PyTorch's in the
// last bits, and those bits propagate through the conditioning into the
// projected depths that key the intersection sort.  So this translation unit
// is compiled WITHOUT --use_fast_math: one pass writes the activated values
// that the fused per-primitive kernels read.
//
// Layout: act = [N, D] scales, then [N, D - 2] betas, then [N] opacities
// (float, contiguous), inside the fused render's workspace.  Each thread
// activates four consecutive values with 16-byte accesses where aligned, in
// a grid-stride loop over eight CTAs per SM.
#include "ubs_common.cuh"

namespace ubs {

namespace {

// softplus with PyTorch's formulation: x > threshold ? x : log1p(exp(x))
__device__ __forceinline__ float torch_softplus(float x) {
    return x > 20.f ? x : log1pf(expf(x));
}
// sigmoid with PyTorch's formulation: 1 / (1 + exp(-x))
__device__ __forceinline__ float torch_sigmoid(float x) { return 1.f / (1.f + expf(-x)); }

template <int OP> __device__ __forceinline__ float activate(float x) {
    if (OP == 0) return torch_softplus(x);
    if (OP == 1) return 4.f * expf(x);
    return torch_sigmoid(x);
}

// Four consecutive values [4q, 4q + 4) of one section (len values): one
// 16-byte load and store when both sides are 16-byte aligned and the four are
// all in range, else value by value.
template <int OP>
__device__ __forceinline__ void act_quad(const float *__restrict__ src, float *__restrict__ dst,
                                         int64_t q, int64_t len, bool vec) {
    const int64_t i = q * 4;
    if (vec && i + 4 <= len) {
        const float4 x = *reinterpret_cast<const float4 *>(src + i);
        *reinterpret_cast<float4 *>(dst + i) =
            make_float4(activate<OP>(x.x), activate<OP>(x.y), activate<OP>(x.z), activate<OP>(x.w));
        return;
    }
    for (int64_t k = i; k < len && k < i + 4; ++k) dst[k] = activate<OP>(src[k]);
}

// The three sections (D scales, D - 2 betas, one opacity per primitive) as
// one space of four-value quads, walked by a grid-stride loop; `vec` bit s
// says section s is 16-byte aligned on both sides.
__global__ void scene_act_kernel(int64_t N, int D, const float *__restrict__ scale,
                                 const float *__restrict__ beta, const float *__restrict__ opac,
                                 float *__restrict__ act, int vec) {
    const int64_t ns = N * D, nb = N * (D - 2);
    const int64_t qs = (ns + 3) / 4, qb = (nb + 3) / 4, qo = (N + 3) / 4;
    float *act_b = act + act_beta_off(N, D), *act_o = act + act_opac_off(N, D);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < qs + qb + qo;
         q += stride) {
        if (q < qs) act_quad<0>(scale, act, q, ns, vec & 1);
        else if (q < qs + qb) act_quad<1>(beta, act_b, q - qs, nb, vec & 2);
        else act_quad<2>(opac, act_o, q - qs - qb, N, vec & 4);
    }
}

} // namespace

int launch_scene_act(int64_t N, int D, const float *scale, const float *beta, const float *opac,
                     float *act, cudaStream_t st) {
    if (N == 0) return UBS_OK;
    const int64_t ns = N * D, nb = N * (D - 2);
    auto a16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
    const int vec = (a16(scale) && a16(act) ? 1 : 0) |
                    (a16(beta) && a16(act + act_beta_off(N, D)) ? 2 : 0) |
                    (a16(opac) && a16(act + act_opac_off(N, D)) ? 4 : 0);
    const int64_t quads = (ns + 3) / 4 + (nb + 3) / 4 + (N + 3) / 4;
    int dev = 0, sms = 152;
    if (cudaGetDevice(&dev) == cudaSuccess)
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (quads + 255) / 256, cap = (int64_t)sms * 8;
    const unsigned grid = (unsigned)(want < cap ? want : cap);
    UBS_TIMED("scene_act", st,
              scene_act_kernel<<<grid, 256, 0, st>>>(N, D, scale, beta, opac, act, vec));
    note_launch();
    return check_launch("scene_act");
}

} // namespace ubs
