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
// (float, contiguous), inside the fused render's workspace.
#include "ubs_common.cuh"

namespace ubs {

namespace {

// softplus with PyTorch's formulation: x > threshold ? x : log1p(exp(x))
__device__ __forceinline__ float torch_softplus(float x) {
    return x > 20.f ? x : log1pf(expf(x));
}
// sigmoid with PyTorch's formulation: 1 / (1 + exp(-x))
__device__ __forceinline__ float torch_sigmoid(float x) { return 1.f / (1.f + expf(-x)); }

// One thread per (primitive, value): rows of D scales, D - 2 betas and one
// opacity are activated by consecutive threads, so reads and writes coalesce.
__global__ void scene_act_kernel(int64_t N, int D, const float *__restrict__ scale,
                                 const float *__restrict__ beta, const float *__restrict__ opac,
                                 float *__restrict__ act) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t ns = N * D, nb = N * (D - 2);
    if (i < ns) {
        act[i] = torch_softplus(scale[i]);
    } else if (i < ns + nb) {
        act[i] = 4.f * expf(beta[i - ns]);
    } else if (i < ns + nb + N) {
        act[i] = torch_sigmoid(opac[i - ns - nb]);
    }
}

} // namespace

int launch_scene_act(int64_t N, int D, const float *scale, const float *beta, const float *opac,
                     float *act, cudaStream_t st) {
    const int64_t total = N * (2 * D - 1);
    if (total == 0) return UBS_OK;
    UBS_TIMED("scene_act", st,
              scene_act_kernel<<<grid_for(total, 256), 256, 0, st>>>(N, D, scale, beta, opac,
                                                                      act));
    note_launch();
    return check_launch("scene_act");
}

} // namespace ubs
