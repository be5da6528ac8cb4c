// mcmc.cu -- MCMC densification of a scene, device-side end to end.
//
// The reference (scene/beta_model.py:553-658, called from train.py:156-171
// every 100 iterations) finds dead primitives, draws replacement sources with
// torch.multinomial over the live opacities, counts repeats with bincount,
// splits the sources' opacity, copies the seven parameter tensors with
// index_copy and resets Adam moments, with host synchronisations in between
// (mask sums, nonzero, multinomial).  Here the same steps are a fixed
// sequence of launches whose sizes do not depend on the data, so nothing
// waits for the device and the sequence can be captured in a CUDA graph:
//   1. weights: w_i = sigmoid(raw_opacity_i) (0 for dead primitives when
//      relocating), per-block sums (FP64) and dead counts
//   2. one CTA scans the block sums -> block offsets, total weight, #dead
//   3. the inclusive CDF of w (FP64) and the dead list (index order, as
//      nonzero() gives it)
//   4. one draw per dead (or new) slot: u = total * U[0,1) from a counter-
//      based generator, source = first i with cdf_i > u (sampling with
//      replacement proportional to w, as multinomial does); atomic counts
//   5. copies and opacity split; 6. sources take the split opacity and lose
//      their Adam moments (relocation, in place) -- or one grow kernel writes
//      the enlarged tensors (addition).
// The random stream differs from torch.multinomial's; given the same draws
// (the given_src arguments) the results are the reference's.
#include <cfloat>
#include <cstdint>

#include "ubs_common.cuh"

namespace ubs {
namespace {

constexpr int MC_THREADS = 256;
constexpr int MC_PER = 4;                       // elements per thread
constexpr int MC_BLOCK = MC_THREADS * MC_PER;   // elements per block

struct McmcHeader {
    double total;     // sum of the weights
    long long n_dead; // dead primitives (relocation)
    long long pad[6];
};

struct McmcSet {
    int32_t n, opac;
    int32_t w[UBS_MCMC_MAX_TENSORS];
    float *p[UBS_MCMC_MAX_TENSORS];
    float *m[UBS_MCMC_MAX_TENSORS];
    float *v[UBS_MCMC_MAX_TENSORS];
};

struct Ws {
    McmcHeader *hdr;
    double *block_sum;
    long long *block_dead;
    double *cdf;
    int32_t *dead_list;
    int32_t *src;
    int32_t *count;
};

__host__ __device__ inline size_t align_up(size_t x) { return (x + 255) & ~(size_t)255; }

inline Ws carve(void *base, int64_t n, int64_t n_draw) {
    const int64_t nb = (n + MC_BLOCK - 1) / MC_BLOCK;
    char *p = static_cast<char *>(base);
    Ws w;
    w.hdr = reinterpret_cast<McmcHeader *>(p);
    p += align_up(sizeof(McmcHeader));
    w.block_sum = reinterpret_cast<double *>(p);
    p += align_up(sizeof(double) * (nb + 1));
    w.block_dead = reinterpret_cast<long long *>(p);
    p += align_up(sizeof(long long) * (nb + 1));
    w.cdf = reinterpret_cast<double *>(p);
    p += align_up(sizeof(double) * (n + 1));
    w.dead_list = reinterpret_cast<int32_t *>(p);
    p += align_up(sizeof(int32_t) * (n + 1));
    w.src = reinterpret_cast<int32_t *>(p);
    p += align_up(sizeof(int32_t) * (n_draw + 1));
    w.count = reinterpret_cast<int32_t *>(p);
    return w;
}

inline size_t ws_bytes(int64_t n, int64_t n_draw) {
    const int64_t nb = (n + MC_BLOCK - 1) / MC_BLOCK;
    return align_up(sizeof(McmcHeader)) + align_up(sizeof(double) * (nb + 1)) +
           align_up(sizeof(long long) * (nb + 1)) + align_up(sizeof(double) * (n + 1)) +
           align_up(sizeof(int32_t) * (n + 1)) + align_up(sizeof(int32_t) * (n_draw + 1)) +
           align_up(sizeof(int32_t) * (n + 1));
}

__device__ __forceinline__ float sigmoid_fast(float x) { return 1.f / (1.f + __expf(-x)); }

// SplitMix64 output function (Steele, Lea & Flood, OOPSLA 2014) over a
// Weyl sequence: a counter-based generator, one independent value per index.
__device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform01(uint64_t seed, uint64_t i) {
    return (double)(splitmix64(seed + (i + 1) * 0x9e3779b97f4a7c15ull) >> 11) * 0x1.0p-53;
}

// The opacity a source sampled `count` times shares with its copies
// (scene/beta_model.py:553-562): logit(clamp(1 - (1 - o)^(1/(count+1)),
// 0.005, 1 - eps)), o = sigmoid(raw), in FP32.
__device__ __forceinline__ float split_opacity(float raw, int count) {
    const float o = sigmoid_fast(raw);
    const float e = 1.f / (float)(count + 1);
    float n = 1.f - powf(1.f - o, e);
    n = fminf(fmaxf(n, 0.005f), 1.f - FLT_EPSILON);
    return logf(n / (1.f - n));
}

__device__ __forceinline__ bool is_dead(const float *op, const uint8_t *mask, float thresh,
                                        int64_t i) {
    return mask ? mask[i] != 0 : sigmoid_fast(op[i]) <= thresh;
}

// ---- 1. weights: block sums and dead counts
__global__ void __launch_bounds__(MC_THREADS) weights_kernel(const float *__restrict__ op,
                                                             const uint8_t *__restrict__ mask,
                                                             float thresh, int relocate,
                                                             int64_t n, Ws w) {
    const int64_t base = (int64_t)blockIdx.x * MC_BLOCK + threadIdx.x * MC_PER;
    double s = 0.0;
    long long d = 0;
#pragma unroll
    for (int k = 0; k < MC_PER; ++k) {
        const int64_t i = base + k;
        if (i >= n) break;
        const bool dead = relocate && is_dead(op, mask, thresh, i);
        d += dead;
        if (!dead) s += (double)sigmoid_fast(op[i]);
    }
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        d += __shfl_xor_sync(0xffffffffu, d, o);
    }
    __shared__ double ss[MC_THREADS / 32];
    __shared__ long long sd[MC_THREADS / 32];
    if ((threadIdx.x & 31) == 0) {
        ss[threadIdx.x >> 5] = s;
        sd[threadIdx.x >> 5] = d;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ts = 0.0;
        long long td = 0;
        for (int i = 0; i < MC_THREADS / 32; ++i) {
            ts += ss[i];
            td += sd[i];
        }
        w.block_sum[blockIdx.x] = ts;
        w.block_dead[blockIdx.x] = td;
    }
}

// ---- 2. exclusive scan of the block sums (one CTA, chunks of 1024)
__global__ void __launch_bounds__(1024) scan_blocks_kernel(int64_t nb, Ws w) {
    __shared__ double ws_[32];
    __shared__ long long wd[32];
    __shared__ double carry_s;
    __shared__ long long carry_d;
    if (threadIdx.x == 0) {
        carry_s = 0.0;
        carry_d = 0;
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int64_t c0 = 0; c0 < nb; c0 += 1024) {
        const int64_t i = c0 + threadIdx.x;
        const double own_s = i < nb ? w.block_sum[i] : 0.0;
        const long long own_d = i < nb ? w.block_dead[i] : 0;
        double s = own_s;
        long long d = own_d;
        // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const double ts = __shfl_up_sync(0xffffffffu, s, o);
            const long long td = __shfl_up_sync(0xffffffffu, d, o);
            if (lane >= o) {
                s += ts;
                d += td;
            }
        }
        if (lane == 31) {
            ws_[wid] = s;
            wd[wid] = d;
        }
        __syncthreads();
        if (wid == 0) {
            double x = ws_[lane];
            long long y = wd[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const double tx = __shfl_up_sync(0xffffffffu, x, o);
                const long long ty = __shfl_up_sync(0xffffffffu, y, o);
                if (lane >= o) {
                    x += tx;
                    y += ty;
                }
            }
            ws_[lane] = x;
            wd[lane] = y;
        }
        __syncthreads();
        const double before_s = carry_s + (wid ? ws_[wid - 1] : 0.0);
        const long long before_d = carry_d + (wid ? wd[wid - 1] : 0);
        if (i < nb) {
            // exclusive = inclusive - own
            w.block_sum[i] = before_s + s - own_s;
            w.block_dead[i] = before_d + d - own_d;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            carry_s += ws_[31];
            carry_d += wd[31];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        w.hdr->total = carry_s;
        w.hdr->n_dead = carry_d;
    }
}

// ---- 3. inclusive CDF and the dead list
__global__ void __launch_bounds__(MC_THREADS) cdf_kernel(const float *__restrict__ op,
                                                         const uint8_t *__restrict__ mask,
                                                         float thresh, int relocate, int64_t n,
                                                         Ws w) {
    const int64_t base = (int64_t)blockIdx.x * MC_BLOCK + threadIdx.x * MC_PER;
    double ws[MC_PER];
    int dd[MC_PER];
    double s = 0.0;
    int d = 0;
#pragma unroll
    for (int k = 0; k < MC_PER; ++k) {
        const int64_t i = base + k;
        const bool in = i < n;
        const bool dead = in && relocate && is_dead(op, mask, thresh, i);
        ws[k] = (in && !dead) ? (double)sigmoid_fast(op[i]) : 0.0;
        dd[k] = dead;
        s += ws[k];
        d += dead;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double is = s;
    int id = d;
    for (int o = 1; o < 32; o <<= 1) {
        const double ts = __shfl_up_sync(0xffffffffu, is, o);
        const int td = __shfl_up_sync(0xffffffffu, id, o);
        if (lane >= o) {
            is += ts;
            id += td;
        }
    }
    __shared__ double ws_[MC_THREADS / 32];
    __shared__ int wd[MC_THREADS / 32];
    if (lane == 31) {
        ws_[wid] = is;
        wd[wid] = id;
    }
    __syncthreads();
    double off_s = w.block_sum[blockIdx.x];
    long long off_d = w.block_dead[blockIdx.x];
    for (int i = 0; i < wid; ++i) {
        off_s += ws_[i];
        off_d += wd[i];
    }
    off_s += is - s; // exclusive within the block
    off_d += id - d;
#pragma unroll
    for (int k = 0; k < MC_PER; ++k) {
        const int64_t i = base + k;
        if (i >= n) break;
        off_s += ws[k];
        w.cdf[i] = off_s;
        if (dd[k]) w.dead_list[off_d++] = (int32_t)i;
    }
}

// ---- 4. draws: one per slot j < n_draw (n_draw from the header when
// relocating); given sources are copied instead
__global__ void __launch_bounds__(MC_THREADS) draw_kernel(int64_t n, int64_t n_draw_host,
                                                          int relocate, uint64_t seed,
                                                          const int64_t *__restrict__ given,
                                                          int64_t n_given, Ws w,
                                                          uint32_t *status) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t n_draw = relocate ? (int64_t)w.hdr->n_dead : n_draw_host;
    if (j >= n_draw) return;
    int32_t s = -1;
    if (given) {
        if (j < n_given) {
            const int64_t g = given[j];
            if (g >= 0 && g < n) s = (int32_t)g;
            else atomicOr(status, DEV_ERR_OVERFLOW);
        } else {
            atomicOr(status, DEV_ERR_OVERFLOW); // fewer given sources than slots
        }
    } else {
        // the CDF's last entry is the total the draws scale to (the header's
        // total sums the same weights in another order)
        const double total = n > 0 ? w.cdf[n - 1] : 0.0;
        if (total > 0.0) {
            double u = uniform01(seed, (uint64_t)j) * total;
            int64_t lo = 0, hi = n - 1; // first i with cdf[i] > u
            while (lo < hi) {
                const int64_t mid = (lo + hi) >> 1;
                if (w.cdf[mid] > u) hi = mid;
                else lo = mid + 1;
            }
            if (!(w.cdf[lo] > u)) {
                // u rounded up to the total: take the last primitive with
                // weight, the first i whose cdf reaches the total
                lo = 0;
                hi = n - 1;
                while (lo < hi) {
                    const int64_t mid = (lo + hi) >> 1;
                    if (w.cdf[mid] >= total) hi = mid;
                    else lo = mid + 1;
                }
            }
            s = (int32_t)lo;
        }
    }
    w.src[j] = s;
    if (s >= 0) atomicAdd(&w.count[s], 1);
}

// ---- 5. relocation: dead slot <- copy of its source, split opacity
__global__ void __launch_bounds__(MC_THREADS) relocate_copy_kernel(McmcSet t, Ws w) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int64_t)w.hdr->n_dead) return;
    const int32_t s = w.src[j];
    if (s < 0) return;
    const int32_t i = w.dead_list[j];
    for (int k = 0; k < t.n; ++k) {
        const int wd = t.w[k];
        const float *from = t.p[k] + (int64_t)s * wd;
        float *to = t.p[k] + (int64_t)i * wd;
        if (k == t.opac) {
            to[0] = split_opacity(from[0], w.count[s]);
        } else {
            for (int c = 0; c < wd; ++c) to[c] = from[c];
        }
    }
}

// ---- 6. relocation: sources take the split opacity, lose their moments
__global__ void __launch_bounds__(MC_THREADS) relocate_sources_kernel(McmcSet t, Ws w) {
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= (int64_t)w.hdr->n_dead) return;
    const int32_t s = w.src[j];
    if (s < 0) return;
    const int32_t i = w.dead_list[j];
    t.p[t.opac][s] = t.p[t.opac][i];
    for (int k = 0; k < t.n; ++k) {
        const int wd = t.w[k];
        if (t.m[k])
            for (int c = 0; c < wd; ++c) t.m[k][(int64_t)s * wd + c] = 0.f;
        if (t.v[k])
            for (int c = 0; c < wd; ++c) t.v[k][(int64_t)s * wd + c] = 0.f;
    }
}

// ---- addition: the grown tensors, element-parallel.  blockIdx.y = tensor
// * 3 + role (0 parameter, 1 exp_avg, 2 exp_avg_sq).
__global__ void __launch_bounds__(MC_THREADS) grow_kernel(McmcSet old, McmcSet grown,
                                                          int64_t n, int64_t n_add, Ws w) {
    const int k = blockIdx.y / 3, role = blockIdx.y % 3;
    const float *src_t = role == 0 ? old.p[k] : (role == 1 ? old.m[k] : old.v[k]);
    float *dst_t = role == 0 ? grown.p[k] : (role == 1 ? grown.m[k] : grown.v[k]);
    if (!dst_t) return;
    const int wd = old.w[k];
    const int64_t total = (n + n_add) * wd;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const bool small = total < INT32_MAX; // 32-bit row / column split (the usual case)
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int64_t row;
        int col;
        if (small) {
            const uint32_t e32 = (uint32_t)e, r32 = e32 / (uint32_t)wd;
            row = r32;
            col = (int)(e32 - r32 * (uint32_t)wd);
        } else {
            row = e / wd;
            col = (int)(e - row * wd);
        }
        float val;
        if (row < n) {
            const int c = w.count[row];
            if (role == 0)
                val = (k == old.opac && c > 0) ? split_opacity(src_t[row], c) : src_t[e];
            else
                val = (c > 0 || !src_t) ? 0.f : src_t[e];
        } else {
            const int32_t s = w.src[row - n];
            if (role != 0 || s < 0) {
                val = 0.f;
            } else if (k == old.opac) {
                val = split_opacity(src_t[s], w.count[s]);
            } else {
                val = src_t[(int64_t)s * wd + col];
            }
        }
        dst_t[e] = val;
    }
}

// ---- the position noise of train.py:164-171
__global__ void __launch_bounds__(MC_THREADS) perturb_kernel(int64_t n, int dim, float *xyz,
                                                             const float *__restrict__ op,
                                                             const float *__restrict__ scale,
                                                             const float *__restrict__ ltri,
                                                             float factor, uint64_t seed,
                                                             const float *__restrict__ noise) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nl = dim * (dim - 1) / 2;
    float z[3];
    if (noise) {
        for (int c = 0; c < 3; ++c) z[c] = noise[i * 3 + c];
    } else {
        // Box-Muller on two pairs of uniforms (the fourth normal is unused)
        for (int pr = 0; pr < 2; ++pr) {
            const double u1 = uniform01(seed, (uint64_t)i * 4 + 2 * pr);
            const double u2 = uniform01(seed, (uint64_t)i * 4 + 2 * pr + 1);
            const float r = sqrtf(-2.f * logf(1.f - (float)u1));
            float sn, cs;
            sincospif(2.f * (float)u2, &sn, &cs);
            z[2 * pr] = r * cs;
            if (2 * pr + 1 < 3) z[2 * pr + 1] = r * sn;
        }
    }
    // (1 - o)^100 by repeated squaring: x^64 x^32 x^4
    const float x = 1.f - sigmoid_fast(op[i]);
    const float x2 = x * x, x4 = x2 * x2, x8 = x4 * x4, x16 = x8 * x8, x32 = x16 * x16;
    const float f = x32 * x32 * x32 * x4 * factor;
    float s[3];
    for (int c = 0; c < 3; ++c) {
        const float r = scale[i * dim + c];
        s[c] = r > 20.f ? r : log1pf(expf(r));
    }
    const float *l = ltri + i * nl;
    const float R[9] = {1.f, l[0], l[1], -l[0], 1.f, l[2], -l[1], -l[2], 1.f};
    float M[9];
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) M[r * 3 + c] = R[r * 3 + c] * s[c];
    float nz[3];
    for (int c = 0; c < 3; ++c) nz[c] = z[c] * f;
    // Sigma n = M (M^T n)
    float t[3];
    for (int c = 0; c < 3; ++c) t[c] = M[0 * 3 + c] * nz[0] + M[1 * 3 + c] * nz[1] + M[2 * 3 + c] * nz[2];
    for (int r = 0; r < 3; ++r)
        xyz[i * 3 + r] += M[r * 3 + 0] * t[0] + M[r * 3 + 1] * t[1] + M[r * 3 + 2] * t[2];
}

int load_set(const ubs_mcmc_tensors *in, McmcSet &out, bool need_params) {
    UBS_REQUIRE(in, "mcmc: null tensor set");
    UBS_REQUIRE(in->n_tensors >= 1 && in->n_tensors <= UBS_MCMC_MAX_TENSORS,
                "mcmc: 1..%d tensors", UBS_MCMC_MAX_TENSORS);
    UBS_REQUIRE(in->opacity_index >= 0 && in->opacity_index < in->n_tensors &&
                    in->width[in->opacity_index] == 1,
                "mcmc: the opacity tensor must be one of the set, one float per primitive");
    out.n = in->n_tensors;
    out.opac = in->opacity_index;
    for (int k = 0; k < UBS_MCMC_MAX_TENSORS; ++k) {
        const bool used = k < in->n_tensors;
        out.w[k] = used ? in->width[k] : 0;
        out.p[k] = used ? in->param[k] : nullptr;
        out.m[k] = used ? in->exp_avg[k] : nullptr;
        out.v[k] = used ? in->exp_avg_sq[k] : nullptr;
        if (used) {
            UBS_REQUIRE(in->width[k] >= 1 && in->width[k] <= 4096, "mcmc: bad width");
            UBS_REQUIRE(!need_params || in->param[k], "mcmc: null parameter tensor");
        }
    }
    return UBS_OK;
}

// steps 1-4
int sample(const McmcSet &t, int64_t n, const uint8_t *mask, float thresh, int relocate,
           int64_t n_draw, uint64_t seed, const int64_t *given, int64_t n_given, const Ws &w,
           uint32_t *status, cudaStream_t st) {
    const int64_t nb = (n + MC_BLOCK - 1) / MC_BLOCK;
    const float *op = t.p[t.opac];
    if (cudaMemsetAsync(w.count, 0, sizeof(int32_t) * (n + 1), st) != cudaSuccess)
        return set_error(UBS_ERR_CUDA, "mcmc: memset failed");
    UBS_TIMED("mcmc_weights", st,
              weights_kernel<<<(unsigned)nb, MC_THREADS, 0, st>>>(op, mask, thresh, relocate, n,
                                                                  w));
    UBS_TIMED("mcmc_scan", st, scan_blocks_kernel<<<1, 1024, 0, st>>>(nb, w));
    UBS_TIMED("mcmc_cdf", st,
              cdf_kernel<<<(unsigned)nb, MC_THREADS, 0, st>>>(op, mask, thresh, relocate, n, w));
    const int64_t slots = relocate ? n : n_draw;
    if (slots > 0)
        UBS_TIMED("mcmc_draw", st,
                  draw_kernel<<<grid_for(slots, MC_THREADS), MC_THREADS, 0, st>>>(
                      n, n_draw, relocate, seed, given, n_given, w, status));
    note_launch(slots > 0 ? 4 : 3);
    return UBS_OK;
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_mcmc_workspace_bytes(int64_t n_prims, int64_t n_draw_max) {
    if (n_prims < 0) n_prims = 0;
    if (n_draw_max < n_prims) n_draw_max = n_prims;
    return ws_bytes(n_prims, n_draw_max) + 256;
}

int ubs_mcmc_relocate(const ubs_mcmc_tensors *scene, int64_t n_prims, const uint8_t *dead_mask,
                      float dead_threshold, uint64_t seed, const int64_t *given_src,
                      int64_t n_given, uint32_t *status, void *workspace,
                      size_t workspace_bytes, void *stream) {
    McmcSet t;
    const int rc = load_set(scene, t, true);
    if (rc != UBS_OK) return rc;
    UBS_REQUIRE(n_prims >= 0 && n_prims < ((int64_t)1 << 31), "mcmc_relocate: bad size");
    UBS_REQUIRE(status, "mcmc_relocate: null status word");
    if (n_prims == 0) return UBS_OK;
    UBS_REQUIRE(workspace && workspace_bytes >= ubs_mcmc_workspace_bytes(n_prims, n_prims),
                "mcmc_relocate: workspace too small");
    UBS_REQUIRE(!given_src || n_given >= 0, "mcmc_relocate: bad given count");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const Ws w = carve(workspace, n_prims, n_prims);
    int r = sample(t, n_prims, dead_mask, dead_threshold, 1, 0, seed, given_src, n_given, w,
                   status, st);
    if (r != UBS_OK) return r;
    const unsigned g = grid_for(n_prims, MC_THREADS);
    UBS_TIMED("mcmc_relocate_copy", st, relocate_copy_kernel<<<g, MC_THREADS, 0, st>>>(t, w));
    UBS_TIMED("mcmc_relocate_sources", st,
              relocate_sources_kernel<<<g, MC_THREADS, 0, st>>>(t, w));
    note_launch(2);
    return check_launch("mcmc_relocate");
}

int ubs_mcmc_add(const ubs_mcmc_tensors *scene, const ubs_mcmc_tensors *grown, int64_t n_prims,
                 int64_t n_add, uint64_t seed, const int64_t *given_src, uint32_t *status,
                 void *workspace, size_t workspace_bytes, void *stream) {
    McmcSet t, g;
    int rc = load_set(scene, t, true);
    if (rc != UBS_OK) return rc;
    rc = load_set(grown, g, true);
    if (rc != UBS_OK) return rc;
    UBS_REQUIRE(t.n == g.n && t.opac == g.opac, "mcmc_add: tensor sets differ");
    for (int k = 0; k < t.n; ++k) {
        UBS_REQUIRE(t.w[k] == g.w[k], "mcmc_add: widths differ");
        UBS_REQUIRE(!g.m[k] == !t.m[k] && !g.v[k] == !t.v[k],
                    "mcmc_add: optimizer moments must be given for both sets or neither");
    }
    UBS_REQUIRE(n_prims > 0 && n_add >= 0 && n_prims + n_add < ((int64_t)1 << 31),
                "mcmc_add: bad sizes");
    UBS_REQUIRE(status, "mcmc_add: null status word");
    UBS_REQUIRE(workspace && workspace_bytes >= ubs_mcmc_workspace_bytes(n_prims, n_add),
                "mcmc_add: workspace too small");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n_draw = n_add;
    const Ws w = carve(workspace, n_prims, n_draw > n_prims ? n_draw : n_prims);
    int r = sample(t, n_prims, nullptr, 0.f, 0, n_draw, seed, given_src, n_add, w, status, st);
    if (r != UBS_OK) return r;
    int sms = 152, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const dim3 grid((unsigned)sms * 4, (unsigned)(3 * t.n));
    UBS_TIMED("mcmc_grow", st, grow_kernel<<<grid, MC_THREADS, 0, st>>>(t, g, n_prims, n_add, w));
    note_launch();
    return check_launch("mcmc_add");
}

int ubs_mcmc_perturb_xyz(int64_t n_prims, int32_t dim, float *xyz, const float *raw_opacity,
                         const float *raw_scale, const float *l_triangle, float factor,
                         uint64_t seed, const float *given_noise, void *stream) {
    UBS_REQUIRE(n_prims >= 0 && dim >= 3 && dim <= 11, "mcmc_perturb_xyz: bad sizes");
    if (n_prims == 0) return UBS_OK;
    UBS_REQUIRE(xyz && raw_opacity && raw_scale && l_triangle,
                "mcmc_perturb_xyz: null tensor");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    UBS_TIMED("mcmc_perturb_xyz", st,
              perturb_kernel<<<grid_for(n_prims, MC_THREADS), MC_THREADS, 0, st>>>(
                  n_prims, dim, xyz, raw_opacity, raw_scale, l_triangle, factor, seed,
                  given_noise));
    note_launch();
    return check_launch("mcmc_perturb_xyz");
}

} // extern "C"
