// viewer.cu -- the per-frame work of the reference's viewer render function
// (BetaModel.view, scene/beta_model.py:725-831) around the rasteriser:
//
// * Beta quantile masks: the reference keeps primitives whose raw spatial
//   beta, mean raw view beta (and raw time beta) lie within torch.quantile
//   bounds, sorting each of those N-vectors on every frame.  Here the bounds
//   come from an exact batched radix select (four 8-bit passes over the
//   order-preserving integer image of the floats) for all requested ranks at
//   once, interpolated as torch.quantile's "linear" method does
//   (rank = q (N - 1) in float32, lerp of the neighbouring order statistics,
//   NaN anywhere -> NaN bound), and one kernel writes the mask.  The value
//   arrays are the caller's (strided views are fine), so they are the very
//   values the reference forms.
// * Depth colormap (utils/general_utils.py:172-218): min and max of the
//   image on the device, normalisation, clip, index = trunc(255 x) into a
//   256-entry colour table -- without the host round trips of float(min).
#include <cmath>

#include "ubs_common.cuh"

namespace ubs {
namespace {

constexpr int QM_MAX_ARR = 3;            // spatial, view, time
constexpr int QM_MAX_T = 4 * QM_MAX_ARR; // below/above rank of lo/hi quantiles
constexpr int QM_THREADS = 256;

struct QTarget {
    int32_t arr;      // which value array
    int32_t pad;
    int64_t rank;     // order statistic sought (0-based)
};
struct QTargets {     // passed by value: no host copies, capturable launches
    int32_t n, pad;
    QTarget t[QM_MAX_T];
};

struct QState {            // per target, device
    uint32_t prefix, known; // key bits fixed so far and their mask
    int64_t rank;           // remaining rank inside the current prefix
};

struct QArrays {        // the value arrays (device) and their element strides
    const float *p[QM_MAX_ARR];
    int64_t stride[QM_MAX_ARR];
};

struct QWs {
    uint32_t *nan;      // [QM_MAX_ARR]
    uint32_t *hist;     // [QM_MAX_T][256]
    QState *state;      // [QM_MAX_T]
    float *bounds;      // [QM_MAX_ARR][2]
};

__host__ __device__ inline size_t al(size_t x) { return (x + 255) & ~(size_t)255; }

inline size_t qws_bytes() {
    return al(sizeof(uint32_t) * QM_MAX_ARR) + al(sizeof(uint32_t) * QM_MAX_T * 256) +
           al(sizeof(QState) * QM_MAX_T) + al(sizeof(float) * QM_MAX_ARR * 2);
}

inline QWs qws(void *base) {
    char *p = static_cast<char *>(base);
    QWs w;
    w.nan = reinterpret_cast<uint32_t *>(p);
    p += al(sizeof(uint32_t) * QM_MAX_ARR);
    w.hist = reinterpret_cast<uint32_t *>(p);
    p += al(sizeof(uint32_t) * QM_MAX_T * 256);
    w.state = reinterpret_cast<QState *>(p);
    p += al(sizeof(QState) * QM_MAX_T);
    w.bounds = reinterpret_cast<float *>(p);
    return w;
}

// float -> uint32 with the same order (NaNs are counted apart)
__device__ __forceinline__ uint32_t fkey(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// state, NaN flags and histograms to their starting values
__global__ void init_kernel(QTargets tg, QWs w) {
    for (int i = threadIdx.x; i < QM_MAX_T * 256; i += blockDim.x) w.hist[i] = 0u;
    if (threadIdx.x < QM_MAX_ARR) w.nan[threadIdx.x] = 0u;
    if (threadIdx.x < tg.n) w.state[threadIdx.x] = QState{0u, 0u, tg.t[threadIdx.x].rank};
}

// histogram of the next 8-bit digit of the values that share each target's
// prefix
__global__ void __launch_bounds__(QM_THREADS) hist_kernel(int64_t N, int n_arr, QArrays va,
                                                          QTargets tg, int shift, QWs w) {
    __shared__ uint32_t h[QM_MAX_T][256];
    const int n_t = tg.n;
    for (int i = threadIdx.x; i < n_t * 256; i += blockDim.x) h[i / 256][i % 256] = 0;
    __shared__ QState s[QM_MAX_T];
    if (threadIdx.x < n_t) s[threadIdx.x] = w.state[threadIdx.x];
    __syncthreads();
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += stride) {
        const float v0 = va.p[0][i * va.stride[0]], v1 = va.p[1][i * va.stride[1]];
        const float v2 = n_arr > 2 ? va.p[2][i * va.stride[2]] : 0.f;
        if (shift == 24) { // first pass: NaN flags
            if (v0 != v0) atomicOr(&w.nan[0], 1u);
            if (v1 != v1) atomicOr(&w.nan[1], 1u);
            if (v2 != v2) atomicOr(&w.nan[2], 1u);
        }
        const uint32_t k0 = fkey(v0), k1 = fkey(v1), k2 = fkey(v2);
        for (int t = 0; t < n_t; ++t) {
            const int a = tg.t[t].arr;
            const uint32_t key = a == 0 ? k0 : (a == 1 ? k1 : k2);
            if ((key & s[t].known) == s[t].prefix) atomicAdd(&h[t][(key >> shift) & 255u], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < n_t * 256; i += blockDim.x) {
        const uint32_t c = h[i / 256][i % 256];
        if (c) atomicAdd(&w.hist[i], c);
    }
}

// per target: the digit holding its rank; narrow the prefix, clear the
// histogram for the next pass.  One warp per target.
__global__ void select_kernel(int n_t, int shift, QWs w) {
    const int t = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (t >= n_t) return;
    uint32_t *h = w.hist + t * 256;
    QState st = w.state[t];
    // each lane owns 8 consecutive bins
    uint32_t c[8], tot = 0;
    for (int k = 0; k < 8; ++k) {
        c[k] = h[lane * 8 + k];
        tot += c[k];
    }
    uint32_t incl = tot;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t x = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += x;
    }
    const uint32_t excl = incl - tot;
    const int64_t r = st.rank;
    // the lane whose range of cumulative counts holds r
    const bool mine = (int64_t)excl <= r && r < (int64_t)incl;
    const unsigned who = __ballot_sync(0xffffffffu, mine);
    if (mine) {
        int64_t acc = excl;
        int d = 0;
        for (int k = 0; k < 8; ++k) {
            if (r < acc + (int64_t)c[k]) {
                d = lane * 8 + k;
                break;
            }
            acc += c[k];
        }
        st.prefix |= (uint32_t)d << shift;
        st.known |= 255u << shift;
        st.rank = r - acc;
        w.state[t] = st;
    }
    (void)who;
    __syncwarp();
    for (int k = 0; k < 8; ++k) h[lane * 8 + k] = 0;
}

// bounds = lerp(below, above, weight) as torch.lerp forms it; NaN in an
// array makes both of its bounds NaN (torch.quantile's rank of the last,
// NaN, element)
struct QBound {
    int32_t arr, t_below, t_above, pad;
    float weight;
};
struct QBounds {
    int32_t n;
    QBound b[2 * QM_MAX_ARR];
};

__global__ void bounds_kernel(QBounds qb, QWs w) {
    const int i = threadIdx.x;
    if (i >= qb.n) return;
    const QBound b = qb.b[i];
    float v;
    if (w.nan[b.arr]) {
        v = __int_as_float(0x7fc00000);
    } else {
        const float lo = fkey_inv(w.state[b.t_below].prefix);
        const float hi = fkey_inv(w.state[b.t_above].prefix);
        const float wt = b.weight;
        v = fabsf(wt) < 0.5f ? lo + wt * (hi - lo) : hi - (hi - lo) * (1.f - wt);
    }
    w.bounds[i] = v;
}

__global__ void __launch_bounds__(QM_THREADS) mask_kernel(int64_t N, int n_arr, QArrays va,
                                                          QWs w, uint8_t *__restrict__ mask) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= N) return;
    bool m = true;
    for (int a = 0; a < n_arr; ++a) {
        const float v = va.p[a][i * va.stride[a]];
        m = m && (v >= w.bounds[2 * a]) && (v <= w.bounds[2 * a + 1]);
    }
    mask[i] = m ? 1 : 0;
}

// ---- depth colormap
__global__ void mm_init_kernel(unsigned int *mm) {
    if (threadIdx.x == 0) {
        mm[0] = 0xffffffffu;
        mm[1] = 0u;
        mm[2] = 0u;
    }
}

__global__ void __launch_bounds__(256) minmax_kernel(const float *__restrict__ img, int64_t n,
                                                     unsigned int *mm) {
    float lo = INFINITY, hi = -INFINITY;
    bool nan = false;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const float v = img[i];
        if (v != v) nan = true;
        lo = fminf(lo, v);
        hi = fmaxf(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    nan = __any_sync(0xffffffffu, nan);
    if ((threadIdx.x & 31) == 0) {
        // ordered-integer min / max; NaN (torch.min / max propagate it) flagged
        atomicMin(&mm[0], fkey(lo));
        atomicMax(&mm[1], fkey(hi));
        if (nan) atomicOr(&mm[2], 1u);
    }
}

__global__ void __launch_bounds__(256) colormap_kernel(const float *__restrict__ img, int64_t n,
                                                       const unsigned int *mm,
                                                       const float *__restrict__ table,
                                                       float *__restrict__ out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int idx = 0;
    if (!mm[2]) {
        const float lo = fkey_inv(mm[0]), hi = fkey_inv(mm[1]);
        // (depth - near) / (far - near + 1e-10) with the Python-double
        // denominator rounded to float, clip, trunc(255 x)
        const float den = (float)((double)hi - (double)lo + 1e-10);
        float d = (img[i] - lo) / den;
        d = fminf(fmaxf(d, 0.f), 1.f);
        if (d != d) d = 0.f;
        idx = (int)(d * 255.f);
    }
    out[i * 3 + 0] = table[idx * 3 + 0];
    out[i * 3 + 1] = table[idx * 3 + 1];
    out[i * 3 + 2] = table[idx * 3 + 2];
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_quantile_mask_workspace_bytes(void) { return qws_bytes(); }

int ubs_quantile_mask(int64_t n, int32_t n_arrays, const float *const *arrays,
                      const int64_t *strides, const double *quantiles, uint8_t *mask,
                      void *workspace, size_t workspace_bytes, void *stream) {
    UBS_REQUIRE(n >= 0 && n_arrays >= 1 && n_arrays <= QM_MAX_ARR, "quantile_mask: bad sizes");
    if (n == 0) return UBS_OK;
    UBS_REQUIRE(arrays && strides && quantiles && mask, "quantile_mask: null pointer");
    UBS_REQUIRE(workspace && workspace_bytes >= qws_bytes(), "quantile_mask: workspace too small");
    QArrays va{};
    for (int a = 0; a < QM_MAX_ARR; ++a) {
        const int src = a < n_arrays ? a : 0; // unused slots alias array 0
        va.p[a] = arrays[src];
        va.stride[a] = strides[src];
        UBS_REQUIRE(va.p[a] && va.stride[a] >= 1, "quantile_mask: bad array %d", a);
    }
    for (int i = 0; i < 2 * n_arrays; ++i)
        UBS_REQUIRE(quantiles[i] >= 0.0 && quantiles[i] <= 1.0,
                    "quantile_mask: quantile %g outside [0, 1]", quantiles[i]);
    const QWs w = qws(workspace);
    // ranks as torch.quantile forms them: q in float32, q * (N - 1) in float32
    QTargets tgs{};
    QTarget *tg = tgs.t;
    QBounds qb{};
    int n_t = 0;
    qb.n = 2 * n_arrays;
    for (int i = 0; i < 2 * n_arrays; ++i) {
        const float q = (float)quantiles[i];
        const float rank = q * (float)(n - 1);
        const int64_t below = (int64_t)rank;
        const int64_t above = (int64_t)ceilf(rank);
        QBound b{};
        b.arr = i / 2;
        b.weight = rank - (float)below;
        b.t_below = n_t;
        tg[n_t++] = QTarget{b.arr, 0, below};
        b.t_above = n_t;
        tg[n_t++] = QTarget{b.arr, 0, above};
        qb.b[i] = b;
    }
    tgs.n = n_t;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned g = grid_for(n, QM_THREADS);
    const unsigned gh = (unsigned)((int64_t)g < (int64_t)sms * 4 ? g : sms * 4);
    UBS_TIMED("quantile_init", st, init_kernel<<<1, 256, 0, st>>>(tgs, w));
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 24 - 8 * pass;
        UBS_TIMED("quantile_hist", st,
                  hist_kernel<<<gh, QM_THREADS, 0, st>>>(n, n_arrays, va, tgs, shift, w));
        UBS_TIMED("quantile_select", st, select_kernel<<<1, 32 * n_t, 0, st>>>(n_t, shift, w));
    }
    UBS_TIMED("quantile_bounds", st, bounds_kernel<<<1, 32, 0, st>>>(qb, w));
    UBS_TIMED("quantile_mask", st,
              mask_kernel<<<g, QM_THREADS, 0, st>>>(n, n_arrays, va, w, mask));
    note_launch(11);
    return check_launch("quantile_mask");
}

int ubs_quantile_mask_bounds(const void *workspace, int32_t n_arrays, float *bounds_out,
                             void *stream) {
    UBS_REQUIRE(workspace && bounds_out && n_arrays >= 1 && n_arrays <= QM_MAX_ARR,
                "quantile_mask_bounds: bad arguments");
    const QWs w = qws(const_cast<void *>(workspace));
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(bounds_out, w.bounds, sizeof(float) * 2 * n_arrays,
                        cudaMemcpyDeviceToDevice, st) != cudaSuccess)
        return check_launch("quantile_mask_bounds");
    return UBS_OK;
}

int ubs_depth_colormap(const float *image, int64_t n_pixels, const float *table, float *out,
                       void *workspace, void *stream) {
    UBS_REQUIRE(n_pixels >= 0 && image && table && out && workspace,
                "depth_colormap: bad arguments");
    if (n_pixels == 0) return UBS_OK;
    unsigned int *mm = static_cast<unsigned int *>(workspace);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    mm_init_kernel<<<1, 32, 0, st>>>(mm);
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const unsigned g = grid_for(n_pixels, 256);
    UBS_TIMED("depth_minmax", st,
              minmax_kernel<<<(unsigned)((int64_t)g < sms * 4 ? g : sms * 4), 256, 0, st>>>(
                  image, n_pixels, mm));
    UBS_TIMED("depth_colormap", st,
              colormap_kernel<<<g, 256, 0, st>>>(image, n_pixels, mm, table, out));
    note_launch(3);
    return check_launch("depth_colormap");
}

} // extern "C"
