// ssim.cu -- the training loss (1 - l) L1 + l (1 - SSIM) and its gradient in
// one pass.
//
// SSIM as the reference defines it (utils/loss_utils.py:26-80, the function
// the fused_ssim package used by train.py:117-121 evaluates): an 11 x 11
// Gaussian window (sigma 1.5) applied with zero padding ("same" output size)
// to x, y, x^2, y^2 and x y; C1 = 0.01^2, C2 = 0.03^2;
//   map = (2 mx my + C1)(2 sxy + C2) / ((mx^2 + my^2 + C1)(sxx + syy + C2))
// with sxx = E[x^2] - mx^2, sxy = E[xy] - mx my, and the loss reads the mean
// of the map (optionally cropped by the window radius, fused_ssim's "valid").
//
// One CTA owns a 32 x 32 tile of one (image, channel).  The window is
// separable, so the moments are a horizontal then a vertical 11-tap pass over
// shared memory.  For the gradient the CTA also evaluates the map on the
// 5-pixel ring around its tile (recomputing the moments there from a 10-pixel
// input halo) and forms, per map point q,
//   D0 = d map / d mx,  D1 = d map / d E[x^2],  D2 = d map / d E[xy]
// (derivatives with the E[.] moments as the free variables); the gradient at
// pixel p is then  sum_q w(q - p) (D0 + 2 x_p D1 + y_p D2), two more
// separable passes.  Nothing but the inputs and the gradient touches HBM.
//
// Loss sums: one partial per CTA, reduced in a fixed order by the last CTA to
// finish (a ticket counter that the last CTA resets), so the result is
// deterministic and the launch can be replayed from a CUDA graph.
#include <cmath>

#include "ubs_common.cuh"

namespace ubs {
namespace {

constexpr int SS_T = 32;       // output tile edge
constexpr int SS_R = 5;        // window radius (11 taps)
constexpr int SS_W = 2 * SS_R + 1;
constexpr int SS_THREADS = 384;

struct SsimArgs {
    const float *img;
    const float *gt;
    float *grad;                 // null: loss only
    int64_t is[4], gs[4], ds[4]; // element strides (image, channel, row, column)
    int32_t n, c, h, w;
    int32_t tiles_x, tiles_y;
    int32_t valid;               // count only map points >= SS_R from every edge
    float c1, c2;
    float ga, gb;                // d loss / d |x - y| (per pixel), d loss / d map (per point)
    double inv_px, inv_map;      // 1 / pixels, 1 / counted map points
    double wl1, wssim, wconst;   // loss = wl1 mean|x-y| + wssim mean(map) + wconst
    float g[SS_W];               // normalised 1-D window
    float *partials;             // [n_ctas][2]
    unsigned *counter;
    float *out;                  // [3]: mean(map), mean|x-y|, loss
};

// Region sizes: the loss-only variant needs moments on the tile itself; the
// gradient variant on the tile plus a ring of SS_R.
template <bool GRAD> struct Geom {
    static constexpr int MO = SS_T + (GRAD ? 2 * SS_R : 0); // moment / map points per edge
    static constexpr int IN = MO + 2 * SS_R;                // input pixels per edge
    static constexpr int IP = IN + 1;                       // padded pitch of input planes
    static constexpr int MP = MO + 1;                       // padded pitch of moment planes
    static constexpr int OFF = (IN - SS_T) / 2;             // tile origin inside the input region
    static constexpr int SEG = GRAD ? 6 : 8;                // outputs per item, moment passes
    static constexpr int NSEG = MO / SEG;
    static_assert(MO % SEG == 0, "segments must tile the moment region");
    // input planes x, y, x^2, y^2, xy; horizontal moments (5 planes IN x MO)
    static constexpr int IN_PLANE = IN * IP;
    static constexpr int HM_PLANE = IN * MP;
    static constexpr size_t FLOATS = 5 * (size_t)IN_PLANE + 5 * (size_t)HM_PLANE;
    static constexpr size_t BYTES = FLOATS * sizeof(float) + 64;
};

__device__ __forceinline__ float block_sum(float v, float *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    float s = 0.f;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s; // valid in thread 0
}

template <bool GRAD>
__global__ void __launch_bounds__(SS_THREADS, 2) ssim_kernel(const SsimArgs a) {
    using G = Geom<GRAD>;
    extern __shared__ float4 smem4[];
    float *sm = reinterpret_cast<float *>(smem4);
    float *in = sm;                         // 5 input planes
    float *hm = sm + 5 * G::IN_PLANE;       // 5 horizontal-moment planes
    __shared__ float red[SS_THREADS / 32];
    __shared__ bool last;

    const int img = blockIdx.z / a.c, ch = blockIdx.z % a.c;
    const int y0 = blockIdx.y * SS_T, x0 = blockIdx.x * SS_T;
    const float *X = a.img + img * a.is[0] + ch * a.is[1];
    const float *Y = a.gt + img * a.gs[0] + ch * a.gs[1];

    // ---- inputs (zero outside the image) and their products
    for (int i = threadIdx.x; i < G::IN * G::IN; i += SS_THREADS) {
        const int r = i / G::IN, cc = i % G::IN;
        const int gy = y0 - G::OFF + r, gx = x0 - G::OFF + cc;
        float xv = 0.f, yv = 0.f;
        if (gy >= 0 && gy < a.h && gx >= 0 && gx < a.w) {
            xv = __ldg(X + gy * a.is[2] + gx * a.is[3]);
            yv = __ldg(Y + gy * a.gs[2] + gx * a.gs[3]);
        }
        const int o = r * G::IP + cc;
        in[o] = xv;
        in[G::IN_PLANE + o] = yv;
        in[2 * G::IN_PLANE + o] = xv * xv;
        in[3 * G::IN_PLANE + o] = yv * yv;
        in[4 * G::IN_PLANE + o] = xv * yv;
    }
    __syncthreads();

    // ---- horizontal pass: item = (row, segment); consecutive threads take
    // consecutive rows (odd pitch: conflict-free)
    for (int it = threadIdx.x; it < G::IN * G::NSEG; it += SS_THREADS) {
        const int r = it % G::IN, c0 = (it / G::IN) * G::SEG;
#pragma unroll 1
        for (int k = 0; k < 5; ++k) {
            const float *src = in + k * G::IN_PLANE + r * G::IP + c0;
            float v[G::SEG + 2 * SS_R];
#pragma unroll
            for (int j = 0; j < G::SEG + 2 * SS_R; ++j) v[j] = src[j];
            float acc[G::SEG];
#pragma unroll
            for (int o = 0; o < G::SEG; ++o) acc[o] = 0.f;
#pragma unroll
            for (int t = 0; t < SS_W; ++t) {
                const float wt = a.g[t];
#pragma unroll
                for (int o = 0; o < G::SEG; ++o) acc[o] = fmaf(wt, v[o + t], acc[o]);
            }
            float *dst = hm + k * G::HM_PLANE + r * G::MP + c0;
#pragma unroll
            for (int o = 0; o < G::SEG; ++o) dst[o] = acc[o];
        }
    }
    __syncthreads();

    // ---- vertical pass, the map and (GRAD) its derivatives.  The product
    // planes are free from here on: D0..D2 (MO x MP each) go there; x and y
    // stay for the gradient.
    float *dmap = in + 2 * G::IN_PLANE;
    float ssim_sum = 0.f;
    for (int it = threadIdx.x; it < G::MO * G::NSEG; it += SS_THREADS) {
        const int m = it % G::MO, r0 = (it / G::MO) * G::SEG;
        float mom[5][G::SEG];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const float *src = hm + k * G::HM_PLANE + r0 * G::MP + m;
            float v[G::SEG + 2 * SS_R];
#pragma unroll
            for (int j = 0; j < G::SEG + 2 * SS_R; ++j) v[j] = src[j * G::MP];
#pragma unroll
            for (int o = 0; o < G::SEG; ++o) mom[k][o] = 0.f;
#pragma unroll
            for (int t = 0; t < SS_W; ++t) {
                const float wt = a.g[t];
#pragma unroll
                for (int o = 0; o < G::SEG; ++o) mom[k][o] = fmaf(wt, v[o + t], mom[k][o]);
            }
        }
#pragma unroll
        for (int o = 0; o < G::SEG; ++o) {
            const int r = r0 + o;
            const int gy = y0 - (G::MO - SS_T) / 2 + r, gx = x0 - (G::MO - SS_T) / 2 + m;
            bool counted = gy >= 0 && gy < a.h && gx >= 0 && gx < a.w;
            if (a.valid)
                counted = counted && gy >= SS_R && gy < a.h - SS_R && gx >= SS_R && gx < a.w - SS_R;
            const float mx = mom[0][o], my = mom[1][o];
            const float mxx = mx * mx, myy = my * my, mxy = mx * my;
            const float vx = mom[2][o] - mxx, vy = mom[3][o] - myy, cxy = mom[4][o] - mxy;
            const float A1 = 2.f * mxy + a.c1, A2 = 2.f * cxy + a.c2;
            const float B1 = mxx + myy + a.c1, B2 = vx + vy + a.c2;
            const float s = (A1 * A2) / (B1 * B2);
            const bool own = r >= (G::MO - SS_T) / 2 && r < (G::MO + SS_T) / 2 &&
                             m >= (G::MO - SS_T) / 2 && m < (G::MO + SS_T) / 2;
            if (counted && own) ssim_sum += s;
            if (GRAD) {
                float d0 = 0.f, d1 = 0.f, d2 = 0.f;
                if (counted) {
                    const float iB1 = 1.f / B1, iB2 = 1.f / B2, iBB = iB1 * iB2;
                    d0 = 2.f * my * (A2 - A1) * iBB - 2.f * mx * s * (iB1 - iB2);
                    d1 = -s * iB2;
                    d2 = 2.f * A1 * iBB;
                }
                dmap[r * G::MP + m] = d0;
                dmap[G::HM_PLANE + r * G::MP + m] = d1;
                dmap[2 * G::HM_PLANE + r * G::MP + m] = d2;
            }
        }
    }

    float l1_sum = 0.f;
    if (GRAD) {
        __syncthreads();
        // ---- horizontal pass over D0..D2 (MO rows -> SS_T columns), 16
        // outputs per item; results into the moment planes (free now)
        float *dh = hm;
        constexpr int DSEG = 16, DNS = SS_T / DSEG;
        for (int it = threadIdx.x; it < 3 * G::MO * DNS; it += SS_THREADS) {
            const int r = it % G::MO, rest = it / G::MO;
            const int c0 = (rest % DNS) * DSEG, k = rest / DNS;
            const float *src = dmap + k * G::HM_PLANE + r * G::MP + c0;
            float v[DSEG + 2 * SS_R];
#pragma unroll
            for (int j = 0; j < DSEG + 2 * SS_R; ++j) v[j] = src[j];
            float acc[DSEG];
#pragma unroll
            for (int o = 0; o < DSEG; ++o) acc[o] = 0.f;
#pragma unroll
            for (int t = 0; t < SS_W; ++t) {
                const float wt = a.g[t];
#pragma unroll
                for (int o = 0; o < DSEG; ++o) acc[o] = fmaf(wt, v[o + t], acc[o]);
            }
            float *dst = dh + k * G::HM_PLANE + r * G::MP + c0;
#pragma unroll
            for (int o = 0; o < DSEG; ++o) dst[o] = acc[o];
        }
        __syncthreads();
        // ---- vertical pass (SS_T x SS_T), 8 outputs per item, into the
        // D planes (free now)
        float *gv = dmap;
        constexpr int VSEG = 8, VNS = SS_T / VSEG;
        for (int it = threadIdx.x; it < 3 * SS_T * VNS; it += SS_THREADS) {
            const int cx = it % SS_T, rest = it / SS_T;
            const int r0 = (rest % VNS) * VSEG, k = rest / VNS;
            const float *src = dh + k * G::HM_PLANE + r0 * G::MP + cx;
            float v[VSEG + 2 * SS_R];
#pragma unroll
            for (int j = 0; j < VSEG + 2 * SS_R; ++j) v[j] = src[j * G::MP];
#pragma unroll
            for (int o = 0; o < VSEG; ++o) {
                float acc = 0.f;
#pragma unroll
                for (int t = 0; t < SS_W; ++t) acc = fmaf(a.g[t], v[o + t], acc);
                gv[k * G::HM_PLANE + (r0 + o) * G::MP + cx] = acc;
            }
        }
        __syncthreads();
        // ---- gradient and the L1 term at the tile's pixels
        float *D = a.grad + img * a.ds[0] + ch * a.ds[1];
        for (int i = threadIdx.x; i < SS_T * SS_T; i += SS_THREADS) {
            const int r = i / SS_T, cx = i % SS_T;
            const int gy = y0 + r, gx = x0 + cx;
            if (gy >= a.h || gx >= a.w) continue;
            const int o = (r + G::OFF) * G::IP + cx + G::OFF;
            const float xv = in[o], yv = in[G::IN_PLANE + o];
            const float d = xv - yv;
            l1_sum += fabsf(d);
            const float s0 = gv[r * G::MP + cx], s1 = gv[G::HM_PLANE + r * G::MP + cx],
                        s2 = gv[2 * G::HM_PLANE + r * G::MP + cx];
            const float sg = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
            D[gy * a.ds[2] + gx * a.ds[3]] =
                fmaf(a.gb, fmaf(2.f * xv, s1, fmaf(yv, s2, s0)), a.ga * sg);
        }
    } else {
        for (int i = threadIdx.x; i < SS_T * SS_T; i += SS_THREADS) {
            const int r = i / SS_T, cx = i % SS_T;
            if (y0 + r >= a.h || x0 + cx >= a.w) continue;
            const int o = (r + G::OFF) * G::IP + cx + G::OFF;
            l1_sum += fabsf(in[o] - in[G::IN_PLANE + o]);
        }
    }

    // ---- loss: per-CTA partials, reduced by the last CTA in a fixed order
    const float bs = block_sum(ssim_sum, red);
    const float bl = block_sum(l1_sum, red);
    const unsigned cta = blockIdx.x + gridDim.x * (blockIdx.y + gridDim.y * blockIdx.z);
    const unsigned n_cta = gridDim.x * gridDim.y * gridDim.z;
    if (threadIdx.x == 0) {
        a.partials[2 * cta] = bs;
        a.partials[2 * cta + 1] = bl;
        __threadfence();
        last = atomicAdd(a.counter, 1u) == n_cta - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0, l = 0.0;
    for (unsigned i = threadIdx.x; i < n_cta; i += SS_THREADS) {
        s += (double)__ldcg(a.partials + 2 * i);
        l += (double)__ldcg(a.partials + 2 * i + 1);
    }
    __shared__ double dred[2][SS_THREADS / 32];
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        l += __shfl_xor_sync(0xffffffffu, l, o);
    }
    if ((threadIdx.x & 31) == 0) {
        dred[0][threadIdx.x >> 5] = s;
        dred[1][threadIdx.x >> 5] = l;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double ts = 0.0, tl = 0.0;
        for (int i = 0; i < SS_THREADS / 32; ++i) {
            ts += dred[0][i];
            tl += dred[1][i];
        }
        const double ms = ts * a.inv_map, ml = tl * a.inv_px;
        a.out[0] = (float)ms;
        a.out[1] = (float)ml;
        a.out[2] = (float)(a.wl1 * ml + a.wssim * ms + a.wconst);
        *a.counter = 0u;
    }
}

template <bool GRAD> void set_smem() {
    static bool done = false;
    if (!done) {
        cudaFuncSetAttribute(ssim_kernel<GRAD>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)Geom<GRAD>::BYTES);
        done = true;
    }
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_ssim_workspace_bytes(int32_t n_images, int32_t channels, int32_t height,
                                int32_t width) {
    if (n_images <= 0 || channels <= 0 || height <= 0 || width <= 0) return 256;
    const size_t ctas = (size_t)n_images * channels * ((height + SS_T - 1) / SS_T) *
                        ((width + SS_T - 1) / SS_T);
    return 256 + ctas * 2 * sizeof(float);
}

int ubs_ssim_loss(const float *img, const int64_t *img_strides, const float *gt,
                  const int64_t *gt_strides, float *grad, const int64_t *grad_strides,
                  int32_t n_images, int32_t channels, int32_t height, int32_t width,
                  int32_t valid_padding, double weight_l1, double weight_ssim,
                  double weight_const, float *out, void *workspace, size_t workspace_bytes,
                  void *stream) {
    UBS_REQUIRE(n_images > 0 && channels > 0 && height > 0 && width > 0,
                "ssim_loss: empty image batch");
    UBS_REQUIRE((int64_t)n_images * channels <= 65535, "ssim_loss: too many image channels");
    UBS_REQUIRE(!valid_padding || (height > 2 * SS_R && width > 2 * SS_R),
                "ssim_loss: 'valid' padding needs images larger than the window");
    UBS_REQUIRE(img && gt && out && img_strides && gt_strides, "ssim_loss: null pointer");
    UBS_REQUIRE(!grad || grad_strides, "ssim_loss: gradient strides missing");
    UBS_REQUIRE(workspace && workspace_bytes >= ubs_ssim_workspace_bytes(n_images, channels,
                                                                         height, width),
                "ssim_loss: workspace too small");
    SsimArgs a;
    a.img = img;
    a.gt = gt;
    a.grad = grad;
    for (int i = 0; i < 4; ++i) {
        a.is[i] = img_strides[i];
        a.gs[i] = gt_strides[i];
        a.ds[i] = grad ? grad_strides[i] : 0;
    }
    a.n = n_images;
    a.c = channels;
    a.h = height;
    a.w = width;
    a.tiles_x = (width + SS_T - 1) / SS_T;
    a.tiles_y = (height + SS_T - 1) / SS_T;
    a.valid = valid_padding ? 1 : 0;
    a.c1 = (float)(0.01 * 0.01);
    a.c2 = (float)(0.03 * 0.03);
    const double px = (double)n_images * channels * height * width;
    const double pts = valid_padding
                           ? (double)n_images * channels * (height - 2 * SS_R) * (width - 2 * SS_R)
                           : px;
    a.inv_px = 1.0 / px;
    a.inv_map = 1.0 / pts;
    a.wl1 = weight_l1;
    a.wssim = weight_ssim;
    a.wconst = weight_const;
    a.ga = (float)(weight_l1 / px);
    a.gb = (float)(weight_ssim / pts);
    // normalised Gaussian of sigma 1.5 over the 11 taps
    double gs[SS_W], tot = 0.0;
    for (int i = 0; i < SS_W; ++i) {
        const double d = i - SS_R;
        gs[i] = std::exp(-d * d / (2.0 * 1.5 * 1.5));
        tot += gs[i];
    }
    for (int i = 0; i < SS_W; ++i) a.g[i] = (float)(gs[i] / tot);
    a.counter = static_cast<unsigned *>(workspace);
    a.partials = reinterpret_cast<float *>(static_cast<char *>(workspace) + 256);
    a.out = out;
    const dim3 grid(a.tiles_x, a.tiles_y, n_images * channels);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (grad) {
        set_smem<true>();
        UBS_TIMED("ssim_loss_grad", st,
                  ssim_kernel<true><<<grid, SS_THREADS, Geom<true>::BYTES, st>>>(a));
    } else {
        set_smem<false>();
        UBS_TIMED("ssim_loss", st,
                  ssim_kernel<false><<<grid, SS_THREADS, Geom<false>::BYTES, st>>>(a));
    }
    note_launch();
    return check_launch("ssim_loss");
}

} // extern "C"
