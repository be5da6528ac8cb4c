// ssim.cu -- the training loss (1 - l) L1 + l (1 - SSIM) and its gradient.
//
// SSIM as the reference defines it (utils/loss_utils.py:26-80, the function
// the fused_ssim package used by train.py:117-121 evaluates): an 11 x 11
// Gaussian window (sigma 1.5) applied with zero padding ("same" output size)
// to x, y, x^2, y^2 and x y; C1 = 0.01^2, C2 = 0.03^2;
//   map = (2 mx my + C1)(2 sxy + C2) / ((mx^2 + my^2 + C1)(sxx + syy + C2))
// with sxx = E[x^2] - mx^2, sxy = E[xy] - mx my, and the loss reads the mean
// of the map (optionally cropped by the window radius, fused_ssim's "valid").
//
// Two kernels, each over 32 x 32 tiles of one (image, channel); quantities
// that are filtered with the same window travel in pairs through Blackwell's
// packed FP32x2 FMA ((x, y), (x^2, y^2), (D1, D2)):
//  * ssim_map_kernel: the five windowed moments of the tile (separable: a
//    horizontal then a vertical 11-tap pass over shared memory, the products
//    formed in registers), the map, the loss partials and -- for the
//    gradient -- the map's derivatives with the E[.] moments as the free
//    variables, D0 = d map / d mx, D1 = d map / d E[x^2],
//    D2 = d map / d E[xy], stored as a D0 plane and a (D1, D2) plane (12 B
//    per pixel-channel, mostly L2-resident between the two launches);
//  * ssim_grad_kernel: d loss / d x_p = gb sum_q w(q - p) (D0 + 2 x_p D1 +
//    y_p D2) + ga sign(x_p - y_p): the window over the three planes and the
//    combination with the image and target.
// Loss sums: one partial per CTA, reduced in a fixed order by the last CTA to
// finish (a ticket counter that the last CTA resets), so the result is
// deterministic and the launches can be replayed from a CUDA graph.
#include <cmath>

#include "ubs_common.cuh"

namespace ubs {
namespace {

constexpr int SS_T = 32;                // output tile edge
constexpr int SS_R = 5;                 // window radius (11 taps)
constexpr int SS_W = 2 * SS_R + 1;
constexpr int SS_IN = SS_T + 2 * SS_R;  // 42: tile plus halo
constexpr int SS_IP = SS_IN + 1;        // padded pitch of the halo planes
constexpr int SS_HP = SS_T + 1;         // padded pitch of the horizontal results
constexpr int SS_THREADS = 256;
constexpr int SS_LOADS = (SS_IN * SS_IN + SS_THREADS - 1) / SS_THREADS; // halo loads per thread

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
    float *dmap0;                // [n c][h][w] D0 plane (gradient only)
    float2 *dmap12;              // [n c][h][w] (D1, D2) plane
    float *partials;             // [n_ctas][2]
    unsigned *counter;
    float *out;                  // [3]: mean(map), mean|x-y|, loss
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

// 4 outputs of an 11-tap window over 14 consecutive values: scalar, and two
// streams at once with the packed FP32x2 FMA (same rounding per component)
__device__ __forceinline__ void taps4(const float (&g)[SS_W], const float (&v)[14],
                                      float (&acc)[4]) {
#pragma unroll
    for (int o = 0; o < 4; ++o) acc[o] = 0.f;
#pragma unroll
    for (int t = 0; t < SS_W; ++t)
#pragma unroll
        for (int o = 0; o < 4; ++o) acc[o] = fmaf(g[t], v[o + t], acc[o]);
}
__device__ __forceinline__ void taps4x2(const float (&g)[SS_W], const float2 (&v)[14],
                                        float2 (&acc)[4]) {
#pragma unroll
    for (int o = 0; o < 4; ++o) acc[o] = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < SS_W; ++t) {
        const float2 g2 = make_float2(g[t], g[t]);
#pragma unroll
        for (int o = 0; o < 4; ++o) acc[o] = __ffma2_rn(g2, v[o + t], acc[o]);
    }
}

// Asynchronous global -> shared copies of 4 or 8 bytes (no register staging,
// so every halo load of a thread is in flight at once); src_bytes 0 writes
// zeros, which is the window's zero padding outside the image.
template <int BYTES>
__device__ __forceinline__ void cp_async(void *dst, const void *src, bool in) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src),
                 "n"(BYTES), "r"(in ? BYTES : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\ncp.async.wait_group 0;\n" ::: "memory");
}

// the CTA's partials -> the last CTA reduces all of them in a fixed order
__device__ void finish_loss(const SsimArgs &a, float ssim_sum, float l1_sum) {
    __shared__ float red[SS_THREADS / 32];
    __shared__ bool last;
    __shared__ double dred[2][SS_THREADS / 32];
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

template <bool GRAD>
__global__ void __launch_bounds__(SS_THREADS, 4) ssim_map_kernel(const SsimArgs a) {
    __shared__ float2 sxy[SS_IN * SS_IP];          // (x, y) over tile + halo
    __shared__ float2 hA[SS_IN * SS_HP];           // horizontal (E x, E y)
    __shared__ float2 hB[SS_IN * SS_HP];           // horizontal (E x^2, E y^2)
    __shared__ float hP[SS_IN * SS_HP];            // horizontal E xy
    const int plane = blockIdx.z;
    const int img = plane / a.c, ch = plane % a.c;
    const int y0 = blockIdx.y * SS_T, x0 = blockIdx.x * SS_T;
    const float *X = a.img + img * a.is[0] + ch * a.is[1];
    const float *Y = a.gt + img * a.gs[0] + ch * a.gs[1];
    float g[SS_W];
#pragma unroll
    for (int t = 0; t < SS_W; ++t) g[t] = a.g[t];

    // ---- tile and halo of the image and the target (zero outside), as
    // asynchronous copies into the x and y halves of the pairs
#pragma unroll
    for (int k = 0; k < SS_LOADS; ++k) {
        const int i = threadIdx.x + k * SS_THREADS;
        if (i < SS_IN * SS_IN) {
            const int r = i / SS_IN, cc = i - r * SS_IN;
            const int gy = y0 - SS_R + r, gx = x0 - SS_R + cc;
            const bool in = gy >= 0 && gy < a.h && gx >= 0 && gx < a.w;
            const int64_t ox = in ? gy * a.is[2] + gx * a.is[3] : 0;
            const int64_t oy = in ? gy * a.gs[2] + gx * a.gs[3] : 0;
            float *d = reinterpret_cast<float *>(&sxy[r * SS_IP + cc]);
            cp_async<4>(d, X + ox, in);
            cp_async<4>(d + 1, Y + oy, in);
        }
    }
    cp_async_wait_all();
    __syncthreads();

    // ---- horizontal pass: (row, 4 outputs) per item; x and y (then x^2
    // and y^2) share packed FMAs, xy runs scalar
    for (int it = threadIdx.x; it < SS_IN * (SS_T / 4); it += SS_THREADS) {
        const int r = it % SS_IN, c0 = (it / SS_IN) * 4;
        float2 v[14], acc2[4];
        float p[14], acc[4];
#pragma unroll
        for (int j = 0; j < 14; ++j) {
            v[j] = sxy[r * SS_IP + c0 + j];
            p[j] = v[j].x * v[j].y;
        }
        const int o0 = r * SS_HP + c0;
        taps4x2(g, v, acc2);
#pragma unroll
        for (int o = 0; o < 4; ++o) hA[o0 + o] = acc2[o];
        taps4(g, p, acc);
#pragma unroll
        for (int o = 0; o < 4; ++o) hP[o0 + o] = acc[o];
#pragma unroll
        for (int j = 0; j < 14; ++j) v[j] = __fmul2_rn(v[j], v[j]);
        taps4x2(g, v, acc2);
#pragma unroll
        for (int o = 0; o < 4; ++o) hB[o0 + o] = acc2[o];
    }
    __syncthreads();

    // ---- vertical pass, map, derivatives: (column, 4 rows) per thread
    float ssim_sum = 0.f;
    {
        const int cx = threadIdx.x % SS_T, r0 = (threadIdx.x / SS_T) * 4;
        float2 mA[4], mB[4];
        float mP[4];
        {
            float2 v[14];
#pragma unroll
            for (int j = 0; j < 14; ++j) v[j] = hA[(r0 + j) * SS_HP + cx];
            taps4x2(g, v, mA);
#pragma unroll
            for (int j = 0; j < 14; ++j) v[j] = hB[(r0 + j) * SS_HP + cx];
            taps4x2(g, v, mB);
            float q[14];
#pragma unroll
            for (int j = 0; j < 14; ++j) q[j] = hP[(r0 + j) * SS_HP + cx];
            taps4(g, q, mP);
        }
        const int gx = x0 + cx;
        const int64_t hw = (int64_t)a.h * a.w;
#pragma unroll
        for (int o = 0; o < 4; ++o) {
            const int gy = y0 + r0 + o;
            const bool inside = gy < a.h && gx < a.w;
            bool counted = inside;
            if (a.valid)
                counted = counted && gy >= SS_R && gy < a.h - SS_R && gx >= SS_R && gx < a.w - SS_R;
            const float mx = mA[o].x, my = mA[o].y;
            const float mxx = mx * mx, myy = my * my, mxy = mx * my;
            const float vx = mB[o].x - mxx, vy = mB[o].y - myy, cxy = mP[o] - mxy;
            const float A1 = 2.f * mxy + a.c1, A2 = 2.f * cxy + a.c2;
            const float B1 = mxx + myy + a.c1, B2 = vx + vy + a.c2;
            const float s = (A1 * A2) / (B1 * B2);
            if (counted) ssim_sum += s;
            if (GRAD && inside) {
                float d0 = 0.f, d1 = 0.f, d2 = 0.f;
                if (counted) {
                    const float iB1 = 1.f / B1, iB2 = 1.f / B2, iBB = iB1 * iB2;
                    d0 = 2.f * my * (A2 - A1) * iBB - 2.f * mx * s * (iB1 - iB2);
                    d1 = -s * iB2;
                    d2 = 2.f * A1 * iBB;
                }
                const int64_t at = (int64_t)plane * hw + (int64_t)gy * a.w + gx;
                a.dmap0[at] = d0;
                a.dmap12[at] = make_float2(d1, d2);
            }
        }
    }
    // ---- L1 over the tile
    float l1_sum = 0.f;
    for (int i = threadIdx.x; i < SS_T * SS_T; i += SS_THREADS) {
        const int r = i / SS_T, cx = i % SS_T;
        if (y0 + r >= a.h || x0 + cx >= a.w) continue;
        const float2 v = sxy[(r + SS_R) * SS_IP + cx + SS_R];
        l1_sum += fabsf(v.x - v.y);
    }
    finish_loss(a, ssim_sum, l1_sum);
}

__global__ void __launch_bounds__(SS_THREADS, 4) ssim_grad_kernel(const SsimArgs a) {
    __shared__ float2 s12[SS_IN * SS_IP];  // (D1, D2) over tile + halo
    __shared__ float s0[SS_IN * SS_IP];    // D0
    __shared__ float2 h12[SS_IN * SS_HP];  // horizontal pass of (D1, D2)
    __shared__ float h0[SS_IN * SS_HP];
    // tiles in the reverse of the map kernel's order: the derivative planes
    // it wrote last are the likeliest to still be in L2
    const int plane = gridDim.z - 1 - blockIdx.z;
    const int img = plane / a.c, ch = plane % a.c;
    const int y0 = (gridDim.y - 1 - blockIdx.y) * SS_T, x0 = (gridDim.x - 1 - blockIdx.x) * SS_T;
    const int64_t hw = (int64_t)a.h * a.w;
    const float *D0 = a.dmap0 + (int64_t)plane * hw;
    const float2 *D12 = a.dmap12 + (int64_t)plane * hw;
    float g[SS_W];
#pragma unroll
    for (int t = 0; t < SS_W; ++t) g[t] = a.g[t];

    // ---- the derivative planes over the tile and halo (zero outside), as
    // asynchronous copies
#pragma unroll
    for (int k = 0; k < SS_LOADS; ++k) {
        const int i = threadIdx.x + k * SS_THREADS;
        if (i < SS_IN * SS_IN) {
            const int r = i / SS_IN, cc = i - r * SS_IN;
            const int gy = y0 - SS_R + r, gx = x0 - SS_R + cc;
            const bool in = gy >= 0 && gy < a.h && gx >= 0 && gx < a.w;
            const int64_t at = in ? (int64_t)gy * a.w + gx : 0;
            cp_async<8>(&s12[r * SS_IP + cc], D12 + at, in);
            cp_async<4>(&s0[r * SS_IP + cc], D0 + at, in);
        }
    }
    cp_async_wait_all();
    __syncthreads();
    // ---- horizontal pass: (row, 4 outputs) per item, D1 and D2 packed
    for (int it = threadIdx.x; it < SS_IN * (SS_T / 4); it += SS_THREADS) {
        const int r = it % SS_IN, c0 = (it / SS_IN) * 4;
        {
            float2 v[14], acc2[4];
#pragma unroll
            for (int j = 0; j < 14; ++j) v[j] = s12[r * SS_IP + c0 + j];
            taps4x2(g, v, acc2);
#pragma unroll
            for (int o = 0; o < 4; ++o) h12[r * SS_HP + c0 + o] = acc2[o];
        }
        {
            float q[14], acc[4];
#pragma unroll
            for (int j = 0; j < 14; ++j) q[j] = s0[r * SS_IP + c0 + j];
            taps4(g, q, acc);
#pragma unroll
            for (int o = 0; o < 4; ++o) h0[r * SS_HP + c0 + o] = acc[o];
        }
    }
    __syncthreads();
    // ---- vertical pass and the gradient: (column, 4 rows) per thread
    const int cx = threadIdx.x % SS_T, r0 = (threadIdx.x / SS_T) * 4;
    float2 G12[4];
    float G0[4];
    {
        float2 v[14];
#pragma unroll
        for (int j = 0; j < 14; ++j) v[j] = h12[(r0 + j) * SS_HP + cx];
        taps4x2(g, v, G12);
    }
    {
        float q[14];
#pragma unroll
        for (int j = 0; j < 14; ++j) q[j] = h0[(r0 + j) * SS_HP + cx];
        taps4(g, q, G0);
    }
    const float *X = a.img + img * a.is[0] + ch * a.is[1];
    const float *Y = a.gt + img * a.gs[0] + ch * a.gs[1];
    float *Gd = a.grad + img * a.ds[0] + ch * a.ds[1];
    const int gx = x0 + cx;
#pragma unroll
    for (int o = 0; o < 4; ++o) {
        const int gy = y0 + r0 + o;
        if (gy >= a.h || gx >= a.w) continue;
        const float xv = __ldg(X + gy * a.is[2] + gx * a.is[3]);
        const float yv = __ldg(Y + gy * a.gs[2] + gx * a.gs[3]);
        const float d = xv - yv;
        const float sg = d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f);
        Gd[gy * a.ds[2] + gx * a.ds[3]] =
            fmaf(a.gb, fmaf(2.f * xv, G12[o].x, fmaf(yv, G12[o].y, G0[o])), a.ga * sg);
    }
}

// ---- L1 alone (train.py's l1_loss, utils/loss_utils.py:18-19): mean |x - y|
// over contiguous arrays and its gradient sign(x - y) w / n, one pass; the
// sums reduced like the SSIM partials (fixed order, last CTA).
constexpr int L1_THREADS = 256;
constexpr int L1_PER = 8; // float4 per thread per pass

__global__ void __launch_bounds__(L1_THREADS) l1_kernel(const float *__restrict__ x,
                                                        const float *__restrict__ y,
                                                        float *__restrict__ grad, int64_t n,
                                                        float gscale, double inv_n, double w,
                                                        float *partials, unsigned *counter,
                                                        float *out) {
    float acc = 0.f;
    const int64_t n4 = n >> 2;
    const bool vec = ((reinterpret_cast<uintptr_t>(x) | reinterpret_cast<uintptr_t>(y) |
                       reinterpret_cast<uintptr_t>(grad)) & 15) == 0;
    const int64_t stride = (int64_t)gridDim.x * L1_THREADS;
    if (vec) {
        // two quads per step, both loads issued before either is used
        auto quad = [&](const float4 &a, const float4 &b, int64_t i) {
            const float d0 = a.x - b.x, d1 = a.y - b.y, d2 = a.z - b.z, d3 = a.w - b.w;
            acc += fabsf(d0) + fabsf(d1) + fabsf(d2) + fabsf(d3);
            if (grad) {
                auto sg = [](float d) { return d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f); };
                reinterpret_cast<float4 *>(grad)[i] = make_float4(
                    gscale * sg(d0), gscale * sg(d1), gscale * sg(d2), gscale * sg(d3));
            }
        };
        for (int64_t i = (int64_t)blockIdx.x * L1_THREADS + threadIdx.x; i < n4; i += 2 * stride) {
            const int64_t j = i + stride;
            const float4 a = reinterpret_cast<const float4 *>(x)[i];
            const float4 b = reinterpret_cast<const float4 *>(y)[i];
            float4 a2 = make_float4(0.f, 0.f, 0.f, 0.f), b2 = a2;
            if (j < n4) {
                a2 = reinterpret_cast<const float4 *>(x)[j];
                b2 = reinterpret_cast<const float4 *>(y)[j];
            }
            quad(a, b, i);
            if (j < n4) quad(a2, b2, j);
        }
    }
    for (int64_t i = (vec ? n4 * 4 : 0) + (int64_t)blockIdx.x * L1_THREADS + threadIdx.x; i < n;
         i += stride) {
        const float d = x[i] - y[i];
        acc += fabsf(d);
        if (grad) grad[i] = gscale * (d > 0.f ? 1.f : (d < 0.f ? -1.f : 0.f));
    }
    __shared__ float red[L1_THREADS / 32];
    __shared__ bool last;
    __shared__ double dred[L1_THREADS / 32];
    const float bs = block_sum(acc, red);
    if (threadIdx.x == 0) {
        partials[blockIdx.x] = bs;
        __threadfence();
        last = atomicAdd(counter, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    double s = 0.0;
    for (unsigned i = threadIdx.x; i < gridDim.x; i += L1_THREADS) s += (double)__ldcg(partials + i);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) dred[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < L1_THREADS / 32; ++i) t += dred[i];
        out[0] = (float)(t * inv_n);
        out[1] = (float)(w * t * inv_n);
        *counter = 0u;
    }
}

int l1_grid(int64_t n) {
    int dev = 0, sms = 152;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int64_t want = (n / 4 + (int64_t)L1_THREADS * L1_PER - 1) / ((int64_t)L1_THREADS * L1_PER);
    const int64_t cap = (int64_t)sms * 8;
    return (int)(want < 1 ? 1 : (want < cap ? want : cap));
}

size_t ws_header() { return 256; }

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_ssim_workspace_bytes(int32_t n_images, int32_t channels, int32_t height,
                                int32_t width) {
    if (n_images <= 0 || channels <= 0 || height <= 0 || width <= 0) return ws_header();
    const size_t ctas = (size_t)n_images * channels * ((height + SS_T - 1) / SS_T) *
                        ((width + SS_T - 1) / SS_T);
    const size_t part = (ctas * 2 * sizeof(float) + 255) & ~(size_t)255;
    const size_t maps = (size_t)3 * n_images * channels * height * width * sizeof(float);
    return ws_header() + part + maps;
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
    const size_t ctas = (size_t)n_images * channels * a.tiles_x * a.tiles_y;
    a.counter = static_cast<unsigned *>(workspace);
    a.partials = reinterpret_cast<float *>(static_cast<char *>(workspace) + ws_header());
    char *maps = static_cast<char *>(workspace) + ws_header() +
                 ((ctas * 2 * sizeof(float) + 255) & ~(size_t)255);
    const size_t px_all = (size_t)n_images * channels * height * width;
    a.dmap12 = reinterpret_cast<float2 *>(maps);
    a.dmap0 = reinterpret_cast<float *>(maps + px_all * sizeof(float2));
    a.out = out;
    const dim3 grid(a.tiles_x, a.tiles_y, n_images * channels);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (grad) {
        UBS_TIMED("ssim_map", st, ssim_map_kernel<true><<<grid, SS_THREADS, 0, st>>>(a));
        UBS_TIMED("ssim_grad", st, ssim_grad_kernel<<<grid, SS_THREADS, 0, st>>>(a));
        note_launch(2);
    } else {
        UBS_TIMED("ssim_map", st, ssim_map_kernel<false><<<grid, SS_THREADS, 0, st>>>(a));
        note_launch();
    }
    return check_launch("ssim_loss");
}

size_t ubs_l1_loss_workspace_bytes(int64_t n) {
    return ws_header() + (((size_t)l1_grid(n < 1 ? 1 : n) * sizeof(float) + 255) & ~(size_t)255);
}

int ubs_l1_loss(const float *x, const float *y, float *grad, int64_t n, double weight,
                float *out, void *workspace, size_t workspace_bytes, void *stream) {
    UBS_REQUIRE(n > 0 && x && y && out, "l1_loss: bad arguments");
    UBS_REQUIRE(workspace && workspace_bytes >= ubs_l1_loss_workspace_bytes(n),
                "l1_loss: workspace too small");
    const int grid = l1_grid(n);
    unsigned *counter = static_cast<unsigned *>(workspace);
    float *partials = reinterpret_cast<float *>(static_cast<char *>(workspace) + ws_header());
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // d mean / d x as torch forms it: the mean's 1/n in float, times the weight
    const float gscale = (float)weight * (float)(1.0 / (double)n);
    UBS_TIMED("l1_loss", st,
              l1_kernel<<<grid, L1_THREADS, 0, st>>>(x, y, grad, n, gscale, 1.0 / (double)n,
                                                     weight, partials, counter, out));
    note_launch();
    return check_launch("l1_loss");
}

} // extern "C"
