// scene.cu -- fused multi-view render path for Universal Beta Splatting scenes.
//
// The reference renders one view per call through separate operators
// (scene/beta_model.py:660-722 -> rendering.py:17-232): PyTorch activations,
// l_triangle_to_rotmat, rot_scale_l_triangle_to_covar (a materialised
// [N, D, D] covariance), cond_mean_convariance_opacity, a [N, 6] gather,
// fully_fused_projection, isect_tiles (+ host sync), isect_offset_encode and
// rasterize_to_pixels.  Here the same mathematics runs as:
//   1. scene_prim_fwd: one thread per (view, primitive) -- activations,
//      rotation, D x D covariance, conditioning on the view ray (and time),
//      EWA projection, tile counting into per-(view, tile) buckets;
//   2. a device-side scan, bucketed emit and per-bucket sort of (depth,
//      entry) keys (no host round trip; the intersection count stays on the
//      device);
//   3. the blend over a flattened (view, tile) work list whose views may have
//      different resolutions, copying each batch of records from the
//      per-entry tables by the sorted keys (no sorted copy of the records);
//   4. scene_prim_bwd: one thread per (view, primitive) recomputes the forward
//      chain and back-propagates blend gradients to the raw parameters.
// Every launch is stream ordered with fixed grids, so a whole forward or
// backward can be captured in a CUDA graph.
//
// The l_triangle layout is the reference model's (scene/beta_model.py:69-73):
// entries 0..2 are the rotation's skew parameters (a01, a02, a12); the rest are
// the strictly-lower entries of rows 3..D-1 in row-major order.
#include <algorithm>

#include "prim_math.cuh"
#include "sort_common.cuh"

namespace ubs {

// raster.cu: the blend kernels in multi-view mode, gathering each batch's
// records from the per-entry tables through the sorted keys
int scene_blend(int fwd, int32_t C, int64_t CN, int32_t n_buckets, int32_t tile_size,
                const int32_t *offsets, const int32_t *order, const int64_t *T_dev, int64_t cap,
                const uint64_t *keys, const void *entry_recs, const float4 *prim_cols,
                const float *bg, const int32_t *tile_base,
                const int32_t *dims, const int64_t *pix_base, float *out_c, float *out_a,
                int32_t *last_ids, const float *render_alphas, const int32_t *last_in,
                const float *v_out_c, const float *v_out_a, float *v_rows, uint32_t *status,
                cudaStream_t st);

// scene_act.cu (compiled with IEEE math): activated scales, betas and
// opacities, act = [N, D] | [N, D - 2] | [N] at the 16-byte aligned section
// offsets 0, act_beta_off, act_opac_off
int launch_scene_act(int64_t N, int D, const float *scale, const float *beta, const float *opac,
                     float *act, cudaStream_t st);

namespace {

constexpr int kTileMaxViews = 1 << 16;
// Replicas of the per-bucket intersection counters and cursors: entry idx
// counts and emits through replica idx % kCountReplicas, which spreads a
// bucket's atomics over that many L2 lines (a 1080p frame has about 520
// intersections per bucket).  A bucket's keys stay one contiguous range: the
// replicas own consecutive sub-ranges of it.
constexpr int kCountReplicas = 8;
// floats per primitive of the activation section (D + D - 2 + 1, D <= 7),
// plus up to 8 floats of section alignment
constexpr int kActPerPrim = 13;
// floats per gradient row of the backward blend (GRAD_ROW in raster.cu)
constexpr int kGradRow = 12;

struct __align__(16) Rec {
    float x, y, opac, beta;
    float cxx, cxy, cyy;
    int32_t gid;
};

struct SceneHeader {
    int64_t total;   // intersections counted on the device
    uint32_t status; // DeviceError bits
    int32_t n_big;   // buckets longer than SMALL_SEG
    int32_t n_mid;   // buckets longer than WARP_SEG, at most SMALL_SEG
    int32_t pad0;
    int64_t pad[5];
};

struct SceneArgs {
    int64_t N;
    int C;
    const float *xyz, *mean, *scale, *ltri, *opac, *beta, *rgb;
    const float *viewmats, *intr, *centers, *times;
    const int32_t *dims, *tile_base;
    float tile_size, eps2d, near_p, far_p, radius_clip;
    const float *act;         // activated scale [N,D] | beta [N,D-2] | opacity [N]
    const float *act_b, *act_o; // its beta and opacity sections (act_beta_off, act_opac_off)
    const uint8_t *prim_mask; // optional: primitives with 0 are not rendered
    int color_mode;           // 0: rgb; 1: depth in channel 0 (one view, forward only)
    // outputs / workspace
    Rec *recs;
    float4 *cols_n; // colour row per primitive (written by the view-0 entries)
    int32_t *radius;
    float *depth;
    int32_t *bucket_counts; // [kCountReplicas][n_buckets]
    int32_t n_buckets;
    uint32_t *status;
    // backward
    // gradient row per (view, primitive) entry from the backward blend:
    // [v_xy(2), v_conic(3), v_opacity, v_beta, v_rgb(3), 0, 0]
    const float *v_rows;
    float *g_xyz, *g_mean, *g_scale, *g_ltri, *g_opac, *g_beta, *g_rgb;
    int exact;
};

__device__ __forceinline__ float sigmoid_f(float x) { return 1.f / (1.f + expf(-x)); }

__device__ __forceinline__ Cam view_cam(const SceneArgs &a, int v) {
    Cam c;
    const float *vm = a.viewmats + (int64_t)v * 16;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
#pragma unroll
        for (int k = 0; k < 3; ++k) c.R(r, k) = vm[r * 4 + k];
        c.t[r] = vm[r * 4 + 3];
    }
    c.fx = a.intr[v * 4 + 0];
    c.fy = a.intr[v * 4 + 1];
    c.cx = a.intr[v * 4 + 2];
    c.cy = a.intr[v * 4 + 3];
    return c;
}

// The conditioning query of the reference model, view_dir / |view_dir| with
// view_dir = xyz - camera_center (scene/beta_model.py:676-678), rounded as
// PyTorch's kernels round it: IEEE subtraction, the norm as PyTorch's
// reduction sums the three squares (pairwise, (x0^2 + x2^2) + x1^2), IEEE
// square root and division.  Explicitly rounded intrinsics keep fast math
// from contracting or approximating any step.
__device__ __forceinline__ void view_direction(const float *xyz, const float *center, float *q) {
    const float d0 = __fsub_rn(xyz[0], center[0]);
    const float d1 = __fsub_rn(xyz[1], center[1]);
    const float d2 = __fsub_rn(xyz[2], center[2]);
    const float ss = __fadd_rn(__fadd_rn(__fmul_rn(d0, d0), __fmul_rn(d2, d2)), __fmul_rn(d1, d1));
    const float nrm = __fsqrt_rn(ss);
    q[0] = __fdiv_rn(d0, nrm);
    q[1] = __fdiv_rn(d1, nrm);
    q[2] = __fdiv_rn(d2, nrm);
}

// Forward state of one (view, primitive), shared by both kernels.
template <int D> struct PrimFwd {
    static constexpr int K = D - 3;
    float s[D];        // activated scales
    float L[D * D];    // covariance factor
    float V[D * D];    // D x D covariance
    float m[D];        // means (xyz, angular / temporal)
    float o;           // activated opacity
    float b[K];        // activated conditional betas
    float b0;          // activated spatial beta
    float q[K];        // query (view direction [, time])
    float om[3], oV[9], oo; // conditioned mean, covariance, opacity
};

// One primitive's parameter rows: xyz (3), mean (K), activated scale (D),
// l_triangle (NL), activated beta (D - 2), and its activated opacity.
struct PrimRows {
    const float *xyz, *mean, *s, *lt, *b;
    float o;
};

// Floats of one warp's parameter stage: the rows of 32 primitives.
template <int D> constexpr int stage_floats() {
    return 32 * (3 + (D - 3) + D + D * (D - 1) / 2 + (D - 2));
}

// The rows of the 32 consecutive primitives [n0, n0 + 32) of a [N, W] array
// are one contiguous span: the warp reads it with W coalesced 128-byte loads
// into its stage, and each lane then reads its own row from shared memory
// (after the caller's __syncwarp; no CTA barrier, so warps keep overlapping).
template <int W>
__device__ __forceinline__ const float *stage_rows(const float *__restrict__ src, int64_t n0,
                                                   float *st, int lane) {
    const float *p = src + n0 * W;
#pragma unroll
    for (int k = 0; k < W; ++k) st[k * 32 + lane] = __ldg(p + k * 32 + lane);
    return st + lane * W;
}

// Rows of primitive n: staged for the warp when its 32 entries are 32
// consecutive primitives of one view (every warp but the one straddling a
// view boundary or the end), else read in place.  Returns whether staged;
// the caller syncs the warp before reading staged rows.
template <int D>
__device__ __forceinline__ bool prim_rows(const SceneArgs &a, int64_t idx, int64_t n, int lane,
                                          float *stage, PrimRows &r) {
    constexpr int K = D - 3, NL = D * (D - 1) / 2;
    const float *act_s = a.act, *act_b = a.act_b, *act_o = a.act_o;
    const int64_t w0 = idx - lane, n0 = n - lane;
    const bool staged = w0 + 32 <= (int64_t)a.C * a.N && n0 >= 0 && n0 + 32 <= a.N;
    if (__all_sync(0xffffffffu, staged)) {
        float *st = stage;
        r.xyz = stage_rows<3>(a.xyz, n0, st, lane);
        st += 32 * 3;
        r.mean = stage_rows<K>(a.mean, n0, st, lane);
        st += 32 * K;
        r.s = stage_rows<D>(act_s, n0, st, lane);
        st += 32 * D;
        r.lt = stage_rows<NL>(a.ltri, n0, st, lane);
        st += 32 * NL;
        r.b = stage_rows<D - 2>(act_b, n0, st, lane);
        r.o = act_o[n];
        return true;
    }
    if (n >= 0 && n < a.N) {
        r.xyz = a.xyz + n * 3;
        r.mean = a.mean + n * K;
        r.s = act_s + n * D;
        r.lt = a.ltri + n * NL;
        r.b = act_b + n * (D - 2);
        r.o = act_o[n];
    }
    return false;
}

template <int D>
__device__ __forceinline__ void prim_forward(const SceneArgs &a, const PrimRows &rw, int v,
                                             PrimFwd<D> &f) {
    constexpr int K = D - 3;
    constexpr int NL = D * (D - 1) / 2;
    float lt[NL];
    // activations as the reference's PyTorch kernels round them (scene_act.cu)
#pragma unroll
    for (int k = 0; k < NL; ++k) lt[k] = rw.lt[k];
#pragma unroll
    for (int k = 0; k < D; ++k) f.s[k] = rw.s[k];
    // L: top-left R diag(s[0:3]) with R = I + A(a01, a02, a12); L[r][r] = s[r] (r >= 3);
    // rest entries row-major below the diagonal
    const float R[9] = {1.f, lt[0], lt[1], -lt[0], 1.f, lt[2], -lt[1], -lt[2], 1.f};
#pragma unroll
    for (int k = 0; k < D * D; ++k) f.L[k] = 0.f;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) f.L[r * D + c] = R[r * 3 + c] * f.s[c];
    int m = 3;
#pragma unroll
    for (int r = 3; r < D; ++r) {
#pragma unroll
        for (int c = 0; c < r; ++c) f.L[r * D + c] = lt[m++];
        f.L[r * D + r] = f.s[r];
    }
    covar_from_L<D>(f.L, f.V);
#pragma unroll
    for (int k = 0; k < 3; ++k) f.m[k] = rw.xyz[k];
#pragma unroll
    for (int k = 0; k < K; ++k) f.m[3 + k] = rw.mean[k];
    f.o = rw.o;
    f.b0 = rw.b[0];
#pragma unroll
    for (int k = 0; k < K; ++k) f.b[k] = rw.b[1 + k];
    // view direction query (+ timestamp for the 7-D model)
    const float *cc = a.centers + v * 3;
    view_direction(f.m, cc, f.q);
    if (K == 4) f.q[3 % K] = a.times[v];
    cond_forward<K>(f.m, f.V, f.o, f.b, f.q, f.om, f.oV, &f.oo);
}

// conditioned covariance -> world covariance used by the projection: the
// reference hands the upper triangle of the [3, 3] result to the projection
__device__ __forceinline__ M3 upper_sym(const float *oV) {
    M3 S;
    S(0, 0) = oV[0]; S(0, 1) = oV[1]; S(0, 2) = oV[2];
    S(1, 0) = oV[1]; S(1, 1) = oV[4]; S(1, 2) = oV[5];
    S(2, 0) = oV[2]; S(2, 1) = oV[5]; S(2, 2) = oV[8];
    return S;
}

constexpr int PRIM_THREADS = 128;

template <int D>
__global__ void __launch_bounds__(PRIM_THREADS, D == 6 ? 8 : 6) scene_prim_fwd_kernel(SceneArgs a) {
    __shared__ float stage[PRIM_THREADS / 32][stage_floats<D>()];
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int v = (int)(idx / a.N);
    const int64_t n = idx - (int64_t)v * a.N;
    PrimRows rows;
    if (prim_rows<D>(a, idx, n, lane, stage[threadIdx.x >> 5], rows)) __syncwarp();
    if (idx >= (int64_t)a.C * a.N) return;
    PrimFwd<D> f;
    prim_forward<D>(a, rows, v, f);
    const Cam cam = view_cam(a, v);
    const uint32_t W = (uint32_t)a.dims[v * 4], H = (uint32_t)a.dims[v * 4 + 1];
    const uint32_t TW = (uint32_t)a.dims[v * 4 + 2], TH = (uint32_t)a.dims[v * 4 + 3];
    float pc[3];
    world_to_cam(cam, f.om, pc);
    Proj2D p;
    p.radius = 0;
    const bool shown = !a.prim_mask || a.prim_mask[n] != 0;
    if (shown && !(pc[2] < a.near_p || pc[2] > a.far_p)) {
        const M3 Sw = upper_sym(f.oV);
        const M3 Sc = mm(mm(cam.R, Sw), tr(cam.R));
        p = project_2d(pc, Sc, cam, W, H, a.eps2d, a.radius_clip);
    }
    Rec r;
    r.gid = (int32_t)idx;
    r.opac = f.oo;
    r.beta = f.b0;
    if (p.radius > 0) {
        r.x = p.mx;
        r.y = p.my;
        r.cxx = p.conic[0];
        r.cxy = p.conic[1];
        r.cyy = p.conic[2];
    } else {
        r.x = r.y = r.cxx = r.cxy = r.cyy = 0.f;
    }
    float4 *dst = reinterpret_cast<float4 *>(a.recs + idx);
    dst[0] = make_float4(r.x, r.y, r.opac, r.beta);
    dst[1] = make_float4(r.cxx, r.cxy, r.cyy, __int_as_float(r.gid));
    if (v == 0) { // one colour row per primitive, gathered by the blend
        if (a.color_mode == 1)
            a.cols_n[n] = make_float4(p.radius > 0 ? p.depth : 0.f, 0.f, 0.f, 0.f);
        else
            a.cols_n[n] = make_float4(a.rgb[n * 3], a.rgb[n * 3 + 1], a.rgb[n * 3 + 2], 0.f);
    }
    a.radius[idx] = p.radius;
    a.depth[idx] = p.radius > 0 ? p.depth : 0.f;
    if (p.radius <= 0) return;
    // tile box (isect_tiles.cu:46-66) and bucket counts
    const float ts = a.tile_size;
    const float rr = (float)p.radius / ts, tx = p.mx / ts, ty = p.my / ts;
    const uint32_t x0 = min(max(0u, __float2uint_rz(floorf(tx - rr))), TW);
    const uint32_t y0 = min(max(0u, __float2uint_rz(floorf(ty - rr))), TH);
    const uint32_t x1 = min(max(0u, __float2uint_rz(ceilf(tx + rr))), TW);
    const uint32_t y1 = min(max(0u, __float2uint_rz(ceilf(ty + rr))), TH);
    if (x1 <= x0 || y1 <= y0) return;
    if (__float_as_int(p.depth) < 0) atomicOr(a.status, DEV_ERR_NEG_DEPTH);
    int32_t *bc = a.bucket_counts + (int64_t)(idx % kCountReplicas) * a.n_buckets + a.tile_base[v];
    for (uint32_t y = y0; y < y1; ++y)
        for (uint32_t x = x0; x < x1; ++x) atomicAdd(&bc[y * TW + x], 1);
}

// Writes one sort key per (view, primitive, tile) at the tile's cursor.  A
// warp flattens the tile rectangles of its 32 (view, primitive) entries into
// one list of (entry, tile) pairs and emits 32 pairs per round, so a warp's
// rounds follow the warp's total tile count rather than its largest entry and
// the 32 cursor atomics of a round are independent.
__global__ void scene_emit_kernel(int64_t CN, int64_t N, const Rec *__restrict__ recs,
                                  const int32_t *__restrict__ radius,
                                  const float *__restrict__ depth,
                                  const int32_t *__restrict__ dims,
                                  const int32_t *__restrict__ tile_base, int32_t nb, float ts,
                                  int32_t *__restrict__ cursor, uint64_t *__restrict__ keys,
                                  int64_t cap, uint32_t *status) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t bw = 1, n = 0, pitch = 0;
    int32_t *cur = cursor;
    uint64_t key = 0;
    if (idx < CN && radius[idx] > 0) {
        const int v = (int)(idx / N);
        const uint32_t TW = (uint32_t)dims[v * 4 + 2], TH = (uint32_t)dims[v * 4 + 3];
        const float4 xy = reinterpret_cast<const float4 *>(recs + idx)[0];
        const float rr = (float)radius[idx] / ts, tx = xy.x / ts, ty = xy.y / ts;
        const uint32_t x0 = min(max(0u, __float2uint_rz(floorf(tx - rr))), TW);
        const uint32_t y0 = min(max(0u, __float2uint_rz(floorf(ty - rr))), TH);
        const uint32_t x1 = min(max(0u, __float2uint_rz(ceilf(tx + rr))), TW);
        const uint32_t y1 = min(max(0u, __float2uint_rz(ceilf(ty + rr))), TH);
        if (x1 > x0 && y1 > y0) {
            bw = x1 - x0;
            n = bw * (y1 - y0);
            cur = cursor + (idx % kCountReplicas) * nb + tile_base[v] + (int64_t)y0 * TW + x0;
            key = ((uint64_t)(uint32_t)__float_as_int(depth[idx]) << 32) | (uint64_t)idx;
            pitch = TW;
        }
    }
    warp_emit_rects(n, bw, pitch, cur, key, lane, keys, cap, status);
}


// Sorted-entry writer of the fused path: the sort leaves each sorted key in
// place; the blend kernels gather each batch's records and colours from the
// per-entry tables by the keys' low words.
struct KeyWriter {
    uint64_t *keys;
    __device__ __forceinline__ void operator()(uint64_t key, int64_t pos, int64_t) const {
        keys[pos] = key;
    }
};

template <int D> __global__ void __launch_bounds__(PRIM_THREADS) scene_prim_bwd_kernel(SceneArgs a) {
    constexpr int K = D - 3;
    constexpr int NL = D * (D - 1) / 2;
    __shared__ float stage[PRIM_THREADS / 32][stage_floats<D>()];
    __shared__ float sraw[PRIM_THREADS / 32][32 * D]; // raw scale rows (softplus derivative)
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    const int v = (int)(idx / a.N);
    const int64_t n = idx - (int64_t)v * a.N;
    // the entry's own rows are requested before the warp stages the
    // parameter rows, so both sets of loads are in flight together
    const bool in = idx < (int64_t)a.C * a.N;
    int32_t rad = 0;
    float4 vr0 = make_float4(0.f, 0.f, 0.f, 0.f), vr1 = vr0, vr2 = vr0, c1 = vr0;
    if (in) {
        rad = a.radius[idx];
        const float4 *vrow = reinterpret_cast<const float4 *>(a.v_rows + idx * kGradRow);
        vr0 = vrow[0];
        vr1 = vrow[1];
        vr2 = vrow[2];
        c1 = reinterpret_cast<const float4 *>(a.recs + idx)[1];
    }
    PrimRows rows;
    const float *raw_s = a.scale + n * D;
    if (prim_rows<D>(a, idx, n, lane, stage[threadIdx.x >> 5], rows)) {
        raw_s = stage_rows<D>(a.scale, n - lane, sraw[threadIdx.x >> 5], lane);
        __syncwarp();
    }
    if (!in) return;
    const bool direct = a.C == 1; // one view: plain stores, else atomics into zeroed grads
    if (rad <= 0) {
        if (direct) {
#pragma unroll
            for (int k = 0; k < 3; ++k) a.g_xyz[n * 3 + k] = 0.f;
#pragma unroll
            for (int k = 0; k < K; ++k) a.g_mean[n * K + k] = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) a.g_scale[n * D + k] = 0.f;
#pragma unroll
            for (int k = 0; k < NL; ++k) a.g_ltri[n * NL + k] = 0.f;
            a.g_opac[n] = 0.f;
#pragma unroll
            for (int k = 0; k < D - 2; ++k) a.g_beta[n * (D - 2) + k] = 0.f;
#pragma unroll
            for (int k = 0; k < 3; ++k) a.g_rgb[n * 3 + k] = 0.f;
        }
        return;
    }
    PrimFwd<D> f;
    prim_forward<D>(a, rows, v, f);
    const Cam cam = view_cam(a, v);
    const uint32_t W = (uint32_t)a.dims[v * 4], H = (uint32_t)a.dims[v * 4 + 1];
    // projection VJP (fully_fused_projection_bwd.cu:69-174) with the saved conic
    const float cn[3] = {c1.x, c1.y, c1.z};
    const float vcn[3] = {vr0.z, vr0.w, vr1.x};
    float vc2[4];
    conic_vjp(cn, vcn, a.eps2d, false, 0.f, 0.f, vc2);
    float pc[3];
    world_to_cam(cam, f.om, pc);
    const M3 Sw = upper_sym(f.oV);
    const M3 Sc = mm(mm(cam.R, Sw), tr(cam.R));
    M3 vSc;
#pragma unroll
    for (int k = 0; k < 9; ++k) vSc.m[k] = 0.f;
    float vpc[3] = {0.f, 0.f, 0.f};
    persp_vjp(pc, Sc, cam, W, H, vc2, vr0.x, vr0.y, vSc, vpc);
    float gM[3];
#pragma unroll
    for (int k = 0; k < 3; ++k)
        gM[k] = cam.R(0, k) * vpc[0] + cam.R(1, k) * vpc[1] + cam.R(2, k) * vpc[2];
    const M3 vSw = mm(mm(tr(cam.R), vSc), cam.R);
    // upper-triangle gather VJP: packed entries back onto the upper triangle
    float gVc[9];
    gVc[0] = vSw(0, 0);
    gVc[1] = vSw(0, 1) + vSw(1, 0);
    gVc[2] = vSw(0, 2) + vSw(2, 0);
    gVc[3] = 0.f;
    gVc[4] = vSw(1, 1);
    gVc[5] = vSw(1, 2) + vSw(2, 1);
    gVc[6] = 0.f;
    gVc[7] = 0.f;
    gVc[8] = vSw(2, 2);
    // conditioning VJP (cond_mean_convariance_opacity_bwd.cu:102-563)
    float gm[D], gV[D * D], go, gb[K];
    cond_backward<K>(f.m, f.V, f.o, f.b, f.q, gM, gVc, vr1.y, a.exact != 0, gm, gV, &go,
                     gb);
    // Sigma = L L^T: dL = (gV + gV^T) L (rot_scale_l_triangle_to_covar_bwd.cu)
    float dL[D * D];
#pragma unroll
    for (int r = 0; r < D; ++r)
#pragma unroll
        for (int c = 0; c < D; ++c) {
            float acc = 0.f;
#pragma unroll
            for (int k = 0; k < D; ++k) acc += (gV[r * D + k] + gV[k * D + r]) * f.L[k * D + c];
            dL[r * D + c] = acc;
        }
    float gs[D], gl[NL];
    const float *lt_raw = rows.lt;
    const float R[9] = {1.f, lt_raw[0], lt_raw[1], -lt_raw[0], 1.f, lt_raw[2], -lt_raw[1],
                        -lt_raw[2], 1.f};
    float dR[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) dR[r * 3 + c] = dL[r * D + c] * f.s[c];
#pragma unroll
    for (int c = 0; c < 3; ++c)
        gs[c] = dL[0 * D + c] * R[0 * 3 + c] + dL[1 * D + c] * R[1 * 3 + c] +
                dL[2 * D + c] * R[2 * 3 + c];
#pragma unroll
    for (int r = 3; r < D; ++r) gs[r] = dL[r * D + r];
    // l_triangle_to_rotmat VJP (l_triagnle_to_rotmat_bwd.cu:8-25) + rest entries
    gl[0] = dR[1] - dR[3];
    gl[1] = dR[2] - dR[6];
    gl[2] = dR[5] - dR[7];
    int m = 3;
#pragma unroll
    for (int r = 3; r < D; ++r)
#pragma unroll
        for (int c = 0; c < r; ++c) gl[m++] = dL[r * D + c];
    // activation VJPs and stores
    auto put = [&](float *p, float val) {
        if (direct) *p = val;
        else if (val != 0.f) atomicAdd(p, val);
    };
#pragma unroll
    for (int k = 0; k < 3; ++k) put(&a.g_xyz[n * 3 + k], gm[k]);
#pragma unroll
    for (int k = 0; k < K; ++k) put(&a.g_mean[n * K + k], gm[3 + k]);
#pragma unroll
    for (int k = 0; k < D; ++k) put(&a.g_scale[n * D + k], gs[k] * sigmoid_f(raw_s[k]));
#pragma unroll
    for (int k = 0; k < NL; ++k) put(&a.g_ltri[n * NL + k], gl[k]);
    put(&a.g_opac[n], go * f.o * (1.f - f.o));
    put(&a.g_beta[n * (D - 2)], vr1.z * f.b0);
#pragma unroll
    for (int k = 0; k < K; ++k) put(&a.g_beta[n * (D - 2) + 1 + k], gb[k] * f.b[k]);
    put(&a.g_rgb[n * 3], vr1.w);
    put(&a.g_rgb[n * 3 + 1], vr2.x);
    put(&a.g_rgb[n * 3 + 2], vr2.y);
}

size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

struct SceneWs {
    SceneHeader *hdr;
    Rec *recs;
    int32_t *radius;
    float *depth;
    int32_t *bucket_counts, *offsets, *cursor, *big_list, *order, *totals;
    int64_t *block_sums;
    uint64_t *keys, *scratch;
    float4 *cols_n;
    float *grads; // one kGradRow-float gradient row per (view, primitive) entry
    float *act;   // activated parameters (scene_act.cu)
    size_t bytes;
};

SceneWs scene_ws(void *base, int32_t C, int64_t N, int32_t nb, int64_t cap) {
    SceneWs w{};
    unsigned char *p = static_cast<unsigned char *>(base);
    const int64_t CN = (int64_t)C * N;
    size_t o = 0;
    auto take = [&](size_t bytes) {
        unsigned char *q = p + o;
        o = al256(o + bytes);
        return q;
    };
    w.hdr = reinterpret_cast<SceneHeader *>(take(sizeof(SceneHeader)));
    w.recs = reinterpret_cast<Rec *>(take(CN * sizeof(Rec)));
    w.radius = reinterpret_cast<int32_t *>(take(CN * 4));
    w.depth = reinterpret_cast<float *>(take(CN * 4));
    w.bucket_counts = reinterpret_cast<int32_t *>(take((size_t)nb * kCountReplicas * 4));
    w.offsets = reinterpret_cast<int32_t *>(take((size_t)(nb + 1) * 4));
    w.cursor = reinterpret_cast<int32_t *>(take((size_t)nb * kCountReplicas * 4));
    w.totals = reinterpret_cast<int32_t *>(take((size_t)nb * 4));
    w.big_list = reinterpret_cast<int32_t *>(take((size_t)nb * 4));
    w.order = reinterpret_cast<int32_t *>(take((size_t)nb * 4));
    w.block_sums = reinterpret_cast<int64_t *>(take(((nb + SCAN_TILE - 1) / SCAN_TILE + 1) * 8));
    w.keys = reinterpret_cast<uint64_t *>(take(cap * 8));
    w.scratch = reinterpret_cast<uint64_t *>(take(cap * 8));
    w.cols_n = reinterpret_cast<float4 *>(take((size_t)N * 16));
    w.grads = reinterpret_cast<float *>(take(CN * kGradRow * 4));
    w.act = reinterpret_cast<float *>(take(((size_t)N * kActPerPrim + 8) * 4));
    w.bytes = o;
    return w;
}

#define UBS_SCENE_DIM(D, ...)                                                             \
    switch (D) {                                                                          \
    case 6: { constexpr int DD = 6; __VA_ARGS__; } break;                                 \
    case 7: { constexpr int DD = 7; __VA_ARGS__; } break;                                 \
    default: return set_error(UBS_ERR_UNSUPPORTED, "scene: dimension %d (supported 6, 7)", D); \
    }

int scene_common(SceneArgs &a, int32_t dim, int64_t N, const float *xyz, const float *mean,
                 const float *scale, const float *ltri, const float *opac, const float *beta,
                 const float *rgb, int32_t C, const float *viewmats, const float *intr,
                 const float *centers, const float *times, const int32_t *dims,
                 const int32_t *tile_base, int32_t tile_size, float eps2d, float near_p,
                 float far_p, float radius_clip) {
    UBS_REQUIRE(N >= 0 && C >= 1 && C <= kTileMaxViews, "scene: bad sizes N=%lld C=%d",
                (long long)N, C);
    UBS_REQUIRE((int64_t)C * N < (1ll << 31), "scene: views x primitives must fit in int32");
    UBS_REQUIRE(tile_size == 8 || tile_size == 16 || tile_size == 24 || tile_size == 32,
                "scene: tile_size %d (supported 8, 16, 24, 32)", tile_size);
    // an empty scene (N = 0) may pass null parameter pointers: it renders the
    // background
    UBS_REQUIRE((N == 0 || (xyz && mean && scale && ltri && opac && beta && rgb)) && viewmats &&
                    intr && centers && dims && tile_base && (dim == 6 || times),
                "scene: null input pointer");
    a.N = N;
    a.C = C;
    a.xyz = xyz;
    a.mean = mean;
    a.scale = scale;
    a.ltri = ltri;
    a.opac = opac;
    a.beta = beta;
    a.rgb = rgb;
    a.viewmats = viewmats;
    a.intr = intr;
    a.centers = centers;
    a.times = times;
    a.dims = dims;
    a.tile_base = tile_base;
    a.tile_size = (float)tile_size;
    a.eps2d = eps2d;
    a.near_p = near_p;
    a.far_p = far_p;
    a.radius_clip = radius_clip;
    return UBS_OK;
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_scene_workspace_bytes(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity) {
    return scene_ws(nullptr, C, N, n_buckets, capacity < 1 ? 1 : capacity).bytes;
}

int ubs_scene_workspace_offsets(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity,
                                int64_t *radius_offset, int64_t *depth_offset) {
    UBS_REQUIRE(radius_offset && depth_offset, "scene_workspace_offsets: null output");
    const SceneWs w = scene_ws(nullptr, C, N, n_buckets, capacity < 1 ? 1 : capacity);
    *radius_offset = (int64_t)reinterpret_cast<uintptr_t>(w.radius);
    *depth_offset = (int64_t)reinterpret_cast<uintptr_t>(w.depth);
    return UBS_OK;
}

int ubs_scene_workspace_layout(int32_t C, int64_t N, int32_t n_buckets, int64_t capacity,
                               int64_t *sections, int32_t n_sections) {
    UBS_REQUIRE(sections && n_sections >= 0 && n_sections <= UBS_SCENE_WS_N_SECTIONS,
                "scene_workspace_layout: bad section array (n=%d)", n_sections);
    const SceneWs w = scene_ws(nullptr, C, N, n_buckets, capacity < 1 ? 1 : capacity);
    const void *at[UBS_SCENE_WS_N_SECTIONS] = {w.recs, w.radius, w.depth, w.offsets, w.keys};
    for (int i = 0; i < n_sections; ++i)
        sections[i] = (int64_t)reinterpret_cast<uintptr_t>(at[i]);
    return UBS_OK;
}

int ubs_scene_forward(int32_t dim, int64_t N, const float *xyz, const float *mean,
                      const float *scale, const float *l_triangle, const float *opacity,
                      const float *beta, const float *rgb, int32_t C, const float *viewmats,
                      const float *intrinsics, const float *centers, const float *timestamps,
                      const int32_t *view_dims, const int32_t *tile_base,
                      const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                      float eps2d, float near_plane, float far_plane, float radius_clip,
                      const float *backgrounds, float *render_colors, float *render_alphas,
                      int32_t *last_ids, int64_t capacity, void *workspace,
                      size_t workspace_bytes, void *stream) {
    return ubs_scene_forward_masked(dim, N, xyz, mean, scale, l_triangle, opacity, beta, rgb, C,
                                    viewmats, intrinsics, centers, timestamps, view_dims,
                                    tile_base, pix_base, n_buckets, tile_size, eps2d, near_plane,
                                    far_plane, radius_clip, backgrounds, render_colors,
                                    render_alphas, last_ids, capacity, workspace,
                                    workspace_bytes, nullptr, 0, stream);
}

int ubs_scene_forward_masked(int32_t dim, int64_t N, const float *xyz, const float *mean,
                             const float *scale, const float *l_triangle, const float *opacity,
                             const float *beta, const float *rgb, int32_t C,
                             const float *viewmats, const float *intrinsics,
                             const float *centers, const float *timestamps,
                             const int32_t *view_dims, const int32_t *tile_base,
                             const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                             float eps2d, float near_plane, float far_plane, float radius_clip,
                             const float *backgrounds, float *render_colors,
                             float *render_alphas, int32_t *last_ids, int64_t capacity,
                             void *workspace, size_t workspace_bytes, const uint8_t *prim_mask,
                             int32_t color_mode, void *stream) {
    SceneArgs a{};
    if (int e = scene_common(a, dim, N, xyz, mean, scale, l_triangle, opacity, beta, rgb, C,
                             viewmats, intrinsics, centers, timestamps, view_dims, tile_base,
                             tile_size, eps2d, near_plane, far_plane, radius_clip))
        return e;
    UBS_REQUIRE(color_mode == 0 || (color_mode == 1 && C == 1),
                "scene_forward: colour mode %d (0 rgb; 1 depth, one view)", color_mode);
    a.prim_mask = prim_mask;
    a.color_mode = color_mode;
    UBS_REQUIRE(n_buckets >= 1 && capacity >= 1 && pix_base && render_colors && render_alphas &&
                    last_ids,
                "scene_forward: bad buckets / capacity / outputs");
    // bucket offsets are int32: one call holds fewer than 2^31 intersections
    UBS_REQUIRE(capacity < (1ll << 31), "scene_forward: capacity %lld exceeds 2^31 - 1 "
                "intersections; render fewer views per call", (long long)capacity);
    UBS_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0,
                "scene_forward: workspace must be 256-byte aligned");
    const SceneWs w = scene_ws(workspace, C, N, n_buckets, capacity);
    if (workspace_bytes < w.bytes)
        return set_error(UBS_ERR_OVERFLOW, "scene_forward: workspace %zu < %zu", workspace_bytes,
                         w.bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t CN = (int64_t)C * N;
    if (cudaMemsetAsync(w.hdr, 0, sizeof(SceneHeader), st) != cudaSuccess ||
        cudaMemsetAsync(w.bucket_counts, 0, (size_t)n_buckets * kCountReplicas * 4, st) !=
            cudaSuccess)
        return check_launch("scene_forward memset");
    a.recs = w.recs;
    a.cols_n = w.cols_n;
    a.radius = w.radius;
    a.depth = w.depth;
    a.bucket_counts = w.bucket_counts;
    a.n_buckets = n_buckets;
    a.status = &w.hdr->status;
    a.act = w.act;
    a.act_b = w.act + act_beta_off(N, dim);
    a.act_o = w.act + act_opac_off(N, dim);
    if (CN > 0) {
        if (int e = launch_scene_act(N, dim, scale, beta, opacity, w.act, st)) return e;
        UBS_TIMED("scene_prim_fwd", st,
                  UBS_SCENE_DIM(dim, scene_prim_fwd_kernel<DD><<<grid_for(CN, PRIM_THREADS),
                                                                PRIM_THREADS, 0, st>>>(a)));
        note_launch();
        if (int e = check_launch("scene_prim_fwd")) return e;
    }
    // bucket offsets, total and heaviest-first order: one CTA when the
    // buckets fit it, else a device-wide scan and the order kernel below
    const bool one_cta = n_buckets <= SCAN_ORDER_MAX;
    if (one_cta) {
        UBS_TIMED("bucket_scan_order", st,
                  bucket_scan_order_kernel<kCountReplicas><<<1, 1024, 0, st>>>(
                      w.bucket_counts, n_buckets, w.offsets, &w.hdr->total, w.order, w.cursor,
                      w.totals));
        note_launch();
        if (int e = check_launch("bucket_scan_order")) return e;
    } else {
        UBS_TIMED("fold_replicas", st,
                  fold_replicas_kernel<kCountReplicas><<<grid_for(n_buckets, 256), 256, 0, st>>>(
                      w.bucket_counts, n_buckets, w.totals));
        note_launch();
        if (int e = check_launch("fold_replicas")) return e;
        if (int e = device_exclusive_scan<int32_t>(w.totals, w.offsets, n_buckets, w.block_sums,
                                                   &w.hdr->total, st))
            return e;
        UBS_TIMED("replica_cursors", st,
                  replica_cursors_kernel<kCountReplicas><<<grid_for(n_buckets, 256), 256, 0, st>>>(
                      w.bucket_counts, n_buckets, w.offsets, w.cursor));
        note_launch();
        if (int e = check_launch("replica_cursors")) return e;
    }
    if (CN > 0) {
        UBS_TIMED("scene_emit", st,
                  scene_emit_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
                      CN, N, w.recs, w.radius, w.depth, view_dims, tile_base, n_buckets,
                      (float)tile_size, w.cursor, w.keys, capacity, &w.hdr->status));
        note_launch();
        if (int e = check_launch("scene_emit")) return e;
    }
    const KeyWriter wr{w.keys};
    if (int e = launch_bucket_sort(n_buckets, w.offsets, &w.hdr->total, capacity, w.keys,
                                   w.scratch, w.big_list, &w.hdr->n_big, wr, st))
        return e;
    if (!one_cta) {
        UBS_TIMED("bucket_order", st,
                  bucket_order_kernel<<<1, 1024, 0, st>>>(w.offsets, &w.hdr->total, capacity,
                                                          n_buckets, w.order));
        note_launch();
        if (int e = check_launch("bucket_order")) return e;
    }
    return scene_blend(1, C, CN, n_buckets, tile_size, w.offsets, w.order, &w.hdr->total, capacity,
                       w.keys, w.recs, w.cols_n, backgrounds, tile_base, view_dims, pix_base,
                       render_colors, render_alphas, last_ids, nullptr, nullptr, nullptr, nullptr,
                       nullptr, &w.hdr->status, st);
}

int ubs_scene_backward(int32_t dim, int64_t N, const float *xyz, const float *mean,
                       const float *scale, const float *l_triangle, const float *opacity,
                       const float *beta, const float *rgb, int32_t C, const float *viewmats,
                       const float *intrinsics, const float *centers, const float *timestamps,
                       const int32_t *view_dims, const int32_t *tile_base,
                       const int64_t *pix_base, int32_t n_buckets, int32_t tile_size,
                       float eps2d, float near_plane, float far_plane, float radius_clip,
                       const float *backgrounds, const float *render_alphas,
                       const int32_t *last_ids, const float *v_render_colors,
                       const float *v_render_alphas, float *v_xyz, float *v_mean, float *v_scale,
                       float *v_l_triangle, float *v_opacity, float *v_beta, float *v_rgb,
                       int32_t exact_cond_grad, int64_t capacity, void *workspace,
                       size_t workspace_bytes, void *stream) {
    SceneArgs a{};
    if (int e = scene_common(a, dim, N, xyz, mean, scale, l_triangle, opacity, beta, rgb, C,
                             viewmats, intrinsics, centers, timestamps, view_dims, tile_base,
                             tile_size, eps2d, near_plane, far_plane, radius_clip))
        return e;
    UBS_REQUIRE(n_buckets >= 1 && capacity >= 1 && pix_base && render_alphas && last_ids &&
                    v_render_colors && v_render_alphas &&
                    (N == 0 || (v_xyz && v_mean && v_scale && v_l_triangle && v_opacity &&
                                v_beta && v_rgb)),
                "scene_backward: null argument");
    UBS_REQUIRE(capacity < (1ll << 31), "scene_backward: capacity %lld exceeds 2^31 - 1",
                (long long)capacity);
    UBS_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0,
                "scene_backward: workspace must be 256-byte aligned");
    const SceneWs w = scene_ws(workspace, C, N, n_buckets, capacity);
    if (workspace_bytes < w.bytes)
        return set_error(UBS_ERR_OVERFLOW, "scene_backward: workspace %zu < %zu", workspace_bytes,
                         w.bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t CN = (int64_t)C * N;
    if (cudaMemsetAsync(w.grads, 0, CN * kGradRow * 4, st) != cudaSuccess)
        return check_launch("scene_backward memset");
    if (int e = scene_blend(0, C, CN, n_buckets, tile_size, w.offsets, w.order, &w.hdr->total,
                            capacity, w.keys, w.recs, w.cols_n, backgrounds, tile_base,
                            view_dims, pix_base,
                            nullptr, nullptr, nullptr, render_alphas, last_ids, v_render_colors,
                            v_render_alphas, w.grads, &w.hdr->status, st))
        return e;
    if (CN == 0) return UBS_OK;
    if (C > 1) {
        const int K = dim - 3, NL = dim * (dim - 1) / 2;
        if (cudaMemsetAsync(v_xyz, 0, N * 12, st) || cudaMemsetAsync(v_mean, 0, N * K * 4, st) ||
            cudaMemsetAsync(v_scale, 0, N * dim * 4, st) ||
            cudaMemsetAsync(v_l_triangle, 0, N * NL * 4, st) ||
            cudaMemsetAsync(v_opacity, 0, N * 4, st) ||
            cudaMemsetAsync(v_beta, 0, N * (dim - 2) * 4, st) ||
            cudaMemsetAsync(v_rgb, 0, N * 12, st))
            return check_launch("scene_backward grad memset");
    }
    a.recs = w.recs;
    a.radius = w.radius;
    a.depth = w.depth;
    a.status = &w.hdr->status;
    a.act = w.act; // left by the forward
    a.act_b = w.act + act_beta_off(N, dim);
    a.act_o = w.act + act_opac_off(N, dim);
    a.v_rows = w.grads;
    a.g_xyz = v_xyz;
    a.g_mean = v_mean;
    a.g_scale = v_scale;
    a.g_ltri = v_l_triangle;
    a.g_opac = v_opacity;
    a.g_beta = v_beta;
    a.g_rgb = v_rgb;
    a.exact = exact_cond_grad;
    UBS_TIMED("scene_prim_bwd", st,
              UBS_SCENE_DIM(dim, scene_prim_bwd_kernel<DD><<<grid_for(CN, PRIM_THREADS),
                                                                PRIM_THREADS, 0, st>>>(a)));
    note_launch();
    return check_launch("scene_prim_bwd");
}

int ubs_scene_stats(const void *workspace, int64_t *n_isects, uint32_t *status, void *stream) {
    UBS_REQUIRE(workspace, "scene_stats: null workspace");
    SceneHeader h;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(&h, workspace, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("scene_stats");
    if (n_isects) *n_isects = h.total;
    if (status) *status = h.status;
    return UBS_OK;
}

} // extern "C"
