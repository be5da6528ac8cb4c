// raster.cu -- per-tile Beta-kernel blend, forward and backward, for sm_103a.
//
// Reference: submodules/gsplat/cuda/csrc/rasterize_to_pixels_fwd.cu:17-191 and
// rasterize_to_pixels_bwd.cu:17-276.  The per-pixel arithmetic (sigma, alpha,
// transmittance, exclusive termination at T <= 1e-4, back-to-front
// transmittance recovery from 1 - render_alpha) follows the reference so that
// images agree to FP32 rounding.  The data movement is new:
//   * records are 32-byte geometry records (+16-byte colour records for <= 4
//     channels).  The drop-in operators pack one per sorted intersection, so
//     a tile's front-to-back list is one contiguous span that a CTA streams
//     through shared memory with bulk async copies (cp.async.bulk + mbarrier,
//     double-buffered, bounded waits).  The fused scene path keeps them as
//     per-entry tables and every thread gathers its batch slots by the sorted
//     keys (16-byte cp.async, arrival on the batch's mbarrier), so no sorted
//     copy is ever written;
//   * each thread owns two vertically adjacent pixels (a warp an 8x8 block),
//     so record loads, loop control and the backward's warp reductions are
//     shared by two pixels;
//   * every batch, each record's ellipse is tested exactly against the
//     8x8-pixel footprint of every warp and the results turned into per-warp
//     bitmasks by ballot, so a warp only visits records that can touch its
//     pixels;
//   * the backward sums the 7 + channels gradients of a record over a warp with
//     transpose reductions (14 shuffles for 10 values), each warp writes its
//     totals into its own list of rows in shared memory with plain stores, and
//     per batch the rows of a record are summed and added to its gradient row
//     with three 16-byte vector atomics (fused path) or one scalar atomic per
//     value (drop-in arrays).
#include <atomic>
#include <cstdio>

#include "ubs_common.cuh"

namespace ubs {

struct __align__(16) GeoRec {
    float x, y, opac, beta;
    float cxx, cxy, cyy;
    int32_t gid;
};
static_assert(sizeof(GeoRec) == 32, "GeoRec must be 32 bytes");

constexpr uint32_t DEV_ERR_BAD_INDEX = 8u;
constexpr int GRAD_ROW = 12; // floats per gradient row (7 + up to 5 channels)

struct RasterArgs {
    int C, W, H, TS, TW, TH, n_tiles;
    int64_t n_isects, n_prims; // n_prims = C * N
    const int32_t *offsets;
    const GeoRec *recs;
    const float4 *rcols; // packed colours (channels <= 4) or nullptr
    const float *colors; // [C*N, CD], gathered when rcols == nullptr
    const float *bg;
    const uint8_t *masks;
    // forward outputs
    float *out_c;
    float *out_a;
    int32_t *last_ids;
    // backward inputs / outputs
    const float *render_alphas;
    const int32_t *last_in;
    const float *v_out_c;
    const float *v_out_a;
    float *v_m2, *v_cn, *v_col, *v_op, *v_be;
    // or, when not null, one gradient row per entry instead of the five arrays:
    // [v_xy(2), v_conic(3), v_opacity, v_beta, v_colour(CD), 0...], GRAD_ROW
    // floats (16-byte aligned rows, added with vector atomics)
    float *v_rows;
    uint32_t *status;
    // counters of the COUNT forward, or nullptr: [0] contributing (pixel,
    // record) pairs, [1] pairs a per-pixel loop evaluates up to termination,
    // [2] pairs up to each pixel's last contributor
    unsigned long long *pair_count;
    // multi-view grids (nullptr: C views of W x H with the same TW x TH grid)
    const int32_t *v_tile_base; // [C+1] first (view, tile) bucket of each view
    const int32_t *v_dims;      // [C, 4] width, height, tile columns, tile rows
    const int64_t *v_pix_base;  // [C] first pixel of each view in the image buffer
    int32_t n_buckets;          // total (view, tile) buckets
    const int64_t *n_isects_dev; // device-side intersection count (nullptr: n_isects)
    const int32_t *order;        // CTA -> bucket launch order (nullptr: identity)
    // gather mode (fused scene path, packed colours): records are copied per
    // batch from the per-entry tables, addressed by the low word of the
    // sorted (depth, entry) keys, instead of from sorted copies
    const uint64_t *keys;       // nullptr: sorted copies in recs / rcols
    const GeoRec *entry_recs;   // [C*N] one record per (view, primitive) entry
    const float4 *prim_cols;    // [N] packed colour per primitive
    int64_t n_per_view;         // N
};

// Where a (view, tile) bucket lives: view, tile within the view, image size,
// tile columns and the view's first pixel.
struct TileLoc {
    int cam, tile, W, H, TW;
    int64_t pix_base;
};
__device__ __forceinline__ TileLoc locate_tile(const RasterArgs &a, int bt) {
    TileLoc l;
    if (a.v_tile_base == nullptr) {
        l.cam = bt / a.n_tiles;
        l.tile = bt - l.cam * a.n_tiles;
        l.W = a.W;
        l.H = a.H;
        l.TW = a.TW;
        l.pix_base = (int64_t)l.cam * a.H * a.W;
        return l;
    }
    int lo = 0, hi = a.C - 1; // last view whose first bucket is <= bt
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (a.v_tile_base[mid] <= bt) lo = mid;
        else hi = mid - 1;
    }
    l.cam = lo;
    l.tile = bt - a.v_tile_base[lo];
    l.W = a.v_dims[lo * 4];
    l.H = a.v_dims[lo * 4 + 1];
    l.TW = a.v_dims[lo * 4 + 2];
    l.pix_base = a.v_pix_base[lo];
    return l;
}

// Number of valid sorted records: the device count (clamped to the record
// capacity n_isects) when the counts never left the device.
__device__ __forceinline__ int32_t isect_total(const RasterArgs &a) {
    int64_t T = a.n_isects;
    if (a.n_isects_dev) T = min(T, *a.n_isects_dev);
    return (int32_t)T;
}

// ---------------------------------------------------------------- packing
template <int CD, bool PACK>
__global__ void pack_records_kernel(int64_t T, int64_t n_prims, const int32_t *__restrict__ fl,
                                    const float *__restrict__ m2, const float *__restrict__ cn,
                                    const float *__restrict__ op, const float *__restrict__ be,
                                    const float *__restrict__ col, GeoRec *__restrict__ recs,
                                    float4 *__restrict__ rcols, uint32_t *status) {
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < T; i += stride) {
        int32_t g = fl[i];
        if (g < 0 || g >= n_prims) {
            atomicOr(status, DEV_ERR_BAD_INDEX);
            g = 0;
        }
        float4 a, b;
        a.x = m2[2 * (int64_t)g];
        a.y = m2[2 * (int64_t)g + 1];
        a.z = op[g];
        a.w = be[g];
        b.x = cn[3 * (int64_t)g];
        b.y = cn[3 * (int64_t)g + 1];
        b.z = cn[3 * (int64_t)g + 2];
        b.w = __int_as_float(g);
        float4 *dst = reinterpret_cast<float4 *>(recs + i);
        dst[0] = a;
        dst[1] = b;
        if (PACK) {
            float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
            const float *cp = col + (int64_t)g * CD;
            c.x = cp[0];
            if (CD > 1) c.y = cp[1];
            if (CD > 2) c.z = cp[2];
            if (CD > 3) c.w = cp[3];
            rcols[i] = c;
        }
    }
}

// ------------------------------------------------------ shared helpers
// Thread layout: every thread owns two vertically adjacent pixels, a warp an
// 8x8-pixel footprint; a TS x TS tile has (TS/8)^2 warps = TS*TS/2 threads and
// streams its records in batches of RB*TS*TS/2, RB batch slots per thread in
// the culling phase (RB = 1 in the backward of tiles up to 16 x 16 with packed
// colours of at most 4 channels, whose smaller shared footprint lets 8 CTAs
// share an SM; else 2).
// The backward accumulates a batch's per-record gradient sums in one of two
// ways.  KE = 0: one shared accumulator row per batch slot (BR x NV floats),
// which every warp adds its reduced sums to with shared-memory atomics, and a
// touched flag per slot.  KE > 0: every warp owns a list of KE entry rows
// (NV floats each) that it fills with plain stores, one row per record it
// visits, and a byte per batch slot naming the row (0xFF: none); the flush
// sums the warps' rows of a slot.  Shared float atomics cost about as much as
// the rest of a visit's reduction, so the small tiles use the lists.
struct SmemLayout {
    int mask_off, rec_off, col_off, gacc_off, touched_off, total;
};

template <int CD, bool PACK, bool BWD>
__host__ __device__ inline SmemLayout smem_layout(int NT, int RB = 2, int KE = 0) {
    constexpr int NV = 7 + CD; // gradient values per record
    const int nw = NT / 32, BR = RB * NT;
    SmemLayout L;
    L.mask_off = 16; // after two mbarriers
    // per-target-warp masks (nw x RB nw words), then one int per warp
    L.rec_off = (L.mask_off + nw * RB * nw * 4 + nw * 4 + 127) & ~127;
    const int colbytes = PACK ? 16 : CD * 4;
    L.col_off = L.rec_off + 2 * BR * (int)sizeof(GeoRec);
    L.gacc_off = (L.col_off + 2 * BR * colbytes + 15) & ~15;
    if (BWD && KE > 0) {
        L.touched_off = L.gacc_off + nw * KE * NV * 4; // entry rows, then the slot maps
        L.total = L.touched_off + nw * BR;
    } else {
        L.touched_off = L.gacc_off + (BWD ? BR * NV * 4 : 0);
        L.total = L.touched_off + (BWD ? BR * 4 : 0);
    }
    return L;
}

// Whether the ellipse {d : d^T Q d < 1} of a record (Q its conic, d = centre -
// pixel) can hold a pixel centre of the 8x8 box [bx0, bx0 + 7] x [by0, by0 + 7].
// The quadratic is minimised over the box: it is zero when the centre lies in
// the box; otherwise the minimum lies on an edge whose outside holds the
// centre (for a convex function the segment from the box minimiser towards the
// unconstrained minimiser leaves the box), so only the one or two facing edges
// are searched, each in closed form.  The test is conservative: the pixel grid
// is treated as continuous and the threshold has 1% slack for FP32 rounding of
// sigma; conics that are not positive definite or are so elongated that
// rounding could matter are never culled (pd == false).
__device__ __forceinline__ bool conic_pd(const GeoRec &r) {
    const float det = r.cxx * r.cyy - r.cxy * r.cxy;
    return (r.cxx > 0.f) && (r.cyy > 0.f) && (det > 1e-3f * r.cxx * r.cyy);
}
__device__ __forceinline__ bool ellipse_hits_box(const GeoRec &r, bool pd, float bx0, float by0) {
    if (!pd) return true;
    const float ex = fminf(fmaxf(r.x, bx0), bx0 + 7.f); // nearest box point to the centre
    const float ey = fminf(fmaxf(r.y, by0), by0 + 7.f);
    const bool out_x = ex != r.x, out_y = ey != r.y;
    if (!out_x && !out_y) return true;
    float best = 3.0e38f;
    if (out_x) { // edge x = ex: minimise over y in [by0, by0 + 7]
        const float dx = r.x - ex;
        const float y = fminf(fmaxf(r.y + r.cxy * dx / r.cyy, by0), by0 + 7.f);
        const float dy = r.y - y;
        best = r.cxx * dx * dx + 2.f * r.cxy * dx * dy + r.cyy * dy * dy;
    }
    if (out_y) { // edge y = ey: minimise over x in [bx0, bx0 + 7]
        const float dy = r.y - ey;
        const float x = fminf(fmaxf(r.x + r.cxy * dy / r.cxx, bx0), bx0 + 7.f);
        const float dx = r.x - x;
        best = fminf(best, r.cxx * dx * dx + 2.f * r.cxy * dx * dy + r.cyy * dy * dy);
    }
    return best < 1.01f;
}

// Gather mode: thread tid copies batch slots tid + h NT (h < RB) with
// cp.async and arrives on the batch's mbarrier once its copies have landed;
// the mbarrier expects one arrival per thread.  Entry indices are loaded one
// batch ahead of their copies (load_entries) so the copies never wait on the
// key reads.  The keys of a bucket address entries of the bucket's view,
// [lo_e, hi_e]; indices are clamped to that range.
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src)
                 : "memory");
}
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}

template <int RB>
__device__ __forceinline__ void load_entries(const RasterArgs &a, int32_t bs, int cnt, int NT,
                                             int tid, int32_t (&ent)[RB]) {
#pragma unroll
    for (int h = 0; h < RB; ++h) {
        const int s = tid + h * NT;
        ent[h] = s < cnt ? (int32_t)(uint32_t)a.keys[bs + s] : 0;
    }
}

template <int RB>
__device__ __forceinline__ void gather_batch(const RasterArgs &a, GeoRec *srec, float4 *scol4,
                                             uint64_t *mbar, int BR, int buf, int cnt,
                                             const int32_t (&ent)[RB], int64_t lo_e,
                                             int64_t hi_e, int NT, int tid) {
#pragma unroll
    for (int h = 0; h < RB; ++h) {
        const int s = tid + h * NT;
        if (s < cnt) {
            // clamped for memory safety; a key outside the bucket's view
            // (corrupt or stale) is reported like a bad flatten index
            int64_t e = (int64_t)ent[h];
            if (e < lo_e || e > hi_e) {
                atomicOr(a.status, DEV_ERR_BAD_INDEX);
                e = min(max(e, lo_e), hi_e);
            }
            const char *src = reinterpret_cast<const char *>(a.entry_recs + e);
            char *dst = reinterpret_cast<char *>(srec + buf * BR + s);
            cp_async16(dst, src);
            cp_async16(dst + 16, src + 16);
            cp_async16(scol4 + buf * BR + s, a.prim_cols + (e - lo_e));
        }
    }
    cp_async_arrive(&mbar[buf]);
}

// Issues the bulk copies of batch [bs, bs+cnt) into buffer `buf` (thread 0).
template <bool PACK>
__device__ __forceinline__ void issue_batch(const RasterArgs &a, GeoRec *srec, float4 *scol4,
                                            uint64_t *mbar, int BR, int buf, int32_t bs,
                                            int cnt) {
    fence_proxy_async_smem();
    const uint32_t bytes = (uint32_t)cnt * (32u + (PACK ? 16u : 0u));
    mbar_arrive_expect_tx(&mbar[buf], bytes);
    bulk_g2s(srec + buf * BR, a.recs + bs, (uint32_t)cnt * 32u, &mbar[buf]);
    if (PACK) bulk_g2s(scol4 + buf * BR, a.rcols + bs, (uint32_t)cnt * 16u, &mbar[buf]);
}

// Per-batch culling masks.  Thread tid describes batch slots tid + h NT
// (h < RB); for every warp w one ballot per slot gives 32 bits of w's
// RB*nw-word mask (word k covers slots 32k .. 32k+31, so ascending bits are
// front to back).  limit[w] (backward) drops records past warp w's last
// contributor.
template <int RB = 2>
__device__ __forceinline__ void build_masks(const GeoRec *batch, int cnt, int lo, int NT, int nw,
                                            int wpr, int tile_x0, int tile_y0, int tid, int lane,
                                            uint32_t *wmask, const int32_t *limit) {
#pragma unroll
    for (int half = 0; half < RB; ++half) {
        const int s = tid + half * NT;
        const bool valid = s < cnt;
        GeoRec r;
        bool pd = false;
        if (valid) {
            r = batch[s];
            pd = conic_pd(r);
        }
        const int word = s >> 5;
        for (int w = 0; w < nw; ++w) {
            const float x0 = (float)(tile_x0 + (w % wpr) * 8) + 0.5f;
            const float y0 = (float)(tile_y0 + (w / wpr) * 8) + 0.5f;
            bool ov = valid && ellipse_hits_box(r, pd, x0, y0);
            if (limit) ov = ov && (lo + s <= limit[w]);
            const uint32_t bits = __ballot_sync(0xffffffffu, ov);
            if (lane == 0) wmask[w * RB * nw + word] = bits;
        }
    }
}

template <int CD, bool PACK>
__device__ __forceinline__ void load_color(const float4 *scol4, const float *scol, int slot,
                                           float (&col)[CD]) {
    if (PACK) {
        const float4 c = scol4[slot];
        col[0] = c.x;
        if (CD > 1) col[1 % CD] = c.y;
        if (CD > 2) col[2 % CD] = c.z;
        if (CD > 3) col[3 % CD] = c.w;
    } else {
#pragma unroll
        for (int k = 0; k < CD; ++k) col[k] = scol[slot * CD + k];
    }
}

// One front-to-back blend step of a thread's two pixels (column px, rows py0
// and py0 + 1) over record q (rasterize_to_pixels_fwd.cu:139-171): skip when
// sigma is outside [0, 1), alpha = min(0.999, opacity (1 - sigma)^beta), stop
// (exclusively) once the transmittance would reach 1e-4.  The pixel pair is
// evaluated two-wide with Blackwell's packed FP32x2 instructions (__ffma2_rn,
// __fadd2_rn, __fmul2_rn: per component the same rounding as the scalar
// operations); (1 - sigma)^beta is formed as 2^(beta log2(1 - sigma)).  The
// updates are select-based so that a warp issues them once for both pixels
// and all lanes; lanes whose record is skipped evaluate dummies (NaN where
// sigma >= 1) that the selects discard.  Records no lane can use are
// evaluated the same way rather than skipped after a warp vote: under 1% of
// the culled visits are such.
template <int CD, bool COUNT>
__device__ __forceinline__ void blend_pair(const GeoRec &q, const float (&col)[CD], float px,
                                           float2 npy, float2 &T, float2 (&acc)[CD],
                                           int32_t &cur0, int32_t &cur1, bool &d0, bool &d1,
                                           int32_t idx, uint32_t &n_contrib, int32_t &term0,
                                           int32_t &term1) {
    const float dx = q.x - px;
    const float2 dy = __fadd2_rn(make_float2(q.y, q.y), npy);
    const float A = q.cxx * dx * dx;
    const float B = 2.f * q.cxy * dx;
    float2 s = __fmul2_rn(make_float2(q.cyy, q.cyy), dy);
    s = __ffma2_rn(s, dy, make_float2(A, A));
    s = __ffma2_rn(make_float2(B, B), dy, s);
    const bool v0 = !d0 && !(s.x < 0.f || s.x >= 1.f);
    const bool v1 = !d1 && !(s.y < 0.f || s.y >= 1.f);
    const float2 om = __ffma2_rn(s, make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
    const float2 l = make_float2(__log2f(om.x), __log2f(om.y));
    const float2 e = __fmul2_rn(l, make_float2(q.beta, q.beta));
    const float2 p = make_float2(exp2f(e.x), exp2f(e.y));
    float2 a = __fmul2_rn(make_float2(q.opac, q.opac), p);
    a.x = fminf(0.999f, a.x);
    a.y = fminf(0.999f, a.y);
    const float2 n = __fmul2_rn(T, __ffma2_rn(a, make_float2(-1.f, -1.f), make_float2(1.f, 1.f)));
    const bool t0 = v0 && n.x <= 1e-4f, t1 = v1 && n.y <= 1e-4f;
    const bool b0 = v0 && !t0, b1 = v1 && !t1;
    d0 = d0 || t0;
    d1 = d1 || t1;
    float2 w = __fmul2_rn(a, T);
    w.x = b0 ? w.x : 0.f;
    w.y = b1 ? w.y : 0.f;
#pragma unroll
    for (int k = 0; k < CD; ++k) acc[k] = __ffma2_rn(make_float2(col[k], col[k]), w, acc[k]);
    T.x = b0 ? n.x : T.x;
    T.y = b1 ? n.y : T.y;
    cur0 = b0 ? idx : cur0;
    cur1 = b1 ? idx : cur1;
    if (COUNT) {
        n_contrib += (uint32_t)b0 + (uint32_t)b1;
        term0 = t0 ? idx : term0;
        term1 = t1 ? idx : term1;
    }
}

// --------------------------------------------------------------- forward
// MINB > 1: tiles of at most 128 threads, MINB CTAs per SM.
template <int CD, bool PACK, bool COUNT, int RB, int MINB>
__global__ void __launch_bounds__(MINB > 1 ? 128 : 512, MINB) raster_fwd_kernel(RasterArgs a) {
    extern __shared__ __align__(128) unsigned char sm[];
    const int NT = blockDim.x, nw = NT >> 5, BR = RB * NT;
    const SmemLayout L = smem_layout<CD, PACK, false>(NT, RB);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm);
    uint32_t *wmask = reinterpret_cast<uint32_t *>(sm + L.mask_off);
    GeoRec *srec = reinterpret_cast<GeoRec *>(sm + L.rec_off);
    float4 *scol4 = reinterpret_cast<float4 *>(sm + L.col_off);
    float *scol = reinterpret_cast<float *>(sm + L.col_off);

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bt = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    const TileLoc loc = locate_tile(a, bt);
    const int cam = loc.cam;
    const int ty = loc.tile / loc.TW, tx = loc.tile - ty * loc.TW;
    const int wpr = a.TS >> 3;
    const int j = tx * a.TS + (warp % wpr) * 8 + (lane & 7);
    const int i0 = ty * a.TS + (warp / wpr) * 8 + (lane >> 3) * 2;
    const bool in0 = (i0 < loc.H) && (j < loc.W);
    const bool in1 = (i0 + 1 < loc.H) && (j < loc.W);
    const int64_t pix0 = loc.pix_base + (int64_t)i0 * loc.W + j;
    const int64_t pix1 = pix0 + loc.W;
    const float *bg = a.bg ? a.bg + (int64_t)cam * CD : nullptr;

    if (a.masks && !a.masks[bt]) {
#pragma unroll
        for (int k = 0; k < CD; ++k) {
            if (in0) a.out_c[pix0 * CD + k] = bg ? bg[k] : 0.f;
            if (in1) a.out_c[pix1 * CD + k] = bg ? bg[k] : 0.f;
        }
        if (in0) { a.out_a[pix0] = 0.f; a.last_ids[pix0] = 0; }
        if (in1) { a.out_a[pix1] = 0.f; a.last_ids[pix1] = 0; }
        return;
    }

    const int32_t T_all = isect_total(a);
    int32_t rs = a.offsets[bt];
    int32_t re = (bt == a.n_buckets - 1) ? T_all : a.offsets[bt + 1];
    rs = max(0, min(rs, T_all));
    re = max(rs, min(re, T_all));
    const int nb = (re - rs + BR - 1) / BR;

    const float px = (float)j + 0.5f, py0 = (float)i0 + 0.5f, py1 = py0 + 1.f;
    const float2 npy = make_float2(-py0, -py1);
    float2 T = make_float2(1.0f, 1.0f);
    int32_t cur0 = 0, cur1 = 0;
    uint32_t n_contrib = 0;
    int32_t term0 = -1, term1 = -1; // COUNT: record at which a pixel terminated
    float2 acc[CD];
#pragma unroll
    for (int k = 0; k < CD; ++k) acc[k] = make_float2(0.f, 0.f);
    bool d0 = !in0, d1 = !in1;

    if (nb > 0) {
        const bool gather = PACK && a.keys != nullptr;
        const int64_t lo_e = gather ? (int64_t)cam * a.n_per_view : 0;
        const int64_t hi_e = lo_e + a.n_per_view - 1;
        int32_t ent[RB];
        if (tid == 0) {
            mbar_init(&mbar[0], gather ? NT : 1);
            mbar_init(&mbar[1], gather ? NT : 1);
            fence_barrier_init();
        }
        __syncthreads();
        int issued = 0, waited = 0;
        if (gather) {
            load_entries<RB>(a, rs, min(BR, re - rs), NT, tid, ent);
            gather_batch<RB>(a, srec, scol4, mbar, BR, 0, min(BR, re - rs), ent, lo_e, hi_e, NT,
                             tid);
            if (nb > 1) load_entries<RB>(a, rs + BR, min(BR, re - rs - BR), NT, tid, ent);
            issued = 1;
        } else if (tid == 0) {
            issue_batch<PACK>(a, srec, scol4, mbar, BR, 0, rs, min(BR, re - rs));
            issued = 1;
        }
        for (int b = 0; b < nb; ++b) {
            const int32_t bs = rs + b * BR;
            const int cnt = min(BR, re - bs);
            const int buf = b & 1;
            if (b + 1 < nb) {
                const int32_t bn = bs + BR;
                if (gather) {
                    gather_batch<RB>(a, srec, scol4, mbar, BR, buf ^ 1, min(BR, re - bn), ent,
                                     lo_e, hi_e, NT, tid);
                    if (b + 2 < nb)
                        load_entries<RB>(a, bn + BR, min(BR, re - bn - BR), NT, tid, ent);
                    issued = b + 2;
                } else if (tid == 0) {
                    issue_batch<PACK>(a, srec, scol4, mbar, BR, buf ^ 1, bn, min(BR, re - bn));
                    issued = b + 2;
                }
            }
            const bool ok = mbar_wait_bounded(&mbar[buf], (b >> 1) & 1);
            if (tid == 0 && ok) waited = b + 1;
            const GeoRec *batch = srec + buf * BR;
            build_masks<RB>(batch, cnt, 0, NT, nw, wpr, tx * a.TS, ty * a.TS, tid, lane, wmask,
                            nullptr);
            if (!PACK) {
#pragma unroll
                for (int half = 0; half < RB; ++half) {
                    const int s = tid + half * NT;
                    if (s < cnt) {
                        const float *cp = a.colors + (int64_t)batch[s].gid * CD;
#pragma unroll
                        for (int k = 0; k < CD; ++k) scol[(buf * BR + s) * CD + k] = cp[k];
                    }
                }
            }
            if (__syncthreads_or(!ok)) {
                if (tid == 0) atomicOr(a.status, DEV_ERR_WAIT_TIMEOUT);
                d0 = d1 = true;
                break;
            }
            if (!__all_sync(0xffffffffu, d0 && d1)) {
                bool warp_done = false;
                for (int k = 0; k < RB * nw && !warp_done; ++k) {
                    uint32_t m = wmask[warp * RB * nw + k];
                    while (m) {
                        const int bit = __ffs(m) - 1;
                        m &= m - 1;
                        const int t = k * 32 + bit;
                        const GeoRec q = batch[t];
                        float col[CD];
                        load_color<CD, PACK>(scol4, scol, buf * BR + t, col);
                        blend_pair<CD, COUNT>(q, col, px, npy, T, acc, cur0, cur1, d0, d1,
                                              bs + t, n_contrib, term0, term1);
                        if (__all_sync(0xffffffffu, d0 && d1)) {
                            warp_done = true;
                            break;
                        }
                    }
                }
            }
            if (__syncthreads_count(d0 && d1) == NT) break;
        }
        // no copy may still target this CTA's shared memory at exit
        if (gather) cp_async_wait_all();
        if (tid == 0)
            for (int b = waited; b < issued; ++b)
                if (!mbar_wait_bounded(&mbar[b & 1], (b >> 1) & 1))
                    atomicOr(a.status, DEV_ERR_WAIT_TIMEOUT);
    }

    if (COUNT) {
        const uint32_t w = __reduce_add_sync(0xffffffffu, n_contrib);
        if (lane == 0 && w) atomicAdd(a.pair_count, (unsigned long long)w);
        // evaluated pairs of a per-pixel loop: up to the terminating record,
        // else the whole range; backward pairs: up to the last contributor
        uint32_t ev = 0, bw = 0;
        if (in0) {
            ev += (uint32_t)(term0 >= 0 ? term0 - rs + 1 : re - rs);
            bw += (uint32_t)(cur0 >= rs && cur0 > 0 ? cur0 - rs + 1 : 0);
        }
        if (in1) {
            ev += (uint32_t)(term1 >= 0 ? term1 - rs + 1 : re - rs);
            bw += (uint32_t)(cur1 >= rs && cur1 > 0 ? cur1 - rs + 1 : 0);
        }
        const uint32_t we = __reduce_add_sync(0xffffffffu, ev);
        const uint32_t wb = __reduce_add_sync(0xffffffffu, bw);
        if (lane == 0 && we) atomicAdd(a.pair_count + 1, (unsigned long long)we);
        if (lane == 0 && wb) atomicAdd(a.pair_count + 2, (unsigned long long)wb);
    }
    if (in0) {
        a.out_a[pix0] = 1.0f - T.x;
#pragma unroll
        for (int k = 0; k < CD; ++k) a.out_c[pix0 * CD + k] = bg ? acc[k].x + T.x * bg[k] : acc[k].x;
        a.last_ids[pix0] = cur0;
    }
    if (in1) {
        a.out_a[pix1] = 1.0f - T.y;
#pragma unroll
        for (int k = 0; k < CD; ++k) a.out_c[pix1 * CD + k] = bg ? acc[k].y + T.y * bg[k] : acc[k].y;
        a.last_ids[pix1] = cur1;
    }
}

// -------------------------------------------------------------- backward
// Per-pixel state of the back-to-front pass.  The reference keeps the colour
// accumulated behind the current record per channel (buf_k) and forms
// sum_k (c_k T - buf_k ra) v_k + T_final ra (v_a - bg.v); only the scalar
// S = sum_k buf_k v_k enters, so it is carried instead of buf, and
// K = T_final (v_a - bg.v) is folded once per pixel.
template <int CD> struct BwdPair {
    float2 T, S, K;
    float2 vrc[CD];
    int32_t bin0, bin1;
    bool in0, in1;
};

template <int CD>
__device__ __forceinline__ void bwd_pair_init(BwdPair<CD> &s, const RasterArgs &a, int64_t pix0,
                                              int64_t pix1, bool in0, bool in1, const float *bg) {
    s.in0 = in0;
    s.in1 = in1;
    const float T0 = 1.0f - a.render_alphas[pix0], T1 = 1.0f - a.render_alphas[pix1];
    s.T = make_float2(T0, T1);
    s.bin0 = in0 ? a.last_in[pix0] : 0;
    s.bin1 = in1 ? a.last_in[pix1] : 0;
    float bg0 = 0.f, bg1 = 0.f;
#pragma unroll
    for (int k = 0; k < CD; ++k) {
        s.vrc[k] = make_float2(a.v_out_c[pix0 * CD + k], a.v_out_c[pix1 * CD + k]);
        if (bg) {
            bg0 += bg[k] * s.vrc[k].x;
            bg1 += bg[k] * s.vrc[k].y;
        }
    }
    s.K = make_float2(T0 * (a.v_out_a[pix0] - bg0), T1 * (a.v_out_a[pix1] - bg1));
    s.S = make_float2(0.f, 0.f);
}

// One back-to-front step of both pixels of a thread against record q
// (rasterize_to_pixels_bwd.cu:158-247: transmittance recovered as
// T / (1 - alpha), v_alpha from the colour behind and the final alpha, the
// sigma chain when opacity (1 - sigma)^beta <= 0.999), packed two-wide (one
// FP32x2 instruction per step for the pixel pair); valid lanes are inside,
// at or before their last contributor, with sigma in [0, 1), others evaluate
// finite dummies (1 - sigma replaced by 1) that selects zero.  A record no
// lane can use is evaluated too: under 1% of the culled visits are such, and
// a warp vote to skip them cost more than it saved.  g receives the pair's sums
//   [w dx, w dy, w dx^2, w dx dy, w dy^2, vis v_alpha, vis v_alpha log2(1-s),
//    fac v_colour (CD)],  w = v_alpha (1 - sigma)^(beta - 1),
// turned into [v_xy, v_conic, v_opacity, v_beta, v_colour] per record at
// the flush (the conic, -opacity beta and opacity ln 2 factors).
template <int CD>
__device__ __forceinline__ void grad_pair(const GeoRec &q, const float (&col)[CD], float px,
                                          float2 npy, int32_t idx, BwdPair<CD> &s,
                                          float (&g)[7 + CD]) {
    const float dx = q.x - px;
    const float2 dy = __fadd2_rn(make_float2(q.y, q.y), npy);
    const float A = q.cxx * dx * dx;
    const float B = 2.f * q.cxy * dx;
    float2 sg = __fmul2_rn(make_float2(q.cyy, q.cyy), dy);
    sg = __ffma2_rn(sg, dy, make_float2(A, A));
    sg = __ffma2_rn(make_float2(B, B), dy, sg);
    const bool v0 = s.in0 && idx <= s.bin0 && !(sg.x < 0.f || sg.x >= 1.f);
    const bool v1 = s.in1 && idx <= s.bin1 && !(sg.y < 0.f || sg.y >= 1.f);
    float2 om = __ffma2_rn(sg, make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
    om.x = v0 ? om.x : 1.f;
    om.y = v1 ? om.y : 1.f;
    const float2 l = make_float2(__log2f(om.x), __log2f(om.y));
    const float2 e = __fmul2_rn(l, make_float2(q.beta, q.beta));
    const float2 vis = make_float2(exp2f(e.x), exp2f(e.y));
    const float2 ov = __fmul2_rn(make_float2(q.opac, q.opac), vis);
    const float2 alpha = make_float2(fminf(0.999f, ov.x), fminf(0.999f, ov.y));
    const float2 oma = __ffma2_rn(alpha, make_float2(-1.f, -1.f), make_float2(1.f, 1.f));
    const float2 ra = make_float2(1.0f / oma.x, 1.0f / oma.y);
    const float2 Tn = __fmul2_rn(s.T, ra);
    float2 fac = __fmul2_rn(alpha, Tn);
    fac.x = v0 ? fac.x : 0.f;
    fac.y = v1 ? fac.y : 0.f;
    float2 cv = __fmul2_rn(make_float2(col[0], col[0]), s.vrc[0]);
#pragma unroll
    for (int k = 1; k < CD; ++k)
        cv = __ffma2_rn(make_float2(col[k], col[k]), s.vrc[k], cv);
#pragma unroll
    for (int k = 0; k < CD; ++k) {
        const float2 gc = __fmul2_rn(fac, s.vrc[k]);
        g[7 + k] = gc.x + gc.y;
    }
    const float2 kms = __ffma2_rn(s.S, make_float2(-1.f, -1.f), s.K);
    float2 va = __ffma2_rn(Tn, cv, __fmul2_rn(ra, kms));
    va.x = (v0 && ov.x <= 0.999f) ? va.x : 0.f;
    va.y = (v1 && ov.y <= 0.999f) ? va.y : 0.f;
    const float2 u = __fmul2_rn(vis, va);
    const float2 w = __fmul2_rn(u, make_float2(__fdividef(1.f, om.x), __fdividef(1.f, om.y)));
    const float ws = w.x + w.y;
    const float2 wdy = __fmul2_rn(w, dy);
    const float2 wdy2 = __fmul2_rn(wdy, dy);
    const float2 ul = __fmul2_rn(u, l);
    g[0] = ws * dx;
    g[1] = wdy.x + wdy.y;
    g[2] = ws * (dx * dx);
    g[3] = g[1] * dx;
    g[4] = wdy2.x + wdy2.y;
    g[5] = u.x + u.y;
    g[6] = ul.x + ul.y;
    s.S = __ffma2_rn(fac, cv, s.S);
    s.T.x = v0 ? Tn.x : s.T.x;
    s.T.y = v1 ? Tn.y : s.T.y;
}

// Factor turning the reduced sum g[u] (u >= 2) of a record into its gradient
// value u of [v_xy(2), v_conic(3), v_opacity, v_beta, v_colour(CD)]; v_xy is
// -2 opacity beta (conic [w dx, w dy]) and is formed at the flush.  With
// the entry lists the first two sums are multiplied by the conic per lane
// before the reduction, so every value is a factor times its sum
// (pre_conic = true).
__device__ __forceinline__ float record_scale(int u, float opac, float beta,
                                              bool pre_conic = false) {
    const float ob = opac * beta;
    if (u == 3 || (pre_conic && u < 2)) return -2.f * ob;
    if (u < 5) return -ob;
    if (u == 6) return opac * 0.6931471805599453f;
    return 1.f;
}

// Gradient array element of value u of primitive entry gid.
template <int CD>
__device__ __forceinline__ float *grad_dst(const RasterArgs &a, int u, int64_t gid) {
    if (a.v_rows) return a.v_rows + gid * GRAD_ROW + u;
    if (u < 2) return a.v_m2 + 2 * gid + u;
    if (u < 5) return a.v_cn + 3 * gid + (u - 2);
    if (u == 5) return a.v_op + gid;
    if (u == 6) return a.v_be + gid;
    return a.v_col + gid * CD + (u - 7);
}

// Sums g[OFF .. OFF+REM) over the warp in power-of-two chunks; every lane
// calls sink(u, total, owner) for the value u whose total it holds, owner
// being true for exactly one lane per value.
template <int OFF, int REM> struct ReduceChunks {
    template <int NV, class Sink>
    static __device__ __forceinline__ void run(const float (&g)[NV], const LaneMasks &lm, int lane,
                                               Sink &sink) {
        constexpr int S = REM >= 32 ? 32 : REM >= 16 ? 16 : REM >= 8 ? 8 : REM >= 4 ? 4
                                                                         : REM >= 2 ? 2 : 1;
        float v[S];
#pragma unroll
        for (int i = 0; i < S; ++i) v[i] = g[OFF + i];
        const float tot = tr_reduce<S>(v, lm);
        sink(OFF + tr_index<S>(lane), tot, (lane & (32 / S - 1)) == 0);
        ReduceChunks<OFF + S, REM - S>::run(g, lm, lane, sink);
    }
};
template <int OFF> struct ReduceChunks<OFF, 0> {
    template <int NV, class Sink>
    static __device__ __forceinline__ void run(const float (&)[NV], const LaneMasks &, int,
                                               Sink &) {}
};

// MINB > 1: tiles of at most 128 threads, MINB CTAs per SM.  KE > 0: entry
// lists of KE rows per warp (see smem_layout).
template <int CD, bool PACK, int RB, int MINB, int KE>
__global__ void __launch_bounds__(MINB > 1 ? 128 : 512, MINB) raster_bwd_kernel(RasterArgs a) {
    constexpr int NV = 7 + CD;
    static_assert(KE < 255, "entry rows are named by a byte");
    extern __shared__ __align__(128) unsigned char sm[];
    const int NT = blockDim.x, nw = NT >> 5, BR = RB * NT;
    const SmemLayout L = smem_layout<CD, PACK, true>(NT, RB, KE);
    uint64_t *mbar = reinterpret_cast<uint64_t *>(sm);
    uint32_t *wmask = reinterpret_cast<uint32_t *>(sm + L.mask_off);
    int32_t *wbin = reinterpret_cast<int32_t *>(sm + L.mask_off + nw * RB * nw * 4);
    GeoRec *srec = reinterpret_cast<GeoRec *>(sm + L.rec_off);
    float4 *scol4 = reinterpret_cast<float4 *>(sm + L.col_off);
    float *scol = reinterpret_cast<float *>(sm + L.col_off);
    float *gacc = reinterpret_cast<float *>(sm + L.gacc_off);       // KE > 0: entry rows
    int32_t *touched = reinterpret_cast<int32_t *>(sm + L.touched_off);
    uint8_t *slot_row = reinterpret_cast<uint8_t *>(sm + L.touched_off); // KE > 0

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int bt = a.order ? a.order[blockIdx.x] : (int)blockIdx.x;
    if (a.masks && !a.masks[bt]) return;
    const TileLoc loc = locate_tile(a, bt);
    const int cam = loc.cam;
    const int ty = loc.tile / loc.TW, tx = loc.tile - ty * loc.TW;
    const int wpr = a.TS >> 3;
    const int j = tx * a.TS + (warp % wpr) * 8 + (lane & 7);
    const int i0 = ty * a.TS + (warp / wpr) * 8 + (lane >> 3) * 2;
    const bool in0 = (i0 < loc.H) && (j < loc.W);
    const bool in1 = (i0 + 1 < loc.H) && (j < loc.W);
    // outside pixels read a clamped pixel, like the reference, and never contribute
    const int64_t img = (int64_t)loc.W * loc.H;
    const int64_t pix0 = loc.pix_base + min((int64_t)i0 * loc.W + j, img - 1);
    const int64_t pix1 = loc.pix_base + min((int64_t)(i0 + 1) * loc.W + j, img - 1);
    const float *bg = a.bg ? a.bg + (int64_t)cam * CD : nullptr;

    const int32_t T_all = isect_total(a);
    int32_t rs = a.offsets[bt];
    int32_t re = (bt == a.n_buckets - 1) ? T_all : a.offsets[bt + 1];
    rs = max(0, min(rs, T_all));
    re = max(rs, min(re, T_all));

    const float px = (float)j + 0.5f, py0 = (float)i0 + 0.5f, py1 = py0 + 1.f;
    const float2 npy = make_float2(-py0, -py1);
    BwdPair<CD> sp;
    bwd_pair_init<CD>(sp, a, pix0, pix1, in0, in1, bg);

    const int32_t wb = __reduce_max_sync(
        0xffffffffu, max(in0 ? sp.bin0 : INT32_MIN, in1 ? sp.bin1 : INT32_MIN));
    if (lane == 0) wbin[warp] = wb;
    if (KE > 0) {
        for (int t = tid; t < nw * BR; t += NT) slot_row[t] = 0xFF;
    } else {
        for (int t = tid; t < BR * NV; t += NT) gacc[t] = 0.f;
        for (int t = tid; t < BR; t += NT) touched[t] = 0;
    }
    const bool gather = PACK && a.keys != nullptr;
    const int64_t lo_e = gather ? (int64_t)cam * a.n_per_view : 0;
    const int64_t hi_e = lo_e + a.n_per_view - 1;
    if (tid == 0) {
        mbar_init(&mbar[0], gather ? NT : 1);
        mbar_init(&mbar[1], gather ? NT : 1);
        fence_barrier_init();
    }
    __syncthreads();
    int32_t block_bin = INT32_MIN;
    for (int w = 0; w < nw; ++w) block_bin = max(block_bin, wbin[w]);
    const int32_t hi_end = max(rs, min(re, block_bin + 1)); // exclusive upper index
    const int nb = (hi_end - rs + BR - 1) / BR;

    const LaneMasks lm = lane_masks(lane);
    // batch b covers [max(rs, hi_end - (b + 1) BR), hi_end - b BR): back to front
    int issued = 0, waited = 0;
    int32_t ent[RB];
    if (nb > 0) {
        const int32_t lo = max(rs, hi_end - BR);
        if (gather) {
            load_entries<RB>(a, lo, hi_end - lo, NT, tid, ent);
            gather_batch<RB>(a, srec, scol4, mbar, BR, 0, hi_end - lo, ent, lo_e, hi_e, NT, tid);
            if (nb > 1) {
                const int32_t l1 = max(rs, lo - BR);
                load_entries<RB>(a, l1, lo - l1, NT, tid, ent);
            }
            issued = 1;
        } else if (tid == 0) {
            issue_batch<PACK>(a, srec, scol4, mbar, BR, 0, lo, hi_end - lo);
            issued = 1;
        }
    }
    for (int b = 0; b < nb; ++b) {
        const int32_t hi = hi_end - b * BR;
        const int32_t lo = max(rs, hi - BR);
        const int cnt = hi - lo;
        const int buf = b & 1;
        if (b + 1 < nb) {
            const int32_t hn = hi - BR;
            const int32_t ln = max(rs, hn - BR);
            if (gather) {
                gather_batch<RB>(a, srec, scol4, mbar, BR, buf ^ 1, hn - ln, ent, lo_e, hi_e, NT,
                                 tid);
                if (b + 2 < nb) {
                    const int32_t l2 = max(rs, ln - BR);
                    load_entries<RB>(a, l2, ln - l2, NT, tid, ent);
                }
                issued = b + 2;
            } else if (tid == 0) {
                issue_batch<PACK>(a, srec, scol4, mbar, BR, buf ^ 1, ln, hn - ln);
                issued = b + 2;
            }
        }
        const bool ok = mbar_wait_bounded(&mbar[buf], (b >> 1) & 1);
        if (tid == 0 && ok) waited = b + 1;
        const GeoRec *batch = srec + buf * BR;
        const int32_t gid0 = (tid < cnt) ? batch[tid].gid : 0;
        const int32_t gid1 = (RB > 1 && tid + NT < cnt) ? batch[tid + NT].gid : 0;
        // per-slot opacity and beta for the flush (the buffer may be refilled
        // while other threads still flush)
        const float op0 = (tid < cnt) ? batch[tid].opac : 0.f;
        const float be0 = (tid < cnt) ? batch[tid].beta : 0.f;
        const float op1 = (RB > 1 && tid + NT < cnt) ? batch[tid + NT].opac : 0.f;
        const float be1 = (RB > 1 && tid + NT < cnt) ? batch[tid + NT].beta : 0.f;
        const float3 cn0 = (tid < cnt) ? make_float3(batch[tid].cxx, batch[tid].cxy, batch[tid].cyy)
                                       : make_float3(0.f, 0.f, 0.f);
        const float3 cn1 = (RB > 1 && tid + NT < cnt)
                               ? make_float3(batch[tid + NT].cxx, batch[tid + NT].cxy,
                                             batch[tid + NT].cyy)
                               : make_float3(0.f, 0.f, 0.f);
        build_masks<RB>(batch, cnt, lo, NT, nw, wpr, tx * a.TS, ty * a.TS, tid, lane, wmask,
                        wbin);
        if (!PACK) {
#pragma unroll
            for (int half = 0; half < RB; ++half) {
                const int sl = tid + half * NT;
                if (sl < cnt) {
                    const float *cp = a.colors + (int64_t)(half ? gid1 : gid0) * CD;
#pragma unroll
                    for (int k = 0; k < CD; ++k) scol[(buf * BR + sl) * CD + k] = cp[k];
                }
            }
        }
        if (__syncthreads_or(!ok)) {
            if (tid == 0) atomicOr(a.status, DEV_ERR_WAIT_TIMEOUT);
            break;
        }
        int rows = 0; // KE > 0: entry rows this warp has filled in this batch
        for (int k = RB * nw - 1; k >= 0; --k) {
            uint32_t m = wmask[warp * RB * nw + k];
            while (m) {
                const int bit = 31 - __clz(m);
                m &= ~(1u << bit);
                const int t = k * 32 + bit;
                const int32_t idx = lo + t;
                const GeoRec q = batch[t];
                float col[CD];
                load_color<CD, PACK>(scol4, scol, buf * BR + t, col);
                float g[NV];
                grad_pair<CD>(q, col, px, npy, idx, sp, g);
                if constexpr (KE > 0) {
                    const float g0 = g[0], g1 = g[1];
                    g[0] = q.cxx * g0 + q.cxy * g1;
                    g[1] = q.cxy * g0 + q.cyy * g1;
                    if (rows < KE) {
                        float *row = gacc + (warp * KE + rows) * NV;
                        // every lane of a group holds the same total: all store it
                        auto put = [row](int u, float tot, bool) { row[u] = tot; };
                        ReduceChunks<0, NV>::run(g, lm, lane, put);
                        if (lane == 0) slot_row[warp * BR + t] = (uint8_t)rows;
                        ++rows;
                    } else { // list full: this record's sums go straight to the arrays
                        auto add = [&](int u, float tot, bool owner) {
                            if (owner && tot != 0.f)
                                atomicAdd(grad_dst<CD>(a, u, q.gid),
                                          record_scale(u, q.opac, q.beta, true) * tot);
                        };
                        ReduceChunks<0, NV>::run(g, lm, lane, add);
                    }
                } else {
                    float *acc = gacc + t * NV;
                    auto add = [acc](int u, float tot, bool owner) {
                        if (owner && tot != 0.f) atomicAdd(&acc[u], tot);
                    };
                    ReduceChunks<0, NV>::run(g, lm, lane, add);
                    if (lane == 0) touched[t] = 1;
                }
            }
        }
        __syncthreads();
        if constexpr (KE > 0) {
#pragma unroll
            for (int half = 0; half < RB; ++half) {
                const int sl = tid + half * NT;
                if (sl >= cnt) continue;
                float sum[NV];
                bool any = false;
#pragma unroll
                for (int u = 0; u < NV; ++u) sum[u] = 0.f;
                for (int w = 0; w < nw; ++w) {
                    const int r = slot_row[w * BR + sl];
                    if (r == 0xFF) continue;
                    slot_row[w * BR + sl] = 0xFF;
                    any = true;
                    const float *row = gacc + (w * KE + r) * NV;
#pragma unroll
                    for (int u = 0; u < NV; ++u) sum[u] += row[u];
                }
                if (!any) continue;
                const int64_t gg = half ? gid1 : gid0;
                const float op = half ? op1 : op0, be = half ? be1 : be0;
#pragma unroll
                for (int u = 0; u < NV; ++u) sum[u] *= record_scale(u, op, be, true);
                if (NV <= GRAD_ROW && a.v_rows) {
                    // three 16-byte vector atomics per row instead of NV scalar ones
                    float4 *row = reinterpret_cast<float4 *>(a.v_rows + gg * GRAD_ROW);
#pragma unroll
                    for (int c = 0; c < (NV + 3) / 4; ++c) {
                        float4 v;
                        v.x = sum[4 * c];
                        v.y = 4 * c + 1 < NV ? sum[(4 * c + 1) % NV] : 0.f;
                        v.z = 4 * c + 2 < NV ? sum[(4 * c + 2) % NV] : 0.f;
                        v.w = 4 * c + 3 < NV ? sum[(4 * c + 3) % NV] : 0.f;
                        atomicAdd(row + c, v);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < NV; ++u)
                        if (sum[u] != 0.f) atomicAdd(grad_dst<CD>(a, u, gg), sum[u]);
                }
            }
            continue;
        }
#pragma unroll
        for (int half = 0; half < RB; ++half) {
            const int sl = tid + half * NT;
            if (sl < cnt && touched[sl]) {
                const int64_t gg = half ? gid1 : gid0;
                const float op = half ? op1 : op0, be = half ? be1 : be0;
                const float3 cn = half ? cn1 : cn0;
                float *ga = gacc + sl * NV;
                const float f2 = -2.f * op * be;
                const float m0 = f2 * (cn.x * ga[0] + cn.y * ga[1]);
                const float m1 = f2 * (cn.y * ga[0] + cn.z * ga[1]);
#pragma unroll
                for (int u = 0; u < NV; ++u) {
                    const float val = u == 0 ? m0 : u == 1 ? m1 : ga[u] * record_scale(u, op, be);
                    if (val != 0.f) atomicAdd(grad_dst<CD>(a, u, gg), val);
                    ga[u] = 0.f;
                }
                touched[sl] = 0;
            }
        }
    }
    // no copy may still target this CTA's shared memory at exit
    if (gather) cp_async_wait_all();
    if (tid == 0)
        for (int b = waited; b < issued; ++b)
            if (!mbar_wait_bounded(&mbar[b & 1], (b >> 1) & 1))
                atomicOr(a.status, DEV_ERR_WAIT_TIMEOUT);
}

// ------------------------------------------------------------- host side
static bool channels_supported(int ch) {
    switch (ch) {
    case 1: case 2: case 3: case 4: case 5: case 8: case 9:
    case 16: case 17: case 32: case 33:
        return true;
    default:
        return false;
    }
}

size_t raster_ws_bytes(int64_t T, int ch) {
    size_t b = 256 + (size_t)T * sizeof(GeoRec);
    if (ch <= 4) b += (size_t)T * 16;
    return b;
}

template <int CD>
static int launch_pack(int64_t T, int64_t n_prims, const int32_t *fl, const float *m2,
                       const float *cn, const float *op, const float *be, const float *col,
                       GeoRec *recs, float4 *rcols, uint32_t *status, cudaStream_t st) {
    constexpr bool PACK = CD <= 4;
    const int blk = 256;
    const int64_t nblk = (T + blk - 1) / blk;
    const unsigned grid = (unsigned)(nblk < 152 * 16 ? nblk : 152 * 16);
    UBS_TIMED("raster_pack", st,
              pack_records_kernel<CD, PACK><<<grid, blk, 0, st>>>(
                  T, n_prims, fl, m2, cn, op, be, col, recs, PACK ? rcols : nullptr, status));
    note_launch();
    return check_launch("pack_records");
}

// Variants of the 3-channel blend kernels for tiles of at most 128 threads
// (16 x 16 pixels and smaller), selected process-wide by
// ubs_set_blend_variant.  The forward's trade records per staged batch (RB)
// against CTAs per SM (MINB, the register bound it implies); the backward's
// the register bound and the accumulation scheme (see smem_layout) --
//   forward:  0: RB 2, 8 CTAs/SM;  1: RB 1, 10 CTAs/SM;  2: RB 2, 6 CTAs/SM
//   backward: 0: RB 1, 8 CTAs/SM, per-warp row lists of 64 entries;
//             1: the same at 7 CTAs/SM (72 registers);
//             2: RB 1, 8 CTAs/SM, shared accumulators with shared atomics
// Every variant computes the same images; the backward's gradient sums are
// the same up to the order of their additions.
// A warp that visits more than KE_SMALL records of one 128-record batch adds
// the rest straight to the gradient arrays; on the 1M-primitive 1080p frame
// 64 of 5.6M visits do.
std::atomic<int> g_blend_fwd_variant{0}, g_blend_bwd_variant{0};
constexpr int kBlendVariants = 3;
constexpr int KE_SMALL = 64; // backward entry rows per warp in tiles of at most 128 threads

template <int CD, bool BWD>
static int launch_blend(RasterArgs &a, cudaStream_t st) {
    constexpr bool PACK = CD <= 4;
    const int NT = a.TS * a.TS / 2; // two pixels per thread
    // Tiles of at most 128 threads with packed colours run 8 CTAs per SM (7
    // for the backward of 4 channels; wider colour rows need more registers),
    // the backward in batches of NT records to fit its shared memory.
    const bool small = PACK && NT <= 128;
    const int variant = (small && CD == 3 && !a.pair_count)
                            ? (BWD ? g_blend_bwd_variant.load() : g_blend_fwd_variant.load())
                            : 0;
    int RB = (small && BWD) ? 1 : 2;
    if (!BWD && variant == 1) RB = 1;
    const int KE = (BWD && small && !(CD == 3 && variant == 2)) ? KE_SMALL : 0;
    const SmemLayout L = smem_layout<CD, PACK, BWD>(NT, RB, KE);
    if (L.total > 227 * 1024)
        return set_error(UBS_ERR_UNSUPPORTED, "raster: tile_size %d with %d channels needs %d B "
                                              "of shared memory", a.TS, CD, L.total);
    const unsigned nblocks = (unsigned)a.n_buckets;
    if (nblocks == 0) return UBS_OK;
    void (*k)(RasterArgs) = nullptr;
    if constexpr (CD == 3) {
        if (small && variant == 1)
            k = BWD ? raster_bwd_kernel<3, true, 1, 7, KE_SMALL>
                    : raster_fwd_kernel<3, true, false, 1, 10>;
        else if (small && variant == 2)
            k = BWD ? raster_bwd_kernel<3, true, 1, 8, 0> : raster_fwd_kernel<3, true, false, 2, 6>;
    }
    if constexpr (PACK) {
        if (small && !k)
            k = BWD ? raster_bwd_kernel<CD, PACK, 1, (CD < 4 ? 8 : 7), KE_SMALL>
                    : (a.pair_count ? raster_fwd_kernel<CD, PACK, true, 2, 8>
                                    : raster_fwd_kernel<CD, PACK, false, 2, 8>);
    }
    if (!k)
        k = BWD ? raster_bwd_kernel<CD, PACK, 2, 1, 0>
                : (a.pair_count ? raster_fwd_kernel<CD, PACK, true, 2, 1>
                                : raster_fwd_kernel<CD, PACK, false, 2, 1>);
    if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, L.total) !=
        cudaSuccess)
        return check_launch("raster smem attribute");
    UBS_TIMED(BWD ? "raster_bwd" : "raster_fwd", st, k<<<nblocks, NT, L.total, st>>>(a));
    note_launch();
    return check_launch(BWD ? "raster_bwd" : "raster_fwd");
}

#define UBS_CHANNEL_SWITCH(ch, ...)                                                        \
    switch (ch) {                                                                          \
    case 1: { constexpr int CDV = 1; __VA_ARGS__; }                                        \
    case 2: { constexpr int CDV = 2; __VA_ARGS__; }                                        \
    case 3: { constexpr int CDV = 3; __VA_ARGS__; }                                        \
    case 4: { constexpr int CDV = 4; __VA_ARGS__; }                                        \
    case 5: { constexpr int CDV = 5; __VA_ARGS__; }                                        \
    case 8: { constexpr int CDV = 8; __VA_ARGS__; }                                        \
    case 9: { constexpr int CDV = 9; __VA_ARGS__; }                                        \
    case 16: { constexpr int CDV = 16; __VA_ARGS__; }                                      \
    case 17: { constexpr int CDV = 17; __VA_ARGS__; }                                      \
    case 32: { constexpr int CDV = 32; __VA_ARGS__; }                                      \
    case 33: { constexpr int CDV = 33; __VA_ARGS__; }                                      \
    default: return set_error(UBS_ERR_UNSUPPORTED, "raster: %d channels", ch);           \
    }

static bool channels_ok(int ch) {
    switch (ch) {
    case 1: case 2: case 3: case 4: case 5: case 8: case 9:
    case 16: case 17: case 32: case 33:
        return true;
    default:
        return false;
    }
}

static int validate_ws(int32_t ch, int64_t T, void *ws, size_t ws_bytes) {
    UBS_REQUIRE(T >= 0 && T < (1ll << 31), "raster: n_isects %lld out of range", (long long)T);
    if (!channels_ok(ch))
        return set_error(UBS_ERR_UNSUPPORTED, "raster: %d channels (supported 1-5, 8, 9, 16, "
                                              "17, 32, 33)", ch);
    UBS_REQUIRE(ws != nullptr && ((uintptr_t)ws & 255) == 0,
                "raster: workspace must be 256-byte aligned");
    if (ws_bytes < raster_ws_bytes(T, ch))
        return set_error(UBS_ERR_OVERFLOW, "raster: workspace %zu B < %zu B needed", ws_bytes,
                         raster_ws_bytes(T, ch));
    return UBS_OK;
}

static int validate_raster(int32_t C, int64_t N, int32_t ch, int64_t T, int32_t W, int32_t H,
                           int32_t ts, int32_t tw, int32_t th, void *ws, size_t ws_bytes) {
    UBS_REQUIRE(C >= 1 && N >= 0 && W >= 0 && H >= 0, "raster: bad sizes C=%d N=%lld W=%d H=%d",
                C, (long long)N, W, H);
    UBS_REQUIRE((int64_t)C * N < (1ll << 31), "raster: C*N must fit in int32");
    if (!(ts == 8 || ts == 16 || ts == 24 || ts == 32))
        return set_error(UBS_ERR_UNSUPPORTED, "raster: tile_size %d (supported 8, 16, 24, 32)",
                         ts);
    UBS_REQUIRE(tw >= 1 && th >= 1 && (int64_t)tw * ts >= W && (int64_t)th * ts >= H,
                "raster: tile grid %dx%d of %d px does not cover %dx%d", tw, th, ts, W, H);
    return validate_ws(ch, T, ws, ws_bytes);
}

static void fill_common(RasterArgs &a, int32_t C, int64_t N, int32_t ch, int64_t T, int32_t W,
                        int32_t H, int32_t ts, int32_t tw, int32_t th, const int32_t *offs,
                        const float *colors, const float *bg, const uint8_t *masks, void *ws) {
    a.C = C;
    a.W = W;
    a.H = H;
    a.TS = ts;
    a.TW = tw;
    a.TH = th;
    a.n_tiles = tw * th;
    a.n_isects = T;
    a.n_prims = (int64_t)C * N;
    a.offsets = offs;
    unsigned char *w = static_cast<unsigned char *>(ws);
    a.status = reinterpret_cast<uint32_t *>(w);
    a.recs = reinterpret_cast<const GeoRec *>(w + 256);
    a.rcols = ch <= 4 ? reinterpret_cast<const float4 *>(w + 256 + T * sizeof(GeoRec)) : nullptr;
    a.colors = colors;
    a.bg = bg;
    a.masks = masks;
    a.pair_count = nullptr;
    a.v_tile_base = nullptr;
    a.v_dims = nullptr;
    a.v_pix_base = nullptr;
    a.n_buckets = C * tw * th;
    a.n_isects_dev = nullptr;
    a.order = nullptr;
}

// Blend of the fused multi-view path (scene.cu): 3 colour channels packed
// with the records, per-view grids, intersection count read on the device.
int scene_blend(int fwd, int32_t C, int64_t CN, int32_t n_buckets, int32_t tile_size,
                const int32_t *offsets, const int32_t *order, const int64_t *T_dev, int64_t cap,
                const uint64_t *keys, const void *entry_recs, const float4 *prim_cols,
                const float *bg, const int32_t *tile_base,
                const int32_t *dims, const int64_t *pix_base, float *out_c, float *out_a,
                int32_t *last_ids, const float *render_alphas, const int32_t *last_in,
                const float *v_out_c, const float *v_out_a, float *v_rows, uint32_t *status,
                cudaStream_t st) {
    RasterArgs a{};
    a.C = C;
    a.TS = tile_size;
    a.n_isects = cap;
    a.n_prims = CN;
    a.offsets = offsets;
    a.keys = keys;
    a.entry_recs = static_cast<const GeoRec *>(entry_recs);
    a.prim_cols = prim_cols;
    a.n_per_view = CN / C;
    a.bg = bg;
    a.status = status;
    a.v_tile_base = tile_base;
    a.v_dims = dims;
    a.v_pix_base = pix_base;
    a.n_buckets = n_buckets;
    a.n_isects_dev = T_dev;
    a.order = order;
    if (fwd) {
        a.out_c = out_c;
        a.out_a = out_a;
        a.last_ids = last_ids;
        return launch_blend<3, false>(a, st);
    }
    a.render_alphas = render_alphas;
    a.last_in = last_in;
    a.v_out_c = v_out_c;
    a.v_out_a = v_out_a;
    a.v_rows = v_rows;
    return launch_blend<3, true>(a, st);
}

} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_raster_workspace_bytes(int64_t n_isects, int32_t channels) {
    return raster_ws_bytes(n_isects < 0 ? 0 : n_isects, channels);
}

int ubs_raster_pack(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                    const int32_t *flatten_ids, const float *means2d, const float *conics,
                    const float *opacities, const float *betas, const float *colors,
                    void *workspace, size_t workspace_bytes, void *stream) {
    UBS_REQUIRE(C >= 1 && N >= 0 && (int64_t)C * N < (1ll << 31), "raster_pack: bad sizes");
    if (int e = validate_ws(channels, n_isects, workspace, workspace_bytes)) return e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    unsigned char *w = static_cast<unsigned char *>(workspace);
    if (cudaMemsetAsync(w, 0, 256, st) != cudaSuccess) return check_launch("raster_pack memset");
    if (n_isects == 0) return UBS_OK;
    GeoRec *recs = reinterpret_cast<GeoRec *>(w + 256);
    float4 *rcols = reinterpret_cast<float4 *>(w + 256 + n_isects * sizeof(GeoRec));
    uint32_t *status = reinterpret_cast<uint32_t *>(w);
    const int64_t P = (int64_t)C * N;
    UBS_CHANNEL_SWITCH(channels, return launch_pack<CDV>(n_isects, P, flatten_ids, means2d,
                                                         conics, opacities, betas, colors, recs,
                                                         rcols, status, st));
}

int ubs_raster_fwd_packed(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                          const float *colors, const float *backgrounds, const uint8_t *masks,
                          int32_t width, int32_t height, int32_t tile_size, int32_t tile_width,
                          int32_t tile_height, const int32_t *isect_offsets,
                          float *render_colors, float *render_alphas, int32_t *last_ids,
                          int32_t count_pairs, void *workspace, size_t workspace_bytes,
                          void *stream) {
    if (int e = validate_raster(C, N, channels, n_isects, width, height, tile_size, tile_width,
                                tile_height, workspace, workspace_bytes))
        return e;
    RasterArgs a{};
    fill_common(a, C, N, channels, n_isects, width, height, tile_size, tile_width, tile_height,
                isect_offsets, colors, backgrounds, masks, workspace);
    a.out_c = render_colors;
    a.out_a = render_alphas;
    a.last_ids = last_ids;
    if (count_pairs)
        a.pair_count = reinterpret_cast<unsigned long long *>(static_cast<unsigned char *>(workspace) + 8);
    UBS_CHANNEL_SWITCH(channels, return launch_blend<CDV, false>(a, static_cast<cudaStream_t>(stream)));
}

int ubs_raster_bwd_packed(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                          const float *colors, const float *backgrounds, const uint8_t *masks,
                          int32_t width, int32_t height, int32_t tile_size, int32_t tile_width,
                          int32_t tile_height, const int32_t *isect_offsets,
                          const float *render_alphas, const int32_t *last_ids,
                          const float *v_render_colors, const float *v_render_alphas,
                          float *v_means2d, float *v_conics, float *v_colors, float *v_opacities,
                          float *v_betas, int32_t zero_outputs, void *workspace,
                          size_t workspace_bytes, void *stream) {
    if (int e = validate_raster(C, N, channels, n_isects, width, height, tile_size, tile_width,
                                tile_height, workspace, workspace_bytes))
        return e;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t P = (int64_t)C * N;
    if (zero_outputs &&
        (cudaMemsetAsync(v_means2d, 0, P * 2 * 4, st) ||
         cudaMemsetAsync(v_conics, 0, P * 3 * 4, st) ||
         cudaMemsetAsync(v_colors, 0, P * channels * 4, st) ||
         cudaMemsetAsync(v_opacities, 0, P * 4, st) || cudaMemsetAsync(v_betas, 0, P * 4, st)))
        return check_launch("raster_bwd memset");
    if (n_isects == 0) return UBS_OK;
    RasterArgs a{};
    fill_common(a, C, N, channels, n_isects, width, height, tile_size, tile_width, tile_height,
                isect_offsets, colors, backgrounds, masks, workspace);
    a.render_alphas = render_alphas;
    a.last_in = last_ids;
    a.v_out_c = v_render_colors;
    a.v_out_a = v_render_alphas;
    a.v_m2 = v_means2d;
    a.v_cn = v_conics;
    a.v_col = v_colors;
    a.v_op = v_opacities;
    a.v_be = v_betas;
    UBS_CHANNEL_SWITCH(channels, return launch_blend<CDV, true>(a, st));
}

int ubs_raster_fwd(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                   const float *means2d, const float *conics, const float *colors,
                   const float *opacities, const float *betas, const float *backgrounds,
                   const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                   int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                   const int32_t *flatten_ids, float *render_colors, float *render_alphas,
                   int32_t *last_ids, void *workspace, size_t workspace_bytes, void *stream) {
    if (int e = validate_raster(C, N, channels, n_isects, width, height, tile_size, tile_width,
                                tile_height, workspace, workspace_bytes))
        return e;
    if (int e = ubs_raster_pack(C, N, channels, n_isects, flatten_ids, means2d, conics,
                                opacities, betas, colors, workspace, workspace_bytes, stream))
        return e;
    return ubs_raster_fwd_packed(C, N, channels, n_isects, colors, backgrounds, masks, width,
                                 height, tile_size, tile_width, tile_height, isect_offsets,
                                 render_colors, render_alphas, last_ids, 0, workspace,
                                 workspace_bytes, stream);
}

int ubs_raster_bwd(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                   const float *means2d, const float *conics, const float *colors,
                   const float *opacities, const float *betas, const float *backgrounds,
                   const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                   int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                   const int32_t *flatten_ids, const float *render_alphas,
                   const int32_t *last_ids, const float *v_render_colors,
                   const float *v_render_alphas, float *v_means2d, float *v_conics,
                   float *v_colors, float *v_opacities, float *v_betas, void *workspace,
                   size_t workspace_bytes, void *stream) {
    if (int e = validate_raster(C, N, channels, n_isects, width, height, tile_size, tile_width,
                                tile_height, workspace, workspace_bytes))
        return e;
    if (int e = ubs_raster_pack(C, N, channels, n_isects, flatten_ids, means2d, conics,
                                opacities, betas, colors, workspace, workspace_bytes, stream))
        return e;
    return ubs_raster_bwd_packed(C, N, channels, n_isects, colors, backgrounds, masks, width,
                                 height, tile_size, tile_width, tile_height, isect_offsets,
                                 render_alphas, last_ids, v_render_colors, v_render_alphas,
                                 v_means2d, v_conics, v_colors, v_opacities, v_betas, 1,
                                 workspace, workspace_bytes, stream);
}

int ubs_set_blend_variant(int32_t forward, int32_t backward) {
    UBS_REQUIRE(forward >= 0 && forward < kBlendVariants && backward >= 0 &&
                    backward < kBlendVariants,
                "set_blend_variant: variants %d, %d (supported 0 .. %d)", forward, backward,
                kBlendVariants - 1);
    g_blend_fwd_variant.store(forward);
    g_blend_bwd_variant.store(backward);
    return UBS_OK;
}

int ubs_get_blend_variant(int32_t *forward, int32_t *backward) {
    UBS_REQUIRE(forward && backward, "get_blend_variant: null pointer");
    *forward = g_blend_fwd_variant.load();
    *backward = g_blend_bwd_variant.load();
    return UBS_OK;
}

int ubs_raster_status(const void *workspace, uint32_t *status, uint64_t *pair_count,
                      void *stream) {
    UBS_REQUIRE(workspace && status, "raster_status: null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t hdr[2];
    if (cudaMemcpyAsync(hdr, workspace, 16, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("raster_status");
    *status = (uint32_t)(hdr[0] & 0xffffffffu);
    if (pair_count) *pair_count = hdr[1];
    return UBS_OK;
}

int ubs_raster_pair_counts(const void *workspace, uint64_t *counts, void *stream) {
    UBS_REQUIRE(workspace && counts, "raster_pair_counts: null pointer");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    uint64_t hdr[4];
    if (cudaMemcpyAsync(hdr, workspace, 32, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("raster_pair_counts");
    counts[0] = hdr[1];
    counts[1] = hdr[2];
    counts[2] = hdr[3];
    return UBS_OK;
}

} // extern "C"
