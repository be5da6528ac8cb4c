// isect.cu -- tile intersection, key build, (tile, depth) sort and offsets.
//
// Reference: submodules/gsplat/cuda/csrc/isect_tiles.cu:17-285 (two passes,
// torch cumsum, a blocking .item() and cub::DeviceRadixSort::SortPairs over
// bits [0, 32 + tile_bits + cam_bits)) and isect_tiles.cu:287-367 (offsets).
//
// Design here: the order the reference produces is "stable sort by
// (camera, tile, depth bits)", and within one (camera, tile) bucket a primitive
// appears at most once, so equal depths are ordered by flatten index.  The
// kernels therefore
//   1. count intersections per primitive and per (camera, tile) bucket,
//   2. scan the bucket counts on the device (these are the tile offsets the
//      reference computes separately with isect_offset_encode),
//   3. scatter each intersection into its bucket with a 64-bit key
//      (depth bits << 32 | flatten index), unique per bucket,
//   4. sort each bucket in shared memory (bitonic) or, for long buckets, with a
//      CTA merge sort in global memory, and write isect_ids / flatten_ids.
// Because the per-bucket keys are unique the result is bit-identical to the
// reference's stable radix sort, independent of scatter order.
#include <algorithm>

#include "ubs_common.cuh"

namespace ubs {

constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_TILE = SCAN_ITEMS * SCAN_THREADS;
constexpr int SMALL_SEG = 4096;       // largest bucket sorted in shared memory
constexpr int SORT_THREADS = 256;
constexpr int BIG_THREADS = 1024;
constexpr int MERGE_ITEMS = 8;

struct IsectHeader {
    int64_t total;     // number of intersections
    uint32_t status;   // DeviceError bits
    int32_t n_big;     // number of buckets longer than SMALL_SEG
    int64_t pad[6];
};
static_assert(sizeof(IsectHeader) <= 256, "header too large");

static uint32_t bit_width_u32(uint32_t v) {
    uint32_t b = 0;
    while (v) {
        ++b;
        v >>= 1;
    }
    return b;
}

static size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

struct CountWs {
    IsectHeader *hdr;
    int32_t *bucket_counts; // [C*n_tiles]
    int64_t *block_sums;    // [n_scan_blocks]
    size_t bytes;
};
static CountWs count_ws_layout(void *base, int32_t C, int64_t N, int32_t n_tiles) {
    CountWs w{};
    unsigned char *p = static_cast<unsigned char *>(base);
    const int64_t nb = (int64_t)C * n_tiles;
    const int64_t nblocks = (std::max<int64_t>(nb, (int64_t)C * N) + SCAN_TILE - 1) / SCAN_TILE;
    size_t off = 256;
    w.hdr = reinterpret_cast<IsectHeader *>(p);
    w.bucket_counts = reinterpret_cast<int32_t *>(p + off);
    off = align256(off + nb * 4);
    w.block_sums = reinterpret_cast<int64_t *>(p + off);
    off = align256(off + (nblocks + 1) * 8);
    w.bytes = off;
    return w;
}

struct SortWs {
    CountWs cw;
    int32_t *cursor;     // [C*n_tiles]
    uint64_t *keys;      // [T]
    uint64_t *scratch;   // [T]
    int32_t *big_list;   // [C*n_tiles]
    int64_t *prim_start; // [C*N] (generation-order emit)
    size_t bytes;
};
static SortWs sort_ws_layout(void *base, int32_t C, int64_t N, int32_t n_tiles, int64_t T) {
    SortWs w{};
    w.cw = count_ws_layout(base, C, N, n_tiles);
    unsigned char *p = static_cast<unsigned char *>(base);
    const int64_t nb = (int64_t)C * n_tiles;
    size_t off = w.cw.bytes;
    w.cursor = reinterpret_cast<int32_t *>(p + off);
    off = align256(off + nb * 4);
    w.keys = reinterpret_cast<uint64_t *>(p + off);
    off = align256(off + T * 8);
    w.scratch = reinterpret_cast<uint64_t *>(p + off);
    off = align256(off + T * 8);
    w.big_list = reinterpret_cast<int32_t *>(p + off);
    off = align256(off + nb * 4);
    w.prim_start = reinterpret_cast<int64_t *>(p + off);
    off = align256(off + (int64_t)C * N * 8);
    w.bytes = off;
    return w;
}

// -------------------------------------------------------- tile bounding box
// isect_tiles.cu:46-66: float tile coordinates, floor/ceil, float -> uint32
// conversion (truncating, saturating at 0 for negatives), clamp to the grid.
struct Box {
    uint32_t x0, y0, x1, y1;
};
__device__ __forceinline__ Box tile_box(float mx, float my, int32_t radius, float ts,
                                        uint32_t tw, uint32_t th) {
    const float r = (float)radius / ts;
    const float tx = mx / ts, ty = my / ts;
    Box b;
    b.x0 = min(max(0u, __float2uint_rz(floorf(tx - r))), tw);
    b.y0 = min(max(0u, __float2uint_rz(floorf(ty - r))), th);
    b.x1 = min(max(0u, __float2uint_rz(ceilf(tx + r))), tw);
    b.y1 = min(max(0u, __float2uint_rz(ceilf(ty + r))), th);
    return b;
}

__global__ void isect_count_kernel(int64_t CN, int64_t N, const float2 *__restrict__ means2d,
                                   const int32_t *__restrict__ radii,
                                   const float *__restrict__ depths, float ts, uint32_t tw,
                                   uint32_t th, int32_t *__restrict__ tiles_per_gauss,
                                   int32_t *__restrict__ bucket_counts, uint32_t *status) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= CN) return;
    const int32_t rad = radii[idx];
    if (rad <= 0) {
        tiles_per_gauss[idx] = 0;
        return;
    }
    const float2 m = means2d[idx];
    const Box b = tile_box(m.x, m.y, rad, ts, tw, th);
    tiles_per_gauss[idx] = (int32_t)((b.y1 - b.y0) * (b.x1 - b.x0));
    if (b.x1 <= b.x0 || b.y1 <= b.y0) return;
    if (__float_as_int(depths[idx]) < 0) atomicOr(status, DEV_ERR_NEG_DEPTH);
    const int64_t cam = idx / N;
    int32_t *bc = bucket_counts + cam * (int64_t)tw * th;
    for (uint32_t y = b.y0; y < b.y1; ++y)
        for (uint32_t x = b.x0; x < b.x1; ++x) atomicAdd(&bc[y * tw + x], 1);
}

// ------------------------------------------------------------------- scan
// Exclusive scan of int32 counts.  Per block: SCAN_TILE items; block-local
// prefixes go to out, block totals to block_sums; a single block scans the
// totals, a last pass adds them.  OutT is int32_t or int64_t.
template <typename OutT>
__global__ void __launch_bounds__(SCAN_THREADS) scan_blocks_kernel(const int32_t *__restrict__ in,
                                                                  OutT *__restrict__ out,
                                                                  int64_t n,
                                                                  int64_t *__restrict__ sums) {
    __shared__ int64_t warp_tot[32];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE + (int64_t)tid * SCAN_ITEMS;
    int64_t v[SCAN_ITEMS];
    int64_t run = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k) {
        const int64_t x = (base + k < n) ? (int64_t)in[base + k] : 0;
        v[k] = run;
        run += x;
    }
    // inclusive warp scan of thread totals
    int64_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) warp_tot[warp] = inc;
    __syncthreads();
    if (warp == 0) {
        int64_t w = warp_tot[lane];
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        warp_tot[lane] = wi - w; // exclusive
        if (lane == 31) sums[blockIdx.x] = wi;
    }
    __syncthreads();
    const int64_t off = warp_tot[warp] + (inc - run);
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; ++k)
        if (base + k < n) out[base + k] = (OutT)(v[k] + off);
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_sums_kernel(int64_t *sums, int64_t nblocks,
                                                                 int64_t *total) {
    __shared__ int64_t warp_tot[32];
    __shared__ int64_t carry;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) carry = 0;
    __syncthreads();
    for (int64_t base = 0; base < nblocks; base += SCAN_THREADS) {
        const int64_t i = base + tid;
        const int64_t x = i < nblocks ? sums[i] : 0;
        int64_t inc = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += y;
        }
        if (lane == 31) warp_tot[warp] = inc;
        __syncthreads();
        if (warp == 0) {
            const int64_t w = warp_tot[lane];
            int64_t wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int64_t y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            warp_tot[lane] = wi - w;
        }
        __syncthreads();
        const int64_t c0 = carry;
        if (i < nblocks) sums[i] = c0 + warp_tot[warp] + inc - x;
        __syncthreads();
        if (tid == SCAN_THREADS - 1) carry = c0 + warp_tot[warp] + inc;
        __syncthreads();
    }
    if (tid == 0) *total = carry;
}

template <typename OutT>
__global__ void scan_add_kernel(OutT *out, int64_t n, const int64_t *__restrict__ sums) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = (OutT)((int64_t)out[i] + sums[i / SCAN_TILE]);
}

template <typename OutT>
static int device_exclusive_scan(const int32_t *in, OutT *out, int64_t n, int64_t *sums,
                                 int64_t *total, cudaStream_t st) {
    if (n == 0) {
        if (cudaMemsetAsync(total, 0, 8, st) != cudaSuccess) return check_launch("scan memset");
        return UBS_OK;
    }
    const int64_t nblocks = (n + SCAN_TILE - 1) / SCAN_TILE;
    scan_blocks_kernel<OutT><<<(unsigned)nblocks, SCAN_THREADS, 0, st>>>(in, out, n, sums);
    ::ubs::note_launch();
    scan_sums_kernel<<<1, SCAN_THREADS, 0, st>>>(sums, nblocks, total);
    ::ubs::note_launch();
    if (nblocks > 1) scan_add_kernel<OutT><<<grid_for(n, 256), 256, 0, st>>>(out, n, sums);
    ::ubs::note_launch();
    return check_launch("exclusive scan");
}

// ------------------------------------------------------------------- emit
__global__ void isect_emit_bucket_kernel(int64_t CN, int64_t N, const float2 *__restrict__ means2d,
                                         const int32_t *__restrict__ radii,
                                         const float *__restrict__ depths, float ts, uint32_t tw,
                                         uint32_t th, int32_t *__restrict__ cursor,
                                         uint64_t *__restrict__ keys, int64_t cap,
                                         uint32_t *status) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= CN) return;
    const int32_t rad = radii[idx];
    if (rad <= 0) return;
    const float2 m = means2d[idx];
    const Box b = tile_box(m.x, m.y, rad, ts, tw, th);
    const uint64_t key = ((uint64_t)(uint32_t)__float_as_int(depths[idx]) << 32) | (uint64_t)idx;
    const int64_t cam = idx / N;
    int32_t *cur = cursor + cam * (int64_t)tw * th;
    for (uint32_t y = b.y0; y < b.y1; ++y)
        for (uint32_t x = b.x0; x < b.x1; ++x) {
            const int32_t pos = atomicAdd(&cur[y * tw + x], 1);
            if (pos >= 0 && pos < cap) keys[pos] = key;
            else atomicOr(status, DEV_ERR_OVERFLOW);
        }
}

// reference generation order: primitive by primitive, tiles row-major
__global__ void isect_emit_ordered_kernel(int64_t CN, int64_t N, const float2 *__restrict__ means2d,
                                          const int32_t *__restrict__ radii,
                                          const float *__restrict__ depths, float ts,
                                          uint32_t tw, uint32_t th, uint32_t tile_bits,
                                          const int64_t *__restrict__ prim_start,
                                          int64_t *__restrict__ isect_ids,
                                          int32_t *__restrict__ flatten_ids, int64_t cap,
                                          uint32_t *status) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= CN) return;
    const int32_t rad = radii[idx];
    if (rad <= 0) return;
    const float2 m = means2d[idx];
    const Box b = tile_box(m.x, m.y, rad, ts, tw, th);
    const int64_t cam = idx / N;
    const int64_t denc = (int64_t)__float_as_int(depths[idx]); // sign-extended
    int64_t pos = prim_start[idx];
    for (uint32_t y = b.y0; y < b.y1; ++y)
        for (uint32_t x = b.x0; x < b.x1; ++x) {
            const int64_t tile = (int64_t)y * tw + x;
            if (pos < cap) {
                isect_ids[pos] = (cam << (32 + tile_bits)) | (tile << 32) | denc;
                flatten_ids[pos] = (int32_t)idx;
            } else {
                atomicOr(status, DEV_ERR_OVERFLOW);
            }
            ++pos;
        }
}

// ------------------------------------------------------------ bucket sort
__device__ __forceinline__ void write_sorted(uint64_t key, int64_t pos, int64_t cam,
                                             int64_t tile, uint32_t tile_bits,
                                             int64_t *isect_ids, int32_t *flatten_ids) {
    const int32_t dbits = (int32_t)(key >> 32);
    isect_ids[pos] = (cam << (32 + tile_bits)) | (tile << 32) | (int64_t)dbits;
    flatten_ids[pos] = (int32_t)(key & 0xffffffffu);
}

// In-place bitonic sort of s[0..n2) (n2 a power of two) by the whole CTA.
__device__ void block_bitonic(uint64_t *s, int n2) {
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < n2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const uint64_t a = s[i], b = s[ixj];
                    const bool up = (i & k) == 0;
                    if ((a > b) == up) {
                        s[i] = b;
                        s[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void __launch_bounds__(SORT_THREADS) bucket_sort_small_kernel(
    int64_t n_buckets, int32_t n_tiles, uint32_t tile_bits, const int32_t *__restrict__ offsets,
    int64_t T, const uint64_t *__restrict__ keys, int64_t *__restrict__ isect_ids,
    int32_t *__restrict__ flatten_ids, int32_t *big_list, IsectHeader *hdr) {
    __shared__ uint64_t s[SMALL_SEG];
    const int64_t bkt = blockIdx.x;
    const int64_t lo = offsets[bkt];
    const int64_t hi = (bkt + 1 < n_buckets) ? (int64_t)offsets[bkt + 1] : T;
    const int n = (int)(hi - lo);
    if (n <= 0) return;
    if (n > SMALL_SEG) {
        if (threadIdx.x == 0) big_list[atomicAdd(&hdr->n_big, 1)] = (int32_t)bkt;
        return;
    }
    int n2 = 1;
    while (n2 < n) n2 <<= 1;
    for (int i = threadIdx.x; i < n2; i += blockDim.x) s[i] = i < n ? keys[lo + i] : ~0ull;
    __syncthreads();
    block_bitonic(s, n2);
    const int64_t cam = bkt / n_tiles, tile = bkt - cam * n_tiles;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        write_sorted(s[i], lo + i, cam, tile, tile_bits, isect_ids, flatten_ids);
}

// merge path: number of elements taken from a for output diagonal d
__device__ __forceinline__ int64_t merge_split(const uint64_t *a, int64_t na, const uint64_t *b,
                                               int64_t nb, int64_t d) {
    int64_t lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (a[mid] < b[d - 1 - mid]) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// One CTA per long bucket: sort SMALL_SEG chunks in shared memory, then merge
// runs pairwise in global memory (keys <-> scratch), then write the result.
__global__ void __launch_bounds__(BIG_THREADS) bucket_sort_big_kernel(
    int32_t n_tiles, int64_t n_buckets, uint32_t tile_bits, const int32_t *__restrict__ offsets,
    int64_t T, uint64_t *keys, uint64_t *scratch, int64_t *__restrict__ isect_ids,
    int32_t *__restrict__ flatten_ids, const int32_t *big_list, const IsectHeader *hdr) {
    __shared__ uint64_t s[SMALL_SEG];
    const int n_big = hdr->n_big;
    for (int item = blockIdx.x; item < n_big; item += gridDim.x) {
    __syncthreads();
    const int64_t bkt = big_list[item];
    const int64_t lo = offsets[bkt];
    const int64_t hi = (bkt + 1 < n_buckets) ? (int64_t)offsets[bkt + 1] : T;
    const int64_t n = hi - lo;
    uint64_t *src = keys + lo, *dst = scratch + lo;
    for (int64_t c0 = 0; c0 < n; c0 += SMALL_SEG) {
        const int cn = (int)imin64(SMALL_SEG, n - c0);
        for (int i = threadIdx.x; i < SMALL_SEG; i += blockDim.x) s[i] = i < cn ? src[c0 + i] : ~0ull;
        __syncthreads();
        block_bitonic(s, SMALL_SEG);
        for (int i = threadIdx.x; i < cn; i += blockDim.x) src[c0 + i] = s[i];
        __syncthreads();
    }
    for (int64_t width = SMALL_SEG; width < n; width <<= 1) {
        for (int64_t r0 = 0; r0 < n; r0 += 2 * width) {
            const int64_t na = imin64(width, n - r0);
            const int64_t nb = imin64(width, n - r0 - na);
            const uint64_t *A = src + r0, *Bv = src + r0 + na;
            uint64_t *O = dst + r0;
            const int64_t total = na + nb;
            for (int64_t o0 = (int64_t)threadIdx.x * MERGE_ITEMS; o0 < total;
                 o0 += (int64_t)blockDim.x * MERGE_ITEMS) {
                int64_t ia = merge_split(A, na, Bv, nb, o0);
                int64_t ib = o0 - ia;
                const int64_t oend = imin64(total, o0 + MERGE_ITEMS);
                for (int64_t o = o0; o < oend; ++o) {
                    const bool take_a = ib >= nb || (ia < na && A[ia] < Bv[ib]);
                    O[o] = take_a ? A[ia++] : Bv[ib++];
                }
            }
        }
        __syncthreads();
        uint64_t *t = src;
        src = dst;
        dst = t;
    }
    const int64_t cam = bkt / n_tiles, tile = bkt - cam * n_tiles;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
        write_sorted(src[i], lo + i, cam, tile, tile_bits, isect_ids, flatten_ids);
    }
}

// ---------------------------------------------------------- offset encode
// offsets[b] = first sorted index whose (camera, tile) field is >= b: a
// binary search per bucket, equivalent to isect_tiles.cu:287-333 on sorted ids.
__global__ void offset_encode_kernel(int64_t T, const int64_t *__restrict__ ids, int64_t n_buckets,
                                     int32_t n_tiles, uint32_t tile_bits,
                                     int32_t *__restrict__ offsets) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n_buckets) return;
    const int64_t cam = b / n_tiles, tile = b - cam * n_tiles;
    const int64_t target = (cam << tile_bits) | tile;
    int64_t lo = 0, hi = T;
    while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if ((ids[mid] >> 32) < target) lo = mid + 1;
        else hi = mid;
    }
    offsets[b] = (int32_t)lo;
}

} // namespace ubs

using namespace ubs;

extern "C" {

size_t ubs_isect_count_workspace_bytes(int32_t C, int64_t N, int32_t n_tiles) {
    return count_ws_layout(nullptr, C, N, n_tiles).bytes;
}

size_t ubs_isect_sort_workspace_bytes(int32_t C, int64_t N, int32_t n_tiles, int64_t n_isects) {
    return sort_ws_layout(nullptr, C, N, n_tiles, n_isects < 0 ? 0 : n_isects).bytes;
}

int ubs_isect_count(int32_t C, int64_t N, const float *means2d, const int32_t *radii,
                    const float *depths, int32_t tile_size, int32_t tile_width,
                    int32_t tile_height, int32_t *tiles_per_gauss, int32_t *isect_offsets,
                    int64_t *n_isects, void *workspace, size_t workspace_bytes, void *stream) {
    UBS_REQUIRE(C >= 1 && N >= 0 && tile_size > 0 && tile_width > 0 && tile_height > 0,
                "isect_count: bad sizes");
    const int64_t n_tiles = (int64_t)tile_width * tile_height;
    UBS_REQUIRE(bit_width_u32((uint32_t)n_tiles) + bit_width_u32((uint32_t)C) <= 32,
                "isect_count: %lld tiles x %d cameras do not fit the 32-bit key field",
                (long long)n_tiles, C);
    UBS_REQUIRE((int64_t)C * N < (1ll << 31), "isect_count: C*N must fit in int32");
    UBS_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0,
                "isect_count: workspace must be 256-byte aligned");
    const CountWs w = count_ws_layout(workspace, C, N, (int32_t)n_tiles);
    if (workspace_bytes < w.bytes)
        return set_error(UBS_ERR_OVERFLOW, "isect_count: workspace %zu < %zu", workspace_bytes,
                         w.bytes);
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t CN = (int64_t)C * N;
    const int64_t nb = (int64_t)C * n_tiles;
    if (cudaMemsetAsync(w.hdr, 0, sizeof(IsectHeader), st) != cudaSuccess ||
        cudaMemsetAsync(w.bucket_counts, 0, nb * 4, st) != cudaSuccess)
        return check_launch("isect_count memset");
    if (CN > 0)
        isect_count_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
            CN, N, reinterpret_cast<const float2 *>(means2d), radii, depths, (float)tile_size,
            (uint32_t)tile_width, (uint32_t)tile_height, tiles_per_gauss, w.bucket_counts,
            &w.hdr->status);
    ::ubs::note_launch();
    if (int e = check_launch("isect_count")) return e;
    if (int e = device_exclusive_scan<int32_t>(w.bucket_counts, isect_offsets, nb, w.block_sums,
                                               &w.hdr->total, st))
        return e;
    IsectHeader h;
    if (cudaMemcpyAsync(&h, w.hdr, sizeof(h), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return check_launch("isect_count readback");
    if (h.status & DEV_ERR_NEG_DEPTH)
        return set_error(UBS_ERR_DEVICE, "isect_count: a visible primitive has a negative depth");
    if (h.total >= (1ll << 31))
        return set_error(UBS_ERR_OVERFLOW, "isect_count: %lld intersections exceed int32 indexing",
                         (long long)h.total);
    *n_isects = h.total;
    return UBS_OK;
}

int ubs_isect_emit(int32_t C, int64_t N, const float *means2d, const int32_t *radii,
                   const float *depths, int32_t tile_size, int32_t tile_width,
                   int32_t tile_height, const int32_t *tiles_per_gauss,
                   const int32_t *isect_offsets, int64_t n_isects, int32_t sort,
                   int64_t *isect_ids, int32_t *flatten_ids, void *workspace,
                   size_t workspace_bytes, void *stream) {
    UBS_REQUIRE(C >= 1 && N >= 0 && tile_size > 0 && tile_width > 0 && tile_height > 0 &&
                    n_isects >= 0,
                "isect_emit: bad sizes");
    UBS_REQUIRE(workspace && ((uintptr_t)workspace & 255) == 0,
                "isect_emit: workspace must be 256-byte aligned");
    const int64_t n_tiles = (int64_t)tile_width * tile_height;
    const SortWs w = sort_ws_layout(workspace, C, N, (int32_t)n_tiles, n_isects);
    if (workspace_bytes < w.bytes)
        return set_error(UBS_ERR_OVERFLOW, "isect_emit: workspace %zu < %zu", workspace_bytes,
                         w.bytes);
    if (n_isects == 0) return UBS_OK;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t CN = (int64_t)C * N;
    const int64_t nb = (int64_t)C * n_tiles;
    const uint32_t tile_bits = bit_width_u32((uint32_t)n_tiles);
    const float ts = (float)tile_size;
    const float2 *m2 = reinterpret_cast<const float2 *>(means2d);
    if (!sort) {
        int64_t *tot = &w.cw.hdr->pad[0];
        if (int e = device_exclusive_scan<int64_t>(tiles_per_gauss, w.prim_start, CN,
                                                   w.cw.block_sums, tot, st))
            return e;
        isect_emit_ordered_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
            CN, N, m2, radii, depths, ts, (uint32_t)tile_width, (uint32_t)tile_height, tile_bits,
            w.prim_start, isect_ids, flatten_ids, n_isects, &w.cw.hdr->status);
    ::ubs::note_launch();
        return check_launch("isect_emit_ordered");
    }
    if (cudaMemcpyAsync(w.cursor, isect_offsets, nb * 4, cudaMemcpyDeviceToDevice, st) !=
            cudaSuccess ||
        cudaMemsetAsync(&w.cw.hdr->n_big, 0, 4, st) != cudaSuccess)
        return check_launch("isect_emit init");
    isect_emit_bucket_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
        CN, N, m2, radii, depths, ts, (uint32_t)tile_width, (uint32_t)tile_height, w.cursor,
        w.keys, n_isects, &w.cw.hdr->status);
    ::ubs::note_launch();
    bucket_sort_small_kernel<<<(unsigned)nb, SORT_THREADS, 0, st>>>(
        nb, (int32_t)n_tiles, tile_bits, isect_offsets, n_isects, w.keys, isect_ids, flatten_ids,
        w.big_list, w.cw.hdr);
    ::ubs::note_launch();
    if (int e = check_launch("isect bucket sort")) return e;
    // long buckets (their number is only known on the device): a fixed grid
    // walks the device-side list, so the host never waits here
    if (n_isects > SMALL_SEG) {
        const int64_t max_big = n_isects / (SMALL_SEG + 1);
        const unsigned grid = (unsigned)imin64(imin64(max_big, nb), 304);
        bucket_sort_big_kernel<<<grid, BIG_THREADS, 0, st>>>(
            (int32_t)n_tiles, nb, tile_bits, isect_offsets, n_isects, w.keys, w.scratch,
            isect_ids, flatten_ids, w.big_list, w.cw.hdr);
    ::ubs::note_launch();
    }
    return check_launch("isect big-bucket sort");
}

int ubs_isect_offset_encode(int64_t n_isects, const int64_t *isect_ids, int32_t C,
                            int32_t tile_width, int32_t tile_height, int32_t *offsets,
                            void *stream) {
    UBS_REQUIRE(C >= 1 && tile_width > 0 && tile_height > 0 && n_isects >= 0,
                "isect_offset_encode: bad sizes");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int64_t n_tiles = (int64_t)tile_width * tile_height;
    const int64_t nb = (int64_t)C * n_tiles;
    if (n_isects == 0) {
        if (cudaMemsetAsync(offsets, 0, nb * 4, st) != cudaSuccess)
            return check_launch("offset_encode memset");
        return UBS_OK;
    }
    offset_encode_kernel<<<grid_for(nb, 256), 256, 0, st>>>(
        n_isects, isect_ids, nb, (int32_t)n_tiles, bit_width_u32((uint32_t)n_tiles), offsets);
    ::ubs::note_launch();
    return check_launch("offset_encode");
}

} // extern "C"
