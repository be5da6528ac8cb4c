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

#include "sort_common.cuh"

namespace ubs {

struct IsectHeader {
    int64_t total;     // number of intersections
    uint32_t status;   // DeviceError bits
    int32_t n_big;     // number of buckets longer than SMALL_SEG
    int32_t n_mid;     // number of buckets longer than WARP_SEG, at most SMALL_SEG
    int32_t pad0;
    int64_t pad[5];
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

// Per-tile counters of the count pass in kCountReplicas replicas
// ([replica][C * n_tiles], primitive entry idx counts in replica idx % R):
// a tile's atomics spread over that many L2 lines; they are folded into
// bucket_counts before the scan.
constexpr int kCountReplicas = 8;

struct CountWs {
    IsectHeader *hdr;
    int32_t *bucket_counts; // [C*n_tiles]
    int32_t *replicas;      // [kCountReplicas][C*n_tiles]
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
    w.replicas = reinterpret_cast<int32_t *>(p + off);
    off = align256(off + nb * kCountReplicas * 4);
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
                                   uint32_t th, int64_t nb, int32_t *__restrict__ tiles_per_gauss,
                                   int32_t *__restrict__ replicas, uint32_t *status) {
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
    int32_t *bc = replicas + (idx % kCountReplicas) * nb + cam * (int64_t)tw * th;
    for (uint32_t y = b.y0; y < b.y1; ++y)
        for (uint32_t x = b.x0; x < b.x1; ++x) atomicAdd(&bc[y * tw + x], 1);
}

__global__ void fold_count_replicas_kernel(const int32_t *__restrict__ replicas, int64_t nb,
                                           int32_t *__restrict__ counts) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= nb) return;
    int32_t c = 0;
#pragma unroll
    for (int r = 0; r < kCountReplicas; ++r) c += replicas[r * nb + b];
    counts[b] = c;
}

// ------------------------------------------------------------------- emit
__global__ void isect_emit_bucket_kernel(int64_t CN, int64_t N, const float2 *__restrict__ means2d,
                                         const int32_t *__restrict__ radii,
                                         const float *__restrict__ depths, float ts, uint32_t tw,
                                         uint32_t th, int32_t *__restrict__ cursor,
                                         uint64_t *__restrict__ keys, int64_t cap,
                                         uint32_t *status) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31;
    uint32_t n = 0, bw = 1;
    int32_t *cur = cursor;
    uint64_t key = 0;
    if (idx < CN && radii[idx] > 0) {
        const float2 m = means2d[idx];
        const Box b = tile_box(m.x, m.y, radii[idx], ts, tw, th);
        if (b.x1 > b.x0 && b.y1 > b.y0) {
            bw = b.x1 - b.x0;
            n = bw * (b.y1 - b.y0);
            const int64_t cam = idx / N;
            cur = cursor + cam * (int64_t)tw * th + (int64_t)b.y0 * tw + b.x0;
            key = ((uint64_t)(uint32_t)__float_as_int(depths[idx]) << 32) | (uint64_t)idx;
        }
    }
    warp_emit_rects(n, bw, tw, cur, key, lane, keys, cap, status);
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

// Sorted-entry writer of the drop-in operator: isect_ids (camera | tile |
// depth bits, the reference's key) and flatten_ids.
struct IdsWriter {
    int64_t *isect_ids;
    int32_t *flatten_ids;
    int32_t n_tiles;
    uint32_t tile_bits;
    __device__ __forceinline__ void operator()(uint64_t key, int64_t pos, int64_t bkt) const {
        const int64_t cam = bkt / n_tiles, tile = bkt - cam * n_tiles;
        const int32_t dbits = (int32_t)(key >> 32);
        isect_ids[pos] = (cam << (32 + tile_bits)) | (tile << 32) | (int64_t)dbits;
        flatten_ids[pos] = (int32_t)(key & 0xffffffffu);
    }
};

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
        cudaMemsetAsync(w.replicas, 0, nb * kCountReplicas * 4, st) != cudaSuccess)
        return check_launch("isect_count memset");
    if (CN > 0)
        UBS_TIMED("isect_count", st,
                  isect_count_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
                      CN, N, reinterpret_cast<const float2 *>(means2d), radii, depths,
                      (float)tile_size, (uint32_t)tile_width, (uint32_t)tile_height, nb,
                      tiles_per_gauss, w.replicas, &w.hdr->status));
    ::ubs::note_launch();
    if (int e = check_launch("isect_count")) return e;
    UBS_TIMED("isect_count_fold", st,
              fold_count_replicas_kernel<<<grid_for(nb, 256), 256, 0, st>>>(w.replicas, nb,
                                                                           w.bucket_counts));
    ::ubs::note_launch();
    if (int e = check_launch("isect_count fold")) return e;
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
        UBS_TIMED("isect_emit_ordered", st,
                  isect_emit_ordered_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
                      CN, N, m2, radii, depths, ts, (uint32_t)tile_width, (uint32_t)tile_height,
                      tile_bits, w.prim_start, isect_ids, flatten_ids, n_isects,
                      &w.cw.hdr->status));
    ::ubs::note_launch();
        return check_launch("isect_emit_ordered");
    }
    if (cudaMemcpyAsync(w.cursor, isect_offsets, nb * 4, cudaMemcpyDeviceToDevice, st) !=
        cudaSuccess)
        return check_launch("isect_emit init");
    UBS_TIMED("isect_emit", st,
              isect_emit_bucket_kernel<<<grid_for(CN, 256), 256, 0, st>>>(
                  CN, N, m2, radii, depths, ts, (uint32_t)tile_width, (uint32_t)tile_height,
                  w.cursor, w.keys, n_isects, &w.cw.hdr->status));
    ::ubs::note_launch();
    if (int e = check_launch("isect emit")) return e;
    const IdsWriter wr{isect_ids, flatten_ids, (int32_t)n_tiles, tile_bits};
    return launch_bucket_sort(nb, isect_offsets, nullptr, n_isects, w.keys, w.scratch, w.big_list,
                              &w.cw.hdr->n_big, wr, st);
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
    UBS_TIMED("offset_encode", st,
              offset_encode_kernel<<<grid_for(nb, 256), 256, 0, st>>>(
                  n_isects, isect_ids, nb, (int32_t)n_tiles, bit_width_u32((uint32_t)n_tiles),
                  offsets));
    ::ubs::note_launch();
    return check_launch("offset_encode");
}

} // extern "C"
