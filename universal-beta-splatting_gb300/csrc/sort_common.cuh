// sort_common.cuh -- device-wide exclusive scan and per-bucket key sort shared
// by the drop-in intersection operator (isect.cu) and the fused multi-view
// render path (scene.cu).
#pragma once

#include "ubs_common.cuh"

namespace ubs {

constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_TILE = SCAN_ITEMS * SCAN_THREADS;
constexpr int WARP_SEG = 1024;  // longest bucket sorted by one warp in registers
constexpr int SMALL_SEG = 4096; // longest bucket sorted by one CTA in shared memory
constexpr int SORT_THREADS = 256;
constexpr int BIG_THREADS = 1024;
constexpr int MERGE_ITEMS = 8;
constexpr int EMIT_ROUNDS = 4; // (entry, tile) rounds of 32 whose cursor atomics overlap

__host__ __device__ __forceinline__ int64_t imin64(int64_t a, int64_t b) { return a < b ? a : b; }

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

static __global__ void __launch_bounds__(SCAN_THREADS) scan_sums_kernel(int64_t *sums, int64_t nblocks,
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
inline int device_exclusive_scan(const int32_t *in, OutT *out, int64_t n, int64_t *sums,
                                 int64_t *total, cudaStream_t st) {
    if (n == 0) {
        if (cudaMemsetAsync(total, 0, 8, st) != cudaSuccess) return check_launch("scan memset");
        return UBS_OK;
    }
    const int64_t nblocks = (n + SCAN_TILE - 1) / SCAN_TILE;
    UBS_TIMED("scan", st,
              scan_blocks_kernel<OutT><<<(unsigned)nblocks, SCAN_THREADS, 0, st>>>(in, out, n,
                                                                                  sums);
              scan_sums_kernel<<<1, SCAN_THREADS, 0, st>>>(sums, nblocks, total);
              if (nblocks > 1) scan_add_kernel<OutT><<<grid_for(n, 256), 256, 0, st>>>(out, n,
                                                                                       sums));
    ::ubs::note_launch(nblocks > 1 ? 3 : 2);
    return check_launch("exclusive scan");
}


// ------------------------------------------------------------ bucket sort
// Buckets hold unique 64-bit keys (depth bits << 32 | flatten index), so any
// correct sort yields the reference's stable order.  Writer::operator()(key,
// sorted position, bucket) stores one sorted entry.  The intersection count
// is read on the device when T_dev is given (clamped to the key capacity
// cap), else it is cap, so no host round trip is needed.

// In-place bitonic sort of s[0..n2) (n2 a power of two) by the whole CTA.
__device__ __forceinline__ void block_bitonic(uint64_t *s, int n2) {
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

__device__ __forceinline__ void bucket_range(const int32_t *offsets, int64_t bkt, int64_t n_buckets,
                                             int64_t T, int64_t &lo, int64_t &hi) {
    lo = imin64(offsets[bkt], T);
    hi = (bkt + 1 < n_buckets) ? imin64(offsets[bkt + 1], T) : T;
    if (hi < lo) hi = lo;
}

// Warp-flattened emission of sort keys: every lane holds the tile rectangle
// of one (view, primitive) entry -- n tiles, bw columns, row pitch `pitch`,
// cursor of its first tile `cur` -- and the warp walks the concatenation of
// the 32 rectangles 32 (entry, tile) pairs per round, so its rounds follow the
// warp's total tile count rather than its largest entry and the cursor
// atomics of a round are independent.  Each pair takes the next slot of its
// tile's cursor and stores the entry's key there (slots past `cap` set the
// overflow bit instead).
__device__ __forceinline__ void warp_emit_rects(uint32_t n, uint32_t bw, uint32_t pitch,
                                                int32_t *cur, uint64_t key, int lane,
                                                uint64_t *__restrict__ keys, int64_t cap,
                                                uint32_t *status) {
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    // pair j of the flattened list: the cursor of its tile and its entry's key
    auto locate = [&](uint32_t j, int32_t *&slot, uint64_t &k) {
        int owner = 0; // first lane whose inclusive count exceeds j
#pragma unroll
        for (int step = 16; step > 0; step >>= 1) {
            const uint32_t c = __shfl_sync(0xffffffffu, incl, owner + step - 1);
            if (c <= j) owner += step;
        }
        const uint32_t o_incl = __shfl_sync(0xffffffffu, incl, owner);
        const uint32_t o_n = __shfl_sync(0xffffffffu, n, owner);
        const uint32_t o_bw = __shfl_sync(0xffffffffu, bw, owner);
        const uint32_t o_pitch = __shfl_sync(0xffffffffu, pitch, owner);
        k = __shfl_sync(0xffffffffu, key, owner);
        int32_t *o_cur = reinterpret_cast<int32_t *>(
            __shfl_sync(0xffffffffu, reinterpret_cast<uintptr_t>(cur), owner));
        const uint32_t local = j - (o_incl - o_n);
        const uint32_t ry = local / o_bw, rx = local - ry * o_bw;
        slot = o_cur + (int64_t)ry * o_pitch + rx;
    };
    // EMIT_ROUNDS rounds per iteration: all their cursor atomics are in
    // flight before any of them stores its key
    for (uint32_t base = 0; base < total; base += 32 * EMIT_ROUNDS) {
        int32_t *sl[EMIT_ROUNDS];
        uint64_t kk[EMIT_ROUNDS];
        int32_t pos[EMIT_ROUNDS];
#pragma unroll
        for (int r = 0; r < EMIT_ROUNDS; ++r)
            if (base + 32 * r < total) locate(base + 32 * r + lane, sl[r], kk[r]); // uniform
#pragma unroll
        for (int r = 0; r < EMIT_ROUNDS; ++r)
            pos[r] = base + 32 * r + lane < total ? atomicAdd(sl[r], 1) : -1;
#pragma unroll
        for (int r = 0; r < EMIT_ROUNDS; ++r) {
            if (base + 32 * r + lane < total) {
                if (pos[r] >= 0 && pos[r] < cap) keys[pos[r]] = kk[r];
                else atomicOr(status, DEV_ERR_OVERFLOW);
            }
        }
    }
}

// Heaviest-first order of the buckets for the blend (longest-processing-time
// scheduling): one CTA counting-sorts the buckets by record count into
// ORDER_BINS bins of 4 records (descending; counts >= 4 * ORDER_BINS share the
// first bin).  Order within a bin is arbitrary, which only changes the launch
// order of the blend's CTAs, never a result.
constexpr int ORDER_BINS = 1024;
static __global__ void __launch_bounds__(1024) bucket_order_kernel(const int32_t *__restrict__ offsets,
                                                            const int64_t *T_dev, int64_t cap,
                                                            int32_t n_buckets,
                                                            int32_t *__restrict__ order) {
    __shared__ int32_t bins[ORDER_BINS];
    __shared__ int32_t warp_tot[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int64_t T = T_dev ? imin64(*T_dev, cap) : cap;
    for (int i = tid; i < ORDER_BINS; i += blockDim.x) bins[i] = 0;
    __syncthreads();
    auto bin_of = [&](int32_t b) {
        int64_t lo, hi;
        bucket_range(offsets, b, n_buckets, T, lo, hi);
        const int64_t c = (hi - lo) >> 2;
        return ORDER_BINS - 1 - (int)(c < ORDER_BINS - 1 ? c : ORDER_BINS - 1);
    };
    for (int32_t b = tid; b < n_buckets; b += blockDim.x) atomicAdd(&bins[bin_of(b)], 1);
    __syncthreads();
    // exclusive scan of the 1024 bins (one per thread)
    const int v = tid < ORDER_BINS ? bins[tid] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = warp_tot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t; // inclusive
    }
    __syncthreads();
    if (tid < ORDER_BINS) bins[tid] = x - v + (wid ? warp_tot[wid - 1] : 0);
    __syncthreads();
    for (int32_t b = tid; b < n_buckets; b += blockDim.x) order[atomicAdd(&bins[bin_of(b)], 1)] = b;
}

// Both per-bucket passes of a frame whose buckets fit one CTA (n <=
// SCAN_ORDER_MAX), in one launch: the exclusive scan of the bucket counts
// (bucket offsets, int32, and the intersection total) and the heaviest-first
// bucket order of bucket_order_kernel (a counting sort by record count).
// Each of the 1024 threads scans a contiguous run of buckets.
constexpr int SCAN_ORDER_MAX = 1024 * 64;
// The counts come in R replicas ([R][n], replica-major: the atomics of a
// bucket spread over R lines).  First the CTA folds them into totals[b] (the
// bucket's count) with consecutive threads on consecutive buckets; the scan
// and the order work on the totals; last, cursor[r n + b] receives the start
// of replica r's sub-range of bucket b (its bucket offset plus the counts of
// replicas 0 .. r - 1), again on consecutive buckets.
template <int R>
__global__ void __launch_bounds__(1024) bucket_scan_order_kernel(
    const int32_t *__restrict__ counts, int32_t n, int32_t *__restrict__ offsets,
    int64_t *__restrict__ total, int32_t *__restrict__ order, int32_t *__restrict__ cursor,
    int32_t *__restrict__ totals) {
    __shared__ int32_t bins[ORDER_BINS];
    __shared__ int64_t wtot[32];
    __shared__ int32_t btot[32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int per = (n + 1023) / 1024;
    const int b0 = min(n, tid * per), b1 = min(n, b0 + per);
    for (int i = tid; i < ORDER_BINS; i += blockDim.x) bins[i] = 0;
    for (int b = tid; b < n; b += blockDim.x) {
        int32_t c = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) c += counts[(int64_t)r * n + b];
        totals[b] = c;
    }
    __syncthreads();
    auto count = [&](int b) { return totals[b]; };
    int64_t run = 0;
    for (int b = b0; b < b1; ++b) {
        const int32_t c = count(b);
        run += c;
        const int64_t q = c >> 2;
        atomicAdd(&bins[ORDER_BINS - 1 - (int)(q < ORDER_BINS - 1 ? q : ORDER_BINS - 1)], 1);
    }
    int64_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) wtot[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        const int64_t w = wtot[lane];
        int64_t wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += y;
        }
        wtot[lane] = wi - w; // exclusive
    }
    __syncthreads();
    int64_t off = wtot[wid] + inc - run;
    for (int b = b0; b < b1; ++b) {
        offsets[b] = (int32_t)off;
        off += count(b);
    }
    if (tid == blockDim.x - 1) *total = off;
    // heaviest-first order: exclusive scan of the bins, then a scatter
    const int v = bins[tid];
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) btot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = btot[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        btot[lane] = t; // inclusive
    }
    __syncthreads();
    bins[tid] = x - v + (wid ? btot[wid - 1] : 0);
    __syncthreads();
    for (int b = b0; b < b1; ++b) {
        const int64_t q = count(b) >> 2;
        order[atomicAdd(&bins[ORDER_BINS - 1 - (int)(q < ORDER_BINS - 1 ? q : ORDER_BINS - 1)],
                        1)] = b;
    }
    for (int b = tid; b < n; b += blockDim.x) { // offsets written above by this CTA
        int32_t o = offsets[b];
#pragma unroll
        for (int r = 0; r < R; ++r) {
            cursor[(int64_t)r * n + b] = o;
            o += counts[(int64_t)r * n + b];
        }
    }
}

// Larger frames (more buckets than one CTA scans): the replicas' sums ...
template <int R>
__global__ void fold_replicas_kernel(const int32_t *__restrict__ counts, int32_t n,
                                     int32_t *__restrict__ totals) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int32_t c = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) c += counts[(int64_t)r * n + b];
    totals[b] = c;
}
// ... and, after their exclusive scan, the replicas' cursors.
template <int R>
__global__ void replica_cursors_kernel(const int32_t *__restrict__ counts, int32_t n,
                                       const int32_t *__restrict__ offsets,
                                       int32_t *__restrict__ cursor) {
    const int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= n) return;
    int32_t off = offsets[b];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        cursor[(int64_t)r * n + b] = off;
        off += counts[(int64_t)r * n + b];
    }
}

// Bitonic sort of the 32 * E keys of a warp held E per lane in registers,
// blocked (element i = lane * E + e): exchange distances below E stay inside
// a lane, larger ones are lane-xor shuffles.  The network runs in two phases
// so that no compare-exchange recomputes its direction:
//   * stages k < E sort runs inside a lane: distances and directions are
//     compile-time (element e of a run of k ascends when e & k == 0);
//   * stages k >= E: the direction of all E elements of a lane is the same,
//     ((lane * E) & k) == 0, one predicate per stage; the stage loop runs at
//     run time with one unrolled body per in-lane distance, which keeps the
//     code small enough for the instruction cache.
// The network is the same as the textbook bitonic sort, so the result is.
template <int E, int J, int K>
__device__ __forceinline__ void bitonic_run_pass(uint64_t (&v)[E]) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int p = e ^ J;
        if (p > e) {
            const uint64_t a = v[e], b = v[p];
            const bool sw = ((e & K) == 0) ? (a > b) : (a < b);
            v[e] = sw ? b : a;
            v[p] = sw ? a : b;
        }
    }
}
template <int E, int K, int J> struct BitonicRunStage {
    static __device__ __forceinline__ void run(uint64_t (&v)[E]) {
        bitonic_run_pass<E, J, K>(v);
        BitonicRunStage<E, K, J / 2>::run(v);
    }
};
template <int E, int K> struct BitonicRunStage<E, K, 0> {
    static __device__ __forceinline__ void run(uint64_t (&)[E]) {}
};
template <int E, int K> struct BitonicRuns { // stages K, 2K, .. < E
    static __device__ __forceinline__ void run(uint64_t (&v)[E]) {
        BitonicRunStage<E, K, K / 2>::run(v);
        BitonicRuns<E, (2 * K < E ? 2 * K : 0)>::run(v);
    }
};
template <int E> struct BitonicRuns<E, 0> {
    static __device__ __forceinline__ void run(uint64_t (&)[E]) {}
};

// One in-lane pass of distance J with the lane's direction `up`.
template <int E, int J>
__device__ __forceinline__ void bitonic_in_lane(uint64_t (&v)[E], bool up) {
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int p = e ^ J;
        if (p > e) {
            const uint64_t a = v[e], b = v[p];
            const bool sw = (a > b) == up;
            v[e] = sw ? b : a;
            v[p] = sw ? a : b;
        }
    }
}

template <int E>
__device__ __forceinline__ void warp_bitonic(uint64_t (&v)[E], int lane) {
    constexpr int N = 32 * E;
    BitonicRuns<E, (E >= 4 ? 2 : 0)>::run(v); // k = 2 .. E / 2 inside the lane
#pragma unroll 1
    for (int k = E >= 2 ? E : 2; k <= N; k <<= 1) {
        const bool up = ((lane * E) & k) == 0;
#pragma unroll 1
        for (int j = k >> 1; j >= E; j >>= 1) { // across lanes
            const int lj = j / E;
            const bool keep_min = ((lane & lj) == 0) == up;
#pragma unroll
            for (int e = 0; e < E; ++e) {
                const uint64_t o = __shfl_xor_sync(0xffffffffu, v[e], lj);
                v[e] = (keep_min == (o < v[e])) ? o : v[e];
            }
        }
        // inside a lane: distances E / 2 .. 1
        if (E >= 32) bitonic_in_lane<E, (E >= 32 ? 16 : 1)>(v, up);
        if (E >= 16) bitonic_in_lane<E, (E >= 16 ? 8 : 1)>(v, up);
        if (E >= 8) bitonic_in_lane<E, (E >= 8 ? 4 : 1)>(v, up);
        if (E >= 4) bitonic_in_lane<E, (E >= 4 ? 2 : 1)>(v, up);
        if (E >= 2) bitonic_in_lane<E, 1>(v, up);
    }
}

template <int E, typename Writer>
__device__ __forceinline__ void warp_sort_bucket(const uint64_t *__restrict__ keys, int64_t lo,
                                                 int n, int64_t bkt, int lane, const Writer &w) {
    uint64_t v[E];
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = lane * E + e;
        v[e] = i < n ? keys[lo + i] : ~0ull;
    }
    warp_bitonic<E>(v, lane);
#pragma unroll
    for (int e = 0; e < E; ++e) {
        const int i = lane * E + e;
        if (i < n) w(v[e], lo + i, bkt);
    }
}

// One warp per bucket for buckets of at most WARP_SEG keys (padded to the
// next power of two >= 32 with all-ones keys, which sort last); longer
// buckets go to the device-side lists: mid (<= SMALL_SEG) from the front of
// `lists`, big from the back.  counters = {n_big, n_mid}.
template <typename Writer>
__global__ void __launch_bounds__(256, 3) bucket_sort_warp_kernel(
    int64_t n_buckets, const int32_t *__restrict__ offsets, const int64_t *T_dev, int64_t cap,
    const uint64_t *__restrict__ keys, int32_t *lists, int32_t *counters, Writer w) {
    const int lane = threadIdx.x & 31;
    const int64_t bkt = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (bkt >= n_buckets) return;
    const int64_t T = T_dev ? imin64(*T_dev, cap) : cap;
    int64_t lo, hi;
    bucket_range(offsets, bkt, n_buckets, T, lo, hi);
    const int64_t n = hi - lo;
    if (n <= 0) return;
    if (n > WARP_SEG) {
        if (lane == 0) {
            if (n > SMALL_SEG) lists[n_buckets - 1 - atomicAdd(&counters[0], 1)] = (int32_t)bkt;
            else lists[atomicAdd(&counters[1], 1)] = (int32_t)bkt;
        }
        return;
    }
    const int m = (int)n;
    if (m <= 32) warp_sort_bucket<1>(keys, lo, m, bkt, lane, w);
    else if (m <= 64) warp_sort_bucket<2>(keys, lo, m, bkt, lane, w);
    else if (m <= 128) warp_sort_bucket<4>(keys, lo, m, bkt, lane, w);
    else if (m <= 256) warp_sort_bucket<8>(keys, lo, m, bkt, lane, w);
    else if (m <= 512) warp_sort_bucket<16>(keys, lo, m, bkt, lane, w);
    else warp_sort_bucket<32>(keys, lo, m, bkt, lane, w);
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

// Buckets of WARP_SEG < n <= SMALL_SEG keys (the mid list): a fixed grid walks
// the device-side list with one CTA of MID_WARPS warps per bucket.  Warp c
// sorts keys [c WARP_SEG, (c + 1) WARP_SEG) in registers (warp_bitonic, 32 per
// lane), the sorted runs are merged pairwise in shared memory by merge path,
// and the last merge hands the sorted keys to the writer: two barriers per
// merge level instead of one per bitonic stage (78 for 4096 keys).
constexpr int MID_WARPS = SMALL_SEG / WARP_SEG;
constexpr size_t MID_SMEM = 2 * SMALL_SEG * sizeof(uint64_t);
template <typename Writer>
__global__ void __launch_bounds__(MID_WARPS * 32, 3) bucket_sort_mid_kernel(
    int64_t n_buckets, const int32_t *__restrict__ offsets, const int64_t *T_dev, int64_t cap,
    const uint64_t *__restrict__ keys, const int32_t *lists, const int32_t *counters, Writer w) {
    extern __shared__ __align__(16) uint64_t mid_runs[]; // two buffers of SMALL_SEG
    const int n_mid = counters[1];
    const int64_t T = T_dev ? imin64(*T_dev, cap) : cap;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (int item = blockIdx.x; item < n_mid; item += gridDim.x) {
        __syncthreads();
        const int64_t bkt = lists[item];
        int64_t lo, hi;
        bucket_range(offsets, bkt, n_buckets, T, lo, hi);
        const int n = (int)(hi - lo);
        const int c0 = warp * WARP_SEG;
        if (c0 < n) {
            uint64_t v[32];
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                const int i = c0 + lane * 32 + e;
                v[e] = i < n ? keys[lo + i] : ~0ull;
            }
            warp_bitonic<32>(v, lane);
#pragma unroll
            for (int e = 0; e < 32; ++e) { // the padding keys sort last: only real keys
                const int i = c0 + lane * 32 + e;
                if (i < n) mid_runs[i] = v[e];
            }
        }
        __syncthreads();
        uint64_t *src = mid_runs, *dst = mid_runs + SMALL_SEG;
        for (int width = WARP_SEG; width < n; width <<= 1) {
            const bool last = 2 * width >= n;
            for (int r0 = 0; r0 < n; r0 += 2 * width) {
                const int na = min(width, n - r0), nb = min(width, n - r0 - na);
                const uint64_t *A = src + r0, *Bv = src + r0 + na;
                const int total = na + nb;
                for (int o0 = threadIdx.x * MERGE_ITEMS; o0 < total;
                     o0 += blockDim.x * MERGE_ITEMS) {
                    int ia = (int)merge_split(A, na, Bv, nb, o0);
                    int ib = o0 - ia;
                    const int oend = min(total, o0 + MERGE_ITEMS);
                    for (int o = o0; o < oend; ++o) {
                        const bool take_a = ib >= nb || (ia < na && A[ia] < Bv[ib]);
                        const uint64_t key = take_a ? A[ia++] : Bv[ib++];
                        if (last) w(key, lo + r0 + o, bkt);
                        else dst[r0 + o] = key;
                    }
                }
            }
            __syncthreads();
            uint64_t *t = src;
            src = dst;
            dst = t;
        }
    }
}

// Long buckets (their number is known only on the device): a fixed grid walks
// the device-side list; each CTA sorts SMALL_SEG chunks in shared memory, then
// merges runs pairwise in global memory (keys <-> scratch).
template <typename Writer>
__global__ void __launch_bounds__(BIG_THREADS) bucket_sort_big_kernel(
    int64_t n_buckets, const int32_t *__restrict__ offsets, const int64_t *T_dev, int64_t cap,
    uint64_t *keys, uint64_t *scratch, const int32_t *lists, const int32_t *counters, Writer w) {
    __shared__ uint64_t s[SMALL_SEG];
    const int n_big = counters[0];
    const int64_t T = T_dev ? imin64(*T_dev, cap) : cap;
    for (int item = blockIdx.x; item < n_big; item += gridDim.x) {
        __syncthreads();
        const int64_t bkt = lists[n_buckets - 1 - item];
        int64_t lo, hi;
        bucket_range(offsets, bkt, n_buckets, T, lo, hi);
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
        for (int64_t i = threadIdx.x; i < n; i += blockDim.x) w(src[i], lo + i, bkt);
    }
}

// Launches the per-bucket sort: buckets of <= WARP_SEG keys one warp each in
// registers, <= SMALL_SEG one CTA each in shared memory, longer ones merged on
// a fixed grid.  lists ([n_buckets]) and counters ([2], zeroed here) are
// scratch.
template <typename Writer>
inline int launch_bucket_sort(int64_t n_buckets, const int32_t *offsets, const int64_t *T_dev,
                              int64_t cap, uint64_t *keys, uint64_t *scratch, int32_t *lists,
                              int32_t *counters, Writer w, cudaStream_t st) {
    if (n_buckets <= 0 || cap <= 0) return UBS_OK;
    if (cudaMemsetAsync(counters, 0, 8, st) != cudaSuccess) return check_launch("sort memset");
    UBS_TIMED("bucket_sort_warp", st,
              bucket_sort_warp_kernel<Writer><<<grid_for(n_buckets, 8), 256, 0, st>>>(
                  n_buckets, offsets, T_dev, cap, keys, lists, counters, w));
    note_launch();
    if (cap > WARP_SEG) {
        const int64_t max_mid = cap / (WARP_SEG + 1);
        const unsigned grid = (unsigned)imin64(imin64(max_mid, n_buckets), 152 * 6);
        if (cudaFuncSetAttribute(bucket_sort_mid_kernel<Writer>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)MID_SMEM) != cudaSuccess)
            return check_launch("bucket_sort_mid attribute");
        UBS_TIMED("bucket_sort_mid", st,
                  bucket_sort_mid_kernel<Writer><<<grid, MID_WARPS * 32, MID_SMEM, st>>>(
                      n_buckets, offsets, T_dev, cap, keys, lists, counters, w));
        note_launch();
    }
    if (cap > SMALL_SEG) {
        const int64_t max_big = cap / (SMALL_SEG + 1);
        const unsigned grid = (unsigned)imin64(imin64(max_big, n_buckets), 304);
        if (grid > 0) {
            UBS_TIMED("bucket_sort_big", st,
                      bucket_sort_big_kernel<Writer><<<grid, BIG_THREADS, 0, st>>>(
                          n_buckets, offsets, T_dev, cap, keys, scratch, lists, counters, w));
            note_launch();
        }
    }
    return check_launch("bucket sort");
}

} // namespace ubs
