// raster_noalloc.cu -- forward blend that uses no caller workspace.
//
// ubs_raster_fwd stages one packed record per sorted intersection in a
// workspace the caller allocates.  Some callers cannot allocate device memory
// at the point where they render: a host callback or a real-time thread that
// must not enter the CUDA allocator (which can synchronise the device or
// block), or an embedding application whose memory pool is fixed and fully
// handed out.  ubs_raster_fwd_noalloc serves them: it runs the same pack and
// blend kernels as ubs_raster_fwd, on a scratch array that lives in this
// library's static device memory, and allocates nothing itself.
//
// Scratch: one static __device__ array per device, sized for
// UBS_RASTER_NOALLOC_MAX_ISECTS intersections (the layout ubs_raster_fwd uses
// in its workspace: a 256-byte status header, then 32-byte geometry records,
// then 16-byte colour records for up to 4 channels).  Its address on each
// device is looked up once with cudaGetSymbolAddress, on the first call made
// while that device is current; that first call therefore does set-up work
// and should come before any stream capture.  Nothing in the scratch has to
// start at zero: every call clears the status header on its stream before the
// pack kernel writes the records the blend reads.
//
// There is one scratch per device, so calls on the same device must not
// overlap: two calls in flight at once (different streams, or different host
// threads without ordering between them) race on the records.
//
// The looked-up address is kept for the life of the process.  cudaDeviceReset
// (or anything else that tears the device's primary context down) unloads the
// library's device code, and the array may come back elsewhere: a process
// that resets a device must not call the no-allocation entry points on it
// again.
//
// Device-side status (a flatten index outside [0, C*N), a bounded wait that
// ran out) lands in the scratch's header like it lands in a workspace's;
// ubs_raster_noalloc_status reads it back.
#include <atomic>
#include <mutex>

#include "ubs_common.cuh"

namespace ubs {
namespace {

constexpr int64_t kMaxIsects = UBS_RASTER_NOALLOC_MAX_ISECTS;
// header + geometry record (32 B) + packed colour record (16 B) per intersection
constexpr size_t kScratchBytes = 256 + (size_t)kMaxIsects * 48;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_raster_scratch[kScratchBytes];

std::atomic<void *> g_scratch_addr[kMaxDevices];
std::mutex g_setup_mu;

// Address of the scratch on the current device (set-up on the first call).
int scratch_for_current_device(void **out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) return check_launch("raster_fwd_noalloc device");
    if (dev < 0 || dev >= kMaxDevices)
        return set_error(UBS_ERR_UNSUPPORTED, "raster_fwd_noalloc: device ordinal %d >= %d", dev,
                         kMaxDevices);
    void *p = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lk(g_setup_mu);
        p = g_scratch_addr[dev].load(std::memory_order_relaxed);
        if (!p) {
            if (cudaGetSymbolAddress(&p, g_raster_scratch) != cudaSuccess || !p)
                return check_launch("raster_fwd_noalloc scratch address");
            g_scratch_addr[dev].store(p, std::memory_order_release);
        }
    }
    *out = p;
    return UBS_OK;
}

} // namespace
} // namespace ubs

using namespace ubs;

extern "C" {

int ubs_raster_fwd_noalloc(int32_t C, int64_t N, int32_t channels, int64_t n_isects,
                           const float *means2d, const float *conics, const float *colors,
                           const float *opacities, const float *betas, const float *backgrounds,
                           const uint8_t *masks, int32_t width, int32_t height, int32_t tile_size,
                           int32_t tile_width, int32_t tile_height, const int32_t *isect_offsets,
                           const int32_t *flatten_ids, float *render_colors, float *render_alphas,
                           int32_t *last_ids, void *stream) {
    if (n_isects > kMaxIsects)
        return set_error(UBS_ERR_OVERFLOW,
                         "raster_fwd_noalloc: %lld intersections exceed the fixed scratch limit "
                         "of %lld; use ubs_raster_fwd with a workspace",
                         (long long)n_isects, (long long)kMaxIsects);
    void *scratch = nullptr;
    if (int e = scratch_for_current_device(&scratch)) return e;
    return ubs_raster_fwd(C, N, channels, n_isects, means2d, conics, colors, opacities, betas,
                          backgrounds, masks, width, height, tile_size, tile_width, tile_height,
                          isect_offsets, flatten_ids, render_colors, render_alphas, last_ids,
                          scratch, kScratchBytes, stream);
}

int ubs_raster_noalloc_status(uint32_t *status, void *stream) {
    UBS_REQUIRE(status, "raster_noalloc_status: null pointer");
    void *scratch = nullptr;
    if (int e = scratch_for_current_device(&scratch)) return e;
    return ubs_raster_status(scratch, status, nullptr, stream);
}

} // extern "C"
