// noalloc.cu - the reference-compatible curl generator without any device allocation.
//
// mm_noise_fill(MM_NOISE_REF_CURL) needs scratch for the 128x128 curl vectors and their per-channel
// min/max before it can normalise them to 8 bits (ImageUtils.cpp:179-219), and allocates it on the
// stream for every call.  Some callers cannot allocate device memory at that point: a render
// engine or plugin host that reserves the whole device heap up front and hands out only its own
// buffers, or a frame loop that must not risk the allocator's synchronisation.  This entry point uses a fixed scratch array compiled into the
// library instead.  The array lives in every GPU that loads the library until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "mm_internal.h"

namespace {

constexpr int kMaxSide = 128;                                    // the reference's CURL_DIM
constexpr size_t kCurlFloats = (size_t)kMaxSide * kMaxSide * 3;  // curl vectors
constexpr size_t kScratchFloats = kCurlFloats + 8;               // + 6 bounds, padded

// Shared by every call on a device; it keeps the last call's contents.
static __device__ __align__(256) float g_ref_curl_scratch[kScratchFloats];

constexpr int kMaxDevices = 64;
std::mutex g_mutex;
float* g_scratch_ptr[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once per device and kept
// for the life of the process.  A device reset (cudaDeviceReset) after the first call reloads the
// module and may move the array; calling this entry point after such a reset is not supported.
int scratch_for_current_device(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return mm::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= kMaxDevices) return mm::fail(MM_ERR_UNSUPPORTED, "noalloc: device index %d too large", dev);
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_ptr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_ref_curl_scratch);
        if (e != cudaSuccess) return mm::cuda_fail(e, "cudaGetSymbolAddress(ref curl scratch)");
        g_scratch_ptr[dev] = static_cast<float*>(ptr);
    }
    *out = g_scratch_ptr[dev];
    return MM_OK;
}

}  // namespace

extern "C" int mm_noise_fill_ref_curl_noalloc(int width, int height, void* d_texels, size_t bytes, void* stream) {
    using mm::fail;
    if (width == 0) width = kMaxSide;
    if (height == 0) height = kMaxSide;
    if (width > kMaxSide || height > kMaxSide)
        return fail(MM_ERR_INVALID_ARGUMENT,
                    "noalloc ref curl: %dx%d exceeds the %dx%d maximum of the library's static scratch", width, height,
                    kMaxSide, kMaxSide);
    if (width != kMaxSide || height != kMaxSide)
        return fail(MM_ERR_INVALID_ARGUMENT, "noalloc ref curl: the reference curl is %dx%d only", kMaxSide, kMaxSide);
    if (!d_texels) return fail(MM_ERR_INVALID_ARGUMENT, "noalloc ref curl: null output");
    const size_t need = (size_t)width * height * 4;
    if (bytes < need) return fail(MM_ERR_INVALID_ARGUMENT, "noalloc ref curl: output smaller than %zu bytes", need);
    float* scratch = nullptr;
    int r = scratch_for_current_device(&scratch);
    if (r) return r;
    // Nothing in the scratch has to start at zero: the curl kernel overwrites every vector and the
    // normalise kernel recomputes the bounds before it reads them.
    return mm::launch_ref_curl(static_cast<uint8_t*>(d_texels), scratch, scratch + kCurlFloats, (cudaStream_t)stream);
}
