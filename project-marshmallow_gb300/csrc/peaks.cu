// peaks.cu - microbenchmarks of the two on-chip limits the cloud march runs against: the
// texture unit's filtered-fetch rate (trilinear 3D and bilinear 2D, RGBA8 texels that stay in
// L1/TEX) and the FP32 FMA rate.  HBM is not the march's bound: its textures (~9 MB) live in L2.
#include <cuda_runtime.h>
#include <string.h>

#include "mm_internal.h"

namespace mm {
namespace peaks {

constexpr int kFetches = 2048;

// Each thread walks its own coordinate sequence with a fixed stride; the sum keeps every fetch live.
__global__ void __launch_bounds__(256) tex3d_rate(cudaTextureObject_t t, float* sink, float step) {
    float u = (blockIdx.x * 256 + threadIdx.x) * (0.25f / 128.0f), v = blockIdx.x * 0.0071f, w = blockIdx.x * 0.0031f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
    for (int i = 0; i < kFetches; ++i) {
        float4 r = tex3D<float4>(t, u, v, w);
        acc.x += r.x;
        acc.y += r.y;
        acc.z += r.z;
        acc.w += r.w;
        u += step;
        v += 0.37f * step;
        w += 0.11f * step;
    }
    if (acc.x + acc.y + acc.z + acc.w == -1.0f) sink[0] = acc.x;
}

__global__ void __launch_bounds__(256) tex2d_rate(cudaTextureObject_t t, float* sink, float step) {
    float u = (blockIdx.x * 256 + threadIdx.x) * (0.25f / 512.0f), v = blockIdx.x * 0.0071f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
    for (int i = 0; i < kFetches; ++i) {
        float4 r = tex2D<float4>(t, u, v);
        acc.x += r.x;
        acc.y += r.y;
        acc.z += r.z;
        acc.w += r.w;
        u += step;
        v += 0.37f * step;
    }
    if (acc.x + acc.y + acc.z + acc.w == -1.0f) sink[0] = acc.x;
}

constexpr int kFmaIters = 16384;

__global__ void __launch_bounds__(256) fma_rate(float* sink, float a) {
    float x0 = threadIdx.x, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f, x4 = x0 + 4.f, x5 = x0 + 5.f,
          x6 = x0 + 6.f, x7 = x0 + 7.f;
#pragma unroll 16
    for (int i = 0; i < kFmaIters; ++i) {
        x0 = fmaf(x0, a, 0.5f);
        x1 = fmaf(x1, a, 0.5f);
        x2 = fmaf(x2, a, 0.5f);
        x3 = fmaf(x3, a, 0.5f);
        x4 = fmaf(x4, a, 0.5f);
        x5 = fmaf(x5, a, 0.5f);
        x6 = fmaf(x6, a, 0.5f);
        x7 = fmaf(x7, a, 0.5f);
    }
    float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == -1.0f) sink[0] = s;
}

}  // namespace peaks
}  // namespace mm

extern "C" int mm_measure_peaks(mm_texture tex3d, mm_texture tex2d, double* out, void* stream) {
    using namespace mm;
    if (!tex3d || !tex2d || !out) return fail(MM_ERR_INVALID_ARGUMENT, "peaks: null argument");
    if (!tex3d->tex || !tex2d->tex || tex3d->channels != 4 || tex2d->channels != 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "peaks: textures must be RGBA with texture objects");
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    MM_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    float* sink = nullptr;
    MM_CUDA_TRY(cudaMallocAsync((void**)&sink, 16, s));
    cudaEvent_t e0, e1;
    MM_CUDA_TRY(cudaEventCreate(&e0));
    MM_CUDA_TRY(cudaEventCreate(&e1));
    const int blocks = sms * 8;
    const double threads = (double)blocks * 256;
    float ms = 0.f;
    double res[3] = {0, 0, 0};
    for (int which = 0; which < 3; ++which) {
        for (int rep = 0; rep < 2; ++rep) {  // first launch warms up
            cudaEventRecord(e0, s);
            if (which == 0)
                peaks::tex3d_rate<<<blocks, 256, 0, s>>>(tex3d->tex, sink, 1.0f / 128.0f);
            else if (which == 1)
                peaks::tex2d_rate<<<blocks, 256, 0, s>>>(tex2d->tex, sink, 1.0f / 512.0f);
            else
                peaks::fma_rate<<<blocks, 256, 0, s>>>(sink, 0.999f);
            cudaEventRecord(e1, s);
            count_launch();
        }
        MM_CUDA_TRY(cudaEventSynchronize(e1));
        MM_CUDA_TRY(cudaEventElapsedTime(&ms, e0, e1));
        const double work = which < 2 ? threads * peaks::kFetches : threads * peaks::kFmaIters * 8.0 * 2.0;
        res[which] = work / (ms * 1e-3);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFreeAsync(sink, s);
    out[0] = res[0] * 1e-9;   // trilinear 3D fetches, G/s
    out[1] = res[1] * 1e-9;   // bilinear 2D fetches, G/s
    out[2] = res[2] * 1e-12;  // FP32 FMA, TFLOP/s
    return MM_OK;
}
