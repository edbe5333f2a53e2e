// shadow_kernel.cuh - the cloud-shadow march of the mesh pass (model.frag:52-162, 221-222, 240-276) as CUDA
// device code over a G-buffer of world positions.
//
// One thread per G-buffer pixel: the sun ray from the fragment meets the inner atmosphere sphere
// (the start parameter t, with the march's isect.t quirk, :158), then up to six low-res density
// samples march from 4 * fragPositionWC along L, the sun direction in view space (:221-222, :257),
// 1 km apart (:253); the shadow is the largest density met, 1 once above 0.99 (:269-274).  The
// density model has the mesh shader's own constants (radius 1e6, weather scale 1e-5, low-res
// scale 5.7e-5, wind 20 (wind + (0, 0.2 rh, 0)) (t + 200 rh)) and its cloudLayerDensity, whose
// second blend goes to stratus, not cumulus (:95).  Where the sun ray misses the inner sphere the
// shader leaves t unset; t = 0 is used (as in the CPU restatement).
//
// Template parameters as for the march (march_kernel.cuh): kExact selects the shader's arithmetic
// (bit-identical to the FP32 oracle with the software sampler, in a -fmad=false translation unit)
// or the fast forms; kSampler the software or the hardware (texture unit) sampler.
#ifndef MM_SHADOW_KERNEL_CUH_
#define MM_SHADOW_KERNEL_CUH_

#include "march_kernel.cuh"

namespace mm {

struct ShadowLaunch {
    mm_uniforms u;
    TexView weather, low;
    const float4* pos;
    size_t pos_pitch;  // bytes
    float* shadow;     // may be null
    size_t shadow_pitch;
    float4* rgba;      // may be null: lit mesh colour darkened in place (model.frag:283-284)
    size_t rgba_pitch;
    int width, height;
    float coverage_offset;
};

namespace shadow {

using march::F4;
using march::M;
using march::V3;
using march::clampf;
using march::mixf;

constexpr float kRadius = 1000000.0f;  // ATMOSPHERE_RADIUS (model.frag:61)
constexpr int kSteps = 6;              // NUM_SHADOW_STEPS (:62)

template <bool E>
__device__ __forceinline__ float layerDensity(float rh, float type) {  // :87-97
    rh = clampf(rh, 0.0f, 1.0f);
    const float ramp = march::remap<E>(rh, 0.0f, 0.2f, 0.0f, 1.0f);
    float stratocumulus = fmaxf(0.0f, ramp * march::remap<E>(rh, 0.2f, 0.7f, 1.0f, 0.0f));
    float stratus = fmaxf(0.0f, march::remap<E>(rh, 0.0f, 0.1f, 0.0f, 1.0f) * march::remap<E>(rh, 0.2f, 0.3f, 1.0f, 0.0f));
    float d1 = mixf(stratus, stratocumulus, clampf(type * 2.0f, 0.0f, 1.0f));
    float d2 = mixf(stratocumulus, stratus, clampf((type - 0.5f) * 2.0f, 0.0f, 1.0f));
    return mixf(d1, d2, type);
}

template <bool E>
__device__ __forceinline__ float sphereT(V3 ro, V3 rd, V3 c, float w) {  // :132-162 (.t)
    ro = ro - c;
    ro = {M<E>::div(ro.x, w), M<E>::div(ro.y, w), M<E>::div(ro.z, w)};
    const float A = march::dot(rd, rd);
    const float B = 2.0f * march::dot(rd, ro);
    const float C = march::dot(ro, ro) - 0.25f;
    const float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return 0.0f;
    float t = M<E>::div(-M<E>::sqrt(disc) - B, A) * 0.5f;
    if (t < 0.0f) t = M<E>::div(M<E>::sqrt(disc) - B, A) * 0.5f;
    if (!(t >= 0.0f)) return 0.0f;
    V3 p = ro + rd * t;
    p = p * w;
    p = p + c;
    return march::length<E>(p - ro);
}

template <bool E, int S>
__device__ __forceinline__ float cloudTest(const ShadowLaunch& p, V3 center, V3 cam, V3 pos, float rh) {  // :104-129
    float u, v;
    if (E) {
        const V3 proj = (0.5f * kRadius) * march::normalize<E>(pos - center) + center;
        u = 0.00001f * (proj.x - cam.x);
        v = 0.00001f * (proj.z - cam.z);
    } else {
        // proj.xz - camera.xz = R * d.xz / |d| (the centre shares the camera's x and z, :244-245)
        const V3 d = pos - center;
        const float k = 5.0f * rsqrtf(march::dot(d, d));
        u = d.x * k;
        v = d.z * k;
    }
    const F4 info = march::sample2d<E, S>(p.weather, u, v);
    const float layer = layerDensity<E>(rh, info.z);
    const F4 n = march::sample3d<E, S>(p.low, 0.000057f * pos);
    float density = layer * march::remapClamped<E>(n.x, 0.3f, 1.0f, 0.0f, 1.0f);
    // The production path evaluates the tail for every sample and turns the early return (:118)
    // into a select, as the march does (a divergent branch costs more than the arithmetic).
    if (E && density < 0.0001f) return 0.0f;
    // heightBiasCoverage(relativeHeight, min(0.85, weather.r)), arguments swapped as in the shader (:120)
    const float h = fminf(0.85f, info.x + p.coverage_offset);
    const float coverage = M<E>::pow(rh, clampf(march::remap<E>(h, 0.7f, 0.8f, 1.0f, 0.6f), 0.6f, 1.0f));
    float erosion = (0.625f * n.y + 0.25f * n.z) + 0.125f * n.w;
    erosion = march::remapClamped<E>(erosion, coverage, 1.0f, 0.0f, 1.0f);
    const float out = march::remapClamped<E>(density, erosion, 1.0f, 0.0f, 1.0f);
    return density < 0.0001f ? 0.0f : out;
}

template <bool E, int S>
__global__ void __launch_bounds__(256) shadow_kernel(ShadowLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    const float4 wc4 = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(p.pos) + (size_t)y * p.pos_pitch) + x);
    float accum = 0.0f;
    if (wc4.w != 0.0f) {
        const mm_uniforms& u = p.u;
        const float* vm = u.camera.view;
        const V3 db1 = march::ld3(u.sun.direction_basis + 4);
        V3 L = march::normalize<E>(V3{(vm[0] * db1.x + vm[4] * db1.y) + vm[8] * db1.z,
                                      (vm[1] * db1.x + vm[5] * db1.y) + vm[9] * db1.z,
                                      (vm[2] * db1.x + vm[6] * db1.y) + vm[10] * db1.z});
        if (L.y < -0.05f) L = L * -1.0f;
        const V3 cam = march::ld3(u.camera.camera_position);
        V3 center = cam;
        center.y = -kRadius * 0.5f * 0.99f;
        const float thickness = 0.5f * kRadius * 0.02f;
        const float step = 0.1f * thickness;
        const V3 wind = march::ld3(u.sky.wind);
        const float time = u.sky.wind[3];
        const V3 wc = {wc4.x, wc4.y, wc4.z};
        float t = sphereT<E>(wc, db1, center, kRadius);
        const V3 origin = wc * 4.0f;
#pragma unroll 1
        for (int i = 0; i < kSteps; ++i) {
            const V3 pos = origin + L * t;
            float rh;
            if (E) {
                const V3 proj = (0.5f * kRadius) * march::normalize<E>(pos - center) + center;
                rh = clampf(M<E>::div(march::length<E>(pos - proj), thickness), 0.0f, 1.0f);
            } else {
                const V3 d = pos - center;
                const float dd = march::dot(d, d);
                rh = __saturatef(fabsf(dd * rsqrtf(dd) - 0.5f * kRadius) * (1.0f / 10000.0f));
            }
            const V3 w = wind + V3{0.0f, 0.2f * rh, 0.0f};
            const V3 windOffset = (20.0f * w) * (time + rh * 200.0f);
            const float density = cloudTest<E, S>(p, center, cam, pos + windOffset, rh);
            accum = fmaxf(density, accum);
            if (accum > 0.99f) {
                accum = 1.0f;
                break;
            }
            t = t + step;
        }
        if (p.rgba) {
            float4* c = reinterpret_cast<float4*>(reinterpret_cast<char*>(p.rgba) + (size_t)y * p.rgba_pitch) + x;
            float4 v = *c;
            const float k = 1.0f - accum * 2.0f;
            v.x = fmaxf(v.x * k, 0.0f);
            v.y = fmaxf(v.y * k, 0.0f);
            v.z = fmaxf(v.z * k, 0.0f);
            v.w = 1.0f;
            *c = v;
        }
    }
    if (p.shadow) *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.shadow) + (size_t)y * p.shadow_pitch) + x) = accum;
}

template <bool E, int S>
int launch(const ShadowLaunch& p, cudaStream_t s) {
    dim3 block(32, 8), grid((p.width + 31) / 32, (p.height + 7) / 8);
    shadow_kernel<E, S><<<grid, block, 0, s>>>(p);
    count_launch();
    MM_CUDA_TRY(cudaGetLastError());
    return MM_OK;
}

}  // namespace shadow
}  // namespace mm

#endif  // MM_SHADOW_KERNEL_CUH_
