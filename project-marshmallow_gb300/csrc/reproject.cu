// reproject.cu - the reprojection pass of reproject.comp:91-152 (mm_clouds_reproject; this file
// holds the exact-arithmetic kernel, reproject_fast.cu the production one) and the
// reference's per-frame compute work (mm_clouds_frame: reprojection of every pixel, then the march
// of one pixel in 16, VulkanApplication.cpp:1053-1071).
//
// Built with -fmad=false: the pass uses only IEEE +, -, *, /, sqrt and round, so it equals the CPU
// restatement bit for bit.  Per pixel: the ray of the pixel (uv = pixel / image size, :93-94) meets
// the inner atmosphere sphere; the hit point in the previous camera's view space gives the pixel's
// previous uv; ten taps along the motion vector are averaged (:142-148); alpha (and depth, which
// the reference does not have) come from the centre tap (:150-151).
#include <cuda_runtime.h>

#include "mm_internal.h"

namespace mm {
namespace rep {

struct P {
    mm_uniforms u;
    const float4* src;
    size_t src_pitch;
    const float* src_depth;
    size_t src_depth_pitch;
    float4* dst;
    size_t dst_pitch;
    float* dst_depth;
    size_t dst_depth_pitch;
    int w, h;
    int skip_phase;  // >= 0: leave the pixels of this 1/16 phase alone (the march writes them)
};

struct v3 {
    float x, y, z;
};
__device__ __forceinline__ v3 add(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ v3 sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ v3 mul(float s, v3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ v3 mulv(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ v3 normalize(v3 a) { return mulv(a, __fdiv_rn(1.0f, __fsqrt_rn(dot(a, a)))); }

__device__ __forceinline__ v3 sphere_point(v3 ro, v3 rd, v3 c, float w) {  // :57-87 (.point)
    ro = sub(ro, c);
    ro = {__fdiv_rn(ro.x, w), __fdiv_rn(ro.y, w), __fdiv_rn(ro.z, w)};
    const float A = dot(rd, rd);
    const float B = 2.0f * dot(rd, ro);
    const float C = dot(ro, ro) - 0.25f;
    const float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return {0.0f, 0.0f, 0.0f};
    float t = __fdiv_rn(-__fsqrt_rn(disc) - B, A) * 0.5f;
    if (t < 0.0f) t = __fdiv_rn(__fsqrt_rn(disc) - B, A) * 0.5f;
    if (!(t >= 0.0f)) return {0.0f, 0.0f, 0.0f};
    v3 p = add(ro, mulv(rd, t));
    p = mulv(p, w);
    return add(p, c);
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

__global__ void __launch_bounds__(256) reproject_kernel(P p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.w || y >= p.h) return;
    if (p.skip_phase >= 0 && (x & 3) == (p.skip_phase & 3) && (y & 3) == (p.skip_phase >> 2)) return;
    const float* view = p.u.camera.view;
    const float* pv = p.u.camera_prev.view;
    const v3 cam = {p.u.camera.camera_position[0], p.u.camera.camera_position[1], p.u.camera.camera_position[2]};
    const float cpx = p.u.camera.camera_params[0], cpy = p.u.camera.camera_params[1];
    const v3 look = {view[2], view[6], view[10]}, right = {view[0], view[4], view[8]}, up = {view[1], view[5], view[9]};
    v3 center = cam;
    center.y = -2000000.0f * 0.5f * 0.995f;
    const float uvx = __fdiv_rn((float)x, (float)p.w), uvy = __fdiv_rn((float)y, (float)p.h);
    const float sx = uvx * 2.0f - 1.0f, sy = uvy * 2.0f - 1.0f;
    const v3 ref = sub(cam, look);
    const v3 q0 = sub(add(ref, mul(cpx * sx * cpy, right)), mul(sy * cpy, up));
    const v3 rd = normalize(sub(q0, cam));
    const v3 ip = sphere_point(cam, rd, center, 2000000.0f);
    // (cameraPrev.view * vec4(ip, 1)).xyz, summed pairwise as the CPU restatement does
    const v3 q = {(pv[0] * ip.x + pv[4] * ip.y) + (pv[8] * ip.z + pv[12]),
                  (pv[1] * ip.x + pv[5] * ip.y) + (pv[9] * ip.z + pv[13]),
                  (pv[2] * ip.x + pv[6] * ip.y) + (pv[10] * ip.z + pv[14])};
    v3 od = normalize(q);
    const float nz = -od.z;
    od = {__fdiv_rn(od.x, nz), __fdiv_rn(od.y, nz), __fdiv_rn(od.z, nz)};
    float oldU = __fdiv_rn(__fdiv_rn(od.x, cpy), cpx);
    oldU = oldU * 0.5f + 0.5f;
    float oldV = __fdiv_rn(-od.y, cpy);
    oldV = oldV * 0.5f + 0.5f;
    const float bx = oldU - uvx, by = oldV - uvy;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int s = 0; s < 10; ++s) {
        const float k = __fdiv_rn((float)s, 9.0f) - 0.5f;
        const float ox = bx * k, oy = by * k;
        const int cx = clampi((int)roundf((oldU - ox) * (float)p.w), 0, p.w - 1);
        const int cy = clampi((int)roundf((oldV - oy) * (float)p.h), 0, p.h - 1);
        const float4 t = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(p.src) + (size_t)cy * p.src_pitch) + cx);
        acc.x += t.x;
        acc.y += t.y;
        acc.z += t.z;
        acc.w += t.w;
    }
    acc = make_float4(__fdiv_rn(acc.x, 10.0f), __fdiv_rn(acc.y, 10.0f), __fdiv_rn(acc.z, 10.0f), __fdiv_rn(acc.w, 10.0f));
    const int cx = clampi((int)roundf(oldU * (float)p.w), 0, p.w - 1), cy = clampi((int)roundf(oldV * (float)p.h), 0, p.h - 1);
    acc.w = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(p.src) + (size_t)cy * p.src_pitch) + cx).w;
    *(reinterpret_cast<float4*>(reinterpret_cast<char*>(p.dst) + (size_t)y * p.dst_pitch) + x) = acc;
    if (p.dst_depth && p.src_depth)
        *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.dst_depth) + (size_t)y * p.dst_depth_pitch) + x) =
            __ldg(reinterpret_cast<const float*>(reinterpret_cast<const char*>(p.src_depth) + (size_t)cy * p.src_depth_pitch) + cx);
}

}  // namespace rep
}  // namespace mm

namespace mm {
int launch_reproject_fast(const mm_uniforms& u, const mm_image& src, const mm_image& dst, int skip_phase,
                          cudaStream_t s);

// mm_clouds_reproject with the pixels of one 1/16 phase left alone (skip_phase >= 0), for
// mm_clouds_frame, whose march writes them.
static int reproject(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                     const mm_march_options* opt, int skip_phase, void* stream) {
    using mm::fail;
    if (!ctx || !u || !src || !dst) return fail(MM_ERR_INVALID_ARGUMENT, "reproject: null argument");
    const int math = opt ? opt->math : MM_MATH_FAST;
    if (math != MM_MATH_FAST && math != MM_MATH_EXACT) return fail(MM_ERR_INVALID_ARGUMENT, "reproject: bad math %d", math);
    if (!src->rgba || !dst->rgba || src->width != dst->width || src->height != dst->height || dst->width <= 0 ||
        dst->height <= 0 || dst->width > 32768 || dst->height > 32768)
        return fail(MM_ERR_INVALID_ARGUMENT, "reproject: source and target must be images of the same size");
    if (src->rgba == dst->rgba) return fail(MM_ERR_INVALID_ARGUMENT, "reproject: source and target must differ");
    if (src->rgba_pitch_bytes < (size_t)src->width * 16 || dst->rgba_pitch_bytes < (size_t)dst->width * 16 ||
        src->rgba_pitch_bytes % 16 || dst->rgba_pitch_bytes % 16 || ((uintptr_t)src->rgba) % 16 || ((uintptr_t)dst->rgba) % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "reproject: bad rgba pitch or alignment");
    if ((src->depth && src->depth_pitch_bytes < (size_t)src->width * 4) ||
        (dst->depth && dst->depth_pitch_bytes < (size_t)dst->width * 4))
        return fail(MM_ERR_INVALID_ARGUMENT, "reproject: bad depth pitch");
    if (math == MM_MATH_FAST) return mm::launch_reproject_fast(*u, *src, *dst, skip_phase, (cudaStream_t)stream);
    mm::rep::P p;
    p.u = *u;
    p.src = reinterpret_cast<const float4*>(src->rgba);
    p.src_pitch = src->rgba_pitch_bytes;
    p.src_depth = src->depth;
    p.src_depth_pitch = src->depth_pitch_bytes;
    p.dst = reinterpret_cast<float4*>(dst->rgba);
    p.dst_pitch = dst->rgba_pitch_bytes;
    p.dst_depth = dst->depth;
    p.dst_depth_pitch = dst->depth_pitch_bytes;
    p.w = dst->width;
    p.h = dst->height;
    p.skip_phase = skip_phase;
    mm::rep::reproject_kernel<<<dim3((p.w + 31) / 32, (p.h + 7) / 8), dim3(32, 8), 0, (cudaStream_t)stream>>>(p);
    MM_CUDA_TRY(cudaGetLastError());
    mm::count_launch();
    return MM_OK;
}
}  // namespace mm

extern "C" int mm_clouds_reproject(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                                   const mm_march_options* opt, void* stream) {
    return mm::reproject(ctx, u, src, dst, opt, -1, stream);
}

extern "C" int mm_clouds_frame(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_image* prev,
                               const mm_image* out, const mm_march_options* opt, void* stream) {
    mm_march_options o;
    if (opt)
        o = *opt;
    else
        mm_march_options_default(&o);
    o.pixel_mode = MM_PIXELS_PHASE16;
    int r = mm::validate_march(ctx, u, tex, out, &o);
    if (r) return r;
    // The march of one pixel in 16 is bounded by the latency of its longest rays and leaves most of
    // the GPU idle; the reprojection writes the other 15 pixels in 16 (the march overwrites the
    // phase's pixels anyway) on a second stream, concurrently.  Both read only prev and the textures.
    cudaStream_t s = (cudaStream_t)stream;
    if (!ctx->aux_stream) {
        MM_CUDA_TRY(cudaStreamCreateWithFlags(&ctx->aux_stream, cudaStreamNonBlocking));
        MM_CUDA_TRY(cudaEventCreateWithFlags(&ctx->aux_fork, cudaEventDisableTiming));
        MM_CUDA_TRY(cudaEventCreateWithFlags(&ctx->aux_join, cudaEventDisableTiming));
    }
    MM_CUDA_TRY(cudaEventRecord(ctx->aux_fork, s));
    MM_CUDA_TRY(cudaStreamWaitEvent(ctx->aux_stream, ctx->aux_fork, 0));
    r = mm::reproject(ctx, u, prev, out, &o, (int)u->sun.color[3], ctx->aux_stream);
    if (r == MM_OK) r = mm_clouds_march(ctx, u, tex, out, &o, stream);
    // join in every case, so that the caller's stream never runs ahead of the reprojection
    cudaEventRecord(ctx->aux_join, ctx->aux_stream);
    cudaStreamWaitEvent(s, ctx->aux_join, 0);
    return r;
}
