// reproject_fast.cu - the reprojection pass (reproject.comp:91-152) in production arithmetic.
//
// The same quantities as the exact kernel (reproject.cu) by cheaper, algebraically equal forms:
//  - the per-frame terms are computed once on the host: the ray basis (-look, aspect * tanHalfFov *
//    right, tanHalfFov * up), the camera position relative to the inner sphere in its unit frame
//    (ro = (cam - centre) / w) and C = |ro|^2 - 0.25 of the intersection quadratic;
//  - od = normalize(q) followed by od / -od.z is q / -q.z: the normalisation cancels, one
//    reciprocal replaces a square root and five divisions;
//  - ((od.x / tanHalfFov) / aspect) * 0.5 and (-od.y / tanHalfFov) * 0.5 use precomputed
//    reciprocals; tap positions are formed in pixel units with multiply-adds;
//  - the ten-tap sum is scaled by 0.1 instead of divided by 10.
// A tap whose position lands within rounding of a pixel boundary can select the neighbouring texel
// of the exact kernel; everything else matches it to float rounding.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "mm_internal.h"

namespace mm {
namespace repf {

struct P {
    float ax, ay, az;  // -look
    float rx, ry, rz;  // right * aspect * tanHalfFov
    float ux, uy, uz;  // up * tanHalfFov
    float ox, oy, oz;  // (cam - centre) / w
    float C;           // |ro|^2 - 0.25
    float w;           // sphere parameter (2e6)
    float cx, cy, cz;  // centre
    float pv[12];      // rows 0..2 of cameraPrev.view, 4 columns each
    float ku, kv;      // 0.5 / (tanHalfFov * aspect), 0.5 / tanHalfFov
    float sxs, sys;    // 2 / W, 2 / H
    float iw, ih;      // 1 / W, 1 / H
    const float4* src;
    size_t src_pitch;
    const float* src_depth;
    size_t src_depth_pitch;
    float4* dst;
    size_t dst_pitch;
    float* dst_depth;
    size_t dst_depth_pitch;
    int width, height;
    int skip_phase;  // >= 0: leave the pixels of this 1/16 phase alone
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

__device__ __forceinline__ float4 texel(const P& p, int x, int y) {
    return __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(p.src) + (size_t)y * p.src_pitch) + x);
}

__global__ void __launch_bounds__(256) reproject_fast_kernel(P p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    if (p.skip_phase >= 0 && (x & 3) == (p.skip_phase & 3) && (y & 3) == (p.skip_phase >> 2)) return;
    const float sx = fmaf((float)x, p.sxs, -1.0f), sy = fmaf((float)y, p.sys, -1.0f);
    float dx = p.ax + sx * p.rx - sy * p.ux;
    float dy = p.ay + sx * p.ry - sy * p.uy;
    float dz = p.az + sx * p.rz - sy * p.uz;
    const float inv = rsqrtf(dx * dx + dy * dy + dz * dz);
    dx *= inv;
    dy *= inv;
    dz *= inv;
    // raySphereIntersection(...).point (:57-87); (0, 0, 0) without a hit
    float ipx = 0.0f, ipy = 0.0f, ipz = 0.0f;
    const float A = dx * dx + dy * dy + dz * dz;
    const float B = 2.0f * (dx * p.ox + dy * p.oy + dz * p.oz);
    const float disc = B * B - 4.0f * A * p.C;
    if (disc >= 0.0f) {
        const float s = sqrtf(disc), ia = __fdividef(0.5f, A);
        float t = (-s - B) * ia;
        if (t < 0.0f) t = (s - B) * ia;
        if (t >= 0.0f) {
            ipx = fmaf(dx, t, p.ox) * p.w + p.cx;
            ipy = fmaf(dy, t, p.oy) * p.w + p.cy;
            ipz = fmaf(dz, t, p.oz) * p.w + p.cz;
        }
    }
    const float* m = p.pv;
    const float qx = m[0] * ipx + m[1] * ipy + m[2] * ipz + m[3];
    const float qy = m[4] * ipx + m[5] * ipy + m[6] * ipz + m[7];
    const float qz = m[8] * ipx + m[9] * ipy + m[10] * ipz + m[11];
    const float iz = __fdividef(-1.0f, qz);
    const float oldU = fmaf(qx * iz, p.ku, 0.5f);
    const float oldV = fmaf(-qy * iz, p.kv, 0.5f);
    // ten taps along the motion vector (:142-148), in pixel units
    const float W = (float)p.width, H = (float)p.height;
    const float ou = oldU * W, ov = oldV * H;
    const float bu = (oldU - (float)x * p.iw) * W, bv = (oldV - (float)y * p.ih) * H;
    float4 acc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
    for (int s = 0; s < 10; ++s) {
        const float k = (float)s / 9.0f - 0.5f;
        const int tx = clampi(__float2int_rn(fmaf(-bu, k, ou)), 0, p.width - 1);
        const int ty = clampi(__float2int_rn(fmaf(-bv, k, ov)), 0, p.height - 1);
        const float4 t = texel(p, tx, ty);
        acc.x += t.x;
        acc.y += t.y;
        acc.z += t.z;
        acc.w += t.w;
    }
    const int cx = clampi(__float2int_rn(ou), 0, p.width - 1), cy = clampi(__float2int_rn(ov), 0, p.height - 1);
    float4 o = make_float4(acc.x * 0.1f, acc.y * 0.1f, acc.z * 0.1f, texel(p, cx, cy).w);
    *(reinterpret_cast<float4*>(reinterpret_cast<char*>(p.dst) + (size_t)y * p.dst_pitch) + x) = o;
    if (p.dst_depth && p.src_depth)
        *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.dst_depth) + (size_t)y * p.dst_depth_pitch) + x) =
            __ldg(reinterpret_cast<const float*>(reinterpret_cast<const char*>(p.src_depth) + (size_t)cy * p.src_depth_pitch) + cx);
}

}  // namespace repf

// Host side: the per-frame terms, then the launch.  src/dst validated by the caller.
int launch_reproject_fast(const mm_uniforms& u, const mm_image& src, const mm_image& dst, int skip_phase,
                          cudaStream_t s) {
    repf::P p;
    const float* v = u.camera.view;
    const float* pv = u.camera_prev.view;
    const float aspect = u.camera.camera_params[0], tan = u.camera.camera_params[1];
    p.ax = -v[2];
    p.ay = -v[6];
    p.az = -v[10];
    p.rx = v[0] * aspect * tan;
    p.ry = v[4] * aspect * tan;
    p.rz = v[8] * aspect * tan;
    p.ux = v[1] * tan;
    p.uy = v[5] * tan;
    p.uz = v[9] * tan;
    p.w = 2000000.0f;
    p.cx = u.camera.camera_position[0];
    p.cy = -2000000.0f * 0.5f * 0.995f;
    p.cz = u.camera.camera_position[2];
    p.ox = (u.camera.camera_position[0] - p.cx) / p.w;
    p.oy = (u.camera.camera_position[1] - p.cy) / p.w;
    p.oz = (u.camera.camera_position[2] - p.cz) / p.w;
    p.C = p.ox * p.ox + p.oy * p.oy + p.oz * p.oz - 0.25f;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 4; ++c) p.pv[r * 4 + c] = pv[c * 4 + r];
    p.ku = 0.5f / (tan * aspect);
    p.kv = 0.5f / tan;
    p.sxs = 2.0f / (float)dst.width;
    p.sys = 2.0f / (float)dst.height;
    p.iw = 1.0f / (float)dst.width;
    p.ih = 1.0f / (float)dst.height;
    p.src = reinterpret_cast<const float4*>(src.rgba);
    p.src_pitch = src.rgba_pitch_bytes;
    p.src_depth = src.depth;
    p.src_depth_pitch = src.depth_pitch_bytes;
    p.dst = reinterpret_cast<float4*>(dst.rgba);
    p.dst_pitch = dst.rgba_pitch_bytes;
    p.dst_depth = dst.depth;
    p.dst_depth_pitch = dst.depth_pitch_bytes;
    p.width = dst.width;
    p.height = dst.height;
    p.skip_phase = skip_phase;
    repf::reproject_fast_kernel<<<dim3((p.width + 31) / 32, (p.height + 7) / 8), dim3(32, 8), 0, s>>>(p);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    return MM_OK;
}

}  // namespace mm
