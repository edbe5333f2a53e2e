// march_kernel.cuh - the cloud raymarch of compute-clouds.comp:288-500 as CUDA device code.
//
// One thread marches one pixel-ray.  The code is a template over
//   kExact   - true: IEEE +,-,*,/,sqrt and the mm_math.h elementary functions, for a translation
//              unit compiled with -fmad=false (bit-identical to the FP32 CPU oracle when the
//              software sampler is used); false: FMA contraction and the SFU approximations.
//   kSampler - MM_SAMPLER_SOFTWARE (float-weight trilinear from the UNORM8 texels, the sampler
//              definition of the oracle) or MM_SAMPLER_HARDWARE (texture objects: LINEAR, WRAP,
//              normalized coordinates; 8-bit fixed-point filter weights).
// Evaluation order follows the source order of the shader, left to right, like the oracle.
#ifndef MM_MARCH_KERNEL_CUH_
#define MM_MARCH_KERNEL_CUH_

#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "mm_internal.h"
#include "mm_math.h"

namespace mm {
namespace march {

// ------------------------------------------------------------------------------ arithmetic policy

template <bool kExact>
struct M;

template <>
struct M<true> {
    static __device__ __forceinline__ float exp(float x) { return mmx::mm_expf(x); }
    static __device__ __forceinline__ float pow(float x, float y) { return mmx::mm_powf(x, y); }
    static __device__ __forceinline__ float acos(float x) { return mmx::mm_acosf(x); }
    static __device__ __forceinline__ float cos(float x) { return mmx::mm_cosf(x); }
    static __device__ __forceinline__ float sin(float x) { return mmx::mm_sinf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return __fsqrt_rn(x); }
    static __device__ __forceinline__ float rsqrt(float x) { return __fdiv_rn(1.0f, __fsqrt_rn(x)); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};

template <>
struct M<false> {
    static __device__ __forceinline__ float exp(float x) { return __expf(x); }
    static __device__ __forceinline__ float pow(float x, float y) {
        // GLSL pow = exp2(y * log2(x)); x == 0 gives exp2(-inf) = 0 for y > 0.
        return exp2f(y * __log2f(x));
    }
    static __device__ __forceinline__ float acos(float x) { return acosf(x); }
    static __device__ __forceinline__ float cos(float x) { return __cosf(x); }
    static __device__ __forceinline__ float sin(float x) { return __sinf(x); }
    static __device__ __forceinline__ float sqrt(float x) { return sqrtf(x); }
    static __device__ __forceinline__ float rsqrt(float x) { return rsqrtf(x); }
    static __device__ __forceinline__ float div(float a, float b) { return __fdividef(a, b); }
};

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator+(V3 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
__device__ __forceinline__ V3 operator-(float s, V3 a) { return {s - a.x, s - a.y, s - a.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
__device__ __forceinline__ float mixf(float x, float y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 mix3(V3 x, V3 y, float a) { return x * (1.0f - a) + y * a; }
__device__ __forceinline__ V3 ld3(const float* p) { return {p[0], p[1], p[2]}; }

template <bool E>
__device__ __forceinline__ float length(V3 a) { return M<E>::sqrt(dot(a, a)); }
template <bool E>
__device__ __forceinline__ V3 normalize(V3 a) { return a * M<E>::rsqrt(dot(a, a)); }
template <bool E>
__device__ __forceinline__ float remap(float v, float a, float b, float c, float d) {
    return c + ((M<E>::div(v - a, b - a)) * (d - c));
}
template <bool E>
__device__ __forceinline__ float remapClamped(float v, float a, float b, float c, float d) {
    return clampf(c + ((M<E>::div(v - a, b - a)) * (d - c)), c, d);
}
template <bool E>
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    float t = clampf(M<E>::div(x - e0, e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// ------------------------------------------------------------------------------ samplers

__device__ __forceinline__ int wrapi(int i, int n) {
    int m = i % n;
    return m < 0 ? m + n : m;
}

struct F4 {
    float x, y, z, w;
};

template <bool E>
__device__ __forceinline__ F4 fetch_unorm(const TexView& t, int x, int y, int z) {
    const size_t i = ((size_t)z * t.h + y) * t.w + x;
    if (t.channels == 4) {
        uchar4 c = __ldg(reinterpret_cast<const uchar4*>(t.texels) + i);
        return {M<E>::div((float)c.x, 255.0f), M<E>::div((float)c.y, 255.0f), M<E>::div((float)c.z, 255.0f),
                M<E>::div((float)c.w, 255.0f)};
    } else if (t.channels == 2) {
        uchar2 c = __ldg(reinterpret_cast<const uchar2*>(t.texels) + i);
        return {M<E>::div((float)c.x, 255.0f), M<E>::div((float)c.y, 255.0f), 0.0f, 1.0f};
    }
    return {M<E>::div((float)__ldg(t.texels + i), 255.0f), 0.0f, 0.0f, 1.0f};
}

__device__ __forceinline__ F4 mix4(F4 a, F4 b, float w) {
    return {mixf(a.x, b.x, w), mixf(a.y, b.y, w), mixf(a.z, b.z, w), mixf(a.w, b.w, w)};
}

template <bool E, int S>
__device__ __forceinline__ F4 sample2d(const TexView& t, float u, float v) {
    if (S == MM_SAMPLER_HARDWARE) {
        if (t.channels == 2) {
            float2 r = tex2D<float2>(t.tex, u, v);
            return {r.x, r.y, 0.0f, 1.0f};
        }
        float4 r = tex2D<float4>(t.tex, u, v);
        return {r.x, r.y, r.z, r.w};
    } else {
        float x = u * (float)t.w - 0.5f, y = v * (float)t.h - 0.5f;
        float fx = floorf(x), fy = floorf(y);
        float ax = x - fx, ay = y - fy;
        int x0 = wrapi((int)fx, t.w), x1 = wrapi((int)fx + 1, t.w);
        int y0 = wrapi((int)fy, t.h), y1 = wrapi((int)fy + 1, t.h);
        F4 a = mix4(fetch_unorm<E>(t, x0, y0, 0), fetch_unorm<E>(t, x1, y0, 0), ax);
        F4 b = mix4(fetch_unorm<E>(t, x0, y1, 0), fetch_unorm<E>(t, x1, y1, 0), ax);
        return mix4(a, b, ay);
    }
}

template <bool E, int S>
__device__ __forceinline__ F4 sample3d(const TexView& t, V3 p) {
    if (S == MM_SAMPLER_HARDWARE) {
        float4 r = tex3D<float4>(t.tex, p.x, p.y, p.z);
        return {r.x, r.y, r.z, r.w};
    } else {
        float x = p.x * (float)t.w - 0.5f, y = p.y * (float)t.h - 0.5f, z = p.z * (float)t.d - 0.5f;
        float fx = floorf(x), fy = floorf(y), fz = floorf(z);
        float ax = x - fx, ay = y - fy, az = z - fz;
        int x0 = wrapi((int)fx, t.w), x1 = wrapi((int)fx + 1, t.w);
        int y0 = wrapi((int)fy, t.h), y1 = wrapi((int)fy + 1, t.h);
        int z0 = wrapi((int)fz, t.d), z1 = wrapi((int)fz + 1, t.d);
        F4 a = mix4(fetch_unorm<E>(t, x0, y0, z0), fetch_unorm<E>(t, x1, y0, z0), ax);
        F4 b = mix4(fetch_unorm<E>(t, x0, y1, z0), fetch_unorm<E>(t, x1, y1, z0), ax);
        F4 d = mix4(fetch_unorm<E>(t, x0, y0, z1), fetch_unorm<E>(t, x1, y0, z1), ax);
        F4 e = mix4(fetch_unorm<E>(t, x0, y1, z1), fetch_unorm<E>(t, x1, y1, z1), ax);
        return mix4(mix4(a, b, ay), mix4(d, e, ay), az);
    }
}

// ------------------------------------------------------------------------------ shader functions

constexpr float kRadius = 2000000.0f;  // ATMOSPHERE_RADIUS (:56)
constexpr int kMaxIterations = 8192;    // loop-iteration cap per ray (the CPU oracle uses the same)

template <bool E>
__device__ __forceinline__ float hgPhase(float cosTheta, float g) {  // :73-77
    float g2 = g * g;
    float inv = M<E>::div(1.0f, M<E>::pow(1.0f - 2.0f * g * cosTheta + g2, 1.5f));
    return 0.07957747154594767f * ((1.0f - g2) * inv);
}

template <bool E>
__device__ __forceinline__ V3 atmosphereColor(const mm_uniforms& u, V3 dir, V3 sunDir) {  // :88-127
    const float sunE = u.sun.intensity;
    const V3 BetaR = ld3(u.sky.beta_r), BetaM = ld3(u.sky.beta_v);
    float zenith = M<E>::acos(fmaxf(0.0f, dir.y));
    float inverse = M<E>::div(
        1.0f, M<E>::cos(zenith) + 0.15f * M<E>::pow(93.885f - M<E>::div(zenith * 180.0f, 3.14159265f), -1.253f));
    float sR = 8.4E3f * inverse;
    float sM = 1.25E3f * inverse;
    V3 e = (-BetaR) * sR + BetaM * sM;
    V3 fex = {M<E>::exp(e.x), M<E>::exp(e.y), M<E>::exp(e.z)};
    float cosTheta = dot(sunDir, dir);
    float rPhase = 0.05968310365946075f * (1.0f + (cosTheta * 0.5f + 0.5f) * (cosTheta * 0.5f + 0.5f));
    V3 betaRTheta = BetaR * rPhase;
    float mPhase = hgPhase<E>(cosTheta, u.sky.mie_directional);
    V3 betaMTheta = BetaM * mPhase;
    float yDot = 1.0f - sunDir.y;
    yDot *= yDot * yDot * yDot * yDot;
    V3 num = betaRTheta + betaMTheta, den = BetaR + BetaM;
    V3 betas = {M<E>::div(num.x, den.x), M<E>::div(num.y, den.y), M<E>::div(num.z, den.z)};
    V3 a = sunE * betas * (1.0f - fex);
    V3 Lin = {M<E>::pow(a.x, 1.5f), M<E>::pow(a.y, 1.5f), M<E>::pow(a.z, 1.5f)};
    V3 b = sunE * betas * fex;
    V3 pb = {M<E>::pow(b.x, 0.5f), M<E>::pow(b.y, 0.5f), M<E>::pow(b.z, 0.5f)};
    Lin = Lin * mix3(V3{1.0f, 1.0f, 1.0f}, pb, clampf(yDot, 0.0f, 1.0f));
    V3 L0 = 0.1f * fex;
    const float sunDisk = 0.0f;  // :119-120
    L0 = L0 + ((sunE * 15000.0f) * fex) * sunDisk;
    return (Lin + L0) * 0.04f + V3{0.0f, 0.0003f, 0.00075f};
}

template <bool E>
__device__ __forceinline__ V3 projectedShellPoint(V3 pt, V3 center) {  // :180-182
    return 0.5f * kRadius * normalize<E>(pt - center) + center;
}

template <bool E>
__device__ __forceinline__ float relativeHeight(V3 pt, V3 proj, float thickness) {  // :186-188
    return clampf(M<E>::div(length<E>(pt - proj), thickness), 0.0f, 1.0f);
}

template <bool E>
__device__ __forceinline__ float cloudLayerDensity(float rh, float type) {  // :193-204
    rh = clampf(rh, 0.0f, 1.0f);
    float cumulus = fmaxf(0.0f, remap<E>(rh, 0.0f, 0.2f, 0.0f, 1.0f) * remap<E>(rh, 0.7f, 0.9f, 1.0f, 0.0f));
    float stratocumulus = fmaxf(0.0f, remap<E>(rh, 0.0f, 0.2f, 0.0f, 1.0f) * remap<E>(rh, 0.2f, 0.7f, 1.0f, 0.0f));
    float stratus = fmaxf(0.0f, remap<E>(rh, 0.0f, 0.1f, 0.0f, 1.0f) * remap<E>(rh, 0.2f, 0.3f, 1.0f, 0.0f));
    float d1 = mixf(stratus, stratocumulus, clampf(type * 2.0f, 0.0f, 1.0f));
    float d2 = mixf(stratocumulus, cumulus, clampf((type - 0.5f) * 2.0f, 0.0f, 1.0f));
    return mixf(d1, d2, type);
}

struct Scene {
    V3 cam;
    V3 center;
    V3 wind;
    float time;
    float thickness;
    float coverage_offset;
};

template <bool E, int S>
__device__ __forceinline__ float cloudTest(const MarchLaunch& p, const Scene& sc, V3 pos, float rh,
                                           unsigned long long& n_test) {  // :231-253
    ++n_test;
    V3 proj = projectedShellPoint<E>(pos, sc.center);
    F4 info = sample2d<E, S>(p.weather, 0.000009f * (proj.x - sc.cam.x), 0.000009f * (proj.z - sc.cam.z));
    float layer = cloudLayerDensity<E>(rh, info.z);
    F4 dn = sample3d<E, S>(p.low, 0.00002f * pos);
    float density = layer * remapClamped<E>(dn.x, 0.3f, 1.0f, 0.0f, 1.0f);
    if (density < 0.0001f) return 0.0f;
    // heightBiasCoverage(relativeHeight, min(0.85, weather.r)) with its arguments swapped as in :245
    float h = fminf(0.85f, info.x + sc.coverage_offset);
    float coverage = M<E>::pow(rh, clampf(remap<E>(h, 0.7f, 0.8f, 1.0f, 0.8f), 0.8f, 1.0f));
    float erosion = 0.625f * dn.y + 0.25f * dn.z + 0.125f * dn.w;
    erosion = remapClamped<E>(erosion, coverage, 1.0f, 0.0f, 1.0f);
    return remapClamped<E>(density, erosion, 1.0f, 0.0f, 1.0f);
}

template <bool E, int S>
__device__ __forceinline__ float cloudHiRes(const MarchLaunch& p, V3 pos, float curlStrength, float orig, float rh,
                                            unsigned long long& n_hires) {  // :214-228
    ++n_hires;
    F4 c = sample2d<E, S>(p.curl, 0.0001f * pos.x, 0.0001f * pos.z);
    V3 curl = {2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f};
    pos = pos + 1.9f * curlStrength * curl;
    F4 dn = sample3d<E, S>(p.hi, 0.0004f * pos);
    float erosion = 0.625f * dn.x + 0.25f * dn.y + 0.125f * dn.z;
    erosion = mixf(erosion, 1.0f - erosion, clampf(rh * 10.0f, 0.0f, 1.0f));
    return remapClamped<E>(orig, 1.0f * erosion, 1.0f, 0.0f, 1.0f);
}

struct Isect {
    float t;
};

template <bool E>
__device__ __forceinline__ Isect raySphere(V3 ro, V3 rd, V3 c, float w) {  // :147-177
    Isect is{0.0f};
    ro = ro - c;
    ro = {M<E>::div(ro.x, w), M<E>::div(ro.y, w), M<E>::div(ro.z, w)};
    float A = dot(rd, rd);
    float B = 2.0f * dot(rd, ro);
    float C = dot(ro, ro) - 0.25f;
    float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return is;
    float t = M<E>::div(-M<E>::sqrt(disc) - B, A) * 0.5f;
    if (t < 0.0f) t = M<E>::div(M<E>::sqrt(disc) - B, A) * 0.5f;
    if (t >= 0.0f) {
        V3 q = ro + rd * t;
        q = q * w;
        q = q + c;
        is.t = length<E>(q - ro);
    }
    return is;
}

// The whole of main() (:288-500) for pixel (px, py).  Writes colour and depth.
template <bool E, int S>
__device__ void march_pixel(const MarchLaunch& p, int px, int py, unsigned long long* cnt) {
    const mm_uniforms& u = p.u;
    unsigned long long n_test = 0, n_hires = 0, n_iter = 0, n_acc = 0;
    Scene sc;
    sc.time = u.sky.wind[3];
    sc.wind = ld3(u.sky.wind);
    sc.coverage_offset = p.coverage_offset;
    const float* view = u.camera.view;
    float uvx = M<E>::div((float)px, p.uv_w), uvy = M<E>::div((float)py, p.uv_h);
    float spx = uvx * 2.0f - 1.0f, spy = uvy * 2.0f - 1.0f;
    V3 camLook = {view[2], view[6], view[10]};
    V3 camRight = {view[0], view[4], view[8]};
    V3 camUp = {view[1], view[5], view[9]};
    const V3 cameraPos = ld3(u.camera.camera_position);
    sc.cam = cameraPos;
    V3 refPoint = cameraPos - camLook;
    const float cpx = u.camera.camera_params[0], cpy = u.camera.camera_params[1];
    V3 q = refPoint + cpx * spx * cpy * camRight - spy * cpy * camUp;
    V3 rd = normalize<E>(q - cameraPos);

    V3 sunDir = normalize<E>(ld3(u.sun.direction_basis + 4));
    const float sunY = u.sun.direction[1];
    float dotToSun = fmaxf(0.0f, dot(sunDir, rd));
    float skyAmbient = dotToSun * 0.18f;
    skyAmbient *= skyAmbient * skyAmbient;
    const float SUN_ANGULAR_COS = 0.999956676946448443553574619906976478926848692873900859324f;
    float sunDisk = smoothstep<E>(SUN_ANGULAR_COS, SUN_ANGULAR_COS + 0.00003f, dotToSun);
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun;
    if (sunY < 0.0f) dotToSun *= dotToSun * dotToSun * dotToSun * dotToSun * dotToSun * dotToSun;
    sunDisk = fmaxf(sunDisk, dotToSun);
    sunDisk = fmaxf(0.0f, sunDisk);

    float4 fc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    V3 bg = {0.0f, 0.0f, 0.0f};
    if (sunY >= 0.0f) {
        bg = atmosphereColor<E>(u, rd, sunDir);
        fc.w = fmaxf(skyAmbient, sunDisk);
        fc.x = bg.x;
        fc.y = bg.y;
        fc.z = bg.z;
    }
    float4* out = reinterpret_cast<float4*>(reinterpret_cast<char*>(p.rgba) + (size_t)py * p.rgba_pitch) + px;
    float* dout = p.depth ? reinterpret_cast<float*>(reinterpret_cast<char*>(p.depth) + (size_t)py * p.depth_pitch) + px
                          : nullptr;
    if (dot(rd, V3{0.0f, 1.0f, 0.0f}) < 0.0f) {  // :351-354
        *out = fc;
        if (dout) *dout = CUDART_INF_F;
        return;
    }

    V3 center = cameraPos;
    center.y = -kRadius * 0.5f * 0.995f;
    sc.center = center;
    const float thickness = 0.5f * kRadius * 0.02f;
    sc.thickness = thickness;
    Isect inner = raySphere<E>(cameraPos, rd, center, kRadius);
    Isect outer = raySphere<E>(cameraPos, rd, center, kRadius * 1.02f);

    if (sunY < 0.0f) {  // :365-384
        const float nrm = M<E>::rsqrt(2.0f);
        V3 ax = {1.0f * nrm, 0.0f * nrm, 1.0f * nrm};
        float ang = sunY * 0.5f;
        float c = M<E>::cos(ang), s = M<E>::sin(ang);
        V3 c0 = {c + ax.x * ax.x * (1.0f - c), ax.y * ax.x * (1.0f - c) + ax.z * s, ax.z * ax.x * (1.0f - c) - ax.y * s};
        V3 c1 = {ax.x * ax.y * (1.0f - c) - ax.z * s, c + ax.y * ax.y * (1.0f - c), ax.z * ax.y * (1.0f - c) + ax.x * s};
        V3 c2 = {ax.x * ax.z * (1.0f - c) + ax.y * s, ax.y * ax.z * (1.0f - c) - ax.x * s, c + ax.z * ax.z * (1.0f - c)};
        V3 rrd = {(c0.x * rd.x + c1.x * rd.y) + c2.x * rd.z, (c0.y * rd.x + c1.y * rd.y) + c2.y * rd.z,
                  (c0.z * rd.x + c1.z * rd.y) + c2.z * rd.z};
        V3 rro = {(c0.x * cameraPos.x + c1.x * cameraPos.y) + c2.x * cameraPos.z,
                  (c0.y * cameraPos.x + c1.y * cameraPos.y) + c2.y * cameraPos.z,
                  (c0.z * cameraPos.x + c1.z * cameraPos.y) + c2.z * cameraPos.z};
        V3 point = outer.t * rrd + rro;
        V3 pp = projectedShellPoint<E>(point, center);
        F4 ns = sample2d<E, S>(p.night, 0.00002f * (pp.x - cameraPos.x) + 0.35f, 0.00002f * (pp.z - cameraPos.z) + 0.35f);
        bg = {ns.x, ns.y, ns.z};
        bg = bg * (V3{M<E>::sqrt(bg.x), M<E>::sqrt(bg.y), M<E>::sqrt(bg.z)} * 0.75f);
        bg = {M<E>::pow(bg.x, 2.2f), M<E>::pow(bg.y, 2.2f), M<E>::pow(bg.z, 2.2f)};
        bg = bg * 10.0f;
        float falloff = M<E>::pow(rd.y, 6.0f);
        bg = bg * falloff;
        bg = mix3(V3{0.3f, 0.6f, 4.0f} * 0.05f, bg, M<E>::pow(rd.y, 0.03125f));
        bg = bg + sunDisk;
        fc.w = sunDisk;
    }

    const float cosTheta = dot(rd, sunDir);
    float accum = 0.0f, transmittance = 1.0f;
    float stepSize = 0.05f * thickness;
    const V3 b0 = ld3(u.sun.direction_basis + 0), b1 = ld3(u.sun.direction_basis + 4),
             b2 = ld3(u.sun.direction_basis + 8);
    // mat3(directionBasis) * v for the six cone offsets (:392-401)
    auto bm = [&](float x, float y, float z) -> V3 {
        return {(b0.x * x + b1.x * y) + b2.x * z, (b0.y * x + b1.y * y) + b2.y * z, (b0.z * x + b1.z * y) + b2.z * z};
    };
    const V3 samples[6] = {bm(0.0f, 0.6f, 0.0f), bm(0.0f, 0.5f, 0.05f), bm(0.1f, 0.75f, 0.0f),
                           bm(0.2f, 2.5f, 0.3f), bm(0.0f, 6.0f, 0.0f),  bm(-0.1f, 1.0f, -0.2f)};
    bool noHits = true;
    int misses = 0, steps = 0;
    float firstT = CUDART_INF_F;
    const float hg = fmaxf(hgPhase<E>(cosTheta, 0.6f), 0.7f * hgPhase<E>(cosTheta, 0.99f - 0.1f));
    const V3 windScale = {0.1f, 0.05f, 0.0f};

    // :408-482, with an iteration cap (kMaxIterations) that no ray starting inside the shells reaches;
    // it bounds the loop for degenerate uniforms.
    int iterations = 0;
    for (float t = inner.t; t < outer.t && iterations < kMaxIterations; t += stepSize, ++iterations) {
        ++n_iter;
        V3 pos = cameraPos + t * rd;
        V3 proj = projectedShellPoint<E>(pos, center);
        float rh = relativeHeight<E>(pos, proj, thickness);
        V3 windOffset = (20.0f * (sc.wind + rh * windScale)) * (sc.time + rh * 200.0f);
        float density = cloudTest<E, S>(p, sc, pos + windOffset, rh, n_test);
        float loDensity = density;
        if (density > 0.0f) {
            misses = 0;
            if (noHits) {
                t -= stepSize;
                stepSize *= 0.3f;
                noHits = false;
                continue;
            }
            density = cloudHiRes<E, S>(p, pos + windOffset, stepSize, density, rh, n_hires);
            if (density < 0.0001f) continue;
            float densityAlongLight = 0.0f;
#pragma unroll 1
            for (int i = 0; i < 6; i++) {
                V3 lsPos = pos + 3.0f * stepSize * samples[i];
                V3 lsProj = projectedShellPoint<E>(lsPos, center);
                float lsHeight = relativeHeight<E>(lsPos, lsProj, thickness);
                windOffset = (20.0f * (sc.wind + lsHeight * windScale)) * (sc.time + lsHeight * 200.0f);
                float lsDensity = cloudTest<E, S>(p, sc, lsPos + windOffset, lsHeight, n_test);
                if (lsDensity > 0.0f) {
                    lsDensity = cloudHiRes<E, S>(p, lsPos + windOffset, stepSize, lsDensity, lsHeight, n_hires);
                    densityAlongLight += lsDensity;
                }
            }
            float beers = M<E>::exp(-densityAlongLight);
            float beersMod = fmaxf(beers, 0.7f * M<E>::exp(-0.25f * densityAlongLight));
            beers = mixf(beers, beersMod, -cosTheta * 0.5f + 0.5f);
            float inScatter = 0.09f + M<E>::pow(loDensity, remapClamped<E>(rh, 0.3f, 0.85f, 0.5f, 2.0f));
            inScatter *= M<E>::pow(remapClamped<E>(rh, 0.07f, 0.34f, 0.1f, 1.0f), 0.8f);
            transmittance = mixf(transmittance, inScatter * hg * beers, 1.0f - accum);
            ++n_acc;
            if (firstT == CUDART_INF_F) firstT = t;
            accum += density;
        } else if (!noHits) {
            misses++;
            if (misses >= 10) {
                noHits = true;
                stepSize = M<E>::div(stepSize, 0.3f);
            }
        }
        if (accum > 0.99f) {
            accum = 1.0f;
            break;
        }
        if (++steps > 100) break;
    }

    accum *= smoothstep<E>(0.0f, 1.0f, fminf(1.0f, remap<E>(rd.y, 0.0f, 0.1f, 0.0f, 1.0f)));
    accum = fminf(accum, 0.999f);
    const V3 sunColor = ld3(u.sun.color);
    const float I = u.sun.intensity;
    const float et = M<E>::exp(-transmittance);
    const float a = I * fmaxf(0.0f, transmittance);
    V3 cloud;
    if (sunY >= 0.0f) {
        cloud = sunColor * (V3{a, a, a} + (0.08f * bg) * et);
    } else {
        V3 night = V3{0.3f, 0.6f, 4.0f} * 0.05f * M<E>::pow(rd.y, 0.03125f);
        cloud = sunColor * (V3{a, a, a} + (0.08f * night) * et);
    }
    V3 rgb = mix3(bg, cloud, accum);
    fc.x = rgb.x;
    fc.y = rgb.y;
    fc.z = rgb.z;
    fc.w *= fmaxf(1.0f - accum, 0.0f);
    *out = fc;
    if (dout) *dout = firstT;
    if (cnt) {
        atomicAdd(cnt + 0, n_test);
        atomicAdd(cnt + 1, n_hires);
        atomicAdd(cnt + 2, n_iter);
        atomicAdd(cnt + 3, n_acc);
    }
}

// Ray-tile order: a block covers a 32x8 pixel tile; each warp an 8x4 sub-tile, so one warp's 32
// rays are a compact footprint in the density textures.
template <bool E, int S>
__global__ void __launch_bounds__(256) march_tiled_kernel(MarchLaunch p) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int tx = blockIdx.x * 32 + (warp & 3) * 8 + (lane & 7);
    const int ty = blockIdx.y * 8 + (warp >> 2) * 4 + (lane >> 3);
    int px, py;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {  // :292-298 (thread grid covers ceil(W/4) x ceil(H/4))
        px = tx * 4 + (p.phase % 4);
        py = ty * 4 + (p.phase / 4);
    } else {
        px = tx;
        py = ty;
    }
    if (px >= p.width || py >= p.height) return;  // :301 with the runtime image size
    march_pixel<E, S>(p, px, py, p.counters);
}

template <bool E, int S>
int launch_tiled(const MarchLaunch& p, cudaStream_t s) {
    int gw = p.width, gh = p.height;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {
        gw = (p.width + 3) / 4;
        gh = (p.height + 3) / 4;
    }
    dim3 grid((gw + 31) / 32, (gh + 7) / 8);
    march_tiled_kernel<E, S><<<grid, 256, 0, s>>>(p);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "march_tiled_kernel launch");
    count_launch();
    return MM_OK;
}

}  // namespace march
}  // namespace mm

#endif  // MM_MARCH_KERNEL_CUH_
