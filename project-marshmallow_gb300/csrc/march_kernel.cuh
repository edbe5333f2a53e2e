// march_kernel.cuh - the cloud raymarch of compute-clouds.comp:288-500 as CUDA device code.
//
// One thread marches one pixel-ray.  The code is a template over
//   kExact   - true: the shader's arithmetic as written, IEEE +,-,*,/,sqrt and the mm_math.h
//              elementary functions, for a translation unit compiled with -fmad=false
//              (bit-identical to the FP32 CPU oracle when the software sampler is used);
//              false: the same quantities by cheaper, algebraically equal forms (below) with FMA
//              contraction and the SFU approximations.
//   kSampler - MM_SAMPLER_SOFTWARE (float-weight trilinear from the UNORM8 texels, the sampler
//              definition of the oracle) or MM_SAMPLER_HARDWARE (texture objects: LINEAR, WRAP,
//              normalized coordinates; 8-bit fixed-point filter weights).
// Evaluation order follows the source order of the shader, left to right, like the oracle.
#ifndef MM_MARCH_KERNEL_CUH_
#define MM_MARCH_KERNEL_CUH_

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <math_constants.h>
#include <stdint.h>

#include "mm_internal.h"
#include "mm_math.h"

// Build knobs (defaults measured best on GB300 at 3840x2160): warps per block of the tiled kernels
// (4 or 8) and the minimum resident blocks per SM requested from the register allocator for them
// (4 warps x 10 blocks: 48 registers, 40 warps per SM; the inline-cone kernel has no spills there and
// was 4.6% slower at 9 blocks / 56 registers; the pooled-cone kernel spills 64 B in its cone rounds
// and was 2.6% / 5.1% slower at 9 / 11 blocks); the same for the persistent kernel; and the
// speculative curl fetch of the tiled march (off: it costs more occupancy than it hides).
#ifndef MM_TILED_WARPS
#define MM_TILED_WARPS 4
#endif
#ifndef MM_MARCH_MIN_BLOCKS
#define MM_MARCH_MIN_BLOCKS (MM_TILED_WARPS == 4 ? 10 : 5)
#endif
#ifndef MM_PERSISTENT_MIN_BLOCKS
#define MM_PERSISTENT_MIN_BLOCKS 3
#endif
#ifndef MM_SPEC_CURL
#define MM_SPEC_CURL 0
#endif

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

// ------------------------------------------------------------------------------ per-launch constants

struct Frame {
    V3 cam, center, wind, sunDir;
    float time, sunY, thickness, coverage_offset;
    // fast-path forms: 20 * wind and 20 * (0.1, 0.05, 0)
    V3 wind20, wscale20;
};

template <bool E>
__device__ __forceinline__ Frame make_frame(const MarchLaunch& p) {
    const mm_uniforms& u = p.u;
    Frame f;
    f.cam = ld3(u.camera.camera_position);
    f.center = f.cam;
    f.center.y = -kRadius * 0.5f * 0.995f;  // :357-358
    f.wind = ld3(u.sky.wind);
    f.time = u.sky.wind[3];  // :289
    if (E)
        f.sunDir = normalize<E>(ld3(u.sun.direction_basis + 4));  // :324
    else
        f.sunDir = ld3(p.sun_dir);
    f.sunY = u.sun.direction[1];
    f.thickness = 0.5f * kRadius * 0.02f;  // :360
    f.coverage_offset = p.coverage_offset;
    f.wind20 = E ? 20.0f * f.wind : ld3(p.wind20);
    f.wscale20 = {2.0f, 1.0f, 0.0f};
    return f;
}


// Cone offsets mat3(directionBasis) * v (:392-401), computed once per block into shared memory
// by threads 0..5 (the caller synchronizes).
__device__ __forceinline__ void cone_offsets(const mm_uniforms& u, V3* out) {
    const int i = threadIdx.x;
    if (i >= 6) return;
    const float* b = u.sun.direction_basis;
    float x, y, z;
    switch (i) {
        case 0: x = 0.0f; y = 0.6f; z = 0.0f; break;
        case 1: x = 0.0f; y = 0.5f; z = 0.05f; break;
        case 2: x = 0.1f; y = 0.75f; z = 0.0f; break;
        case 3: x = 0.2f; y = 2.5f; z = 0.3f; break;
        case 4: x = 0.0f; y = 6.0f; z = 0.0f; break;
        default: x = -0.1f; y = 1.0f; z = -0.2f; break;
    }
    out[i] = {(b[0] * x + b[4] * y) + b[8] * z, (b[1] * x + b[5] * y) + b[9] * z, (b[2] * x + b[6] * y) + b[10] * z};
}

// ------------------------------------------------------------------------------ sample evaluation
//
// A density sample at point `pos` (a march step or a cone tap): relative height of pos, the wind
// offset at that height (:414, :445) and the wind-displaced point sp that cloudTest/cloudHiRes
// read (:421, :436, :447, :450).
//
// Fast-path identities used when kExact is false (the exact path keeps the shader's forms):
//  - getRelativeHeight(pos, getProjectedShellPoint(pos, c), T) (:180-188): pos - proj is
//    d * (1 - R/|d|) with d = pos - c and R = 0.5 * ATMOSPHERE_RADIUS, so its length is
//    | |d| - R |: one square root instead of a normalize, a subtraction and a length.
//  - the weather coordinate 0.000009 * (proj(sp).xz - camera.xz) (:236): the earth centre shares
//    the camera's x and z (:357-358), so proj.xz - cam.xz = R * d2.xz / |d2| with d2 = sp - c,
//    i.e. 9 * d2.xz * rsqrt(|d2|^2).
//  - remap/remapClamped with constant bounds folded into one multiply-add; the three layer
//    profiles of cloudLayerDensity (:193-204) as h (22.5 - 25 h), h (7 - 10 h), h (30 - 100 h).
//  - cloudTest's low-res fetch is skipped where the layer density is exactly zero (the product
//    layer * remapClamped(...) is zero whatever the texel holds, :240, :243).

struct Geo {
    V3 sp;     // wind-displaced sample point
    V3 d2;     // sp - earth centre (fast path)
    float rh;  // relative height of the undisplaced point
};

template <bool E>
__device__ __forceinline__ Geo geo_at(const Frame& f, V3 pos) {
    Geo g;
    if (E) {
        V3 proj = projectedShellPoint<E>(pos, f.center);
        g.rh = relativeHeight<E>(pos, proj, f.thickness);
        const V3 windScale = {0.1f, 0.05f, 0.0f};
        V3 wo = (20.0f * (f.wind + g.rh * windScale)) * (f.time + g.rh * 200.0f);
        g.sp = pos + wo;
        g.d2 = g.sp - f.center;
    } else {
        const V3 d = pos - f.center;
        const float dd = dot(d, d);
        const float len = dd * rsqrtf(dd);
        g.rh = __saturatef(fabsf(len - 0.5f * kRadius) * (1.0f / 20000.0f));
        const float k = f.time + g.rh * 200.0f;
        V3 wo = {(f.wind20.x + g.rh * f.wscale20.x) * k, (f.wind20.y + g.rh * f.wscale20.y) * k, f.wind20.z * k};
        g.sp = pos + wo;
        g.d2 = d + wo;
    }
    return g;
}

__device__ __forceinline__ float layer_fast(float h, float type) {
    const float cumulus = fmaxf(0.0f, h * (22.5f - 25.0f * h));
    const float strato = fmaxf(0.0f, h * (7.0f - 10.0f * h));
    const float stratus = fmaxf(0.0f, h * (30.0f - 100.0f * h));
    const float d1 = stratus + (strato - stratus) * __saturatef(type * 2.0f);
    const float d2 = strato + (cumulus - strato) * __saturatef(type * 2.0f - 1.0f);
    return d1 + (d2 - d1) * type;
}

// cloudTest (:231-253) in two halves so independent fetches can be in flight together: the
// weather and low-res fetches of one sample (and of several cone taps) are issued before any of
// their results is used.
struct TestFetch {
    float cov, type;  // weather.r, weather.b
    F4 dn;            // low-res density noise
};

template <bool E, int S>
__device__ __forceinline__ TestFetch test_fetch(const MarchLaunch& p, const Frame& f, const Geo& g) {
    TestFetch r;
    F4 info;
    if (E) {
        V3 proj = projectedShellPoint<E>(g.sp, f.center);
        info = sample2d<E, S>(p.weather, 0.000009f * (proj.x - f.cam.x), 0.000009f * (proj.z - f.cam.z));
    } else {
        const float rr = rsqrtf(dot(g.d2, g.d2));
        info = sample2d<E, S>(p.weather, 9.0f * rr * g.d2.x, 9.0f * rr * g.d2.z);
    }
    r.cov = info.x;
    r.type = info.z;
    r.dn = sample3d<E, S>(p.low, 0.00002f * g.sp);
    return r;
}

template <bool E>
__device__ __forceinline__ float test_finish(const Frame& f, const Geo& g, const TestFetch& c,
                                             unsigned long long& n_test) {
    ++n_test;
    if (E) {
        float layer = cloudLayerDensity<E>(g.rh, c.type);
        float density = layer * remapClamped<E>(c.dn.x, 0.3f, 1.0f, 0.0f, 1.0f);
        if (density < 0.0001f) return 0.0f;
        // heightBiasCoverage(relativeHeight, min(0.85, weather.r)) with its arguments swapped (:245)
        float h = fminf(0.85f, c.cov + f.coverage_offset);
        float coverage = M<E>::pow(g.rh, clampf(remap<E>(h, 0.7f, 0.8f, 1.0f, 0.8f), 0.8f, 1.0f));
        float erosion = 0.625f * c.dn.y + 0.25f * c.dn.z + 0.125f * c.dn.w;
        erosion = remapClamped<E>(erosion, coverage, 1.0f, 0.0f, 1.0f);
        return remapClamped<E>(density, erosion, 1.0f, 0.0f, 1.0f);
    } else {
        // Branch-free: the coverage and erosion terms are evaluated for every sample and the
        // shader's early return (:243) becomes a select.  A divergent branch costs more here than
        // the arithmetic it would skip (4K frame 3.41 -> 3.34 ms with this form).  For rh == 0 the
        // power is exp2(-inf) = 0 and a zero divisor gives a NaN or infinity that __saturatef and
        // the select turn into the shader's value.
        const float n = __saturatef(c.dn.x * (1.0f / 0.7f) - (0.3f / 0.7f));
        const float density = layer_fast(g.rh, c.type) * n;
        const float h = fminf(0.85f, c.cov + f.coverage_offset);
        const float e = clampf(1.0f - (h - 0.7f) * 2.0f, 0.8f, 1.0f);
        const float coverage = exp2f(e * __log2f(g.rh));
        const float ero = 0.625f * c.dn.y + 0.25f * c.dn.z + 0.125f * c.dn.w;
        const float erosion = __saturatef((ero - coverage) * __fdividef(1.0f, 1.0f - coverage));
        const float out = __saturatef((density - erosion) * __fdividef(1.0f, 1.0f - erosion));
        return density >= 0.0001f ? out : 0.0f;
    }
}

template <bool E, int S>
__device__ __forceinline__ float cloud_test(const MarchLaunch& p, const Frame& f, const Geo& g,
                                            unsigned long long& n_test) {
    return test_finish<E>(f, g, test_fetch<E, S>(p, f, g), n_test);
}

// cloudHiRes (:214-228) in three stages: curl fetch, displaced hi-res fetch, erosion.
template <bool E, int S>
__device__ __forceinline__ F4 curl_fetch(const MarchLaunch& p, const Geo& g) {
    return sample2d<E, S>(p.curl, 0.0001f * g.sp.x, 0.0001f * g.sp.z);
}

template <bool E>
__device__ __forceinline__ V3 curl_displace(const Geo& g, float curlStrength, const F4& c) {
    const V3 pos = g.sp;
    if (E) {
        V3 curl = {2.0f * c.x - 1.0f, 2.0f * c.y - 1.0f, 2.0f * c.z - 1.0f};
        return pos + 1.9f * curlStrength * curl;
    } else {
        const float k = 1.9f * curlStrength;
        return {pos.x + k * (2.0f * c.x - 1.0f), pos.y + k * (2.0f * c.y - 1.0f), pos.z + k * (2.0f * c.z - 1.0f)};
    }
}

template <bool E, int S>
__device__ __forceinline__ V3 hires_point(const MarchLaunch& p, const Geo& g, float curlStrength) {
    return curl_displace<E>(g, curlStrength, curl_fetch<E, S>(p, g));
}

template <bool E, int S>
__device__ __forceinline__ F4 hires_fetch(const MarchLaunch& p, V3 q) {
    return sample3d<E, S>(p.hi, 0.0004f * q);
}

template <bool E>
__device__ __forceinline__ float hires_finish(const F4& dn, float rh, float orig, unsigned long long& n_hires) {
    ++n_hires;
    if (E) {
        float erosion = 0.625f * dn.x + 0.25f * dn.y + 0.125f * dn.z;
        erosion = mixf(erosion, 1.0f - erosion, clampf(rh * 10.0f, 0.0f, 1.0f));
        return remapClamped<E>(orig, 1.0f * erosion, 1.0f, 0.0f, 1.0f);
    } else {
        float e = 0.625f * dn.x + 0.25f * dn.y + 0.125f * dn.z;
        e = e + (1.0f - 2.0f * e) * __saturatef(rh * 10.0f);
        return __saturatef((orig - e) * __fdividef(1.0f, 1.0f - e));
    }
}

template <bool E, int S>
__device__ __forceinline__ float cloud_hires(const MarchLaunch& p, const Geo& g, float curlStrength, float orig,
                                             unsigned long long& n_hires) {
    return hires_finish<E>(hires_fetch<E, S>(p, hires_point<E, S>(p, g, curlStrength)), g.rh, orig, n_hires);
}

#ifndef MM_CONE_GROUP
#define MM_CONE_GROUP 1  // cone taps whose fetches are issued together (1, 2, 3 or 6)
#endif

// Sun-cone taps i0 .. i0+G-1 of one sample (:441-453): their fetches are issued together; the
// densities are added to densityAlongLight in tap order.
// Cone offset k: from the block's shared copy, or (PC: production path, the cone loop unrolled so k
// is a constant) from the launch parameters, where the host put it.
template <bool E, bool PC>
__device__ __forceinline__ V3 cone_offset(const MarchLaunch& p, const V3* cone, int k) {
    if (!E && PC) return {p.cone[3 * k], p.cone[3 * k + 1], p.cone[3 * k + 2]};
    return cone[k];
}

template <bool E, int S, int G, bool PC = false>
__device__ __forceinline__ float cone_taps(const MarchLaunch& p, const Frame& f, const V3* cone, int i0, V3 pos,
                                           float stepSize, float dal, unsigned long long& n_test,
                                           unsigned long long& n_hires) {
    Geo g[G];
    TestFetch c[G];
#pragma unroll
    for (int j = 0; j < G; ++j) {
        g[j] = geo_at<E>(f, pos + 3.0f * stepSize * cone_offset<E, PC>(p, cone, i0 + j));
        c[j] = test_fetch<E, S>(p, f, g[j]);
    }
    float d[G];
#pragma unroll
    for (int j = 0; j < G; ++j) d[j] = test_finish<E>(f, g[j], c[j], n_test);
    if constexpr (!E) {
        // Production path: nearly every tap has density (144 M of 150 M per 4K frame), so the
        // cloudHiRes of every tap is evaluated and added where the tap's density is positive, without
        // a branch (4K frame 3.34 -> 3.25 ms; the 1/16-pixel launches ~15% faster).
        V3 q[G];
#pragma unroll
        for (int j = 0; j < G; ++j) q[j] = hires_point<E, S>(p, g[j], stepSize);
        F4 hv[G];
#pragma unroll
        for (int j = 0; j < G; ++j) hv[j] = hires_fetch<E, S>(p, q[j]);
#pragma unroll
        for (int j = 0; j < G; ++j) {
            unsigned long long used = 0;
            const float h = hires_finish<E>(hv[j], g[j].rh, d[j], used);
            n_hires += d[j] > 0.0f ? used : 0ull;
            dal += d[j] > 0.0f ? h : 0.0f;
        }
    } else {
        V3 q[G];
#pragma unroll
        for (int j = 0; j < G; ++j)
            if (d[j] > 0.0f) q[j] = hires_point<E, S>(p, g[j], stepSize);
        F4 hv[G];
#pragma unroll
        for (int j = 0; j < G; ++j)
            if (d[j] > 0.0f) hv[j] = hires_fetch<E, S>(p, q[j]);
#pragma unroll
        for (int j = 0; j < G; ++j)
            if (d[j] > 0.0f) dal += hires_finish<E>(hv[j], g[j].rh, d[j], n_hires);
    }
    return dal;
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

// Per-ray set-up of main() (:292-407): ray direction, sky colour, horizon kill, shell
// intersections, night sky, phase function.
struct Ray {
    V3 rd, bg;
    float alpha;    // finalColor.a before the cloud term
    float t0, t1;   // inner / outer shell distances
    float cosTheta, hg;
    bool killed;    // rd.y < 0: stored as is (:351-354)
};

template <bool E, int S>
__device__ __forceinline__ Ray ray_setup(const MarchLaunch& p, const Frame& f, int px, int py) {
    const mm_uniforms& u = p.u;
    Ray r;
    const float* view = u.camera.view;
    float uvx = M<E>::div((float)px, p.uv_w), uvy = M<E>::div((float)py, p.uv_h);
    float spx = uvx * 2.0f - 1.0f, spy = uvy * 2.0f - 1.0f;
    V3 camLook = {view[2], view[6], view[10]};
    V3 camRight = {view[0], view[4], view[8]};
    V3 camUp = {view[1], view[5], view[9]};
    V3 refPoint = f.cam - camLook;
    const float cpx = u.camera.camera_params[0], cpy = u.camera.camera_params[1];
    V3 q = refPoint + cpx * spx * cpy * camRight - spy * cpy * camUp;
    r.rd = normalize<E>(q - f.cam);
    const V3 rd = r.rd;

    float dotToSun = fmaxf(0.0f, dot(f.sunDir, rd));
    float skyAmbient = dotToSun * 0.18f;
    skyAmbient *= skyAmbient * skyAmbient;
    const float SUN_ANGULAR_COS = 0.999956676946448443553574619906976478926848692873900859324f;
    float sunDisk = smoothstep<E>(SUN_ANGULAR_COS, SUN_ANGULAR_COS + 0.00003f, dotToSun);
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun * dotToSun;
    dotToSun *= dotToSun * dotToSun;
    if (f.sunY < 0.0f) dotToSun *= dotToSun * dotToSun * dotToSun * dotToSun * dotToSun * dotToSun;
    sunDisk = fmaxf(sunDisk, dotToSun);
    sunDisk = fmaxf(0.0f, sunDisk);

    r.alpha = 0.0f;
    r.bg = {0.0f, 0.0f, 0.0f};
    if (f.sunY >= 0.0f) {
        r.bg = atmosphereColor<E>(u, rd, f.sunDir);
        r.alpha = fmaxf(skyAmbient, sunDisk);
    }
    r.killed = dot(rd, V3{0.0f, 1.0f, 0.0f}) < 0.0f;
    r.t0 = r.t1 = 0.0f;
    r.cosTheta = 0.0f;
    r.hg = 0.0f;
    if (r.killed) return r;

    r.t0 = raySphere<E>(f.cam, rd, f.center, kRadius).t;
    r.t1 = raySphere<E>(f.cam, rd, f.center, kRadius * 1.02f).t;

    if (f.sunY < 0.0f) {  // :365-384
        const float nrm = M<E>::rsqrt(2.0f);
        V3 ax = {1.0f * nrm, 0.0f * nrm, 1.0f * nrm};
        float ang = f.sunY * 0.5f;
        float c = M<E>::cos(ang), s = M<E>::sin(ang);
        V3 c0 = {c + ax.x * ax.x * (1.0f - c), ax.y * ax.x * (1.0f - c) + ax.z * s, ax.z * ax.x * (1.0f - c) - ax.y * s};
        V3 c1 = {ax.x * ax.y * (1.0f - c) - ax.z * s, c + ax.y * ax.y * (1.0f - c), ax.z * ax.y * (1.0f - c) + ax.x * s};
        V3 c2 = {ax.x * ax.z * (1.0f - c) + ax.y * s, ax.y * ax.z * (1.0f - c) - ax.x * s, c + ax.z * ax.z * (1.0f - c)};
        V3 rrd = {(c0.x * rd.x + c1.x * rd.y) + c2.x * rd.z, (c0.y * rd.x + c1.y * rd.y) + c2.y * rd.z,
                  (c0.z * rd.x + c1.z * rd.y) + c2.z * rd.z};
        const V3 cp = f.cam;
        V3 rro = {(c0.x * cp.x + c1.x * cp.y) + c2.x * cp.z, (c0.y * cp.x + c1.y * cp.y) + c2.y * cp.z,
                  (c0.z * cp.x + c1.z * cp.y) + c2.z * cp.z};
        V3 point = r.t1 * rrd + rro;
        V3 pp = projectedShellPoint<E>(point, f.center);
        F4 ns = sample2d<E, S>(p.night, 0.00002f * (pp.x - cp.x) + 0.35f, 0.00002f * (pp.z - cp.z) + 0.35f);
        V3 bg = {ns.x, ns.y, ns.z};
        bg = bg * (V3{M<E>::sqrt(bg.x), M<E>::sqrt(bg.y), M<E>::sqrt(bg.z)} * 0.75f);
        bg = {M<E>::pow(bg.x, 2.2f), M<E>::pow(bg.y, 2.2f), M<E>::pow(bg.z, 2.2f)};
        bg = bg * 10.0f;
        float falloff = M<E>::pow(rd.y, 6.0f);
        bg = bg * falloff;
        bg = mix3(V3{0.3f, 0.6f, 4.0f} * 0.05f, bg, M<E>::pow(rd.y, 0.03125f));
        r.bg = bg + sunDisk;
        r.alpha = sunDisk;
    }
    r.cosTheta = dot(rd, f.sunDir);  // :386
    r.hg = fmaxf(hgPhase<E>(r.cosTheta, 0.6f), 0.7f * hgPhase<E>(r.cosTheta, 0.99f - 0.1f));  // :407
    return r;
}

// Beer's law, in-scatter and the front-to-back blend of one accumulated sample (:455-464).
template <bool E>
__device__ __forceinline__ float shade(float trans, float accum, float dal, float lo, float rh, float cosTheta,
                                       float hg) {
    float beers = M<E>::exp(-dal);
    float beersMod = fmaxf(beers, 0.7f * M<E>::exp(-0.25f * dal));
    beers = mixf(beers, beersMod, -cosTheta * 0.5f + 0.5f);
    float inScatter = 0.09f + M<E>::pow(lo, remapClamped<E>(rh, 0.3f, 0.85f, 0.5f, 2.0f));
    inScatter *= M<E>::pow(remapClamped<E>(rh, 0.07f, 0.34f, 0.1f, 1.0f), 0.8f);
    return mixf(trans, inScatter * hg * beers, 1.0f - accum);
}

// The blend target inScatter * HG * beersLaw of one accumulated sample (:455-464), the term shade
// mixes in; the same operations in the same order, so mixf(trans, shade_term(...), 1 - accum)
// equals shade(...).
template <bool E>
__device__ __forceinline__ float shade_term(float dal, float lo, float rh, float cosTheta, float hg) {
    float beers = M<E>::exp(-dal);
    float beersMod = fmaxf(beers, 0.7f * M<E>::exp(-0.25f * dal));
    beers = mixf(beers, beersMod, -cosTheta * 0.5f + 0.5f);
    float inScatter = 0.09f + M<E>::pow(lo, remapClamped<E>(rh, 0.3f, 0.85f, 0.5f, 2.0f));
    inScatter *= M<E>::pow(remapClamped<E>(rh, 0.07f, 0.34f, 0.1f, 1.0f), 0.8f);
    return inScatter * hg * beers;
}

// End of main() (:484-499): horizon fade, cloud colour, composite.
template <bool E>
__device__ __forceinline__ float4 composite(const mm_uniforms& u, const Frame& f, V3 rd, V3 bg, float alpha,
                                            float accum, float transmittance) {
    accum *= smoothstep<E>(0.0f, 1.0f, fminf(1.0f, remap<E>(rd.y, 0.0f, 0.1f, 0.0f, 1.0f)));
    accum = fminf(accum, 0.999f);
    const V3 sunColor = ld3(u.sun.color);
    const float I = u.sun.intensity;
    const float et = M<E>::exp(-transmittance);
    const float a = I * fmaxf(0.0f, transmittance);
    V3 cloud;
    if (f.sunY >= 0.0f) {
        cloud = sunColor * (V3{a, a, a} + (0.08f * bg) * et);
    } else {
        V3 night = V3{0.3f, 0.6f, 4.0f} * 0.05f * M<E>::pow(rd.y, 0.03125f);
        cloud = sunColor * (V3{a, a, a} + (0.08f * night) * et);
    }
    V3 rgb = mix3(bg, cloud, accum);
    return make_float4(rgb.x, rgb.y, rgb.z, alpha * fmaxf(1.0f - accum, 0.0f));
}

__device__ __forceinline__ void store_pixel(const MarchLaunch& p, int px, int py, float4 c, float depth) {
    float4* out = reinterpret_cast<float4*>(reinterpret_cast<char*>(p.rgba) + (size_t)py * p.rgba_pitch) + px;
    *out = c;
    if (p.depth) *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.depth) + (size_t)py * p.depth_pitch) + px) = depth;
}

struct Work {
    unsigned long long test = 0, hires = 0, iter = 0, acc = 0;
};

// Adds a thread's work counts to the launch totals: summed over the warp's active lanes first (one
// ray's counts fit 32 bits), then one atomic per counter from the lowest active lane.
__device__ __forceinline__ void flush_work(unsigned long long* cnt, const Work& w) {
    if (!cnt) return;
    const unsigned mask = __activemask();
    const unsigned t = __reduce_add_sync(mask, (unsigned)w.test), h = __reduce_add_sync(mask, (unsigned)w.hires);
    const unsigned i = __reduce_add_sync(mask, (unsigned)w.iter), a = __reduce_add_sync(mask, (unsigned)w.acc);
    if ((threadIdx.x & 31) == (unsigned)(__ffs(mask) - 1)) {
        atomicAdd(cnt + 0, (unsigned long long)t);
        atomicAdd(cnt + 1, (unsigned long long)h);
        atomicAdd(cnt + 2, (unsigned long long)i);
        atomicAdd(cnt + 3, (unsigned long long)a);
    }
}

// ------------------------------------------------------------------------------ tiled kernel

// The whole of main() (:288-500) for pixel (px, py) in one thread, the shader's own loop structure.
// G = cone taps whose fetches are issued together (the densities are still added in tap order);
// SC = in small-step mode, issue the sample's curl fetch with its cloudTest fetches (speculative:
// used only if the sample has density).
// PC = cone offsets from the launch parameters with the cone loop unrolled (see cone_offset).
// ------------------------------------------------------------------------------ large-step pairs
//
// Production arithmetic only.  While the ray marches in large steps (noHits), the loop body of
// sample t and of sample t + s (the next iteration's, reached if sample t has no density) are
// evaluated together: both samples' weather and low-res fetches are in flight at once.  Only the
// `density > 0` decision of a large step is used (:426), so with FP16 density textures (LP = 2)
// the two decisions are made in half2 arithmetic: the low-res texels are fetched as packed FP16
// (tex.3d.v2.f16x2), and the layer profile, remap, erosion and both thresholds run on (sample t,
// sample t + s) pairs; the coverage power stays FP32.  Transmittance, phase and in-scatter are
// not involved (large steps accumulate nothing).  LP = 1 makes the same two decisions in FP32 with
// the production cloudTest.

// Low-res texels of an FP16 texture at normalized p, filtered, as (R, G) and (B, A) half pairs.
__device__ __forceinline__ void tex3d_f16x2(cudaTextureObject_t t, V3 q, __half2& rg, __half2& ba) {
    unsigned a, b;
    asm volatile("tex.3d.v2.f16x2.f32 {%0, %1}, [%2, {%3, %4, %5, %5}];"
                 : "=r"(a), "=r"(b)
                 : "l"(t), "f"(q.x), "f"(q.y), "f"(q.z));
    rg = *reinterpret_cast<__half2*>(&a);
    ba = *reinterpret_cast<__half2*>(&b);
}

// The large-step decisions density > 0 of two samples (low half: the first) from their weather
// data, relative heights, coverage powers and low-res texels, in half2 (cloudTest, :231-253, with
// the production forms of march_kernel's test_finish).
__device__ __forceinline__ void decide_pair_h2(__half2 rg1, __half2 ba1, __half2 rg2, __half2 ba2, float rh1,
                                               float rh2, float type1, float type2, float cov1, float cov2, bool& d1,
                                               bool& d2) {
    const __half2 R = __lows2half2(rg1, rg2), Gc = __highs2half2(rg1, rg2);
    const __half2 B = __lows2half2(ba1, ba2), A = __highs2half2(ba1, ba2);
    const __half2 h = __floats2half2_rn(rh1, rh2), ty = __floats2half2_rn(type1, type2);
    const __half2 zero = __float2half2_rn(0.0f);
    const __half2 n = __hfma2_sat(R, __float2half2_rn(1.0f / 0.7f), __float2half2_rn(-0.3f / 0.7f));
    const __half2 cumulus = __hmax2(__hmul2(h, __hfma2(h, __float2half2_rn(-25.0f), __float2half2_rn(22.5f))), zero);
    const __half2 strato = __hmax2(__hmul2(h, __hfma2(h, __float2half2_rn(-10.0f), __float2half2_rn(7.0f))), zero);
    const __half2 stratus = __hmax2(__hmul2(h, __hfma2(h, __float2half2_rn(-100.0f), __float2half2_rn(30.0f))), zero);
    const __half2 a = __hmul2_sat(ty, __float2half2_rn(2.0f));
    const __half2 b = __hfma2_sat(ty, __float2half2_rn(2.0f), __float2half2_rn(-1.0f));
    const __half2 l1 = __hfma2(__hsub2(strato, stratus), a, stratus);
    const __half2 l2 = __hfma2(__hsub2(cumulus, strato), b, strato);
    const __half2 density = __hmul2(__hfma2(__hsub2(l2, l1), ty, l1), n);
    const __half2 cov = __floats2half2_rn(cov1, cov2);
    const __half2 ero = __hfma2(Gc, __float2half2_rn(0.625f),
                                __hfma2(B, __float2half2_rn(0.25f), __hmul2(A, __float2half2_rn(0.125f))));
    const __half2 erosion = __hmul2_sat(__hsub2(ero, cov), h2rcp(__hsub2(__float2half2_rn(1.0f), cov)));
    const __half2 yes = __hmul2(__hge2(density, __float2half2_rn(0.0001f)), __hgt2(density, erosion));
    d1 = __low2float(yes) > 0.5f;
    d2 = __high2float(yes) > 0.5f;
}

// The coverage power of cloudTest (:245, production form) for one sample.
__device__ __forceinline__ float coverage_fast(const Frame& f, float rh, float cov) {
    const float h = fminf(0.85f, cov + f.coverage_offset);
    const float e = clampf(1.0f - (h - 0.7f) * 2.0f, 0.8f, 1.0f);
    return exp2f(e * __log2f(rh));
}

template <int S, int LP>
__device__ __forceinline__ void large_pair(const MarchLaunch& p, const Frame& f, V3 rd, float t, float t2, bool two,
                                           bool& h1, bool& h2) {
    const Geo g1 = geo_at<false>(f, f.cam + t * rd);
    const Geo g2 = geo_at<false>(f, f.cam + t2 * rd);
    unsigned long long unused = 0;
    if constexpr (LP == 1) {
        const TestFetch c1 = test_fetch<false, S>(p, f, g1);
        TestFetch c2 = c1;
        if (two) c2 = test_fetch<false, S>(p, f, g2);
        h1 = test_finish<false>(f, g1, c1, unused) > 0.0f;
        h2 = two && test_finish<false>(f, g2, c2, unused) > 0.0f;
    } else {
        // weather (UNORM8, filtered to float) and the low-res texels (FP16, as half pairs)
        F4 w1, w2 = {0.0f, 0.0f, 0.0f, 0.0f};
        __half2 rg1, ba1, rg2 = __float2half2_rn(0.0f), ba2 = rg2;
        {
            const float rr = rsqrtf(dot(g1.d2, g1.d2));
            w1 = sample2d<false, S>(p.weather, 9.0f * rr * g1.d2.x, 9.0f * rr * g1.d2.z);
            tex3d_f16x2(p.low.tex, 0.00002f * g1.sp, rg1, ba1);
        }
        if (two) {
            const float rr = rsqrtf(dot(g2.d2, g2.d2));
            w2 = sample2d<false, S>(p.weather, 9.0f * rr * g2.d2.x, 9.0f * rr * g2.d2.z);
            tex3d_f16x2(p.low.tex, 0.00002f * g2.sp, rg2, ba2);
        }
        bool d1, d2;
        decide_pair_h2(rg1, ba1, rg2, ba2, g1.rh, g2.rh, w1.z, w2.z, coverage_fast(f, g1.rh, w1.x),
                       coverage_fast(f, g2.rh, w2.x), d1, d2);
        h1 = d1;
        h2 = two && d2;
    }
}

template <bool E, int S, int G = MM_CONE_GROUP, bool SC = (MM_SPEC_CURL != 0), bool PC = false, int LP = 0>
__device__ __forceinline__ void march_pixel(const MarchLaunch& p, const Frame& f, const V3* cone, int px, int py,
                                            Work& w) {
    const Ray r = ray_setup<E, S>(p, f, px, py);
    if (r.killed) {
        store_pixel(p, px, py, make_float4(r.bg.x, r.bg.y, r.bg.z, r.alpha), CUDART_INF_F);
        return;
    }
    const V3 rd = r.rd;
    float accum = 0.0f, transmittance = 1.0f;
    float stepSize = 0.05f * f.thickness;  // :390
    bool noHits = true;
    int misses = 0, steps = 0;
    float firstT = CUDART_INF_F;
    // :408-482, with an iteration cap (kMaxIterations) that no ray starting inside the shells
    // reaches; it bounds the loop for degenerate uniforms.
    int iterations = 0;
    for (float t = r.t0; t < r.t1 && iterations < kMaxIterations; t += stepSize, ++iterations) {
        ++w.iter;
        if constexpr (!E && LP > 0) {
            if (noHits) {
                // this sample and the next one, which the loop reaches if this one has no density
                const float t2 = t + stepSize;
                const bool two = t2 < r.t1 && iterations + 1 < kMaxIterations && steps < 100;
                bool h1, h2;
                large_pair<S, LP>(p, f, rd, t, t2, two, h1, h2);
                ++w.test;
                if (h1) {  // :428-434
                    misses = 0;
                    t -= stepSize;
                    stepSize *= 0.3f;
                    noHits = false;
                    continue;
                }
                if (++steps > 100) break;
                if (!two) continue;
                t = t2;  // the loop increment to the second sample
                ++iterations;
                ++w.iter;
                ++w.test;
                if (h2) {
                    misses = 0;
                    t -= stepSize;
                    stepSize *= 0.3f;
                    noHits = false;
                    continue;
                }
                if (++steps > 100) break;
                continue;
            }
        }
        const V3 pos = f.cam + t * rd;
        const Geo g = geo_at<E>(f, pos);
        // Once the ray marches in small steps, a sample that finds density goes on to cloudHiRes;
        // with SC its curl fetch is issued before the cloudTest fetches (and used after them), so a
        // sample with density waits two dependent fetch rounds instead of three.
        F4 cu;
        if (SC && !noHits) cu = curl_fetch<E, S>(p, g);
        float density = cloud_test<E, S>(p, f, g, w.test);
        const float loDensity = density;
        if (density > 0.0f) {
            misses = 0;
            if (noHits) {
                t -= stepSize;
                stepSize *= 0.3f;
                noHits = false;
                continue;
            }
            if (SC)
                density = hires_finish<E>(hires_fetch<E, S>(p, curl_displace<E>(g, stepSize, cu)), g.rh, density,
                                          w.hires);
            else
                density = cloud_hires<E, S>(p, g, stepSize, density, w.hires);
            if (density < 0.0001f) continue;
            float densityAlongLight = 0.0f;
            if constexpr (!E && PC) {
#pragma unroll
                for (int i = 0; i < 6; i += G)
                    densityAlongLight = cone_taps<E, S, G, true>(p, f, cone, i, pos, stepSize, densityAlongLight,
                                                                 w.test, w.hires);
            } else {
#pragma unroll 1
                for (int i = 0; i < 6; i += G)
                    densityAlongLight = cone_taps<E, S, G>(p, f, cone, i, pos, stepSize, densityAlongLight, w.test,
                                                           w.hires);
            }
            transmittance = shade<E>(transmittance, accum, densityAlongLight, loDensity, g.rh, r.cosTheta, r.hg);
            ++w.acc;
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
    store_pixel(p, px, py, composite<E>(p.u, f, r.rd, r.bg, r.alpha, accum, transmittance), firstT);
}


// Ray-tile order: each warp marches a kWarpTileW x (32 / kWarpTileW) pixel sub-tile (8x4 by
// default), so one warp's 32 rays are a compact footprint in the density textures; the warps of a
// block sit side by side across a block tile kBlockTileW wide (16 pixels for 4 warps, 32 for 8, or
// one warp tile if that is wider) and stack down it.
#ifndef MM_WARP_TILE_W
#define MM_WARP_TILE_W 8
#endif
constexpr int kWarpTileW = MM_WARP_TILE_W;
constexpr int kWarpTileH = 32 / kWarpTileW;
static_assert(kWarpTileW == 4 || kWarpTileW == 8 || kWarpTileW == 16 || kWarpTileW == 32, "warp tile width");
constexpr int kBlockTileW = (MM_TILED_WARPS == 8 ? 32 : 16) > kWarpTileW ? (MM_TILED_WARPS == 8 ? 32 : 16) : kWarpTileW;
constexpr int kWarpsAcross = kBlockTileW / kWarpTileW;
constexpr int kBlockTileH = kWarpTileH * (MM_TILED_WARPS / kWarpsAcross);

// Pixel (before the 1/16-phase mapping) of a lane of a warp in block tile (bx, by).
__device__ __forceinline__ int tile_px(int bx, int warp, int lane) {
    return bx * kBlockTileW + (warp % kWarpsAcross) * kWarpTileW + lane % kWarpTileW;
}
__device__ __forceinline__ int tile_py(int by, int warp, int lane) {
    return by * kBlockTileH + (warp / kWarpsAcross) * kWarpTileH + lane / kWarpTileW;
}

// Three variants of the same march, chosen per launch:
//  - full frames: one cone tap at a time (G = 1) keeps registers low enough for 10 blocks per SM,
//    and the texture unit is kept busy by the many warps;
//  - launches of at most kLatencyRays rays (a 1920x1080 frame at 1/16 of its pixels, or a small
//    image): such a launch is bounded below by the latency of its longest rays (a few hundred
//    dependent samples just above the horizon, ~0.5 ms on GB300 whatever the launch size), so all
//    six sun-cone taps of a sample are issued together (G = 6: a sample's cone takes 3 dependent
//    fetch rounds instead of up to 18) at 3 blocks per SM for the registers;
//  - larger 1/16-pixel launches (3840x2160/16: several waves): cone taps in threes (G = 3, 6 blocks).
// Measured over the 16-frame sweep (mean of frames 0, 5, 10, 15; production units built with
// denormals flushed): 1920x1080/16 0.48 ms (G = 6); 3840x2160/16 0.68 (G = 1, 10 blocks), 0.56
// (G = 2, 7 or 8 blocks), 0.53 (G = 3, 6 blocks), 0.54 / 0.56 (G = 3, 5 / 7 blocks), 0.60 / 0.67
// (G = 6, 4 / 3 blocks).  Both small-launch variants issue a small-step sample's curl fetch ahead of
// its cloudTest fetches (SC): the longest rays are chains of small-step samples whose density is then
// eroded away by cloudHiRes (~170 of their ~700 dependent fetch rounds), and SC takes one round out
// of each: 1920x1080/16 0.35 -> 0.32 ms, 3840x2160/16 0.42 -> 0.41 ms.  Full frames, bound by
// throughput, lose by the wasted fetches (3.24 -> 3.28 ms) and keep it off.
#ifndef MM_TILED_PARAM_CONE
#define MM_TILED_PARAM_CONE 0  // full frames: cone offsets from the launch parameters, cone loop unrolled
#endif
#ifndef MM_PHASE16_CONE_GROUP
#define MM_PHASE16_CONE_GROUP 3
#endif
#ifndef MM_PHASE16_MIN_BLOCKS
#define MM_PHASE16_MIN_BLOCKS 6
#endif
#ifndef MM_PHASE16_SPEC_CURL
#define MM_PHASE16_SPEC_CURL 1
#endif
#ifndef MM_LATENCY_SPEC_CURL
#define MM_LATENCY_SPEC_CURL 1
#endif
#ifndef MM_LATENCY_MIN_BLOCKS
#define MM_LATENCY_MIN_BLOCKS 3
#endif

#ifndef MM_LATENCY_RAYS
#define MM_LATENCY_RAYS 262144
#endif
constexpr long long kLatencyRays = MM_LATENCY_RAYS;
#ifndef MM_LATENCY_SCHEDULE
#define MM_LATENCY_SCHEDULE 1  // launches of at most kLatencyRays rays: 1 = team march, 0 = one thread per ray
#endif

template <bool E, int S, bool C, int G, bool SC, bool PC = false, int LP = 0>
__device__ __forceinline__ void march_tiled_body(const MarchLaunch& p) {
    __shared__ V3 s_cone[6];
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int by = (int)blockIdx.y < p.row_split ? p.row_split - 1 - (int)blockIdx.y : (int)blockIdx.y;
    const int tx = tile_px((int)blockIdx.x, warp, lane);
    const int ty = tile_py(by, warp, lane);
    int px, py;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {  // :292-298 (thread grid covers ceil(W/4) x ceil(H/4))
        px = tx * 4 + (p.phase % 4);
        py = ty * 4 + (p.phase / 4);
    } else {
        px = tx;
        py = ty;
    }
    if (px >= p.width || py >= p.height) return;  // :301 with the runtime image size
    const Frame f = make_frame<E>(p);
    Work w;  // work counts; dead code unless C (counters requested)
    march_pixel<E, S, G, SC, PC, LP>(p, f, s_cone, px, py, w);
    if (C) flush_work(p.counters, w);
}

// ------------------------------------------------------------------------------ deferred sun cones
//
// Full frames.  The sun cone of an accumulated sample (:441-453) changes only the light term
// (`transmittance`, :462), never the march: the loop's path, `accum` and `firstT` depend on the
// density alone.  So a lane that accumulates a sample appends a record of it -- t, step size, low-res
// density, `accum` before the sample, its lane -- to its warp's FIFO pool in shared memory and marches
// on.  One warp reduction per iteration counts the appends and the rays still marching; once the pool
// holds 32 records the warp computes the 32 oldest cones at once, one record per lane, every lane
// taking part (helpers included: rays that have ended, rays below the horizon, pixels outside the
// image).  Each lane writes its record's blend target inScatter * HG * beers (:455-460) back into the
// pool, and each owner then blends its records of the round into its transmittance in pool order,
// which is its accumulation order, with the sample's own `accum` (:462).  Clouds are coherent, so 19
// of 32 lanes on average accumulate in an iteration in which any does (3840x2160 sweep frame 3, oracle
// trace): the inline cone runs with those lanes while the rest wait; pooled records fill ~92% of the
// lanes.  A record's position and relative height are recomputed from t and the owner's ray by the
// march's own expressions, and the owners' masks of a round reuse the round's slots, so the pool takes
// 4.4 KB a block.  Shared memory is taken from the L1 that caches the textures: with 28-byte records
// (8 KB a block) the 1920x1080 sweep took 1.071 ms, with these 1.012 (inline cone: 1.074; both before
// the per-iteration count became one reduction).  Every sample, tap and blend is the shader's
// arithmetic in its order per ray, so results and work counts equal the one-thread march bit for bit
// in exact mode.
constexpr int kPool = 64;  // records per warp: < 32 after a round, + at most 32 per iteration
// Cone taps a lane of a round issues together (1, 2, 3 or 6).  3840x2160 / 1920x1080 sweeps: one at
// a time 3.215 / 0.992 ms; in pairs 3.347 / 1.036 (spills at 48 registers), 3.328 / 1.025 at 9 blocks
// per SM; in threes 3.819 / 1.186.
#ifndef MM_POOL_CONE_GROUP
#define MM_POOL_CONE_GROUP 1
#endif
// Production rounds: the six cone offsets from the launch parameters (computed on the host) with the
// tap loop unrolled (1), or from the block's shared copy with the loop rolled (0).  3840x2160 /
// 1920x1080 sweeps: 3.184 / 0.986 ms against 3.212 / 0.992 (fewer spills: 64 B against 72 B).
#ifndef MM_POOL_PARAM_CONE
#define MM_POOL_PARAM_CONE 1
#endif
// 1/16-pixel launches above kLatencyRays rays: pooled cones (1) or the inline kernel with cone taps in
// threes at 6 blocks per SM (0).  3840x2160 at 1/16, sweep frames 0/5/10/15: 0.361 against 0.412 ms.
#ifndef MM_PHASE16_POOL
#define MM_PHASE16_POOL 1
#endif
// The team march's one-thread rows: pooled cones (1) or inline cone taps in threes (0).  1920x1080 at
// 1/16, sweep mean: 0.256 ms pooled against 0.247 (the launch is bound by its longest rays, which the
// teams march; the pool's rounds only add latency to the others).
#ifndef MM_HYBRID_POOL
#define MM_HYBRID_POOL 0
#endif
struct ConePool {
    float t[MM_TILED_WARPS][kPool], step[MM_TILED_WARPS][kPool], acc[MM_TILED_WARPS][kPool];
    union {
        float lo;       // the record's low-res density
        unsigned mask;  // during a round, at slot head + o: the round's lanes holding owner o's records
    } lm[MM_TILED_WARPS][kPool];
    unsigned char own[MM_TILED_WARPS][kPool];
    int tail[MM_TILED_WARPS];  // records appended so far (slot = index mod kPool)
};

// One round: the `take` (<= 32) oldest records of the warp's pool, one per lane, then each owner's
// blends in pool order.  Every lane of the warp calls it with the same head and take.
template <bool E, int S>
__device__ __forceinline__ void cone_round(const MarchLaunch& p, const Frame& f, const V3* cone, ConePool& q,
                                           int head, int take, V3 rd, float& trans, float cosTheta, float hg,
                                           Work& w) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    __syncwarp();  // the appended records are visible to the warp
    const bool work = lane < take;
    const int slot = (head + lane) & (kPool - 1);
    const int o = work ? (int)q.own[wp][slot] : 32 + lane;  // idle lanes: a value no owner has
    const int src = o & 31;
    const float rx = __shfl_sync(full, rd.x, src), ry = __shfl_sync(full, rd.y, src);
    const float rz = __shfl_sync(full, rd.z, src);
    const float cosO = __shfl_sync(full, cosTheta, src), hgO = __shfl_sync(full, hg, src);
    if (work) {
        const float t = q.t[wp][slot], stepSize = q.step[wp][slot];
        const V3 pos = f.cam + t * V3{rx, ry, rz};  // the march's own expressions for this sample
        const float rh = geo_at<E>(f, pos).rh;
        float dal = 0.0f;
        if constexpr (!E && MM_POOL_PARAM_CONE) {
#pragma unroll
            for (int i = 0; i < 6; i += MM_POOL_CONE_GROUP)
                dal = cone_taps<E, S, MM_POOL_CONE_GROUP, true>(p, f, cone, i, pos, stepSize, dal, w.test, w.hires);
        } else {
#pragma unroll 1
            for (int i = 0; i < 6; i += MM_POOL_CONE_GROUP)
                dal = cone_taps<E, S, MM_POOL_CONE_GROUP>(p, f, cone, i, pos, stepSize, dal, w.test, w.hires);
        }
        q.t[wp][slot] = shade_term<E>(dal, q.lm[wp][slot].lo, rh, cosO, hgO);
    }
    q.lm[wp][slot].mask = 0u;  // this lane's slot of the round: read above (if it held a record)
    const unsigned same = __match_any_sync(full, o);
    __syncwarp();
    if (work && lane == __ffs(same) - 1) q.lm[wp][(head + o) & (kPool - 1)].mask = same;
    __syncwarp();
    unsigned mine = q.lm[wp][slot].mask;
    while (mine) {  // :462, in accumulation order
        const int sl = (head + __ffs(mine) - 1) & (kPool - 1);
        mine &= mine - 1u;
        trans = mixf(trans, q.t[wp][sl], 1.0f - q.acc[wp][sl]);
    }
    __syncwarp();  // the round's slots are read before later appends reuse them
}

// The march of pixel (px, py) with deferred sun cones (inside = false: no pixel, a helper lane).
template <bool E, int S, bool SC>
__device__ __forceinline__ void march_pixel_q(const MarchLaunch& p, const Frame& f, const V3* cone, ConePool& q,
                                              int px, int py, bool inside, Work& w) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
    Ray r{};
    bool live = false;
    if (inside) {
        r = ray_setup<E, S>(p, f, px, py);
        if (r.killed)
            store_pixel(p, px, py, make_float4(r.bg.x, r.bg.y, r.bg.z, r.alpha), CUDART_INF_F);
        else
            live = true;
    }
    if (lane == 0) q.tail[wp] = 0;
    float accum = 0.0f, trans = 1.0f;
    float stepSize = 0.05f * f.thickness;  // :390
    bool noHits = true;
    int misses = 0, steps = 0, iterations = 0;
    int head = 0, pending = 0;  // records of the warp's pool consumed / waiting (the same in every lane)
    float firstT = CUDART_INF_F;
    float t = r.t0;
    bool alive = live && t < r.t1;  // :408, the loop condition on entry
    __syncwarp();
    for (;;) {
        bool pushed = false;
        if (alive) {  // one iteration of :408-482
            ++w.iter;
            bool next = true;  // false: the loop ends here (no increment)
            const V3 pos = f.cam + t * r.rd;
            const Geo g = geo_at<E>(f, pos);
            F4 cu;
            if (SC && !noHits) cu = curl_fetch<E, S>(p, g);
            float density = cloud_test<E, S>(p, f, g, w.test);
            const float loDensity = density;
            do {  // `break` = the shader's `continue`
                if (density > 0.0f) {
                    misses = 0;
                    if (noHits) {  // :428-434
                        t -= stepSize;
                        stepSize *= 0.3f;
                        noHits = false;
                        break;
                    }
                    if (SC)
                        density = hires_finish<E>(hires_fetch<E, S>(p, curl_displace<E>(g, stepSize, cu)), g.rh,
                                                  density, w.hires);
                    else
                        density = cloud_hires<E, S>(p, g, stepSize, density, w.hires);
                    if (density < 0.0001f) break;
                    // the cone and blend of this sample (:441-462) come later; an owner's records
                    // take increasing slots, so the pool keeps each ray's order
                    const int slot = atomicAdd(&q.tail[wp], 1) & (kPool - 1);
                    q.t[wp][slot] = t;
                    q.step[wp][slot] = stepSize;
                    q.lm[wp][slot].lo = loDensity;
                    q.acc[wp][slot] = accum;
                    q.own[wp][slot] = (unsigned char)lane;
                    pushed = true;
                    ++w.acc;
                    if (firstT == CUDART_INF_F) firstT = t;
                    accum += density;
                } else if (!noHits) {  // :468-474
                    misses++;
                    if (misses >= 10) {
                        noHits = true;
                        stepSize = M<E>::div(stepSize, 0.3f);
                    }
                }
                if (accum > 0.99f) {
                    accum = 1.0f;
                    next = false;
                    break;
                }
                if (++steps > 100) next = false;
            } while (false);
            if (next) {
                t += stepSize;
                ++iterations;
                alive = t < r.t1 && iterations < kMaxIterations;
            } else {
                alive = false;
            }
        }
        // one reduction gives the records appended (low 6 bits) and the rays still marching (x 64)
        const unsigned sum = __reduce_add_sync(full, (pushed ? 1u : 0u) + (alive ? 64u : 0u));
        pending += (int)(sum & 63u);
        if (pending >= 32) {  // < 64 records: < 32 after a round, at most 32 appended since
            cone_round<E, S>(p, f, cone, q, head, 32, r.rd, trans, r.cosTheta, r.hg, w);
            head += 32;
            pending -= 32;
        }
        if (sum < 64u) break;
    }
    if (pending > 0) cone_round<E, S>(p, f, cone, q, head, pending, r.rd, trans, r.cosTheta, r.hg, w);
    if (live) store_pixel(p, px, py, composite<E>(p.u, f, r.rd, r.bg, r.alpha, accum, trans), firstT);
}

template <bool E, int S, bool C, bool SC>
__device__ __forceinline__ void march_tiled_q_body(const MarchLaunch& p) {
    __shared__ V3 s_cone[6];
    __shared__ ConePool s_q;
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int by = (int)blockIdx.y < p.row_split ? p.row_split - 1 - (int)blockIdx.y : (int)blockIdx.y;
    const int tx = tile_px((int)blockIdx.x, warp, lane);
    const int ty = tile_py(by, warp, lane);
    int px = tx, py = ty;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {  // :292-298
        px = tx * 4 + (p.phase % 4);
        py = ty * 4 + (p.phase / 4);
    }
    const Frame f = make_frame<E>(p);
    Work w;
    march_pixel_q<E, S, SC>(p, f, s_cone, s_q, px, py, px < p.width && py < p.height, w);
    if (C) flush_work(p.counters, w);
}

#ifndef MM_POOL_CARVEOUT_PCT
#define MM_POOL_CARVEOUT_PCT 20  // carveout preference of the pooled kernel, percent (0: computed)
#endif
#ifndef MM_MARCH_CARVEOUT
#define MM_MARCH_CARVEOUT 1  // pooled cones: request the smallest shared-memory carveout (the rest is L1)
#endif
#ifndef MM_CONE_POOL
#define MM_CONE_POOL 1  // full frames: sun cones pooled per warp (1) or each lane's inline cone (0)
#endif

#ifndef MM_LARGE_PAIR
// Full frames: large steps in pairs with FP32 decisions (1) or one at a time (0).  Measured on the
// 4K sweep: 3.367 ms in pairs against 3.240 one at a time (the lanes of a warp fall out of step).
#define MM_LARGE_PAIR 0
#endif
#ifndef MM_PAIR_MIN_BLOCKS
#define MM_PAIR_MIN_BLOCKS MM_MARCH_MIN_BLOCKS
#endif

template <bool E, int S, bool C>
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_MARCH_MIN_BLOCKS) march_tiled_kernel(MarchLaunch p) {
    march_tiled_body<E, S, C, MM_CONE_GROUP, (MM_SPEC_CURL != 0), (MM_TILED_PARAM_CONE != 0),
                     (E || S != MM_SAMPLER_HARDWARE) ? 0 : MM_LARGE_PAIR>(p);
}

// Full frames with deferred, pooled sun cones (above).
template <bool E, int S, bool C>
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_MARCH_MIN_BLOCKS) march_tiled_pool_kernel(MarchLaunch p) {
    march_tiled_q_body<E, S, C, (MM_SPEC_CURL != 0)>(p);
}

// Full frames with FP16 (or BF16) density textures under MM_MATH_FAST_HALF2: large-step decisions
// in half2 on packed FP16 texels (the hardware sampler only).
template <bool C>
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_PAIR_MIN_BLOCKS) march_tiled_h2_kernel(MarchLaunch p) {
    march_tiled_body<false, MM_SAMPLER_HARDWARE, C, MM_CONE_GROUP, (MM_SPEC_CURL != 0), (MM_TILED_PARAM_CONE != 0), 2>(p);
}

template <bool E, int S, bool C>
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_PHASE16_MIN_BLOCKS) march_tiled_phase16_kernel(MarchLaunch p) {
    march_tiled_body<E, S, C, MM_PHASE16_CONE_GROUP, (MM_PHASE16_SPEC_CURL != 0), true>(p);
}

template <bool E, int S, bool C>
__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_LATENCY_MIN_BLOCKS) march_tiled_latency_kernel(MarchLaunch p) {
    march_tiled_body<E, S, C, 6, (MM_LATENCY_SPEC_CURL != 0), true>(p);
}

// ------------------------------------------------------------------------------ team march
//
// Launches of few rays (a 1920x1080 frame at 1/16 of its pixels) are bound by the chain of
// dependent texture fetches of their longest rays: a ray just above the horizon takes ~60 large
// steps, ~200 small steps and ~170 cloudHiRes calls, one after another.  Here a team of kTeam
// lanes marches one ray.  In a round, member j evaluates the sample the shader's loop would
// reach j iterations later if nothing changed the step size or the mode: position t + s + ... + s
// (j additions, as the loop's increments make it), its cloudTest, and in small-step mode its
// cloudHiRes, sun cone and shading term where the shader would compute them.  The team then runs
// the loop body (:408-482) sample by sample in order on the shuffled results, every member the
// same state; a step back (:426-434) or a return to large steps (:468-474) changes the step size,
// so the rest of the round is dropped and the next round starts where the loop goes on.  Every
// consumed sample is the computation the sequential loop does, in the same arithmetic, so the
// output (and the work counts, which count consumed samples only) equals the one-thread march.
#ifndef MM_TEAM_LANES
#define MM_TEAM_LANES 4
#endif
#ifndef MM_TEAM_MIN_BLOCKS
#define MM_TEAM_MIN_BLOCKS 4
#endif
// Cone taps a team member issues together (6 or 3).  1920x1080/16 sweep mean, 256x256: taps in
// sixes at 4 blocks/SM (127 registers) 0.247 / 0.160 ms; in threes at 5 / 6 / 8 blocks/SM 0.256 /
// 0.282 / 0.321 and 0.163 / 0.179 / 0.189; sixes at 5 blocks/SM (96 registers) 0.256 / 0.169.
#ifndef MM_TEAM_CONE_GROUP
#define MM_TEAM_CONE_GROUP 6
#endif
constexpr int kTeam = MM_TEAM_LANES;
static_assert(kTeam == 4 || kTeam == 8, "team size");
// Rays of a warp (32 / kTeam) as a 2x2 (teams of 8) or 4x2 (teams of 4) pixel tile; the four warps
// of a block side by side in a 2x2 arrangement.
constexpr int kTeamWarpW = kTeam == 8 ? 2 : 4, kTeamWarpH = 2;
constexpr int kTeamBlockW = 2 * kTeamWarpW, kTeamBlockH = 2 * kTeamWarpH;

// One ray marched by the calling team (member `member` of the kTeam lanes at `base` of the warp).
template <bool E, int S, bool C>
__device__ __forceinline__ void team_ray(const MarchLaunch& p, const Frame& f, const V3* s_cone, int px, int py,
                                         int member, int base, unsigned tmask) {
    Work w;
    const Ray r = ray_setup<E, S>(p, f, px, py);
    if (r.killed) {
        if (member == 0) store_pixel(p, px, py, make_float4(r.bg.x, r.bg.y, r.bg.z, r.alpha), CUDART_INF_F);
        return;
    }
    const V3 rd = r.rd;
    float accum = 0.0f, transmittance = 1.0f;
    float stepSize = 0.05f * f.thickness;  // :390
    bool noHits = true;
    int misses = 0, steps = 0, iterations = 0;
    float firstT = CUDART_INF_F;
    float t = r.t0;
    bool done = false;
    while (!done) {
        // ---- this member's sample of the round
        float tj = t;
        for (int k = 0; k < member; ++k) tj += stepSize;
        const bool valid = tj < r.t1 && iterations + member < kMaxIterations;
        float lo = 0.0f, hi = 0.0f, y = 0.0f;
        unsigned long long nt = 0, nh = 0;
        if (valid) {
            const V3 pos = f.cam + tj * rd;
            const Geo g = geo_at<E>(f, pos);
            F4 cu;
            if (!noHits) cu = curl_fetch<E, S>(p, g);  // issued with the cloudTest fetches
            lo = cloud_test<E, S>(p, f, g, nt);
            if (!noHits && lo > 0.0f) {
                hi = hires_finish<E>(hires_fetch<E, S>(p, curl_displace<E>(g, stepSize, cu)), g.rh, lo, nh);
                if (hi >= 0.0001f) {
                    float dal = 0.0f;
#pragma unroll
                    for (int i = 0; i < 6; i += MM_TEAM_CONE_GROUP)
                        dal = cone_taps<E, S, MM_TEAM_CONE_GROUP, true>(p, f, s_cone, i, pos, stepSize, dal, nt, nh);
                    y = shade_term<E>(dal, lo, g.rh, r.cosTheta, r.hg);
                }
            }
        }
        // ---- the loop body (:408-482) on the round's samples, in order
#pragma unroll 1
        for (int i = 0; i < kTeam; ++i) {
            const bool vi = __shfl_sync(tmask, valid, base + i);
            if (!vi) {  // the loop condition fails at this iteration: the ray is finished
                done = true;
                break;
            }
            const float li = __shfl_sync(tmask, lo, base + i);
            const float hiv = __shfl_sync(tmask, hi, base + i);
            const float yi = __shfl_sync(tmask, y, base + i);
            if (C) {
                w.test += (unsigned)__shfl_sync(tmask, (unsigned)nt, base + i);
                w.hires += (unsigned)__shfl_sync(tmask, (unsigned)nh, base + i);
            }
            ++w.iter;
            bool restart = false;
            if (li > 0.0f) {
                misses = 0;
                if (noHits) {  // :428-434: back half a step, small steps from here
                    t -= stepSize;
                    stepSize *= 0.3f;
                    noHits = false;
                    restart = true;
                } else if (hiv >= 0.0001f) {  // :437-466
                    transmittance = mixf(transmittance, yi, 1.0f - accum);
                    ++w.acc;
                    if (firstT == CUDART_INF_F) firstT = t;
                    accum += hiv;
                    if (accum > 0.99f) {  // :476-479
                        accum = 1.0f;
                        done = true;
                        break;
                    }
                    if (++steps > 100) {
                        done = true;
                        break;
                    }
                }
            } else {
                if (!noHits) {  // :468-474
                    misses++;
                    if (misses >= 10) {
                        noHits = true;
                        stepSize = M<E>::div(stepSize, 0.3f);
                        restart = true;
                    }
                }
                if (++steps > 100) {  // :481
                    done = true;
                    break;
                }
            }
            t += stepSize;  // the loop increment (:408), also after a `continue`
            ++iterations;
            if (restart) break;
        }
    }
    if (member == 0) {
        store_pixel(p, px, py, composite<E>(p.u, f, r.rd, r.bg, r.alpha, accum, transmittance), firstT);
        if (C) flush_work(p.counters, w);
    }
}

// Band of ray rows marched by teams, the rest one thread per ray, in one launch: the first
// team_blocks blocks march kTeamBlockW x kTeamBlockH ray tiles of the band [band0, band1) from its
// bottom row (the horizon) up, the others 16 x 8 tiles of the rows above the band (nearest first)
// and then of the rows below it (rays under the horizon, which end at once).
struct HybridGrid {
    int team_bx, team_blocks;  // team tiles per band row, team blocks in all
    int band0, band1;          // ray rows [band0, band1), multiples of 8
    int single_bx;             // 16-wide tiles per row
    int rows_above;            // 8-row block rows above the band
};

template <bool E, int S, bool C>
__global__ void __launch_bounds__(128, MM_TEAM_MIN_BLOCKS) march_hybrid_kernel(MarchLaunch p, HybridGrid hg) {
    __shared__ V3 s_cone[6];
#if MM_HYBRID_POOL
    __shared__ ConePool s_q;
#endif
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int tx, ty;
    const bool team_block = (int)blockIdx.x < hg.team_blocks;
    if (team_block) {
        const int bx = (int)blockIdx.x % hg.team_bx, byr = (int)blockIdx.x / hg.team_bx;
        const int team = lane / kTeam;
        tx = bx * kTeamBlockW + (warp & 1) * kTeamWarpW + team % kTeamWarpW;
        ty = hg.band1 - kTeamBlockH * (byr + 1) + (warp >> 1) * kTeamWarpH + team / kTeamWarpW;
    } else {
        const int idx = (int)blockIdx.x - hg.team_blocks;
        const int bx = idx % hg.single_bx, k = idx / hg.single_bx;
        const int row0 = k < hg.rows_above ? hg.band0 - 8 * (k + 1) : hg.band1 + 8 * (k - hg.rows_above);
        tx = bx * 16 + (warp & 1) * 8 + (lane & 7);
        ty = row0 + (warp >> 1) * 4 + (lane >> 3);
    }
    int px, py;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {  // :292-298
        px = tx * 4 + (p.phase % 4);
        py = ty * 4 + (p.phase / 4);
    } else {
        px = tx;
        py = ty;
    }
    const bool inside = px < p.width && py < p.height;
#if MM_HYBRID_POOL
    if (!team_block) {  // every lane of the warp stays: the pool's rounds need them all
        const Frame f = make_frame<E>(p);
        Work w;
        march_pixel_q<E, S, (MM_SPEC_CURL != 0)>(p, f, s_cone, s_q, px, py, inside, w);
        if (C) flush_work(p.counters, w);
        return;
    }
#endif
    if (!inside) return;  // a team leaves together: its lanes share (px, py)
    const Frame f = make_frame<E>(p);
    if (team_block) {
        const int team = lane / kTeam, base = team * kTeam;
        team_ray<E, S, C>(p, f, s_cone, px, py, lane % kTeam, base, ((1u << kTeam) - 1u) << base);
    } else {
        Work w;
        march_pixel<E, S, 3, true, true>(p, f, s_cone, px, py, w);
        if (C) flush_work(p.counters, w);
    }
}

// The band for a launch: ray rows whose rays rise at less than MM_TEAM_BAND_DEG degrees (the long
// ones: at 6 degrees a ray crosses ~190 km of the shell and hits the 100-step limit), widened to
// multiples of 8 rows and running down to the horizon; a launch of at most MM_TEAM_ALL_RAYS rays
// marches every row above the horizon by teams.  Empty for a camera with roll (right.y != 0: a
// row's rays then rise at different angles).  Measured over the 16-frame sweep on GB300, mean
// ms per launch, against 0.308 (1920x1080 at 1/16) and 0.312 (256x256) one thread per ray:
//   band 6 deg 0.246 / 0.224, 12 deg 0.264 / 0.193, 25 deg 0.261 / 0.175, every row 0.298 / 0.160.
// A launch of one wave or less gains from teams everywhere; in a larger one the teams' extra
// lanes cost more than they save on rays that are not the longest.
#ifndef MM_TEAM_BAND_DEG
#define MM_TEAM_BAND_DEG 6
#endif
#ifndef MM_TEAM_ALL_RAYS
#define MM_TEAM_ALL_RAYS 65536
#endif
inline HybridGrid hybrid_grid(const MarchLaunch& p, int gw, int gh) {
    HybridGrid g{};
    const int ghp = (gh + 7) / 8 * 8;
    int band0 = ghp, band1 = ghp;
    const float* v = p.u.camera.view;
    if (v[4] == 0.0f) {
        const double cpy = p.u.camera.camera_params[1];
        const double lx = v[2], ly = v[6], lz = v[10], ux = v[1], uy = v[5], uz = v[9];
        const double s_band = (long long)gw * gh <= MM_TEAM_ALL_RAYS
                                  ? 2.0
                                  : sin((double)MM_TEAM_BAND_DEG * 3.14159265358979323846 / 180.0);
        const bool phase16 = p.pixel_mode == MM_PIXELS_PHASE16;
        int first = -1, horizon = gh;
        for (int ty = 0; ty < gh; ++ty) {
            const int py = phase16 ? ty * 4 + p.phase / 4 : ty;
            const double sy = 2.0 * py / p.uv_h - 1.0;
            // centre-column ray direction (compute-clouds.comp:309-322): -look - sy * tan * up
            const double dx = -lx - sy * cpy * ux, dy = -ly - sy * cpy * uy, dz = -lz - sy * cpy * uz;
            const double sin_el = dy / sqrt(dx * dx + dy * dy + dz * dz);
            if (sin_el <= 0.0) {
                horizon = ty;
                break;
            }
            if (first < 0 && sin_el < s_band) first = ty;
        }
        if (first >= 0 && first < horizon) {
            band0 = first / 8 * 8;
            band1 = (horizon + 7) / 8 * 8;
            if (band1 > ghp) band1 = ghp;
        }
    }
    if (band0 >= band1) band0 = band1 = ghp;  // no band: every row one thread per ray
    g.band0 = band0;
    g.band1 = band1;
    g.team_bx = (gw + kTeamBlockW - 1) / kTeamBlockW;
    g.team_blocks = g.team_bx * ((band1 - band0) / kTeamBlockH);
    g.single_bx = (gw + 15) / 16;
    g.rows_above = band0 / 8;
    return g;
}

// Launch order of the block rows.  A ray's cost grows as it nears the horizon (it crosses more of
// the cloud shell: ~124 km at rd.y = 0 against 20 km straight up) and rays below it end at once,
// so the rows just above the horizon are the long ones.  Started last, they would form the tail of
// the launch (at 1/16 of a frame, a launch is only a few waves of rays).  For a camera without roll
// (right.y == 0, as mm_camera_from_angles makes) the ray's y component depends on the row only and
// falls monotonically down the image; the block rows whose centre ray rises are [0, split), and the
// kernel runs them from split - 1 (the horizon) upwards before the rest.  Any other camera keeps
// the launch order.  Only the order changes: every pixel is marched by the same code.
inline int horizon_row_split(const MarchLaunch& p, int block_rows, int rows_per_block = kBlockTileH) {
    const float* v = p.u.camera.view;
    if (v[4] != 0.0f) return 0;
    const float cpy = p.u.camera.camera_params[1];
    const bool phase16 = p.pixel_mode == MM_PIXELS_PHASE16;
    int split = 0;
    for (int r = 0; r < block_rows; ++r) {
        const int row = r * rows_per_block + rows_per_block / 2;
        const int py = phase16 ? row * 4 + p.phase / 4 : row;
        const float spy = 2.0f * (float)py / p.uv_h - 1.0f;
        if (-v[6] - spy * cpy * v[5] > 0.0f)
            split = r + 1;
        else
            break;
    }
    return split;
}

// Pooled cones or each lane's own (MM_CONE_POOL).  The pool pays more where the inline cone leaves more
// lanes idle: neighbouring rays of a warp tile are less alike where a pixel spans a larger angle
// (oracle trace, sweep frame 3: 15 of 32 lanes accumulate together at 1920x1080, 19 at 3840x2160).
// 16-frame sweep, 60 degree field of view, inline -> pooled: 1920x1080 1.074 -> 0.993 ms, 2880x1620
// 1.988 -> 1.924, 3200x1800 2.394 -> 2.338, 3840x2160 3.240 -> 3.212.

// The pooled kernel's shared memory is small (4.4 KB a block), and the rest of the SM's unified L1 is
// its texture cache.  Without a preference the driver gave it a 132 KB shared-memory carveout; the
// preference computed from its need (10 blocks x (4.4 + 1 KB reserved) = 23% of 228 KB) still got
// 100 KB, and 20% (or 12%) got 64 KB, which holds 11 blocks (6%: 32 KB, 5 blocks).  1920x1080, one
// sweep frame: L1 hit rate 88% / 91.4% / 93.0% at 132 / 100 / 64 KB (the inline kernel: 93.0% at its
// 32 KB); 16-frame sweep at 64 KB against 100 KB: 1920x1080 1.012 / 1.021 ms, 3840x2160 3.273 /
// 3.295.  So 20% is requested (MM_POOL_CARVEOUT_PCT = 0: the computed preference) when a context is
// created, outside any stream capture.  A hint only: a failure is cleared and ignored.
template <bool E, int S, bool C>
void pool_carveout() {
    if (!MM_MARCH_CARVEOUT) return;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return;
    }
    int per_sm = 0, reserved = 0;
    cudaFuncAttributes a{};
    if (cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) == cudaSuccess &&
        cudaFuncGetAttributes(&a, march_tiled_pool_kernel<E, S, C>) == cudaSuccess && per_sm > 0) {
        const long long need = (long long)MM_MARCH_MIN_BLOCKS * ((long long)a.sharedSizeBytes + reserved);
        int pct = MM_POOL_CARVEOUT_PCT > 0 ? MM_POOL_CARVEOUT_PCT : (int)((100 * need + per_sm - 1) / per_sm);
        pct = pct < 1 ? 1 : (pct > 100 ? 100 : pct);
        cudaFuncSetAttribute(march_tiled_pool_kernel<E, S, C>, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    }
    cudaGetLastError();
}

// Kernel attributes of this arithmetic's march kernels for the current device.
template <bool E>
void prepare_march_kernels() {
    pool_carveout<E, MM_SAMPLER_HARDWARE, false>();
    pool_carveout<E, MM_SAMPLER_HARDWARE, true>();
    pool_carveout<E, MM_SAMPLER_SOFTWARE, false>();
    pool_carveout<E, MM_SAMPLER_SOFTWARE, true>();
}

template <bool E, int S>
int launch_tiled(const MarchLaunch& p0, cudaStream_t s, bool half2 = false) {
    MarchLaunch p = p0;
    int gw = p.width, gh = p.height;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {
        gw = (p.width + 3) / 4;
        gh = (p.height + 3) / 4;
    }
    dim3 grid((gw + kBlockTileW - 1) / kBlockTileW, (gh + kBlockTileH - 1) / kBlockTileH);
    p.row_split = horizon_row_split(p, (int)grid.y);
    // Kernels that the build knobs leave unused are not instantiated (if constexpr).
    const bool C = p.counters != nullptr;
    const dim3 block(MM_TILED_WARPS * 32);
    if ((long long)gw * gh <= kLatencyRays) {
        if constexpr (MM_LATENCY_SCHEDULE == 1) {
            const HybridGrid hg = hybrid_grid(p, gw, gh);
            const int blocks =
                hg.team_blocks + hg.single_bx * (hg.rows_above + ((gh + 7) / 8 * 8 - hg.band1) / 8);
            if (C)
                march_hybrid_kernel<E, S, true><<<blocks, 128, 0, s>>>(p, hg);
            else
                march_hybrid_kernel<E, S, false><<<blocks, 128, 0, s>>>(p, hg);
        } else {
            if (C)
                march_tiled_latency_kernel<E, S, true><<<grid, block, 0, s>>>(p);
            else
                march_tiled_latency_kernel<E, S, false><<<grid, block, 0, s>>>(p);
        }
    } else if (p.pixel_mode == MM_PIXELS_PHASE16 && !MM_PHASE16_POOL) {
        if constexpr (!MM_PHASE16_POOL) {
            if (C)
                march_tiled_phase16_kernel<E, S, true><<<grid, block, 0, s>>>(p);
            else
                march_tiled_phase16_kernel<E, S, false><<<grid, block, 0, s>>>(p);
        }
    } else if (!E && S == MM_SAMPLER_HARDWARE && half2 && p.pixel_mode != MM_PIXELS_PHASE16) {
        if constexpr (!E && S == MM_SAMPLER_HARDWARE) {
            if (C)
                march_tiled_h2_kernel<true><<<grid, block, 0, s>>>(p);
            else
                march_tiled_h2_kernel<false><<<grid, block, 0, s>>>(p);
        }
    } else if (MM_CONE_POOL != 0 || p.pixel_mode == MM_PIXELS_PHASE16) {
        if (C)
            march_tiled_pool_kernel<E, S, true><<<grid, block, 0, s>>>(p);
        else
            march_tiled_pool_kernel<E, S, false><<<grid, block, 0, s>>>(p);
    } else {
        if constexpr (MM_CONE_POOL == 0) {
            if (C)
                march_tiled_kernel<E, S, true><<<grid, block, 0, s>>>(p);
            else
                march_tiled_kernel<E, S, false><<<grid, block, 0, s>>>(p);
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "march_tiled_kernel launch");
    count_launch();
    return MM_OK;
}

// ------------------------------------------------------------------------------ persistent kernel
//
// Each warp keeps 32 rays in flight.  One iteration of the loop below evaluates, for every lane,
// exactly one cloudTest (either the lane's next march step or its next sun-cone tap) and, where
// the shader would, one cloudHiRes; a lane whose ray ends stores it and takes the next ray of its
// warp's 8x4 pixel tile (ballot over the idle lanes), and a warp that has used up its tile takes
// the next tile from a global counter.  Every ray executes the same sequence of operations as in
// march_pixel; only the interleaving of rays on the SIMT lanes changes.

constexpr int kTileW = 8, kTileH = 4;
constexpr int kWarps = 8;  // warps per block of the persistent kernel


// A ray whose set-up is done, waiting in its warp's queue for an idle lane.
struct Pending {
    float rdx, rdy, rdz, bgx, bgy, bgz, alpha, t0, t1, cosTheta, hg;
    int pix;  // py * 65536 + px
};

template <bool E, int S, bool C>
__global__ void __launch_bounds__(256, MM_PERSISTENT_MIN_BLOCKS) march_persistent_kernel(MarchLaunch p, unsigned int* tile_counter, int tiles_x,
                                                               int n_tiles, int grid_w, int grid_h) {
    __shared__ V3 s_cone[6];
    __shared__ Pending s_queue[kWarps][32];
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const unsigned lane_id = threadIdx.x & 31;
    Pending* queue = s_queue[threadIdx.x >> 5];
    const Frame f = make_frame<E>(p);
    Work w;
    // Lane state of one ray (the locals of main() that live across loop iterations).
    int px = -1, py = 0;  // px < 0: no ray
    V3 rd, bg, pos;
    float alpha = 0.f, t = 0.f, t1 = 0.f, stepSize = 0.f, accum = 0.f, trans = 0.f, firstT = 0.f, cosTheta = 0.f,
          hg = 0.f, rh = 0.f, lo = 0.f, dens = 0.f, dal = 0.f;
    int misses = 0, steps = 0, iterations = 0, cone = -1;
    bool noHits = true;
    int queued = 0;          // warp-uniform: rays waiting in the queue (taken from the top)
    bool exhausted = false;  // warp-uniform: no tiles left

    while (true) {
        unsigned need = __ballot_sync(0xffffffffu, px < 0);
        // ---- the warp sets up the 32 rays of its next tile together, one per lane; rays that
        // leave the frame or point below the horizon (:351-354) are stored here and not queued.
        if (need && queued == 0 && !exhausted) {
            int tv = 0;
            if (lane_id == 0) tv = (int)atomicAdd(tile_counter, 1u);
            const int tile = __shfl_sync(0xffffffffu, tv, 0);
            if (tile >= n_tiles) {
                exhausted = true;
            } else {
                const int gx = (tile % tiles_x) * kTileW + (lane_id % kTileW);
                const int gy = (tile / tiles_x) * kTileH + (lane_id / kTileW);
                int qx = gx, qy = gy;
                if (p.pixel_mode == MM_PIXELS_PHASE16) {
                    qx = gx * 4 + (p.phase % 4);
                    qy = gy * 4 + (p.phase / 4);
                }
                bool live = false;
                Ray r;
                if (gx < grid_w && gy < grid_h && qx < p.width && qy < p.height) {
                    r = ray_setup<E, S>(p, f, qx, qy);
                    if (r.killed)
                        store_pixel(p, qx, qy, make_float4(r.bg.x, r.bg.y, r.bg.z, r.alpha), CUDART_INF_F);
                    else
                        live = true;
                }
                const unsigned lm = __ballot_sync(0xffffffffu, live);
                if (live) {
                    Pending& q = queue[__popc(lm & ((1u << lane_id) - 1u))];
                    q.rdx = r.rd.x; q.rdy = r.rd.y; q.rdz = r.rd.z;
                    q.bgx = r.bg.x; q.bgy = r.bg.y; q.bgz = r.bg.z;
                    q.alpha = r.alpha; q.t0 = r.t0; q.t1 = r.t1; q.cosTheta = r.cosTheta; q.hg = r.hg;
                    q.pix = qy * 65536 + qx;
                }
                queued = __popc(lm);
                __syncwarp();
            }
        }
        // ---- idle lanes take queued rays (ballot rank among the idle lanes)
        if (need && queued > 0) {
            const int rank = __popc(need & ((1u << lane_id) - 1u));
            const int take = min(__popc(need), queued);
            if (((need >> lane_id) & 1u) && rank < take) {
                const Pending& q = queue[queued - 1 - rank];
                px = q.pix & 65535;
                py = q.pix >> 16;
                rd = {q.rdx, q.rdy, q.rdz};
                bg = {q.bgx, q.bgy, q.bgz};
                alpha = q.alpha;
                t = q.t0;
                t1 = q.t1;
                cosTheta = q.cosTheta;
                hg = q.hg;
                stepSize = 0.05f * f.thickness;  // :390
                accum = 0.0f;
                trans = 1.0f;
                firstT = CUDART_INF_F;
                misses = steps = iterations = 0;
                noHits = true;
                cone = -1;
            }
            queued -= take;
            __syncwarp();
        }
        const unsigned active = __ballot_sync(0xffffffffu, px >= 0);
        if (active == 0) {
            if (exhausted) break;
            continue;  // every ray of the last tile was stored during set-up
        }
        if (px >= 0) {
            // ---- the loop condition of :408 for a lane about to take a march step
            bool done = cone < 0 && !(t < t1 && iterations < kMaxIterations);
            if (!done) {
                if (cone < 0) {
                    ++w.iter;
                    pos = f.cam + t * rd;
                }
                // march step: the point itself; cone tap i: pos + 3 stepSize samples[i] (:442)
                const V3 q = cone < 0 ? pos : pos + 3.0f * stepSize * s_cone[cone];
                const Geo g = geo_at<E>(f, q);
                if (cone < 0) rh = g.rh;
                const float d = cloud_test<E, S>(p, f, g, w.test);
                float h = 0.0f;
                if (d > 0.0f && (cone >= 0 || !noHits)) h = cloud_hires<E, S>(p, g, stepSize, d, w.hires);

                bool advance = false, post = false;
                if (cone < 0) {
                    lo = d;
                    if (d > 0.0f) {
                        misses = 0;
                        if (noHits) {  // :428-434
                            t -= stepSize;
                            stepSize *= 0.3f;
                            noHits = false;
                            advance = true;
                        } else if (h < 0.0001f) {  // :437
                            advance = true;
                        } else {
                            dens = h;
                            dal = 0.0f;
                            cone = 0;
                        }
                    } else {
                        if (!noHits) {  // :468-474
                            misses++;
                            if (misses >= 10) {
                                noHits = true;
                                stepSize = M<E>::div(stepSize, 0.3f);
                            }
                        }
                        post = true;
                    }
                } else {
                    if (d > 0.0f) dal += h;  // :449-452
                    if (++cone == 6) {       // :456-466
                        trans = shade<E>(trans, accum, dal, lo, rh, cosTheta, hg);
                        ++w.acc;
                        if (firstT == CUDART_INF_F) firstT = t;
                        accum += dens;
                        cone = -1;
                        post = true;
                    }
                }
                if (post) {  // :476-481
                    if (accum > 0.99f) {
                        accum = 1.0f;
                        done = true;
                    } else if (++steps > 100) {
                        done = true;
                    } else {
                        advance = true;
                    }
                }
                if (advance) {  // the for-loop increment
                    t += stepSize;
                    ++iterations;
                }
            }
            if (done) {
                store_pixel(p, px, py, composite<E>(p.u, f, rd, bg, alpha, accum, trans), firstT);
                px = -1;
            }
        }
    }
    if (C) flush_work(p.counters, w);
}

template <bool E, int S>
int launch_persistent(const MarchLaunch& p, unsigned int* d_counter, int num_sms, cudaStream_t s) {
    int gw = p.width, gh = p.height;
    if (p.pixel_mode == MM_PIXELS_PHASE16) {
        gw = (p.width + 3) / 4;
        gh = (p.height + 3) / 4;
    }
    const int tiles_x = (gw + kTileW - 1) / kTileW, tiles_y = (gh + kTileH - 1) / kTileH;
    const int n_tiles = tiles_x * tiles_y;
    static int per_sm = 0;
    if (per_sm == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, march_persistent_kernel<E, S, false>, 256, 0) !=
                cudaSuccess ||
            per_sm <= 0)
            per_sm = 1;
    }
    int blocks = num_sms * per_sm;
    if (blocks * kWarps > n_tiles) blocks = (n_tiles + kWarps - 1) / kWarps;
    if (blocks < 1) blocks = 1;
    cudaError_t e = cudaMemsetAsync(d_counter, 0, sizeof(unsigned int), s);
    if (e != cudaSuccess) return cuda_fail(e, "work counter reset");
    if (p.counters)
        march_persistent_kernel<E, S, true><<<blocks, 256, 0, s>>>(p, d_counter, tiles_x, n_tiles, gw, gh);
    else
        march_persistent_kernel<E, S, false><<<blocks, 256, 0, s>>>(p, d_counter, tiles_x, n_tiles, gw, gh);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "march_persistent_kernel launch");
    count_launch();
    return MM_OK;
}

}  // namespace march
}  // namespace mm

#endif  // MM_MARCH_KERNEL_CUH_
