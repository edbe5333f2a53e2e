// glsl_shim.h - lets the reference's GLSL shaders compile unchanged as C++ on glm (test
// infrastructure: builds the checker's reference, never the library).
//
// oracle/ref/glsl_to_cpp.py turns a shader into a C++ translation unit: it drops the three lines
// that are GLSL-only syntax (#version, #extension, precision), marks decimal literals as float
// (GLSL literals are single precision, C++ ones double) and includes this header first.  Everything
// else is the shader's own text:
//  - layout(...) qualifiers vanish; `uniform` becomes `struct`, so a uniform block
//    `uniform Camera { ... } camera;` declares a global struct and `uniform sampler2D s;` a global of
//    the sampler type below; `in`/`out` varyings become globals (thread_local: one invocation per
//    host thread at a time); `in`/`inout` parameter qualifiers vanish (the shaders read their
//    inout parameters back nowhere);
//  - vec/mat types and the built-in functions are glm's (swizzles included), with float overloads
//    for the calls GLSL makes with integer literals (clamp(x, 0, 1) and the like), the implicit
//    int -> float conversion of mixed vector arithmetic, and mix in the specification's form;
//  - samplers: LINEAR filter with float weights, REPEAT or CLAMP_TO_EDGE, mip 0, on UNORM8 or float
//    texels — the definition shared with the CPU restatement (x = u*N - 0.5, i0 = floor(x),
//    a = x - i0, interpolated along x, then y, then z);
//  - images: imageStore / imageLoad / imageSize on float4 rows;
//  - main() is renamed glsl_main(); gl_GlobalInvocationID is a thread_local that the harness
//    (oracle/ref/ref_*_main.cpp) sets.
#pragma once

#define GLM_FORCE_SWIZZLE
#include <glm/glm.hpp>

#include <cmath>
#include <cstdint>

using namespace glm;

#define layout(...)
#define uniform struct
#define readonly
#define writeonly
#define highp
#define in
#define inout
#define out
#define main glsl_main

// ---------------------------------------------------------------------------------- built-ins

thread_local uvec3 gl_GlobalInvocationID;

inline float clamp(float x, float a, float b) { return glm::clamp(x, a, b); }
inline float min(float a, float b) { return glm::min(a, b); }
inline float max(float a, float b) { return glm::max(a, b); }
// mix as the GLSL specification defines it, x * (1 - a) + y * a (glm computes x + a * (y - x), which
// differs in the last bit)
inline float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
template <length_t L>
inline vec<L, float> mix(const vec<L, float>& x, const vec<L, float>& y, float a) {
    return x * (1.0f - a) + y * a;
}
template <length_t L>
inline vec<L, float> mix(const vec<L, float>& x, const vec<L, float>& y, const vec<L, float>& a) {
    return x * (vec<L, float>(1.0f) - a) + y * a;
}
inline float smoothstep(float e0, float e1, float x) { return glm::smoothstep(e0, e1, x); }

// GLSL converts an integer vector operand to float implicitly (vec2(uv) / ivec2(dim)); glm does not.
template <length_t L>
inline vec<L, float> operator*(const vec<L, float>& a, const vec<L, int>& b) { return a * vec<L, float>(b); }
template <length_t L>
inline vec<L, float> operator*(const vec<L, int>& a, const vec<L, float>& b) { return vec<L, float>(a) * b; }
template <length_t L>
inline vec<L, float> operator/(const vec<L, float>& a, const vec<L, int>& b) { return a / vec<L, float>(b); }
template <length_t L>
inline vec<L, float> operator+(const vec<L, float>& a, const vec<L, int>& b) { return a + vec<L, float>(b); }
template <length_t L>
inline vec<L, float> operator-(const vec<L, float>& a, const vec<L, int>& b) { return a - vec<L, float>(b); }

// ---------------------------------------------------------------------------------- samplers

struct GlslSampler {
    const void* texels = nullptr;  // UNORM8 (bytes) or float texels, x fastest, then y, then z
    int w = 1, h = 1, d = 1, channels = 4;
    bool is_float = false;         // float texels (framebuffers) instead of UNORM8
    bool clamp_edge = false;       // CLAMP_TO_EDGE instead of REPEAT
    vec4 fetch(int x, int y, int z) const {
        if (clamp_edge) {
            x = x < 0 ? 0 : (x >= w ? w - 1 : x);
            y = y < 0 ? 0 : (y >= h ? h - 1 : y);
            z = z < 0 ? 0 : (z >= d ? d - 1 : z);
        } else {
            x %= w;
            x += x < 0 ? w : 0;
            y %= h;
            y += y < 0 ? h : 0;
            z %= d;
            z += z < 0 ? d : 0;
        }
        const size_t i = (((size_t)z * h + y) * w + x) * channels;
        float v[4] = {0.0f, 0.0f, 0.0f, 1.0f};
        for (int c = 0; c < channels && c < 4; ++c)
            v[c] = is_float ? static_cast<const float*>(texels)[i + c]
                            : (float)static_cast<const uint8_t*>(texels)[i + c] / 255.0f;
        return vec4(v[0], v[1], v[2], v[3]);
    }
};
struct sampler2D : GlslSampler {};
struct sampler3D : GlslSampler {};

inline vec4 mix4(const vec4& a, const vec4& b, float t) {
    return vec4(a.x * (1.0f - t) + b.x * t, a.y * (1.0f - t) + b.y * t, a.z * (1.0f - t) + b.z * t,
                a.w * (1.0f - t) + b.w * t);
}

inline vec4 texture(const sampler2D& s, vec2 uv) {
    const float x = uv.x * (float)s.w - 0.5f, y = uv.y * (float)s.h - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y);
    const float ax = x - fx, ay = y - fy;
    // CLAMP_TO_EDGE may clamp the base texel first (it keeps far coordinates out of int overflow);
    // REPEAT wraps the true floor
    const int x0 = s.clamp_edge ? (int)fminf(fmaxf(fx, -2.0f), (float)s.w + 1.0f) : (int)fx;
    const int y0 = s.clamp_edge ? (int)fminf(fmaxf(fy, -2.0f), (float)s.h + 1.0f) : (int)fy;
    const vec4 a = mix4(s.fetch(x0, y0, 0), s.fetch(x0 + 1, y0, 0), ax);
    const vec4 b = mix4(s.fetch(x0, y0 + 1, 0), s.fetch(x0 + 1, y0 + 1, 0), ax);
    return mix4(a, b, ay);
}

inline vec4 texture(const sampler3D& s, vec3 p) {
    const float x = p.x * (float)s.w - 0.5f, y = p.y * (float)s.h - 0.5f, z = p.z * (float)s.d - 0.5f;
    const float fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    const float ax = x - fx, ay = y - fy, az = z - fz;
    const int x0 = (int)fx, y0 = (int)fy, z0 = (int)fz;
    const vec4 a = mix4(s.fetch(x0, y0, z0), s.fetch(x0 + 1, y0, z0), ax);
    const vec4 b = mix4(s.fetch(x0, y0 + 1, z0), s.fetch(x0 + 1, y0 + 1, z0), ax);
    const vec4 c = mix4(s.fetch(x0, y0, z0 + 1), s.fetch(x0 + 1, y0, z0 + 1), ax);
    const vec4 e = mix4(s.fetch(x0, y0 + 1, z0 + 1), s.fetch(x0 + 1, y0 + 1, z0 + 1), ax);
    return mix4(mix4(a, b, ay), mix4(c, e, ay), az);
}

// ---------------------------------------------------------------------------------- images

struct image2D {
    float* texels = nullptr;  // float4 rows
    int w = 0, h = 0;
};

inline void imageStore(image2D& im, ivec2 p, vec4 v) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    float* t = im.texels + ((size_t)p.y * im.w + p.x) * 4;
    t[0] = v.x;
    t[1] = v.y;
    t[2] = v.z;
    t[3] = v.w;
}

inline vec4 imageLoad(const image2D& im, ivec2 p) {
    if (p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return vec4(0.0f);
    const float* t = im.texels + ((size_t)p.y * im.w + p.x) * 4;
    return vec4(t[0], t[1], t[2], t[3]);
}

inline ivec2 imageSize(const image2D& im) { return ivec2(im.w, im.h); }

// ---------------------------------------------------------------------------------- elementary functions
//
// With GLSL_SHIM_MM_MATH the shader's exp, pow, acos, cos and sin are those of mm_math.h (the
// functions the CPU restatement's float instance and the GPU's exact mode use) instead of the C
// library's.  GLSL leaves their precision to the implementation, so either is the shader; with the
// same functions on both sides every remaining difference would be one of arithmetic or order.
#ifdef GLSL_SHIM_MM_MATH
#include "mm_math.h"

namespace glsl_mm {
inline float pow_(float x, float y) { return mmx::mm_powf(x, y); }
inline float exp_(float x) { return mmx::mm_expf(x); }
inline float acos_(float x) { return mmx::mm_acosf(x); }
inline float cos_(float x) { return mmx::mm_cosf(x); }
inline float sin_(float x) { return mmx::mm_sinf(x); }
template <length_t L>
inline vec<L, float> pow_(const vec<L, float>& x, const vec<L, float>& y) {
    vec<L, float> r;
    for (length_t i = 0; i < L; ++i) r[i] = mmx::mm_powf(x[i], y[i]);
    return r;
}
template <length_t L>
inline vec<L, float> exp_(const vec<L, float>& x) {
    vec<L, float> r;
    for (length_t i = 0; i < L; ++i) r[i] = mmx::mm_expf(x[i]);
    return r;
}
}  // namespace glsl_mm

#define pow glsl_mm::pow_
#define exp glsl_mm::exp_
#define acos glsl_mm::acos_
#define cos glsl_mm::cos_
#define sin glsl_mm::sin_
#endif
