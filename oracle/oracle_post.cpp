// oracle_post.cpp - CPU restatement of the reference's post-processing chain (test infrastructure
// only): god rays (SkyEngine/SkyEngine/Shaders/god-ray.frag:41-76), radial blur
// (radialBlur.frag:36-63), the mesh drawn over the blurred sky in the same render pass
// (VulkanApplication.cpp:955-966) and the Uncharted-2 tonemap with vignette (tonemap.frag:11-33)
// into the 8-bit swapchain image (B8G8R8A8_UNORM, VulkanApplication.cpp:1437-1446).
//
// Conventions shared with the CUDA kernels (post.cu):
//  - every pass draws a full-screen quad whose uv runs 0..1 left to right and top to bottom
//    (Geometry.cpp:91-101), so pixel (x, y) has fragUV = ((x + 0.5) / W, (y + 0.5) / H) and
//    scrPt = fragUV * 2 - 1;
//  - texture(texColor, fragUV) at the fragment's own uv is the texel itself (a texel centre: the
//    LINEAR filter's weights are zero there); taps elsewhere are bilinear with float weights and
//    CLAMP_TO_EDGE (the offscreen sampler, VulkanApplication.cpp:1290-1305): x = u W - 0.5,
//    a = x - floor(x), indices clamped to the image;
//  - camera.proj * camera.view * sun.location is evaluated as (proj * view) * location, the
//    elements of the matrix product summed in index order, the matrix-vector product pairwise
//    (glm's orders, under which the compiled shaders agree with this file);
//  - GLSL constant expressions (SAMPLE_WEIGHT * DENSITY, the tonemap's 0.1 * 0.5 ...) are folded in
//    float; pow is mm_math.h's powf; the float -> UNORM8 conversion rounds to nearest even after
//    clamping to [0, 1] (NaN -> 0).
// Float arithmetic in source order, no contraction (-ffp-contract=off).
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../project-marshmallow_gb300/csrc/mm_math.h"
#include "oracle.h"

namespace {

struct F4 {
    float x, y, z, w;
};

struct Img {
    const float* p;
    int w, h;
    F4 texel(int x, int y) const {
        const float* q = p + ((size_t)y * w + x) * 4;
        return {q[0], q[1], q[2], q[3]};
    }
};

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// Bilinear, CLAMP_TO_EDGE, channel c of the image at normalized (u, v).
float sample_channel(const Img& im, float u, float v, int c) {
    const float x = u * (float)im.w - 0.5f, y = v * (float)im.h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    const int ix = (int)fminf(fmaxf(fx, -1.0f), (float)im.w), iy = (int)fminf(fmaxf(fy, -1.0f), (float)im.h);
    const int x0 = clampi(ix, 0, im.w - 1), x1 = clampi(ix + 1, 0, im.w - 1);
    const int y0 = clampi(iy, 0, im.h - 1), y1 = clampi(iy + 1, 0, im.h - 1);
    auto t = [&](int xx, int yy) { return im.p[((size_t)yy * im.w + xx) * 4 + c]; };
    const float a = mixf(t(x0, y0), t(x1, y0), ax);
    const float b = mixf(t(x0, y1), t(x1, y1), ax);
    return mixf(a, b, ay);
}

// (proj * view) * sun.location, divided by its w (god-ray.frag:44-46, radialBlur.frag:48-49).
// GLSL leaves the order of the sums to its compiler; these are glm's: each element of the matrix
// product summed in index order, the matrix-vector product pairwise, (m0 x + m1 y) + (m2 z + m3 w).
void sun_ndc(const mm_uniforms* u, float* sx, float* sy) {
    const float* P = u->camera.proj;
    const float* V = u->camera.view;
    float pv[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            float s = P[0 * 4 + r] * V[c * 4 + 0];
            for (int k = 1; k < 4; ++k) s = s + P[k * 4 + r] * V[c * 4 + k];
            pv[c * 4 + r] = s;
        }
    const float* L = u->sun.location;
    float q[4];
    for (int r = 0; r < 4; ++r) q[r] = (pv[0 * 4 + r] * L[0] + pv[1 * 4 + r] * L[1]) + (pv[2 * 4 + r] * L[2] + pv[3 * 4 + r] * L[3]);
    *sx = q[0] / q[3];
    *sy = q[1] / q[3];
}

inline void frag(int x, int y, int w, int h, float* u, float* v) {
    *u = ((float)x + 0.5f) / (float)w;
    *v = ((float)y + 0.5f) / (float)h;
}

// god-ray.frag:41-76
void god_rays(const mm_uniforms* un, const Img& src, float* dst) {
    float sx, sy;
    sun_ndc(un, &sx, &sy);
    const bool night = un->sun.direction[1] < 0.0f;
    const float weight_density = 1.0f / 8.0f * 0.75f;  // SAMPLE_WEIGHT * DENSITY
    for (int y = 0; y < src.h; ++y)
        for (int x = 0; x < src.w; ++x) {
            float u, v;
            frag(x, y, src.w, src.h, &u, &v);
            const F4 c = src.texel(x, y);
            float* o = dst + ((size_t)y * src.w + x) * 4;
            o[0] = c.x;
            o[1] = c.y;
            o[2] = c.z;
            if (night) {
                o[3] = 1.0f;
                continue;
            }
            float px = u * 2.0f - 1.0f, py = v * 2.0f - 1.0f;
            const float dx = (px - sx) * weight_density, dy = (py - sy) * weight_density;
            float accum = c.w * 0.5f;
            float decay = 1.0f;
            for (int i = 0; i < 8; ++i) {
                px = px - dx;
                py = py - dy;
                float amt = sample_channel(src, px * 0.5f + 0.5f, py * 0.5f + 0.5f, 3) * 0.5f;
                amt = amt * (1.0f / 8.0f * decay);
                accum = accum + amt;
                decay = decay * 0.99f;
            }
            o[3] = accum * 0.9f;
        }
}

// radialBlur.frag:36-63
void radial_blur(const mm_uniforms* un, const Img& src, float* dst) {
    static const float kTaps[10] = {-0.08f, -0.05f, -0.03f, -0.02f, -0.01f, 0.01f, 0.02f, 0.03f, 0.05f, 0.08f};
    float sx, sy;
    sun_ndc(un, &sx, &sy);
    const bool night = un->sun.direction[1] < 0.0f;
    const float kr = un->sun.color[0] * un->sun.intensity, kg = un->sun.color[1] * un->sun.intensity,
                kb = un->sun.color[2] * un->sun.intensity;
    for (int y = 0; y < src.h; ++y)
        for (int x = 0; x < src.w; ++x) {
            float u, v;
            frag(x, y, src.w, src.h, &u, &v);
            const F4 c = src.texel(x, y);
            float* o = dst + ((size_t)y * src.w + x) * 4;
            o[3] = 1.0f;
            if (night) {
                o[0] = c.x;
                o[1] = c.y;
                o[2] = c.z;
                continue;
            }
            const float px = u * 2.0f - 1.0f, py = v * 2.0f - 1.0f;
            float lx = sx - px, ly = sy - py;
            const float dist = sqrtf(lx * lx + ly * ly);
            lx = lx / dist;
            ly = ly / dist;
            float accum = 0.0f;
            for (int i = 0; i < 10; ++i) {
                const float ox = kTaps[i] * lx * 1.5f * dist, oy = kTaps[i] * ly * 1.5f * dist;
                accum = accum + sample_channel(src, (px + ox) * 0.5f + 0.5f, (py + oy) * 0.5f + 0.5f, 3) * 1.1f;
            }
            accum = accum / 10.0f;
            o[0] = kr * accum + 0.5f * c.x;
            o[1] = kg * accum + 0.5f * c.y;
            o[2] = kb * accum + 0.5f * c.z;
        }
}

// tonemap.frag:11-14
inline float uc2(float x) {
    return ((x * (0.15f * x + 0.1f * 0.5f) + 0.2f * 0.02f) / (x * (0.15f * x + 0.5f) + 0.2f * 0.3f)) - 0.02f / 0.3f;
}

inline uint8_t unorm8(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);  // NaN -> 0
    return (uint8_t)nearbyintf(v * 255.0f);
}

// tonemap.frag:16-33 into 8 bits
void tonemap(const Img& src, uint8_t* out, size_t pitch, int bgra) {
    const float whitemap = 1.0f / uc2(50.2f);
    const float inv_gamma = 1.0f / 2.2f;
    for (int y = 0; y < src.h; ++y)
        for (int x = 0; x < src.w; ++x) {
            float u, v;
            frag(x, y, src.w, src.h, &u, &v);
            const F4 c = src.texel(x, y);
            float col[3] = {c.x, c.y, c.z};
            const float du = u - 0.5f, dv = v - 0.5f;
            const float vignette = du * du + dv * dv;
            const float tint[3] = {0.1f, 0.05f, 0.13f};
            uint8_t b[3];
            for (int k = 0; k < 3; ++k) {
                float t = uc2(0.7f * col[k]);
                t = t * whitemap;
                t = mmx::mm_powf(t, inv_gamma);
                b[k] = unorm8(mixf(t, tint[k], vignette));
            }
            uint8_t* o = out + (size_t)y * pitch + (size_t)x * 4;
            o[0] = bgra ? b[2] : b[0];
            o[1] = b[1];
            o[2] = bgra ? b[0] : b[2];
            o[3] = 255;
        }
}

}  // namespace

extern "C" {

int oracle_post_god_rays(const mm_uniforms* u, const float* src, int w, int h, float* dst) {
    if (!u || !src || !dst || w <= 0 || h <= 0) return MM_ERR_INVALID_ARGUMENT;
    god_rays(u, Img{src, w, h}, dst);
    return MM_OK;
}

int oracle_post_radial_blur(const mm_uniforms* u, const float* src, int w, int h, float* dst) {
    if (!u || !src || !dst || w <= 0 || h <= 0) return MM_ERR_INVALID_ARGUMENT;
    radial_blur(u, Img{src, w, h}, dst);
    return MM_OK;
}

int oracle_post_tonemap(const float* src, int w, int h, uint8_t* out, size_t pitch, int bgra) {
    if (!src || !out || w <= 0 || h <= 0) return MM_ERR_INVALID_ARGUMENT;
    tonemap(Img{src, w, h}, out, pitch, bgra);
    return MM_OK;
}

int oracle_post_chain(const mm_uniforms* u, const float* clouds, const float* mesh, int w, int h, uint8_t* out,
                      size_t pitch, int bgra) {
    if (!u || !clouds || !out || w <= 0 || h <= 0) return MM_ERR_INVALID_ARGUMENT;
    const size_t n = (size_t)w * h * 4;
    std::vector<float> fb1(n), fb2(n);
    god_rays(u, Img{clouds, w, h}, fb1.data());
    radial_blur(u, Img{fb1.data(), w, h}, fb2.data());
    if (mesh)
        for (size_t i = 0; i < (size_t)w * h; ++i)
            if (mesh[4 * i + 3] != 0.0f) memcpy(&fb2[4 * i], mesh + 4 * i, 16);
    tonemap(Img{fb2.data(), w, h}, out, pitch, bgra);
    return MM_OK;
}

}  // extern "C"
