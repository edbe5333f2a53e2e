// oracle_noise.cpp - CPU oracle of the noise-texture generators (test infrastructure only).
//
// Two parts:
//  1. oracle_ref_curl: SkyEngine/SkyEngine/ImageUtils.cpp:7-222 (GenerateCurlNoise) restated with
//     the same float/double typing as the reference build, so the 128x128 output equals the
//     shipped Textures/CurlNoiseFBM.tga byte for byte.  The reference hashes with float sinf
//     (ImageUtils.cpp:26); sinf here is the correctly rounded mmx::mm_sinf_cr, which the tests
//     show reproduces the shipped texture.
//  2. oracle_noise_fill: the seeded generators that replace the pre-baked Nubis textures of
//     Textures/3DTextures (no generator for them exists in the reference).  The generator
//     definition (hash, lattice, octave weights, output maps) is stated once here, in plain
//     sequential code; the CUDA kernels restate it and must match it bit for bit.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "../project-marshmallow_gb300/csrc/mm_math.h"
#include "oracle.h"

namespace {

// ------------------------------------------------------------------ reference curl generator

struct f3 {
    float x, y, z;
};

// ImageUtils.cpp:10-23 (glm::vec3 of float; the literals are rounded to float)
const float kRefBasis[12][3] = {
    {0.7071f, 0.7071f, 0.f},  {0.7071f, -0.7071f, 0.f},  {-0.7071f, 0.7071f, 0.f},
    {-0.7071f, -0.7071f, 0.f}, {0.7071f, 0.f, 0.7071f},  {0.7071f, 0.f, -0.7071f},
    {-0.7071f, 0.f, 0.7071f},  {-0.7071f, 0.f, -0.7071f}, {0.f, 0.7071f, 0.7071f},
    {0.f, 0.7071f, -0.7071f},  {0.f, -0.7071f, 0.7071f},  {0.f, -0.7071f, -0.7071f},
};

// ImageUtils.cpp:25-29: fract(sinf(dot(p, (12.9898, 78.233, 47.387))) * 43758.5453), all float;
// glm::dot sums (x*a + y*b) + z*c.
float ref_hash_noise(float x, float y, float z) {
    float d = x * 12.9898f + y * 78.233f;
    d = d + z * (float)47.387;
    float n = mmx::mm_sinf_cr(d) * 43758.5453f;
    n = n - floorf(n);
    return n;
}

int ref_hash_index(float x, float y, float z) {
    return (int)floorf(12.f * ref_hash_noise(x, y, z));
}

float ref_dot(int gi, f3 r) {
    const float* g = kRefBasis[gi];
    float a = g[0] * r.x + g[1] * r.y;
    return a + g[2] * r.z;
}

// ImageUtils.cpp:36-38: (1.0 - t) * a + t * b evaluates in double (1.0 is a double literal,
// t * b is a float product), then returns float.
float ref_lerp(float a, float b, float t) {
    return (float)((1.0 - (double)t) * (double)a + (double)(t * b));
}

// ImageUtils.cpp:41-73
float ref_perlin(f3 p, float freq) {
    p.x *= freq;
    p.y *= freq;
    p.z *= freq;
    f3 f = {floorf(p.x), floorf(p.y), floorf(p.z)};
    f3 r = {p.x - f.x, p.y - f.y, p.z - f.z};
    auto fade = [](float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); };
    f3 u = {fade(r.x), fade(r.y), fade(r.z)};
    f3 f1 = {f.x + 1.f, f.y + 1.f, f.z + 1.f};
    if (fabsf(f1.x - freq) < 0.001f) f1.x = freq;
    if (fabsf(f1.y - freq) < 0.001f) f1.y = freq;
    if (fabsf(f1.z - freq) < 0.001f) f1.z = freq;
    float nnn = ref_dot(ref_hash_index(f.x, f.y, f.z), r);
    float nnp = ref_dot(ref_hash_index(f.x, f.y, f1.z), {r.x, r.y, r.z - 1.f});
    float npn = ref_dot(ref_hash_index(f.x, f1.y, f.z), {r.x, r.y - 1.f, r.z});
    float npp = ref_dot(ref_hash_index(f.x, f1.y, f1.z), {r.x, r.y - 1.f, r.z - 1.f});
    float pnn = ref_dot(ref_hash_index(f1.x, f.y, f.z), {r.x - 1.f, r.y, r.z});
    float pnp = ref_dot(ref_hash_index(f1.x, f.y, f1.z), {r.x - 1.f, r.y, r.z - 1.f});
    float ppn = ref_dot(ref_hash_index(f1.x, f1.y, f.z), {r.x - 1.f, r.y - 1.f, r.z});
    float ppp = ref_dot(ref_hash_index(f1.x, f1.y, f1.z), {r.x - 1.f, r.y - 1.f, r.z - 1.f});
    float nn = ref_lerp(nnn, pnn, u.x);
    float np = ref_lerp(nnp, pnp, u.x);
    float pn = ref_lerp(npn, ppn, u.x);
    float pp = ref_lerp(npp, ppp, u.x);
    float n = ref_lerp(nn, pn, u.y);
    float q = ref_lerp(np, pp, u.y);
    return ref_lerp(n, q, u.z);
}

// ImageUtils.cpp:75-87
float ref_fbm(f3 p, float freq, int octaves) {
    float noise = 0.0f, weight = 1.0f, total = 0.0f;
    const float persistence = 0.4f;
    for (int i = 0; i < octaves; i++) {
        total += weight;
        noise += weight * ref_perlin(p, freq);
        freq *= 2.0f;
        weight *= persistence;
    }
    return noise / total;
}

// ImageUtils.cpp:130-169; EPS = 0.0005 is a double literal: the coordinates are rounded to float
// by the glm::vec3 constructor and the difference quotient divides by the double 2*EPS.
f3 ref_curl_fbm(float px, float py, float freq, int octaves) {
    const double EPS = 0.0005;
    auto q = [&](f3 a, f3 b) {
        float fa = ref_fbm(a, freq, octaves), fb = ref_fbm(b, freq, octaves);
        return (float)((double)(fb - fa) / (2.f * EPS));
    };
    float dydx = q({(float)(px - EPS), py, 0.5f}, {(float)(px + EPS), py, 0.5f});
    float dxdy = q({px, (float)(py - EPS), 0.5f}, {px, (float)(py + EPS), 0.5f});
    float dxdz = q({px, 0.5f, (float)(py - EPS)}, {px, 0.5f, (float)(py + EPS)});
    float dzdx = q({(float)(px - EPS), 0.5f, py}, {(float)(px + EPS), 0.5f, py});
    float dzdy = q({0.5f, (float)(py - EPS), px}, {0.5f, (float)(py + EPS), px});
    float dydz = q({0.5f, py, (float)(px - EPS)}, {0.5f, py, (float)(px + EPS)});
    return {dzdy - dydz, dxdz - dzdx, dydx - dxdy};
}

// ------------------------------------------------------------------ seeded generators

inline uint32_t hash32(uint32_t x) {  // "lowbias32" integer mixer (C. Wellons, public domain)
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

inline uint32_t hash3(int32_t x, int32_t y, int32_t z, uint32_t s) {
    return hash32((uint32_t)x + hash32((uint32_t)y + hash32((uint32_t)z + s)));
}

inline float rand01(uint32_t h) { return (float)(h >> 8) * 0x1p-24f; }

inline uint32_t stream_seed(uint32_t seed, int kind, int channel, int octave) {
    return hash32(seed ^ hash32(0x9E3779B9u * (uint32_t)(1 + kind * 64 + channel * 8 + octave)));
}

inline int wrapi(int c, int f) {
    int m = c % f;
    return m < 0 ? m + f : m;
}

// Lattice coordinate of texel centre i of n at frequency f: ((2i+1) f) / (2n), one rounding.
inline float lattice(int i, int n, int f) { return (float)((2 * i + 1) * f) / (float)(2 * n); }

// Worley F1, inverted: 1 - min(F1, 1); one feature point per cell; tileable with period f.
float worley3(float qx, float qy, float qz, int f, uint32_t s) {
    int cx = (int)floorf(qx), cy = (int)floorf(qy), cz = (int)floorf(qz);
    float fx = qx - (float)cx, fy = qy - (float)cy, fz = qz - (float)cz;
    float best = 4.0f;
    for (int dz = -1; dz <= 1; ++dz)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                uint32_t h = hash3(wrapi(cx + dx, f), wrapi(cy + dy, f), wrapi(cz + dz, f), s);
                float px = (float)dx + rand01(h);
                float py = (float)dy + rand01(hash32(h + 0x9E3779B9u));
                float pz = (float)dz + rand01(hash32(h + 0x3C6EF372u));
                float ex = px - fx, ey = py - fy, ez = pz - fz;
                float d2 = (ex * ex + ey * ey) + ez * ez;
                best = fminf(best, d2);
            }
    return 1.0f - fminf(sqrtf(best), 1.0f);
}

// 0.625 W(f) + 0.25 W(2f) + 0.125 W(4f)
float worley_fbm(int i, int j, int k, int n, int f, uint32_t seed, int kind, int ch) {
    float a = worley3(lattice(i, n, f), lattice(j, n, f), lattice(k, n, f), f,
                      stream_seed(seed, kind, ch, 0));
    float b = worley3(lattice(i, n, 2 * f), lattice(j, n, 2 * f), lattice(k, n, 2 * f), 2 * f,
                      stream_seed(seed, kind, ch, 1));
    float c = worley3(lattice(i, n, 4 * f), lattice(j, n, 4 * f), lattice(k, n, 4 * f), 4 * f,
                      stream_seed(seed, kind, ch, 2));
    return (0.625f * a + 0.25f * b) + 0.125f * c;
}

const int kGrad3[12][3] = {{1, 1, 0},  {-1, 1, 0},  {1, -1, 0}, {-1, -1, 0},
                           {1, 0, 1},  {-1, 0, 1},  {1, 0, -1}, {-1, 0, -1},
                           {0, 1, 1},  {0, -1, 1},  {0, 1, -1}, {0, -1, -1}};

inline float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
inline float lerpf(float a, float b, float t) { return a + t * (b - a); }

inline float grad3(uint32_t h, float x, float y, float z) {
    const int* g = kGrad3[h % 12u];
    return ((float)g[0] * x + (float)g[1] * y) + (float)g[2] * z;
}

// Gradient noise with period f on every axis, output roughly in [-1, 1].
float perlin3(float qx, float qy, float qz, int f, uint32_t s) {
    int cx = (int)floorf(qx), cy = (int)floorf(qy), cz = (int)floorf(qz);
    float x = qx - (float)cx, y = qy - (float)cy, z = qz - (float)cz;
    int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f);
    int y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    int z0 = wrapi(cz, f), z1 = wrapi(cz + 1, f);
    float n000 = grad3(hash3(x0, y0, z0, s), x, y, z);
    float n100 = grad3(hash3(x1, y0, z0, s), x - 1.0f, y, z);
    float n010 = grad3(hash3(x0, y1, z0, s), x, y - 1.0f, z);
    float n110 = grad3(hash3(x1, y1, z0, s), x - 1.0f, y - 1.0f, z);
    float n001 = grad3(hash3(x0, y0, z1, s), x, y, z - 1.0f);
    float n101 = grad3(hash3(x1, y0, z1, s), x - 1.0f, y, z - 1.0f);
    float n011 = grad3(hash3(x0, y1, z1, s), x, y - 1.0f, z - 1.0f);
    float n111 = grad3(hash3(x1, y1, z1, s), x - 1.0f, y - 1.0f, z - 1.0f);
    float u = fade(x), v = fade(y), w = fade(z);
    float n00 = lerpf(n000, n100, u), n10 = lerpf(n010, n110, u);
    float n01 = lerpf(n001, n101, u), n11 = lerpf(n011, n111, u);
    float n0 = lerpf(n00, n10, v), n1 = lerpf(n01, n11, v);
    return lerpf(n0, n1, w);
}

const float kGrad2[8][2] = {{1.f, 1.f}, {-1.f, 1.f}, {1.f, -1.f}, {-1.f, -1.f},
                            {1.f, 0.f}, {-1.f, 0.f}, {0.f, 1.f},  {0.f, -1.f}};

float perlin2(float qx, float qy, int f, uint32_t s) {
    int cx = (int)floorf(qx), cy = (int)floorf(qy);
    float x = qx - (float)cx, y = qy - (float)cy;
    int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f), y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    auto g = [&](int ix, int iy, float dx, float dy) {
        const float* gg = kGrad2[hash3(ix, iy, 0, s) & 7u];
        return gg[0] * dx + gg[1] * dy;
    };
    float n00 = g(x0, y0, x, y), n10 = g(x1, y0, x - 1.0f, y);
    float n01 = g(x0, y1, x, y - 1.0f), n11 = g(x1, y1, x - 1.0f, y - 1.0f);
    float u = fade(x), v = fade(y);
    return lerpf(lerpf(n00, n10, u), lerpf(n01, n11, u), v);
}

float value2(float qx, float qy, int f, uint32_t s) {
    int cx = (int)floorf(qx), cy = (int)floorf(qy);
    float x = qx - (float)cx, y = qy - (float)cy;
    int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f), y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    float v00 = rand01(hash3(x0, y0, 0, s)), v10 = rand01(hash3(x1, y0, 0, s));
    float v01 = rand01(hash3(x0, y1, 0, s)), v11 = rand01(hash3(x1, y1, 0, s));
    float u = x * x * (3.0f - 2.0f * x), v = y * y * (3.0f - 2.0f * y);
    return lerpf(lerpf(v00, v10, u), lerpf(v01, v11, u), v);
}

inline uint8_t quantize(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint8_t)(int)floorf(v * 255.0f + 0.5f);
}

// Affine output maps that give the synthetic channels the first two moments of the shipped
// Nubis textures (low-res R mean 0.504 sd 0.105; Worley channels mean 0.686 sd 0.10).
const float kPwScale = 1.64f, kPwBias = -0.593f;
const float kWorleyScale = 0.866f, kWorleyBias = 0.271f;
const float kCurlScale = 0.03f;

// MM_NOISE_LOWRES_PERLIN_WORLEY R channel: Perlin FBM (3 octaves from f, halving amplitude)
// remapped with the Worley FBM of the same base frequency as its lower bound.
float perlin_worley(int i, int j, int k, int n, uint32_t seed) {
    const int f = 4;
    float sum = 0.0f, amp = 1.0f, norm = 0.0f;
    for (int o = 0; o < 3; ++o) {
        int fo = f << o;
        sum += amp * perlin3(lattice(i, n, fo), lattice(j, n, fo), lattice(k, n, fo), fo,
                             stream_seed(seed, MM_NOISE_LOWRES_PERLIN_WORLEY, 0, 4 + o));
        norm += amp;
        amp *= 0.5f;
    }
    float p01 = (sum / norm) * 0.5f + 0.5f;
    float wf = worley_fbm(i, j, k, n, f, seed, MM_NOISE_LOWRES_PERLIN_WORLEY, 0);
    // remap(p01, wf - 1, 1, 0, 1)
    return (p01 - (wf - 1.0f)) / (1.0f - (wf - 1.0f));
}

float curl_potential(float qx, float qy, int n_unused, uint32_t seed) {
    (void)n_unused;
    float sum = 0.0f, amp = 1.0f, norm = 0.0f;
    for (int o = 0; o < 5; ++o) {
        int fo = 4 << o;
        sum += amp * perlin2(qx * (float)fo, qy * (float)fo, fo,
                             stream_seed(seed, MM_NOISE_CURL2D, 0, o));
        norm += amp;
        amp *= 0.5f;
    }
    return sum / norm;
}

// Runs fn(k) for k in [0, n) on the host's hardware threads (slices are independent).
template <class F>
void parallel_slices(int n, F fn) {
    unsigned nt = std::max(1u, std::min(std::thread::hardware_concurrency(), 64u));
    std::atomic<int> next(0);
    std::vector<std::thread> pool;
    for (unsigned t = 0; t < nt; ++t)
        pool.emplace_back([&]() {
            for (int k = next++; k < n; k = next++) fn(k);
        });
    for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

uint32_t oracle_hash32(uint32_t x) { return hash32(x); }
uint32_t oracle_hash3(int32_t x, int32_t y, int32_t z, uint32_t s) { return hash3(x, y, z, s); }

int oracle_ref_curl_hash_index(float x, float y, float z) { return ref_hash_index(x, y, z); }
float oracle_ref_curl_hash(float x, float y, float z) { return ref_hash_noise(x, y, z); }

// The elementary functions shared with the GPU's exact mode, exposed for accuracy tests.
float oracle_mm_math(int fn, float x, float y) {
    switch (fn) {
        case 0: return mmx::mm_expf(x);
        case 1: return mmx::mm_exp2f(x);
        case 2: return mmx::mm_log2f(x);
        case 3: return mmx::mm_powf(x, y);
        case 4: return mmx::mm_acosf(x);
        case 5: return mmx::mm_cosf(x);
        case 6: return mmx::mm_sinf(x);
        case 7: return mmx::mm_sinf_cr(x);
        default: return 0.0f;
    }
}

// ImageUtils.cpp:176-222
int oracle_ref_curl(uint8_t* out) {
    if (!out) return MM_ERR_INVALID_ARGUMENT;
    const int N = 128;
    std::vector<f3> c((size_t)N * N);
    float lo[3] = {3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f};
    float hi[3] = {-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f};
    for (int row = 0; row < N; row++)
        for (int col = 0; col < N; col++) {
            f3 v = ref_curl_fbm((float)col / N, (float)row / N, 3.f, 4);
            c[(size_t)row * N + col] = v;
            float a[3] = {v.x, v.y, v.z};
            for (int k = 0; k < 3; k++) {
                lo[k] = std::min(lo[k], a[k]);
                hi[k] = std::max(hi[k], a[k]);
            }
        }
    for (int i = 0; i < N * N; i++) {
        float a[3] = {c[i].x, c[i].y, c[i].z};
        for (int k = 0; k < 3; k++) {
            float m = 0.f + ((a[k] - lo[k]) / (hi[k] - lo[k]) * (1.f - 0.f));
            out[4 * i + k] = (uint8_t)(int)roundf(m * 255.f);
        }
        out[4 * i + 3] = 255;
    }
    return MM_OK;
}

int oracle_noise_fill(int kind, uint32_t seed, int w, int h, int d, uint8_t* out) {
    if (!out || w <= 0 || h <= 0 || d <= 0) return MM_ERR_INVALID_ARGUMENT;
    switch (kind) {
        case MM_NOISE_LOWRES_PERLIN_WORLEY:
        case MM_NOISE_HIRES_WORLEY: {
            if (w != h || h != d) return MM_ERR_INVALID_ARGUMENT;
            const int n = w;
            const bool low = kind == MM_NOISE_LOWRES_PERLIN_WORLEY;
            parallel_slices(n, [&](int k) {
                for (int j = 0; j < n; ++j)
                    for (int i = 0; i < n; ++i) {
                        uint8_t* t = out + 4 * (((size_t)k * n + j) * n + i);
                        if (low) {
                            t[0] = quantize(kPwScale * perlin_worley(i, j, k, n, seed) + kPwBias);
                            for (int c = 1; c < 4; ++c) {
                                float wf = worley_fbm(i, j, k, n, 4 << (c - 1), seed, kind, c);
                                t[c] = quantize(kWorleyScale * wf + kWorleyBias);
                            }
                        } else {
                            for (int c = 0; c < 3; ++c) {
                                float wf = worley_fbm(i, j, k, n, 2 << c, seed, kind, c);
                                t[c] = quantize(kWorleyScale * wf + kWorleyBias);
                            }
                            t[3] = 0;
                        }
                    }
            });
            return MM_OK;
        }
        case MM_NOISE_CURL2D: {
            if (d != 1) return MM_ERR_INVALID_ARGUMENT;
            // psi = 2D Perlin FBM (5 octaves from 4 cells); curl = (dpsi/dy, -dpsi/dx) by central
            // differences a quarter texel apart; stored as 0.5 + kCurlScale * curl.
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    float xm = (float)(4 * i + 1) / (float)(4 * w), xp = (float)(4 * i + 3) / (float)(4 * w);
                    float ym = (float)(4 * j + 1) / (float)(4 * h), yp = (float)(4 * j + 3) / (float)(4 * h);
                    float xc = (float)(2 * i + 1) / (float)(2 * w), yc = (float)(2 * j + 1) / (float)(2 * h);
                    float dpx = (curl_potential(xp, yc, w, seed) - curl_potential(xm, yc, w, seed)) *
                                (float)(2 * w);
                    float dpy = (curl_potential(xc, yp, h, seed) - curl_potential(xc, ym, h, seed)) *
                                (float)(2 * h);
                    uint8_t* t = out + 2 * ((size_t)j * w + i);
                    t[0] = quantize(0.5f + kCurlScale * dpy);
                    t[1] = quantize(0.5f - kCurlScale * dpx);
                }
            return MM_OK;
        }
        case MM_NOISE_WEATHER: {
            if (d != 1) return MM_ERR_INVALID_ARGUMENT;
            for (int j = 0; j < h; ++j)
                for (int i = 0; i < w; ++i) {
                    float ch[2];
                    for (int c = 0; c < 2; ++c) {
                        const int f = c == 0 ? 8 : 4;
                        float sum = 0.0f, amp = 1.0f, norm = 0.0f;
                        for (int o = 0; o < 4; ++o) {
                            int fo = f << o;
                            sum += amp * value2(lattice(i, w, fo), lattice(j, h, fo), fo,
                                                stream_seed(seed, kind, c, o));
                            norm += amp;
                            amp *= 0.5f;
                        }
                        ch[c] = sum / norm;
                    }
                    uint8_t* t = out + 4 * ((size_t)j * w + i);
                    t[0] = quantize(ch[0]);
                    t[1] = 0;
                    t[2] = quantize(ch[1]);
                    t[3] = 255;
                }
            return MM_OK;
        }
        case MM_NOISE_REF_CURL:
            if (w != 128 || h != 128 || d != 1) return MM_ERR_INVALID_ARGUMENT;
            return oracle_ref_curl(out);
        default:
            return MM_ERR_INVALID_ARGUMENT;
    }
}

}  // extern "C"
