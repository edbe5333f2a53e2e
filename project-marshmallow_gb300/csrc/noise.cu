// noise.cu - GPU generators for the cloud textures (mm_noise_generate / mm_noise_fill).
//
// Built with -fmad=false so every float operation rounds exactly as the sequential definition
// in the CPU oracle does: the integer hash and lattice stages are exact by construction and the
// 8-bit texels come out identical.
//
// Generator definition (the reference ships these textures pre-baked, README.md:68, so the
// seeded generators below are this library's own):
//   hash32     lowbias32 integer mixer; hash3(x,y,z,s) = hash32(x + hash32(y + hash32(z + s)))
//   stream     s = hash32(seed ^ hash32(0x9E3779B9 * (1 + 64 kind + 8 channel + octave)))
//   lattice    texel centre i of n at frequency f: ((2i+1) f) / (2n)
//   Worley     inverted F1 (1 - min(F1, 1)), one feature point per cell, period f on each axis
//   WorleyFBM  0.625 W(f) + 0.25 W(2f) + 0.125 W(4f)
//   Perlin     gradient noise, 12 edge gradients, quintic fade, period f
//   low-res    R = remap(PerlinFBM01(4, 3 oct), WorleyFBM(4) - 1, 1, 0, 1) * 1.64 - 0.593,
//              G/B/A = WorleyFBM(4/8/16) * 0.866 + 0.271              (128^3 RGBA8)
//   hi-res     R/G/B = WorleyFBM(2/4/8) * 0.866 + 0.271, A = 0          (32^3 RGBA8)
//   curl       psi = 2D Perlin FBM (4 cells, 5 octaves); (dpsi/dy, -dpsi/dx) by central
//              differences a quarter texel apart, stored as 0.5 + 0.03 curl  (128^2 RG8)
//   weather    R = value-noise FBM (8 cells, 4 oct), G = 0, B = value-noise FBM (4 cells,
//              4 oct), A = 255                                          (512^2 RGBA8)
// The affine output maps give the channels the mean/deviation of the shipped Nubis textures.
//
// The reference-compatible curl (MM_NOISE_REF_CURL) restates ImageUtils.cpp:7-222 with the
// reference's float/double typing and a correctly rounded sinf (mmx::mm_sinf_cr).
#include <cuda_runtime.h>
#include <stdint.h>

#include "mm_internal.h"
#include "mm_math.h"

namespace mm {
namespace noise {

__device__ __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ uint32_t hash3(int x, int y, int z, uint32_t s) {
    return hash32((uint32_t)x + hash32((uint32_t)y + hash32((uint32_t)z + s)));
}

__device__ __forceinline__ float rand01(uint32_t h) { return (float)(h >> 8) * 0x1p-24f; }

__device__ __forceinline__ uint32_t stream_seed(uint32_t seed, int kind, int ch, int oct) {
    return hash32(seed ^ hash32(0x9E3779B9u * (uint32_t)(1 + kind * 64 + ch * 8 + oct)));
}

__device__ __forceinline__ int wrapi(int c, int f) {
    int m = c % f;
    return m < 0 ? m + f : m;
}

__device__ __forceinline__ float lattice(int i, int n, int f) {
    return __fdiv_rn((float)((2 * i + 1) * f), (float)(2 * n));
}

__device__ __forceinline__ uint8_t quantize(float v) {
    v = fminf(fmaxf(v, 0.0f), 1.0f);
    return (uint8_t)(int)floorf(v * 255.0f + 0.5f);
}

__device__ float worley3(float qx, float qy, float qz, int f, uint32_t s) {
    const int cx = (int)floorf(qx), cy = (int)floorf(qy), cz = (int)floorf(qz);
    const float fx = qx - (float)cx, fy = qy - (float)cy, fz = qz - (float)cz;
    float best = 4.0f;
#pragma unroll 1
    for (int dz = -1; dz <= 1; ++dz) {
        const uint32_t hz = (uint32_t)wrapi(cz + dz, f) + s;
        const uint32_t hz2 = hash32(hz);
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy) {
            const uint32_t hy = hash32((uint32_t)wrapi(cy + dy, f) + hz2);
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const uint32_t h = hash32((uint32_t)wrapi(cx + dx, f) + hy);
                const float px = (float)dx + rand01(h);
                const float py = (float)dy + rand01(hash32(h + 0x9E3779B9u));
                const float pz = (float)dz + rand01(hash32(h + 0x3C6EF372u));
                const float ex = px - fx, ey = py - fy, ez = pz - fz;
                const float d2 = (ex * ex + ey * ey) + ez * ez;
                best = fminf(best, d2);
            }
        }
    }
    return 1.0f - fminf(__fsqrt_rn(best), 1.0f);
}

__device__ float worley_fbm(int i, int j, int k, int n, int f, uint32_t seed, int kind, int ch) {
    const float a = worley3(lattice(i, n, f), lattice(j, n, f), lattice(k, n, f), f, stream_seed(seed, kind, ch, 0));
    const float b = worley3(lattice(i, n, 2 * f), lattice(j, n, 2 * f), lattice(k, n, 2 * f), 2 * f,
                            stream_seed(seed, kind, ch, 1));
    const float c = worley3(lattice(i, n, 4 * f), lattice(j, n, 4 * f), lattice(k, n, 4 * f), 4 * f,
                            stream_seed(seed, kind, ch, 2));
    return (0.625f * a + 0.25f * b) + 0.125f * c;
}

__device__ __forceinline__ float fade(float t) { return t * t * t * (t * (t * 6.0f - 15.0f) + 10.0f); }
__device__ __forceinline__ float lerpf(float a, float b, float t) { return a + t * (b - a); }

// 12 edge gradients (+-1,+-1,0), (+-1,0,+-1), (0,+-1,+-1) in the oracle's table order.
__device__ __forceinline__ float grad3(uint32_t h, float x, float y, float z) {
    const int g = (int)(h % 12u);
    float gx, gy, gz;
    if (g < 4) {
        gx = (g & 1) ? -1.0f : 1.0f;
        gy = (g & 2) ? -1.0f : 1.0f;
        gz = 0.0f;
    } else if (g < 8) {
        gx = (g & 1) ? -1.0f : 1.0f;
        gy = 0.0f;
        gz = (g & 2) ? -1.0f : 1.0f;
    } else {
        gx = 0.0f;
        gy = (g & 1) ? -1.0f : 1.0f;
        gz = (g & 2) ? -1.0f : 1.0f;
    }
    return (gx * x + gy * y) + gz * z;
}

__device__ float perlin3(float qx, float qy, float qz, int f, uint32_t s) {
    const int cx = (int)floorf(qx), cy = (int)floorf(qy), cz = (int)floorf(qz);
    const float x = qx - (float)cx, y = qy - (float)cy, z = qz - (float)cz;
    const int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f);
    const int y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    const int z0 = wrapi(cz, f), z1 = wrapi(cz + 1, f);
    const float n000 = grad3(hash3(x0, y0, z0, s), x, y, z);
    const float n100 = grad3(hash3(x1, y0, z0, s), x - 1.0f, y, z);
    const float n010 = grad3(hash3(x0, y1, z0, s), x, y - 1.0f, z);
    const float n110 = grad3(hash3(x1, y1, z0, s), x - 1.0f, y - 1.0f, z);
    const float n001 = grad3(hash3(x0, y0, z1, s), x, y, z - 1.0f);
    const float n101 = grad3(hash3(x1, y0, z1, s), x - 1.0f, y, z - 1.0f);
    const float n011 = grad3(hash3(x0, y1, z1, s), x, y - 1.0f, z - 1.0f);
    const float n111 = grad3(hash3(x1, y1, z1, s), x - 1.0f, y - 1.0f, z - 1.0f);
    const float u = fade(x), v = fade(y), w = fade(z);
    const float n00 = lerpf(n000, n100, u), n10 = lerpf(n010, n110, u);
    const float n01 = lerpf(n001, n101, u), n11 = lerpf(n011, n111, u);
    return lerpf(lerpf(n00, n10, v), lerpf(n01, n11, v), w);
}

// 8 gradients (+-1,+-1), (+-1,0), (0,+-1) in the oracle's table order.
__device__ __forceinline__ float grad2(uint32_t h, float x, float y) {
    const int g = (int)(h & 7u);
    float gx, gy;
    if (g < 4) {
        gx = (g & 1) ? -1.0f : 1.0f;
        gy = (g & 2) ? -1.0f : 1.0f;
    } else if (g < 6) {
        gx = (g & 1) ? -1.0f : 1.0f;
        gy = 0.0f;
    } else {
        gx = 0.0f;
        gy = (g & 1) ? -1.0f : 1.0f;
    }
    return gx * x + gy * y;
}

__device__ float perlin2(float qx, float qy, int f, uint32_t s) {
    const int cx = (int)floorf(qx), cy = (int)floorf(qy);
    const float x = qx - (float)cx, y = qy - (float)cy;
    const int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f), y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    const float n00 = grad2(hash3(x0, y0, 0, s), x, y), n10 = grad2(hash3(x1, y0, 0, s), x - 1.0f, y);
    const float n01 = grad2(hash3(x0, y1, 0, s), x, y - 1.0f), n11 = grad2(hash3(x1, y1, 0, s), x - 1.0f, y - 1.0f);
    const float u = fade(x), v = fade(y);
    return lerpf(lerpf(n00, n10, u), lerpf(n01, n11, u), v);
}

__device__ float value2(float qx, float qy, int f, uint32_t s) {
    const int cx = (int)floorf(qx), cy = (int)floorf(qy);
    const float x = qx - (float)cx, y = qy - (float)cy;
    const int x0 = wrapi(cx, f), x1 = wrapi(cx + 1, f), y0 = wrapi(cy, f), y1 = wrapi(cy + 1, f);
    const float v00 = rand01(hash3(x0, y0, 0, s)), v10 = rand01(hash3(x1, y0, 0, s));
    const float v01 = rand01(hash3(x0, y1, 0, s)), v11 = rand01(hash3(x1, y1, 0, s));
    const float u = x * x * (3.0f - 2.0f * x), v = y * y * (3.0f - 2.0f * y);
    return lerpf(lerpf(v00, v10, u), lerpf(v01, v11, u), v);
}

// 3D density volumes: a block is a 32x8 (x,y) tile of one z slice; each thread one texel, one
// 4-byte store, so a warp writes 128 contiguous bytes.
__global__ void __launch_bounds__(256) volume_kernel(int kind, uint32_t seed, int n, uchar4* out) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    const int k = blockIdx.z;
    if (i >= n || j >= n) return;
    uchar4 t;
    if (kind == MM_NOISE_LOWRES_PERLIN_WORLEY) {
        const int f = 4;
        float sum = 0.0f, amp = 1.0f, norm = 0.0f;
#pragma unroll 1
        for (int o = 0; o < 3; ++o) {
            const int fo = f << o;
            sum += amp * perlin3(lattice(i, n, fo), lattice(j, n, fo), lattice(k, n, fo), fo,
                                 stream_seed(seed, kind, 0, 4 + o));
            norm += amp;
            amp *= 0.5f;
        }
        const float p01 = __fdiv_rn(sum, norm) * 0.5f + 0.5f;
        const float wf = worley_fbm(i, j, k, n, f, seed, kind, 0);
        const float pw = __fdiv_rn(p01 - (wf - 1.0f), 1.0f - (wf - 1.0f));
        t.x = quantize(1.64f * pw + -0.593f);
        t.y = quantize(0.866f * worley_fbm(i, j, k, n, 4, seed, kind, 1) + 0.271f);
        t.z = quantize(0.866f * worley_fbm(i, j, k, n, 8, seed, kind, 2) + 0.271f);
        t.w = quantize(0.866f * worley_fbm(i, j, k, n, 16, seed, kind, 3) + 0.271f);
    } else {
        t.x = quantize(0.866f * worley_fbm(i, j, k, n, 2, seed, kind, 0) + 0.271f);
        t.y = quantize(0.866f * worley_fbm(i, j, k, n, 4, seed, kind, 1) + 0.271f);
        t.z = quantize(0.866f * worley_fbm(i, j, k, n, 8, seed, kind, 2) + 0.271f);
        t.w = 0;
    }
    out[((size_t)k * n + j) * n + i] = t;
}

__device__ float curl_potential(float qx, float qy, uint32_t seed) {
    float sum = 0.0f, amp = 1.0f, norm = 0.0f;
#pragma unroll 1
    for (int o = 0; o < 5; ++o) {
        const int fo = 4 << o;
        sum += amp * perlin2(qx * (float)fo, qy * (float)fo, fo, stream_seed(seed, MM_NOISE_CURL2D, 0, o));
        norm += amp;
        amp *= 0.5f;
    }
    return __fdiv_rn(sum, norm);
}

__global__ void __launch_bounds__(256) curl_kernel(uint32_t seed, int w, int h, uchar2* out) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= w || j >= h) return;
    const float xm = __fdiv_rn((float)(4 * i + 1), (float)(4 * w)), xp = __fdiv_rn((float)(4 * i + 3), (float)(4 * w));
    const float ym = __fdiv_rn((float)(4 * j + 1), (float)(4 * h)), yp = __fdiv_rn((float)(4 * j + 3), (float)(4 * h));
    const float xc = __fdiv_rn((float)(2 * i + 1), (float)(2 * w)), yc = __fdiv_rn((float)(2 * j + 1), (float)(2 * h));
    const float dpx = (curl_potential(xp, yc, seed) - curl_potential(xm, yc, seed)) * (float)(2 * w);
    const float dpy = (curl_potential(xc, yp, seed) - curl_potential(xc, ym, seed)) * (float)(2 * h);
    out[(size_t)j * w + i] = make_uchar2(quantize(0.5f + 0.03f * dpy), quantize(0.5f - 0.03f * dpx));
}

__global__ void __launch_bounds__(256) weather_kernel(uint32_t seed, int w, int h, uchar4* out) {
    const int i = blockIdx.x * 32 + threadIdx.x;
    const int j = blockIdx.y * 8 + threadIdx.y;
    if (i >= w || j >= h) return;
    float ch[2];
#pragma unroll
    for (int c = 0; c < 2; ++c) {
        const int f = c == 0 ? 8 : 4;
        float sum = 0.0f, amp = 1.0f, norm = 0.0f;
#pragma unroll 1
        for (int o = 0; o < 4; ++o) {
            const int fo = f << o;
            sum += amp * value2(lattice(i, w, fo), lattice(j, h, fo), fo, stream_seed(seed, MM_NOISE_WEATHER, c, o));
            norm += amp;
            amp *= 0.5f;
        }
        ch[c] = __fdiv_rn(sum, norm);
    }
    out[(size_t)j * w + i] = make_uchar4(quantize(ch[0]), 0, quantize(ch[1]), 255);
}

// ---------------------------------------------------------------- reference-compatible curl

__constant__ float kRefBasis[12][3] = {
    {0.7071f, 0.7071f, 0.f},  {0.7071f, -0.7071f, 0.f},  {-0.7071f, 0.7071f, 0.f},
    {-0.7071f, -0.7071f, 0.f}, {0.7071f, 0.f, 0.7071f},  {0.7071f, 0.f, -0.7071f},
    {-0.7071f, 0.f, 0.7071f},  {-0.7071f, 0.f, -0.7071f}, {0.f, 0.7071f, 0.7071f},
    {0.f, 0.7071f, -0.7071f},  {0.f, -0.7071f, 0.7071f},  {0.f, -0.7071f, -0.7071f},
};

__device__ __forceinline__ int ref_index(float x, float y, float z) {  // ImageUtils.cpp:25-34
    float d = x * 12.9898f + y * 78.233f;
    d = d + z * 47.387f;
    float n = mmx::mm_sinf_cr(d) * 43758.5453f;
    n = n - floorf(n);
    return (int)floorf(12.f * n);
}

__device__ __forceinline__ float ref_dot(int g, float rx, float ry, float rz) {
    float a = kRefBasis[g][0] * rx + kRefBasis[g][1] * ry;
    return a + kRefBasis[g][2] * rz;
}

__device__ __forceinline__ float ref_lerp(float a, float b, float t) {  // ImageUtils.cpp:36-38
    return (float)((1.0 - (double)t) * (double)a + (double)(t * b));
}

__device__ float ref_perlin(float px, float py, float pz, float freq) {  // ImageUtils.cpp:41-73
    px *= freq;
    py *= freq;
    pz *= freq;
    const float fx = floorf(px), fy = floorf(py), fz = floorf(pz);
    const float rx = px - fx, ry = py - fy, rz = pz - fz;
    const float ux = rx * rx * rx * (rx * (rx * 6.0f - 15.0f) + 10.0f);
    const float uy = ry * ry * ry * (ry * (ry * 6.0f - 15.0f) + 10.0f);
    const float uz = rz * rz * rz * (rz * (rz * 6.0f - 15.0f) + 10.0f);
    float f1x = fx + 1.f, f1y = fy + 1.f, f1z = fz + 1.f;
    if (fabsf(f1x - freq) < 0.001f) f1x = freq;
    if (fabsf(f1y - freq) < 0.001f) f1y = freq;
    if (fabsf(f1z - freq) < 0.001f) f1z = freq;
    const float nnn = ref_dot(ref_index(fx, fy, fz), rx, ry, rz);
    const float nnp = ref_dot(ref_index(fx, fy, f1z), rx, ry, rz - 1.f);
    const float npn = ref_dot(ref_index(fx, f1y, fz), rx, ry - 1.f, rz);
    const float npp = ref_dot(ref_index(fx, f1y, f1z), rx, ry - 1.f, rz - 1.f);
    const float pnn = ref_dot(ref_index(f1x, fy, fz), rx - 1.f, ry, rz);
    const float pnp = ref_dot(ref_index(f1x, fy, f1z), rx - 1.f, ry, rz - 1.f);
    const float ppn = ref_dot(ref_index(f1x, f1y, fz), rx - 1.f, ry - 1.f, rz);
    const float ppp = ref_dot(ref_index(f1x, f1y, f1z), rx - 1.f, ry - 1.f, rz - 1.f);
    const float nn = ref_lerp(nnn, pnn, ux), np = ref_lerp(nnp, pnp, ux);
    const float pn = ref_lerp(npn, ppn, ux), pp = ref_lerp(npp, ppp, ux);
    const float n = ref_lerp(nn, pn, uy), q = ref_lerp(np, pp, uy);
    return ref_lerp(n, q, uz);
}

__device__ float ref_fbm(float x, float y, float z, float freq) {  // ImageUtils.cpp:75-87, 4 octaves
    float noise = 0.0f, weight = 1.0f, total = 0.0f;
#pragma unroll 1
    for (int i = 0; i < 4; i++) {
        total += weight;
        noise += weight * ref_perlin(x, y, z, freq);
        freq *= 2.0f;
        weight *= 0.4f;
    }
    return __fdiv_rn(noise, total);
}

__device__ __forceinline__ float ref_quot(float fa, float fb) {
    const double EPS = 0.0005;
    return (float)((double)(fb - fa) / (double)(2.f * EPS));
}

// One thread per texel: the curl vector of ImageUtils.cpp:130-169 at (col/128, row/128).
__global__ void __launch_bounds__(128) ref_curl_vectors(float* curls) {
    const int col = threadIdx.x, row = blockIdx.x;
    const double EPS = 0.0005;
    const float px = __fdiv_rn((float)col, 128.0f), py = __fdiv_rn((float)row, 128.0f);
    const float xm = (float)((double)px - EPS), xp = (float)((double)px + EPS);
    const float ym = (float)((double)py - EPS), yp = (float)((double)py + EPS);
    const float F = 3.f;
    const float dydx = ref_quot(ref_fbm(xm, py, 0.5f, F), ref_fbm(xp, py, 0.5f, F));
    const float dxdy = ref_quot(ref_fbm(px, ym, 0.5f, F), ref_fbm(px, yp, 0.5f, F));
    const float dxdz = ref_quot(ref_fbm(px, 0.5f, ym, F), ref_fbm(px, 0.5f, yp, F));
    const float dzdx = ref_quot(ref_fbm(xm, 0.5f, py, F), ref_fbm(xp, 0.5f, py, F));
    const float dzdy = ref_quot(ref_fbm(0.5f, ym, px, F), ref_fbm(0.5f, yp, px, F));
    const float dydz = ref_quot(ref_fbm(0.5f, py, xm, F), ref_fbm(0.5f, py, xp, F));
    float* c = curls + 3 * ((size_t)row * 128 + col);
    c[0] = dzdy - dydz;
    c[1] = dxdz - dzdx;
    c[2] = dydx - dxdy;
}

// One block: per-channel min/max over the 128x128 vectors (ImageUtils.cpp:179-198), then the
// remap to [0,1] and 8-bit rounding (ImageUtils.cpp:200-219).
__global__ void __launch_bounds__(1024) ref_curl_normalize(const float* curls, float* bounds, uchar4* out) {
    __shared__ float s_lo[3][32], s_hi[3][32];
    float lo[3] = {3.402823466e+38f, 3.402823466e+38f, 3.402823466e+38f};
    float hi[3] = {-3.402823466e+38f, -3.402823466e+38f, -3.402823466e+38f};
    for (int i = threadIdx.x; i < 128 * 128; i += blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            lo[k] = fminf(lo[k], curls[3 * i + k]);
            hi[k] = fmaxf(hi[k], curls[3 * i + k]);
        }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = fminf(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = fmaxf(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0)
        for (int k = 0; k < 3; ++k) {
            s_lo[k][warp] = lo[k];
            s_hi[k][warp] = hi[k];
        }
    __syncthreads();
    if (threadIdx.x < 3) {
        const int k = threadIdx.x;
        float a = s_lo[k][0], b = s_hi[k][0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            a = fminf(a, s_lo[k][w]);
            b = fmaxf(b, s_hi[k][w]);
        }
        bounds[k] = a;
        bounds[3 + k] = b;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 128 * 128; i += blockDim.x) {
        unsigned char b[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float m = 0.f + (__fdiv_rn(curls[3 * i + k] - bounds[k], bounds[3 + k] - bounds[k]) * (1.f - 0.f));
            b[k] = (unsigned char)(int)roundf(m * 255.f);
        }
        out[i] = make_uchar4(b[0], b[1], b[2], 255);
    }
}

__global__ void hash3_kernel(const int* xyz, uint32_t s, size_t n, uint32_t* out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = hash3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], s);
}

__global__ void ref_hash_kernel(const float* xyz, size_t n, float* out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float d = xyz[3 * i] * 12.9898f + xyz[3 * i + 1] * 78.233f;
    d = d + xyz[3 * i + 2] * 47.387f;
    float v = mmx::mm_sinf_cr(d) * 43758.5453f;
    out[i] = v - floorf(v);
}

}  // namespace noise

int launch_hash_stage(int which, const void* in, uint32_t seed, size_t n, void* out, cudaStream_t s) {
    const unsigned blocks = (unsigned)((n + 255) / 256);
    if (which == 0)
        noise::hash3_kernel<<<blocks, 256, 0, s>>>((const int*)in, seed, n, (uint32_t*)out);
    else
        noise::ref_hash_kernel<<<blocks, 256, 0, s>>>((const float*)in, n, (float*)out);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "hash stage launch");
    count_launch();
    return MM_OK;
}

int launch_noise(int kind, uint32_t seed, int w, int h, int d, uint8_t* out, cudaStream_t s) {
    using namespace noise;
    switch (kind) {
        case MM_NOISE_LOWRES_PERLIN_WORLEY:
        case MM_NOISE_HIRES_WORLEY: {
            dim3 grid((w + 31) / 32, (h + 7) / 8, d);
            volume_kernel<<<grid, dim3(32, 8), 0, s>>>(kind, seed, w, reinterpret_cast<uchar4*>(out));
            break;
        }
        case MM_NOISE_CURL2D:
            curl_kernel<<<dim3((w + 31) / 32, (h + 7) / 8), dim3(32, 8), 0, s>>>(seed, w, h,
                                                                                 reinterpret_cast<uchar2*>(out));
            break;
        case MM_NOISE_WEATHER:
            weather_kernel<<<dim3((w + 31) / 32, (h + 7) / 8), dim3(32, 8), 0, s>>>(seed, w, h,
                                                                                    reinterpret_cast<uchar4*>(out));
            break;
        default:
            return fail(MM_ERR_INVALID_ARGUMENT, "launch_noise: kind %d", kind);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "noise kernel launch");
    count_launch();
    return MM_OK;
}

int launch_ref_curl(uint8_t* out_rgba, float* scratch_curl, float* scratch_bounds, cudaStream_t s) {
    noise::ref_curl_vectors<<<128, 128, 0, s>>>(scratch_curl);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "ref_curl_vectors launch");
    noise::ref_curl_normalize<<<1, 1024, 0, s>>>(scratch_curl, scratch_bounds, reinterpret_cast<uchar4*>(out_rgba));
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "ref_curl_normalize launch");
    count_launch(2);
    return MM_OK;
}

}  // namespace mm
