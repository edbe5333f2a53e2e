// post_kernel.cuh - the reference's post-processing chain as CUDA kernels, headless: god rays
// (god-ray.frag:41-76), radial blur (radialBlur.frag:36-63), the mesh drawn over the blurred
// sky (VulkanApplication.cpp:955-966) and the Uncharted-2 tonemap with vignette
// (tonemap.frag:11-33) into an 8-bit image laid out as the B8G8R8A8 swapchain (or R8G8B8A8).
//
// The reference runs each pass as a full-screen quad into an RGBA32F framebuffer.  The chain here
// is two kernels: the god-ray term (the only value of the god-ray framebuffer that is not a copy
// of the cloud image) goes to a float plane; one fused kernel then reads its ten radial-blur taps
// from that plane, the centre colour from the cloud image, overlays the mesh, tonemaps and stores
// 8 bits.  In production arithmetic the chain first copies the cloud alpha into a float plane so
// that both tap loops run on the texture unit (one filtered fetch per tap instead of four loads and
// three lerps; 8-bit fixed-point filter weights).  The three single-pass kernels (float4 in,
// float4 or 8 bits out) exist for callers that keep the reference's intermediate framebuffers.
//
// Sampling (shared with the CPU restatement): pixel (x, y) has fragUV = ((x + 0.5) / W,
// (y + 0.5) / H); a fetch at the fragment's own uv is the texel itself (a texel centre); taps
// elsewhere are bilinear with float weights and CLAMP_TO_EDGE (VulkanApplication.cpp:1290-1305).
// Per-launch constants (the sun's NDC position (proj * view) * location / w, sun colour *
// intensity, the tonemap's white-point scale) are computed on the host in IEEE float.
//
// kExact: the shaders' arithmetic in a -fmad=false translation unit with mm_math.h's pow
// (bit-identical to the CPU restatement); otherwise FMA contraction and the SFU exp2/log2 pow.
#ifndef MM_POST_KERNEL_CUH_
#define MM_POST_KERNEL_CUH_

#include <cuda_runtime.h>
#include <stdint.h>

#include "mm_internal.h"
#include "mm_math.h"

namespace mm {

struct PostLaunch {
    const float* src;  // float4 rows
    size_t src_pitch;  // bytes
    float4* dst;       // float4 rows (god rays, radial blur)
    size_t dst_pitch;
    float* plane;      // god-ray term, float rows (chain)
    size_t plane_pitch;
    const float4* mesh;  // optional mesh layer (chain), float4 rows; a != 0 marks mesh pixels
    size_t mesh_pitch;
    uint8_t* out8;       // 8-bit output (tonemap, chain)
    size_t out8_pitch;
    float* aplane;       // fast chain: the cloud image's alpha, float rows (pitch = plane_pitch)
    cudaTextureObject_t atex, gtex;  // fast chain: LINEAR / CLAMP texture objects on aplane and plane
    int width, height;
    int night;         // sun.direction.y < 0: both passes copy the colour, alpha 1
    float sun_x, sun_y;  // sun position in NDC
    float kr, kg, kb;    // sun.color.rgb * sun.intensity
    float whitemap;      // 1 / uc2(50.2)
    int bgra;
};

namespace post {

// Channel `ch` of texel (x, y) of float rows with `stride` floats per texel.
struct Plane {
    const float* p;
    size_t pitch;  // bytes
    int stride, ch, w, h;
    __device__ __forceinline__ float at(int x, int y) const {
        return __ldg(reinterpret_cast<const float*>(reinterpret_cast<const char*>(p) + (size_t)y * pitch) +
                     (size_t)x * stride + ch);
    }
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }

__device__ __forceinline__ float bilinear(const Plane& pl, float u, float v) {
    const float x = u * (float)pl.w - 0.5f, y = v * (float)pl.h - 0.5f;
    const float fx = floorf(x), fy = floorf(y);
    const float ax = x - fx, ay = y - fy;
    const int ix = (int)fminf(fmaxf(fx, -1.0f), (float)pl.w), iy = (int)fminf(fmaxf(fy, -1.0f), (float)pl.h);
    const int x0 = clampi(ix, 0, pl.w - 1), x1 = clampi(ix + 1, 0, pl.w - 1);
    const int y0 = clampi(iy, 0, pl.h - 1), y1 = clampi(iy + 1, 0, pl.h - 1);
    const float a = mixf(pl.at(x0, y0), pl.at(x1, y0), ax);
    const float b = mixf(pl.at(x0, y1), pl.at(x1, y1), ax);
    return mixf(a, b, ay);
}

// Tap samplers: float-weight bilinear from memory (both arithmetic modes of the single passes, the
// exact chain) or the texture unit's LINEAR filter (the fast chain; 8-bit fixed-point weights).
struct SoftTaps {
    Plane pl;
    __device__ __forceinline__ float operator()(float u, float v) const { return bilinear(pl, u, v); }
};
struct TexTaps {
    cudaTextureObject_t t;
    __device__ __forceinline__ float operator()(float u, float v) const { return tex2D<float>(t, u, v); }
};

__device__ __forceinline__ void frag(int x, int y, int w, int h, float* px, float* py, float* u, float* v) {
    *u = ((float)x + 0.5f) / (float)w;
    *v = ((float)y + 0.5f) / (float)h;
    *px = *u * 2.0f - 1.0f;
    *py = *v * 2.0f - 1.0f;
}

// god-ray.frag:56-75 for the fragment at NDC (px, py) with centre alpha ca.
template <class Taps>
__device__ __forceinline__ float god_ray_term(const PostLaunch& p, const Taps& alpha, float px, float py, float ca) {
    const float weight_density = 1.0f / 8.0f * 0.75f;  // SAMPLE_WEIGHT * DENSITY
    const float dx = (px - p.sun_x) * weight_density, dy = (py - p.sun_y) * weight_density;
    float accum = ca * 0.5f;
    float decay = 1.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        px = px - dx;
        py = py - dy;
        float amt = alpha(px * 0.5f + 0.5f, py * 0.5f + 0.5f) * 0.5f;
        amt = amt * (1.0f / 8.0f * decay);
        accum = accum + amt;
        decay = decay * 0.99f;
    }
    return accum * 0.9f;
}

// radialBlur.frag:51-60: the mean of ten taps of the god-ray term along the line to the sun.
template <class Taps>
__device__ __forceinline__ float radial_term(const PostLaunch& p, const Taps& g, float px, float py) {
    float lx = p.sun_x - px, ly = p.sun_y - py;
    const float dist = sqrtf(lx * lx + ly * ly);
    lx = lx / dist;
    ly = ly / dist;
    const float taps[10] = {-0.08f, -0.05f, -0.03f, -0.02f, -0.01f, 0.01f, 0.02f, 0.03f, 0.05f, 0.08f};
    float accum = 0.0f;
#pragma unroll
    for (int i = 0; i < 10; ++i) {
        const float ox = taps[i] * lx * 1.5f * dist, oy = taps[i] * ly * 1.5f * dist;
        accum = accum + g((px + ox) * 0.5f + 0.5f, (py + oy) * 0.5f + 0.5f) * 1.1f;
    }
    return accum / 10.0f;
}

__device__ __forceinline__ float uc2(float x) {  // tonemap.frag:11-14
    return ((x * (0.15f * x + 0.1f * 0.5f) + 0.2f * 0.02f) / (x * (0.15f * x + 0.5f) + 0.2f * 0.3f)) - 0.02f / 0.3f;
}

template <bool E>
__device__ __forceinline__ float powf_(float x, float y) {
    if (E) return mmx::mm_powf(x, y);
    return exp2f(y * __log2f(x));
}

__device__ __forceinline__ uint32_t unorm8(float v) { return (uint32_t)__float2int_rn(fminf(fmaxf(v, 0.0f), 1.0f) * 255.0f); }

// tonemap.frag:24-33 for colour c at uv (u, v); packed 8-bit texel.
template <bool E>
__device__ __forceinline__ uint32_t tonemap8(const PostLaunch& p, float r, float g, float b, float u, float v) {
    const float inv_gamma = 1.0f / 2.2f;
    const float du = u - 0.5f, dv = v - 0.5f;
    const float vignette = du * du + dv * dv;
    const float c0 = powf_<E>(uc2(0.7f * r) * p.whitemap, inv_gamma);
    const float c1 = powf_<E>(uc2(0.7f * g) * p.whitemap, inv_gamma);
    const float c2 = powf_<E>(uc2(0.7f * b) * p.whitemap, inv_gamma);
    const uint32_t R = unorm8(mixf(c0, 0.1f, vignette)), G = unorm8(mixf(c1, 0.05f, vignette)),
                   B = unorm8(mixf(c2, 0.13f, vignette));
    return p.bgra ? (B | (G << 8) | (R << 16) | (255u << 24)) : (R | (G << 8) | (B << 16) | (255u << 24));
}

__device__ __forceinline__ float4 ld4(const float* base, size_t pitch, int x, int y) {
    return __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(base) + (size_t)y * pitch) + x);
}

// god-ray.frag as one pass: dst = (src.rgb, term) (plane == nullptr) or the term alone into the plane.
template <bool E>
__global__ void __launch_bounds__(256) god_rays_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    const float4 c = ld4(p.src, p.src_pitch, x, y);
    float term = 1.0f;
    if (!p.night) {
        float px, py, u, v;
        frag(x, y, p.width, p.height, &px, &py, &u, &v);
        const SoftTaps alpha{Plane{p.src, p.src_pitch, 4, 3, p.width, p.height}};
        term = god_ray_term(p, alpha, px, py, c.w);
    }
    if (p.plane) {
        *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.plane) + (size_t)y * p.plane_pitch) + x) = term;
    } else {
        *(reinterpret_cast<float4*>(reinterpret_cast<char*>(p.dst) + (size_t)y * p.dst_pitch) + x) =
            make_float4(c.x, c.y, c.z, term);
    }
}

// radialBlur.frag as one pass: dst = (k * blur(src.a) + 0.5 src.rgb, 1).
template <bool E>
__global__ void __launch_bounds__(256) radial_blur_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    const float4 c = ld4(p.src, p.src_pitch, x, y);
    float4 o = make_float4(c.x, c.y, c.z, 1.0f);
    if (!p.night) {
        float px, py, u, v;
        frag(x, y, p.width, p.height, &px, &py, &u, &v);
        const SoftTaps alpha{Plane{p.src, p.src_pitch, 4, 3, p.width, p.height}};
        const float a = radial_term(p, alpha, px, py);
        o.x = p.kr * a + 0.5f * c.x;
        o.y = p.kg * a + 0.5f * c.y;
        o.z = p.kb * a + 0.5f * c.z;
    }
    *(reinterpret_cast<float4*>(reinterpret_cast<char*>(p.dst) + (size_t)y * p.dst_pitch) + x) = o;
}

// tonemap.frag as one pass: src.rgb -> 8 bits.
template <bool E>
__global__ void __launch_bounds__(256) tonemap_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    const float4 c = ld4(p.src, p.src_pitch, x, y);
    float px, py, u, v;
    frag(x, y, p.width, p.height, &px, &py, &u, &v);
    *(reinterpret_cast<uint32_t*>(p.out8 + (size_t)y * p.out8_pitch) + x) = tonemap8<E>(p, c.x, c.y, c.z, u, v);
}

// Radial blur of the god-ray plane + mesh overlay + tonemap, fused: src = the cloud image (whose
// colour the god-ray framebuffer copies), plane = the god-ray term (read through the texture unit
// when kTex).
template <bool E, bool kTex = false>
__global__ void __launch_bounds__(256) chain_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    float px, py, u, v;
    frag(x, y, p.width, p.height, &px, &py, &u, &v);
    float r, g, b;
    float4 m = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (p.mesh) m = __ldg(reinterpret_cast<const float4*>(reinterpret_cast<const char*>(p.mesh) + (size_t)y * p.mesh_pitch) + x);
    if (m.w != 0.0f) {
        r = m.x;
        g = m.y;
        b = m.z;
    } else {
        const float4 c = ld4(p.src, p.src_pitch, x, y);
        if (p.night) {
            r = c.x;
            g = c.y;
            b = c.z;
        } else {
            float a;
            if (kTex) {
                a = radial_term(p, TexTaps{p.gtex}, px, py);
            } else {
                const SoftTaps term{Plane{p.plane, p.plane_pitch, 1, 0, p.width, p.height}};
                a = radial_term(p, term, px, py);
            }
            r = p.kr * a + 0.5f * c.x;
            g = p.kg * a + 0.5f * c.y;
            b = p.kb * a + 0.5f * c.z;
        }
    }
    *(reinterpret_cast<uint32_t*>(p.out8 + (size_t)y * p.out8_pitch) + x) = tonemap8<E>(p, r, g, b, u, v);
}

// Fast chain, first kernel: the cloud image's alpha into a float plane (read by the texture unit).
template <bool E>
__global__ void __launch_bounds__(256) alpha_plane_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.aplane) + (size_t)y * p.plane_pitch) + x) =
        ld4(p.src, p.src_pitch, x, y).w;
}

// Fast chain, second kernel: the god-ray term with its eight taps filtered by the texture unit.
template <bool E>
__global__ void __launch_bounds__(256) god_rays_tex_kernel(PostLaunch p) {
    const int x = blockIdx.x * 32 + threadIdx.x, y = blockIdx.y * 8 + threadIdx.y;
    if (x >= p.width || y >= p.height) return;
    float px, py, u, v;
    frag(x, y, p.width, p.height, &px, &py, &u, &v);
    const float ca = *(reinterpret_cast<const float*>(reinterpret_cast<const char*>(p.aplane) + (size_t)y * p.plane_pitch) + x);
    *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.plane) + (size_t)y * p.plane_pitch) + x) =
        god_ray_term(p, TexTaps{p.atex}, px, py, ca);
}

// which: 0 god rays, 1 radial blur, 2 tonemap, 3 chain (god-ray plane, then the fused kernel),
// 4 fast chain (alpha plane, god-ray plane with texture-unit taps, fused kernel with texture-unit taps).
template <bool E>
int launch(const PostLaunch& p, int which, cudaStream_t s) {
    const dim3 block(32, 8), grid((p.width + 31) / 32, (p.height + 7) / 8);
    switch (which) {
        case 0: god_rays_kernel<E><<<grid, block, 0, s>>>(p); break;
        case 1: radial_blur_kernel<E><<<grid, block, 0, s>>>(p); break;
        case 2: tonemap_kernel<E><<<grid, block, 0, s>>>(p); break;
        case 4:
            if (!p.night) {
                alpha_plane_kernel<E><<<grid, block, 0, s>>>(p);
                count_launch();
                MM_CUDA_TRY(cudaGetLastError());
                god_rays_tex_kernel<E><<<grid, block, 0, s>>>(p);
                count_launch();
                MM_CUDA_TRY(cudaGetLastError());
            }
            chain_kernel<E, true><<<grid, block, 0, s>>>(p);
            break;
        default:
            if (!p.night) {
                god_rays_kernel<E><<<grid, block, 0, s>>>(p);
                count_launch();
                MM_CUDA_TRY(cudaGetLastError());
            }
            chain_kernel<E><<<grid, block, 0, s>>>(p);
            break;
    }
    count_launch();
    MM_CUDA_TRY(cudaGetLastError());
    return MM_OK;
}

}  // namespace post
}  // namespace mm

#endif  // MM_POST_KERNEL_CUH_
