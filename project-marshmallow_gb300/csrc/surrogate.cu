// surrogate.cu - the cloud march with the learned sun-cone surrogate, and its training samples.
//
// The six-tap sun cone of every accumulated sample (compute-clouds.comp:441-453) is replaced by the
// cone taps' low-res cloudTest densities (all six by default, two with MM_SUR_TAPS=2) and a small MLP
// that predicts Beer's transmittance exp(-sum) of the six-tap density sum, i.e. the taps' hi-res
// erosion (two curl + hi-res fetches per tap) is what the network stands in for.  Because accumDensity never depends on the cone
// (compute-clouds.comp:464-466), the march can run without the prediction: the front-to-back blend
//     T_k = A_{k-1} T_{k-1} + (1 - A_{k-1}) y_k,   y_k = inScatter_k * HG * beers_k
// (A = accumDensity before the sample) is linear in the beers_k, so
//     T_n = U_n + sum_{k deferred} c_k beers_k exp(l_n - l_k),
// with c_k = inScatter_k HG (1 - A_{k-1}), l_k = sum_{j=2..k} ln A_{j-1} (l of the ray's last sample
// is l_n), and U the blend run with y_k = 0 for deferred samples.  The march writes one record per
// deferred sample: 16 BF16 features (32 B) and (ray, g_k = ln c_k - l_k) (8 B); per ray it keeps
// (U, accum, rd.y) and (l_n, beers mix factor).  The MLP evaluates all records on the tensor cores
// and its epilogue adds c_k beers_k exp(l_n - l_k) = beers_k exp(g_k + l_n) to the ray's U (an
// atomic per record; no prediction goes back to memory), and a composite kernel finishes the pixels
// (compute-clouds.comp:484-499).  A sample that finds the record buffer full takes the plain cone
// inline.
//
// Features, six-tap set (features6): relative height, low-res density of the sample, cloudTest
// density at cone taps 0..5, sun direction (3), weather coverage and type at the sample, fractional
// low-res texture coordinate of the wind-displaced point (x, z, y).  Two-tap set (features):
// relative height, sample density, taps 1 and 4, sun direction, coverage, type, fractional
// coordinate (3), sin/cos of 2 pi times its x and z.  The view direction is not an input: the cone
// does not depend on it (HG and the beers/beersMod mix stay analytic).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "march_kernel.cuh"
#include "tc.cuh"

namespace mm {
namespace sur {

using namespace march;

constexpr int kFeatures = 16;

#ifndef MM_SUR_TAPS
#define MM_SUR_TAPS 6  // cone taps whose cloudTest density is a network input (2 or 6)
#endif

// 16 features with all six cone-tap densities: relative height, sample density, tap densities
// 0..5, sun direction, weather coverage and type, fractional low-res coordinate x and z.
__device__ __forceinline__ void features6(float* out, const Frame& f, const Geo& g, float lo, const float* d6,
                                          float cov, float type) {
    out[0] = g.rh;
    out[1] = lo;
#pragma unroll
    for (int i = 0; i < 6; ++i) out[2 + i] = d6[i];
    out[8] = f.sunDir.x;
    out[9] = f.sunDir.y;
    out[10] = f.sunDir.z;
    out[11] = cov;
    out[12] = type;
    const float ux = 0.00002f * g.sp.x, uz = 0.00002f * g.sp.z;
    out[13] = ux - floorf(ux);
    out[14] = uz - floorf(uz);
    out[15] = 0.00002f * g.sp.y - floorf(0.00002f * g.sp.y);
}

// 16 features of one accumulated sample (shared by the training-sample generator and the march).
__device__ __forceinline__ void features(float* out, const Frame& f, const Geo& g, float lo, float da, float db,
                                         float cov, float type) {
    out[0] = g.rh;
    out[1] = lo;
    out[2] = da;
    out[3] = db;
    out[4] = f.sunDir.x;
    out[5] = f.sunDir.y;
    out[6] = f.sunDir.z;
    out[7] = cov;
    out[8] = type;
    const float ux = 0.00002f * g.sp.x, uy = 0.00002f * g.sp.y, uz = 0.00002f * g.sp.z;
    const float fx = ux - floorf(ux), fy = uy - floorf(uy), fz = uz - floorf(uz);
    out[9] = fx;
    out[10] = fy;
    out[11] = fz;
    float s, c;
    __sincosf(6.2831853f * fx, &s, &c);
    out[12] = s;
    out[13] = c;
    __sincosf(6.2831853f * fz, &s, &c);
    out[14] = s;
    out[15] = c;
}

__device__ __forceinline__ void store_features(__nv_bfloat16* X, unsigned idx, const float* v) {
    uint4* dst = reinterpret_cast<uint4*>(X + (size_t)idx * kFeatures);
    dst[0] = tc::pack8_bf16(v);
    dst[1] = tc::pack8_bf16(v + 8);
}

// The plain six-tap cone at position pos (:441-453), also returning the six tap densities.
template <int S>
__device__ __forceinline__ float plain_cone(const MarchLaunch& p, const Frame& f, const V3* cone, V3 pos, float stepSize,
                                            float* d6, Work& w) {
    float dal = 0.0f;
#pragma unroll 1
    for (int i = 0; i < 6; ++i) {
        const Geo gl = geo_at<false>(f, pos + 3.0f * stepSize * cone[i]);
        float d = cloud_test<false, S>(p, f, gl, w.test);
        d6[i] = d;
        if (d > 0.0f) dal += cloud_hires<false, S>(p, gl, stepSize, d, w.hires);
    }
    return dal;
}

struct Records {
    __nv_bfloat16* X;    // [cap][16] features
    float2* meta;        // [cap]: ray index (int bits), g_k = ln c_k - l_k
    unsigned int* count;
    float4* ray;         // [height][width]: U, accum, rd.y (rd.y < 0: a killed ray, pixel final)
    float2* ray_b;       // [height][width]: l_n, beers mix factor -cos(theta)/2 + 1/2
    int cap;
};

// ------------------------------------------------------------------------------ surrogate march

template <int S, bool C>
// Resident blocks per SM for the surrogate march (its record writes need more registers than the
// plain march: 9 blocks leave 56 per thread and no spills).
#ifndef MM_SUR_MIN_BLOCKS
#define MM_SUR_MIN_BLOCKS 9
#endif

__global__ void __launch_bounds__(MM_TILED_WARPS * 32, MM_SUR_MIN_BLOCKS) march_sur_kernel(MarchLaunch p, Records rec) {
    __shared__ V3 s_cone[6];
    cone_offsets(p.u, s_cone);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int px = tile_px((int)blockIdx.x, warp, lane);
    const int py = tile_py((int)blockIdx.y, warp, lane);
    if (px >= p.width || py >= p.height) return;
    const Frame f = make_frame<false>(p);
    Work w;
    const Ray r = ray_setup<false, S>(p, f, px, py);
    const size_t ray_index = (size_t)py * p.width + px;
    // Background and alpha go to the image now; the composite kernel reads them back.
    store_pixel(p, px, py, make_float4(r.bg.x, r.bg.y, r.bg.z, r.alpha), CUDART_INF_F);
    if (r.killed) {
        rec.ray[ray_index] = make_float4(1.0f, 0.0f, -1.0f, 0.0f);  // rd.y < 0: the composite leaves the pixel
        return;
    }
    const V3 rd = r.rd;
    const float mixf_beers = -r.cosTheta * 0.5f + 0.5f;
    float accum = 0.0f, U = 1.0f, l = 0.0f;
    float stepSize = 0.05f * f.thickness;
    bool noHits = true;
    int misses = 0, steps = 0, nsamp = 0;
    float firstT = CUDART_INF_F;
    int iterations = 0;
    for (float t = r.t0; t < r.t1 && iterations < kMaxIterations; t += stepSize, ++iterations) {
        ++w.iter;
        const V3 pos = f.cam + t * rd;
        const Geo g = geo_at<false>(f, pos);
        const TestFetch tf = test_fetch<false, S>(p, f, g);
        float density = test_finish<false>(f, g, tf, w.test);
        const float loDensity = density;
        if (density > 0.0f) {
            misses = 0;
            if (noHits) {
                t -= stepSize;
                stepSize *= 0.3f;
                noHits = false;
                continue;
            }
            density = cloud_hires<false, S>(p, g, stepSize, density, w.hires);
            if (density < 0.0001f) continue;
            // the deferred blend weight of this sample (:461-464 without beers)
            float inScatter = 0.09f + exp2f(remapClamped<false>(g.rh, 0.3f, 0.85f, 0.5f, 2.0f) * __log2f(loDensity));
            inScatter *= exp2f(0.8f * __log2f(remapClamped<false>(g.rh, 0.07f, 0.34f, 0.1f, 1.0f)));
            if (nsamp > 0) l += __logf(accum);
            const float ck = inScatter * r.hg * (1.0f - accum);
            unsigned idx = 0xffffffffu;
            if (rec.cap > 0) idx = atomicAdd(rec.count, 1u);
            if (idx < (unsigned)rec.cap) {
                float v[kFeatures];
#if MM_SUR_TAPS == 6
                float d6[6];
#pragma unroll 1
                for (int i = 0; i < 6; ++i) d6[i] = cloud_test<false, S>(p, f, geo_at<false>(f, pos + 3.0f * stepSize * s_cone[i]), w.test);
                features6(v, f, g, loDensity, d6, tf.cov, tf.type);
#else
                const V3 l1 = pos + 3.0f * stepSize * s_cone[1], l4 = pos + 3.0f * stepSize * s_cone[4];
                const Geo g1 = geo_at<false>(f, l1), g4 = geo_at<false>(f, l4);
                const float da = cloud_test<false, S>(p, f, g1, w.test);
                const float db = cloud_test<false, S>(p, f, g4, w.test);
                features(v, f, g, loDensity, da, db, tf.cov, tf.type);
#endif
                store_features(rec.X, idx, v);
                rec.meta[idx] = make_float2(__int_as_float(py * p.width + px), __logf(ck) - l);
                U = accum * U;  // y_k = 0 in U; the accumulate kernel adds it
            } else {            // buffer full: the plain cone, inline
                float d6[6];
                const float dal = plain_cone<S>(p, f, s_cone, pos, stepSize, d6, w);
                float beers = __expf(-dal);
                beers = mixf(beers, fmaxf(beers, 0.7f * __expf(-0.25f * dal)), mixf_beers);
                U = accum * U + ck * beers;
            }
            ++nsamp;
            ++w.acc;
            if (firstT == CUDART_INF_F) firstT = t;
            accum += density;
        } else if (!noHits) {
            misses++;
            if (misses >= 10) {
                noHits = true;
                stepSize = __fdividef(stepSize, 0.3f);
            }
        }
        if (accum > 0.99f) {
            accum = 1.0f;
            break;
        }
        if (++steps > 100) break;
    }
    rec.ray[ray_index] = make_float4(U, accum, rd.y, 0.0f);
    rec.ray_b[ray_index] = make_float2(l, mixf_beers);
    if (p.depth) *(reinterpret_cast<float*>(reinterpret_cast<char*>(p.depth) + (size_t)py * p.depth_pitch) + px) = firstT;
    if (C) flush_work(p.counters, w);
}

// Finishes the pixels of a surrogate frame (:484-499).
__global__ void composite_kernel(MarchLaunch p, Records rec) {
    const int px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y;
    if (px >= p.width) return;
    const float4 rr = rec.ray[(size_t)py * p.width + px];  // U, accum, rd.y
    if (rr.z < 0.0f) return;  // below the horizon: stored during the march
    const Frame f = make_frame<false>(p);
    float4* out = reinterpret_cast<float4*>(reinterpret_cast<char*>(p.rgba) + (size_t)py * p.rgba_pitch) + px;
    const float4 bgA = *out;
    V3 rd = {0.0f, rr.z, 0.0f};
    *out = composite<false>(p.u, f, rd, V3{bgA.x, bgA.y, bgA.z}, bgA.w, rr.y, rr.x);
}

// ------------------------------------------------------------------------------ training samples

struct SampleParams {
    MarchLaunch p;   // textures of one seed; uniforms unused except the camera
    __nv_bfloat16* X;
    float* T;
    unsigned int* count;
    int cap;
    uint32_t seed;
    unsigned long long first;  // index of the first candidate
    float half_extent;         // horizontal half-size of the sampled region (m)
};

__device__ __forceinline__ uint32_t h32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

__device__ __forceinline__ float u01(uint32_t& s) {
    s = h32(s + 0x9E3779B9u);
    return (float)(s >> 8) * 0x1p-24f;
}

// One candidate per thread: a uniform random point in the cloud layer, a random sun (elevation
// 0-90 deg, any azimuth) and wind time; kept if the march would accumulate a sample there
// (cloudTest > 0 and cloudHiRes >= 1e-4 at the small step), with the plain cone's exp(-sum) as
// the target.
__global__ void __launch_bounds__(128) sample_kernel(SampleParams sp, unsigned long long n) {
    const unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t s = h32(sp.seed * 0x85EBCA6Bu ^ h32((uint32_t)(sp.first + i)) ^ (uint32_t)((sp.first + i) >> 32));
    Frame f;
    f.cam = {0.0f, 10.0f, 0.0f};
    f.center = {0.0f, -kRadius * 0.5f * 0.995f, 0.0f};
    f.wind = {1.0f, 0.05f, 1.0f};
    f.time = 2.0f * u01(s);
    f.thickness = 0.5f * kRadius * 0.02f;
    f.coverage_offset = 0.0f;
    f.wind20 = 20.0f * f.wind;
    f.wscale20 = {2.0f, 1.0f, 0.0f};
    const float el = 1.5707963f * u01(s), az = 6.2831853f * u01(s);
    const V3 dir = {cosf(el) * cosf(az), sinf(el), cosf(el) * sinf(az)};
    f.sunDir = dir;
    f.sunY = dir.y;
    // SkyManager TBN (SkyManager.cpp:55-69): columns N, dir, B
    const V3 right = fabsf(dir.y) < 0.001f ? (dir.z < 0.0f ? V3{0.0f, 1.0f, 0.0f} : V3{0.0f, -1.0f, 0.0f})
                                            : V3{0.0f, 0.0f, 1.0f};
    auto cross = [](V3 a, V3 b) { return V3{a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; };
    const V3 N = normalize<false>(cross(dir, right));
    const V3 B = normalize<false>(cross(dir, N));
    const float cx[6] = {0.0f, 0.0f, 0.1f, 0.2f, 0.0f, -0.1f}, cy[6] = {0.6f, 0.5f, 0.75f, 2.5f, 6.0f, 1.0f},
                cz[6] = {0.0f, 0.05f, 0.0f, 0.3f, 0.0f, -0.2f};
    V3 cone[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) cone[k] = N * cx[k] + dir * cy[k] + B * cz[k];
    // a point at relative height h of the layer, horizontally uniform in the square
    const float x = (2.0f * u01(s) - 1.0f) * sp.half_extent, z = (2.0f * u01(s) - 1.0f) * sp.half_extent;
    const float R = 0.5f * kRadius + u01(s) * f.thickness;
    const float yy = R * R - x * x - z * z;
    if (yy <= 0.0f) return;
    const V3 pos = {x, f.center.y + sqrtf(yy), z};
    const float stepSize = 0.05f * f.thickness * 0.3f;  // the step of every accumulated sample
    Work w;
    const Geo g = geo_at<false>(f, pos);
    const TestFetch tf = test_fetch<false, MM_SAMPLER_HARDWARE>(sp.p, f, g);
    const float lo = test_finish<false>(f, g, tf, w.test);
    if (!(lo > 0.0f)) return;
    const float hd = cloud_hires<false, MM_SAMPLER_HARDWARE>(sp.p, g, stepSize, lo, w.hires);
    if (hd < 0.0001f) return;
    float d6[6];
    const float dal = plain_cone<MM_SAMPLER_HARDWARE>(sp.p, f, cone, pos, stepSize, d6, w);
    const unsigned idx = atomicAdd(sp.count, 1u);
    if (idx >= (unsigned)sp.cap) return;
    float v[kFeatures];
#if MM_SUR_TAPS == 6
    features6(v, f, g, lo, d6, tf.cov, tf.type);
#else
    features(v, f, g, lo, d6[1], d6[4], tf.cov, tf.type);
#endif
    store_features(sp.X, idx, v);
    sp.T[idx] = __expf(-dal);
}

}  // namespace sur

int surrogate_reserve(mm_context ctx, size_t pixels) {
    using namespace sur;
    // Record capacity: 4 per pixel (a 4K frame of the benchmark sweep defers ~3 per marched ray).
    const size_t want_cap = pixels * 4;
    if (ctx->sur_cap < want_cap || ctx->sur_pixels < pixels) {
        cudaFree(ctx->sur_x);
        cudaFree(ctx->sur_meta);
        cudaFree(ctx->sur_y);
        cudaFree(ctx->sur_ray);
        ctx->sur_x = nullptr;
        ctx->sur_meta = nullptr;
        ctx->sur_y = nullptr;
        ctx->sur_ray = nullptr;
        ctx->sur_cap = 0;
        ctx->sur_pixels = 0;
        MM_CUDA_TRY(cudaMalloc(&ctx->sur_x, want_cap * kFeatures * sizeof(__nv_bfloat16)));
        MM_CUDA_TRY(cudaMalloc(&ctx->sur_meta, want_cap * sizeof(float2)));
        MM_CUDA_TRY(cudaMalloc(&ctx->sur_y, pixels * sizeof(float2)));  // per-ray (l_n, mix)
        MM_CUDA_TRY(cudaMalloc(&ctx->sur_ray, pixels * sizeof(float4)));
        ctx->sur_cap = want_cap;
        ctx->sur_pixels = pixels;
    }
    return MM_OK;
}

int launch_surrogate_frame(const MarchLaunch& p, mm_context ctx, mm_mlp net, cudaStream_t s) {
    using namespace sur;
    const size_t pixels = (size_t)p.width * p.height;
    int rr = surrogate_reserve(ctx, pixels);
    if (rr) return rr;
    Records rec;
    rec.X = (__nv_bfloat16*)ctx->sur_x;
    rec.meta = (float2*)ctx->sur_meta;
    rec.count = ctx->d_work + 1;
    rec.ray = (float4*)ctx->sur_ray;
    rec.ray_b = (float2*)ctx->sur_y;
    rec.cap = (int)(ctx->sur_cap < 0x7fffffff ? ctx->sur_cap : 0x7fffffff);
    MM_CUDA_TRY(cudaMemsetAsync(rec.count, 0, sizeof(unsigned int), s));
    dim3 grid((p.width + kBlockTileW - 1) / kBlockTileW, (p.height + kBlockTileH - 1) / kBlockTileH);
    if (p.counters)
        march_sur_kernel<MM_SAMPLER_HARDWARE, true><<<grid, MM_TILED_WARPS * 32, 0, s>>>(p, rec);
    else
        march_sur_kernel<MM_SAMPLER_HARDWARE, false><<<grid, MM_TILED_WARPS * 32, 0, s>>>(p, rec);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    int r = mlp_infer_accumulate(net, rec.X, rec.cap, rec.count, rec.meta, rec.ray_b, rec.ray, s);
    if (r) return r;
    composite_kernel<<<dim3((p.width + 127) / 128, p.height), 128, 0, s>>>(p, rec);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch(1);
    return MM_OK;
}

int launch_surrogate_samples(const MarchLaunch& p, uint32_t seed, unsigned long long first, unsigned long long n,
                             float half_extent, void* d_x, float* d_t, unsigned int* d_count, int cap,
                             cudaStream_t s) {
    sur::SampleParams sp;
    sp.p = p;
    sp.X = (__nv_bfloat16*)d_x;
    sp.T = d_t;
    sp.count = d_count;
    sp.cap = cap;
    sp.seed = seed;
    sp.first = first;
    sp.half_extent = half_extent;
    sur::sample_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(sp, n);
    MM_CUDA_TRY(cudaGetLastError());
    count_launch();
    return MM_OK;
}

}  // namespace mm
