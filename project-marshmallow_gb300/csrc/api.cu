// api.cu - the C ABI of include/mm.h: error state, textures, contexts and the march/noise entry
// points.  Replaces the Vulkan descriptor/dispatch plumbing of the reference
// (Shader.cpp:633-994, Texture.cpp, VulkanApplication.cpp:1027-1078).
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <new>

#include "mm_internal.h"

namespace mm {

namespace {
thread_local char g_last_error[512] = "";
std::atomic<uint64_t> g_launches(0);
}  // namespace

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
    va_end(ap);
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    int code = (e == cudaErrorMemoryAllocation) ? MM_ERR_OUT_OF_MEMORY
               : (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) ? MM_ERR_NO_DEVICE
                                                                                : MM_ERR_CUDA;
    return fail(code, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
}

void count_launch(uint64_t n) { g_launches += n; }

}  // namespace mm

using mm::fail;

namespace {

bool valid_kind(int k) { return k >= MM_NOISE_LOWRES_PERLIN_WORLEY && k <= MM_NOISE_REF_CURL; }

// Fills in default sizes and validates the shape of a noise request.
int resolve_desc(const mm_noise_desc* d, int* w, int* h, int* z, int* ch) {
    if (!d) return fail(MM_ERR_INVALID_ARGUMENT, "noise: null descriptor");
    if (!valid_kind(d->kind)) return fail(MM_ERR_INVALID_ARGUMENT, "noise: unknown kind %d", d->kind);
    static const int def[5][4] = {{128, 128, 128, 4}, {32, 32, 32, 4}, {128, 128, 1, 2}, {512, 512, 1, 4}, {128, 128, 1, 4}};
    const int* df = def[d->kind];
    *w = d->width ? d->width : df[0];
    *h = d->height ? d->height : df[1];
    *z = d->depth ? d->depth : df[2];
    *ch = df[3];
    const bool is3d = d->kind <= MM_NOISE_HIRES_WORLEY;
    if (*w <= 0 || *h <= 0 || *z <= 0) return fail(MM_ERR_INVALID_ARGUMENT, "noise: non-positive size");
    if (is3d && (*w != *h || *h != *z)) return fail(MM_ERR_INVALID_ARGUMENT, "noise: 3D kinds are cubes");
    if (!is3d && *z != 1) return fail(MM_ERR_INVALID_ARGUMENT, "noise: 2D kinds have depth 1");
    if (*w > 4096 || *h > 4096 || (is3d && *w > 512))
        return fail(MM_ERR_INVALID_ARGUMENT, "noise: size above the supported maximum");
    if (d->kind == MM_NOISE_REF_CURL && (*w != 128 || *h != 128))
        return fail(MM_ERR_INVALID_ARGUMENT, "noise: the reference curl is 128x128 only");
    return MM_OK;
}

// Hardware-filtered copy: CUDA array of the texel format with a LINEAR/WRAP/normalized texture
// object (the reference samplers, Texture.cpp:29-52 and 315-338).
// texel/255 rounded to FP16 (bf16 == false) or to bfloat16 (bf16 == true; round to nearest even on
// the float's bits).  A bfloat16 value of texel/255 (8 significant bits, >= 1/255 or 0) is exactly
// an FP16 value, so both are stored in FP16 arrays and filtered by the texture unit's FP16 path.
__global__ void unorm8_to_half(const uint8_t* in, __half* out, size_t n, bool bf16) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = __fdiv_rn((float)in[i], 255.0f);
    if (bf16) {
        const uint32_t b = __float_as_uint(v);
        v = __uint_as_float((b + 0x7FFFu + ((b >> 16) & 1u)) & 0xFFFF0000u);
    }
    out[i] = __float2half_rn(v);
}

int build_hw_copy(mm_texture t, int format, cudaStream_t s) {
    if (t->tex) {
        cudaDestroyTextureObject(t->tex);
        t->tex = 0;
    }
    if (t->array) {
        cudaFreeArray(t->array);
        t->array = nullptr;
    }
    const int ch = t->channels;
    cudaChannelFormatDesc cd;
    size_t elem = 1;
    if (format == MM_FORMAT_UNORM8) {
        cd = cudaCreateChannelDesc(8, ch >= 2 ? 8 : 0, ch >= 4 ? 8 : 0, ch >= 4 ? 8 : 0, cudaChannelFormatKindUnsigned);
        elem = 1;
    } else if (format == MM_FORMAT_FP16 || format == MM_FORMAT_BF16) {
        // The CUDA runtime has no bfloat16 channel kind; bfloat16-rounded texels are held in an FP16
        // array (exactly, see unorm8_to_half) and filtered by the FP16 path.
        cd = cudaCreateChannelDesc(16, ch >= 2 ? 16 : 0, ch >= 4 ? 16 : 0, ch >= 4 ? 16 : 0, cudaChannelFormatKindFloat);
        elem = 2;
    } else {
        return fail(MM_ERR_INVALID_ARGUMENT, "texture: unknown format %d", format);
    }
    const bool is3d = t->depth > 1;
    cudaExtent ext = make_cudaExtent(t->width, t->height, is3d ? t->depth : 0);
    MM_CUDA_TRY(cudaMalloc3DArray(&t->array, &cd, ext, 0));
    const size_t n = (size_t)t->width * t->height * t->depth * ch;
    const void* src = t->texels;
    void* conv = nullptr;
    if (format != MM_FORMAT_UNORM8) {
        MM_CUDA_TRY(cudaMallocAsync(&conv, n * elem, s));
        const unsigned blocks = (unsigned)((n + 255) / 256);
        unorm8_to_half<<<blocks, 256, 0, s>>>(t->texels, (__half*)conv, n, format == MM_FORMAT_BF16);
        MM_CUDA_TRY(cudaGetLastError());
        mm::count_launch();
        src = conv;
    }
    cudaMemcpy3DParms cp;
    memset(&cp, 0, sizeof(cp));
    cp.srcPtr = make_cudaPitchedPtr(const_cast<void*>(src), (size_t)t->width * ch * elem, t->width, t->height);
    cp.dstArray = t->array;
    cp.extent = make_cudaExtent(t->width, t->height, t->depth);
    cp.kind = cudaMemcpyDeviceToDevice;
    MM_CUDA_TRY(cudaMemcpy3DAsync(&cp, s));
    if (conv) MM_CUDA_TRY(cudaFreeAsync(conv, s));
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = t->array;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeWrap;
    td.filterMode = cudaFilterModeLinear;
    td.readMode = format == MM_FORMAT_UNORM8 ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
    td.normalizedCoords = 1;
    MM_CUDA_TRY(cudaCreateTextureObject(&t->tex, &rd, &td, nullptr));
    t->format = format;
    return MM_OK;
}

void release(mm_texture t) {
    if (!t) return;
    if (t->tex) cudaDestroyTextureObject(t->tex);
    if (t->array) cudaFreeArray(t->array);
    if (t->texels) cudaFree(t->texels);
    delete t;
}

int make_texture(int w, int h, int d, int ch, mm_texture* out) {
    mm_texture t = new (std::nothrow) mm_texture_s;
    if (!t) return fail(MM_ERR_OUT_OF_MEMORY, "texture: host allocation failed");
    t->width = w;
    t->height = h;
    t->depth = d;
    t->channels = ch;
    cudaGetDevice(&t->device);
    cudaError_t e = cudaMalloc(&t->texels, (size_t)w * h * d * ch);
    if (e != cudaSuccess) {
        delete t;
        return mm::cuda_fail(e, "texture texels");
    }
    *out = t;
    return MM_OK;
}

}  // namespace

mm::TexView mm::texture_view(mm_texture t) {
    mm::TexView v;
    memset(&v, 0, sizeof(v));
    if (t) {
        v.tex = t->tex;
        v.texels = t->texels;
        v.w = t->width;
        v.h = t->height;
        v.d = t->depth;
        v.channels = t->channels;
    }
    return v;
}

namespace {

mm::TexView view_of(mm_texture t) {
    mm::TexView v;
    memset(&v, 0, sizeof(v));
    if (t) {
        v.tex = t->tex;
        v.texels = t->texels;
        v.w = t->width;
        v.h = t->height;
        v.d = t->depth;
        v.channels = t->channels;
    }
    return v;
}

}  // namespace

extern "C" {

const char* mm_last_error_string(void) { return mm::g_last_error; }
int mm_abi_version(void) { return MM_ABI_VERSION; }
uint64_t mm_kernel_launch_count(void) { return mm::g_launches.load(); }

int mm_noise_texel_bytes(const mm_noise_desc* desc, size_t* bytes) {
    int w, h, d, ch;
    int r = resolve_desc(desc, &w, &h, &d, &ch);
    if (r) return r;
    if (!bytes) return fail(MM_ERR_INVALID_ARGUMENT, "noise: null size pointer");
    *bytes = (size_t)w * h * d * ch;
    return MM_OK;
}

int mm_noise_fill(const mm_noise_desc* desc, void* d_texels, size_t bytes, void* stream) {
    int w, h, d, ch;
    int r = resolve_desc(desc, &w, &h, &d, &ch);
    if (r) return r;
    if (!d_texels) return fail(MM_ERR_INVALID_ARGUMENT, "noise: null output");
    if (bytes < (size_t)w * h * d * ch) return fail(MM_ERR_INVALID_ARGUMENT, "noise: output smaller than %zu bytes",
                                                   (size_t)w * h * d * ch);
    cudaStream_t s = (cudaStream_t)stream;
    if (desc->kind == MM_NOISE_REF_CURL) {
        float* scratch = nullptr;
        MM_CUDA_TRY(cudaMallocAsync((void**)&scratch, (128 * 128 * 3 + 8) * sizeof(float), s));
        r = mm::launch_ref_curl((uint8_t*)d_texels, scratch, scratch + 128 * 128 * 3, s);
        cudaError_t e = cudaFreeAsync(scratch, s);
        if (r) return r;
        if (e != cudaSuccess) return mm::cuda_fail(e, "cudaFreeAsync");
        return MM_OK;
    }
    return mm::launch_noise(desc->kind, desc->seed, w, h, d, (uint8_t*)d_texels, s);
}

int mm_noise_hash3(const int32_t* d_xyz, uint32_t stream_seed, size_t n, uint32_t* d_out, void* stream) {
    if (!d_xyz || !d_out) return fail(MM_ERR_INVALID_ARGUMENT, "hash: null pointer");
    if (n == 0) return MM_OK;
    return mm::launch_hash_stage(0, d_xyz, stream_seed, n, d_out, (cudaStream_t)stream);
}

int mm_ref_curl_hash(const float* d_xyz, size_t n, float* d_out, void* stream) {
    if (!d_xyz || !d_out) return fail(MM_ERR_INVALID_ARGUMENT, "hash: null pointer");
    if (n == 0) return MM_OK;
    return mm::launch_hash_stage(1, d_xyz, 0, n, d_out, (cudaStream_t)stream);
}

int mm_noise_generate(const mm_noise_desc* desc, mm_texture* out, void* stream) {
    int w, h, d, ch;
    int r = resolve_desc(desc, &w, &h, &d, &ch);
    if (r) return r;
    if (!out) return fail(MM_ERR_INVALID_ARGUMENT, "noise: null output handle");
    mm_texture t = nullptr;
    if ((r = make_texture(w, h, d, ch, &t))) return r;
    cudaStream_t s = (cudaStream_t)stream;
    if ((r = mm_noise_fill(desc, t->texels, (size_t)w * h * d * ch, stream)) || (r = build_hw_copy(t, MM_FORMAT_UNORM8, s))) {
        cudaStreamSynchronize(s);
        release(t);
        return r;
    }
    *out = t;
    return MM_OK;
}

int mm_texture_create(const void* texels, int src_is_device, int width, int height, int depth, int channels, int format,
                      mm_texture* out, void* stream) {
    if (!texels || !out) return fail(MM_ERR_INVALID_ARGUMENT, "texture: null pointer");
    if (width <= 0 || height <= 0 || depth <= 0 || width > 16384 || height > 16384 || depth > 2048)
        return fail(MM_ERR_INVALID_ARGUMENT, "texture: bad size %dx%dx%d", width, height, depth);
    if (channels != 1 && channels != 2 && channels != 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "texture: channels must be 1, 2 or 4");
    mm_texture t = nullptr;
    int r = make_texture(width, height, depth, channels, &t);
    if (r) return r;
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n = (size_t)width * height * depth * channels;
    cudaError_t e = cudaMemcpyAsync(t->texels, texels, n, src_is_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, s);
    if (e != cudaSuccess) {
        release(t);
        return mm::cuda_fail(e, "texture upload");
    }
    if ((r = build_hw_copy(t, format, s))) {
        cudaStreamSynchronize(s);
        release(t);
        return r;
    }
    if (!src_is_device) cudaStreamSynchronize(s);  // the host buffer may be freed after return
    *out = t;
    return MM_OK;
}

int mm_texture_info(mm_texture t, int* w, int* h, int* d, int* ch, int* format) {
    if (!t) return fail(MM_ERR_INVALID_ARGUMENT, "texture: null handle");
    if (w) *w = t->width;
    if (h) *h = t->height;
    if (d) *d = t->depth;
    if (ch) *ch = t->channels;
    if (format) *format = t->format;
    return MM_OK;
}

int mm_texture_copy_to_host(mm_texture t, void* dst, size_t bytes) {
    if (!t || !dst) return fail(MM_ERR_INVALID_ARGUMENT, "texture: null pointer");
    const size_t n = (size_t)t->width * t->height * t->depth * t->channels;
    if (bytes < n) return fail(MM_ERR_INVALID_ARGUMENT, "texture: destination smaller than %zu bytes", n);
    MM_CUDA_TRY(cudaMemcpy(dst, t->texels, n, cudaMemcpyDeviceToHost));
    return MM_OK;
}

int mm_texture_set_format(mm_texture t, int format, void* stream) {
    if (!t) return fail(MM_ERR_INVALID_ARGUMENT, "texture: null handle");
    return build_hw_copy(t, format, (cudaStream_t)stream);
}

}  // extern "C"

namespace {

// One filtered fetch of the texture's hardware copy per coordinate: (u, v) pairs for a 2D texture,
// (u, v, w) triples for a 3D one; four floats out per fetch.
__global__ void texture_sample_kernel(cudaTextureObject_t tex, int dims, int channels, const float* coords, size_t n,
                                      float4* out) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 r;
    if (dims == 3) {
        r = tex3D<float4>(tex, coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]);
    } else if (channels == 2) {
        const float2 q = tex2D<float2>(tex, coords[2 * i], coords[2 * i + 1]);
        r = make_float4(q.x, q.y, 0.0f, 1.0f);
    } else if (channels == 1) {
        r = make_float4(tex2D<float>(tex, coords[2 * i], coords[2 * i + 1]), 0.0f, 0.0f, 1.0f);
    } else {
        r = tex2D<float4>(tex, coords[2 * i], coords[2 * i + 1]);
    }
    out[i] = r;
}

}  // namespace

extern "C" {

int mm_texture_sample(mm_texture t, const float* d_coords, size_t n, float* d_out, void* stream) {
    if (!t || (n && (!d_coords || !d_out))) return fail(MM_ERR_INVALID_ARGUMENT, "texture sample: null pointer");
    if (n == 0) return MM_OK;
    if (n > ((size_t)1 << 30)) return fail(MM_ERR_INVALID_ARGUMENT, "texture sample: too many coordinates");
    const int dims = t->depth > 1 ? 3 : 2;
    const int threads = 256;
    texture_sample_kernel<<<(unsigned)((n + threads - 1) / threads), threads, 0, (cudaStream_t)stream>>>(
        t->tex, dims, t->channels, d_coords, n, reinterpret_cast<float4*>(d_out));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return mm::cuda_fail(e, "texture_sample_kernel launch");
    mm::count_launch();
    return MM_OK;
}

int mm_texture_destroy(mm_texture t) {
    if (!t) return fail(MM_ERR_INVALID_ARGUMENT, "texture: null handle");
    release(t);
    return MM_OK;
}

int mm_context_create(mm_context* out) {
    if (!out) return fail(MM_ERR_INVALID_ARGUMENT, "context: null output");
    int dev = 0, count = 0;
    MM_CUDA_TRY(cudaGetDeviceCount(&count));
    if (count <= 0) return fail(MM_ERR_NO_DEVICE, "context: no CUDA device");
    MM_CUDA_TRY(cudaGetDevice(&dev));
    mm_context c = new (std::nothrow) mm_context_s;
    if (!c) return fail(MM_ERR_OUT_OF_MEMORY, "context: host allocation failed");
    c->device = dev;
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    mm::prepare_march_fast();
    mm::prepare_march_exact();
    cudaError_t e = cudaMalloc(&c->d_work, 64 * sizeof(unsigned int));
    if (e != cudaSuccess) {
        delete c;
        return mm::cuda_fail(e, "context scratch");
    }
    *out = c;
    return MM_OK;
}

int mm_context_destroy(mm_context c) {
    if (!c) return fail(MM_ERR_INVALID_ARGUMENT, "context: null handle");
    mm::batch_state_destroy(c);
    if (c->d_work) cudaFree(c->d_work);
    cudaFree(c->sur_x);
    cudaFree(c->sur_meta);
    cudaFree(c->sur_y);
    cudaFree(c->sur_ray);
    mm::post_state_destroy(c);
    if (c->aux_stream) {
        cudaStreamSynchronize(c->aux_stream);
        cudaStreamDestroy(c->aux_stream);
    }
    if (c->aux_fork) cudaEventDestroy(c->aux_fork);
    if (c->aux_join) cudaEventDestroy(c->aux_join);
    delete c;
    return MM_OK;
}

int mm_surrogate_generate(uint32_t first_seed, int n_seeds, int per_seed, float half_extent, void* d_x, float* d_t,
                          int* produced, void* stream) {
    if (!d_x || !d_t || n_seeds <= 0 || per_seed <= 0 || !(half_extent > 0.0f) ||
        (long long)n_seeds * per_seed > 0x7fffffffLL)
        return fail(MM_ERR_INVALID_ARGUMENT, "surrogate samples: bad arguments");
    if (((uintptr_t)d_x) % 16) return fail(MM_ERR_INVALID_ARGUMENT, "surrogate samples: features must be 16-byte aligned");
    cudaStream_t s = (cudaStream_t)stream;
    unsigned int* d_count = nullptr;
    MM_CUDA_TRY(cudaMalloc(&d_count, sizeof(unsigned int)));
    int total = 0, r = MM_OK;
    for (int k = 0; k < n_seeds && r == MM_OK; ++k) {
        const uint32_t seed = first_seed + (uint32_t)k;
        mm_texture t[4] = {nullptr, nullptr, nullptr, nullptr};
        const int kinds[4] = {MM_NOISE_WEATHER, MM_NOISE_CURL2D, MM_NOISE_LOWRES_PERLIN_WORLEY, MM_NOISE_HIRES_WORLEY};
        for (int i = 0; i < 4 && r == MM_OK; ++i) {
            mm_noise_desc d = {kinds[i], seed, 0, 0, 0};
            r = mm_noise_generate(&d, &t[i], stream);
        }
        if (r == MM_OK) {
            mm::MarchLaunch p;
            memset(&p, 0, sizeof(p));
            p.weather = mm::texture_view(t[0]);
            p.curl = mm::texture_view(t[1]);
            p.low = mm::texture_view(t[2]);
            p.hi = mm::texture_view(t[3]);
            uint8_t* xk = (uint8_t*)d_x + (size_t)total * 16 * 2;
            float* tk = d_t + total;
            cudaError_t e = cudaMemsetAsync(d_count, 0, sizeof(unsigned int), s);
            if (e != cudaSuccess) r = mm::cuda_fail(e, "surrogate count reset");
            unsigned int got = 0;
            const unsigned long long chunk = 1ull << 23;
            for (unsigned long long first = 0; r == MM_OK && got < (unsigned)per_seed && first < (1ull << 32);
                 first += chunk) {
                r = mm::launch_surrogate_samples(p, seed, first, chunk, half_extent, xk, tk, d_count, per_seed, s);
                if (r == MM_OK && (e = cudaMemcpyAsync(&got, d_count, sizeof(got), cudaMemcpyDeviceToHost, s)) != cudaSuccess)
                    r = mm::cuda_fail(e, "surrogate count");
                if (r == MM_OK && (e = cudaStreamSynchronize(s)) != cudaSuccess) r = mm::cuda_fail(e, "surrogate samples");
            }
            total += got < (unsigned)per_seed ? (int)got : per_seed;
        }
        cudaStreamSynchronize(s);
        for (int i = 0; i < 4; ++i)
            if (t[i]) mm_texture_destroy(t[i]);
    }
    cudaFree(d_count);
    if (produced) *produced = total;
    return r;
}

int mm_march_options_default(mm_march_options* o) {
    if (!o) return fail(MM_ERR_INVALID_ARGUMENT, "options: null pointer");
    memset(o, 0, sizeof(*o));
    o->pixel_mode = MM_PIXELS_FULL;
    o->sampler = MM_SAMPLER_HARDWARE;
    o->math = MM_MATH_FAST;
    o->density_format = MM_FORMAT_UNORM8;
    return MM_OK;
}

}  // extern "C"

// Checks one march request (the argument contract of mm_clouds_march).
int mm::validate_march(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_image* out,
                       const mm_march_options* opt) {
    if (!ctx || !u || !tex || !out || !opt) return fail(MM_ERR_INVALID_ARGUMENT, "march: null argument");
    const mm_march_options& o = *opt;
    if (o.pixel_mode != MM_PIXELS_FULL && o.pixel_mode != MM_PIXELS_PHASE16)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad pixel_mode %d", o.pixel_mode);
    if (o.sampler != MM_SAMPLER_HARDWARE && o.sampler != MM_SAMPLER_SOFTWARE)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad sampler %d", o.sampler);
    if (o.math != MM_MATH_FAST && o.math != MM_MATH_EXACT && o.math != MM_MATH_FAST_HALF2)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad math %d", o.math);
    if (o.math == MM_MATH_FAST_HALF2 &&
        (o.density_format == MM_FORMAT_UNORM8 || o.sampler != MM_SAMPLER_HARDWARE || o.schedule != MM_SCHEDULE_TILED))
        return fail(MM_ERR_INVALID_ARGUMENT,
                    "march: the half2 coverage test needs FP16/BF16 density, the hardware sampler and the tiled schedule");
    if (o.schedule != MM_SCHEDULE_PERSISTENT && o.schedule != MM_SCHEDULE_TILED)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad schedule %d", o.schedule);
    if (o.cone != MM_CONE_PLAIN && o.cone != MM_CONE_SURROGATE) return fail(MM_ERR_INVALID_ARGUMENT, "march: bad cone %d", o.cone);
    if (o.cone == MM_CONE_SURROGATE) {
        if (!o.surrogate) return fail(MM_ERR_INVALID_ARGUMENT, "march: surrogate cone without a network");
        if (o.pixel_mode != MM_PIXELS_FULL || o.sampler != MM_SAMPLER_HARDWARE || o.math != MM_MATH_FAST ||
            o.schedule != MM_SCHEDULE_TILED)
            return fail(MM_ERR_UNSUPPORTED, "march: the surrogate cone runs full frames with the hardware sampler, "
                                            "fast math and the tiled schedule");
    }
    if (o.density_format < MM_FORMAT_UNORM8 || o.density_format > MM_FORMAT_BF16)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad density_format %d", o.density_format);
    if (!(o.coverage_offset == o.coverage_offset) || o.coverage_offset < -1.0f || o.coverage_offset > 1.0f)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: coverage_offset must be in [-1, 1]");
    if (!out->rgba || out->width <= 0 || out->height <= 0 || out->width > 32768 || out->height > 32768)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: bad output image");
    if (out->rgba_pitch_bytes < (size_t)out->width * 16 || out->rgba_pitch_bytes % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: rgba pitch must be >= 16*width and a multiple of 16");
    if (out->depth && out->depth_pitch_bytes < (size_t)out->width * 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: depth pitch must be >= 4*width");
    if (((uintptr_t)out->rgba) % 16) return fail(MM_ERR_INVALID_ARGUMENT, "march: rgba must be 16-byte aligned");
    const mm_texture need[4] = {tex->weather, tex->curl, tex->low_res, tex->hi_res};
    const char* names[4] = {"weather", "curl", "low_res", "hi_res"};
    for (int i = 0; i < 4; ++i)
        if (!need[i]) return fail(MM_ERR_INVALID_ARGUMENT, "march: missing %s texture", names[i]);
    if (tex->low_res->depth < 2 || tex->hi_res->depth < 2 || tex->weather->depth != 1 || tex->curl->depth != 1)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: low_res/hi_res must be 3D and weather/curl 2D");
    if (tex->low_res->channels != 4 || tex->hi_res->channels < 4 || tex->weather->channels != 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: low_res, hi_res and weather must have 4 channels");
    for (int i = 0; i < 4; ++i)
        if (!need[i]->tex) return fail(MM_ERR_INVALID_ARGUMENT, "march: %s has no texture object", names[i]);
    if (u->sun.direction[1] < 0.0f && !tex->night_sky)
        return fail(MM_ERR_INVALID_ARGUMENT, "march: the sun is below the horizon and no night_sky texture is bound");
    const float ph = u->sun.color[3];
    if (o.pixel_mode == MM_PIXELS_PHASE16 && !(ph >= 0.0f && ph < 16.0f))
        return fail(MM_ERR_INVALID_ARGUMENT, "march: sun.color.a must be a pixel phase in [0, 16)");
    if (o.math == MM_MATH_EXACT && o.density_format != MM_FORMAT_UNORM8)
        return fail(MM_ERR_UNSUPPORTED, "march: exact math runs on UNORM8 density only");
    if (o.density_format != MM_FORMAT_UNORM8 &&
        (tex->low_res->format != o.density_format || tex->hi_res->format != o.density_format))
        return fail(MM_ERR_INVALID_ARGUMENT, "march: density textures are not in the requested format "
                                             "(use mm_texture_set_format)");
    if (o.density_format == MM_FORMAT_UNORM8 && o.sampler == MM_SAMPLER_HARDWARE &&
        (tex->low_res->format != MM_FORMAT_UNORM8 || tex->hi_res->format != MM_FORMAT_UNORM8))
        return fail(MM_ERR_INVALID_ARGUMENT, "march: density textures are not UNORM8");
    return MM_OK;
}

// The kernel-side record of one view.
void mm::fill_march_launch(const mm_uniforms& u, const mm_scene_textures* tex, const mm_image& out,
                           const mm_march_options& o, MarchLaunch* pp) {
    MarchLaunch& p = *pp;
    memset(&p, 0, sizeof(p));
    p.u = u;
    p.weather = view_of(tex->weather);
    p.night = view_of(tex->night_sky);
    p.curl = view_of(tex->curl);
    p.low = view_of(tex->low_res);
    p.hi = view_of(tex->hi_res);
    p.rgba = reinterpret_cast<float4*>(out.rgba);
    p.rgba_pitch = out.rgba_pitch_bytes;
    p.depth = out.depth;
    p.depth_pitch = out.depth_pitch_bytes;
    p.width = out.width;
    p.height = out.height;
    p.pixel_mode = o.pixel_mode;
    p.phase = (int)u.sun.color[3];
    p.uv_w = o.ref_uv_1080p ? 1920.0f : (float)out.width;
    p.uv_h = o.ref_uv_1080p ? 1080.0f : (float)out.height;
    p.coverage_offset = o.coverage_offset;
    p.counters = reinterpret_cast<unsigned long long*>(o.d_counters);
    march_host_consts(p);
}

extern "C" {

int mm_clouds_march(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_image* out,
                    const mm_march_options* opt, void* stream) {
    mm_march_options o;
    if (opt)
        o = *opt;
    else
        mm_march_options_default(&o);
    int r = mm::validate_march(ctx, u, tex, out, &o);
    if (r) return r;
    mm::MarchLaunch p;
    mm::fill_march_launch(*u, tex, *out, o, &p);
    cudaStream_t s = (cudaStream_t)stream;
    // The surrogate was trained on sun elevations 0-90 degrees (mm_surrogate_generate); with the sun
    // below the horizon a frame is outside that envelope and takes the plain cone march.
    if (o.cone == MM_CONE_SURROGATE && u->sun.direction[1] >= 0.0f)
        return mm::launch_surrogate_frame(p, ctx, o.surrogate, s);
    if (o.math == MM_MATH_EXACT) return mm::launch_march_exact(p, o.sampler, o.schedule, ctx->d_work, ctx->num_sms, s);
    return mm::launch_march_fast(p, o.sampler, o.density_format, o.schedule, o.math == MM_MATH_FAST_HALF2, ctx->d_work,
                                 ctx->num_sms, s);
}

}  // extern "C"
