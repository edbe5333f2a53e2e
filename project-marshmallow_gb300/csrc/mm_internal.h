// mm_internal.h - library-internal declarations shared by the C ABI and the kernel launchers.
#ifndef MM_INTERNAL_H_
#define MM_INTERNAL_H_

#include <stddef.h>
#include <stdint.h>

#include <math.h>

#include "../../include/mm.h"

#if defined(MM_HAVE_CUDA_RUNTIME) || defined(__CUDACC__)
#include <cuda_runtime.h>
#endif

namespace mm {

// Records `msg` as the calling thread's last error and returns `code`.
int fail(int code, const char* fmt, ...);
// Counts device kernel launches made by the library.
void count_launch(uint64_t n = 1);

#if defined(MM_HAVE_CUDA_RUNTIME) || defined(__CUDACC__)

// Maps a CUDA error to MM_ERR_CUDA / MM_ERR_OUT_OF_MEMORY with the call site in the message.
int cuda_fail(cudaError_t e, const char* what);

#define MM_CUDA_TRY(call)                                          \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return ::mm::cuda_fail(e_, #call); \
    } while (0)

}  // namespace mm

// Library-owned texture: UNORM8 texels in linear device memory (software sampling, copies) and a
// hardware-filtered copy in a CUDA array with its texture object.
struct mm_texture_s {
    int width = 0, height = 0, depth = 0, channels = 0;
    int format = MM_FORMAT_UNORM8;   // format of the hardware-filtered copy
    uint8_t* texels = nullptr;       // device, width*height*depth*channels bytes
    cudaArray_t array = nullptr;
    cudaTextureObject_t tex = 0;
    int device = 0;
};

struct mm_context_s {
    int device = 0;
    unsigned int* d_work = nullptr;  // [0] persistent-march tile counter, [1] surrogate record count
    int num_sms = 0;
    // surrogate-cone records (surrogate.cu)
    void* sur_x = nullptr;
    void* sur_meta = nullptr;
    void* sur_y = nullptr;     // per-ray (l_n, beers mix factor) of the surrogate march
    void* sur_ray = nullptr;
    size_t sur_cap = 0, sur_pixels = 0;
    void* batch = nullptr;  // multi-view launch state (batch.cu)
    // post chain (post.cu): god-ray term and cloud alpha planes of the last frame size, with
    // LINEAR / CLAMP texture objects on them for the production-arithmetic chain
    void* post_raw = nullptr;  // the allocation holding both planes
    float* post_plane = nullptr;
    float* post_aplane = nullptr;
    size_t post_pitch = 0;
    int post_w = 0, post_h = 0;
    cudaTextureObject_t post_gtex = 0, post_atex = 0;
    // mm_clouds_frame: second stream for the reprojection beside the 1/16 march
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t aux_fork = nullptr, aux_join = nullptr;
};

namespace mm {

// Device-side view of one texture for the kernels.
struct TexView {
    cudaTextureObject_t tex;
    const uint8_t* texels;
    int w, h, d, channels;
};

struct MarchLaunch {
    mm_uniforms u;
    TexView weather, night, curl, low, hi;
    float4* rgba;
    size_t rgba_pitch;  // bytes
    float* depth;
    size_t depth_pitch;  // bytes
    int width, height;
    int pixel_mode;
    int phase;
    float uv_w, uv_h;
    float coverage_offset;
    unsigned long long* counters;
    int row_split;  // tiled march: block rows [0, row_split) run in reverse order first (0 = launch order)
    // Per-frame constants of the production-arithmetic march, computed once on the host
    // (march_host_consts) so the kernels read them from the parameter bank instead of holding them
    // in registers: the normalized sun direction and 20 * wind.
    float sun_dir[3], wind20[3];
    float cone[18];  // the six sun-cone offsets mat3(directionBasis) * v (compute-clouds.comp:392-401)
};

// Kernel launchers (one translation unit per arithmetic mode).
// Kernel attributes of the march kernels (the pooled kernels' shared-memory carveout) for the current
// device; called when a context is created, outside any stream capture.
void prepare_march_fast();
void prepare_march_exact();
void prepare_march_exact_sw();
// The exact march with the software sampler (march_exact_sw.cu); launch_march_exact forwards to it.
int launch_march_exact_sw(const MarchLaunch& p, int schedule, unsigned int* work, int num_sms, cudaStream_t s);
int launch_march_exact(const MarchLaunch& p, int sampler, int schedule, unsigned int* work, int num_sms,
                       cudaStream_t s);
int launch_march_fast(const MarchLaunch& p, int sampler, int format, int schedule, int half2, unsigned int* work,
                      int num_sms, cudaStream_t s);

// Noise generators (noise.cu).
int launch_noise(int kind, uint32_t seed, int w, int h, int d, uint8_t* out, cudaStream_t s);
int launch_ref_curl(uint8_t* out_rgba, float* scratch_curl, float* scratch_bounds, cudaStream_t s);
int launch_hash_stage(int which, const void* in, uint32_t seed, size_t n, void* out, cudaStream_t s);

// Surrogate network (mlp.cu): inference over the deferred cone samples of a surrogate frame (count
// held in device memory), each prediction added to its ray's transmittance.
int mlp_infer_accumulate(mm_mlp m, const void* d_x, int cap, const unsigned int* d_count, const float2* meta,
                         const float2* ray_b, float4* ray_u, cudaStream_t s);
int* mlp_status_ptr(mm_mlp m);

// Surrogate march and training samples (surrogate.cu).
int launch_surrogate_frame(const MarchLaunch& p, mm_context ctx, mm_mlp net, cudaStream_t s);
// Allocates the context's deferred-sample records for frames of up to `pixels` pixels (no-op if
// they are large enough): a surrogate frame launched during a stream capture must find them there.
int surrogate_reserve(mm_context ctx, size_t pixels);
int launch_surrogate_samples(const MarchLaunch& p, uint32_t seed, unsigned long long first, unsigned long long n,
                             float half_extent, void* d_x, float* d_t, unsigned int* d_count, int cap,
                             cudaStream_t s);
TexView texture_view(mm_texture t);

// Argument contract of mm_clouds_march and the kernel record of one view (api.cu).
int validate_march(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_image* out,
                   const mm_march_options* opt);
// Host side of the production frame constants (make_frame<false> reads them): normalize(sun
// direction basis column 1) and 20 * wind.
inline void march_host_consts(MarchLaunch& p) {
    const float* b = p.u.sun.direction_basis + 4;
    const float inv = 1.0f / sqrtf((b[0] * b[0] + b[1] * b[1]) + b[2] * b[2]);
    for (int i = 0; i < 3; ++i) {
        p.sun_dir[i] = b[i] * inv;
        p.wind20[i] = 20.0f * p.u.sky.wind[i];
    }
    static const float v[6][3] = {{0.0f, 0.6f, 0.0f}, {0.0f, 0.5f, 0.05f}, {0.1f, 0.75f, 0.0f},
                                  {0.2f, 2.5f, 0.3f}, {0.0f, 6.0f, 0.0f},  {-0.1f, 1.0f, -0.2f}};
    const float* m = p.u.sun.direction_basis;
    for (int k = 0; k < 6; ++k)
        for (int r = 0; r < 3; ++r)
            p.cone[3 * k + r] = (m[r] * v[k][0] + m[4 + r] * v[k][1]) + m[8 + r] * v[k][2];
}

void fill_march_launch(const mm_uniforms& u, const mm_scene_textures* tex, const mm_image& out,
                       const mm_march_options& o, MarchLaunch* p);
void batch_state_destroy(mm_context ctx);
void post_state_destroy(mm_context ctx);

#endif  // CUDA runtime available

}  // namespace mm

#endif  // MM_INTERNAL_H_
