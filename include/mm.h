/*
 * mm.h - C ABI of the GB300 cloud raymarch pass and its noise-texture generators.
 *
 * This library replaces one Vulkan compute pass of Project-Marshmallow: the cloud raymarch shader
 * SkyEngine/SkyEngine/Shaders/compute-clouds.comp, its descriptor contract
 * (SkyEngine/SkyEngine/Shader.cpp:662-693) and its dispatch
 * (SkyEngine/SkyEngine/VulkanApplication.cpp:1062-1071), plus the textures that feed it.
 *
 * Conventions
 *  - Every entry point returns an mm_status; none throws or aborts.  mm_last_error_string()
 *    describes the most recent failure of the calling thread.
 *  - Device work is stream ordered and asynchronous.  `stream` is a cudaStream_t passed as void*
 *    (NULL = the legacy default stream).
 *  - Device pointers are plain CUDA device pointers owned by the caller unless stated otherwise.
 *  - Matrices are column-major float[16] (glm / GLSL layout), element [col*4 + row].
 */
#ifndef MM_H_
#define MM_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MM_ABI_VERSION 1

typedef enum mm_status {
    MM_OK = 0,
    MM_ERR_INVALID_ARGUMENT = 1, /* null pointer, bad size, bad enum, wrong texture shape */
    MM_ERR_CUDA = 2,             /* a CUDA runtime call failed (text in mm_last_error_string) */
    MM_ERR_OUT_OF_MEMORY = 3,    /* a device or host allocation failed */
    MM_ERR_UNSUPPORTED = 4,      /* valid request the library does not implement */
    MM_ERR_TIMEOUT = 5,          /* a bounded device-side wait gave up */
    MM_ERR_NO_DEVICE = 6         /* no usable CUDA device */
} mm_status;

/* ------------------------------------------------------------------------------------------ */
/* Uniform blocks.  Byte layout = std140 layout of the shader's UBOs                           */
/* (compute-clouds.comp:12-41; host structs Shader.h:24-28, SkyManager.h:8-37).               */
/* ------------------------------------------------------------------------------------------ */

/* UniformCameraObject (Shader.h:24-28): 160 bytes. */
typedef struct mm_camera_ubo {
    float view[16];            /* world -> view; rows 0..2 of the 3x3 part = right, up, forward */
    float proj[16];            /* perspective with proj[1][1] negated (VulkanApplication.cpp:362) */
    float camera_position[4];  /* xyz = eye, w = 1 */
    float camera_params[4];    /* x = aspect, y = tan(0.5 * 0.01745 * fov_deg) (camera.h:72) */
} mm_camera_ubo;

/* UniformCameraObjectPrev (compute-clouds.comp:19-23): 144 bytes; read only by reprojection. */
typedef struct mm_camera_prev_ubo {
    float view[16];
    float proj[16];
    float camera_position[4];
} mm_camera_prev_ubo;

/* UniformSunObject (SkyManager.h:8-15): 116 bytes of data, padded to 128 as std140 does. */
typedef struct mm_sun_ubo {
    float location[4];
    float direction[4];
    float color[4];            /* rgb = sun colour; a = pixel phase 0..15 of the 1/16 update */
    float direction_basis[16]; /* columns: N, sun direction, B (SkyManager.cpp:46-70) */
    float intensity;
    float pad_[3];
} mm_sun_ubo;

/* UniformSkyObject (SkyManager.h:28-37): 52 bytes of data, padded to 64. */
typedef struct mm_sky_ubo {
    float beta_r[4];
    float beta_v[4];
    float wind[4];             /* xyz = wind direction, w = time */
    float mie_directional;
    float pad_[3];
} mm_sky_ubo;

/* All four blocks of descriptor set 2 bindings 0..3, in binding order (496 bytes). */
typedef struct mm_uniforms {
    mm_camera_ubo camera;
    mm_camera_prev_ubo camera_prev;
    mm_sun_ubo sun;
    mm_sky_ubo sky;
} mm_uniforms;

/* ------------------------------------------------------------------------------------------ */
/* Host scene set-up: camera and sky math of camera.cpp / SkyManager.cpp, restated.            */
/* ------------------------------------------------------------------------------------------ */

/* Camera from eye position and angles.  The march casts rays along -m_forward
 * (compute-clouds.comp:312-322 with camera.cpp:27-39), so `pitch_deg`/`yaw_deg` give the
 * direction the image centre looks at: d = (cos yaw cos pitch, sin pitch, sin yaw cos pitch)
 * and m_forward = -d; right/up follow camera.cpp:139-148.  `fov_deg` is the vertical field of
 * view converted with DEG2RAD = 0.01745 (camera.h:15,72).  camera_prev is set equal to camera. */
int mm_camera_from_angles(const float eye[3], float yaw_deg, float pitch_deg, float fov_deg,
                          int width, int height, mm_uniforms* u);

/* Sun/sky blocks from a sun direction given as elevation/azimuth in degrees:
 * dir = (cos el cos az, sin el, cos el sin az), then the TBN, intensity, colour and
 * scattering coefficients of SkyManager.cpp:15-70 (SkyManager::calcSun*, calcSkyBeta*).
 * wind = (1, 0.05, 1, time) (SkyManager.cpp:85-90); mie_directional = 0.8, rayleigh = 2,
 * mie = 0.005, turbidity = 10.  sun.color.a = pixel_phase. */
int mm_sky_from_sun_angles(float elevation_deg, float azimuth_deg, float time, int pixel_phase,
                           mm_uniforms* u);

/* Same blocks from SkyManager::rebuildSkyFromNewSun's fractional parameters
 * (SkyManager.cpp:108-116, 46-52): theta = 2 pi (elevation - 0.5), phi = 2 pi (azimuth - 0.5). */
int mm_sky_from_reference_fractions(float elevation, float azimuth, float time, int pixel_phase,
                                    mm_uniforms* u);

/* ------------------------------------------------------------------------------------------ */
/* Textures (replace Texture.cpp / Texture3D and the stb-loaded assets of                      */
/* VulkanApplication.cpp:240-265).  Sampling follows the reference samplers: LINEAR filter,    */
/* REPEAT wrap on every axis, normalized coordinates, mip level 0 only (Texture.cpp:29-52,     */
/* 315-338).                                                                                   */
/* ------------------------------------------------------------------------------------------ */

typedef enum mm_noise_kind {
    MM_NOISE_LOWRES_PERLIN_WORLEY = 0, /* 3D RGBA8: R Perlin-Worley, GBA Worley FBM (4/8/16 cells) */
    MM_NOISE_HIRES_WORLEY = 1,         /* 3D RGBA8: RGB Worley FBM (2/4/8 cells), A = 0 */
    MM_NOISE_CURL2D = 2,               /* 2D RG8: curl of 2D Perlin FBM (5 octaves) */
    MM_NOISE_WEATHER = 3,              /* 2D RGBA8: R coverage, G 0, B cloud type, A 255 */
    MM_NOISE_REF_CURL = 4              /* 2D RGBA8: ImageUtils.cpp GenerateCurlNoise (freq 3, 4 oct) */
} mm_noise_kind;

typedef enum mm_texel_format {
    MM_FORMAT_UNORM8 = 0, /* texel/255, as VK_FORMAT_R8G8B8A8_UNORM (Texture.h:29) */
    MM_FORMAT_FP16 = 1,   /* IEEE half, value = texel/255 rounded to half */
    MM_FORMAT_BF16 = 2    /* bfloat16, value = texel/255 rounded to bf16 (held exactly in an FP16 array: the
                             CUDA runtime has no bfloat16 texture channel kind) */
} mm_texel_format;

typedef struct mm_noise_desc {
    int kind;       /* mm_noise_kind */
    uint32_t seed;  /* ignored by MM_NOISE_REF_CURL, which has no seed */
    int width;      /* texels per side; 0 = the kind's default size */
    int height;
    int depth;      /* 1 for 2D kinds */
} mm_noise_desc;

typedef struct mm_texture_s* mm_texture;
typedef struct mm_mlp_s* mm_mlp; /* the learned sun-cone surrogate (see below) */

/* Generates a noise texture on the GPU into a new library-owned texture (device texels plus
 * a hardware texture object).  Default sizes: low-res 128^3, hi-res 32^3, curl 128^2,
 * weather 512^2, reference curl 128^2.  Replaces the pre-baked TGA/PNG assets loaded at
 * VulkanApplication.cpp:253-262. */
int mm_noise_generate(const mm_noise_desc* desc, mm_texture* out, void* stream);

/* Bytes of raw UNORM8 texels mm_noise_fill writes for `desc` (after defaults are applied). */
int mm_noise_texel_bytes(const mm_noise_desc* desc, size_t* bytes);

/* Writes the raw UNORM8 texels of a noise kind into caller device memory (x fastest, then y,
 * then z; 4 bytes per texel, 2 for MM_NOISE_CURL2D).  No texture object is made.
 * MM_NOISE_REF_CURL needs device scratch for its min/max normalisation and allocates it per
 * call. */
int mm_noise_fill(const mm_noise_desc* desc, void* d_texels, size_t bytes, void* stream);

/* MM_NOISE_REF_CURL without any device allocation, for callers that cannot allocate when they
 * generate (an engine or plugin host that owns the whole device heap, a frame loop that must not
 * hit the allocator).  No counterpart in the reference,
 * which generates this texture offline on the CPU.  Writes the same 128x128 RGBA8 texels as
 * mm_noise_fill with kind MM_NOISE_REF_CURL.  width/height: 0 or 128 (the maximum: sizes beyond
 * it are rejected with MM_ERR_INVALID_ARGUMENT).  Its scratch is one static device array of the
 * library (~192 KB, held by every GPU that loads the library until exit) shared by all calls:
 * calls whose GPU work overlaps (different streams, or threads) race on it and must be ordered by
 * the caller.  The first call on a device looks up the array's address on that device, so make it
 * before any stream capture; later calls only launch kernels.  The address is kept for the life of
 * the process: calls after a device reset (cudaDeviceReset) are not supported. */
int mm_noise_fill_ref_curl_noalloc(int width, int height, void* d_texels, size_t bytes, void* stream);

/* Hash stage of the seeded generators, for bit-exactness checks: out[i] = hash3(x, y, z, s) for
 * the n int32 triples at d_xyz (device), with hash3(x,y,z,s) = h(x + h(y + h(z + s))) and h the
 * lowbias32 integer mixer. */
int mm_noise_hash3(const int32_t* d_xyz, uint32_t stream_seed, size_t n, uint32_t* d_out, void* stream);

/* Hash stage of the reference curl generator: out[i] = hashNoise(x, y, z) of ImageUtils.cpp:25-29
 * (fract(sinf(dot(p, (12.9898, 78.233, 47.387))) * 43758.5453)) for n float triples (device). */
int mm_ref_curl_hash(const float* d_xyz, size_t n, float* d_out, void* stream);

/* Creates a texture from UNORM8 texels already in caller memory (`src_is_device` 0 = host).
 * channels is 1, 2 or 4; depth 1 makes a 2D texture.  `format` selects the storage of the
 * hardware-filtered copy; the UNORM8 texels are always kept for software sampling. */
int mm_texture_create(const void* texels, int src_is_device, int width, int height, int depth,
                      int channels, int format, mm_texture* out, void* stream);

/* Shipped assets (Texture::initFromFile / Texture3D::initFromFile, Texture.cpp:212-246, 502-538, with
 * stb_image's stbi_load(..., STBI_rgb_alpha)).  Decodes TGA (uncompressed or RLE; 8-bit grey,
 * 24/32-bit; either row order) and PNG (8- or 16-bit grey, grey+alpha, RGB, RGBA; not interlaced)
 * to RGBA8 rows top to bottom as stbi_load does: grey g -> (g, g, g, 255), missing alpha -> 255,
 * 16-bit samples -> their high byte, TGA rows flipped unless the descriptor has the top-left
 * origin bit.  Other variants (palettes, interlacing, 16-bit TGA) return MM_ERR_UNSUPPORTED. */

/* Decodes one file into a malloc'ed RGBA8 buffer (release with mm_image_free). */
int mm_image_decode_file(const char* path, uint8_t** rgba, int* width, int* height);
int mm_image_free(uint8_t* rgba);

/* Texture::initFromFile: one image file -> a 2D RGBA texture (e.g. Textures/CloudPlacement.png
 * for the weather map, NightSky/nightSky.png, CurlNoiseFBM.tga). */
int mm_texture_load_file(const char* path, int format, mm_texture* out, void* stream);

/* Texture3D::initFromFile: `depth` slices named prefix + "(" + i + ").tga", i = 0..depth-1
 * (Texture.cpp:511; the reference passes ".../lowResCloudShape/lowResCloud" with depth 128 and
 * ".../hiResCloudShape/hiResClouds " with depth 32, VulkanApplication.cpp:259-262) -> a 3D RGBA
 * texture, slice i at z = i. */
int mm_texture_load_slices(const char* prefix, int depth, int format, mm_texture* out, void* stream);

/* Width/height/depth/channels/format of a texture. */
int mm_texture_info(mm_texture tex, int* width, int* height, int* depth, int* channels,
                    int* format);

/* Copies the UNORM8 texels of a texture to host memory (synchronous). */
int mm_texture_copy_to_host(mm_texture tex, void* dst, size_t bytes);

/* Re-encodes the hardware-filtered copy of a texture in another mm_texel_format. */
int mm_texture_set_format(mm_texture tex, int format, void* stream);

/* Filtered fetches of a texture's hardware copy (the texture unit's LINEAR filter with WRAP
 * addressing and normalized coordinates, as the march reads it) at n caller coordinates, for
 * checking a filter model against the hardware: d_coords holds (u, v) pairs for a 2D texture or
 * (u, v, w) triples for a 3D one, d_out receives 4 floats per fetch (channels the texture lacks
 * read 0, 0, 1).  Device pointers; stream ordered.  Stands in for the GLSL texture() calls of
 * compute-clouds.comp:218,223,236,238 on the bound samplers (Texture.cpp:29-52, 315-338). */
int mm_texture_sample(mm_texture tex, const float* d_coords, size_t n, float* d_out, void* stream);

int mm_texture_destroy(mm_texture tex);

/* The five samplers of descriptor set 2 bindings 4..8 (compute-clouds.comp:43-47).
 * night_sky may be NULL when the sun is above the horizon. */
typedef struct mm_scene_textures {
    mm_texture weather;   /* cloudPlacement, 2D */
    mm_texture night_sky; /* nightSkyMap, 2D */
    mm_texture curl;      /* curlNoise, 2D */
    mm_texture low_res;   /* lowResCloudShape, 3D */
    mm_texture hi_res;    /* hiResCloudShape, 3D */
} mm_scene_textures;

/* ------------------------------------------------------------------------------------------ */
/* The cloud march (compute-clouds.comp:288-500).                                              */
/* ------------------------------------------------------------------------------------------ */

/* Output images (set 0 binding 0 `resultImage`, rgba32f), plus a depth image the reference
 * does not have: the march distance t of the first sample whose density is accumulated
 * (compute-clouds.comp:466), +INF where no sample is accumulated. */
typedef struct mm_image {
    float* rgba;              /* device, width*height float4 rows */
    size_t rgba_pitch_bytes;  /* >= 16*width, multiple of 16 */
    float* depth;             /* device, may be NULL */
    size_t depth_pitch_bytes; /* >= 4*width */
    int width;
    int height;
} mm_image;

typedef enum mm_pixel_mode {
    MM_PIXELS_FULL = 0,   /* every pixel is marched */
    MM_PIXELS_PHASE16 = 1 /* only pixels (4i + p%4, 4j + p/4), p = int(sun.color.a)
                             (compute-clouds.comp:292-298); other pixels are untouched */
} mm_pixel_mode;

typedef enum mm_sampler_mode {
    MM_SAMPLER_HARDWARE = 0, /* CUDA texture objects (8-bit fixed-point filter weights) */
    MM_SAMPLER_SOFTWARE = 1  /* software trilinear/bilinear with float weights */
} mm_sampler_mode;

typedef enum mm_math_mode {
    MM_MATH_FAST = 0,  /* FMA contraction and hardware transcendental approximations */
    MM_MATH_FAST_HALF2 = 2, /* MM_MATH_FAST with the large-step coverage test (the density > 0
                               decision of a large step, compute-clouds.comp:421-426) made in half2
                               on pairs of consecutive samples from FP16 texels; transmittance,
                               phase and in-scatter stay FP32.  Full frames with FP16/BF16 density,
                               hardware sampler, tiled schedule only. */
    MM_MATH_EXACT = 1  /* IEEE +,-,*,/,sqrt without contraction and the library's own
                          elementary functions: reproduces the FP32 CPU oracle bit for bit
                          when combined with MM_SAMPLER_SOFTWARE */
} mm_math_mode;

typedef enum mm_schedule {
    MM_SCHEDULE_TILED = 0,      /* one thread marches one pixel start to end (the shader's own loop
                                   nest), 8x4 pixel tiles per warp, block rows just above the horizon
                                   first; the sun-cone taps of a sample are fetched one at a time in
                                   full frames, in pairs in large 1/16-pixel launches and all six
                                   together in launches of <= 262144 rays (latency-bound) */
    MM_SCHEDULE_PERSISTENT = 1  /* persistent warps; each iteration evaluates one cloudTest per lane
                                   (a march step or a sun-cone tap); finished lanes take the next ray
                                   of their warp's 8x4 pixel tile (ballot compaction).  Full SIMT
                                   lanes, but a warp's texture requests scatter over more texels */
} mm_schedule;

typedef enum mm_cone_mode {
    MM_CONE_PLAIN = 0,     /* the six-tap sun cone of compute-clouds.comp:441-453 */
    MM_CONE_SURROGATE = 1  /* the cone taps' low-res densities + the trained MLP
                              (mm_march_options.surrogate) predict Beer's transmittance of the
                              six-tap sum; full frames, hardware sampler, fast math and the tiled
                              schedule only.  Frames with the sun below the horizon lie outside the
                              training envelope (elevations 0-90 degrees) and take the plain cone */
} mm_cone_mode;

typedef struct mm_march_options {
    int pixel_mode;        /* mm_pixel_mode */
    int sampler;           /* mm_sampler_mode */
    int math;              /* mm_math_mode */
    int density_format;    /* mm_texel_format of the hardware-filtered density textures */
    float coverage_offset; /* added to weather.r before min(0.85, .) (0 = reference) */
    int ref_uv_1080p;      /* 1: uv = pixel / (1920,1080) as the shader hard-codes
                              (compute-clouds.comp:283-285,305); 0: uv = pixel / (width,height) */
    uint64_t* d_counters;  /* optional device uint64[4]: cloudTest calls, cloudHiRes calls,
                              loop iterations, accumulated samples (atomically added) */
    int schedule;          /* mm_schedule */
    int cone;              /* mm_cone_mode */
    mm_mlp surrogate;      /* trained network for MM_CONE_SURROGATE */
} mm_march_options;

/* Fills `o` with the defaults: full frame, hardware sampler, fast math, UNORM8, offset 0,
 * uv = pixel/(width,height), no counters, tiled schedule. */
int mm_march_options_default(mm_march_options* o);

typedef struct mm_context_s* mm_context;

/* A context owns the per-device scratch the march uses (work-queue counters; for the surrogate
 * cone, the deferred-sample records: 4 per pixel, ~212 bytes per pixel, allocated by the first
 * surrogate march of a frame size).  Create it with the target device current.  Contexts must not
 * be shared by concurrent streams. */
int mm_context_create(mm_context* out);
int mm_context_destroy(mm_context ctx);

/* Renders one cloud frame (replaces vkCmdDispatch of the compute pipeline,
 * VulkanApplication.cpp:1062-1071).  `u` is read on the host at call time (no device copy is
 * kept).  Stream ordered; returns after the launch. */
int mm_clouds_march(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex,
                    const mm_image* out, const mm_march_options* opt, void* stream);

/* The reprojection pass (reproject.comp:91-152): every pixel of dst takes the previous frame src at
 * the point where its ray meets the inner atmosphere sphere, seen by u->camera_prev (ten taps along
 * the motion vector averaged; alpha, and depth when both images have one, from the centre tap).
 * src and dst are different images of the same size.  uv = pixel / image size.  opt->math (NULL =
 * defaults, FAST): EXACT is bit-identical to the shader's arithmetic restated on the CPU; FAST
 * uses equal algebraic forms (a tap within rounding of a pixel boundary may take the neighbour). */
int mm_clouds_reproject(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                        const mm_march_options* opt, void* stream);

/* One frame of the reference's compute work (VulkanApplication.cpp:1053-1071): reproject prev into
 * out, then march the pixels of phase int(u->sun.color.a) (one in 16) into out.  opt->pixel_mode is
 * ignored (PHASE16); opt->math applies to both passes. */
int mm_clouds_frame(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_image* prev,
                    const mm_image* out, const mm_march_options* opt, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* Mesh cloud shadows: the low-res march of the mesh fragment shader (model.frag:52-162,       */
/* 221-222, 240-276), run over a G-buffer instead of rasterized fragments.                    */
/* ------------------------------------------------------------------------------------------ */

/* Per pixel, the world position of the mesh fragment that covers it (model.vert:39,
 * fragPositionWC): float4 rows, xyz the position, w != 0 where a fragment covers the pixel and 0
 * where none does.  Device memory; pitch >= 16 * width and a multiple of 16. */
typedef struct mm_gbuffer {
    const float* world_pos;
    size_t world_pos_pitch_bytes;
    int width, height;
} mm_gbuffer;

/* For every covered pixel: six low-res density samples from the fragment towards the sun; the
 * shadow is the largest density met (1 once above 0.99).  Writes it to `shadow` (float rows,
 * 0 on uncovered pixels; may be NULL) and, if `rgba` (float4 rows holding the lit mesh colour,
 * may be NULL) is given, darkens covered pixels in place to (max(rgb * (1 - 2 shadow), 0), 1) as
 * the shader's last lines do (:275-277).  Reads tex->weather (the reference's cloudPlacement) and
 * tex->low_res.  opt (NULL = defaults) supplies sampler, math and coverage_offset; its other fields
 * are ignored.  Replaces the cloud-shadow part of the mesh draw (VulkanApplication.cpp:965). */
int mm_mesh_shadow(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex, const mm_gbuffer* gbuf,
                   float* shadow, size_t shadow_pitch_bytes, float* rgba, size_t rgba_pitch_bytes,
                   const mm_march_options* opt, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* Post chain: the reference's offscreen passes after the clouds (VulkanApplication.cpp:926-1010)  */
/* as CUDA kernels on device buffers (no graphics API): god rays (god-ray.frag:41-76), radial      */
/* blur (radialBlur.frag:36-63), the mesh over the blurred sky, Uncharted-2 tonemap + vignette  */
/* (tonemap.frag:11-33) into the 8-bit swapchain layout.                                        */
/* ------------------------------------------------------------------------------------------ */

typedef struct mm_post_options {
    int math; /* mm_math_mode: EXACT = the shaders' arithmetic (bit-reproducible), FAST = FMA + SFU pow */
    int bgra; /* 1: bytes B,G,R,A as the B8G8R8A8_UNORM swapchain (VulkanApplication.cpp:1437-1446); 0: R,G,B,A */
} mm_post_options;

/* math FAST, bgra 1. */
int mm_post_options_default(mm_post_options* o);

/* Pixel (x, y) of every pass has fragUV = ((x + 0.5) / W, (y + 0.5) / H) (the full-screen quad of
 * Geometry.cpp:91-101); a fetch at the fragment's own uv returns the texel, other taps are bilinear
 * with CLAMP_TO_EDGE (the offscreen sampler, VulkanApplication.cpp:1290-1305).  Images are RGBA32F
 * (mm_image; depth fields ignored); src and dst must not overlap.  With the sun below the horizon
 * both passes copy the colour with alpha 1, as the shaders do. */

/* god-ray.frag: dst = (src.rgb, god-ray term from eight taps of src.a towards the sun). */
int mm_post_god_rays(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                     const mm_post_options* opt, void* stream);
/* radialBlur.frag: dst = (sun.color.rgb * sun.intensity * mean of ten taps of src.a * 1.1
 * + 0.5 src.rgb, 1). */
int mm_post_radial_blur(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                        const mm_post_options* opt, void* stream);
/* tonemap.frag: Uncharted-2 (exposure 0.7, white 50.2, gamma 1/2.2), vignette towards
 * (0.1, 0.05, 0.13), UNORM8 (round to nearest even, alpha 255) into `out` (4 bytes per pixel). */
int mm_post_tonemap(mm_context ctx, const mm_image* src, void* out, size_t out_pitch_bytes,
                    const mm_post_options* opt, void* stream);
/* The whole chain in two kernels: clouds -> god rays -> radial blur -> mesh layer (pixels with
 * a != 0 replace the blurred sky, as the mesh draw after the blur does; may be NULL) -> tonemap
 * -> 8 bits.  Equal to the four passes above run through RGBA32F framebuffers.  Keeps a float
 * scratch plane of the frame size in the context. */
int mm_post_chain(mm_context ctx, const mm_uniforms* u, const mm_image* clouds, const mm_image* mesh, void* out,
                  size_t out_pitch_bytes, const mm_post_options* opt, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* Many views in one launch.  No counterpart in the reference, which renders one camera.          */
/* ------------------------------------------------------------------------------------------ */

/* One view of a batch: its own uniform blocks (camera, sun, wind/time) and output image. */
typedef struct mm_view {
    mm_uniforms u;
    mm_image out;
    float coverage_offset;
} mm_view;

typedef enum mm_batch_schedule {
    MM_BATCH_PERSISTENT = 0, /* persistent warps take warp tiles of all views from one global queue */
    MM_BATCH_BLOCKS = 1,     /* one launch of 16x8-pixel blocks over all views, hardware-scheduled */
    MM_BATCH_GRAPH = 2       /* one CUDA graph of the views' own launches (each view's kernel variant) on
                                four concurrent branches, largest views first */
} mm_batch_schedule;

typedef struct mm_batch_options {
    int warp_tile_w;    /* persistent schedule: pixels across one warp's 32-ray tile: 4, 8 (default), 16, 32 */
    int tiles_per_grab; /* persistent schedule: warp tiles taken from the queue at a time, 1..64 (default 4) */
    int use_graph;      /* 1 (default): replay a captured CUDA graph (upload, reset, kernel) */
    int schedule;       /* mm_batch_schedule (default MM_BATCH_GRAPH, the fastest on the 70-view batch) */
    int density_format; /* mm_texel_format of the density textures' hardware copies (default UNORM8) */
    mm_mlp surrogate;   /* non-NULL: the learned sun cone for every view with the sun above the horizon
                           (MM_BATCH_GRAPH only; such views run one after another, sharing the
                           context's deferred-sample records) */
} mm_batch_options;

int mm_batch_options_default(mm_batch_options* o);

/* Renders n views (full frames, hardware sampler, fast math, plain or surrogate cone) with the shared textures:
 * blocks of all views in one grid (MM_BATCH_BLOCKS; one launch per 72 views), a persistent kernel
 * whose warps take tiles of all views from one queue (MM_BATCH_PERSISTENT), or one CUDA graph of the
 * views' own launches on concurrent branches (MM_BATCH_GRAPH, re-captured and updated in place on
 * every call).  The host-side records are
 * staged in pinned memory owned by the context; a call waits for the previous batch of the same
 * context to finish reading them.  The graph is re-captured when the view count or the options
 * change. */
int mm_clouds_march_batch(mm_context ctx, const mm_view* views, int n, const mm_scene_textures* tex,
                          const mm_batch_options* opt, void* stream);

/* Autotuner: times the persistent schedule with warp_tile_w in {4, 8, 16, 32} x tiles_per_grab in
 * {1, 2, 4, 8, 16}, the block schedule and the graph schedule on this batch (ms_table, optional:
 * 22 floats, the 20 persistent ones row-major in that order, then blocks, then graph) and returns
 * the fastest options.  Synchronizes `stream`. */
int mm_batch_autotune(mm_context ctx, const mm_view* views, int n, const mm_scene_textures* tex,
                      mm_batch_options* best, float* ms_table, void* stream);

/* ------------------------------------------------------------------------------------------ */
/* Learned sun-cone surrogate: a 16 -> 64 -> 64 -> 64 -> 1 MLP (ReLU, sigmoid output) trained and  */
/* run on the tensor cores (tcgen05, BF16 operands, FP32 accumulation).  No counterpart in the     */
/* reference, whose sun cone (compute-clouds.comp:441-460) is always marched.                      */
/* ------------------------------------------------------------------------------------------ */

/* Number of FP32 parameters: W1[64x16], b1[64], W2[64x64], b2[64], W3[64x64], b3[64], w4[64], b4
 * (row-major [out][in]), in that order. */
int mm_mlp_param_count(void);
/* New network on the current device, He-uniform weights from `seed`, zero biases. */
int mm_mlp_create(uint32_t seed, mm_mlp* out);
int mm_mlp_destroy(mm_mlp m);
int mm_mlp_get_params(mm_mlp m, float* host, int n);
int mm_mlp_set_params(mm_mlp m, const float* host, int n);
/* y[i] = network(x[i]) for n samples; x: device bf16 [n][16] (16-byte aligned), y: device FP32. */
int mm_mlp_forward(mm_mlp m, const void* d_x, int n, float* d_y, void* stream);
/* Gradient of mean((y - t)^2) over the n samples w.r.t. the parameters into d_grad (device, FP32,
 * mm_mlp_param_count() values); *h_loss (optional) = the loss.  Synchronizes `stream`. */
int mm_mlp_gradients(mm_mlp m, const void* d_x, const float* d_t, int n, float* d_grad, float* h_loss, void* stream);
/* `steps` Adam steps (beta 0.9/0.999) of `batch` samples (a multiple of 128) taken in order from
 * the n samples, wrapping around; h_loss_history (optional, host, `steps` floats) gets each step's
 * mean squared error.  Synchronizes `stream`. */
int mm_mlp_train(mm_mlp m, const void* d_x, const float* d_t, int n, int batch, int steps, float lr,
                 float* h_loss_history, void* stream);
/* Training samples for the surrogate: for each texture seed first_seed .. first_seed+n_seeds-1
 * (the four seeded textures regenerated on the GPU), `per_seed` samples at uniform random points
 * of the cloud layer within +-half_extent m of the origin where the march would accumulate, with a
 * random sun (elevation 0-90 deg, any azimuth) and wind time in [0, 2] s; features as the surrogate
 * march computes them (d_x: bf16 [n_seeds*per_seed][16]) and the target exp(-sum of the plain
 * six-tap cone) (d_t: FP32).  *produced = samples written.  Synchronizes `stream`. */
int mm_surrogate_generate(uint32_t first_seed, int n_seeds, int per_seed, float half_extent, void* d_x,
                          float* d_t, int* produced, void* stream);

/* Checkpoint of parameters and Adam state ("MMMLP001" header, count, step, P, M, V). */
int mm_mlp_save(mm_mlp m, const char* path);
int mm_mlp_load(mm_mlp m, const char* path);

/* ------------------------------------------------------------------------------------------ */
/* Diagnostics                                                                                 */
/* ------------------------------------------------------------------------------------------ */

const char* mm_last_error_string(void);
int mm_abi_version(void);
/* Number of device kernels this library has launched since load (all entry points). */
uint64_t mm_kernel_launch_count(void);

/* Measures the on-chip rates the march is bound by, on the current device:
 * out[0] trilinear 3D filtered fetches (G/s) from `tex3d`, out[1] bilinear 2D filtered fetches
 * (G/s) from `tex2d` (both RGBA textures with texture objects), out[2] FP32 FMA throughput
 * (TFLOP/s).  Synchronizes `stream`.  No reference counterpart (the reference has no timing). */
int mm_measure_peaks(mm_texture tex3d, mm_texture tex2d, double* out, void* stream);

/* Tensor-core self-check: out[128 x N] = A[128 x K] * B[N x K]^T (bf16 in, FP32 out, row-major,
 * device pointers) through one tcgen05 MMA pipeline of the surrogate's kernels.  K, N multiples of
 * 16 in [16, 128].  variant 0 is the operand layout the kernels use; 1 swaps the descriptors'
 * leading/stride fields.  *d_status is set to 1 if a bounded wait gave up.  No reference
 * counterpart. */
int mm_tc_gemm_check(const void* d_a, const void* d_b, int K, int N, int variant, float* d_out, int* d_status,
                     void* stream);

/* The same GEMM with A and/or B read MN-major from shared memory (the in-place transposed operands
 * of the training kernel's weight-gradient and delta GEMMs): d_a holds A^T ([K][128] row-major)
 * when a_mn, d_b holds B^T ([K][N]) when b_mn.  lbo_k = 1 puts the stride between K groups of an
 * MN-major operand in the descriptor's leading-byte-offset field, 0 in its stride field (the
 * kernels use 1).  No reference counterpart. */
int mm_tc_gemm_mn_check(const void* d_a, const void* d_b, int K, int N, int a_mn, int b_mn, int lbo_k, float* d_out,
                        int* d_status, void* stream);

/* Self-test of the bounded mbarrier wait every tensor-core kernel uses: one thread initializes an
 * mbarrier, arrives on it (arrive != 0) or not, and waits for its phase for at most poll_limit polls
 * (1 .. 2^24).  *d_status becomes 0 if the phase completed and 1 if the wait gave up — the path a
 * kernel takes when an expected arrival never comes: it reports and returns instead of hanging.
 * No reference counterpart. */
int mm_tc_wait_check(int arrive, unsigned int poll_limit, int* d_status, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MM_H_ */
