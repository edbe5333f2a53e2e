/*
 * oracle.h - CPU oracle for the cloud raymarch pass and the noise generators.
 *
 * TEST INFRASTRUCTURE ONLY.  The oracle is the checker of the CUDA library: the parity tests,
 * the smoke check and the CPU-baseline leg of the benchmark call it; the library never does.
 *
 *  - oracle_march_*: a line-by-line restatement of SkyEngine/SkyEngine/Shaders/compute-clouds.comp
 *    (:65-500) in C++, instantiated in float (the FP32 parity twin and the timed CPU baseline) and
 *    in double (the FP64 yardstick for errors), with software samplers that implement the reference
 *    samplers (LINEAR, REPEAT, normalized coordinates, mip 0; Texture.cpp:29-52, 315-338).
 *  - oracle_ref_curl: a restatement of SkyEngine/SkyEngine/ImageUtils.cpp:25-222
 *    (GenerateCurlNoise), pinned against the shipped Textures/CurlNoiseFBM.tga.
 *  - oracle_shadow_*: the cloud-shadow march of the mesh pass, SkyEngine/SkyEngine/Shaders/model.frag.
 *  - oracle_reproject_f32: the reprojection pass, SkyEngine/SkyEngine/Shaders/reproject.comp.
 *  - oracle_post_*: the post chain (god rays, radial blur, tonemap) of the reference's offscreen passes.
 *  - oracle_noise_fill: the seeded Perlin-Worley / Worley / curl / weather generators that stand in
 *    for the pre-baked Nubis textures (which have no generator in the reference).
 */
#ifndef MM_ORACLE_H_
#define MM_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#include "../include/mm.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_texture {
    const uint8_t* texels; /* UNORM8, x fastest, then y, then z */
    int width, height, depth;
    int channels; /* 1, 2 or 4 */
} oracle_texture;

typedef struct oracle_textures {
    oracle_texture weather, night_sky, curl, low_res, hi_res;
} oracle_textures;

/* Pixel sample of a frame: rows row_begin, row_begin+row_step, ... < row_end and in each row the
 * columns col_begin, col_begin+col_step, ... < width.  Outputs are written compactly
 * (n_rows x n_cols), rgba as 4 floats per pixel.  pixel_mode 1 (PHASE16) marches the reference's
 * 1/16 subset: only pixels with (x%4, y%4) == (p%4, p/4), p = int(sun.color.a); others are
 * left untouched.  counters (may be NULL) receive cloudTest calls, cloudHiRes calls, loop
 * iterations and accumulated samples. */
typedef struct oracle_frame {
    int width, height;
    int pixel_mode;
    float coverage_offset;
    int ref_uv_1080p;
    int row_begin, row_end, row_step;
    int col_begin, col_step;
    int filter; /* 0: exact filter weights; 1: the texture unit's 8-bit fixed-point filter */
} oracle_frame;

int oracle_march_f32(const mm_uniforms* u, const oracle_textures* t, const oracle_frame* f,
                     float* out_rgba, float* out_depth, uint64_t* counters, int nthreads);
int oracle_march_f64(const mm_uniforms* u, const oracle_textures* t, const oracle_frame* f,
                     float* out_rgba, float* out_depth, uint64_t* counters, int nthreads);

/* The texture unit's LINEAR/WRAP filter (oracle_glsl.h) of an oracle texture at n normalized
 * coordinates: dims 2 reads (u, v) pairs, dims 3 (u, v, w) triples from coords; out gets 4 floats
 * per fetch (channels the texture lacks read 0, 0, 1).  filter 0 uses exact float weights instead. */
int oracle_sample(const oracle_texture* t, int dims, const float* coords, size_t n, int filter, float* out);

/* ImageUtils.cpp GenerateCurlNoise: 128x128 RGBA8 (A = 255), rows top to bottom. */
int oracle_ref_curl(uint8_t* out_rgba);
/* Gradient-table index hashVec picks for lattice point (x,y,z) (ImageUtils.cpp:25-34). */
int oracle_ref_curl_hash_index(float x, float y, float z);
/* hashNoise(x, y, z) of ImageUtils.cpp:25-29. */
float oracle_ref_curl_hash(float x, float y, float z);
/* mm_math.h functions: 0 exp, 1 exp2, 2 log2, 3 pow(x,y), 4 acos, 5 cos, 6 sin, 7 sinf_cr. */
float oracle_mm_math(int fn, float x, float y);

/* Seeded generators; kind = mm_noise_kind; out holds w*h*d*channels bytes. */
int oracle_noise_fill(int kind, uint32_t seed, int w, int h, int d, uint8_t* out);
/* Integer hash stage: lowbias32 and the 3D lattice hash used by the generators. */
uint32_t oracle_hash32(uint32_t x);
uint32_t oracle_hash3(int32_t x, int32_t y, int32_t z, uint32_t s);

/* reproject.comp:91-152 over a w x h frame: dst from src (rgba float4 rows; depth optional) with the
 * camera and camera_prev blocks of u.  Depth (new) follows the centre tap, as alpha does. */
int oracle_reproject_f32(const mm_uniforms* u, const float* src_rgba, const float* src_depth, int w, int h,
                         float* dst_rgba, float* dst_depth);

/* Cloud shadow of the mesh pass (model.frag:52-162, 221-222, 240-276) for n G-buffer pixels: world_pos holds
 * float4 (xyz world position, w != 0 where a mesh fragment covers the pixel); out_shadow gets the
 * accumulated density (0 on uncovered pixels).  coverage_offset is added to weather.r, as in the march. */
int oracle_shadow_f32(const mm_uniforms* u, const oracle_textures* t, const float* world_pos, size_t n,
                      float coverage_offset, float* out_shadow, int nthreads);
int oracle_shadow_f64(const mm_uniforms* u, const oracle_textures* t, const float* world_pos, size_t n,
                      float coverage_offset, float* out_shadow, int nthreads);

/* The post chain (god-ray.frag:41-76, radialBlur.frag:36-63, tonemap.frag:11-33) on w x h RGBA32F
 * images (rows of 4 floats).  god_rays: dst = (src.rgb, god-ray term); radial_blur: dst =
 * (sun colour * intensity * blur(src.a) + 0.5 src.rgb, 1); tonemap: 8-bit (bgra: B,G,R,A byte order
 * as the B8G8R8A8 swapchain, else R,G,B,A; A = 255).  chain: clouds -> god rays -> radial blur ->
 * mesh pixels (a != 0) drawn over it (mesh may be NULL) -> tonemap. */
int oracle_post_god_rays(const mm_uniforms* u, const float* src, int w, int h, float* dst);
int oracle_post_radial_blur(const mm_uniforms* u, const float* src, int w, int h, float* dst);
int oracle_post_tonemap(const float* src, int w, int h, uint8_t* out, size_t pitch, int bgra);
int oracle_post_chain(const mm_uniforms* u, const float* clouds, const float* mesh, int w, int h, uint8_t* out,
                      size_t pitch, int bgra);

/* The four uniform blocks as the reference's host fills them each frame: Camera (camera.cpp:27-39,
 * 139-147; near 0.1, far 1000; proj[1][1] negated) looking along (cos yaw cos pitch, sin pitch,
 * sin yaw cos pitch) with its m_forward the reverse of that, and SkyManager (SkyManager.cpp:15-100)
 * for the sun at (cos el cos az, sin el, cos el sin az); wind time `time`, sun.color.a = pixel_phase.
 * camera_prev = camera.  Returns 0, or 1 for invalid arguments. */
int oracle_uniforms(const float eye[3], float yaw_deg, float pitch_deg, float fov_deg, int width, int height,
                    float sun_elevation_deg, float sun_azimuth_deg, float time, int pixel_phase, mm_uniforms* u);

/* Uncharted-2 tonemap of tonemap.frag:10-28 (exposure 0.7, white 50.2, gamma 1/2.2) applied to
 * n rgb triples (stride 4 floats), written as n*3 floats. */
void oracle_tonemap(const float* rgba, size_t n, float* out_rgb);

#ifdef __cplusplus
}
#endif

#endif /* MM_ORACLE_H_ */
