// ref_clouds_main.cpp - runs the reference's own compute-clouds.comp, compiled unchanged as C++
// (oracle/ref/glsl_to_cpp.py + glsl_shim.h), on the CPU over a list of pixels (test infrastructure:
// builds oracle/_ref/libref_clouds.so, which only regenerates and re-checks golden fixtures).
//
// The shader's uniform blocks, samplers and result image are globals of the generated translation
// unit; this file fills them from an mm_uniforms block and oracle_textures (the same inputs the CPU
// restatement takes), then runs main() once per requested pixel with gl_GlobalInvocationID set the
// way the dispatch of VulkanApplication.cpp does: invocation (x/4, y/4) of the 1/16 pixel phase
// p = int(sun.color.a) writes pixel (4*gid.x + p%4, 4*gid.y + p/4).
#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../oracle.h"

#include "compute_clouds.gen.cpp"
// the shim's GLSL keywords end with the shader
#undef main
#undef layout
#undef uniform
#undef readonly
#undef writeonly
#undef highp
#undef in
#undef inout
#undef out

namespace {

mat4 to_mat4(const float* m) {  // std140 column-major, as glm stores it
    mat4 r;
    std::memcpy(&r[0][0], m, 16 * sizeof(float));
    return r;
}

vec4 to_vec4(const float* v) { return vec4(v[0], v[1], v[2], v[3]); }

void bind(GlslSampler& s, const oracle_texture& t) {
    s.texels = t.texels;
    s.w = t.width;
    s.h = t.height;
    s.d = t.depth > 0 ? t.depth : 1;
    s.channels = t.channels;
    s.is_float = false;
    s.clamp_edge = false;  // every sampler of the cloud pass is REPEAT (Texture.cpp:29-52)
}

}  // namespace

extern "C" {

// Marches the n pixels (xs[i], ys[i]) of a WIDTH x HEIGHT frame and writes their rgba (4 floats each)
// to out.  Every pixel must belong to the phase int(sun.color.a).  Returns 0, or -1 on bad input.
int ref_clouds_march(const mm_uniforms* u, const oracle_textures* t, const int* xs, const int* ys, size_t n,
                     float* out, int nthreads) {
    if (!u || !t || (n && (!xs || !ys || !out))) return -1;
    const int phase = (int)u->sun.color[3];
    for (size_t i = 0; i < n; ++i) {
        if (xs[i] < 0 || ys[i] < 0 || xs[i] >= WIDTH || ys[i] >= HEIGHT) return -1;
        if (xs[i] % 4 != phase % 4 || ys[i] % 4 != phase / 4) return -1;
    }
    camera.view = to_mat4(u->camera.view);
    camera.proj = to_mat4(u->camera.proj);
    camera.cameraPosition = to_vec4(u->camera.camera_position);
    camera.cameraParams = to_vec4(u->camera.camera_params);
    cameraPrev.view = to_mat4(u->camera_prev.view);
    cameraPrev.proj = to_mat4(u->camera_prev.proj);
    cameraPrev.cameraPosition = to_vec4(u->camera_prev.camera_position);
    sun.location = to_vec4(u->sun.location);
    sun.direction = to_vec4(u->sun.direction);
    sun.color = to_vec4(u->sun.color);
    sun.directionBasis = to_mat4(u->sun.direction_basis);
    sun.intensity = u->sun.intensity;
    sky.betaR = to_vec4(u->sky.beta_r);
    sky.betaV = to_vec4(u->sky.beta_v);
    sky.wind = to_vec4(u->sky.wind);
    sky.mie_directional = u->sky.mie_directional;
    bind(cloudPlacement, t->weather);
    bind(nightSkyMap, t->night_sky);
    bind(curlNoise, t->curl);
    bind(lowResCloudShape, t->low_res);
    bind(hiResCloudShape, t->hi_res);

    std::vector<float> image((size_t)WIDTH * HEIGHT * 4, 0.0f);
    resultImage.texels = image.data();
    resultImage.w = WIDTH;
    resultImage.h = HEIGHT;

    if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < n;) {
            gl_GlobalInvocationID = uvec3((unsigned)xs[i] / 4u, (unsigned)ys[i] / 4u, 0u);
            glsl_main();
        }
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < nthreads; ++k) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();

    for (size_t i = 0; i < n; ++i)
        std::memcpy(out + 4 * i, &image[((size_t)ys[i] * WIDTH + xs[i]) * 4], 4 * sizeof(float));
    return 0;
}

}  // extern "C"
