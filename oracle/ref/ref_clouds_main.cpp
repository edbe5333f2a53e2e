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

#include "compute_clouds.gen.cpp"
#include "ref_uniforms.h"

namespace {

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
    refshader::load_blocks(u, camera, cameraPrev, sun, sky);
    bind(cloudPlacement, t->weather);
    bind(nightSkyMap, t->night_sky);
    bind(curlNoise, t->curl);
    bind(lowResCloudShape, t->low_res);
    bind(hiResCloudShape, t->hi_res);

    std::vector<float> image((size_t)WIDTH * HEIGHT * 4, 0.0f);
    resultImage.texels = image.data();
    resultImage.w = WIDTH;
    resultImage.h = HEIGHT;

    refshader::parallel_for(n, nthreads, [&](size_t i) {
        gl_GlobalInvocationID = uvec3((unsigned)xs[i] / 4u, (unsigned)ys[i] / 4u, 0u);
        glsl_main();
    });

    for (size_t i = 0; i < n; ++i)
        std::memcpy(out + 4 * i, &image[((size_t)ys[i] * WIDTH + xs[i]) * 4], 4 * sizeof(float));
    return 0;
}

}  // extern "C"
