// ref_reproject_main.cpp - runs the reference's own reproject.comp, compiled unchanged as C++
// (oracle/ref/glsl_to_cpp.py + glsl_shim.h), on the CPU (test infrastructure: builds
// oracle/_ref/libref_reproject.so, which only regenerates and re-checks golden fixtures).
//
// The shader is dispatched at full resolution: invocation (x, y) writes targetImage pixel (x, y)
// from sourceImage (RGBA32F, the same size) with the camera and cameraPrev blocks.
#include "reproject.gen.cpp"
#include "ref_uniforms.h"

extern "C" {

// dst (w x h float4 rows) = reproject.comp applied to src (w x h float4 rows).  Returns 0, or -1.
int ref_reproject(const mm_uniforms* u, const float* src, int w, int h, float* dst, int nthreads) {
    if (!u || !src || !dst || w <= 0 || h <= 0) return -1;
    refshader::load_blocks(u, camera, cameraPrev, sun, sky);
    sourceImage.texels = const_cast<float*>(src);  // read only: the shader declares it readonly
    sourceImage.w = w;
    sourceImage.h = h;
    targetImage.texels = dst;
    targetImage.w = w;
    targetImage.h = h;
    refshader::parallel_for((size_t)w * h, nthreads, [&](size_t i) {
        gl_GlobalInvocationID = uvec3((unsigned)(i % (size_t)w), (unsigned)(i / (size_t)w), 0u);
        glsl_main();
    });
    return 0;
}

}  // extern "C"
