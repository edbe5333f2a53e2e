// ref_post_main.cpp - runs one of the reference's post-pass fragment shaders (god-ray.frag,
// radialBlur.frag, tonemap.frag), compiled unchanged as C++ (oracle/ref/glsl_to_cpp.py +
// glsl_shim.h), on the CPU over a whole image (test infrastructure: builds
// oracle/_ref/libref_god_ray.so, libref_radial_blur.so, libref_tonemap.so).
//
// Built once per shader: REF_SHADER_GEN names the generated translation unit, REF_ENTRY the
// exported function, REF_HAS_BLOCKS whether the shader declares the camera and sun blocks.  The
// full-screen pass shades pixel (x, y) of a w x h target with fragUV at the pixel centre,
// ((x + 0.5) / w, (y + 0.5) / h); texColor is the RGBA32F input (LINEAR, CLAMP_TO_EDGE).
#include REF_SHADER_GEN
#include "ref_uniforms.h"

extern "C" {

// dst (w x h float4 rows) = the shader's outColor for every pixel of src (w x h float4 rows).
int REF_ENTRY(const mm_uniforms* u, const float* src, int w, int h, float* dst, int nthreads) {
    if (!src || !dst || w <= 0 || h <= 0) return -1;
#if REF_HAS_BLOCKS
    if (!u) return -1;
    camera.view = refshader::to_mat4(u->camera.view);
    camera.proj = refshader::to_mat4(u->camera.proj);
    camera.cameraPosition = vec3(u->camera.camera_position[0], u->camera.camera_position[1],
                                 u->camera.camera_position[2]);
    sun.location = refshader::to_vec4(u->sun.location);
    sun.direction = refshader::to_vec4(u->sun.direction);
    sun.color = refshader::to_vec4(u->sun.color);
    sun.directionBasis = refshader::to_mat4(u->sun.direction_basis);
    sun.intensity = u->sun.intensity;
#else
    (void)u;
#endif
    texColor.texels = src;
    texColor.w = w;
    texColor.h = h;
    texColor.d = 1;
    texColor.channels = 4;
    texColor.is_float = true;
    texColor.clamp_edge = true;
    refshader::parallel_for((size_t)w * h, nthreads, [&](size_t i) {
        const int x = (int)(i % (size_t)w), y = (int)(i / (size_t)w);
        fragUV = vec2(((float)x + 0.5f) / (float)w, ((float)y + 0.5f) / (float)h);
        glsl_main();
        float* o = dst + 4 * i;
        o[0] = outColor.x;
        o[1] = outColor.y;
        o[2] = outColor.z;
        o[3] = outColor.w;
    });
    return 0;
}

}  // extern "C"
