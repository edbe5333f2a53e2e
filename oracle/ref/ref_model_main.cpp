// ref_model_main.cpp - runs the reference's own model.frag (the mesh pass), compiled unchanged as
// C++ (oracle/ref/glsl_to_cpp.py + glsl_shim.h), on the CPU for a list of mesh fragments (test
// infrastructure: builds oracle/_ref/libref_model.so).
//
// The shader lights a fragment and then darkens it by the cloud shadow it marches:
// color *= 1 - 2 * accumDensity, clamped at 0 (model.frag:283-284).  The shadow is not an output of
// the shader, so each fragment is shaded twice, with the caller's low-res cloud texture and with an
// all-zero one (density 0, so accumDensity = 0); the caller recovers accumDensity from the ratio of
// the two colours wherever the shadowed colour is not clamped (accumDensity < 0.5).
//
// Fragment inputs: fragPositionWC = the world position; fragPosition = (camera.view * (wc, 1)).xyz;
// fragNormal / fragTangent / fragBitangent = the view-space images of +y / +x / +z; fragUV = (0.5,
// 0.5) on 1x1 material textures (albedo 0.5 grey, roughness 0.5, metalness 0, occlusion 1, flat
// normal).  None of them enters the shadow march, which reads only fragPositionWC, the camera,
// sun and sky blocks and the two cloud textures.
#include "model.gen.cpp"
#include "ref_uniforms.h"

namespace {

void bind(GlslSampler& s, const uint8_t* texels, int w, int h, int d, int channels) {
    s.texels = texels;
    s.w = w;
    s.h = h;
    s.d = d;
    s.channels = channels;
    s.is_float = false;
    s.clamp_edge = false;
}

}  // namespace

extern "C" {

// color_clouds / color_clear: n x 3 floats, the fragment's outColor.rgb with the caller's clouds and
// without clouds.  world_pos: n x 4 floats (xyz used).  Returns 0, or -1 on bad input.
int ref_model_shade(const mm_uniforms* u, const oracle_textures* t, const float* world_pos, size_t n,
                    float* color_clouds, float* color_clear, int nthreads) {
    if (!u || !t || (n && (!world_pos || !color_clouds || !color_clear))) return -1;
    camera.view = refshader::to_mat4(u->camera.view);
    camera.proj = refshader::to_mat4(u->camera.proj);
    camera.cameraPosition = refshader::to_vec4(u->camera.camera_position);
    model.model = mat4(1.0f);
    model.invTranspose = mat4(1.0f);
    sun.location = refshader::to_vec4(u->sun.location);
    sun.direction = refshader::to_vec4(u->sun.direction);
    sun.color = refshader::to_vec4(u->sun.color);
    sun.directionBasis = refshader::to_mat4(u->sun.direction_basis);
    sun.intensity = u->sun.intensity;
    sky.betaR = refshader::to_vec4(u->sky.beta_r);
    sky.betaV = refshader::to_vec4(u->sky.beta_v);
    sky.wind = refshader::to_vec4(u->sky.wind);
    sky.mie_directional = u->sky.mie_directional;

    static const uint8_t albedo[4] = {128, 128, 128, 255}, pbr[4] = {128, 0, 255, 255},
                         flat[4] = {128, 128, 255, 255}, zero[4] = {0, 0, 0, 0};
    bind(texColor, albedo, 1, 1, 1, 4);
    bind(pbrInfo, pbr, 1, 1, 1, 4);
    bind(normalMap, flat, 1, 1, 1, 4);
    bind(cloudPlacement, t->weather.texels, t->weather.width, t->weather.height, 1, t->weather.channels);

    for (int pass = 0; pass < 2; ++pass) {
        if (pass == 0)
            bind(lowResCloudShape, t->low_res.texels, t->low_res.width, t->low_res.height, t->low_res.depth,
                 t->low_res.channels);
        else
            bind(lowResCloudShape, zero, 1, 1, 1, 4);
        float* out = pass == 0 ? color_clouds : color_clear;
        refshader::parallel_for(n, nthreads, [&](size_t i) {
            const vec3 wc(world_pos[4 * i], world_pos[4 * i + 1], world_pos[4 * i + 2]);
            fragPositionWC = wc;
            fragPosition = vec3(camera.view * vec4(wc, 1.0f));
            fragNormal = vec3(camera.view * vec4(0.0f, 1.0f, 0.0f, 0.0f));
            fragTangent = vec3(camera.view * vec4(1.0f, 0.0f, 0.0f, 0.0f));
            fragBitangent = vec3(camera.view * vec4(0.0f, 0.0f, 1.0f, 0.0f));
            fragUV = vec2(0.5f, 0.5f);
            fragColor = vec3(1.0f);
            glsl_main();
            out[3 * i] = outColor.x;
            out[3 * i + 1] = outColor.y;
            out[3 * i + 2] = outColor.z;
        });
    }
    return 0;
}

}  // extern "C"
