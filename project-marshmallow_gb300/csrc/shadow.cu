// shadow.cu - mm_mesh_shadow: argument checks and the fast-arithmetic instance of the mesh
// cloud-shadow march (shadow_kernel.cuh); the exact instance is in shadow_exact.cu.
#include <stdint.h>
#include <string.h>

#include "shadow_kernel.cuh"

namespace mm {

int launch_shadow_exact(const ShadowLaunch& p, int sampler, cudaStream_t s);

}  // namespace mm

extern "C" int mm_mesh_shadow(mm_context ctx, const mm_uniforms* u, const mm_scene_textures* tex,
                              const mm_gbuffer* g, float* shadow, size_t shadow_pitch_bytes, float* rgba,
                              size_t rgba_pitch_bytes, const mm_march_options* opt, void* stream) {
    using mm::fail;
    if (!ctx || !u || !tex || !g) return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: null argument");
    mm_march_options o;
    if (opt)
        o = *opt;
    else
        mm_march_options_default(&o);
    if (o.sampler != MM_SAMPLER_HARDWARE && o.sampler != MM_SAMPLER_SOFTWARE)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: bad sampler %d", o.sampler);
    if (o.math != MM_MATH_FAST && o.math != MM_MATH_EXACT)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: bad math %d", o.math);
    if (!(o.coverage_offset == o.coverage_offset) || o.coverage_offset < -1.0f || o.coverage_offset > 1.0f)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: coverage_offset must be in [-1, 1]");
    if (!g->world_pos || g->width <= 0 || g->height <= 0 || g->width > 32768 || g->height > 32768)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: bad G-buffer");
    if (g->world_pos_pitch_bytes < (size_t)g->width * 16 || g->world_pos_pitch_bytes % 16 ||
        ((uintptr_t)g->world_pos) % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: world_pos must be 16-byte aligned rows of >= 16*width bytes");
    if (!shadow && !rgba) return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: neither shadow nor rgba output");
    if (shadow && (shadow_pitch_bytes < (size_t)g->width * 4 || shadow_pitch_bytes % 4 || ((uintptr_t)shadow) % 4))
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: bad shadow pitch");
    if (rgba && (rgba_pitch_bytes < (size_t)g->width * 16 || rgba_pitch_bytes % 16 || ((uintptr_t)rgba) % 16))
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: bad rgba pitch or alignment");
    if (!tex->weather || !tex->low_res) return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: missing weather or low_res");
    if (tex->weather->depth != 1 || tex->low_res->depth < 2 || tex->weather->channels != 4 ||
        tex->low_res->channels != 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: weather must be 2D RGBA and low_res 3D RGBA");
    if (!tex->weather->tex || !tex->low_res->tex)
        return fail(MM_ERR_INVALID_ARGUMENT, "mesh_shadow: texture without a texture object");
    mm::ShadowLaunch p;
    memset(&p, 0, sizeof(p));
    p.u = *u;
    p.weather = mm::texture_view(tex->weather);
    p.low = mm::texture_view(tex->low_res);
    p.pos = reinterpret_cast<const float4*>(g->world_pos);
    p.pos_pitch = g->world_pos_pitch_bytes;
    p.shadow = shadow;
    p.shadow_pitch = shadow_pitch_bytes;
    p.rgba = reinterpret_cast<float4*>(rgba);
    p.rgba_pitch = rgba_pitch_bytes;
    p.width = g->width;
    p.height = g->height;
    p.coverage_offset = o.coverage_offset;
    cudaStream_t s = (cudaStream_t)stream;
    if (o.math == MM_MATH_EXACT) return mm::launch_shadow_exact(p, o.sampler, s);
    if (o.sampler == MM_SAMPLER_SOFTWARE) return mm::shadow::launch<false, MM_SAMPLER_SOFTWARE>(p, s);
    return mm::shadow::launch<false, MM_SAMPLER_HARDWARE>(p, s);
}
