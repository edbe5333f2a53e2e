// post.cu - the post-chain entry points (mm_post_*): argument checks, the per-launch constants
// computed on the host, the fast-arithmetic kernels (post_kernel.cuh); the exact instance is in
// post_exact.cu.
#include <stdint.h>
#include <string.h>

#include "post_kernel.cuh"

namespace mm {

int launch_post_exact(const PostLaunch& p, int which, cudaStream_t s);

namespace {

float uc2_host(float x) {  // tonemap.frag:11-14, host twin of post::uc2
    return ((x * (0.15f * x + 0.1f * 0.5f) + 0.2f * 0.02f) / (x * (0.15f * x + 0.5f) + 0.2f * 0.3f)) - 0.02f / 0.3f;
}

// (proj * view) * sun.location / w (god-ray.frag:44-46): the product of the matrices first (each
// element summed in index order), then the matrix-vector product summed pairwise,
// (m0 x + m1 y) + (m2 z + m3 w), as the CPU restatement evaluates both.
void sun_ndc(const mm_uniforms& u, float* sx, float* sy) {
    const float* P = u.camera.proj;
    const float* V = u.camera.view;
    float pv[16];
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) {
            float s = P[r] * V[c * 4];
            for (int k = 1; k < 4; ++k) s = s + P[k * 4 + r] * V[c * 4 + k];
            pv[c * 4 + r] = s;
        }
    const float* L = u.sun.location;
    float q[4];
    for (int r = 0; r < 4; ++r) q[r] = (pv[r] * L[0] + pv[4 + r] * L[1]) + (pv[8 + r] * L[2] + pv[12 + r] * L[3]);
    *sx = q[0] / q[3];
    *sy = q[1] / q[3];
}

int check_image(const mm_image* im, const char* what) {
    if (!im || !im->rgba || im->width <= 0 || im->height <= 0 || im->width > 32768 || im->height > 32768)
        return fail(MM_ERR_INVALID_ARGUMENT, "post: bad %s image", what);
    if (im->rgba_pitch_bytes < (size_t)im->width * 16 || im->rgba_pitch_bytes % 16 || ((uintptr_t)im->rgba) % 16)
        return fail(MM_ERR_INVALID_ARGUMENT, "post: %s must be 16-byte aligned float4 rows of >= 16*width bytes", what);
    return MM_OK;
}

int check_out8(const void* out, size_t pitch, int w) {
    if (!out || pitch < (size_t)w * 4 || pitch % 4 || ((uintptr_t)out) % 4)
        return fail(MM_ERR_INVALID_ARGUMENT, "post: 8-bit output must be 4-byte aligned rows of >= 4*width bytes");
    return MM_OK;
}

int resolve(const mm_post_options* opt, mm_post_options* o) {
    if (opt)
        *o = *opt;
    else
        mm_post_options_default(o);
    if (o->math != MM_MATH_FAST && o->math != MM_MATH_EXACT) return fail(MM_ERR_INVALID_ARGUMENT, "post: bad math %d", o->math);
    if (o->bgra != 0 && o->bgra != 1) return fail(MM_ERR_INVALID_ARGUMENT, "post: bgra must be 0 or 1");
    return MM_OK;
}

void fill_constants(const mm_uniforms* u, PostLaunch* p) {
    if (u) {
        p->night = u->sun.direction[1] < 0.0f;
        sun_ndc(*u, &p->sun_x, &p->sun_y);
        p->kr = u->sun.color[0] * u->sun.intensity;
        p->kg = u->sun.color[1] * u->sun.intensity;
        p->kb = u->sun.color[2] * u->sun.intensity;
    }
    p->whitemap = 1.0f / uc2_host(50.2f);
}

int run(const PostLaunch& p, int which, int math, cudaStream_t s) {
    if (math == MM_MATH_EXACT) return launch_post_exact(p, which, s);
    return post::launch<false>(p, which, s);
}

cudaTextureObject_t plane_texture(float* base, size_t pitch, int w, int h) {
    cudaResourceDesc rd;
    memset(&rd, 0, sizeof(rd));
    rd.resType = cudaResourceTypePitch2D;
    rd.res.pitch2D.devPtr = base;
    rd.res.pitch2D.desc = cudaCreateChannelDesc<float>();
    rd.res.pitch2D.width = (size_t)w;
    rd.res.pitch2D.height = (size_t)h;
    rd.res.pitch2D.pitchInBytes = pitch;
    cudaTextureDesc td;
    memset(&td, 0, sizeof(td));
    td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;  // CLAMP_TO_EDGE
    td.filterMode = cudaFilterModeLinear;
    td.readMode = cudaReadModeElementType;
    td.normalizedCoords = 1;
    cudaTextureObject_t t = 0;
    if (cudaCreateTextureObject(&t, &rd, &td, nullptr) != cudaSuccess) return 0;
    return t;
}

// The two float planes of the chain (god-ray term, cloud alpha) for a w x h frame, with texture
// objects; kept in the context while the frame size stays the same.
int ensure_planes(mm_context ctx, int w, int h) {
    if (ctx->post_plane && ctx->post_w == w && ctx->post_h == h) return MM_OK;
    post_state_destroy(ctx);  // synchronizes with work that may still read the old planes
    // A texture object's base address must be a multiple of the device's texture alignment and its
    // pitch a multiple of the texture pitch alignment: both planes start on such a boundary.
    int align = 512, pitch_align = 32;
    cudaDeviceGetAttribute(&align, cudaDevAttrTextureAlignment, ctx->device);
    cudaDeviceGetAttribute(&pitch_align, cudaDevAttrTexturePitchAlignment, ctx->device);
    const size_t pa = (size_t)(pitch_align > 128 ? pitch_align : 128), ba = (size_t)(align > 256 ? align : 256);
    const size_t pitch = ((size_t)w * 4 + pa - 1) / pa * pa;
    const size_t plane = (pitch * (size_t)h + ba - 1) / ba * ba;
    char* raw = nullptr;
    MM_CUDA_TRY(cudaMalloc(&raw, 2 * plane + ba));
    char* base = raw + ((ba - ((uintptr_t)raw % ba)) % ba);
    ctx->post_raw = raw;
    ctx->post_plane = reinterpret_cast<float*>(base);
    ctx->post_aplane = reinterpret_cast<float*>(base + plane);
    ctx->post_pitch = pitch;
    ctx->post_w = w;
    ctx->post_h = h;
    ctx->post_gtex = plane_texture(ctx->post_plane, pitch, w, h);
    ctx->post_atex = plane_texture(ctx->post_aplane, pitch, w, h);
    if (!ctx->post_gtex || !ctx->post_atex) {
        post_state_destroy(ctx);
        return fail(MM_ERR_CUDA, "post: cannot create the plane texture objects");
    }
    return MM_OK;
}

bool overlaps(const mm_image* a, const mm_image* b) {
    const char* a0 = (const char*)a->rgba;
    const char* a1 = a0 + a->rgba_pitch_bytes * (size_t)a->height;
    const char* b0 = (const char*)b->rgba;
    const char* b1 = b0 + b->rgba_pitch_bytes * (size_t)b->height;
    return a0 < b1 && b0 < a1;
}

}  // namespace

void post_state_destroy(mm_context ctx) {
    if (ctx->post_gtex) cudaDestroyTextureObject(ctx->post_gtex);
    if (ctx->post_atex) cudaDestroyTextureObject(ctx->post_atex);
    cudaFree(ctx->post_raw);
    ctx->post_raw = nullptr;
    ctx->post_plane = ctx->post_aplane = nullptr;
    ctx->post_gtex = ctx->post_atex = 0;
    ctx->post_pitch = 0;
    ctx->post_w = ctx->post_h = 0;
}

}  // namespace mm

extern "C" int mm_post_options_default(mm_post_options* o) {
    if (!o) return mm::fail(MM_ERR_INVALID_ARGUMENT, "post: null options");
    o->math = MM_MATH_FAST;
    o->bgra = 1;
    return MM_OK;
}

static int post_pass(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                     const mm_post_options* opt, void* stream, int which) {
    using namespace mm;
    if (!ctx || !u) return fail(MM_ERR_INVALID_ARGUMENT, "post: null argument");
    mm_post_options o;
    int r;
    if ((r = resolve(opt, &o)) || (r = check_image(src, "source")) || (r = check_image(dst, "destination"))) return r;
    if (src->width != dst->width || src->height != dst->height)
        return fail(MM_ERR_INVALID_ARGUMENT, "post: source and destination differ in size");
    if (overlaps(src, dst)) return fail(MM_ERR_INVALID_ARGUMENT, "post: source and destination overlap");
    PostLaunch p;
    memset(&p, 0, sizeof(p));
    p.src = src->rgba;
    p.src_pitch = src->rgba_pitch_bytes;
    p.dst = reinterpret_cast<float4*>(dst->rgba);
    p.dst_pitch = dst->rgba_pitch_bytes;
    p.width = src->width;
    p.height = src->height;
    p.bgra = o.bgra;
    fill_constants(u, &p);
    return run(p, which, o.math, (cudaStream_t)stream);
}

extern "C" int mm_post_god_rays(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                                const mm_post_options* opt, void* stream) {
    return post_pass(ctx, u, src, dst, opt, stream, 0);
}

extern "C" int mm_post_radial_blur(mm_context ctx, const mm_uniforms* u, const mm_image* src, const mm_image* dst,
                                   const mm_post_options* opt, void* stream) {
    return post_pass(ctx, u, src, dst, opt, stream, 1);
}

extern "C" int mm_post_tonemap(mm_context ctx, const mm_image* src, void* out, size_t out_pitch_bytes,
                               const mm_post_options* opt, void* stream) {
    using namespace mm;
    if (!ctx) return fail(MM_ERR_INVALID_ARGUMENT, "post: null context");
    mm_post_options o;
    int r;
    if ((r = resolve(opt, &o)) || (r = check_image(src, "source")) || (r = check_out8(out, out_pitch_bytes, src->width)))
        return r;
    PostLaunch p;
    memset(&p, 0, sizeof(p));
    p.src = src->rgba;
    p.src_pitch = src->rgba_pitch_bytes;
    p.out8 = static_cast<uint8_t*>(out);
    p.out8_pitch = out_pitch_bytes;
    p.width = src->width;
    p.height = src->height;
    p.bgra = o.bgra;
    fill_constants(nullptr, &p);
    return run(p, 2, o.math, (cudaStream_t)stream);
}

extern "C" int mm_post_chain(mm_context ctx, const mm_uniforms* u, const mm_image* clouds, const mm_image* mesh,
                             void* out, size_t out_pitch_bytes, const mm_post_options* opt, void* stream) {
    using namespace mm;
    if (!ctx || !u) return fail(MM_ERR_INVALID_ARGUMENT, "post: null argument");
    mm_post_options o;
    int r;
    if ((r = resolve(opt, &o)) || (r = check_image(clouds, "cloud")) ||
        (r = check_out8(out, out_pitch_bytes, clouds->width)))
        return r;
    if (mesh) {
        if ((r = check_image(mesh, "mesh"))) return r;
        if (mesh->width != clouds->width || mesh->height != clouds->height)
            return fail(MM_ERR_INVALID_ARGUMENT, "post: mesh layer and cloud image differ in size");
    }
    if ((r = ensure_planes(ctx, clouds->width, clouds->height))) return r;
    PostLaunch p;
    memset(&p, 0, sizeof(p));
    p.src = clouds->rgba;
    p.src_pitch = clouds->rgba_pitch_bytes;
    p.plane = ctx->post_plane;
    p.aplane = ctx->post_aplane;
    p.plane_pitch = ctx->post_pitch;
    p.gtex = ctx->post_gtex;
    p.atex = ctx->post_atex;
    p.mesh = mesh ? reinterpret_cast<const float4*>(mesh->rgba) : nullptr;
    p.mesh_pitch = mesh ? mesh->rgba_pitch_bytes : 0;
    p.out8 = static_cast<uint8_t*>(out);
    p.out8_pitch = out_pitch_bytes;
    p.width = clouds->width;
    p.height = clouds->height;
    p.bgra = o.bgra;
    fill_constants(u, &p);
    if (o.math == MM_MATH_EXACT) return launch_post_exact(p, 3, (cudaStream_t)stream);
    return post::launch<false>(p, 4, (cudaStream_t)stream);
}
