// oracle_reproject.cpp - CPU restatement of SkyEngine/SkyEngine/Shaders/reproject.comp:91-152
// (test infrastructure only).  Float arithmetic in source order without contraction, so the GPU
// kernel (built without FMA contraction) must match it bit for bit.
#include <math.h>

#include "oracle.h"

namespace {

struct v3 {
    float x, y, z;
};
inline v3 add(v3 a, v3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline v3 sub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline v3 mul(float s, v3 a) { return {s * a.x, s * a.y, s * a.z}; }
inline v3 mulv(v3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline float dot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline v3 normalize(v3 a) { return mulv(a, 1.0f / sqrtf(dot(a, a))); }

// raySphereIntersection(...).point (reproject.comp:57-87); (0,0,0) when there is no hit.
v3 sphere_point(v3 ro, v3 rd, v3 c, float w) {
    ro = sub(ro, c);
    ro = {ro.x / w, ro.y / w, ro.z / w};
    float A = dot(rd, rd);
    float B = 2.0f * dot(rd, ro);
    float C = dot(ro, ro) - 0.25f;
    float disc = B * B - 4.0f * A * C;
    if (disc < 0.0f) return {0.0f, 0.0f, 0.0f};
    float t = (-sqrtf(disc) - B) / A * 0.5f;
    if (t < 0.0f) t = (sqrtf(disc) - B) / A * 0.5f;
    if (!(t >= 0.0f)) return {0.0f, 0.0f, 0.0f};
    v3 p = add(ro, mulv(rd, t));
    p = mulv(p, w);
    return add(p, c);
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace

extern "C" int oracle_reproject_f32(const mm_uniforms* u, const float* src_rgba, const float* src_depth, int w, int h,
                                    float* dst_rgba, float* dst_depth) {
    if (!u || !src_rgba || !dst_rgba || w <= 0 || h <= 0) return MM_ERR_INVALID_ARGUMENT;
    const float* view = u->camera.view;
    const float* pv = u->camera_prev.view;
    const v3 cam = {u->camera.camera_position[0], u->camera.camera_position[1], u->camera.camera_position[2]};
    const float cpx = u->camera.camera_params[0], cpy = u->camera.camera_params[1];
    const v3 look = {view[2], view[6], view[10]}, right = {view[0], view[4], view[8]}, up = {view[1], view[5], view[9]};
    v3 center = cam;
    center.y = -2000000.0f * 0.5f * 0.995f;
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const float uvx = (float)x / (float)w, uvy = (float)y / (float)h;  // :93-94
            const float sx = uvx * 2.0f - 1.0f, sy = uvy * 2.0f - 1.0f;
            const v3 ref = sub(cam, look);
            v3 p = sub(add(ref, mul(cpx * sx * cpy, right)), mul(sy * cpy, up));
            const v3 rd = normalize(sub(p, cam));
            v3 ip = sphere_point(cam, rd, center, 2000000.0f);  // :120
            // (cameraPrev.view * vec4(ip, 1)).xyz (:125).  GLSL leaves the order of the sum to its
            // compiler; this is glm's, (m0 x + m1 y) + (m2 z + m3 w), so the restatement equals the
            // shader compiled on glm bit for bit.
            v3 q = {(pv[0] * ip.x + pv[4] * ip.y) + (pv[8] * ip.z + pv[12]),
                    (pv[1] * ip.x + pv[5] * ip.y) + (pv[9] * ip.z + pv[13]),
                    (pv[2] * ip.x + pv[6] * ip.y) + (pv[10] * ip.z + pv[14])};
            v3 od = normalize(q);
            const float nz = -od.z;
            od = {od.x / nz, od.y / nz, od.z / nz};  // :132
            float oldU = od.x / cpy / cpx;
            oldU = oldU * 0.5f + 0.5f;
            float oldV = -od.y / cpy;
            oldV = oldV * 0.5f + 0.5f;
            const float bx = oldU - uvx, by = oldV - uvy;
            float acc[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            for (int s = 0; s < 10; ++s) {  // :142-147
                const float k = (float)s / 9.0f - 0.5f;
                const float ox = bx * k, oy = by * k;
                const float ix = roundf((oldU - ox) * (float)w), iy = roundf((oldV - oy) * (float)h);
                const int cx = clampi((int)ix, 0, w - 1), cy = clampi((int)iy, 0, h - 1);
                const float* t = src_rgba + 4 * ((size_t)cy * w + cx);
                for (int c = 0; c < 4; ++c) acc[c] += t[c];
            }
            for (int c = 0; c < 4; ++c) acc[c] /= 10.0f;
            const int cx = clampi((int)roundf(oldU * (float)w), 0, w - 1), cy = clampi((int)roundf(oldV * (float)h), 0, h - 1);
            acc[3] = src_rgba[4 * ((size_t)cy * w + cx) + 3];  // :150-151
            float* o = dst_rgba + 4 * ((size_t)y * w + x);
            for (int c = 0; c < 4; ++c) o[c] = acc[c];
            if (dst_depth && src_depth) dst_depth[(size_t)y * w + x] = src_depth[(size_t)cy * w + cx];
        }
    return MM_OK;
}
