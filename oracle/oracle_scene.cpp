// oracle_scene.cpp - CPU restatement of the host-side uniform set-up (test infrastructure only).
//
// The benchmark's reference arm and the oracle tests build the four uniform blocks here, without the
// CUDA library: the camera block as Camera builds it (SkyEngine/SkyEngine/camera.cpp:27-39 getView,
// :139-147 the yaw/pitch basis, glm::perspective for getProj with proj[1][1] negated as
// VulkanApplication.cpp:361-362 does, cameraParams = (aspect, tan(0.5 * DEG2RAD * fov)) with
// DEG2RAD = 0.01745f, camera.h:15,72; near 0.1, far 1000 as VulkanApplication.cpp:76 builds the
// camera), and the sun/sky blocks as SkyManager fills them (SkyManager.cpp:15-70 with the
// constructor's constants, :72-100).  SkyManager leaves `turbidity` uninitialised; 10 is used (its
// only effect, betaV, is ~1e-19 for any finite value).
//
// Angles: (yaw, pitch) name the direction the image centre looks at, (cos yaw cos pitch, sin pitch,
// sin yaw cos pitch); the shader's rays travel along -m_forward (compute-clouds.comp:312-322), so
// m_forward is the reverse of that direction.  The sun direction is (cos el cos az, sin el,
// cos el sin az).  pixel_phase goes to sun.color.a (VulkanApplication.cpp:386).
#include <math.h>
#include <string.h>

#include <algorithm>

#include "oracle.h"

namespace {

struct Vec {
    float x, y, z;
};

Vec scale(Vec a, float s) { return {a.x * s, a.y * s, a.z * s}; }
float dotp(Vec a, Vec b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// glm::cross
Vec crossp(Vec a, Vec b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
// glm::normalize: v * inversesqrt(dot(v, v))
Vec unit(Vec a) { return scale(a, 1.0f / sqrtf(dotp(a, a))); }

void camera_block(const float eye[3], double yaw_deg, double pitch_deg, float fov_deg, int w, int h,
                  mm_uniforms* u) {
    const double r = 3.14159265358979323846 / 180.0;
    const double cy = cos(yaw_deg * r), sy = sin(yaw_deg * r), cp = cos(pitch_deg * r), sp = sin(pitch_deg * r);
    const Vec look = {(float)(cy * cp), (float)sp, (float)(sy * cp)};
    const Vec fwd = scale(look, -1.0f);
    // camera.cpp:143-146: world up, or +z when the forward is (anti)parallel to it (EPSILON 1e-5)
    const Vec wup = (1.0f - fabsf(dotp(fwd, Vec{0.0f, 1.0f, 0.0f})) < 0.00001f) ? Vec{0, 0, 1} : Vec{0, 1, 0};
    const Vec right = unit(crossp(fwd, wup));
    const Vec up = unit(crossp(right, fwd));
    const Vec pos = {eye[0], eye[1], eye[2]};
    mm_camera_ubo& c = u->camera;
    memset(&c, 0, sizeof(c));
    // getView = view * trans, view's columns (right.i, up.i, fwd.i, 0), trans[3] = (-pos, 1)
    const Vec rows[3] = {right, up, fwd};
    for (int i = 0; i < 3; ++i) {
        c.view[4 * 0 + i] = i == 0 ? right.x : i == 1 ? up.x : fwd.x;
        c.view[4 * 1 + i] = i == 0 ? right.y : i == 1 ? up.y : fwd.y;
        c.view[4 * 2 + i] = i == 0 ? right.z : i == 1 ? up.z : fwd.z;
        c.view[12 + i] = -dotp(rows[i], pos);
    }
    c.view[15] = 1.0f;
    // glm::perspective(DEG2RAD * fov, aspect, 0.1, 1000), then proj[1][1] *= -1
    const float deg2rad = 0.01745f, zn = 0.1f, zf = 1000.0f;
    const float aspect = (float)w / (float)h;
    const float tanHalf = tanf(deg2rad * fov_deg / 2.0f);
    c.proj[0] = 1.0f / (aspect * tanHalf);
    c.proj[5] = -(1.0f / tanHalf);
    c.proj[10] = -(zf + zn) / (zf - zn);
    c.proj[11] = -1.0f;
    c.proj[14] = -(2.0f * zf * zn) / (zf - zn);
    c.camera_position[0] = pos.x;
    c.camera_position[1] = pos.y;
    c.camera_position[2] = pos.z;
    c.camera_position[3] = 1.0f;
    c.camera_params[0] = aspect;
    c.camera_params[1] = tanf(0.5f * deg2rad * fov_deg);
    // the previous frame's camera: the same camera (a still frame)
    memcpy(u->camera_prev.view, c.view, sizeof(c.view));
    memcpy(u->camera_prev.proj, c.proj, sizeof(c.proj));
    memcpy(u->camera_prev.camera_position, c.camera_position, sizeof(c.camera_position));
}

void sun_sky_blocks(Vec dir, float time, int phase, mm_uniforms* u) {
    mm_sun_ubo& s = u->sun;
    mm_sky_ubo& k = u->sky;
    memset(&s, 0, sizeof(s));
    memset(&k, 0, sizeof(k));
    const bool below = dir.y < 0.0f;
    // calcSunPosition (SkyManager.cpp:52-69)
    const float dist = 400000.0f;
    const float d4[4] = {dir.x, dir.y, dir.z, 0.0f};
    const float l4[4] = {dist * dir.x, dist * dir.y, dist * dir.z, 1.0f};
    for (int i = 0; i < 4; ++i) {
        s.direction[i] = d4[i];
        s.location[i] = below ? -l4[i] : l4[i];
    }
    Vec side;
    if (fabsf(dir.y) < 0.001f)
        side = dir.z < 0.0f ? Vec{0, 1, 0} : Vec{0, -1, 0};
    else
        side = Vec{0, 0, 1};
    const Vec n = unit(crossp(dir, side));
    const Vec b = unit(crossp(dir, n));
    const float basis[16] = {n.x, n.y, n.z, 0.0f, dir.x, dir.y, dir.z, 0.0f, b.x, b.y, b.z, 0.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    for (int i = 0; i < 16; ++i) s.direction_basis[i] = below ? -basis[i] : basis[i];
    // calcSunIntensity (:28-34)
    const float zc = std::max(-1.0f, std::min(1.0f, dir.y));
    s.intensity = below ? 2.0f
                        : 1000.0f * std::max(0.0f, 1.0f - powf(2.718281828459f,
                                                               -((1.6110731557f - acosf(zc)) / 1.5f)));
    // calcSunColor (:15-26)
    if (below) {
        s.color[0] = 0.8f;
        s.color[1] = 0.9f;
        s.color[2] = 1.0f;
    } else {
        const float t = std::max(0.0f, std::min(1.0f, dir.y * 13.0f));
        const float sunset[3] = {2.0f, 0.33922f, 0.0431f};
        for (int i = 0; i < 3; ++i) s.color[i] = (1.0f - t) * sunset[i] + t * 1.0f;
    }
    s.color[3] = (float)phase;
    // calcSkyBetaR / calcSkyBetaV (:36-44): rayleigh 2, mie 0.005, mie_directional 0.8, wind (1, 0.05, 1)
    const double rt[3] = {5.804542996261093E-6, 1.3562911419845635E-5, 3.0265902468824876E-5};
    const float mc[3] = {1.839991851443397f, 2.779802391966052f, 4.079047954386109f};
    const float fade = 1.0f - std::max(0.0f, std::min(1.0f, (float)(1.0f - exp(s.location[1] / 450000.0))));
    const float cm = (0.2f * 10.0f) * 10E-18f;
    for (int i = 0; i < 3; ++i) {
        k.beta_r[i] = (float)rt[i] * (2.0f - 1.0f + fade);
        k.beta_v[i] = 0.434f * cm * mc[i] * 0.005f;
    }
    k.wind[0] = 1.0f;
    k.wind[1] = 0.05f;
    k.wind[2] = 1.0f;
    k.wind[3] = time;
    k.mie_directional = 0.8f;
}

}  // namespace

extern "C" int oracle_uniforms(const float eye[3], float yaw_deg, float pitch_deg, float fov_deg, int width,
                               int height, float sun_elevation_deg, float sun_azimuth_deg, float time,
                               int pixel_phase, mm_uniforms* u) {
    if (!eye || !u || width <= 0 || height <= 0 || !(fov_deg > 0.0f && fov_deg < 180.0f) || pixel_phase < 0 ||
        pixel_phase > 15)
        return 1;
    camera_block(eye, yaw_deg, pitch_deg, fov_deg, width, height, u);
    const double r = 3.14159265358979323846 / 180.0;
    const double ce = cos(sun_elevation_deg * r), se = sin(sun_elevation_deg * r);
    const double ca = cos(sun_azimuth_deg * r), sa = sin(sun_azimuth_deg * r);
    sun_sky_blocks(Vec{(float)(ce * ca), (float)se, (float)(ce * sa)}, time, pixel_phase, u);
    return 0;
}
