// scene.cpp - host "scene -> uniforms" set-up: the camera and sky math that fills the reference's
// uniform blocks each frame (VulkanApplication.cpp:351-395), restated without glm/GLFW.
//
//  - camera: Camera::addYaw/addPitch basis (camera.cpp:139-148 / SE camera.cpp:230-238), the view
//    matrix layout of Camera::getView (camera.cpp:27-39), glm::perspective for proj with
//    proj[1][1] negated (VulkanApplication.cpp:361-362) and cameraParams = (aspect,
//    tan(0.5 * DEG2RAD * fov)) with DEG2RAD = 0.01745f (camera.h:15,72).
//  - sky: SkyManager::calcSunPosition/calcSunIntensity/calcSunColor/calcSkyBetaR/calcSkyBetaV
//    (SkyManager.cpp:15-70) with the constructor's constants (SkyManager.cpp:72-100).
//    SkyManager leaves `turbidity` uninitialised; it is fixed at 10 here.  Its only effect is
//    on betaV, which is ~1e-19 for any finite value because MIE_CONST lacks the 1e14 factor of
//    the Preetham constants it was taken from.
#include <math.h>
#include <string.h>

#include <algorithm>

#include "../../include/mm.h"
#include "mm_internal.h"

namespace {

struct v3f {
    float x, y, z;
};

v3f cross(v3f a, v3f b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
float dot(v3f a, v3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
v3f normalize(v3f a) {
    float s = 1.0f / sqrtf(dot(a, a));
    return {a.x * s, a.y * s, a.z * s};
}

const float kDeg2RadRef = 0.01745f;  // camera.h:15

// Shared tail of SkyManager::calcSunPosition (SkyManager.cpp:54-69) and the calcSun*/calcSky*
// functions that rebuildSkyFromNewSun runs after it (SkyManager.cpp:108-116).
void fill_sky(v3f dir, float time, int phase, mm_uniforms* u) {
    mm_sun_ubo& sun = u->sun;
    mm_sky_ubo& sky = u->sky;
    memset(&sun, 0, sizeof(sun));
    memset(&sky, 0, sizeof(sky));
    // calcSunPosition
    sun.direction[0] = dir.x;
    sun.direction[1] = dir.y;
    sun.direction[2] = dir.z;
    sun.direction[3] = 0.0f;
    const float SUN_DISTANCE = 400000.0f;
    sun.location[0] = SUN_DISTANCE * dir.x;
    sun.location[1] = SUN_DISTANCE * dir.y;
    sun.location[2] = SUN_DISTANCE * dir.z;
    sun.location[3] = 1.0f;
    if (sun.direction[1] < 0.0f)
        for (int i = 0; i < 4; ++i) sun.location[i] *= -1.0f;
    v3f right = (fabsf(dir.y) < 0.001f) ? ((dir.z < 0) ? v3f{0, 1, 0} : v3f{0, -1, 0}) : v3f{0, 0, 1};
    v3f n = normalize(cross(dir, right));
    v3f b = normalize(cross(dir, n));
    float* m = sun.direction_basis;  // column-major; starts as identity
    for (int i = 0; i < 16; ++i) m[i] = (i % 5 == 0) ? 1.0f : 0.0f;
    m[4] = dir.x; m[5] = dir.y; m[6] = dir.z; m[7] = 0.0f;
    m[0] = n.x;   m[1] = n.y;   m[2] = n.z;   m[3] = 0.0f;
    m[8] = b.x;   m[9] = b.y;   m[10] = b.z;  m[11] = 0.0f;
    if (sun.direction[1] < 0.0f)
        for (int i = 0; i < 16; ++i) m[i] *= -1.0f;
    // calcSunIntensity (SkyManager.cpp:28-34)
    const float EE = 1000.0f, E = 2.718281828459f, SHADOW_CUTOFF = 1.6110731557f, SHADOW_STEEPNESS = 1.5f;
    float zc = std::max(-1.f, std::min(1.f, sun.direction[1]));
    sun.intensity = EE * std::max(0.f, 1.f - powf(E, -((SHADOW_CUTOFF - acosf(zc)) / SHADOW_STEEPNESS)));
    if (sun.direction[1] < 0.0f) sun.intensity = 2.0f;
    // calcSunColor (SkyManager.cpp:15-26)
    if (sun.direction[1] < 0.0f) {
        sun.color[0] = 0.8f; sun.color[1] = 0.9f; sun.color[2] = 1.0f;
    } else {
        const float sunset[3] = {2.f, 0.33922f, 0.0431f};
        float t = std::max(0.f, std::min(1.f, sun.direction[1] * 13.f));
        for (int i = 0; i < 3; ++i) sun.color[i] = (1.f - t) * sunset[i] + t * 1.0f;
    }
    sun.color[3] = (float)phase;
    // calcSkyBetaR / calcSkyBetaV (SkyManager.cpp:36-44) with rayleigh = 2, mie = 0.005
    const float rayleigh = 2.f, mie = 0.005f, turbidity = 10.f;
    const float RT[3] = {5.804542996261093E-6f, 1.3562911419845635E-5f, 3.0265902468824876E-5f};
    const float MC[3] = {1.839991851443397f, 2.779802391966052f, 4.079047954386109f};
    float sunFade = 1.0f - std::max(0.0f, std::min(1.0f, (float)(1.0f - exp(sun.location[1] / 450000.0))));
    for (int i = 0; i < 3; ++i) sky.beta_r[i] = RT[i] * (rayleigh - 1.f + sunFade);
    float c = (0.2f * turbidity) * 10E-18f;
    for (int i = 0; i < 3; ++i) sky.beta_v[i] = 0.434f * c * MC[i] * mie;
    sky.wind[0] = 1.0f;
    sky.wind[1] = 0.05f;
    sky.wind[2] = 1.0f;
    sky.wind[3] = time;
    sky.mie_directional = 0.8f;
}

}  // namespace

extern "C" {

int mm_camera_from_angles(const float eye[3], float yaw_deg, float pitch_deg, float fov_deg, int width,
                          int height, mm_uniforms* u) {
    if (!eye || !u) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mm_camera_from_angles: null pointer");
    if (width <= 0 || height <= 0 || !(fov_deg > 0.0f && fov_deg < 180.0f))
        return mm::fail(MM_ERR_INVALID_ARGUMENT, "mm_camera_from_angles: bad size or fov");
    const double d2r = 3.14159265358979323846 / 180.0;
    const double yaw = yaw_deg * d2r, pitch = pitch_deg * d2r;
    v3f d = {(float)(cos(yaw) * cos(pitch)), (float)sin(pitch), (float)(sin(yaw) * cos(pitch))};
    v3f fwd = {-d.x, -d.y, -d.z};
    // camera.cpp:234-237 (SE/camera.cpp addYaw): world up unless the forward is vertical
    v3f wup = (1.0f - fabsf(dot(fwd, v3f{0, 1, 0})) < 0.00001f) ? v3f{0, 0, 1} : v3f{0, 1, 0};
    v3f right = normalize(cross(fwd, wup));
    v3f up = normalize(cross(right, fwd));
    mm_camera_ubo& c = u->camera;
    memset(&c, 0, sizeof(c));
    float* v = c.view;  // Camera::getView: rows of the rotation = right, up, forward; then * trans
    v[0] = right.x; v[1] = up.x; v[2] = fwd.x;  v[3] = 0.f;
    v[4] = right.y; v[5] = up.y; v[6] = fwd.y;  v[7] = 0.f;
    v[8] = right.z; v[9] = up.z; v[10] = fwd.z; v[11] = 0.f;
    v[12] = -(right.x * eye[0] + right.y * eye[1] + right.z * eye[2]);
    v[13] = -(up.x * eye[0] + up.y * eye[1] + up.z * eye[2]);
    v[14] = -(fwd.x * eye[0] + fwd.y * eye[1] + fwd.z * eye[2]);
    v[15] = 1.f;
    const float aspect = (float)width / (float)height;
    const float n = 0.1f, f = 1000.0f;  // VulkanApplication.cpp:76 frustum
    const float th = tanf(kDeg2RadRef * fov_deg / 2.0f);  // glm::perspective(DEG2RAD * fov, ...)
    float* p = c.proj;
    p[0] = 1.0f / (aspect * th);
    p[5] = -(1.0f / th);  // proj[1][1] *= -1
    p[10] = -(f + n) / (f - n);
    p[11] = -1.0f;
    p[14] = -(2.0f * f * n) / (f - n);
    c.camera_position[0] = eye[0];
    c.camera_position[1] = eye[1];
    c.camera_position[2] = eye[2];
    c.camera_position[3] = 1.0f;
    c.camera_params[0] = aspect;
    c.camera_params[1] = tanf(0.5f * kDeg2RadRef * fov_deg);
    memcpy(u->camera_prev.view, c.view, sizeof(c.view));
    memcpy(u->camera_prev.proj, c.proj, sizeof(c.proj));
    memcpy(u->camera_prev.camera_position, c.camera_position, sizeof(c.camera_position));
    return MM_OK;
}

int mm_sky_from_sun_angles(float elevation_deg, float azimuth_deg, float time, int pixel_phase, mm_uniforms* u) {
    if (!u) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mm_sky_from_sun_angles: null pointer");
    if (pixel_phase < 0 || pixel_phase > 15) return mm::fail(MM_ERR_INVALID_ARGUMENT, "pixel_phase must be 0..15");
    const double d2r = 3.14159265358979323846 / 180.0;
    const double el = elevation_deg * d2r, az = azimuth_deg * d2r;
    v3f dir = {(float)(cos(el) * cos(az)), (float)sin(el), (float)(cos(el) * sin(az))};
    fill_sky(dir, time, pixel_phase, u);
    return MM_OK;
}

int mm_sky_from_reference_fractions(float elevation, float azimuth, float time, int pixel_phase, mm_uniforms* u) {
    if (!u) return mm::fail(MM_ERR_INVALID_ARGUMENT, "mm_sky_from_reference_fractions: null pointer");
    if (pixel_phase < 0 || pixel_phase > 15) return mm::fail(MM_ERR_INVALID_ARGUMENT, "pixel_phase must be 0..15");
    const float PI = 3.14159265f;  // SkyManager.cpp:6
    float theta = (float)(2.0 * PI * (elevation - 0.5));
    float phi = (float)(2.0 * PI * (azimuth - 0.5));
    v3f dir = {cosf(phi), sinf(phi) * sinf(theta), sinf(phi) * cosf(theta)};
    fill_sky(dir, time, pixel_phase, u);
    return MM_OK;
}

}  // extern "C"
