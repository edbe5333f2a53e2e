/* abi_host.c - a plain C99 host of include/mm.h (test infrastructure): the header compiles as C, the
 * std140 uniform blocks have the reference's sizes and offsets, and the host-only entry points of
 * libmm.so work from C without a device: the camera and sky fills that replace the reference's
 * uniform-buffer update, the ABI version, and the status / message of a rejected dispatch.
 * Prints "ok" and exits 0 on success. */
#include <stddef.h>
#include <stdio.h>
#include <string.h>

#include "mm.h"

_Static_assert(sizeof(mm_camera_ubo) == 160, "UniformCameraObject, std140");
_Static_assert(sizeof(mm_camera_prev_ubo) == 144, "UniformCameraObjectPrev, std140");
_Static_assert(sizeof(mm_sun_ubo) == 128, "UniformSunObject, std140");
_Static_assert(sizeof(mm_sky_ubo) == 64, "UniformSkyObject, std140");
_Static_assert(sizeof(mm_uniforms) == 496, "set 2 bindings 0-3");
_Static_assert(offsetof(mm_uniforms, sun) == 304, "sun block offset");
_Static_assert(offsetof(mm_sun_ubo, intensity) == 112, "sun.intensity offset");

static int fail(const char* what) {
    fprintf(stderr, "FAIL: %s (%s)\n", what, mm_last_error_string());
    return 1;
}

int main(void) {
    if (mm_abi_version() != 1) return fail("abi version");
    mm_uniforms u;
    memset(&u, 0, sizeof(u));
    const float eye[3] = {0.0f, 10.0f, 0.0f};
    if (mm_camera_from_angles(eye, 0.0f, 15.0f, 60.0f, 3840, 2160, &u) != MM_OK) return fail("camera");
    if (mm_sky_from_sun_angles(30.0f, 0.0f, 0.0f, 5, &u) != MM_OK) return fail("sky");
    /* camera_params = (aspect, tan(half fov)); the sun phase travels in sun.color.a */
    if (u.camera.camera_params[0] < 1.777f || u.camera.camera_params[0] > 1.778f) return fail("aspect");
    if (u.camera.camera_params[1] < 0.57f || u.camera.camera_params[1] > 0.58f) return fail("tan half fov");
    if (u.sun.color[3] != 5.0f) return fail("pixel phase");
    if (u.sun.direction[1] < 0.49f || u.sun.direction[1] > 0.51f) return fail("sun elevation");
    /* a dispatch with no context is rejected with a status and a message, nothing launched */
    if (mm_clouds_march(NULL, &u, NULL, NULL, NULL, NULL) != MM_ERR_INVALID_ARGUMENT) return fail("null context");
    if (mm_last_error_string()[0] == '\0') return fail("error message");
    printf("ok\n");
    return 0;
}
