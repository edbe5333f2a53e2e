// Driver for the reference Camera (camera.cpp): for each "ex ey ez yaw_deg pitch_deg fov_deg width
// height" line on stdin, builds Camera(pos, target, 0.1, 1000, fov) as the application does
// (VulkanApplication.cpp:76) with the target placed so that lookAt (camera.cpp:179-194) sets
// m_yaw = yaw and m_pitch = pitch, sets the aspect ratio, and prints getView(), getProj() with
// proj[1][1] negated (VulkanApplication.cpp:361-362), getAspect() and getHTanFov() as one JSON object.
#include <cmath>
#include <cstdio>

#include "camera.h"

static void arr(const char* name, const float* p, int n, bool comma) {
    printf("\"%s\": [", name);
    for (int i = 0; i < n; ++i) printf("%s%.9g", i ? ", " : "", p[i]);
    printf("]%s", comma ? ", " : "");
}

int main() {
    float ex, ey, ez, yaw, pitch, fov;
    int w, h;
    printf("[\n");
    bool first = true;
    while (scanf("%f %f %f %f %f %f %d %d", &ex, &ey, &ez, &yaw, &pitch, &fov, &w, &h) == 8) {
        const float Y = yaw * 0.017453292519943295f, P = pitch * 0.017453292519943295f;
        const glm::vec3 pos(ex, ey, ez);
        const glm::vec3 dir(std::sin(Y) * std::cos(P), std::sin(P), std::cos(Y) * std::cos(P));
        Camera cam(pos, pos + 100.0f * dir, 0.1f, 1000.0f, fov);
        cam.setAspect((float)w, (float)h);
        glm::mat4 view = cam.getView();
        glm::mat4 proj = cam.getProj();
        proj[1][1] *= -1.0f;
        const float aspect = cam.getAspect(), tanh = cam.getHTanFov();
        printf("%s{\"eye\": [%.9g, %.9g, %.9g], \"yaw\": %.9g, \"pitch\": %.9g, \"fov\": %.9g, \"width\": %d, "
               "\"height\": %d, ", first ? "" : ",\n", ex, ey, ez, yaw, pitch, fov, w, h);
        arr("view", &view[0][0], 16, true);
        arr("proj", &proj[0][0], 16, true);
        arr("aspect", &aspect, 1, true);
        arr("tan_half_fov", &tanh, 1, false);
        printf("}");
        first = false;
    }
    printf("\n]\n");
    return 0;
}
