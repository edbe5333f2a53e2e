// Driver for the reference SkyManager (SkyManager.cpp): for each "elevation azimuth time" triple
// on stdin, prints one JSON object with the UniformSunObject and UniformSkyObject floats after
// rebuildSkyFromNewSun(elevation, azimuth) and setTime(time) (VulkanApplication.cpp:374-376).
#include <cstdio>
#include "SkyManager.h"

static void arr(const char* name, const float* p, int n, bool comma) {
    printf("\"%s\": [", name);
    for (int i = 0; i < n; ++i) printf("%s%.9g", i ? ", " : "", p[i]);
    printf("]%s", comma ? ", " : "");
}

int main() {
    float e, a, t;
    SkyManager sm;
    printf("[\n");
    bool first = true;
    while (scanf("%f %f %f", &e, &a, &t) == 3) {
        sm.rebuildSkyFromNewSun(e, a);
        sm.setTime(t);
        UniformSunObject& sun = sm.getSun();
        UniformSkyObject sky = sm.getSky();
        printf("%s{\"elevation\": %.9g, \"azimuth\": %.9g, \"time\": %.9g, ", first ? "" : ",\n", e, a, t);
        arr("location", &sun.location[0], 4, true);
        arr("direction", &sun.direction[0], 4, true);
        arr("color_rgb", &sun.color[0], 3, true);
        arr("direction_basis", &sun.directionBasis[0][0], 16, true);
        arr("intensity", &sun.intensity, 1, true);
        arr("beta_r", &sky.betaR[0], 4, true);
        arr("wind", &sky.wind[0], 4, true);
        arr("mie_directional", &sky.mie_directional, 1, false);
        printf("}");
        first = false;
    }
    printf("\n]\n");
    return 0;
}
