// oracle_shadow.cpp - CPU restatement of the cloud-shadow march of the mesh pass,
// SkyEngine/SkyEngine/Shaders/model.frag:52-162, :221-222 and :240-276 (test infrastructure only).
//
// The mesh fragment shader marches six low-res density samples from the fragment towards the sun
// and darkens the fragment by the largest density it meets.  Its density model is a copy of
// compute-clouds.comp's with other constants, kept here as the shader has them:
//  - ATMOSPHERE_RADIUS 1e6 (:61; the sphere radius is half of it, raySphereIntersection uses 0.25),
//    earth centre y = -0.5 * 0.99 * 1e6 (:245), shell thickness 0.5 * 1e6 * 0.02 = 10 km (:247);
//  - weather coordinate 0.00001 * (proj.xz - camera.xz), low-res coordinate 0.000057 * pos (:109, :112);
//  - cloudLayerDensity's second blend goes from stratocumulus to *stratus* (:95) and cumulus, though
//    computed, is unused; cumulus fades over 0.7..1.0 (:90);
//  - heightBiasCoverage gets its arguments swapped, as in the march (:120);
//  - wind 20 * (wind.xyz + (0, 0.2 rh, 0)) * (wind.w + 200 rh) (:265);
//  - the march runs along L, the sun direction in *view* space (:221-222), from 4 * fragPositionWC
//    (:257), starting at t = the world-space intersection parameter of the quirk shared with the
//    march (isect.t = length(p_world - ro_normalized), :158), stepping 0.1 * thickness (:253);
//  - the shadow is max over the samples (:269), 1 once above 0.99 (:271-274).
// raySphereIntersection leaves isect.t unset when the sun ray misses the inner sphere (a fragment
// above the cloud floor looking away from it); t = 0 is used there, here and on the GPU.
//
// Float arithmetic in source order without contraction (built with -ffp-contract=off); float
// elementary functions from mm_math.h, so the GPU's exact variant matches this bit for bit.
#include <math.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "oracle_glsl.h"

namespace {

template <class T>
struct Shadow {
    const mm_uniforms* u;
    const oracle_textures* tex;
    T coverage_offset;
    V3<T> cam, center, L, db1, wind;
    T time, thickness, step;

    static constexpr double kRadius = 1000000.0;  // ATMOSPHERE_RADIUS (:61)

    // model.frag:65-71
    static T remap(T v, T lo0, T hi0, T lo1, T hi1) { return lo1 + (((v - lo0) / (hi0 - lo0)) * (hi1 - lo1)); }
    static T remapClamped(T v, T lo0, T hi0, T lo1, T hi1) {
        return clampT(lo1 + (((v - lo0) / (hi0 - lo0)) * (hi1 - lo1)), lo1, hi1);
    }

    // :74-76
    static V3<T> shellPoint(V3<T> pt, V3<T> c) { return (T(0.5) * T(kRadius)) * normalize(pt - c) + c; }
    // :80-82
    static T relativeHeight(V3<T> pt, V3<T> proj, T thick) { return clampT(length(pt - proj) / thick, T(0), T(1)); }

    // :87-97
    static T layerDensity(T rh, T type) {
        rh = clampT(rh, T(0), T(1));
        T cumulus = Fn<T>::max(T(0), remap(rh, T(0), T(0.2), T(0), T(1)) * remap(rh, T(0.7), T(1), T(1), T(0)));
        (void)cumulus;
        T stratocumulus = Fn<T>::max(T(0), remap(rh, T(0), T(0.2), T(0), T(1)) * remap(rh, T(0.2), T(0.7), T(1), T(0)));
        T stratus = Fn<T>::max(T(0), remap(rh, T(0), T(0.1), T(0), T(1)) * remap(rh, T(0.2), T(0.3), T(1), T(0)));
        T d1 = mixT(stratus, stratocumulus, clampT(type * T(2), T(0), T(1)));
        T d2 = mixT(stratocumulus, stratus, clampT((type - T(0.5)) * T(2), T(0), T(1)));
        return mixT(d1, d2, type);
    }

    // :99-101
    static T heightBiasCoverage(T coverage, T height) {
        return Fn<T>::pow(coverage, clampT(remap(height, T(0.7), T(0.8), T(1), T(0.6)), T(0.6), T(1)));
    }

    // :104-129
    T cloudTest(V3<T> pos, T rh) const {
        V3<T> proj = shellPoint(pos, center);
        V4<T> info = sample2d<T>(tex->weather, T(0.00001) * (proj.x - cam.x), T(0.00001) * (proj.z - cam.z));
        T layer = layerDensity(rh, info.z);
        V4<T> n = sample3d<T>(tex->low_res, T(0.000057) * pos);
        T density = layer * remapClamped(n.x, T(0.3), T(1), T(0), T(1));
        if (density < T(0.0001)) return T(0);
        T coverage = heightBiasCoverage(rh, Fn<T>::min(T(0.85), info.x + coverage_offset));
        T erosion = (T(0.625) * n.y + T(0.25) * n.z) + T(0.125) * n.w;
        erosion = remapClamped(erosion, coverage, T(1), T(0), T(1));
        return remapClamped(density, erosion, T(1), T(0), T(1));
    }

    // raySphereIntersection(ro, rd, (c, w)).t (:132-162); 0 where it leaves t unset.
    static T sphereT(V3<T> ro, V3<T> rd, V3<T> c, T w) {
        ro = ro - c;
        ro = {ro.x / w, ro.y / w, ro.z / w};
        T A = dot(rd, rd);
        T B = T(2) * dot(rd, ro);
        T C = dot(ro, ro) - T(0.25);
        T disc = B * B - T(4) * A * C;
        if (disc < T(0)) return T(0);
        T t = (-Fn<T>::sqrt(disc) - B) / A * T(0.5);
        if (t < T(0)) t = (Fn<T>::sqrt(disc) - B) / A * T(0.5);
        if (!(t >= T(0))) return T(0);
        V3<T> p = ro + rd * t;
        p = p * w;
        p = p + c;
        return length(p - ro);
    }

    void setup() {
        const float* v = u->camera.view;
        cam = {(T)u->camera.camera_position[0], (T)u->camera.camera_position[1], (T)u->camera.camera_position[2]};
        const float* b = u->sun.direction_basis + 4;  // directionBasis[1]
        db1 = {(T)b[0], (T)b[1], (T)b[2]};
        // L = normalize((camera.view * vec4(directionBasis[1], 0)).xyz), flipped below -0.05 (:221-222)
        V3<T> l = {((T)v[0] * db1.x + (T)v[4] * db1.y) + (T)v[8] * db1.z,
                   ((T)v[1] * db1.x + (T)v[5] * db1.y) + (T)v[9] * db1.z,
                   ((T)v[2] * db1.x + (T)v[6] * db1.y) + (T)v[10] * db1.z};
        L = normalize(l);
        if (L.y < T(-0.05)) L = L * T(-1);
        center = cam;
        center.y = -T(kRadius) * T(0.5) * T(0.99);  // :245
        thickness = T(0.5) * T(kRadius) * T(0.02);    // :247
        step = T(0.1) * thickness;                    // :253
        wind = {(T)u->sky.wind[0], (T)u->sky.wind[1], (T)u->sky.wind[2]};
        time = (T)u->sky.wind[3];
    }

    // :249-276 for the fragment at world position wc
    T shadow(V3<T> wc) const {
        T t = sphereT(wc, db1, center, T(kRadius));
        T accum = T(0);
        const V3<T> origin = wc * T(4);
        for (int i = 0; i < 6; ++i) {
            V3<T> pos = origin + L * t;
            V3<T> proj = shellPoint(pos, center);
            T rh = relativeHeight(pos, proj, thickness);
            V3<T> w = wind + V3<T>{T(0), T(0.2) * rh, T(0)};
            V3<T> windOffset = (T(20) * w) * (time + rh * T(200));
            T density = cloudTest(pos + windOffset, rh);
            accum = Fn<T>::max(density, accum);
            if (accum > T(0.99)) {
                accum = T(1);
                break;
            }
            t = t + step;
        }
        return accum;
    }
};

template <class T>
int run(const mm_uniforms* u, const oracle_textures* tex, const float* pos, size_t n, float coverage_offset,
        float* out, int nthreads) {
    if (!u || !tex || !pos || !out) return MM_ERR_INVALID_ARGUMENT;
    if (!tex->weather.texels || !tex->low_res.texels) return MM_ERR_INVALID_ARGUMENT;
    Shadow<T> s;
    s.u = u;
    s.tex = tex;
    s.coverage_offset = (T)coverage_offset;
    s.setup();
    auto work = [&](size_t b, size_t e) {
        for (size_t i = b; i < e; ++i) {
            const float* p = pos + 4 * i;
            out[i] = p[3] != 0.0f ? (float)s.shadow({(T)p[0], (T)p[1], (T)p[2]}) : 0.0f;
        }
    };
    if (nthreads <= 1 || n < 4096) {
        work(0, n);
        return MM_OK;
    }
    std::vector<std::thread> th;
    const size_t chunk = (n + nthreads - 1) / nthreads;
    for (int k = 0; k < nthreads; ++k) {
        size_t b = k * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back(work, b, e);
    }
    for (auto& x : th) x.join();
    return MM_OK;
}

}  // namespace

extern "C" {

int oracle_shadow_f32(const mm_uniforms* u, const oracle_textures* t, const float* world_pos, size_t n,
                      float coverage_offset, float* out_shadow, int nthreads) {
    return run<float>(u, t, world_pos, n, coverage_offset, out_shadow, nthreads);
}

int oracle_shadow_f64(const mm_uniforms* u, const oracle_textures* t, const float* world_pos, size_t n,
                      float coverage_offset, float* out_shadow, int nthreads) {
    return run<double>(u, t, world_pos, n, coverage_offset, out_shadow, nthreads);
}

}  // extern "C"
