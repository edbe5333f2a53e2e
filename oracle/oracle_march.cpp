// oracle_march.cpp - CPU restatement of the cloud raymarch compute pass (test infrastructure only).
//
// Follows SkyEngine/SkyEngine/Shaders/compute-clouds.comp line by line; each function names the
// lines it restates.  The template runs in float (T = float: the FP32 parity twin of the CUDA
// kernel and the timed CPU baseline) and in double (T = double: the yardstick for errors).
//
// Arithmetic conventions (these fix the evaluation order the GLSL source leaves to the compiler):
//  - expressions are evaluated left to right as written, no contraction into fused multiply-add
//    (built with -ffp-contract=off);
//  - dot(a, b) = (a.x*b.x + a.y*b.y) + a.z*b.z; length = sqrt(dot); normalize(v) = v * (1/length);
//  - mix(x, y, a) = x*(1-a) + y*a; clamp(x, lo, hi) = min(max(x, lo), hi) with the IEEE
//    minNum/maxNum NaN rule of GPU min/max; smoothstep per GLSL 4.50 section 8.3;
//  - mat3 * vec3 = col0*v.x + col1*v.y + col2*v.z summed left to right;
//  - float: exp/pow/acos/cos/sin are the mmx:: functions of mm_math.h (bit-reproducible on the
//    GPU); double: the C library's;
//  - samplers (Texture.cpp:29-52, 315-338: LINEAR, REPEAT, normalized coords, mip 0, UNORM8):
//    x = u*N - 0.5, i0 = floor(x), a = x - i0, texel indices wrapped modulo N, value texel/255,
//    interpolated along x, then y, then z with mix; channels a 2-channel texture lacks read
//    (.., 0, 1) as Vulkan format conversion does.  oracle_frame.filter = 1 replaces the exact
//    weights with the texture unit's fixed-point filter (oracle_glsl.h), the filter the GPU
//    applies to the same request.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <limits>
#include <thread>
#include <vector>

#include "../project-marshmallow_gb300/csrc/mm_math.h"
#include "oracle_glsl.h"

// Per-iteration event trace (built into _build/liboracle_trace.so only, -DORACLE_TRACE): one byte
// per iteration of the march loop of every traced pixel -- 1 large step without density, 2 large step
// with density (step back, :428-434), 3 small step without density, 4 small step eroded below 1e-4 by
// cloudHiRes (:437), 5 accumulated sample (sun cone, :441-466).  oracle/lane_model.py groups the
// traces into the GPU kernel's warp tiles to model lane utilization.
#ifdef ORACLE_TRACE
static uint8_t* g_trace = nullptr;
static size_t g_trace_cap = 0;
static thread_local uint8_t* t_trace = nullptr;
static thread_local size_t t_trace_n = 0;
static inline void trace_event(int e) {
    if (t_trace && t_trace_n < g_trace_cap) t_trace[t_trace_n++] = (uint8_t)e;
}
static inline void trace_pixel(size_t o) {
    t_trace = g_trace ? g_trace + o * g_trace_cap : nullptr;
    t_trace_n = 0;
}
extern "C" void oracle_trace_set(uint8_t* buf, size_t cap_per_pixel) {
    g_trace = buf;
    g_trace_cap = cap_per_pixel;
}
#else
static inline void trace_event(int) {}
static inline void trace_pixel(size_t) {}
#endif

namespace {

// ---------------------------------------------------------------------------------- the pass

struct Counters {
    uint64_t cloud_test = 0, cloud_hires = 0, iterations = 0, accumulated = 0;
};

template <class T>
struct March {
    const mm_uniforms* u;
    const oracle_textures* tex;
    T coverage_offset;
    Counters* cnt;
    int filter;  // 0: exact filter weights in T; 1: the texture unit's fixed-point filter

    // compute-clouds.comp:65-71
    static T remap(T v, T lo0, T hi0, T lo1, T hi1) { return lo1 + (((v - lo0) / (hi0 - lo0)) * (hi1 - lo1)); }
    static T remapClamped(T v, T lo0, T hi0, T lo1, T hi1) {
        return clampT(lo1 + (((v - lo0) / (hi0 - lo0)) * (hi1 - lo1)), lo1, hi1);
    }

    // compute-clouds.comp:73-77
    static T hgPhase(T cosTheta, T g) {
        T g2 = g * g;
        T inv = T(1) / Fn<T>::pow(T(1) - T(2) * g * cosTheta + g2, T(1.5));
        return T(0.07957747154594767) * ((T(1) - g2) * inv);
    }

    // compute-clouds.comp:84-86
    static T rayleighPhase(T cosTheta) { return T(0.05968310365946075) * (T(1) + cosTheta * cosTheta); }

    V3<T> v3(const float* p) const { return {(T)p[0], (T)p[1], (T)p[2]}; }

    // compute-clouds.comp:88-127
    V3<T> atmosphereColor(V3<T> dir, V3<T> sunDir) const {
        T sunE = (T)u->sun.intensity;
        V3<T> BetaR = v3(u->sky.beta_r), BetaM = v3(u->sky.beta_v);
        T zenith = Fn<T>::acos(Fn<T>::max(T(0), dir.y));
        T inverse = T(1) / (Fn<T>::cos(zenith) +
                            T(0.15) * Fn<T>::pow(T(93.885) - ((zenith * T(180)) / T(3.14159265)), T(-1.253)));
        T sR = T(8.4E3) * inverse;
        T sM = T(1.25E3) * inverse;
        V3<T> fex = exp3((-BetaR) * sR + BetaM * sM);
        T cosTheta = dot(sunDir, dir);
        T rPhase = rayleighPhase(cosTheta * T(0.5) + T(0.5));
        V3<T> betaRTheta = BetaR * rPhase;
        T mPhase = hgPhase(cosTheta, (T)u->sky.mie_directional);
        V3<T> betaMTheta = BetaM * mPhase;
        T yDot = T(1) - sunDir.y;
        yDot *= yDot * yDot * yDot * yDot;
        V3<T> betas = (betaRTheta + betaMTheta) / (BetaR + BetaM);
        V3<T> Lin = pow3(sunE * betas * (T(1) - fex), T(1.5));
        Lin = Lin * mix3(V3<T>{T(1), T(1), T(1)}, pow3(sunE * betas * fex, T(0.5)), clampT(yDot, T(0), T(1)));
        V3<T> L0 = T(0.1) * fex;
        // :119-121: the sun disk term is forced to zero; L0 += (sunE * 15000 * fex) * 0
        T sunDisk = T(0);
        L0 = L0 + ((sunE * T(15000.0)) * fex) * sunDisk;
        return (Lin + L0) * T(0.04) + V3<T>{T(0.0), T(0.0003), T(0.00075)};
    }

    // compute-clouds.comp:180-182
    static V3<T> projectedShellPoint(V3<T> pt, V3<T> center) {
        return T(0.5) * T(2000000.0) * normalize(pt - center) + center;
    }
    // compute-clouds.comp:186-188
    static T relativeHeight(V3<T> pt, V3<T> proj, T thickness) {
        return clampT(length(pt - proj) / thickness, T(0), T(1));
    }
    // compute-clouds.comp:193-204
    static T cloudLayerDensity(T rh, T cloudType) {
        rh = clampT(rh, T(0), T(1));
        T cumulus = Fn<T>::max(T(0), remap(rh, T(0), T(0.2), T(0), T(1)) * remap(rh, T(0.7), T(0.9), T(1), T(0)));
        T stratocumulus = Fn<T>::max(T(0), remap(rh, T(0), T(0.2), T(0), T(1)) * remap(rh, T(0.2), T(0.7), T(1), T(0)));
        T stratus = Fn<T>::max(T(0), remap(rh, T(0), T(0.1), T(0), T(1)) * remap(rh, T(0.2), T(0.3), T(1), T(0)));
        T d1 = mixT(stratus, stratocumulus, clampT(cloudType * T(2), T(0), T(1)));
        T d2 = mixT(stratocumulus, cumulus, clampT((cloudType - T(0.5)) * T(2), T(0), T(1)));
        return mixT(d1, d2, cloudType);
    }
    // compute-clouds.comp:206-208
    static T heightBiasCoverage(T coverage, T height) {
        return Fn<T>::pow(coverage, clampT(remap(height, T(0.7), T(0.8), T(1), T(0.8)), T(0.8), T(1)));
    }

    // compute-clouds.comp:214-228
    T cloudHiRes(V3<T> pos, T curlStrength, T origDensity, T rh) const {
        cnt->cloud_hires++;
        T c = T(0.0001);
        V4<T> cs = sample2d<T>(tex->curl, c * pos.x, c * pos.z, filter);
        V3<T> curl = {cs.x, cs.y, cs.z};
        curl = T(2) * curl - V3<T>{T(1), T(1), T(1)};
        pos = pos + T(1.9) * curlStrength * curl;
        V4<T> dn = sample3d<T>(tex->hi_res, T(0.0004) * pos, filter);
        T erosion = T(0.625) * dn.x + T(0.25) * dn.y + T(0.125) * dn.z;
        erosion = mixT(erosion, T(1) - erosion, clampT(rh * T(10), T(0), T(1)));
        return remapClamped(origDensity, T(1) * erosion, T(1), T(0), T(1));
    }

    // compute-clouds.comp:231-253 (the coverage out-parameter is unused by every caller)
    T cloudTest(V3<T> pos, T rh, V3<T> center) const {
        cnt->cloud_test++;
        V3<T> proj = projectedShellPoint(pos, center);
        V3<T> cam = v3(u->camera.camera_position);
        V4<T> info = sample2d<T>(tex->weather, T(0.000009) * (proj.x - cam.x), T(0.000009) * (proj.z - cam.z), filter);
        T layer = cloudLayerDensity(rh, info.z);
        V4<T> dn = sample3d<T>(tex->low_res, T(0.00002) * pos, filter);
        T density = layer * remapClamped(dn.x, T(0.3), T(1), T(0), T(1));
        if (density < T(0.0001)) return T(0);
        T coverage = heightBiasCoverage(rh, Fn<T>::min(T(0.85), info.x + coverage_offset));
        T erosion = T(0.625) * dn.y + T(0.25) * dn.z + T(0.125) * dn.w;
        erosion = remapClamped(erosion, coverage, T(1), T(0), T(1));
        density = remapClamped(density, erosion, T(1), T(0), T(1));
        return density;
    }

    struct Isect {
        bool valid;
        T t;
    };
    // compute-clouds.comp:147-177; the returned t is length(p_world - ro_scaled) (:173), as the
    // shader computes it.  A miss leaves t at 0.
    static Isect raySphere(V3<T> ro, V3<T> rd, V3<T> c, T w) {
        Isect is{false, T(0)};
        ro = ro - c;
        ro = ro / V3<T>{w, w, w};
        T A = dot(rd, rd);
        T B = T(2) * dot(rd, ro);
        T C = dot(ro, ro) - T(0.25);
        T disc = B * B - T(4) * A * C;
        if (disc < T(0)) return is;
        T t = (-Fn<T>::sqrt(disc) - B) / A * T(0.5);
        if (t < T(0)) t = (Fn<T>::sqrt(disc) - B) / A * T(0.5);
        if (t >= T(0)) {
            is.valid = true;
            V3<T> p = ro + rd * t;
            p = p * w;
            p = p + c;
            is.t = length(p - ro);
        }
        return is;
    }

    // compute-clouds.comp:256-277
    static M3<T> fromAngleAxis(V3<T> a, T rad) {
        T c = Fn<T>::cos(rad), s = Fn<T>::sin(rad);
        M3<T> r;
        r.c[0] = {c + a.x * a.x * (T(1) - c), a.y * a.x * (T(1) - c) + a.z * s, a.z * a.x * (T(1) - c) - a.y * s};
        r.c[1] = {a.x * a.y * (T(1) - c) - a.z * s, c + a.y * a.y * (T(1) - c), a.z * a.y * (T(1) - c) + a.x * s};
        r.c[2] = {a.x * a.z * (T(1) - c) + a.y * s, a.y * a.z * (T(1) - c) - a.x * s, c + a.z * a.z * (T(1) - c)};
        return r;
    }

    // compute-clouds.comp:288-500 for one pixel
    void pixel(int px, int py, float uv_w, float uv_h, float* rgba, float* depth) const {
        const T timeOffset = (T)u->sky.wind[3];
        V3<T> wind = v3(u->sky.wind);
        const float* view = u->camera.view;
        T uvx = (T)px / (T)uv_w, uvy = (T)py / (T)uv_h;
        T spx = uvx * T(2) - T(1), spy = uvy * T(2) - T(1);
        V3<T> camLook = {(T)view[0 * 4 + 2], (T)view[1 * 4 + 2], (T)view[2 * 4 + 2]};
        V3<T> camRight = {(T)view[0 * 4 + 0], (T)view[1 * 4 + 0], (T)view[2 * 4 + 0]};
        V3<T> camUp = {(T)view[0 * 4 + 1], (T)view[1 * 4 + 1], (T)view[2 * 4 + 1]};
        const V3<T> cameraPos = v3(u->camera.camera_position);
        V3<T> refPoint = cameraPos - camLook;
        T cpx = (T)u->camera.camera_params[0], cpy = (T)u->camera.camera_params[1];
        V3<T> p = refPoint + cpx * spx * cpy * camRight - spy * cpy * camUp;
        V3<T> rd = normalize(p - cameraPos);

        V3<T> sunDir = normalize(v3(u->sun.direction_basis + 4));
        const T sunY = (T)u->sun.direction[1];
        T dotToSun = Fn<T>::max(T(0), dot(sunDir, rd));
        T skyAmbient = dotToSun * T(0.18);
        skyAmbient *= skyAmbient * skyAmbient;
        const T SUN_ANGULAR_COS = T(0.999956676946448443553574619906976478926848692873900859324);
        T sunDisk = smoothstepT(SUN_ANGULAR_COS, SUN_ANGULAR_COS + T(0.00003), dotToSun);
        dotToSun *= dotToSun * dotToSun * dotToSun;
        dotToSun *= dotToSun * dotToSun * dotToSun;
        dotToSun *= dotToSun * dotToSun * dotToSun;
        dotToSun *= dotToSun * dotToSun * dotToSun;
        dotToSun *= dotToSun * dotToSun;
        if (sunY < T(0)) dotToSun *= dotToSun * dotToSun * dotToSun * dotToSun * dotToSun * dotToSun;
        sunDisk = Fn<T>::max(sunDisk, dotToSun);
        sunDisk = Fn<T>::max(T(0), sunDisk);

        V4<T> fc = {T(0), T(0), T(0), T(0)};
        V3<T> bg = {T(0), T(0), T(0)};
        if (sunY >= T(0)) {
            bg = atmosphereColor(rd, sunDir);
            fc.w = Fn<T>::max(skyAmbient, sunDisk);
            fc.x = bg.x;
            fc.y = bg.y;
            fc.z = bg.z;
        }
        if (dot(rd, V3<T>{T(0), T(1), T(0)}) < T(0)) {
            store(fc, std::numeric_limits<float>::infinity(), rgba, depth);
            return;
        }

        V3<T> earthCenter = cameraPos;
        earthCenter.y = -T(2000000.0) * T(0.5) * T(0.995);
        const T R = T(2000000.0);
        T thickness = T(0.5) * R * T(0.02);
        Isect inner = raySphere(cameraPos, rd, earthCenter, R);
        Isect outer = raySphere(cameraPos, rd, earthCenter, R * T(1.02));

        if (sunY < T(0)) {  // :365-384
            M3<T> rot = fromAngleAxis(normalize(V3<T>{T(1), T(0), T(1)}), sunY * T(0.5));
            V3<T> rrd = mul(rot, rd), rro = mul(rot, cameraPos);
            V3<T> point = outer.t * rrd + rro;
            V3<T> pp = projectedShellPoint(point, earthCenter);
            V4<T> ns = sample2d<T>(tex->night_sky, T(0.00002) * (pp.x - cameraPos.x) + T(0.35),
                                   T(0.00002) * (pp.z - cameraPos.z) + T(0.35), filter);
            bg = {ns.x, ns.y, ns.z};
            bg = bg * (V3<T>{Fn<T>::sqrt(bg.x), Fn<T>::sqrt(bg.y), Fn<T>::sqrt(bg.z)} * T(0.75));
            bg = pow3(bg, T(2.2));
            bg = bg * T(10);
            T falloff = Fn<T>::pow(rd.y, T(6));
            bg = bg * falloff;
            bg = mix3(V3<T>{T(0.3), T(0.6), T(4.0)} * T(0.05), bg, Fn<T>::pow(rd.y, T(0.03125)));
            bg = bg + sunDisk;
            fc.w = sunDisk;
        }

        T cosTheta = dot(rd, sunDir);
        T accum = T(0), transmittance = T(1);
        T stepSize = T(0.05) * thickness;
        M3<T> basis;
        basis.c[0] = v3(u->sun.direction_basis + 0);
        basis.c[1] = v3(u->sun.direction_basis + 4);
        basis.c[2] = v3(u->sun.direction_basis + 8);
        const V3<T> samples[6] = {
            mul(basis, V3<T>{T(0), T(0.6), T(0)}),   mul(basis, V3<T>{T(0), T(0.5), T(0.05)}),
            mul(basis, V3<T>{T(0.1), T(0.75), T(0)}), mul(basis, V3<T>{T(0.2), T(2.5), T(0.3)}),
            mul(basis, V3<T>{T(0), T(6), T(0)}),     mul(basis, V3<T>{T(-0.1), T(1), T(-0.2)}),
        };
        bool noHits = true;
        int misses = 0, steps = 0;
        float firstT = std::numeric_limits<float>::infinity();
        const T hg = Fn<T>::max(hgPhase(cosTheta, T(0.6)), T(0.7) * hgPhase(cosTheta, T(0.99) - T(0.1)));
        const V3<T> windScale = {T(0.1), T(0.05), T(0)};

        // :408-482.  The shader's loop ends by t >= outer.t, accumulated density or MAX_STEPS counted
        // steps; the iteration cap below (never reached by a ray that starts inside the shells) bounds
        // rays whose uncounted iterations could otherwise run long on degenerate uniforms.
        int iterations = 0;
        for (T t = inner.t; t < outer.t && iterations < 8192; t += stepSize, ++iterations) {
            cnt->iterations++;
            V3<T> pos = cameraPos + t * rd;
            V3<T> proj = projectedShellPoint(pos, earthCenter);
            T rh = relativeHeight(pos, proj, thickness);
            V3<T> windOffset = (T(20) * (wind + rh * windScale)) * (timeOffset + rh * T(200));
            T density = cloudTest(pos + windOffset, rh, earthCenter);
            T loDensity = density;
            if (density > T(0)) {
                misses = 0;
                if (noHits) {
                    t -= stepSize;
                    stepSize *= T(0.3);
                    noHits = false;
                    trace_event(2);
                    continue;
                }
                density = cloudHiRes(pos + windOffset, stepSize, density, rh);
                if (density < T(0.0001)) {
                    trace_event(4);
                    continue;
                }
                T densityAlongLight = T(0);
                for (int i = 0; i < 6; i++) {
                    V3<T> lsPos = pos + T(3) * stepSize * samples[i];
                    V3<T> lsProj = projectedShellPoint(lsPos, earthCenter);
                    T lsHeight = relativeHeight(lsPos, lsProj, thickness);
                    windOffset = (T(20) * (wind + lsHeight * windScale)) * (timeOffset + lsHeight * T(200));
                    T lsDensity = cloudTest(lsPos + windOffset, lsHeight, earthCenter);
                    if (lsDensity > T(0)) {
                        lsDensity = cloudHiRes(lsPos + windOffset, stepSize, lsDensity, lsHeight);
                        densityAlongLight += lsDensity;
                    }
                }
                T beers = Fn<T>::exp(-densityAlongLight);
                T beersMod = Fn<T>::max(beers, T(0.7) * Fn<T>::exp(T(-0.25) * densityAlongLight));
                beers = mixT(beers, beersMod, -cosTheta * T(0.5) + T(0.5));
                T inScatter = T(0.09) + Fn<T>::pow(loDensity, remapClamped(rh, T(0.3), T(0.85), T(0.5), T(2)));
                inScatter *= Fn<T>::pow(remapClamped(rh, T(0.07), T(0.34), T(0.1), T(1)), T(0.8));
                transmittance = mixT(transmittance, inScatter * hg * beers, T(1) - accum);
                cnt->accumulated++;
                if (firstT == std::numeric_limits<float>::infinity()) firstT = (float)t;
                accum += density;
                trace_event(5);
            } else if (trace_event(noHits ? 1 : 3), !noHits) {
                misses++;
                if (misses >= 10) {
                    noHits = true;
                    stepSize /= T(0.3);
                }
            }
            if (accum > T(0.99)) {
                accum = T(1);
                break;
            }
            if (++steps > 100) break;
        }

        accum *= smoothstepT(T(0), T(1), Fn<T>::min(T(1), remap(rd.y, T(0), T(0.1), T(0), T(1))));
        accum = Fn<T>::min(accum, T(0.999));
        V3<T> sunColor = v3(u->sun.color);
        T I = (T)u->sun.intensity;
        T et = Fn<T>::exp(-transmittance);
        V3<T> cloud;
        if (sunY >= T(0)) {
            T a = I * Fn<T>::max(T(0), transmittance);
            cloud = sunColor * (V3<T>{a, a, a} + (T(0.08) * bg) * et);
        } else {
            T a = I * Fn<T>::max(T(0), transmittance);
            V3<T> night = V3<T>{T(0.3), T(0.6), T(4.0)} * T(0.05) * Fn<T>::pow(rd.y, T(0.03125));
            cloud = sunColor * (V3<T>{a, a, a} + (T(0.08) * night) * et);
        }
        V3<T> rgb = mix3(bg, cloud, accum);
        fc.x = rgb.x;
        fc.y = rgb.y;
        fc.z = rgb.z;
        fc.w *= Fn<T>::max(T(1) - accum, T(0));
        store(fc, firstT, rgba, depth);
    }

    static void store(V4<T> c, float d, float* rgba, float* depth) {
        rgba[0] = (float)c.x;
        rgba[1] = (float)c.y;
        rgba[2] = (float)c.z;
        rgba[3] = (float)c.w;
        if (depth) *depth = d;
    }
};

template <class T>
int run(const mm_uniforms* u, const oracle_textures* t, const oracle_frame* f, float* out_rgba,
        float* out_depth, uint64_t* counters, int nthreads) {
    if (!u || !t || !f || !out_rgba) return MM_ERR_INVALID_ARGUMENT;
    if (f->width <= 0 || f->height <= 0 || f->row_step <= 0 || f->col_step <= 0) return MM_ERR_INVALID_ARGUMENT;
    const oracle_texture* req[4] = {&t->weather, &t->curl, &t->low_res, &t->hi_res};
    for (auto r : req)
        if (!r->texels || r->width <= 0 || r->height <= 0 || r->depth <= 0) return MM_ERR_INVALID_ARGUMENT;
    if (u->sun.direction[1] < 0.f && !t->night_sky.texels) return MM_ERR_INVALID_ARGUMENT;
    const int rows = f->row_end > f->row_begin ? (f->row_end - f->row_begin + f->row_step - 1) / f->row_step : 0;
    const int cols = f->width > f->col_begin ? (f->width - f->col_begin + f->col_step - 1) / f->col_step : 0;
    if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
    const float uv_w = f->ref_uv_1080p ? 1920.f : (float)f->width;
    const float uv_h = f->ref_uv_1080p ? 1080.f : (float)f->height;
    const int phase = (int)u->sun.color[3];
    std::vector<Counters> per(nthreads);
    std::atomic<int> next(0);
    auto worker = [&](int tid) {
        March<T> m{u, t, (T)f->coverage_offset, &per[tid], f->filter};
        for (int r = next++; r < rows; r = next++) {
            int py = f->row_begin + r * f->row_step;
            for (int c = 0; c < cols; ++c) {
                int px = f->col_begin + c * f->col_step;
                if (f->pixel_mode == MM_PIXELS_PHASE16 && ((px & 3) != (phase % 4) || (py & 3) != (phase / 4)))
                    continue;
                size_t o = (size_t)r * cols + c;
                trace_pixel(o);
                m.pixel(px, py, uv_w, uv_h, out_rgba + 4 * o, out_depth ? out_depth + o : nullptr);
            }
        }
    };
    std::vector<std::thread> pool;
    for (int i = 0; i < nthreads; ++i) pool.emplace_back(worker, i);
    for (auto& th : pool) th.join();
    if (counters) {
        Counters s;
        for (auto& c : per) {
            s.cloud_test += c.cloud_test;
            s.cloud_hires += c.cloud_hires;
            s.iterations += c.iterations;
            s.accumulated += c.accumulated;
        }
        counters[0] = s.cloud_test;
        counters[1] = s.cloud_hires;
        counters[2] = s.iterations;
        counters[3] = s.accumulated;
    }
    return MM_OK;
}

}  // namespace

extern "C" {

int oracle_march_f32(const mm_uniforms* u, const oracle_textures* t, const oracle_frame* f,
                     float* out_rgba, float* out_depth, uint64_t* counters, int nthreads) {
    return run<float>(u, t, f, out_rgba, out_depth, counters, nthreads);
}

int oracle_march_f64(const mm_uniforms* u, const oracle_textures* t, const oracle_frame* f,
                     float* out_rgba, float* out_depth, uint64_t* counters, int nthreads) {
    return run<double>(u, t, f, out_rgba, out_depth, counters, nthreads);
}

int oracle_sample(const oracle_texture* t, int dims, const float* coords, size_t n, int filter, float* out) {
    if (!t || !t->texels || !coords || !out || (dims != 2 && dims != 3)) return MM_ERR_INVALID_ARGUMENT;
    for (size_t i = 0; i < n; ++i) {
        V4<float> v;
        if (dims == 2)
            v = sample2d<float>(*t, coords[2 * i], coords[2 * i + 1], filter);
        else
            v = sample3d<float>(*t, V3<float>{coords[3 * i], coords[3 * i + 1], coords[3 * i + 2]}, filter);
        out[4 * i] = v.x;
        out[4 * i + 1] = v.y;
        out[4 * i + 2] = v.z;
        out[4 * i + 3] = v.w;
    }
    return MM_OK;
}

// tonemap.frag:11-22 with the constants of :27-28 (exposure 0.7, white 50.2, gamma 1/2.2).
void oracle_tonemap(const float* rgba, size_t n, float* out) {
    auto uc2 = [](double x) {
        return ((x * (0.15 * x + 0.1 * 0.5) + 0.2 * 0.02) / (x * (0.15 * x + 0.5) + 0.2 * 0.3)) - 0.02 / 0.3;
    };
    const double white = 1.0 / uc2(50.2);
    for (size_t i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            double v = uc2(0.7 * (double)rgba[4 * i + c]) * white;
            out[3 * i + c] = (float)pow(v > 0 ? v : 0.0, 1.0 / 2.2);
        }
}

}  // extern "C"
