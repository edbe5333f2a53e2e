// ref_uniforms.h - fills the uniform blocks of a reference shader compiled by glsl_to_cpp.py from
// an mm_uniforms block (test infrastructure).  Included after the generated translation unit, whose
// globals `camera`, `cameraPrev`, `sun` and `sky` are the four blocks of descriptor set 2 that the
// cloud and reprojection shaders declare identically.
#pragma once

// the shim's GLSL keywords end with the shader
#undef main
#undef layout
#undef uniform
#undef readonly
#undef writeonly
#undef highp
#undef in
#undef inout
#undef out
#undef pow
#undef exp
#undef acos
#undef cos
#undef sin

#include <atomic>
#include <cstring>
#include <thread>
#include <vector>

#include "../oracle.h"

namespace refshader {

inline mat4 to_mat4(const float* m) {  // std140 column-major, as glm stores it
    mat4 r;
    std::memcpy(&r[0][0], m, 16 * sizeof(float));
    return r;
}

inline vec4 to_vec4(const float* v) { return vec4(v[0], v[1], v[2], v[3]); }

template <class Cam, class CamPrev, class Sun, class Sky>
inline void load_blocks(const mm_uniforms* u, Cam& camera, CamPrev& cameraPrev, Sun& sun, Sky& sky) {
    camera.view = to_mat4(u->camera.view);
    camera.proj = to_mat4(u->camera.proj);
    camera.cameraPosition = to_vec4(u->camera.camera_position);
    camera.cameraParams = to_vec4(u->camera.camera_params);
    cameraPrev.view = to_mat4(u->camera_prev.view);
    cameraPrev.proj = to_mat4(u->camera_prev.proj);
    cameraPrev.cameraPosition = to_vec4(u->camera_prev.camera_position);
    sun.location = to_vec4(u->sun.location);
    sun.direction = to_vec4(u->sun.direction);
    sun.color = to_vec4(u->sun.color);
    sun.directionBasis = to_mat4(u->sun.direction_basis);
    sun.intensity = u->sun.intensity;
    sky.betaR = to_vec4(u->sky.beta_r);
    sky.betaV = to_vec4(u->sky.beta_v);
    sky.wind = to_vec4(u->sky.wind);
    sky.mie_directional = u->sky.mie_directional;
}

// Runs body(i) for i in [0, n) on nthreads host threads (0: all cores).
template <class F>
inline void parallel_for(size_t n, int nthreads, F body) {
    if (nthreads <= 0) nthreads = (int)std::thread::hardware_concurrency();
    if (nthreads <= 0) nthreads = 1;
    std::atomic<size_t> next{0};
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < n;) body(i);
    };
    std::vector<std::thread> pool;
    for (int k = 1; k < nthreads; ++k) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
}

}  // namespace refshader
