"""Scene -> uniform blocks for the benchmark configurations (camera.cpp / SkyManager.cpp math runs in
libmm.so: mm_camera_from_angles, mm_sky_from_sun_angles)."""
import ctypes as C

from . import lib as L

# Camera 10 m above the origin, 60 degree vertical field of view; sun at 30 degrees elevation,
# azimuth 0; wind time 0 (the 256x256 CPU configuration).
DEFAULT = dict(eye=(0.0, 10.0, 0.0), yaw=0.0, pitch=15.0, fov=60.0, sun_elevation=30.0, sun_azimuth=0.0, time=0.0)


def uniforms(width, height, eye=(0.0, 10.0, 0.0), yaw=0.0, pitch=15.0, fov=60.0, sun_elevation=30.0,
             sun_azimuth=0.0, time=0.0, phase=0):
    lib = L.load()
    u = L.Uniforms()
    e = (C.c_float * 3)(*eye)
    L.check(lib.mm_camera_from_angles(e, yaw, pitch, fov, width, height, C.byref(u)), "mm_camera_from_angles")
    L.check(lib.mm_sky_from_sun_angles(sun_elevation, sun_azimuth, time, phase, C.byref(u)), "mm_sky_from_sun_angles")
    return u


def sweep_params(k, n=16):
    """Frame k of the 16-frame camera sweep: yaw 0 -> 90 deg, pitch 5 -> 25 deg, t += 0.1 s."""
    f = k / float(n - 1) if n > 1 else 0.0
    return dict(yaw=90.0 * f, pitch=5.0 + 20.0 * f, time=0.1 * k)


def sweep_uniforms(k, width, height, n=16, sun_elevation=30.0, sun_azimuth=0.0):
    p = sweep_params(k, n)
    return uniforms(width, height, yaw=p["yaw"], pitch=p["pitch"], time=p["time"], sun_elevation=sun_elevation,
                    sun_azimuth=sun_azimuth)


def cubemap_views(size=512, eye=(0.0, 10.0, 0.0), time=0.0, sun_elevation=30.0, sun_azimuth=0.0):
    """Six cube-map probe faces (+x, -x, +y, -y, +z, -z) at `size`^2 with a 90 degree field of view."""
    faces = [(0.0, 0.0), (180.0, 0.0), (0.0, 89.9), (0.0, -89.9), (90.0, 0.0), (270.0, 0.0)]
    return [(size, size, uniforms(size, size, eye=eye, yaw=y, pitch=p, fov=90.0, time=time, sun_elevation=sun_elevation,
                                  sun_azimuth=sun_azimuth)) for y, p in faces]


def batch_views(seed=0):
    """The uneven-view batch: 6 cube-map faces at 512^2, 32 cameras at random resolutions between
    640x360 and 1920x1080 and 32 cameras at 3840x2160 with random sun elevation 5-85 deg and yaw
    0-360 deg (seeded).  Returns (width, height, uniforms) triples."""
    import random
    rng = random.Random(seed)
    views = cubemap_views()
    for _ in range(32):
        w = rng.randrange(640, 1921) // 16 * 16
        h = max(360, min(1080, int(w * 9 / 16)))
        views.append((w, h, uniforms(w, h, yaw=rng.uniform(0.0, 360.0), pitch=rng.uniform(5.0, 25.0),
                                     time=rng.uniform(0.0, 2.0))))
    for _ in range(32):
        views.append((3840, 2160, uniforms(3840, 2160, yaw=rng.uniform(0.0, 360.0), pitch=rng.uniform(5.0, 25.0),
                                           time=rng.uniform(0.0, 2.0), sun_elevation=rng.uniform(5.0, 85.0))))
    return views
