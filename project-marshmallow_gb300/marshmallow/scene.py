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
