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


def _camera_rays(u, width, height):
    """Unit ray directions of every pixel, (height, width, 3) float64, as the march forms them
    (compute-clouds.comp:309-322): p = (cam - look) + aspect * sx * tanHalfFov * right
    - sy * tanHalfFov * up, rd = normalize(p - cam), sx, sy = 2 * pixel / size - 1."""
    import numpy as np
    v = np.array(u.camera.view[:], np.float64)
    look, right, up = v[[2, 6, 10]], v[[0, 4, 8]], v[[1, 5, 9]]
    aspect, tan = float(u.camera.camera_params[0]), float(u.camera.camera_params[1])
    sx = 2.0 * np.arange(width, dtype=np.float64) / width - 1.0
    sy = 2.0 * np.arange(height, dtype=np.float64) / height - 1.0
    d = (-look)[None, None, :] + (aspect * tan) * sx[None, :, None] * right - tan * sy[:, None, None] * up
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def terrain_height(x, z, amplitude=40.0):
    import numpy as np
    return amplitude * (0.6 * np.sin(x / 310.0) * np.cos(z / 260.0) + 0.4 * np.sin((x + 2.0 * z) / 95.0))


def terrain_gbuffer(u, width, height, amplitude=40.0, coarse_steps=48, refine_steps=30):
    """A headless G-buffer for the mesh pass: the world position (model.vert's fragPositionWC) where
    each pixel's camera ray first meets the height field y = terrain_height(x, z), as float4 rows
    (height, width, 4) float32 with w = 1 where the ray hits the ground and 0 where it does not.
    The first crossing is found by a coarse march between the planes y = +-amplitude and refined by
    bisection."""
    import numpy as np
    rd = _camera_rays(u, width, height).reshape(-1, 3)
    eye = np.array(u.camera.camera_position[:3], np.float64)
    out = np.zeros((rd.shape[0], 4), np.float32)
    down = rd[:, 1] < -1e-6
    r = rd[down]
    t0 = np.maximum(0.0, (eye[1] - amplitude) / -r[:, 1])
    t1 = (eye[1] + amplitude) / -r[:, 1]

    def g(t):
        p = eye[None, :] + t[:, None] * r
        return p[:, 1] - terrain_height(p[:, 0], p[:, 2], amplitude)

    lo, hi = t0.copy(), t1.copy()
    found = np.zeros(len(r), bool)
    prev_t, prev_g = t0, g(t0)
    for k in range(1, coarse_steps + 1):
        t = t0 + (t1 - t0) * (k / coarse_steps)
        gt = g(t)
        hit = (~found) & (prev_g > 0) & (gt <= 0)
        lo[hit], hi[hit] = prev_t[hit], t[hit]
        found |= hit
        prev_t, prev_g = t, gt
    found &= g(t0) > 0
    for _ in range(refine_steps):
        mid = 0.5 * (lo + hi)
        above = g(mid) > 0
        lo = np.where(above, mid, lo)
        hi = np.where(above, hi, mid)
    p = eye[None, :] + hi[:, None] * r
    sel = np.flatnonzero(down)[found]
    out[sel, :3] = p[found]
    out[sel, 3] = 1.0
    return out.reshape(height, width, 4)


def terrain_gbuffer_cuda(u, width, height, amplitude=40.0, coarse_steps=48, refine_steps=30):
    """terrain_gbuffer computed on the current CUDA device with torch (float64): returns an
    (height, width, 4) float32 CUDA tensor.  Used to build large G-buffers quickly."""
    import torch
    dev = torch.device("cuda")
    f64 = torch.float64
    v = torch.tensor(list(u.camera.view), dtype=f64, device=dev)
    look, right, up = v[[2, 6, 10]], v[[0, 4, 8]], v[[1, 5, 9]]
    aspect, tan = float(u.camera.camera_params[0]), float(u.camera.camera_params[1])
    sx = 2.0 * torch.arange(width, dtype=f64, device=dev) / width - 1.0
    sy = 2.0 * torch.arange(height, dtype=f64, device=dev) / height - 1.0
    d = (-look)[None, None, :] + (aspect * tan) * sx[None, :, None] * right - tan * sy[:, None, None] * up
    rd = (d / torch.linalg.norm(d, dim=-1, keepdim=True)).reshape(-1, 3)
    eye = torch.tensor(list(u.camera.camera_position[:3]), dtype=f64, device=dev)
    out = torch.zeros((rd.shape[0], 4), dtype=torch.float32, device=dev)
    down = rd[:, 1] < -1e-6
    r = rd[down]
    t0 = torch.clamp((eye[1] - amplitude) / -r[:, 1], min=0.0)
    t1 = (eye[1] + amplitude) / -r[:, 1]

    def height_at(x, z):
        return amplitude * (0.6 * torch.sin(x / 310.0) * torch.cos(z / 260.0) + 0.4 * torch.sin((x + 2.0 * z) / 95.0))

    def g(t):
        p = eye[None, :] + t[:, None] * r
        return p[:, 1] - height_at(p[:, 0], p[:, 2])

    lo, hi = t0.clone(), t1.clone()
    found = torch.zeros(len(r), dtype=torch.bool, device=dev)
    prev_t, prev_g = t0, g(t0)
    for k in range(1, coarse_steps + 1):
        t = t0 + (t1 - t0) * (k / coarse_steps)
        gt = g(t)
        hit = (~found) & (prev_g > 0) & (gt <= 0)
        lo = torch.where(hit, prev_t, lo)
        hi = torch.where(hit, t, hi)
        found |= hit
        prev_t, prev_g = t, gt
    found &= g(t0) > 0
    for _ in range(refine_steps):
        mid = 0.5 * (lo + hi)
        above = g(mid) > 0
        lo = torch.where(above, mid, lo)
        hi = torch.where(above, hi, mid)
    p = eye[None, :] + hi[:, None] * r
    sel = torch.nonzero(down).squeeze(1)[found]
    out[sel, :3] = p[found].float()
    out[sel, 3] = 1.0
    return out.reshape(height, width, 4)
