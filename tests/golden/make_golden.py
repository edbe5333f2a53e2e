"""Regenerates the committed golden fixtures from the reference tree (development machine only).

  curl_fbm_128.rgba   Textures/CurlNoiseFBM.tga decoded to 128x128 RGBA8 (rows top to bottom),
                      checked equal to the output of the reference's own GenerateCurlNoise
                      (ImageUtils.cpp compiled by `make -C oracle ref`).
  ref_hash.txt        hashNoise(x, y, z) of ImageUtils.cpp:25 for a set of lattice points, from the
                      compiled reference.
  sky_reference.json  UniformSunObject / UniformSkyObject after SkyManager::rebuildSkyFromNewSun and
                      setTime (SkyManager.cpp, compiled by `make -C oracle ref`).
  nubis_stats.json    mean / deviation of the shipped Nubis density textures (the targets of the
                      seeded generators' output maps).
  camera_reference.json  view/projection/aspect/tanHalfFov of the reference Camera (camera.cpp,
                      compiled by `make -C oracle ref` with forwarding headers for its Windows-style
                      includes) for a set of poses, frusta and image sizes.
  shader_clouds_1080p.npz  the reference's own compute-clouds.comp, compiled unchanged as C++ on the
                      CPU (`make -C oracle ref`: oracle/ref/glsl_to_cpp.py + glsl_shim.h), on the
                      seed-0 generator textures: for five frames (sweep poses, a low sun, a night sky;
                      pixel phases 0, 5, 10, 15, 3) the rgba of every 32nd pixel of the phase in x and y
                      of its hard-coded 1920x1080 frame, with the uniform blocks that made them.
  shader_clouds_mm.json  the same five frames from the shader built with mm_math.h's exp, pow, acos,
                      cos and sin (the restatement's elementary functions): SHA-256 of the rgba of every
                      8th pixel of the phase in x and y, which the FP32 restatement and the GPU's exact
                      kernel reproduce bit for bit.
  shader_passes.npz   the reference's reproject.comp, model.frag, god-ray.frag, radialBlur.frag and
                      tonemap.frag compiled the same way: SHA-256 of the reprojected images of three
                      camera motions (tests/shader_golden.py REPROJECT_CASES, seeded hash images);
                      the god-ray alpha, radial-blur rgb and tonemap rgb (8 bits) of a 64x36 frame;
                      the cloud shadow of a 48x27 terrain G-buffer (positions stored with it).
  asset_digests.json  SHA-256 of the RGBA8 decode (stbi_load(..., STBI_rgb_alpha) conventions) of the
                      shipped textures the reference loads, from the independent decoders in
                      tests/tga.py and tests/png.py; the library's loader must reproduce them.

Usage: python tests/golden/make_golden.py [REFERENCE_ROOT] [--digests-only | --shader-only]

"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))
from png import read_png  # noqa: E402
from tga import read_tga  # noqa: E402

# Files VulkanApplication.cpp:253-262 loads (plus the TGA twin of the curl map), relative to Textures/.
ASSETS = ["CloudPlacement.png", "NightSky/nightSky_noOrange.png", "CurlNoiseFBM.png", "CurlNoiseFBM.tga",
          "3DTextures/lowResCloudShape/lowResCloud(0).tga", "3DTextures/lowResCloudShape/lowResCloud(77).tga",
          "3DTextures/hiResCloudShape/hiResClouds (0).tga", "3DTextures/hiResCloudShape/hiResClouds (31).tga"]


def rgba8(a, depth16=False):
    """stbi_load(..., STBI_rgb_alpha) conversion of decoded samples (h, w, c)."""
    if depth16:
        a = a >> 8
    a = a.astype(np.uint8)
    h, w, c = a.shape
    out = np.full((h, w, 4), 255, np.uint8)
    if c <= 2:
        out[..., :3] = a[..., :1]
        if c == 2:
            out[..., 3] = a[..., 1]
    else:
        out[..., :c] = a
    return out


def asset_digests(se):
    import hashlib
    d = {}
    for name in ASSETS:
        path = os.path.join(se, "Textures", name)
        if name.endswith(".png"):
            a = read_png(path)
            img = rgba8(a, a.dtype == np.uint16)
        else:
            img = rgba8(read_tga(path))
        d[name] = hashlib.sha256(img.tobytes()).hexdigest()
    with open(os.path.join(HERE, "asset_digests.json"), "w") as f:
        json.dump(d, f, indent=1)


SHADER_STRIDE = 32
SHADER_MM_STRIDE = 8


def shader_frames():
    """(name, uniforms, night-sky texels or None) of the compute-clouds.comp golden frames."""
    sys.path.insert(0, os.path.join(REPO, "project-marshmallow_gb300"))
    sys.path.insert(0, REPO)
    import marshmallow as mm
    import marshmallow.lib as L
    import oracle
    night = oracle.noise(L.NOISE_WEATHER, 3, 160, 90, 1, 4)[0]
    frames = [("sweep0", mm.scene.sweep_uniforms(0, 1920, 1080), 0),
              ("sweep7", mm.scene.sweep_uniforms(7, 1920, 1080), 5),
              ("sweep12", mm.scene.sweep_uniforms(12, 1920, 1080), 10),
              ("low_sun", mm.scene.uniforms(1920, 1080, yaw=120.0, pitch=4.0, sun_elevation=3.0, time=40.0), 15),
              ("night", mm.scene.uniforms(1920, 1080, yaw=300.0, pitch=9.0, sun_elevation=-12.0), 3)]
    out = []
    for name, u, phase in frames:
        u.sun.color[3] = float(phase)
        out.append((name, u, night if u.sun.direction[1] < 0 else None))
    return out


def shader_pixels(phase, stride=SHADER_STRIDE):
    """Row and column lists of the golden pixels of a phase: every stride-th pixel of the phase."""
    return np.arange(phase // 4, 1080, stride), np.arange(phase % 4, 1920, stride)


def shader_clouds_golden():
    import ctypes as C
    sys.path.insert(0, os.path.join(REPO, "project-marshmallow_gb300"))
    sys.path.insert(0, REPO)
    import oracle
    import marshmallow.lib as L
    tex = {"low_res": oracle.noise(L.NOISE_LOWRES, 0, 128, 128, 128, 4),
           "hi_res": oracle.noise(L.NOISE_HIRES, 0, 32, 32, 32, 4),
           "curl": oracle.noise(L.NOISE_CURL2D, 0, 128, 128, 1, 2)[0],
           "weather": oracle.noise(L.NOISE_WEATHER, 0, 512, 512, 1, 4)[0]}
    names, ublocks, images = [], [], []
    for name, u, night in shader_frames():
        t = dict(tex, night_sky=night)
        rows, cols = shader_pixels(int(u.sun.color[3]))
        ys, xs = np.meshgrid(rows, cols, indexing="ij")
        rgba = oracle.ref_clouds_march(u, t, xs.ravel(), ys.ravel()).reshape(len(rows), len(cols), 4)
        names.append(name)
        ublocks.append(np.frombuffer(C.string_at(C.addressof(u), C.sizeof(u)), np.uint8))
        images.append(rgba)
    np.savez_compressed(os.path.join(HERE, "shader_clouds_1080p.npz"), names=np.array(names),
                        uniforms=np.stack(ublocks), rgba=np.stack(images), stride=SHADER_STRIDE)

    import hashlib
    mm_frames = []
    for name, u, night in shader_frames():
        t = dict(tex, night_sky=night)
        rows, cols = shader_pixels(int(u.sun.color[3]), SHADER_MM_STRIDE)
        ys, xs = np.meshgrid(rows, cols, indexing="ij")
        rgba = oracle.ref_clouds_march(u, t, xs.ravel(), ys.ravel(), mm_math=True).reshape(len(rows), len(cols), 4)
        mm_frames.append({"name": name, "uniforms": C.string_at(C.addressof(u), C.sizeof(u)).hex(),
                          "sha256": hashlib.sha256(np.ascontiguousarray(rgba, np.float32).tobytes()).hexdigest()})
    with open(os.path.join(HERE, "shader_clouds_mm.json"), "w") as f:
        json.dump({"stride": SHADER_MM_STRIDE, "frames": mm_frames}, f, indent=1)


def shader_passes_golden():
    import ctypes as C
    sys.path.insert(0, os.path.join(REPO, "project-marshmallow_gb300"))
    sys.path.insert(0, REPO)
    import oracle
    import marshmallow as mm
    import marshmallow.lib as L
    import shader_golden as sg

    def ublock(u):
        return np.frombuffer(C.string_at(C.addressof(u), C.sizeof(u)), np.uint8)

    out = {}
    digests, ubs = [], []
    for k, case in enumerate(sg.REPROJECT_CASES):
        u = sg.reproject_uniforms(case)
        src = sg.pattern(case[1], case[0], k)
        digests.append(sg.digest(oracle.ref_reproject(u, src)))
        ubs.append(ublock(u))
    out["reproject_uniforms"] = np.stack(ubs)
    out["reproject_digests"] = np.array(digests)

    u = sg.post_uniforms()
    w, h = sg.POST_SIZE
    src = sg.pattern(h, w, 11)
    g = oracle.ref_post("god_ray", u, src)
    out["post_uniforms"] = ublock(u)
    out["god_ray_alpha"] = g[..., 3]
    out["radial_blur_rgb"] = oracle.ref_post("radial_blur", u, g)[..., :3]
    out["tonemap_rgb"] = oracle.unorm8(oracle.ref_post("tonemap", None, src)[..., :3])

    w, h = sg.SHADOW_SIZE
    u = mm.scene.uniforms(w, h, eye=(0.0, 150.0, 0.0), pitch=-20.0, sun_elevation=35.0, time=20.0)
    gb = mm.scene.terrain_gbuffer(u, w, h).astype(np.float32)
    tex = {"low_res": oracle.noise(L.NOISE_LOWRES, 0, 128, 128, 128, 4),
           "weather": oracle.noise(L.NOISE_WEATHER, 0, 512, 512, 1, 4)[0]}
    out["shadow_uniforms"] = ublock(u)
    out["shadow_world_pos"] = gb
    out["shadow"] = oracle.ref_model_shadow(u, tex, gb.reshape(-1, 4)).reshape(h, w).astype(np.float32)
    np.savez_compressed(os.path.join(HERE, "shader_passes.npz"), **out)


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    ref = args[0] if args else os.environ.get("MM_REF_DIR", "")
    if not os.path.isdir(os.path.join(ref, "SkyEngine")):
        sys.exit("usage: make_golden.py <reference tree root>  (or set MM_REF_DIR)")
    se = os.path.join(ref, "SkyEngine", "SkyEngine")
    asset_digests(se)
    if "--digests-only" in sys.argv:
        return
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "ref", "REF=" + ref], check=True)
    bins = os.path.join(REPO, "oracle", "_ref")
    shader_clouds_golden()
    shader_passes_golden()
    if "--shader-only" in sys.argv:
        return

    shipped = read_tga(os.path.join(se, "Textures", "CurlNoiseFBM.tga"))
    tmp = os.path.join(bins, "curl_from_reference.tga")
    subprocess.run([os.path.join(bins, "ref_curlgen"), tmp], check=True)
    built = read_tga(tmp)
    assert shipped.shape == (128, 128, 4) and np.array_equal(shipped, built), "reference build != shipped TGA"
    shipped.tofile(os.path.join(HERE, "curl_fbm_128.rgba"))

    rng = np.random.default_rng(7)
    pts = [(x, y, z) for x in range(-1, 26, 3) for y in range(-1, 26, 4) for z in range(-1, 26, 5)]
    pts += [tuple(float(v) for v in rng.uniform(-30, 30, 3).astype(np.float32)) for _ in range(200)]
    inp = "".join("%.9g %.9g %.9g\n" % p for p in pts)
    out = subprocess.run([os.path.join(bins, "ref_curlgen"), "--hash"], input=inp, capture_output=True, text=True,
                         check=True).stdout
    with open(os.path.join(HERE, "ref_hash.txt"), "w") as f:
        f.write("# x y z hashNoise(x,y,z) from ImageUtils.cpp:25 (compiled reference)\n" + out)

    triples = [(e, a, t) for e in (0.02, 0.1, 0.2, 0.3, 0.45, 0.6, 0.75, 0.9) for a in (0.25, 0.1, 0.4)
               for t in (0.0, 7.5)]
    inp = "".join("%.9g %.9g %.9g\n" % t for t in triples)
    out = subprocess.run([os.path.join(bins, "ref_sky")], input=inp, capture_output=True, text=True, check=True).stdout
    with open(os.path.join(HERE, "sky_reference.json"), "w") as f:
        json.dump(json.loads(out), f, indent=0)

    poses = []
    for (eye, fov, w, h) in (((0.0, 10.0, 0.0), 60.0, 256, 256), ((0.0, 10.0, 0.0), 60.0, 1920, 1080),
                             ((5.0, 150.0, -3.0), 45.0, 3840, 2160), ((1000.0, 300.0, -2000.0), 90.0, 512, 512)):
        for yaw, pitch in ((0.0, 15.0), (30.0, 5.0), (90.0, 25.0), (200.0, 40.0), (270.0, 0.0), (359.0, 89.9)):
            poses.append("%g %g %g %g %g %g %d %d\n" % (eye + (yaw, pitch, fov, w, h)))
    out = subprocess.run([os.path.join(bins, "ref_camera")], input="".join(poses), capture_output=True, text=True,
                         check=True).stdout
    with open(os.path.join(HERE, "camera_reference.json"), "w") as f:
        json.dump(json.loads(out), f, indent=0)

    d3 = os.path.join(se, "Textures", "3DTextures")
    lo = np.stack([read_tga(os.path.join(d3, "lowResCloudShape", "lowResCloud(%d).tga" % i)) for i in range(128)])
    hi = np.stack([read_tga(os.path.join(d3, "hiResCloudShape", "hiResClouds (%d).tga" % i)) for i in range(32)])
    stats = {}
    for name, a in (("low_res", lo), ("hi_res", hi)):
        f = a.reshape(-1, 4).astype(np.float64) / 255.0
        stats[name] = {"mean": f.mean(0).round(4).tolist(), "std": f.std(0).round(4).tolist()}
    with open(os.path.join(HERE, "nubis_stats.json"), "w") as f:
        json.dump(stats, f, indent=1)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
