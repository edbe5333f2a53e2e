#!/usr/bin/env python3
"""Cloud raymarch throughput at 3840x2160: Mrays/s and ms/frame.

One step = one full 3840x2160 frame of the cloud march (every pixel marched), cycling through the
16-frame camera sweep (yaw 0 -> 90 deg, pitch 5 -> 25 deg, t += 0.1 s; sun 30 deg) over the seed-0
textures that mm_noise_generate makes on the GPU.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm times K frames with CUDA events on the launch stream (L2 flushed between frames by a
256 MB memset outside the events), takes the max over ranks, and prints one JSON line with the
end-to-end figure through the C ABI (host-visible output copied back every frame), the roofline
of the march kernel against the on-chip rates it is bound by, the sampled SM clocks and a CPU
baseline (the FP32 oracle on the host cores over a sample of the same frames).
The reference arm (--impl reference) times the reference's march on the host CPU: the FP32
oracle restatement of compute-clouds.comp over all host threads, one bounded sample per step.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "project-marshmallow_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Mrays/s at 3840x2160 (cloud raymarch frame, every pixel marched)"
SWEEP = 16
PROFILE_SUMMARY = os.path.join(REPO, "profiles", "march_dram_4k.txt")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=48)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--width", type=int, default=3840)
    ap.add_argument("--height", type=int, default=2160)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--sampler", choices=["hardware", "software"], default="hardware")
    ap.add_argument("--math", choices=["fast", "exact"], default="fast")
    ap.add_argument("--schedule", choices=["persistent", "tiled"], default="tiled")
    ap.add_argument("--density", choices=["unorm8", "fp16", "bf16"], default="unorm8")
    ap.add_argument("--no-passes", action="store_true", help="skip the timings of the other passes")
    ap.add_argument("--no-variants", action="store_true",
                    help="skip the metric's variants (FP16/BF16 density, surrogate cone)")
    ap.add_argument("--batch", action="store_true",
                    help="time the uneven-view batch (mm_clouds_march_batch) instead of the 4K frame")
    ap.add_argument("--batch-views", type=int, default=70, help="first N views of the 70-view batch")
    ap.add_argument("--passes-only", action="store_true",
                    help="time only the other passes (one march frame as their input) and print their JSON")
    ap.add_argument("--small-launches", action="store_true",
                    help="time only the 1920x1080 1/16-pixel sweep and the 256x256 camera and print their JSON")
    return ap.parse_args()


def rank_info():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


# ------------------------------------------------------------------------------ clocks


class ClockSampler:
    """nvidia-smi clock/throttle samples taken while the timed region runs."""

    FIELDS = ("index,uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid):
        self.uuid = uuid
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "50"], stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 10:
                continue
            if self.uuid and self.uuid not in f[1]:
                continue
            rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        mhz = sorted(float(r[2]) for r in rows if r[2].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[6 + i].lower() == "active"})
        return {"sm_mhz": mhz[len(mhz) // 2] if mhz else None,
                "sm_max_mhz": float(rows[0][3]) if rows[0][3].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------------ shared


def reduce_max(value, dist, device):
    """The maximum of `value` over all ranks (the slowest rank's time); `dist` None = one process."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(world, units_per_rank, seconds):
    """Whole-job throughput of `world` replicas that each processed `units_per_rank` units, timed by
    the slowest rank (`seconds`): replicas only, no collective on the data path."""
    return world * units_per_rank / seconds


def sweep(k):
    import marshmallow as mm
    return mm.scene.sweep_params(k % SWEEP, SWEEP)


def frame_uniforms(k, w, h):
    import marshmallow as mm
    return mm.scene.sweep_uniforms(k % SWEEP, w, h, n=SWEEP)


def bench_config(args, w, h):
    """The workload both arms report (identical dicts, so the two lines describe the same config)."""
    return {"workload": "cloud march %dx%d, plain FP32 march, %s-filtered %s density textures, 16-frame sweep"
                        % (w, h, args.sampler, args.density.upper()),
            "width": w, "height": h, "frames_cycled": SWEEP, "textures": "seed 0 (Perlin-Worley/Worley/curl/weather)",
            "l2": "flushed between frames (256 MB memset outside the timed events)", "variant": "plain",
            "math": args.math, "sampler": args.sampler, "density": args.density, "schedule": args.schedule}


def cpu_march_sample(u, host_tex, w, h, row0, step):
    """FP32 oracle over rows row0::step and columns row0%step::step; returns (rays, seconds, threads)."""
    import oracle
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    rgba, _, _ = oracle.march(u, host_tex, w, h, precision=32, rows=(row0, h, step), col_begin=row0 % step,
                              col_step=step, nthreads=threads)
    dt = time.perf_counter() - t0
    return rgba.shape[0] * rgba.shape[1], dt, threads


# ------------------------------------------------------------------------------ reference arm


def run_reference(args):
    """The reference's march on the host CPU: the FP32 restatement of compute-clouds.comp (the oracle)
    over all host threads, with uniforms and textures from the oracle's own set-up (no GPU library is
    loaded).  Each step marches 1/64 of one sweep frame (every 8th row and column, offset per step)."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    import oracle
    oracle.build()
    w, h = args.width, args.height
    tex = oracle.seed_textures(0)
    step_px = 8
    for k in range(args.warmup):
        cpu_march_sample(oracle.sweep_uniforms(k % SWEEP, w, h, n=SWEEP), tex, w, h, k % step_px, step_px)
    rays = 0
    secs = 0.0
    threads = 1
    for k in range(args.steps):
        n, dt, threads = cpu_march_sample(oracle.sweep_uniforms(k % SWEEP, w, h, n=SWEEP), tex, w, h, k % step_px,
                                          step_px)
        rays += n
        secs += dt
    value = rays / secs / 1e6
    sample = ("FP32 oracle restatement of compute-clouds.comp on %d host threads; each step marches every 8th row "
              "and column of one sweep frame (1/64 of its rays, %d rays per step on average)"
              % (threads, rays // max(1, args.steps)))
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * secs / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(args, w, h),
        "sample_per_step": "1/64 of a frame: every 8th row and column",
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------ the other passes


def _median_ms(fn, flush, stream, n=10, warm=3):
    import torch
    ts = []
    for i in range(warm + n):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        if i >= warm:
            ts.append(a.elapsed_time(b))
    ts.sort()
    return ts[len(ts) // 2]


def _pass_line(ms, w, h, bytes_px, hbm_peak, note, cpu=None):
    gbs = bytes_px * w * h / (ms * 1e-3) / 1e9
    d = {"ms": round(ms, 4), "mpix_per_s": round(w * h / (ms * 1e-3) / 1e6, 1),
         "algorithmic_bytes_per_pixel": bytes_px, "achieved_gbs": round(gbs, 1),
         "hbm_frac": round(gbs / hbm_peak, 4) if hbm_peak else None, "note": note}
    if cpu:
        d["cpu_baseline"] = cpu
    return d


def _cpu_rate(fn, pixels):
    t0 = time.perf_counter()
    fn()
    dt = time.perf_counter() - t0
    return pixels / dt / 1e6, dt


def measure_passes(renderer, textures, rgba, depth, uniforms, w, h, flush, stream, hbm_peak, with_cpu):
    """Timings of the reference's other per-frame passes at the benchmark size (CUDA events, L2 flushed
    before each launch, median of 10): reprojection, the 16-phase frame (reprojection + 1/16 march),
    the mesh cloud-shadow march over a terrain G-buffer, the post chain to 8 bits; with CPU-oracle
    rates on a 960x540 sample when with_cpu."""
    import numpy as np
    import torch
    import marshmallow as mm
    import marshmallow.lib as L
    out = {}
    src = (rgba, depth)
    dst = (torch.empty_like(rgba), torch.empty_like(depth))
    # Reprojection: motion of one sweep step (6 degrees of yaw) and of a 0.5 degree pan.
    u_sweep = mm.scene.sweep_uniforms(5, w, h, n=SWEEP)
    u_sweep.camera_prev = uniforms[4].camera_prev
    p = sweep(5)
    u_pan = mm.scene.uniforms(w, h, yaw=p["yaw"], pitch=p["pitch"], time=p["time"])
    u_pan.camera_prev = mm.scene.uniforms(w, h, yaw=p["yaw"] - 0.5, pitch=p["pitch"], time=p["time"]).camera_prev
    cpu = None
    sw, sh = 960, 540
    if with_cpu:
        import oracle
        us = mm.scene.sweep_uniforms(5, sw, sh, n=SWEEP)
        us.camera_prev = mm.scene.sweep_uniforms(4, sw, sh, n=SWEEP).camera_prev
        img = np.random.default_rng(0).uniform(0, 1, (sh, sw, 4)).astype(np.float32)
        rate, dt = _cpu_rate(lambda: oracle.reproject(us, img, img[..., 0].copy()), sw * sh)
        cpu = {"value": round(rate, 2), "unit": "Mpix/s", "cores": 1, "kind": "port",
               "sample": "oracle reprojection of one %dx%d frame (%.2f s)" % (sw, sh, dt)}
    out["reproject_sweep_step"] = _pass_line(
        _median_ms(lambda: renderer.reproject(u_sweep, src, dst), flush, stream), w, h, 40.0, hbm_peak,
        "reproject.comp, every pixel, motion of one sweep step (6 deg yaw); RGBA32F + depth in and out", cpu)
    out["reproject_sweep_step_exact"] = _pass_line(
        _median_ms(lambda: renderer.reproject(u_sweep, src, dst, math=L.MATH_EXACT), flush, stream), w, h, 40.0,
        hbm_peak, "the same in exact arithmetic (bit-identical to the CPU restatement)")
    out["reproject_pan_0p5deg"] = _pass_line(
        _median_ms(lambda: renderer.reproject(u_pan, src, dst), flush, stream), w, h, 40.0, hbm_peak,
        "reproject.comp, every pixel, a 0.5 deg pan")
    # The reference's per-frame compute work: reprojection + march of one pixel in 16.
    u_f = mm.scene.sweep_uniforms(5, w, h, n=SWEEP, )
    u_f.camera_prev = uniforms[4].camera_prev
    u_f.sun.color[3] = 5.0
    out["frame_phase16"] = _pass_line(
        _median_ms(lambda: renderer.frame(u_f, textures, src, dst), flush, stream), w, h, 40.0, hbm_peak,
        "mm_clouds_frame: reprojection of every pixel + march of the pixels of phase 5 (1/16)")
    # Mesh cloud shadows over a terrain G-buffer (camera 150 m up, 20 deg down, sun 45 deg).
    u_s = mm.scene.uniforms(w, h, eye=(0.0, 150.0, 0.0), pitch=-20.0, sun_elevation=45.0, time=5.0)
    gbuf = mm.scene.terrain_gbuffer_cuda(u_s, w, h)
    shadow = torch.empty((h, w), dtype=torch.float32, device="cuda")
    cpu = None
    if with_cpu:
        import oracle
        us = mm.scene.uniforms(sw, sh, eye=(0.0, 150.0, 0.0), pitch=-20.0, sun_elevation=45.0, time=5.0)
        g = mm.scene.terrain_gbuffer(us, sw, sh)
        host = {"weather": textures.host("weather"), "low_res": textures.host("low_res")}
        threads = os.cpu_count() or 1
        rate, dt = _cpu_rate(lambda: oracle.shadow(us, host, g, nthreads=threads), sw * sh)
        cpu = {"value": round(rate, 2), "unit": "Mpix/s", "cores": threads, "kind": "port",
               "sample": "oracle shadow march of one %dx%d terrain G-buffer (%.2f s)" % (sw, sh, dt)}
    out["mesh_shadow"] = _pass_line(
        _median_ms(lambda: renderer.mesh_shadow(u_s, textures, gbuf, shadow=shadow), flush, stream), w, h, 20.0,
        hbm_peak, "model.frag cloud-shadow march, %.0f%% of pixels covered; float4 positions in, float shadow out"
        % (100.0 * float((gbuf[..., 3] != 0).float().mean())), cpu)
    del gbuf
    # Post chain: god rays + radial blur + tonemap of a cloud frame looking at the sun -> 8 bits.
    u_p = mm.scene.uniforms(w, h, yaw=0.0, pitch=12.0, sun_elevation=20.0)
    renderer.march(u_p, textures, rgba)
    out8 = torch.empty((h, w, 4), dtype=torch.uint8, device="cuda")
    cpu = None
    if with_cpu:
        import oracle
        up = mm.scene.uniforms(sw, sh, yaw=0.0, pitch=12.0, sun_elevation=20.0)
        img = torch.nn.functional.interpolate(rgba.permute(2, 0, 1)[None], size=(sh, sw)).squeeze(0).permute(1, 2, 0)
        img = img.contiguous().cpu().numpy()
        rate, dt = _cpu_rate(lambda: oracle.post_chain(up, img), sw * sh)
        cpu = {"value": round(rate, 2), "unit": "Mpix/s", "cores": 1, "kind": "port",
               "sample": "oracle post chain of one %dx%d frame (%.2f s)" % (sw, sh, dt)}
    out["post_chain"] = _pass_line(
        _median_ms(lambda: renderer.post_chain(u_p, rgba, out8), flush, stream), w, h, 20.0, hbm_peak,
        "god rays + radial blur + tonemap (alpha plane, god-ray plane, fused blur/tonemap; texture-unit "
        "taps); RGBA32F in, B8G8R8A8 out", cpu)
    out["post_chain_exact"] = _pass_line(
        _median_ms(lambda: renderer.post_chain(u_p, rgba, out8, math=L.MATH_EXACT), flush, stream), w, h, 20.0,
        hbm_peak, "the same in exact arithmetic with float-weight bilinear taps (bit-identical to the CPU "
                  "restatement)")
    out["reference_frame_1080p"] = reference_frame_1080p(renderer, textures, flush, stream)
    return out


def measure_configs(renderer, textures, flush, stream, with_cpu):
    """The two smaller workloads of the baseline plan, GPU beside the CPU restatement: the 256x256
    camera (pitch 15 deg, sun 30 deg, t = 0) and the 1920x1080 16-frame sweep; production arithmetic,
    hardware sampler, full frames.  CPU: the FP32 oracle on all host threads, the whole 256x256 frame
    and every 2nd row and column of the 16 sweep frames."""
    import torch
    import marshmallow as mm
    out = {}
    u0 = mm.scene.uniforms(256, 256)
    rgba = torch.empty((256, 256, 4), device="cuda")
    dep = torch.empty((256, 256), device="cuda")
    ms0 = _median_ms(lambda: renderer.march(u0, textures, rgba, dep), flush, stream)
    out["camera_256"] = {"ms": round(ms0, 4), "mrays_per_s": round(256 * 256 / ms0 / 1e3, 1)}
    W, H = 1920, 1080
    rgba = torch.empty((H, W, 4), device="cuda")
    dep = torch.empty((H, W), device="cuda")
    us = [mm.scene.sweep_uniforms(k, W, H) for k in range(SWEEP)]
    ms1 = sum(_median_ms(lambda: renderer.march(u, textures, rgba, dep), flush, stream, n=3) for u in us) / SWEEP
    out["sweep_1080p"] = {"ms_per_frame": round(ms1, 4), "mrays_per_s": round(W * H / ms1 / 1e3, 1)}
    out["small_launches"] = measure_small_launches(renderer, textures, flush, stream)
    if with_cpu:
        host = textures.host_all()
        n, dt, th = cpu_march_sample(u0, host, 256, 256, 0, 1)
        out["camera_256"]["cpu"] = {"ms": round(1e3 * dt, 2), "mrays_per_s": round(n / dt / 1e6, 3), "cores": th,
                                    "kind": "port"}
        rays = 0
        secs = 0.0
        for k, u in enumerate(us):
            n, dt, th = cpu_march_sample(u, host, W, H, k % 2, 2)
            rays += n
            secs += dt
        out["sweep_1080p"]["cpu"] = {"mrays_per_s": round(rays / secs / 1e6, 3), "cores": th, "kind": "port",
                                     "ms_per_frame_estimated": round(1e3 * secs / SWEEP * (W * H * SWEEP / rays), 1),
                                     "sample": "every 2nd row and column of the 16 frames (%.1f s)" % secs}
    return out


def measure_small_launches(renderer, textures, flush, stream):
    """The reference's own per-frame march (compute-clouds.comp dispatched over one pixel in 16 at
    1920x1080, VulkanApplication.cpp:381-384): the 16 sweep frames, frame k marching phase k,
    CUDA events, L2 flushed before each launch, median of 5 per frame; and the 256x256 camera."""
    import torch
    import marshmallow as mm
    import marshmallow.lib as L
    W, H = 1920, 1080
    rgba = torch.zeros((H, W, 4), device="cuda")
    dep = torch.zeros((H, W), device="cuda")
    per = []
    for k in range(SWEEP):
        u = mm.scene.sweep_uniforms(k, W, H)
        u.sun.color[3] = float(k)
        per.append(_median_ms(lambda: renderer.march(u, textures, rgba, dep, pixel_mode=L.PIXELS_PHASE16), flush,
                              stream, n=5, warm=2))
    mean = sum(per) / len(per)
    u0 = mm.scene.uniforms(256, 256)
    a = torch.zeros((256, 256, 4), device="cuda")
    d = torch.zeros((256, 256), device="cuda")
    ms256 = _median_ms(lambda: renderer.march(u0, textures, a, d), flush, stream, n=5, warm=2)
    W4, H4 = 3840, 2160
    rgba4 = torch.zeros((H4, W4, 4), device="cuda")
    dep4 = torch.zeros((H4, W4), device="cuda")
    per4 = []
    for k in (0, 5, 10, 15):
        u = mm.scene.sweep_uniforms(k, W4, H4)
        u.sun.color[3] = float(k)
        per4.append(_median_ms(lambda: renderer.march(u, textures, rgba4, dep4, pixel_mode=L.PIXELS_PHASE16), flush,
                               stream, n=5, warm=2))
    return {"phase16_1080p": {"ms_mean": round(mean, 4), "ms_per_frame": [round(x, 4) for x in per],
                              "mrays_per_s": round((W // 4) * (H // 4) / mean / 1e3, 1),
                              "note": "march of the pixels of phase k of sweep frame k (1/16 of 1920x1080)"},
            "phase16_4k": {"ms_mean": round(sum(per4) / len(per4), 4), "frames": [0, 5, 10, 15]},
            "camera_256_ms": round(ms256, 4)}


def reference_frame_1080p(renderer, textures, flush, stream, frames=16):
    """The reference application's per-frame GPU work at its own resolution (1920x1080), as this
    library runs it: mm_clouds_frame (reprojection of every pixel + the march of one pixel in 16),
    mm_mesh_shadow over a terrain G-buffer (the lit mesh colour, which the mesh raster pass would
    write, is copied in from a template each frame), mm_post_chain to the 8-bit swapchain layout.
    Camera 150 m up looking 4 degrees down: clouds above, terrain below.  Mean over 16 frames
    (all pixel phases), camera turning 0.25 degrees per frame; L2 flushed before each frame."""
    import torch
    import marshmallow as mm
    W, H = 1920, 1080
    bufs = [(torch.zeros((H, W, 4), device="cuda"), torch.full((H, W), float("inf"), device="cuda")) for _ in range(2)]
    us = [mm.scene.uniforms(W, H, eye=(0.0, 150.0, 0.0), yaw=0.25 * k, pitch=-4.0, time=0.1 * k, sun_elevation=25.0)
          for k in range(frames + 1)]
    for k in range(1, frames + 1):
        us[k].camera_prev = us[k - 1].camera_prev
        us[k].sun.color[3] = float(k % 16)
    gbuf = mm.scene.terrain_gbuffer_cuda(us[0], W, H)
    lit = torch.zeros((H, W, 4), device="cuda")
    lit[..., 0], lit[..., 1], lit[..., 2] = 0.35, 0.32, 0.28
    lit[..., 3] = (gbuf[..., 3] != 0).float()
    mesh = torch.empty_like(lit)
    out8 = torch.empty((H, W, 4), dtype=torch.uint8, device="cuda")
    for k in range(16):  # warm-up: fills the frame history through all 16 phases
        renderer.frame(us[k + 1], textures, bufs[k % 2], bufs[(k + 1) % 2])
    side = torch.cuda.Stream()
    fork, join = torch.cuda.Event(), torch.cuda.Event()
    ts = []
    for k in range(1, frames + 1):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        prev, cur = bufs[k % 2], bufs[(k + 1) % 2]
        # the mesh shadow needs only the G-buffer and the textures: it runs on a second stream while
        # the latency-bound 1/16 march runs; the post chain waits for both
        fork.record(stream)
        side.wait_event(fork)
        with torch.cuda.stream(side):
            mesh.copy_(lit)
            renderer.mesh_shadow(us[k], textures, gbuf, rgba=mesh, stream=side)
        join.record(side)
        renderer.frame(us[k], textures, prev, cur)
        stream.wait_event(join)
        renderer.post_chain(us[k], cur[0], out8, mesh=mesh)
        b.record(stream)
        torch.cuda.synchronize()
        ts.append(a.elapsed_time(b))
    ms = sum(ts) / len(ts)
    return {"ms": round(ms, 4), "fps": round(1000.0 / ms, 1), "frames": frames, "width": W, "height": H,
            "note": "reprojection + 1/16 march (concurrent), mesh cloud shadow (terrain %.0f%% of pixels) on a "
                    "second stream beside them, then the post chain to 8 bits; the lit mesh colour copied in "
                    "from a template stands in for the mesh raster pass"
                    % (100.0 * float((gbuf[..., 3] != 0).float().mean()))}


# ------------------------------------------------------------------------------ the metric's variants


def train_surrogate(lib, stream):
    """The learned sun-cone surrogate as the library trains it: 2^22 samples of the plain six-tap cone
    (texture seeds 1-8, sun 0-90 deg) by mm_surrogate_generate, then 256 Adam steps of batch 131072
    (8 passes over the samples) by mm_mlp_train on the tensor cores.  Returns the network and the
    training cost."""
    import torch
    import marshmallow.lib as L
    sp = C.c_void_p(stream.cuda_stream)
    per_seed = 1 << 19
    x = torch.empty((8 * per_seed, 16), dtype=torch.bfloat16, device="cuda")
    t = torch.empty(8 * per_seed, dtype=torch.float32, device="cuda")
    n = C.c_int()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.check(lib.mm_surrogate_generate(1, 8, per_seed, 150000.0, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()),
                                      C.byref(n), sp), "mm_surrogate_generate")
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    net = C.c_void_p()
    L.check(lib.mm_mlp_create(11, C.byref(net)), "mm_mlp_create")
    steps = 0
    for lr, k in ((8e-3, 128), (2.5e-3, 128)):
        L.check(lib.mm_mlp_train(net, C.c_void_p(x.data_ptr()), C.c_void_p(t.data_ptr()), n.value, 131072, k, lr, None,
                                 sp), "mm_mlp_train")
        steps += k
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    # forward + backward of the 16-64-64-64-1 network: 3 x 2 x 9280 multiply-adds' FLOP per sample
    tflops = 3 * 2 * 9280 * 131072 * steps / (t2 - t1) / 1e12
    peaks_file = os.path.join(REPO, "MEASURED_PEAKS.json")
    bf16 = json.load(open(peaks_file)).get("bf16_tflops") if os.path.exists(peaks_file) else None
    return net, {"samples": n.value, "generate_ms": round(1e3 * (t1 - t0), 2), "train_steps": steps, "batch": 131072,
                 "train_ms": round(1e3 * (t2 - t1), 2), "train_tflops": round(tflops, 1),
                 "train_frac_of_measured_bf16": round(tflops / bf16, 4) if bf16 else None,
                 "note": "one-off cost per texture set, not part of a frame"}


def measure_variants(lib, renderer, textures, w, h, flush, stream, with_oracle, net, training):
    """The benchmark metric itself: the 3840x2160 sweep for each variant of the march -- plain with
    UNORM8 (the reference's texel format), FP16 (also with the large-step coverage test in half2)
    or BF16 density textures, and the learned
    sun-cone surrogate with UNORM8 or FP16 density -- each with its ms/frame (CUDA events, L2 flushed
    before every frame, mean over the 16 sweep frames) and its error against the FP64 oracle (exact
    filter weights) on a fixed grid (every 8th row and column, sweep frames 0, 5, 10, 15)."""
    import numpy as np
    import torch
    import marshmallow as mm
    import marshmallow.lib as L
    variants = [("plain_unorm8", L.FORMAT_UNORM8, None), ("surrogate_unorm8", L.FORMAT_UNORM8, net.value),
                ("plain_fp16", L.FORMAT_FP16, None), ("surrogate_fp16", L.FORMAT_FP16, net.value),
                ("plain_fp16_half2", L.FORMAT_FP16, None), ("plain_bf16", L.FORMAT_BF16, None)]
    err_frames = (0, 5, 10, 15)
    refs = {}
    if with_oracle:
        import oracle
        oracle.build()
        host = textures.host_all()
        for k in err_frames:
            ref, rdep, _ = oracle.march(frame_uniforms(k, w, h), host, w, h, precision=64, rows=(3, h, 8), col_begin=3,
                                        col_step=8)
            refs[k] = (ref, rdep)
    rgba = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    dep = torch.empty((h, w), dtype=torch.float32, device="cuda")
    out = {}
    try:
        for name, fmt, sur in variants:
            textures.set_density_format(fmt)
            opts = dict(density_format=fmt, surrogate=sur)
            if name.endswith("half2"):
                opts["math"] = L.MATH_FAST_HALF2  # large-step coverage test in half2
            for k in range(SWEEP):
                renderer.march(frame_uniforms(k, w, h), textures, rgba, dep, **opts)
            ts = []
            for k in range(SWEEP):
                flush.zero_()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                renderer.march(frame_uniforms(k, w, h), textures, rgba, dep, **opts)
                b.record(stream)
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(b))
            ms = sum(ts) / len(ts)
            d = {"ms_per_frame": round(ms, 4), "mrays_per_s": round(w * h / ms / 1e3, 1)}
            if refs:
                es = []
                for k in err_frames:
                    renderer.march(frame_uniforms(k, w, h), textures, rgba, dep, **opts)
                    torch.cuda.synchronize()
                    img = rgba[3::8, 3::8].cpu().numpy()
                    dd = dep[3::8, 3::8].cpu().numpy()
                    es.append(mm.metrics.frame_errors(img, refs[k][0], dd, refs[k][1]))
                d.update({"rmse_255_mean": round(float(np.mean([e["rmse_255"] for e in es])), 4),
                          "rmse_255_max": round(max(e["rmse_255"] for e in es), 4),
                          "p999_255_max": round(max(e["p999_255"] for e in es), 3),
                          "max_255_max": round(max(e["max_255"] for e in es), 2),
                          "frac_over_4_max": max(e["frac_over_4"] for e in es),
                          "depth_rel_median_max": max(e["depth_rel_median"] for e in es),
                          "within_rmse_2_255": all(e["rmse_255"] <= 2.0 for e in es)})
            out[name] = d
    finally:
        textures.set_density_format(L.FORMAT_UNORM8)
    plain = out["plain_unorm8"]["ms_per_frame"]
    summary = {"surrogate_fp16_vs_plain_speedup": round(plain / out["surrogate_fp16"]["ms_per_frame"], 4),
               "fp16_vs_plain_speedup": round(plain / out["plain_fp16"]["ms_per_frame"], 4),
               "fp16_half2_vs_plain_speedup": round(plain / out["plain_fp16_half2"]["ms_per_frame"], 4),
               "surrogate_fp16_rmse_255_max": out["surrogate_fp16"].get("rmse_255_max"),
               "error_yardstick": "FP64 oracle, exact filter weights, every 8th row and column of sweep frames "
                                  "0, 5, 10, 15" if refs else None}
    return {"variants": out, "surrogate_training": training, "summary": summary}


# ------------------------------------------------------------------------------ our arm


def read_profile_traffic():
    """Per-launch DRAM bytes of the march kernel from the committed ncu summary, if present."""
    try:
        for line in open(PROFILE_SUMMARY):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def run_ours(args):
    import torch
    import marshmallow as mm
    import marshmallow.lib as L

    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    lib = L.load()
    w, h = args.width, args.height
    stream = torch.cuda.current_stream()
    sptr = C.c_void_p(stream.cuda_stream)

    textures = mm.render.Textures(seed=0)
    density_format = {"unorm8": L.FORMAT_UNORM8, "fp16": L.FORMAT_FP16, "bf16": L.FORMAT_BF16}[args.density]
    if density_format != L.FORMAT_UNORM8:
        textures.set_density_format(density_format)
    renderer = mm.render.Renderer()
    rgba = torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    depth = torch.empty((h, w), dtype=torch.float32, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    uniforms = [frame_uniforms(k, w, h) for k in range(SWEEP)]

    sampler_mode = L.SAMPLER_HARDWARE if args.sampler == "hardware" else L.SAMPLER_SOFTWARE
    math_mode = L.MATH_FAST if args.math == "fast" else L.MATH_EXACT
    schedule = L.SCHEDULE_PERSISTENT if args.schedule == "persistent" else L.SCHEDULE_TILED

    def march(k, out_rgba=rgba, out_depth=depth, s=None, counters=None):
        renderer.march(uniforms[k % SWEEP], textures, out_rgba, out_depth, stream=s, counters=counters,
                       sampler=sampler_mode, math=math_mode, schedule=schedule, density_format=density_format)

    for k in range(args.warmup):
        march(k)
    torch.cuda.synchronize()

    if args.small_launches:
        if rank == 0:
            print(json.dumps(measure_small_launches(renderer, textures, flush, stream)), flush=True)
        renderer.close()
        textures.close()
        if dist:
            dist.destroy_process_group()
        return

    if args.passes_only:
        if rank == 0:
            peaks_file = os.path.join(REPO, "MEASURED_PEAKS.json")
            hbm = json.load(open(peaks_file)).get("hbm_gbs") if os.path.exists(peaks_file) else None
            passes = measure_passes(renderer, textures, rgba, depth, uniforms, w, h, flush, stream, hbm,
                                    world == 1 and not args.no_cpu_baseline)
            print(json.dumps({"passes": passes, "width": w, "height": h}), flush=True)
        renderer.close()
        textures.close()
        if dist:
            dist.destroy_process_group()
        return

    props = torch.cuda.get_device_properties(local)
    uuid = str(getattr(props, "uuid", "") or "")
    sampler = ClockSampler(uuid)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sampler.start()
    launches0 = lib.mm_kernel_launch_count()
    for k in range(args.steps):
        flush.zero_()  # L2 flush between frames, outside the timed events
        ev[k][0].record(stream)
        march(k)
        ev[k][1].record(stream)
    torch.cuda.synchronize()
    launches = lib.mm_kernel_launch_count() - launches0
    if dist:
        dist.barrier()
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    total_ms = reduce_max(sum(step_ms), dist, "cuda")
    rays_per_frame = w * h
    value = whole_job_rate(world, rays_per_frame * args.steps, total_ms * 1e-3) / 1e6
    ms_frame = total_ms / args.steps

    # Algorithmic work of the timed frames (same frames, counted in a separate untimed pass).
    cnt = torch.zeros(4, dtype=torch.int64, device="cuda")
    for k in range(args.steps):
        march(k, counters=cnt)
    torch.cuda.synchronize()
    n_test, n_hires, n_iter, n_acc = (int(x) for x in cnt.cpu().tolist())
    f3d = (n_test + n_hires) / args.steps  # trilinear 3D fetches per frame (one per call)
    f2d = (n_test + n_hires) / args.steps  # bilinear 2D fetches per frame (one per call)

    # On-chip peaks measured now on this GPU (MEASURED_PEAKS.json holds HBM and bf16 only).
    pk = (C.c_double * 3)()
    if density_format != L.FORMAT_UNORM8:
        textures.set_density_format(L.FORMAT_UNORM8)
    L.check(lib.mm_measure_peaks(textures.handles["low_res"], textures.handles["weather"], pk, sptr),
            "mm_measure_peaks")
    peak3d, peak2d, peak_fp32 = pk[0], pk[1], pk[2]
    sec_frame = ms_frame * 1e-3
    tex_time_frac = (f3d / (peak3d * 1e9) + f2d / (peak2d * 1e9)) / sec_frame
    achieved_gfetch = (f3d + f2d) / sec_frame / 1e9
    # UNORM8 texel bytes: 8 x 4 B per trilinear RGBA fetch, 4 x 4 B per bilinear weather fetch,
    # 4 x 2 B per bilinear RG curl fetch.
    texel_bytes = 32.0 * f3d + (16.0 * n_test + 8.0 * n_hires) / args.steps
    peak_eff = (f3d + f2d) / (f3d / peak3d + f2d / peak2d) if f3d + f2d > 0 else peak3d
    out_bytes = 20.0 * rays_per_frame  # RGBA32F + depth written once
    peaks_file = os.path.join(REPO, "MEASURED_PEAKS.json")
    hbm_peak = None
    if os.path.exists(peaks_file):
        hbm_peak = json.load(open(peaks_file)).get("hbm_gbs")
    hbm_achieved = (out_bytes + 9.4e6) / sec_frame / 1e9
    traffic = read_profile_traffic()

    # End to end through the C ABI with host buffers: each frame's uniforms go to the device with the
    # launch (mm_uniforms by value), the frame's RGBA32F + depth come back to pinned host memory.
    e2e = None
    if not args.no_e2e:
        s_cmp = torch.cuda.Stream()
        s_cpy = torch.cuda.Stream()
        dev_rgba = [rgba, torch.empty_like(rgba)]
        dev_depth = [depth, torch.empty_like(depth)]
        host_rgba = [torch.empty((h, w, 4), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        host_depth = [torch.empty((h, w), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        done_cmp = [torch.cuda.Event() for _ in range(2)]
        done_cpy = [torch.cuda.Event() for _ in range(2)]
        for i in range(2):
            done_cpy[i].record(s_cpy)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for k in range(args.steps):
            b = k % 2
            s_cmp.wait_event(done_cpy[b])
            march(k, dev_rgba[b], dev_depth[b], s=s_cmp)
            done_cmp[b].record(s_cmp)
            s_cpy.wait_event(done_cmp[b])
            with torch.cuda.stream(s_cpy):
                host_rgba[b].copy_(dev_rgba[b], non_blocking=True)
                host_depth[b].copy_(dev_depth[b], non_blocking=True)
            done_cpy[b].record(s_cpy)
        torch.cuda.synchronize()
        e2e_s = reduce_max(time.perf_counter() - t0, dist, "cuda")
        e2e = {"value": round(whole_job_rate(world, rays_per_frame * args.steps, e2e_s) / 1e6, 3), "unit": "Mrays/s",
               "h2d_bytes_per_step": C.sizeof(L.Uniforms), "d2h_bytes_per_step": 20 * rays_per_frame,
               "ms_per_step": round(1e3 * e2e_s / args.steps, 3)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        host_tex = textures.host_all()
        rays = 0
        secs = 0.0
        threads = 1
        for k in range(SWEEP):  # all 16 sweep frames, every 3rd row and column (~11 s on 16 cores)
            n, dt, threads = cpu_march_sample(uniforms[k], host_tex, w, h, k % 3, 3)
            rays += n
            secs += dt
        cpu = {"value": round(rays / secs / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": "FP32 oracle restatement of compute-clouds.comp on the 16 sweep frames, every 3rd row "
                         "and column (%d rays, %.1f s)" % (rays, secs)}

    configs = None
    if rank == 0 and world == 1 and not args.no_passes:
        configs = measure_configs(renderer, textures, flush, stream, not args.no_cpu_baseline)

    variants = None
    batch = None
    if rank == 0 and world == 1 and not args.no_variants:
        net, training = train_surrogate(lib, stream)
        try:
            variants = measure_variants(lib, renderer, textures, w, h, flush, stream, not args.no_cpu_baseline, net,
                                        training)
            batch = measure_batch(renderer, textures, net.value, flush, stream, steps=3, warmup=2)
        finally:
            lib.mm_mlp_destroy(net)

    passes = None
    if rank == 0 and not args.no_passes:
        passes = measure_passes(renderer, textures, rgba, depth, uniforms, w, h, flush, stream, hbm_peak,
                                world == 1 and not args.no_cpu_baseline)

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_frame, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(args, w, h),
            "roofline": {"bound": "tex", "achieved": round(achieved_gfetch, 2), "peak": round(peak_eff, 1),
                         "unit": "Gfetch/s",
                         "frac": round(tex_time_frac, 4), "traffic": traffic,
                         "peak_3d_gfetch": round(peak3d, 1), "peak_2d_gfetch": round(peak2d, 1),
                         "fetches_3d_per_frame": f3d, "fetches_2d_per_frame": f2d,
                         "texel_bytes_per_frame": texel_bytes,
                         "peak_source": "in-run microbenchmark mm_measure_peaks (texture unit, L1-resident)",
                         "frac_definition": "time the texture unit needs at its measured peak for the frame's "
                                            "algorithmic fetches / kernel time"},
            "roofline_hbm": {"bound": "hbm", "achieved": round(hbm_achieved, 2), "peak": hbm_peak, "unit": "GB/s",
                             "frac": round(hbm_achieved / hbm_peak, 4) if hbm_peak else None,
                             "algorithmic_bytes": out_bytes + 9.4e6, "traffic": traffic},
            "fp32_peak_tflops": round(peak_fp32, 2),
            "work_per_frame": {"cloud_test": n_test / args.steps, "cloud_hires": n_hires / args.steps,
                               "iterations": n_iter / args.steps, "accumulated": n_acc / args.steps},
            "e2e": e2e, "gpu_launches": int(launches), "clocks": clocks, "cpu_baseline": cpu,
            "configs": configs, "variants": variants, "batch": batch, "passes": passes,
        }
        print(json.dumps(line), flush=True)
    renderer.close()
    textures.close()
    if dist:
        dist.destroy_process_group()


def measure_batch(renderer, tex, net, flush, stream, steps, warmup, n_views=70):
    """Many views in one launch: the seeded 70-view batch (6 cube-map faces at 512^2, 32 cameras at
    640x360-1920x1080, 32 cameras at 3840x2160 with random sun and yaw).  Plain cone with UNORM8
    density: one mm_clouds_march_batch per step with the schedule and tile shape the autotuner
    picks, beside the same views as one launch each.  With a trained surrogate (`net`): the batch of
    the mixed-precision learned configuration -- surrogate cone, FP16 density, graph schedule."""
    import torch
    import marshmallow as mm
    import marshmallow.lib as L
    lib = mm.lib.load()
    views = mm.scene.batch_views(seed=0)[:max(1, n_views)]
    outs = [(torch.empty((h, w, 4), device="cuda"), torch.empty((h, w), device="cuda")) for w, h, _ in views]
    rays = sum(w * h for w, h, _ in views)
    arr = renderer.march_batch(views, tex, outs)
    best, table = renderer.autotune_batch(arr, len(views), tex)
    opts = dict(warp_tile_w=best.warp_tile_w, tiles_per_grab=best.tiles_per_grab, schedule=best.schedule)

    def timed(fn, k):
        ts = []
        for i in range(warmup + k):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            if i >= warmup:
                ts.append(a.elapsed_time(b))
        return sum(ts) / len(ts)

    l0 = lib.mm_kernel_launch_count()
    ms = timed(lambda: renderer.march_batch(views, tex, outs, **opts), steps)
    launches = lib.mm_kernel_launch_count() - l0
    ms_seq = timed(lambda: [renderer.march(u, tex, o[0], o[1]) for (w, h, u), o in zip(views, outs)], max(1, steps // 4))
    out = {"views": len(views), "mrays_per_step": round(rays / 1e6, 2),
           "plain_unorm8": {"ms": round(ms, 3), "mrays_per_s": round(rays / ms / 1e3, 1),
                            "schedule": {0: "persistent", 1: "blocks", 2: "graph"}[best.schedule],
                            "warp_tile_w": best.warp_tile_w, "tiles_per_grab": best.tiles_per_grab,
                            "gpu_launches_per_step": int(launches) // max(1, warmup + steps)},
           "one_launch_per_view_ms": round(ms_seq, 3), "autotune_ms": [round(v, 2) for v in table],
           "l2": "flushed between steps"}
    if net is not None:
        tex.set_density_format(L.FORMAT_FP16)
        try:
            sur = dict(density_format=L.FORMAT_FP16, surrogate=net, schedule=L.BATCH_GRAPH)
            ms_s = timed(lambda: renderer.march_batch(views, tex, outs, **sur), steps)
            ms_f = timed(lambda: renderer.march_batch(views, tex, outs, density_format=L.FORMAT_FP16,
                                                      schedule=L.BATCH_GRAPH), steps)
        finally:
            tex.set_density_format(L.FORMAT_UNORM8)
        out["surrogate_fp16"] = {"ms": round(ms_s, 3), "mrays_per_s": round(rays / ms_s / 1e3, 1),
                                 "schedule": "graph (surrogate views one after another)"}
        out["plain_fp16"] = {"ms": round(ms_f, 3), "mrays_per_s": round(rays / ms_f / 1e3, 1), "schedule": "graph"}
    return out


def run_batch(args):
    """The batch alone as its own JSON line (`python bench.py --batch`)."""
    import torch
    import marshmallow as mm
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if rank != 0:
        return
    tex = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    b = measure_batch(r, tex, None, flush, torch.cuda.current_stream(), args.steps, args.warmup, args.batch_views)
    p = b["plain_unorm8"]
    line = {
        "metric": "Mrays/s, %d views of uneven resolution in one batched launch" % b["views"],
        "value": p["mrays_per_s"], "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": p["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "seeded uneven-view batch (cube faces 512^2, 640x360-1920x1080 cameras, 3840x2160 "
                               "cameras with random sun 5-85 deg and yaw 0-360 deg)", "views": b["views"],
                   "mrays_per_step": b["mrays_per_step"], "schedule": p["schedule"], "warp_tile_w": p["warp_tile_w"],
                   "tiles_per_grab": p["tiles_per_grab"], "l2": "flushed between steps"},
        "one_launch_per_view_ms": b["one_launch_per_view_ms"], "autotune_ms": b["autotune_ms"],
        "gpu_launches": p["gpu_launches_per_step"] * args.steps,
    }
    print(json.dumps(line), flush=True)
    r.close()
    tex.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.batch:
        run_batch(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
