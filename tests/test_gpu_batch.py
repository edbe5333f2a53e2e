"""Many views in one persistent, graph-captured launch (mm_clouds_march_batch) and its autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(cuda, mmlib):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    yield t, r
    r.close()
    t.close()


def _outputs(cuda, views):
    return [(cuda.zeros((h, w, 4), device="cuda"), cuda.zeros((h, w), device="cuda")) for w, h, _ in views]


def test_batch_equals_single_views(cuda, env):
    import marshmallow as mm
    tex, r = env
    views = mm.scene.cubemap_views(128) + [(320, 180, mm.scene.uniforms(320, 180, yaw=40.0, pitch=20.0)),
                                          (257, 131, mm.scene.uniforms(257, 131, yaw=200.0, pitch=8.0, time=1.0,
                                                                       sun_elevation=70.0))]
    import marshmallow.lib as L
    for tw, grab, sched in ((8, 4, L.BATCH_PERSISTENT), (4, 1, L.BATCH_PERSISTENT), (32, 16, L.BATCH_PERSISTENT),
                            (8, 4, L.BATCH_BLOCKS), (8, 4, L.BATCH_GRAPH)):
        outs = _outputs(cuda, views)
        r.march_batch(views, tex, outs, warp_tile_w=tw, tiles_per_grab=grab, schedule=sched)
        cuda.cuda.synchronize()
        for (w, h, u), (rgba, dep) in zip(views, outs):
            ref = cuda.zeros((h, w, 4), device="cuda")
            rdep = cuda.zeros((h, w), device="cuda")
            r.march(u, tex, ref, rdep)
            cuda.cuda.synchronize()
            e = mm.metrics.frame_errors(rgba.cpu().numpy(), ref.cpu().numpy(), dep.cpu().numpy(), rdep.cpu().numpy())
            assert e["rmse_255"] < 0.05 and e["frac_over_4"] < 1e-3, (tw, grab, w, h, e)


def test_graph_replay_takes_new_uniforms(cuda, env):
    import marshmallow as mm
    tex, r = env
    a = [(200, 100, mm.scene.uniforms(200, 100, yaw=0.0, pitch=15.0))]
    b = [(200, 100, mm.scene.uniforms(200, 100, yaw=120.0, pitch=10.0, sun_elevation=60.0))]
    outs = _outputs(cuda, a)
    import marshmallow.lib as L
    for sched in (L.BATCH_BLOCKS, L.BATCH_GRAPH, L.BATCH_PERSISTENT):
        r.march_batch(a, tex, outs, schedule=sched)
        first = outs[0][0].cpu().numpy()
        r.march_batch(b, tex, outs, schedule=sched)  # same shape and options: the graph is replayed/updated
        second = outs[0][0].cpu().numpy()
        ref = cuda.zeros((100, 200, 4), device="cuda")
        r.march(b[0][2], tex, ref)
        cuda.cuda.synchronize()
        assert not np.array_equal(first, second)
        assert mm.metrics.frame_errors(second, ref.cpu().numpy())["rmse_255"] < 0.05


def test_uneven_batch_and_autotune(cuda, env):
    """The 70-view batch (cube map, 32 mid-size cameras, 32 4K cameras): one launch vs one launch per
    view, and the autotuner's pick."""
    import marshmallow as mm
    tex, r = env
    views = mm.scene.batch_views(seed=0)
    assert len(views) == 70
    outs = _outputs(cuda, views)
    arr = r.march_batch(views, tex, outs)
    best, table = r.autotune_batch(arr, len(views), tex)
    cuda.cuda.synchronize()
    ev = [cuda.cuda.Event(enable_timing=True) for _ in range(4)]
    ev[0].record()
    r.march_batch(views, tex, outs, warp_tile_w=best.warp_tile_w, tiles_per_grab=best.tiles_per_grab,
                  schedule=best.schedule)
    ev[1].record()
    for (w, h, u), (rgba, dep) in zip(views, outs):
        r.march(u, tex, rgba, dep)
    ev[2].record()
    cuda.cuda.synchronize()
    t_batch, t_seq = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    rays = sum(w * h for w, h, _ in views)
    print("\n70 views, %.1f Mrays: batch %.2f ms (%.0f Mrays/s, schedule %d, warp tile %d, grab %d) vs per-view %.2f ms"
          % (rays / 1e6, t_batch, rays / t_batch / 1e3, best.schedule, best.warp_tile_w, best.tiles_per_grab, t_seq))
    print("autotune table (ms; persistent: rows warp_tile_w 4/8/16/32, cols grab 1/2/4/8/16; then blocks):")
    for i in range(4):
        print("  " + " ".join("%8.2f" % v for v in table[5 * i:5 * i + 5]))
    print("  blocks %8.2f   graph %8.2f" % (table[20], table[21]))
    assert best.warp_tile_w in (4, 8, 16, 32) and 1 <= best.tiles_per_grab <= 16
    assert all(v > 0 for v in table)


def test_batch_fp16_and_surrogate_equal_single_views(cuda, mmlib, env):
    # config[4]'s batch: FP16 density and the learned sun cone, in the graph schedule.  FP16 views
    # are the single-view launches themselves (identical bytes); surrogate views add their deferred
    # terms with atomics, whose order differs from run to run (last-bit differences only).
    import ctypes as C
    import marshmallow as mm
    import marshmallow.lib as L
    from gpu_util import stream_ptr
    tex, r = env
    sp = stream_ptr(cuda)
    per = 1 << 16
    X = cuda.empty((2 * per, 16), dtype=cuda.bfloat16, device="cuda")
    T = cuda.empty(2 * per, dtype=cuda.float32, device="cuda")
    n = C.c_int()
    assert mmlib.mm_surrogate_generate(1, 2, per, 150000.0, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()),
                                       C.byref(n), sp) == 0
    net = C.c_void_p()
    assert mmlib.mm_mlp_create(5, C.byref(net)) == 0
    assert mmlib.mm_mlp_train(net, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()), n.value, 16384, 32, 3e-3,
                              None, sp) == 0
    views = mm.scene.cubemap_views(96) + [(320, 180, mm.scene.uniforms(320, 180, yaw=40.0, pitch=20.0)),
                                         (200, 120, mm.scene.uniforms(200, 120, sun_elevation=-8.0))]
    night = mm.render.Textures.from_arrays({"night_sky": np.full((32, 64, 4), 90, np.uint8)})
    tex.handles["night_sky"] = night.handles["night_sky"]
    tex.set_density_format(L.FORMAT_FP16)
    try:
        for sur in (None, net.value):
            outs = _outputs(cuda, views)
            r.march_batch(views, tex, outs, density_format=L.FORMAT_FP16, surrogate=sur)
            cuda.cuda.synchronize()
            for (w, h, u), (rgba, dep) in zip(views, outs):
                ref = cuda.zeros((h, w, 4), device="cuda")
                rdep = cuda.zeros((h, w), device="cuda")
                r.march(u, tex, ref, rdep, density_format=L.FORMAT_FP16, surrogate=sur)
                cuda.cuda.synchronize()
                a, b = rgba.cpu().numpy(), ref.cpu().numpy()
                if sur is None:
                    assert np.array_equal(a, b), (w, h)
                else:
                    assert np.allclose(a, b, rtol=1e-4, atol=1e-6), (w, h, float(np.abs(a - b).max()))
                assert np.array_equal(dep.cpu().numpy(), rdep.cpu().numpy()), (w, h)
    finally:
        tex.set_density_format(L.FORMAT_UNORM8)
        mmlib.mm_mlp_destroy(net)
        del tex.handles["night_sky"]
        night.close()
