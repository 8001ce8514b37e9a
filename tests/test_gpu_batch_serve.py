"""Batched and served forms: every view in a mixed batch, and every request
served in a mix, must equal the same view rendered alone by the plain
per-frame path (visibility bit-exact, colour identical)."""
import numpy as np
import pytest

import scenes
import swr

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_scenes():
    a = swr.Scene(scenes.small_scene(seed=3))
    b = swr.Scene(scenes.stress_scene(seed=9, triangles=40_000, width=640, height=480, n_textures=2, tex_size=128,
                                      cube_size=16, voxel=32, specular_samples=8, brdf_lut_size=32)[0])
    yield a, b
    a.close()
    b.close()


def sphere_cameras(scene, n, sizes, seed=0):
    rng = np.random.default_rng(seed)
    info = scene.info()
    c = np.array(info.bounds_center[:], np.float64)
    d = float(info.bounds_diagonal)
    out = []
    for i in range(n):
        w, h = sizes[i % len(sizes)]
        u = rng.normal(size=3)
        u /= np.linalg.norm(u)
        r = d * rng.uniform(0.6, 1.6)
        pos = c + u * r
        cam = swr.make_camera(tuple(map(float, pos)), tuple(map(float, c)), np.pi / 3, w, h, float(2 * d + r))
        out.append((cam, w, h))
    return out


def alone(scene, cam, w, h):
    r = swr.Renderer(w, h)
    r.render(scene, cam)
    out = r.blit(), r.visbuffer()
    r.close()
    return out


@pytest.mark.parametrize("tile,graph,fused", [(64, False, False), (32, True, False), (32, False, True),
                                              (16, False, False)])
def test_batch_views_equal_plain(two_scenes, tile, graph, fused):
    sizes = [(320, 240), (160, 96), (257, 131), (64, 64)]
    items = []
    for k, sc in enumerate(two_scenes):
        for cam, w, h in sphere_cameras(sc, 5, sizes, seed=k):
            items.append((sc, cam, w, h))
    b = swr.Batch(sched_tile=tile, use_graph=graph, fused_shade=fused)
    arr = swr.Batch.views([(sc, cam, w, h, 2.0, swr.RSQRT_AARCH64) for sc, cam, w, h in items])
    for rep in range(2):  # the second run replays the captured graph
        b.render(arr)
        b.sync()
        for i, (sc, cam, w, h) in enumerate(items):
            rgba, vis = b.output(i, w, h)
            ref_rgba, ref_vis = alone(sc, cam, w, h)
            assert np.array_equal(vis, ref_vis), "view %d" % i
            rows = h & ~1
            assert np.array_equal(rgba[:rows], ref_rgba[:rows]), "view %d" % i
    b.close()


def test_autotune_picks_a_tile(two_scenes):
    items = [(two_scenes[1], cam, w, h, 2.0, swr.RSQRT_AARCH64)
             for cam, w, h in sphere_cameras(two_scenes[1], 4, [(320, 240)], seed=4)]
    b = swr.Batch()
    arr = swr.Batch.views(items)
    tile, ms = b.autotune(arr)
    assert tile in (8, 16, 32, 64) and ms > 0
    t = b.tuning(arr)
    assert t["tuned"] == 1 and t["sched_tile"] == tile
    assert t["raster_ctas_per_sm"] in (0, 1, 2) and t["bin_capacity"] > 0
    # The tuned configuration (its raster grid, its starting bin capacity)
    # renders every view as the plain path does.
    b.render(arr)
    b.sync()
    for i, (sc, cam, w, h, _, _) in enumerate(items):
        rgba, vis = b.output(i, w, h)
        ref_rgba, ref_vis = alone(sc, cam, w, h)
        assert np.array_equal(vis, ref_vis), "view %d" % i
        assert np.array_equal(rgba[:h & ~1], ref_rgba[:h & ~1]), "view %d" % i
    b.close()


@pytest.mark.parametrize("cap", [1, 2])
def test_raster_ctas_per_sm_equal_plain(two_scenes, cap):
    # The persistent raster with fewer CTAs per SM than fit (autotuner trials).
    sc = two_scenes[1]
    items = [(sc, cam, w, h) for cam, w, h in sphere_cameras(sc, 3, [(320, 240), (200, 130)], seed=6)]
    for tile in (64, 16):
        b = swr.Batch(sched_tile=tile, raster_ctas_per_sm=cap)
        arr = swr.Batch.views([(s, cam, w, h, 2.0, swr.RSQRT_AARCH64) for s, cam, w, h in items])
        b.render(arr)
        b.sync()
        for i, (s, cam, w, h) in enumerate(items):
            rgba, vis = b.output(i, w, h)
            ref_rgba, ref_vis = alone(s, cam, w, h)
            assert np.array_equal(vis, ref_vis), "tile %d view %d" % (tile, i)
        b.close()


def test_served_results_equal_alone(two_scenes):
    srv = swr.Server(memory_budget=8 << 30, max_batch_views=16, inflight=2)
    ids = [srv.add_scene(s) for s in two_scenes]
    reqs = {}
    sizes = [(320, 240), (200, 120), (96, 64)]
    for k, sc in enumerate(two_scenes):
        for cam, w, h in sphere_cameras(sc, 12, sizes, seed=10 + k):
            t = srv.submit(ids[k], cam, w, h, 2.0, tag=len(reqs))
            assert t is not None
            reqs[t] = (sc, cam, w, h)
    got = {}
    for _ in range(2000):
        for c in srv.poll(64, wait_ms=20):
            assert c.status == 0
            sc, cam, w, h = reqs[c.ticket]
            rgba = swr.copy_device_to_host(c.rgba8, w * h * 4, np.zeros((h, w), np.uint32))
            vis = swr.copy_device_to_host(c.vis, w * h * 8, np.zeros((h, w), np.uint64))
            got[c.ticket] = (rgba, vis, c.batch_views)
            srv.release(c.ticket)
        if len(got) == len(reqs):
            break
    assert len(got) == len(reqs)
    assert max(v[2] for v in got.values()) > 1  # requests really were batched
    for t, (sc, cam, w, h) in reqs.items():
        ref_rgba, ref_vis = alone(sc, cam, w, h)
        rgba, vis, _ = got[t]
        assert np.array_equal(vis, ref_vis)
        assert np.array_equal(rgba[:h & ~1], ref_rgba[:h & ~1])
    st = srv.stats()
    assert st.completed == len(reqs) and st.device_bytes <= st.budget
    srv.close()


def test_server_admission_budget(two_scenes):
    srv = swr.Server(memory_budget=1 << 20)
    with pytest.raises(swr.SwrError) as e:
        srv.add_scene(two_scenes[1])
    assert e.value.status == swr.SWR_BUSY
    srv.close()
