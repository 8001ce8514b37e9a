"""Translucent forward path (render_tile's sorted translucent packets,
src/tilerasterizer.rs:92-101, TranslucentForwardShader, src/shader.rs:66-76)
against the oracle: visibility bit-exact, colour within 1/255, tile
luminance bit-exact."""
import numpy as np
import pytest

import oracle
import scenes
import swr
from test_gpu_parity import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trans():
    s = swr.Scene(scenes.translucent_scene())
    yield s
    s.close()


@pytest.mark.parametrize("tile", [8, 16, 64])
def test_translucent_scene(trans, tile):
    cam = swr.make_camera(*scenes.default_camera_params(trans.info(), 320, 200))
    compare(trans, cam, 320, 200, sched_tile=tile)


def test_translucent_odd_size_close_camera(trans):
    # Camera inside the translucent plane's extent, odd frame size: partial
    # tiles, off-screen centre quads, clipped translucent triangles.
    c = np.array(trans.info().bounds_center[:])
    cam = swr.make_camera((float(c[0]) + 0.5, float(c[1]) + 0.3, float(c[2]) + 4.0),
                          (float(c[0]), float(c[1]), float(c[2])), 1.1, 193, 131, 40.0)
    compare(trans, cam, 193, 131)


def test_translucent_with_exposure_step(trans):
    cam = swr.make_camera(*scenes.default_camera_params(trans.info(), 256, 160))
    compare(trans, cam, 256, 160, dt=0.25)


def test_translucent_sort_overflow_retries_smaller_tile():
    # Two layers of 8,192 translucent triangles within about 60 pixels: more
    # than one 64-px (or 32-px) tile's translucent sort holds, so the frame is
    # rendered again with smaller scheduling tiles until every tile fits.
    sd = scenes.translucent_scene(count=2)
    GP, GUV, GF = scenes.grid(64, 64)
    sd["materials"].append({"base_color_factor": (0.8, 0.5, 0.3, 1.0), "metallic": 0.0, "roughness": 0.5,
                            "has_transmission": 1, "transmission": 0.6})
    mi = len(sd["materials"]) - 1
    # Two layers of the same dense grid, slightly apart, facing the camera.
    for z in (0.0, 0.05):
        sd["meshes"].append([{"positions": GP + np.array([0, 0, z], np.float32),
                              "normals": np.tile(np.array([[0, 0, 1]], np.float32), (len(GP), 1)),
                              "texcoords": GUV, "indices": GF, "material": mi}])
        w = scenes.translate_scale(np.array([0.0, 0.0, 3.0], np.float32), 3.0)
        sd["nodes"].append({"world": w, "local": w, "mesh": len(sd["meshes"]) - 1})
    s = swr.Scene(sd)
    cam = swr.make_camera((0.0, 0.0, 9.0), (0.0, 0.0, 0.0), 1.0, 160, 128, 40.0)
    r = swr.Renderer(160, 128, sched_tile=64)
    r.render(s, cam, 0.0)
    rgba = r.blit()
    vis = r.visbuffer()
    st = r.stats()
    assert st.overflow_retries >= 1 and st.sched_tile < 64
    orgba, ovis, otl, res = oracle.render(s, cam, 160, 128, threads=1)
    assert int((vis != ovis).sum()) == 0
    d = np.abs(rgba.view(np.uint8).astype(np.int32) - orgba.view(np.uint8).astype(np.int32))
    assert d.max() <= 1
    r.close()
    s.close()


def test_batched_translucent_views_equal_plain(trans):
    # Translucent views in a batch (engine-owned colour, fused resolve) give
    # the plain renderer's frames.
    info = trans.info()
    sizes = [(320, 200), (160, 96), (97, 65)]
    cams = [swr.make_camera(*scenes.default_camera_params(info, w, h)) for (w, h) in sizes]
    b = swr.Batch(use_graph=True)
    arr = swr.Batch.views([(trans, cams[i], w, h, 2.0, swr.RSQRT_AARCH64) for i, (w, h) in enumerate(sizes)])
    b.render(arr)
    b.sync()
    for i, (w, h) in enumerate(sizes):
        brgba, bvis = b.output(i, w, h)
        r = swr.Renderer(w, h)
        r.render(trans, cams[i], 0.0)
        np.testing.assert_array_equal(bvis, r.visbuffer())
        rows = h & ~1
        np.testing.assert_array_equal(brgba[:rows], r.blit()[:rows])
        r.close()
    b.close()
