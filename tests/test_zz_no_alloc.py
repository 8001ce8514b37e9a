"""swr_render_frame_noalloc, the allocation-free frame for callers that cannot
allocate device memory while rendering (code under CUDA stream capture,
processes whose device memory belongs to another allocator, real-time loops).

Its output must equal the regular entry point's (swr_render_frame + blit +
read_visbuffer) on two calls in a row: the fixed scratch array it uses keeps
the previous call's contents, so the second call checks that everything that
must start at zero is cleared. Collected last so that a failure here does not
stop the rest of a `-x` run.
"""
import ctypes as C

import numpy as np
import pytest

import scenes
import swr

pytestmark = pytest.mark.gpu


def test_noalloc_matches_regular_frame_twice():
    torch = pytest.importorskip("torch")
    L = swr.lib()
    scene = swr.Scene(scenes.small_scene(seed=5))
    W, H = 320, 200
    cam = swr.make_camera(*scenes.default_camera_params(scene.info(), W, H))
    r = swr.Renderer(W, H)
    r.render(scene, cam, 0.0)
    ref_rgba = r.blit()
    ref_vis = r.visbuffer()
    r.close()
    rgba = torch.zeros((H, W), dtype=torch.int32, device="cuda")
    vis = torch.zeros((H, W), dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        rgba.fill_(0x12345678)
        vis.fill_(7)
        st = L.swr_render_frame_noalloc(scene.handle, C.byref(cam), W, H, 2.0, swr.RSQRT_AARCH64,
                                        C.c_void_p(rgba.data_ptr()), C.c_void_p(vis.data_ptr()), C.c_void_p(stream))
        assert st == swr.SWR_OK, L.swr_last_error()
        torch.cuda.synchronize()
        got_vis = vis.cpu().numpy().view(np.uint64)
        got_rgba = rgba.cpu().numpy().view(np.uint32)
        assert np.array_equal(got_vis, ref_vis), "call %d: visibility differs in %d pixels" % (
            call, int((got_vis != ref_vis).sum()))
        d = np.abs(got_rgba.view(np.uint8).astype(np.int32) - ref_rgba.view(np.uint8).astype(np.int32))
        assert d.max() <= 1, "call %d: colour differs by %d/255" % (call, d.max())
    scene.close()


def test_noalloc_rejects_oversized_frames():
    L = swr.lib()
    scene = swr.Scene(scenes.small_scene(seed=5))
    cam = swr.make_camera(*scenes.default_camera_params(scene.info(), 1024, 600))
    dummy = C.c_void_p(16)
    st = L.swr_render_frame_noalloc(scene.handle, C.byref(cam), 1024, 600, 2.0, 1, dummy, dummy, None)
    assert st == swr.SWR_INVALID_ARG
    assert b"512" in L.swr_last_error()
    scene.close()
