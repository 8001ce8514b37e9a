"""Blit target written by the shading pass (swr_renderer_set_blit_target):
the pixels a frame writes straight into host memory equal the copying blit's
(which the parity tests hold against the oracle), rows and padding outside
the frame stay untouched, and a blit elsewhere still copies."""
import numpy as np
import pytest

import oracle
import scenes
import swr

pytestmark = pytest.mark.gpu

SENTINEL = 0x5A5A5A5A


def pinned(rows, cols):
    torch = pytest.importorskip("torch")
    t = torch.full((rows, cols), SENTINEL, dtype=torch.int32, pin_memory=True)
    return t, t.numpy().view(np.uint32)


@pytest.fixture(scope="module")
def small():
    s = swr.Scene(scenes.small_scene(seed=3))
    yield s
    s.close()


@pytest.fixture(scope="module")
def trans():
    s = swr.Scene(scenes.translucent_scene())
    yield s
    s.close()


def frame_via_target(scene, w, h, stride=0, dt=0.0, frames=1):
    cam = swr.make_camera(*scenes.default_camera_params(scene.info(), w, h))
    r = swr.Renderer(w, h)
    cols = stride if stride else w
    t, arr = pinned(h, cols)
    r.set_blit_target(arr.ctypes.data, stride, keep=t)
    for _ in range(frames):
        r.render(scene, cam, dt)
        swr.check(swr.lib().swr_blit(r.handle, arr.ctypes.data, stride, None))
    copied = r.blit()
    r.close()
    return arr, copied, cam


@pytest.mark.parametrize("w,h", [(320, 200), (97, 61), (1, 1)])
def test_target_equals_copy(small, w, h):
    arr, copied, _ = frame_via_target(small, w, h)
    rows = h & ~1
    np.testing.assert_array_equal(arr[:rows, :w], copied[:rows])
    # An odd height leaves the last row alone (chunks_exact, src/renderer.rs:298).
    assert (arr[rows:] == SENTINEL).all()


def test_target_matches_oracle(small):
    w, h = 256, 160
    arr, _, cam = frame_via_target(small, w, h)
    orgba, _, _, _ = oracle.render(small, cam, w, h, threads=1)
    d = np.abs(arr[:h].view(np.uint8).astype(np.int32) - orgba[:h].view(np.uint8).astype(np.int32))
    assert d.max() <= 1


def test_target_row_stride(small):
    w, h, stride = 130, 34, 141
    arr, copied, _ = frame_via_target(small, w, h, stride=stride)
    np.testing.assert_array_equal(arr[:, :w], copied)
    assert (arr[:, w:] == SENTINEL).all()


def test_target_exposure_step_and_translucent(small, trans):
    # dt > 0 and translucent views write the frame from the resolve pass.
    for scene in (small, trans):
        arr, copied, _ = frame_via_target(scene, 192, 128, dt=0.25, frames=3)
        np.testing.assert_array_equal(arr, copied)


def test_detach_and_other_destination(small):
    w, h = 64, 48
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), w, h))
    r = swr.Renderer(w, h)
    t, arr = pinned(h, w)
    r.set_blit_target(arr.ctypes.data, 0, keep=t)
    r.render(small, cam)
    other = r.blit()  # not the target: copied from the device, after the frame
    np.testing.assert_array_equal(other, arr)
    # Detached: the next frame leaves the old target alone until a blit copies into it.
    arr[:] = SENTINEL
    r.set_blit_target(None)
    r.render(small, cam)
    r.sync()
    assert (arr == SENTINEL).all()
    swr.check(swr.lib().swr_blit(r.handle, arr.ctypes.data, 0, None))
    np.testing.assert_array_equal(arr, other)
    r.close()


def test_pageable_target_accepted_or_refused(small):
    # Plain host memory is a valid target only where the GPU reads the host
    # page tables; elsewhere the call refuses it and nothing changes.
    w, h = 64, 48
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), w, h))
    r = swr.Renderer(w, h)
    arr = np.full((h, w), SENTINEL, np.uint32)
    try:
        r.set_blit_target(arr.ctypes.data, 0, keep=arr)
    except swr.SwrError as e:
        assert e.status == swr.SWR_INVALID_ARG
        r.close()
        return
    r.render(small, cam)
    swr.check(swr.lib().swr_blit(r.handle, arr.ctypes.data, 0, None))
    np.testing.assert_array_equal(arr, r.blit())
    r.close()


def test_target_rejects_short_stride(small):
    r = swr.Renderer(64, 48)
    t, arr = pinned(48, 64)
    with pytest.raises(swr.SwrError):
        r.set_blit_target(arr.ctypes.data, 32, keep=t)
    r.close()
