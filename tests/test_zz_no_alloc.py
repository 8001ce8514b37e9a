"""swr_render_frame_noalloc, the allocation-free frame for callers that cannot
allocate device memory while rendering (processes whose device memory belongs
to another allocator or a fixed budget, real-time loops that cannot afford a
cudaMalloc that may synchronize the device).

Its output must equal the regular entry point's (swr_render_frame + blit +
read_visbuffer) on two calls in a row: the fixed scratch array it uses keeps
the previous call's contents, so the second call checks that everything that
must start at zero is cleared. Frames at the size limit (512x512) and with an
odd height (the last row stays untouched) are covered, so are a scene within
the host-side limits whose bins overflow the fixed capacity on the device
(SWR_OVERFLOW, then a correct frame on the next call) and each limit's
rejection. Collected last so that a failure here does not stop the rest of a
`-x` run.
"""
import ctypes as C

import numpy as np
import pytest

import scenes
import swr

pytestmark = pytest.mark.gpu

FILL_RGBA = 0x12345678


def regular(scene, cam, w, h):
    r = swr.Renderer(w, h)
    r.render(scene, cam, 0.0)
    rgba, vis = r.blit(), r.visbuffer()
    r.close()
    return rgba, vis


def noalloc(torch, scene, cam, w, h):
    L = swr.lib()
    rgba = torch.full((h, w), FILL_RGBA, dtype=torch.int32, device="cuda")
    vis = torch.full((h, w), 7, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    st = L.swr_render_frame_noalloc(scene.handle, C.byref(cam), w, h, 2.0, swr.RSQRT_AARCH64,
                                    C.c_void_p(rgba.data_ptr()), C.c_void_p(vis.data_ptr()), C.c_void_p(stream))
    torch.cuda.synchronize()
    return st, rgba.cpu().numpy().view(np.uint32), vis.cpu().numpy().view(np.uint64)


def assert_same(got, ref, h, what):
    got_rgba, got_vis = got
    ref_rgba, ref_vis = ref
    assert np.array_equal(got_vis, ref_vis), "%s: visibility differs in %d pixels" % (
        what, int((got_vis != ref_vis).sum()))
    rows = h & ~1
    d = np.abs(got_rgba[:rows].view(np.uint8).astype(np.int32) - ref_rgba[:rows].view(np.uint8).astype(np.int32))
    assert d.max() <= 1, "%s: colour differs by %d/255" % (what, d.max())
    if h & 1:
        assert (got_rgba[rows:] == FILL_RGBA).all(), "%s: the odd last row was written" % what


@pytest.mark.parametrize("w,h", [(320, 200), (512, 512), (301, 211)])
def test_noalloc_matches_regular_frame_twice(w, h):
    torch = pytest.importorskip("torch")
    L = swr.lib()
    scene = swr.Scene(scenes.small_scene(seed=5))
    cam = swr.make_camera(*scenes.default_camera_params(scene.info(), w, h))
    ref = regular(scene, cam, w, h)
    for call in range(2):
        st, rgba, vis = noalloc(torch, scene, cam, w, h)
        assert st == swr.SWR_OK, L.swr_last_error()
        assert_same((rgba, vis), ref, h, "%dx%d call %d" % (w, h, call))
    scene.close()


def stacked_quads(n=1200, half=2.75, step=0.001):
    """n camera-facing quads one behind the other: 2n triangles inside the
    frustum whose bounding boxes each touch most 64-px tiles of a 512x512
    view, far more (triangle, tile) pairs than the fixed bins hold."""
    rng = np.random.default_rng(2)
    P, UV, F = [], [], []
    for i in range(n):
        z = -i * step
        b = 4 * i
        P += [[-half, -half, z], [half, -half, z], [half, half, z], [-half, half, z]]
        UV += [[0, 0], [1, 0], [1, 1], [0, 1]]
        F += [b, b + 1, b + 2, b, b + 2, b + 3]
    eye = np.eye(4, dtype=np.float32).reshape(16)
    return {"meshes": [[{"positions": np.array(P, np.float32), "normals": None,
                         "texcoords": np.array(UV, np.float32), "indices": np.array(F, np.uint32), "material": 0}]],
            "nodes": [{"world": eye, "local": eye, "mesh": 0}],
            "materials": [{"metallic": 0.2, "roughness": 0.6, "base_color": (0, 0, 0)}],
            "textures": [scenes.noise_texture(rng, 16)], "cubemap": scenes.cubemap_faces(rng, 8),
            "cubemap_face_size": 8, "voxel_grid_size": 8, "specular_samples": 4, "brdf_lut_size": 8}


def test_noalloc_bin_overflow_then_a_correct_frame():
    torch = pytest.importorskip("torch")
    L = swr.lib()
    big = swr.Scene(stacked_quads())
    cam = swr.make_camera((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), np.pi / 3, 512, 512, 30.0)
    st, _, _ = noalloc(torch, big, cam, 512, 512)
    assert st == swr.SWR_OVERFLOW, L.swr_last_error()
    assert b"capacity" in L.swr_last_error()
    # The regular path renders the same frame (its bins grow).
    r = swr.Renderer(512, 512)
    r.render(big, cam, 0.0)
    r.sync()
    assert r.stats().bin_pairs > 65536
    r.close()
    # The next call, on a scene that fits, is exact.
    small = swr.Scene(scenes.small_scene(seed=5))
    cam2 = swr.make_camera(*scenes.default_camera_params(small.info(), 256, 192))
    st, rgba, vis = noalloc(torch, small, cam2, 256, 192)
    assert st == swr.SWR_OK, L.swr_last_error()
    assert_same((rgba, vis), regular(small, cam2, 256, 192), 192, "after overflow")
    big.close()
    small.close()


def one_mesh_scene(mesh_prims, nodes):
    rng = np.random.default_rng(4)
    return {"meshes": [mesh_prims], "nodes": nodes,
            "materials": [{"metallic": 0.2, "roughness": 0.6, "base_color": (0, 0, 0)}],
            "textures": [scenes.noise_texture(rng, 8)], "cubemap": scenes.cubemap_faces(rng, 8),
            "cubemap_face_size": 8, "voxel_grid_size": 8, "specular_samples": 4, "brdf_lut_size": 8}


def tiny_prim():
    return {"positions": np.array([[0, 0, 0], [0.01, 0, 0], [0, 0.01, 0]], np.float32), "normals": None,
            "texcoords": None, "indices": np.array([0, 1, 2], np.uint32), "material": 0}


def grid_nodes(n):
    out = []
    for i in range(n):
        w = scenes.translate_scale(np.array([(i % 64) * 0.05 - 1.6, (i // 64) * 0.05 - 1.6, 0.0], np.float32), 1.0)
        out.append({"world": w, "local": w, "mesh": 0})
    return out


def rejects(scene, w, h, text):
    L = swr.lib()
    cam = swr.make_camera(*scenes.default_camera_params(scene.info(), w, h))
    dummy = C.c_void_p(256)
    st = L.swr_render_frame_noalloc(scene.handle, C.byref(cam), w, h, 2.0, 1, dummy, dummy, None)
    assert st == swr.SWR_INVALID_ARG
    assert text in L.swr_last_error()


def test_noalloc_rejects_inputs_beyond_its_limits():
    small = swr.Scene(scenes.small_scene(seed=5))
    rejects(small, 1024, 600, b"512")
    rejects(small, 512, 513, b"512")
    small.close()
    # 20,480 visible triangles (one icosphere of subdivision 5).
    P, F = scenes.icosphere(5)
    many_tris = swr.Scene(one_mesh_scene([{"positions": P, "normals": None, "texcoords": None, "indices": F,
                                           "material": 0}], grid_nodes(1)))
    rejects(many_tris, 256, 256, b"16384")
    many_tris.close()
    # 2,100 nodes of a two-primitive mesh: 4,200 draws.
    many_draws = swr.Scene(one_mesh_scene([tiny_prim(), tiny_prim()], grid_nodes(2100)))
    rejects(many_draws, 256, 256, b"4096 draws")
    many_draws.close()
    many_nodes = swr.Scene(one_mesh_scene([tiny_prim()], grid_nodes(4097)))
    rejects(many_nodes, 256, 256, b"4096 nodes")
    many_nodes.close()
