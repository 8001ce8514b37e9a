"""Device draw-list build (render_scene's front half, src/renderer.rs:201-210
and 357-420) against the oracle, whose draw list follows the reference's
host loop: scenes of more than 256 nodes (several counting blocks, the last
CTA's scan and k_draw_emit), the 256-slot boundary, frustum-culled and
intersecting nodes, multi-primitive meshes with translucent primitives, and
batches whose views together pass 256 node slots."""
import numpy as np
import pytest

import scenes
import swr
from test_gpu_parity import compare
from test_gpu_batch_serve import alone

pytestmark = pytest.mark.gpu


def many_spheres(count, seed=21):
    return swr.Scene(scenes.spheres_scene(seed=seed, count=count, subdiv=1, box=12.0, radius=(0.3, 1.0), tex_size=64,
                                          cube_size=16, voxel=32, specular_samples=16, brdf_lut_size=32))


@pytest.mark.parametrize("count", [255, 256, 257, 700])
def test_node_counts_around_one_block(count):
    s = many_spheres(count)
    cam = swr.make_camera(*scenes.default_camera_params(s.info(), 256, 160))
    compare(s, cam, 256, 160)
    s.close()


def test_camera_inside_node_cloud():
    # Nodes behind the camera, beside the frustum and cut by its planes.
    s = many_spheres(700, seed=22)
    cam = swr.make_camera((0.5, 0.25, 0.0), (6.0, 1.0, -9.0), 1.2, 240, 160, 60.0)
    compare(s, cam, 240, 160)
    s.close()


def replicated_translucent(copies=30, spacing=20.0):
    sd = scenes.translucent_scene()
    nodes = []
    for k in range(copies):
        off = np.array([(k % 6) * spacing, (k // 6) * spacing, 0.0], np.float32)
        for n in sd["nodes"]:
            w = np.array(n["world"], np.float32).copy()
            w[12:15] += off  # column-major translation
            nodes.append({"world": w, "local": w.copy(), "mesh": n["mesh"]})
    sd["nodes"] = nodes
    return swr.Scene(sd)


def test_translucent_meshes_over_many_nodes():
    s = replicated_translucent()
    assert s.info().node_count > 256
    cam = swr.make_camera(*scenes.default_camera_params(s.info(), 320, 200))
    compare(s, cam, 320, 200, sched_tile=16)
    s.close()


def test_batch_views_over_many_slots():
    big = many_spheres(700, seed=23)
    small = swr.Scene(scenes.small_scene(seed=3))
    items = []
    for sc, n in ((big, 3), (small, 2), (big, 1)):
        info = sc.info()
        for i in range(n):
            w, h = (200 + 24 * i, 120 + 16 * i)
            c = np.array(info.bounds_center[:], np.float64)
            d = float(info.bounds_diagonal)
            pos = c + np.array([0.3 * i, 0.2, 0.6 + 0.2 * i]) * d
            cam = swr.make_camera(tuple(map(float, pos)), tuple(map(float, c)), np.pi / 3, w, h, float(2.5 * d))
            items.append((sc, cam, w, h))
    b = swr.Batch(sched_tile=32)
    b.render(swr.Batch.views([(sc, cam, w, h, 2.0, swr.RSQRT_AARCH64) for sc, cam, w, h in items]))
    b.sync()
    for i, (sc, cam, w, h) in enumerate(items):
        rgba, vis = b.output(i, w, h)
        ref_rgba, ref_vis = alone(sc, cam, w, h)
        assert np.array_equal(vis, ref_vis), "view %d" % i
        assert np.array_equal(rgba[:h & ~1], ref_rgba[:h & ~1]), "view %d" % i
    b.close()
    big.close()
    small.close()


def instanced_grid(n_side=12, depth=16, subdiv=4, seed=24):
    """One icosphere mesh instanced on a grid of n_side x n_side x depth nodes:
    11.8M triangles drawn (more than the 10.5M record slots first sized from
    the scene's bound) from a scene of one small mesh."""
    rng = np.random.default_rng(seed)
    P, F = scenes.icosphere(subdiv)
    UV = scenes.spherical_uv(P)
    nodes = []
    for k in range(depth):
        for j in range(n_side):
            for i in range(n_side):
                w = scenes.translate_scale(np.array([i * 3.0, j * 3.0, -k * 3.0], np.float32), 1.0)
                nodes.append({"world": w, "local": w, "mesh": 0})
    sd = {"meshes": [[{"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": 0}]],
          "nodes": nodes,
          "materials": [{"base_color_factor": (0.8, 0.7, 0.6, 1.0), "metallic": 0.3, "roughness": 0.6,
                         "base_color": (0, scenes.WRAP_REPEAT, scenes.WRAP_REPEAT)}],
          "textures": [scenes.noise_texture(rng, 64)], "cubemap": scenes.cubemap_faces(rng, 16),
          "cubemap_face_size": 16, "voxel_grid_size": 32, "specular_samples": 8, "brdf_lut_size": 32}
    return swr.Scene(sd)


def test_frame_past_initial_record_slots_is_rendered_again():
    s = instanced_grid()
    info = s.info()
    assert info.triangle_count > (8 << 20) * 5 // 4 + 16
    w, h = 96, 64
    cam = swr.make_camera(*scenes.default_camera_params(info, w, h))
    r = swr.Renderer(w, h)
    r.render(s, cam)
    rgba1, vis1 = r.blit(), r.visbuffer()
    st = r.stats()
    assert st.triangles_in == info.triangle_count
    assert st.overflow_retries >= 1  # the first frame found more triangles than slots
    r.render(s, cam)
    rgba2, vis2 = r.blit(), r.visbuffer()
    assert r.stats().overflow_retries == st.overflow_retries  # grown buffers hold the second frame
    np.testing.assert_array_equal(vis1, vis2)
    np.testing.assert_array_equal(rgba1, rgba2)
    assert (vis1 != np.uint64(2**64 - 1)).sum() > w * h // 4
    r.close()
    s.close()
