"""GPU kernels vs the CPU oracle on seeded scenes: the visibility buffer must
be bit-exact and colour must stay within 1/255 per 8-bit channel (mean error
reported)."""
import numpy as np
import pytest

import oracle
import scenes
import swr

pytestmark = pytest.mark.gpu

TOL = 1  # max abs difference per 8-bit channel


def compare(scene, cam, w, h, **kw):
    mode = kw.get("rsqrt_mode", swr.RSQRT_AARCH64)
    r = swr.Renderer(w, h, rsqrt_mode=mode, sched_tile=kw.get("sched_tile", 64))
    r.render(scene, cam, kw.get("dt", 0.0))
    rgba = r.blit()
    vis = r.visbuffer()
    tl = r.tile_luminance()
    orgba, ovis, otl, res = oracle.render(scene, cam, w, h, rsqrt_mode=mode, threads=1, dt=kw.get("dt", 0.0))
    bad = int((vis != ovis).sum())
    assert bad == 0, "visibility differs in %d of %d pixels" % (bad, vis.size)
    rows = h & ~1
    if rows > 0:
        a = rgba[:rows].view(np.uint8).astype(np.int32)
        b = orgba[:rows].view(np.uint8).astype(np.int32)
        d = np.abs(a - b)
        print("max %d mean %.6f exact %.6f" % (d.max(), d.mean(), (d == 0).mean()))
        assert d.max() <= TOL
    np.testing.assert_array_equal(tl, otl)
    r.close()
    return rgba, vis


@pytest.fixture(scope="module")
def small():
    s = swr.Scene(scenes.small_scene(seed=3))
    yield s
    s.close()


@pytest.mark.parametrize("mode", [swr.RSQRT_AARCH64, swr.RSQRT_IEEE])
def test_small_default_camera(small, mode):
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), 320, 200))
    compare(small, cam, 320, 200, rsqrt_mode=mode)


@pytest.mark.parametrize("w,h", [(97, 61), (64, 64), (130, 33), (1, 1), (2, 3)])
def test_odd_sizes(small, w, h):
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), w, h))
    compare(small, cam, w, h)


@pytest.mark.parametrize("tile", [8, 16, 32, 64])
def test_sched_tiles_match(small, tile):
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), 256, 160))
    compare(small, cam, 256, 160, sched_tile=tile)


@pytest.fixture(scope="module")
def big_tris():
    s = swr.Scene(scenes.spheres_scene(seed=5, count=3, subdiv=0, box=3.0, radius=(1.5, 2.5), tex_size=64,
                                       cube_size=16, voxel=32, specular_samples=16, brdf_lut_size=32))
    yield s
    s.close()


@pytest.mark.parametrize("tile", [16, 64])
@pytest.mark.parametrize("dist", [4.0, 6.0])
def test_large_triangles_sequential_regions(big_tris, tile, dist):
    # Icosahedra seen from close by: triangles hundreds of pixels across, so
    # edge values leave the exact-integer range (2^24) inside many 16-px
    # blocks and those regions replay the reference's sequential additions
    # (about half of the quads at distance 4, a fifth at 6).
    c = np.array(big_tris.info().bounds_center[:])
    cam = swr.make_camera((float(c[0]), float(c[1]) + 0.5, float(c[2]) + dist), (float(c[0]), float(c[1]), float(c[2])),
                          1.0, 1024, 768, 100.0)
    compare(big_tris, cam, 1024, 768, sched_tile=tile)


def test_auto_sched_tile(small):
    # sched_tile 0: the largest tile that still gives >= 8 tiles per SM.
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), 320, 200))
    for (w, h) in [(3840, 2160), (320, 200)]:
        r = swr.Renderer(w, h)
        r.render(small, cam, 0.0)
        r.sync()
        st = r.stats().sched_tile
        r.close()
        assert st in (16, 32, 64)
        if (w, h) == (320, 200):
            assert st == 16


def test_camera_inside_scene_clips(small):
    # Camera among the spheres: primitives straddle the near and side planes.
    info = small.info()
    c = np.array(info.bounds_center[:])
    cam = swr.make_camera((float(c[0]) + 0.3, float(c[1]) + 0.2, float(c[2]) + 0.5),
                          (float(c[0]) + 3.0, float(c[1]) - 1.0, float(c[2]) - 4.0), 1.2, 240, 160, 40.0)
    compare(small, cam, 240, 160)


def test_c1_full_frame():
    s = swr.Scene(scenes.spheres_scene())
    cam = swr.make_camera(*scenes.default_camera_params(s.info(), 1280, 720))
    compare(s, cam, 1280, 720)
    s.close()


def test_c1_close_camera_clipping():
    s = swr.Scene(scenes.spheres_scene())
    cam = swr.make_camera((0.0, 0.0, 6.0), (0.0, 0.0, -1.0), np.pi / 3, 1280, 720, 60.0)
    compare(s, cam, 1280, 720)
    s.close()


def test_dt_exposure_path(small):
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), 320, 200))
    compare(small, cam, 320, 200, dt=0.5)


def test_repeat_frames_identical(small):
    cam = swr.make_camera(*scenes.default_camera_params(small.info(), 320, 200))
    r = swr.Renderer(320, 200)
    r.render(small, cam)
    a = r.blit().copy(), r.visbuffer().copy()
    r.render(small, cam)
    b = r.blit(), r.visbuffer()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    r.close()


def quad_stack_scene(n=120, dup_every=10):
    """n screen-covering 2-triangle quads at increasing depth; every
    `dup_every`-th quad is duplicated exactly (same node transform), so the
    two copies tie on depth at every pixel and the later node must win."""
    rng = np.random.default_rng(11)
    P, UV, F = scenes.grid(1, 1)
    tex = scenes.noise_texture(rng, 32)
    meshes, nodes, mats = [], [], []
    for i in range(n):
        mats.append({"metallic": float(rng.random()), "roughness": float(rng.random()), "base_color": (0, 0, 0)})
        meshes.append([{"positions": P, "normals": None, "texcoords": UV, "indices": F, "material": i}])
        z = -2.0 - 0.05 * i
        m = np.eye(4, dtype=np.float32)
        m[0, 0] = m[1, 1] = 8.0 + 0.01 * i
        m[:3, 3] = (0.01 * i, -0.02 * i, z)
        w = m.T.reshape(16).copy()
        nodes.append({"world": w, "local": w, "mesh": i})
        if i % dup_every == 0:
            nodes.append({"world": w, "local": w, "mesh": i})
    return {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": [tex],
            "cubemap": scenes.cubemap_faces(rng, 8), "cubemap_face_size": 8, "voxel_grid_size": 16,
            "specular_samples": 8, "brdf_lut_size": 16}


@pytest.mark.parametrize("tile", [64, 16])
def test_overlapping_large_quads_and_depth_ties(tile):
    s = swr.Scene(quad_stack_scene())
    cam = swr.make_camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 1.0, 192, 128, 40.0)
    rgba, vis = compare(s, cam, 192, 128, sched_tile=tile)
    # The nearest quad is node 0 (triangles 0, 1) with an exact duplicate,
    # node 1 (triangles 2, 3): equal depth everywhere, and the duplicate comes
    # later in the canonical order, so only its triangles are visible.
    covered = vis[vis != np.uint64(2 ** 64 - 1)] >> np.uint64(3)
    assert covered.size > 0 and set(np.unique(covered).tolist()) == {2, 3}
    s.close()


def tie_across_rounds_scene(n=80):
    """n screen-covering quads front to back, then one wide quad in the plane of
    the nearest one. Every vertex of the two lies in one plane facing the
    camera, so they tie on depth at every pixel; the wide quad's bounding
    sphere sits far to the side, so it sorts after every other quad and reaches
    each tile rounds after the quad it ties. Being later in the canonical
    order it must win wherever it covers, so occlusion culling has to keep
    packets that only tie the depths already held."""
    rng = np.random.default_rng(5)
    P, UV, F = scenes.grid(1, 1)
    tex = scenes.noise_texture(rng, 32)
    meshes, nodes, mats = [], [], []

    def world(sx, sy, t):
        m = np.eye(4, dtype=np.float32)
        m[0, 0], m[1, 1] = sx, sy
        m[:3, 3] = t
        return m.T.reshape(16).copy()

    for i in range(n):
        mats.append({"metallic": float(rng.random()), "roughness": float(rng.random()), "base_color": (0, 0, 0)})
        meshes.append([{"positions": P, "normals": None, "texcoords": UV, "indices": F, "material": i}])
        w = world(8.0 + 0.01 * i, 8.0 + 0.01 * i, (0.01 * i, -0.02 * i, -2.0 - 0.05 * i))
        nodes.append({"world": w, "local": w, "mesh": i})
    w = world(44.0, 8.0, (18.0, 0.0, -2.0))
    nodes.append({"world": w, "local": w, "mesh": 0})
    return {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": [tex],
            "cubemap": scenes.cubemap_faces(rng, 8), "cubemap_face_size": 8, "voxel_grid_size": 16,
            "specular_samples": 8, "brdf_lut_size": 16}


@pytest.mark.parametrize("tile", [64, 32])
def test_depth_ties_across_rounds_with_culling(tile):
    n = 80
    s = swr.Scene(tie_across_rounds_scene(n))
    cam = swr.make_camera((0.0, 0.0, 3.0), (0.0, 0.0, 0.0), 1.0, 192, 128, 40.0)
    rgba, vis = compare(s, cam, 192, 128, sched_tile=tile)
    covered = vis[vis != np.uint64(2 ** 64 - 1)] >> np.uint64(3)
    assert np.isin(covered, [2 * n, 2 * n + 1]).mean() > 0.9
    r = swr.Renderer(192, 128, sched_tile=tile)
    r.render(s, cam)
    st = r.stats()
    print("culled %d of %d bin pairs" % (st.culled_pairs, st.bin_pairs))
    # Occlusion culling runs for 64-px scheduling tiles.
    assert (st.culled_pairs > 0) == (tile == 64)
    r.close()
    s.close()


def test_stress_workload_reduced():
    sd, cp = scenes.stress_scene(seed=4, triangles=150_000, width=960, height=540, n_textures=2, tex_size=256,
                                 cube_size=32, voxel=32, specular_samples=16, brdf_lut_size=32)
    s = swr.Scene(sd)
    cam = swr.make_camera(*cp)
    compare(s, cam, 960, 540)
    s.close()


def test_stress_workload_full_4k():
    sd, cp = scenes.stress_scene()
    s = swr.Scene(sd)
    cam = swr.make_camera(*cp)
    compare(s, cam, 3840, 2160)
    s.close()


@pytest.fixture(scope="module")
def textured():
    s = swr.Scene(scenes.textured_scene())
    yield s
    s.close()


@pytest.mark.parametrize("tile", [16, 64])
@pytest.mark.parametrize("mode", [swr.RSQRT_AARCH64, swr.RSQRT_IEEE])
def test_opaque_texture_slots(textured, mode, tile):
    # Opaque materials with normal maps over generated tangents
    # (shader.rs:132-146), metallic-roughness and occlusion textures
    # (shader.rs:182-200) and emissive textures (shader.rs:285-291), present
    # or absent per material, with every wrap mode.
    cam = swr.make_camera(*scenes.default_camera_params(textured.info(), 320, 200))
    compare(textured, cam, 320, 200, rsqrt_mode=mode, sched_tile=tile)


@pytest.mark.parametrize("tile", [8, 32])
def test_opaque_texture_slots_close_up(textured, tile):
    # Close to a displaced grid: magnified textures (mip 0), clipping.
    c = np.array(textured.info().bounds_center[:])
    cam = swr.make_camera((float(c[0]) + 0.3, float(c[1]) + 0.2, float(c[2]) + 2.0),
                          (float(c[0]), float(c[1]), float(c[2]) - 1.0), 1.1, 256, 192, 40.0)
    compare(textured, cam, 256, 192, sched_tile=tile)


def test_stress_all_texture_slots_4k():
    # The 4K workload with every material carrying metallic-roughness,
    # normal, emissive and occlusion textures beside its base colour.
    sd, cp = scenes.stress_scene(all_slots=True)
    s = swr.Scene(sd)
    cam = swr.make_camera(*cp)
    compare(s, cam, 3840, 2160)
    s.close()
