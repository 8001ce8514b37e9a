"""Voxel GI bake (the reference's --gi: bake_voxel_gi + blur_gi_sh4,
src/gi.rs:316-408, src/voxelgrid.rs:422-472) on the device against the
oracle's own build of the scene with its brute-force bake, bit for bit, and
frames shaded with the baked SH4 grid against the oracle's frames from its
own grid (visibility bit-exact, colour within 1/255). The bake samples
surface textures bilinearly on the device and converts them to linear on the
host, so every powf is the host libm's, as in the oracle."""
import numpy as np
import pytest

import oracle
import scenes
import swr
from test_gpu_parity import compare


def gi_scene(kind, voxel=12):
    if kind == "spheres":
        sd = scenes.spheres_scene(seed=31, count=6, subdiv=2, box=4.0, radius=(0.6, 1.8), tex_size=32, cube_size=16,
                                  voxel=voxel, specular_samples=8, brdf_lut_size=32)
        # An emissive sphere: the bounce adds emissive radiance.
        sd["materials"][2]["emissive_factor"] = (0.8, 0.5, 0.2)
        return sd
    if kind == "textured":
        # Every texture slot, emissive textures included.
        return scenes.textured_scene(voxel=voxel)
    sd = scenes.translucent_scene(count=6, tex_size=32, cube_size=16, voxel=voxel)
    return sd


def baked(scene):
    v = scene.export()
    n = v.voxel_size
    assert bool(v.voxel_gi_sh4)
    return np.ctypeslib.as_array(v.voxel_gi_sh4, shape=(n * n * n, 4, 4)).copy(), v


def test_gi_requires_device():
    with pytest.raises(swr.SwrError):
        swr.Scene(gi_scene("spheres"), host_only=True, gi=True)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["spheres", "translucent", "textured"])
def test_bake_matches_oracle(kind):
    sd = gi_scene(kind)
    s = swr.Scene(sd, gi=True)
    grid, v = baked(s)
    o = oracle.Scene(sd, gi=True, threads=16)
    n = o.view.voxel_size
    ref = np.ctypeslib.as_array(o.view.voxel_gi_sh4, shape=(n * n * n, 4, 4)).copy()
    d = np.abs(grid - ref)
    print("max abs %.3g, exact %.4f" % (d.max(), (d == 0).mean()))
    np.testing.assert_array_equal(grid.view(np.uint32), ref.view(np.uint32))
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["spheres", "translucent"])
def test_frames_with_baked_grid_match_oracle(kind):
    s = swr.Scene(gi_scene(kind, voxel=16), gi=True)
    cam = swr.make_camera(*scenes.default_camera_params(s.info(), 256, 160))
    compare(s, cam, 256, 160)
    s.close()


@pytest.mark.gpu
def test_gi_cache_replaces_the_bake(tmp_path):
    """The reference's .gi cache (src/main.rs:248-279): the first load bakes
    and writes the file, the second reads it instead of baking; grids and
    frames are identical. The prefiltered environment goes through its
    cache file the same way."""
    sd = gi_scene("spheres", voxel=16)
    gi_path, ggx_path = tmp_path / "scene.gi", tmp_path / "cubemap.ggx"
    a = swr.Scene(sd, gi=True, gi_cache=gi_path, ggx_cache=ggx_path)
    ia = a.info()
    if swr.CACHE_NO_CODEC in (ia.gi_cache, ia.ggx_cache):
        pytest.skip("no brotli library on this system")
    assert (ia.gi_cache, ia.ggx_cache) == (swr.CACHE_WRITTEN, swr.CACHE_WRITTEN)
    b = swr.Scene(sd, gi=True, gi_cache=gi_path, ggx_cache=ggx_path)
    ib = b.info()
    assert (ib.gi_cache, ib.ggx_cache) == (swr.CACHE_LOADED, swr.CACHE_LOADED)
    ga, _ = baked(a)
    gb, _ = baked(b)
    assert np.array_equal(ga.view(np.uint32), gb.view(np.uint32))
    cam = swr.make_camera(*scenes.default_camera_params(ia, 256, 160))
    out = []
    for s in (a, b):
        r = swr.Renderer(256, 160)
        r.render(s, cam, 0.0)
        out.append((r.blit(), r.visbuffer()))
        r.close()
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    a.close()
    b.close()
