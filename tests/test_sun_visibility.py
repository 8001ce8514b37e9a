"""Voxel sun visibility of the load-time precompute (compute_sun_visibility +
blur_grid, src/gi.rs:267-314, src/voxelgrid.rs:370-419): the host
restatement (host-only scenes, BVH traversal) and the device version (scenes
that go to the GPU, a light-space grid) against the oracle's own build of the
same scene (its grid bounds and light from its own restatement, every ray
against the triangles its conservative BVH keeps, or against every triangle),
bit for bit, on opaque and translucent scenes."""
import numpy as np
import pytest

import oracle
import scenes
import swr


def exported_light(scene):
    v = scene.export()
    n = v.voxel_size
    return np.ctypeslib.as_array(v.voxel_light_intensity, shape=(n * n * n,)).copy(), v


SCENES = {
    "small": lambda: scenes.small_scene(seed=3),
    "translucent": lambda: scenes.translucent_scene(),
    "stress": lambda: scenes.stress_scene(seed=9, triangles=20_000, width=640, height=480, n_textures=1, tex_size=64,
                                          cube_size=16, voxel=24, specular_samples=8, brdf_lut_size=32)[0],
}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_host_matches_oracle(name):
    sd = SCENES[name]()
    s = swr.Scene(sd, host_only=True)
    light, _ = exported_light(s)
    o = oracle.Scene(sd, threads=4)
    ref = oracle.sun_visibility(o.view, threads=4, brute=True)
    assert (ref < 1.0).any() and (ref > 0.0).any()
    np.testing.assert_array_equal(light, ref)
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(SCENES))
def test_device_matches_oracle(name):
    sd = SCENES[name]()
    s = swr.Scene(sd)
    light, _ = exported_light(s)
    o = oracle.Scene(sd, threads=8)
    np.testing.assert_array_equal(light, oracle.sun_visibility(o.view, threads=8, brute=True))
    s.close()


@pytest.mark.gpu
def test_device_matches_oracle_full_grid():
    # A 128^3 grid over 200k triangles: the oracle's build prunes each ray's
    # candidates with its conservative BVH.
    sd = scenes.stress_scene(seed=5, triangles=200_000, width=1280, height=720, n_textures=1, tex_size=64,
                             cube_size=16, voxel=128, specular_samples=8, brdf_lut_size=32)[0]
    dev, _ = exported_light(swr.Scene(sd))
    o = oracle.Scene(sd)
    ref = np.ctypeslib.as_array(o.view.voxel_light_intensity, shape=(128 ** 3,)).copy()
    assert (ref < 1.0).mean() > 0.01
    np.testing.assert_array_equal(dev, ref)
