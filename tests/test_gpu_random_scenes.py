"""Seeded random scenes (sphere, textured with every texture slot, translucent;
cubemap faces of 8 to 64 px, voxel grids of 8 to 24, frame sizes from 64 to
700 px) built on the device and rendered at every scheduling tile size, against
the oracle's own build and frames: every exported table bit-exact, visibility
bit-exact, colour within 1/255, tile luminance exact."""
import numpy as np
import pytest

import oracle
import scenes
import swr
from test_gpu_parity import compare
from test_scene_tables import table_differences

pytestmark = pytest.mark.gpu


def cases(n=9, seed=2026):
    rng = np.random.default_rng(seed)
    out = []
    for it in range(n):
        out.append((it % 3, int(rng.integers(1000, 100000)), int(rng.choice([8, 16, 32, 48, 64])),
                    int(rng.choice([8, 16, 24])), int(rng.integers(64, 700)), int(rng.integers(64, 500))))
    return out


@pytest.mark.parametrize("kind,seed,cube,voxel,w,h", cases())
def test_random_scene_tables_and_frames(kind, seed, cube, voxel, w, h):
    if kind == 0:
        sd = scenes.small_scene(seed=seed, cube_size=cube, voxel=voxel)
    elif kind == 1:
        sd = scenes.textured_scene(seed=seed, cube_size=cube, voxel=voxel)
    else:
        sd = scenes.translucent_scene(seed=seed, cube_size=cube, voxel=voxel)
    p = swr.Scene(sd)
    o = oracle.Scene(sd, threads=16)
    assert table_differences(p.export(), o.view) == []
    cam = swr.make_camera(*scenes.default_camera_params(p.info(), w, h))
    for tile in (8, 16, 32, 64):
        compare(p, cam, w, h, sched_tile=tile)
    p.close()
