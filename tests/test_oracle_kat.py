"""Known answers for the oracle, derived from the reference's formulas
(src/renderer.rs, src/tilerasterizer.rs). CPU only."""
import numpy as np

import oracle
from helpers import BACKGROUND, tri_scene

W, H = 64, 48
CAM = ((0.0, 0.0, 5.0), (0.0, 0.0, 0.0), np.pi / 3, W, H, 20.0)


def render(tris, **kw):
    s = oracle.Scene(tri_scene(tris))
    out = oracle.render(s, oracle.camera(*CAM), W, H, **kw)
    s.close()
    return out


def test_backface_culling():
    ccw = [(-1, -1, 0), (1, -1, 0), (0, 1, 0)]   # counter-clockwise seen from +z: front-facing
    cw = [(-1, -1, 0), (0, 1, 0), (1, -1, 0)]
    _, vis_front, _, _ = render([ccw])
    _, vis_back, _, _ = render([cw])
    assert (vis_front != BACKGROUND).sum() > 100
    assert (vis_back != BACKGROUND).sum() == 0  # signed_area > 0 is culled (renderer.rs:680)


def test_degenerate_triangle_covers_nothing():
    _, vis, _, res = render([[(-1, -1, 0), (0, 0, 0), (1, 1, 0)]])
    assert (vis != BACKGROUND).sum() == 0
    assert res.packets > 0  # zero area is not culled; it is binned and covers no pixel


def test_top_left_rule_partitions_shared_edge():
    # A square split on its diagonal: every pixel of the union belongs to
    # exactly one of the two triangles (tilerasterizer.rs:139-156).
    a = [(-1.3, -1.1, 0), (1.2, -1.1, 0), (1.2, 1.05, 0)]
    b = [(-1.3, -1.1, 0), (1.2, 1.05, 0), (-1.3, 1.05, 0)]
    _, va, _, _ = render([a])
    _, vb, _, _ = render([b])
    _, vab, _, _ = render([a, b])
    sa, sb = va != BACKGROUND, vb != BACKGROUND
    assert not (sa & sb).any()
    assert np.array_equal(vab != BACKGROUND, sa | sb)
    # Triangle IDs: the pair's second triangle has static id 1.
    assert set(np.unique(vab[sa] >> np.uint64(3)).tolist()) == {0}
    assert set(np.unique(vab[sb] >> np.uint64(3)).tolist()) == {1}


def test_near_plane_clip_fans():
    # A big triangle crossing the near plane (near = 0.2 -> clip at ~0.1 in
    # front of the camera) and the side planes: its fan triangles show up as
    # fan indices > 0 (renderer.rs:650-664).
    t = [(-30.0, -30.0, 4.95), (30.0, -30.0, 4.95), (0.0, 30.0, -40.0)]
    _, vis, _, _ = render([t])
    cov = vis[vis != BACKGROUND]
    assert cov.size > 0
    assert (cov & np.uint64(7)).max() >= 1


def test_exposure_update_matches_formula():
    tri = [(-1, -1, 0), (1, -1, 0), (0, 1, 0)]
    _, _, tl, res0 = render([tri], dt=0.0)
    assert res0.exposure == 2.0 and res0.ev == 1.0  # dt = 0 keeps the fresh exposure
    _, _, tl, res = render([tri], dt=0.5)
    # update_auto_exposure (renderer.rs:258-290) restated in float32 numpy.
    s = np.sort(np.log2(np.maximum(tl, np.float32(1e-4))).astype(np.float32))
    n = s.size
    trim = min(int(np.floor(np.float32(n) * np.float32(0.1))), (n - 1) // 2)
    mean = np.float32(np.sum(s[trim:n - trim], dtype=np.float32) / np.float32(n - 2 * trim))
    key = np.float32(0.45) * np.float32(0.2) / (np.float32(1.2) - np.float32(0.45))
    target = np.clip(np.exp2(np.log2(key) - mean), 0.05, 32.0)
    alpha = 1.0 - np.exp(-0.5)
    ev = 1.0 + (np.log2(target) - 1.0) * alpha
    assert abs(res.ev - ev) < 1e-5 and abs(res.exposure - 2.0 ** ev) < 1e-4
