"""The raster's occlusion culling drops a packet when a lower bound of its
depths lies behind every depth its tile cells already hold. The bound (the
raster's own source, evaluated on the host through swr_selftest_depth_floor)
must never exceed a depth the reference's tile raster computes for a covered
lane of the packet: an exhaustive walk of the packet by the oracle
(oracle_packet_depths, src/tilerasterizer.rs:114-383) checks it on seeded
packets of every size, slivers, packets far outside the screen and steep
depth ranges."""
import numpy as np

import oracle
import swr

W, H = 3840, 2160
f32 = np.float32


def record(rng, xy, cw_range=(0.05, 500.0)):
    """Packet record from subpixel vertices as the front end forms it
    (setup_triangle): front-facing order, 1/area, z/w and 1/w interpolants."""
    x = xy[:, 0].astype(np.int64)
    y = xy[:, 1].astype(np.int64)
    area = (x[1] - x[0]) * (y[2] - y[0]) - (x[2] - x[0]) * (y[1] - y[0])
    if area == 0:
        return None
    if area > 0:  # make it front-facing (negative signed area)
        xy = xy[[0, 2, 1]]
        area = -area
    a32 = np.int64(area).astype(np.int32)  # the raster's wrapping int32 area
    ooa = f32(1.0) / f32(abs(int(a32)) if a32 != np.iinfo(np.int32).min else 2.0 ** 31)
    cw = np.exp(rng.uniform(np.log(cw_range[0]), np.log(cw_range[1]), 3)).astype(f32)
    cz = (cw * rng.uniform(-1.0, 1.2, 3).astype(f32)).astype(f32)
    oow = (f32(1.0) / cw).astype(f32)
    zow = (cz * oow).astype(f32)
    rz = np.array([zow[0], zow[1] - zow[0], zow[2] - zow[0]], f32)
    ro = np.array([oow[0], oow[1] - oow[0], oow[2] - oow[0]], f32)
    return xy.reshape(-1).astype(np.int32), ooa, rz, ro


def bbox(p):
    """Pixel bounding box as the front end clamps it to the screen."""
    xs, ys = p[0::2].astype(np.int64), p[1::2].astype(np.int64)
    mnx = max(int(xs.min()), 0) >> 4
    mny = max(int(ys.min()), 0) >> 4
    mxx = (min(int(xs.max()), W * 16) + 16) >> 4
    mxy = (min(int(ys.max()), H * 16) + 16) >> 4
    return mnx, mny, mxx, mxy


def tiles(rng, bb, limit=3):
    mnx, mny, mxx, mxy = bb
    tx = list(range(mnx // 64, min((mxx + 63) // 64, (W + 63) // 64)))
    ty = list(range(mny // 64, min((mxy + 63) // 64, (H + 63) // 64)))
    pairs = [(a, b) for a in tx for b in ty]
    if len(pairs) > limit:
        pairs = [pairs[i] for i in rng.choice(len(pairs), limit, replace=False)]
    for a, b in pairs:
        rect = (max(mnx, 64 * a), max(mny, 64 * b), min(mxx, 64 * a + 64), min(mxy, 64 * b + 64))
        if rect[2] - rect[0] >= 1 and rect[3] - rect[1] >= 1:
            yield np.array(rect, np.int32)


def triangle(rng, kind):
    c = rng.uniform([0, 0], [W, H])
    if kind == "any":
        s = np.exp(rng.uniform(np.log(0.3), np.log(6000.0)))
        v = c + s * rng.uniform(-1, 1, (3, 2))
    elif kind == "sliver":
        s = np.exp(rng.uniform(np.log(2.0), np.log(4000.0)))
        a = c + s * rng.uniform(-1, 1, 2)
        b = c - s * rng.uniform(-1, 1, 2)
        t = rng.uniform(0, 1)
        v = np.array([a, b, a + t * (b - a) + rng.uniform(-0.3, 0.3, 2)])
    else:  # "far": vertices well outside the screen (guard band and beyond)
        s = np.exp(rng.uniform(np.log(1e3), np.log(3e5)))
        v = c + s * rng.uniform(-1, 1, (3, 2))
    return np.round(v * 16).astype(np.int64)


def check(rng, n, kind, cw_range=(0.05, 500.0)):
    taken = covered = 0
    slack = []
    for _ in range(n):
        xy = triangle(rng, kind)
        if np.abs(xy).max() >= 2 ** 31:
            continue
        rec = record(rng, xy.astype(np.int64), cw_range)
        if rec is None:
            continue
        p, ooa, zow, oow = rec
        for rect in tiles(rng, bbox(p)):
            zlo = swr.selftest_depth_floor(p, zow, oow, int(rect[2]) * 16, int(rect[3]) * 16)
            zmin, lanes = oracle.packet_depths(p, ooa, zow, oow, rect)
            if lanes == 0:
                continue
            covered += 1
            if zlo == -np.inf:
                continue
            taken += 1
            assert zlo <= zmin, (kind, p.tolist(), float(ooa), zow.tolist(), oow.tolist(), rect.tolist(), zlo, zmin)
            # Against the nearest vertex depth (the ideal floor of the whole
            # triangle), relative to the depth's magnitude.
            zw = zow.astype(np.float64)
            ow = oow.astype(np.float64)
            zv = min(zw[0] / ow[0], (zw[0] + zw[1]) / (ow[0] + ow[1]), (zw[0] + zw[2]) / (ow[0] + ow[2]))
            slack.append((zv - zlo) / max(1.0, abs(zv)))
    return taken, covered, np.array(slack)


def test_floor_below_every_covered_depth():
    rng = np.random.default_rng(2024)
    taken, covered, slack = check(rng, 3000, "any")
    print("any: floor taken for %d of %d covered packets" % (taken, covered))
    # No floor where the setup's int32 terms could wrap (triangles far
    # larger than the screen) or where 1/w spans so many decades that its
    # interpolant, widened by the rounding margins, could reach 0.
    assert covered > 1000 and taken > 0.85 * covered
    # The floor is the nearest vertex depth up to rounding margins: tight for
    # most packets (what makes culling drop anything).
    assert np.median(slack) < 1e-3


def test_floor_on_slivers_and_far_triangles():
    rng = np.random.default_rng(7)
    for kind in ("sliver", "far"):
        taken, covered, _ = check(rng, 2000, kind)
        print("%s: floor taken for %d of %d covered packets" % (kind, taken, covered))
        assert covered > 200


def test_floor_with_steep_depth_ranges():
    # 1/w spanning five decades across one triangle (near-plane crossings
    # after clipping): the corners of the barycentric triangle bound it.
    rng = np.random.default_rng(99)
    taken, covered, _ = check(rng, 2000, "any", cw_range=(0.001, 100.0))
    print("steep: floor taken for %d of %d covered packets" % (taken, covered))
    assert covered > 500 and taken > 0


def test_no_floor_for_back_faces_and_wrapping_setups():
    p = np.array([0, 0, 320, 0, 0, 320], np.int32)  # positive signed area: back-facing
    assert swr.selftest_depth_floor(p, [0.5, 0.1, 0.2], [1.0, 0.0, 0.0], 1024, 1024) == -np.inf
    big = np.array([-(2 ** 29), 0, 0, 2 ** 29, 2 ** 29, 0], np.int32)  # edge terms beyond int32
    assert swr.selftest_depth_floor(big, [0.5, 0.1, 0.2], [1.0, 0.0, 0.0], 1024, 1024) == -np.inf
    front = np.array([0, 0, 0, 320, 320, 0], np.int32)
    zlo = swr.selftest_depth_floor(front, [0.5, 0.1, 0.2], [1.0, 0.0, 0.0], 1024, 1024)
    assert 0.49 < zlo <= 0.5
    # A 1/w interpolant that reaches 0 inside the triangle: no floor.
    assert swr.selftest_depth_floor(front, [0.5, 0.1, 0.2], [1.0, -1.0, 0.0], 1024, 1024) == -np.inf
