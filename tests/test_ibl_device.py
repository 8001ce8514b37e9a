"""Load-time texture precompute on the device (mip chains, BRDF LUT, GGX
prefilter; csrc/ibl.cu) against the oracle's own build of the same scenes,
bit for bit.

sRGB mips take the way back from linear through host-made byte thresholds,
sound while the host's byte never decreases with its input (checked here
with this host's libm, tests/test_srgb_thresholds.py). The GGX prefilter
takes an interval of +-2 ulp around the device's powf; that is sound only
while the device's and the host libm's powf differ by at most that much,
which the first test checks over every float the tables can pass to powf
(the prefilter's inputs lie in [0.0905, 1]; the range tested also covers the
mips' [0.0031308, 1]). Texels whose byte the interval leaves open are
computed again on the host; the scenes below are large enough that this
happens, and `precompute_host_texels` counts it."""
import ctypes as C

import numpy as np
import pytest

import oracle
import scenes
import swr
from test_scene_tables import SCENES, bounds_differ, table_differences

pytestmark = pytest.mark.gpu

WINDOW = 2  # kPowUlps in csrc/ibl.cu


@pytest.mark.parametrize("mode", [0, 1])
def test_device_powf_stays_inside_the_interval(mode):
    lo = np.array([0.003], np.float32).view(np.uint32)[0]
    hi = np.array([1.001], np.float32).view(np.uint32)[0]
    L = swr.lib()
    worst, chunk = 0, 1 << 23
    for start in range(int(lo), int(hi) + 1, chunk):
        bits = np.arange(start, min(start + chunk, int(hi) + 1), dtype=np.uint32)
        x = bits.view(np.float32)
        dev = np.empty_like(x)
        st = L.swr_selftest_srgb_pow(x.ctypes.data_as(swr.f32p), dev.ctypes.data_as(swr.f32p), x.size, mode)
        assert st == swr.SWR_OK, L.swr_last_error()
        host = oracle.srgb_pow(x, mode)
        d = np.abs(dev.view(np.int32).astype(np.int64) - host.view(np.int32).astype(np.int64))
        worst = max(worst, int(d.max()))
    print("mode %d: largest difference %d ulp" % (mode, worst))
    assert worst <= WINDOW


def test_linear_to_srgb_byte_is_monotone_on_this_host():
    from test_srgb_thresholds import check_monotone_bytes
    n, top = check_monotone_bytes()
    assert n > 60_000_000 and top == 254


def reference_sizes():
    """The reference's table sizes: a 256-px cubemap face (its
    assets/cubemap.jpg is a 1024x768 cross), 64 GGX samples, a 128^2 BRDF
    LUT, with two 512^2 sRGB textures."""
    sd = scenes.spheres_scene(seed=4, count=8, subdiv=2, tex_size=512, cube_size=256, voxel=16,
                              specular_samples=64, brdf_lut_size=128)
    return sd


DEVICE_SCENES = dict(SCENES, reference_sizes=reference_sizes)


@pytest.mark.parametrize("name", list(DEVICE_SCENES))
def test_device_tables_equal_the_oracle_build(name):
    sd = DEVICE_SCENES[name]()
    p = swr.Scene(sd)
    o = oracle.Scene(sd, threads=16)
    info = p.info()
    print("%s: %d texels recomputed on the host" % (name, info.precompute_host_texels))
    assert table_differences(p.export(), o.view) == []
    assert not bounds_differ(info, o.bounds)
    if name in ("c2_reduced", "reference_sizes"):
        # Large enough that the interval leaves some bytes open.
        assert info.precompute_host_texels > 0
    p.close()


def test_planted_powf_error_would_be_caught():
    """The comparison above sees a one-level change in a single texel of a
    device-built table (planted on the oracle's side, on the CPU)."""
    sd = scenes.small_scene(seed=3)
    p = swr.Scene(sd)
    o = oracle.Scene(sd)
    spec = o.view.cubemap_specular
    data = np.ctypeslib.as_array(C.cast(spec.data, C.POINTER(C.c_uint32)), shape=(spec.data_len,))
    data[spec.data_len // 2] ^= np.uint32(1 << 8)
    assert "cubemap_specular texels" in table_differences(p.export(), o.view)
    p.close()
