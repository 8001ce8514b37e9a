"""Known answers for the oracle's Arm FRSQRTE/FRSQRTS emulation, and (on an
aarch64 host, i.e. the GPU machine's Grace CPU) an exhaustive check of the
emulation against the real vrsqrteq_f32 / vrsqrtsq_f32 instructions that
the reference's rsqrt_vec (src/math.rs:17-25) executes there."""
import os
import platform
import subprocess
import tempfile

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))


def test_frsqrte_known_answers():
    L = oracle.lib()
    # RecipSqrtEstimate: 1.0 -> 511/512, 2.0 -> 361/256 * 2^-1, 4.0 -> 1.0 * 2^-1 (x 511/512).
    assert L.oracle_frsqrte(1.0) == 0.998046875
    assert L.oracle_frsqrte(4.0) == 0.4990234375
    assert L.oracle_frsqrte(2.0) == 0.705078125
    assert L.oracle_frsqrte(0.0) == float("inf")
    assert L.oracle_frsqrte(-0.0) == float("-inf")
    assert np.isnan(L.oracle_frsqrte(-1.0))
    assert L.oracle_frsqrte(float("inf")) == 0.0
    # FRSQRTS: (3 - a*b) / 2, inf * 0 -> 1.5.
    assert L.oracle_frsqrts(1.0, 1.0) == 1.0
    assert L.oracle_frsqrts(float("inf"), 0.0) == 1.5
    # One Newton step lands within 2^-15 relative of 1/sqrt(x).
    for x in (0.3, 1.0, 2.0, 7.5, 1e-20, 3e30):
        r = L.oracle_rsqrt_aarch64(x)
        assert abs(r * np.sqrt(np.float64(x)) - 1.0) < 2.0 ** -14


def _inputs():
    xs = []
    # Every 9-bit estimate-table index, for even and odd exponents.
    for e in (126, 127, 128, 129):
        for m in range(256):
            xs.append(np.uint32((e << 23) | (m << 15) | 0x1234))
    xs = np.array(xs, np.uint32).view(np.float32)
    rng = np.random.default_rng(5)
    rnd = rng.integers(1, 0x7F7FFFFF, 200000, dtype=np.uint32).view(np.float32)
    sub = rng.integers(1, 0x007FFFFF, 2000, dtype=np.uint32).view(np.float32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, -1.0, 1.0, np.float32(1e-45), np.float32(3.4e38)], np.float32)
    return np.concatenate([xs, rnd, sub, special]).astype(np.float32)


@pytest.mark.gpu
@pytest.mark.skipif(platform.machine() != "aarch64", reason="needs an aarch64 host")
def test_emulation_matches_arm_hardware():
    L = oracle.lib()
    xs = _inputs()
    with tempfile.TemporaryDirectory() as td:
        exe = os.path.join(td, "neon_rsqrt")
        subprocess.run(["gcc", "-O2", os.path.join(HERE, "native", "neon_rsqrt.c"), "-o", exe], check=True)
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        xs.tofile(fi)
        subprocess.run([exe, fi, fo], check=True)
        hw = np.fromfile(fo, np.float32).reshape(-1, 3)
    bad = 0
    for i, x in enumerate(xs):
        e = np.float32(L.oracle_frsqrte(float(x)))
        r = np.float32(L.oracle_rsqrt_aarch64(float(x)))
        he, hr = hw[i, 0], hw[i, 2]
        same_e = (e.view(np.uint32) == he.view(np.uint32)) or (np.isnan(e) and np.isnan(he))
        same_r = (r.view(np.uint32) == hr.view(np.uint32)) or (np.isnan(r) and np.isnan(hr))
        if not (same_e and same_r):
            bad += 1
            if bad < 5:
                print("mismatch x=%r emu=(%r, %r) hw=(%r, %r)" % (x, e, r, he, hr))
    assert bad == 0, "%d of %d inputs differ from the hardware" % (bad, len(xs))


@pytest.mark.gpu
def test_device_rsqrt_matches_oracle():
    # The shading pass's normalize arithmetic on the device, bit for bit
    # against the oracle's restatement (Arm mode) and IEEE 1/sqrt (IEEE mode).
    import swr
    L = oracle.lib()
    xs = _inputs()
    dev = swr.selftest_rsqrt(xs, swr.RSQRT_AARCH64)
    ref = np.array([L.oracle_rsqrt_aarch64(float(x)) for x in xs], np.float32)
    same = (dev.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(dev) & np.isnan(ref))
    assert same.all(), "%d of %d differ, first x=%r" % ((~same).sum(), xs.size, xs[~same][:3])
    dev = swr.selftest_rsqrt(xs, swr.RSQRT_IEEE)
    with np.errstate(all="ignore"):
        ref = np.float32(1.0) / np.sqrt(xs)
    same = (dev.view(np.uint32) == ref.view(np.uint32)) | (np.isnan(dev) & np.isnan(ref))
    assert same.all(), "%d of %d differ (IEEE)" % ((~same).sum(), xs.size)
