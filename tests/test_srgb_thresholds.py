"""The device builds sRGB mips without powf: a texel's way back from linear
goes through host-made thresholds (the smallest float that packs to each
byte, csrc/ibl.cu linear_to_srgb_byte). That equals the host's
f2u_sat((powf(s, 1/2.4) * 1.055 - 0.055) * 255) for every s only if that byte
never decreases as s grows; this checks it over every float of the powf
branch, (0.0031308, 1], with the host libm (here, and on the GPU host from
tests/test_ibl_device.py)."""
import numpy as np

import oracle


def host_bytes(s):
    p = oracle.srgb_pow(s, 1)
    v = (p * np.float32(1.055) - np.float32(0.055)) * np.float32(255.0)
    assert v.dtype == np.float32
    return np.where(v > 0, np.floor(v), 0).astype(np.uint32)


def check_monotone_bytes():
    first = int(np.array([0.0031308], np.float32).view(np.uint32)[0]) + 1
    last = int(np.array([1.0], np.float32).view(np.uint32)[0])
    prev, total = None, 0
    for start in range(first, last + 1, 1 << 23):
        s = np.arange(start, min(start + (1 << 23), last + 1), dtype=np.uint32).view(np.float32)
        b = host_bytes(s)
        assert np.all(np.diff(b.astype(np.int64)) >= 0)
        if prev is not None:
            assert b[0] >= prev
        prev = b[-1]
        total += s.size
    return total, int(prev)


def test_linear_to_srgb_byte_is_monotone():
    n, top = check_monotone_bytes()
    # Every float of the branch; white packs to 254 (1.055 - 0.055 rounds
    # below 1 in f32), as in the reference.
    assert n > 60_000_000 and top == 254
