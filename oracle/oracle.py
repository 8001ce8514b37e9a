"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the reference's per-frame path on the CPU; tests, the
smoke check and bench.py's CPU-baseline leg use it to check or time against
the CUDA path. The product never imports this module.
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "swr_oracle.cpp")
LIB = os.path.join(HERE, "liboracle.so")
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "swraster-viewer_gb300"))
import swr  # noqa: E402  (structure definitions only)

# -ffp-contract=off: the reference never fuses multiply and add.
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math"]


def build(force=False):
    deps = [SRC, os.path.join(ROOT, "include", "swr.h")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(d) for d in deps):
        cmd = ["g++"] + FLAGS + [SRC, "-o", LIB]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + p.stderr)
    return LIB


class Opts(C.Structure):
    _fields_ = [("rsqrt_mode", C.c_uint32), ("threads", C.c_uint32), ("dt", C.c_float), ("ev", C.c_float)]


class Result(C.Structure):
    _fields_ = [("ev", C.c_float), ("exposure", C.c_float), ("target", C.c_float), ("tiles", C.c_uint32),
                ("packets", C.c_uint64), ("triangles_in", C.c_uint64), ("quads_tested", C.c_uint64),
                ("fragments", C.c_uint64), ("depth_passed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        L.oracle_render.argtypes = [C.POINTER(swr.SceneHostView), C.POINTER(swr.Camera), C.c_int32, C.c_int32,
                                    C.POINTER(Opts), C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(Result)]
        L.oracle_render.restype = C.c_int
        for n in ("oracle_frsqrte", "oracle_rsqrt_aarch64"):
            getattr(L, n).argtypes = [C.c_float]
            getattr(L, n).restype = C.c_float
        L.oracle_frsqrts.argtypes = [C.c_float, C.c_float]
        L.oracle_frsqrts.restype = C.c_float
        L.oracle_sun_visibility.argtypes = [C.POINTER(swr.SceneHostView), C.c_uint32, C.c_void_p]
        L.oracle_sun_visibility.restype = C.c_int
        L.oracle_gi_bake.argtypes = [C.POINTER(swr.SceneHostView), C.c_uint32, C.c_void_p]
        L.oracle_gi_bake.restype = C.c_int
        L.oracle_packet_depths.argtypes = [C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.POINTER(C.c_float), C.POINTER(C.c_uint64)]
        L.oracle_packet_depths.restype = C.c_int
        _lib = L
    return _lib


def render(view, cam, width, height, rsqrt_mode=swr.RSQRT_AARCH64, threads=1, dt=0.0, ev=1.0):
    """Returns (rgba8 (H,W) u32, vis (H,W) u64, tile_lum, Result)."""
    rgba = np.zeros((height, width), np.uint32)
    vis = np.zeros((height, width), np.uint64)
    tl = np.zeros(((width + 63) // 64) * ((height + 63) // 64), np.float32)
    res = Result()
    o = Opts(rsqrt_mode, threads, dt, ev)
    rc = lib().oracle_render(C.byref(view), C.byref(cam), width, height, C.byref(o),
                             rgba.ctypes.data_as(C.c_void_p), vis.ctypes.data_as(C.c_void_p),
                             tl.ctypes.data_as(C.c_void_p), C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle_render failed")
    return rgba, vis, tl, res


def packet_depths(p, ooa, zow, oow, rect):
    """(smallest depth, covered lanes) of one packet as the reference's tile
    raster computes them, without the depth test. p: 6 subpixel vertex
    coordinates; zow, oow: interpolants (vertex 0, then differences); rect:
    the packet's pixel rect clipped to its 64-px tile."""
    p = np.ascontiguousarray(p, np.int32)
    zow = np.ascontiguousarray(zow, np.float32)
    oow = np.ascontiguousarray(oow, np.float32)
    rect = np.ascontiguousarray(rect, np.int32)
    zmin, n = C.c_float(), C.c_uint64()
    lib().oracle_packet_depths(p.ctypes.data, float(ooa), zow.ctypes.data, oow.ctypes.data, rect.ctypes.data,
                               C.byref(zmin), C.byref(n))
    return zmin.value, n.value


def sun_visibility(view, threads=1):
    """Blurred voxel sun visibility (voxel_size^3 floats, x fastest) of the
    scene's load-time precompute, by brute force over every triangle."""
    n = view.voxel_size
    out = np.zeros(n * n * n, np.float32)
    if lib().oracle_sun_visibility(C.byref(view), threads, out.ctypes.data_as(C.c_void_p)) != 0:
        raise RuntimeError("oracle_sun_visibility failed")
    return out


def gi_bake(view, threads=1):
    """Blurred baked SH4 grid (voxel_size^3 x 4 x (r, g, b, w)) of the scene's
    voxel GI bake, by brute force over every triangle."""
    n = view.voxel_size
    out = np.zeros((n * n * n, 4, 4), np.float32)
    if lib().oracle_gi_bake(C.byref(view), threads, out.ctypes.data_as(C.c_void_p)) != 0:
        raise RuntimeError("oracle_gi_bake failed")
    return out


if __name__ == "__main__":
    print(build(force=True))
