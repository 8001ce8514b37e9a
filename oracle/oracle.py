"""ctypes binding of the CPU oracle (test infrastructure only).

The oracle restates the reference's per-frame path and its load-time scene
processing and camera on the CPU; tests, the smoke check and bench.py's CPU
legs use it to check or time against the CUDA path. It renders only scenes
and cameras it built itself from the same inputs the product gets (a scene
dict, camera parameters), so none of the product's tables reach it. The
product never imports this module, and this module never loads libswr (the
binding module is imported for its ctypes structure definitions only).
"""
import ctypes as C
import os
import subprocess
import sys
import weakref

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRCS = [os.path.join(HERE, "swr_oracle.cpp"), os.path.join(HERE, "swr_oracle_scene.cpp")]
LIB = os.path.join(HERE, "liboracle.so")
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "swraster-viewer_gb300"))
import swr  # noqa: E402  (structure definitions only)

# -ffp-contract=off: the reference never fuses multiply and add.
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-pthread", "-ffp-contract=off", "-fno-fast-math"]


def build(force=False):
    deps = SRCS + [os.path.join(ROOT, "include", "swr.h")]
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(d) for d in deps):
        cmd = ["g++"] + FLAGS + SRCS + ["-o", LIB]
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
        L.oracle_srgb_pow.argtypes = [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_void_p]
        L.oracle_srgb_pow.restype = C.c_int
        L.oracle_frsqrts.argtypes = [C.c_float, C.c_float]
        L.oracle_frsqrts.restype = C.c_float
        L.oracle_sun_visibility_ex.argtypes = [C.POINTER(swr.SceneHostView), C.c_uint32, C.c_void_p, C.c_int]
        L.oracle_sun_visibility_ex.restype = C.c_int
        L.oracle_gi_bake.argtypes = [C.POINTER(swr.SceneHostView), C.c_uint32, C.c_void_p]
        L.oracle_gi_bake.restype = C.c_int
        L.oracle_packet_depths.argtypes = [C.c_void_p, C.c_float, C.c_void_p, C.c_void_p, C.c_void_p,
                                           C.POINTER(C.c_float), C.POINTER(C.c_uint64)]
        L.oracle_packet_depths.restype = C.c_int
        L.oracle_scene_build.argtypes = [C.c_void_p, C.c_uint32, C.POINTER(swr.SceneHostView),
                                         C.POINTER(C.c_void_p)]
        L.oracle_scene_build.restype = C.c_int
        L.oracle_scene_bounds.argtypes = [C.c_void_p, C.POINTER(C.c_float)]
        L.oracle_scene_bounds.restype = None
        L.oracle_scene_free.argtypes = [C.c_void_p]
        L.oracle_scene_free.restype = None
        L.oracle_camera_init.argtypes = [C.POINTER(swr.Camera), C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                                         C.c_float, C.c_float, C.c_float]
        L.oracle_camera_init.restype = C.c_int
        L.oracle_node_local.argtypes = [C.c_void_p] * 5
        L.oracle_node_local.restype = None
        L.oracle_mat4_mul.argtypes = [C.c_void_p] * 3
        L.oracle_mat4_mul.restype = None
        _lib = L
    return _lib


class Scene:
    """The processed scene of a scene dict (see scenes.py), built by the
    oracle's restatement of the reference's load path. `view` is a
    swr_scene_host_view of it; `bounds` = (min, max, centre, diagonal)."""

    def __init__(self, sd, gi=False, threads=0):
        desc, keep = swr.scene_desc(sd, swr.SCENE_GI if gi else 0)
        self.view = swr.SceneHostView()
        h = C.c_void_p()
        if lib().oracle_scene_build(C.addressof(desc), threads, C.byref(self.view), C.byref(h)) != 0:
            raise RuntimeError("oracle_scene_build rejected the scene")
        self.handle = h
        self.view._owner = self  # the view points into this scene's arrays
        b = (C.c_float * 10)()
        lib().oracle_scene_bounds(h, b)
        self.bounds = (tuple(b[0:3]), tuple(b[3:6]), tuple(b[6:9]), b[9])

    def close(self):
        if getattr(self, "handle", None):
            lib().oracle_scene_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_scenes = weakref.WeakKeyDictionary()


def scene_of(scene):
    """The oracle's own build of the scene dict a product scene was made from
    (cached per product scene)."""
    if isinstance(scene, Scene):
        return scene
    if getattr(scene, "source", None) is None:
        raise ValueError("the oracle needs the scene dict this scene was made from (scene.source)")
    o = _scenes.get(scene)
    if o is None:
        o = Scene(scene.source, gi=bool(scene.flags & swr.SCENE_GI))
        _scenes[scene] = o
    return o


def camera(position, look_at, fov, width, height, far_plane):
    """RenderCamera::new + update_matrices, as the oracle restates them."""
    cam = swr.Camera()
    p = (C.c_float * 3)(*position)
    t = (C.c_float * 3)(*look_at)
    if lib().oracle_camera_init(C.byref(cam), p, t, fov, float(width), float(height), far_plane) != 0:
        raise RuntimeError("oracle_camera_init failed")
    cam.args = (tuple(position), tuple(look_at), fov, width, height, far_plane)
    return cam


def render(scene, cam, width, height, rsqrt_mode=swr.RSQRT_AARCH64, threads=1, dt=0.0, ev=1.0):
    """Renders `scene` (an oracle Scene, or a product scene whose scene dict
    the oracle rebuilds) from `cam` (rebuilt by the oracle from the
    parameters it was made with). Returns (rgba8 (H,W) u32, vis (H,W) u64,
    tile_lum, Result)."""
    view = scene_of(scene).view
    cam = camera(*cam.args)
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


def srgb_pow(x, mode, threads=16):
    """powf(x, 2.4) (mode 0) or powf(x, 1/2.4) (mode 1) with the host libm."""
    x = np.ascontiguousarray(x, np.float32)
    out = np.empty_like(x)
    if lib().oracle_srgb_pow(x.ctypes.data_as(C.c_void_p), x.size, mode, threads,
                             out.ctypes.data_as(C.c_void_p)) != 0:
        raise RuntimeError("oracle_srgb_pow failed")
    return out


def sun_visibility(view, threads=1, brute=False):
    """Blurred voxel sun visibility (voxel_size^3 floats, x fastest) of the
    scene's load-time precompute: every ray against every triangle (brute),
    or against the candidates of the oracle's conservative BVH."""
    n = view.voxel_size
    out = np.zeros(n * n * n, np.float32)
    if lib().oracle_sun_visibility_ex(C.byref(view), threads, out.ctypes.data_as(C.c_void_p), 1 if brute else 0) != 0:
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
