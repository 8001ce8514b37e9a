"""C ABI surface: the library loads, exports every declared entry point, and
validates arguments without a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import scenes
import swr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "swr.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(swr_[a-z0-9_]+)\s*\(", src)))


def test_every_declared_symbol_is_exported():
    L = swr.lib()
    names = declared_functions()
    assert len(names) >= 18
    for n in names:
        assert hasattr(L, n), n
    assert set(names) == set(swr.EXPORTS)


def test_abi_version():
    assert swr.lib().swr_abi_version() == 2


def test_null_arguments_are_rejected():
    L = swr.lib()
    assert L.swr_scene_create(None, None) == swr.SWR_INVALID_ARG
    assert L.swr_camera_update(None) == swr.SWR_INVALID_ARG
    assert L.swr_render_frame(None, None, None, 0.0, None) == swr.SWR_INVALID_ARG
    assert b"null" in L.swr_last_error()
    h = C.c_void_p()
    assert L.swr_renderer_create(0, 10, None, C.byref(h)) == swr.SWR_INVALID_ARG
    o = swr.RendererOpts(0, 12, 0, 0, 0)
    assert L.swr_renderer_create(64, 64, C.byref(o), C.byref(h)) == swr.SWR_INVALID_ARG


def test_bad_scene_is_rejected():
    sd = scenes.small_scene()
    sd["meshes"][0][0]["indices"] = np.array([0, 1, 100000], np.uint32)
    with pytest.raises(swr.SwrError) as e:
        swr.Scene(sd, host_only=True)
    assert e.value.status == swr.SWR_BAD_SCENE
    sd = scenes.small_scene()
    sd["materials"][0]["base_color"] = (5, 0, 0)
    with pytest.raises(swr.SwrError):
        swr.Scene(sd, host_only=True)
    # Load-time table sizes past their limits (a 2^20 BRDF LUT would be 4 TB).
    for key, value in (("brdf_lut_size", 1 << 20), ("voxel_grid_size", 4097), ("specular_samples", 1 << 31)):
        sd = scenes.small_scene()
        sd[key] = value
        with pytest.raises(swr.SwrError) as e:
            swr.Scene(sd, host_only=True)
        assert e.value.status == swr.SWR_INVALID_ARG


def test_host_only_scene_export():
    sd = scenes.small_scene()
    s = swr.Scene(sd, host_only=True)
    info = s.info()
    assert info.triangle_count == 6 * 320
    v = s.export()
    assert v.primitive_count == 6 and v.node_count == 6
    p = v.primitives[0]
    tan = np.ctypeslib.as_array(p.tangents, (p.vertex_count * 4,)).reshape(-1, 4)
    assert set(np.unique(tan[:, 3])) <= {-1.0, 1.0}
    nrm = np.ctypeslib.as_array(p.normals, (p.vertex_count * 4,)).reshape(-1, 4)
    assert np.allclose(np.linalg.norm(nrm[:, :3], axis=1), 1.0, atol=1e-5)
    # 16^2 cubemap: 5 mips (src/texture.rs:336), BRDF LUT 32^2 with mips.
    assert v.cubemap.mip_count == 5 and v.cubemap_specular.mip_count == 5 and v.brdf_lut.mip_count == 6
    L = np.ctypeslib.as_array(v.voxel_light_intensity, (v.voxel_size ** 3,))
    assert L.min() >= 0.0 and L.max() <= 1.0
    s.close()


def _rx(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])


def _ry(a):
    c, s = np.cos(a), np.sin(a)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def test_camera_matches_float64_model():
    # Yaw only: the look-at point projects to the screen centre.
    cam = swr.make_camera((3.0, 0.0, 10.0), (0.0, 0.0, 0.0), np.pi / 3, 640, 480, 50.0)
    vp = np.array(cam.view_project[:], np.float64).reshape(4, 4).T
    p = vp @ np.array([0.0, 0.0, 0.0, 1.0])
    assert abs(p[0] / p[3]) < 1e-5 and abs(p[1] / p[3]) < 1e-5 and p[3] > 0
    inv = np.array(cam.inverse_view_project[:], np.float64).reshape(4, 4).T
    assert np.allclose(inv @ vp, np.eye(4), atol=1e-4)
    assert abs(cam.near_plane - 0.5) < 1e-7 and cam.far_plane == 50.0
    # With pitch the view rotation is Rx(pitch) * Ry(yaw), pitch = asin(forward.y)
    # (src/rendercamera.rs:40-41, 126-135), which does not re-centre the target.
    cam = swr.make_camera((1.0, 2.0, 10.0), (0.0, 0.0, 0.0), np.pi / 3, 640, 480, 50.0)
    f = -np.array([1.0, 2.0, 10.0]) / np.linalg.norm([1.0, 2.0, 10.0])
    yaw, pitch = np.arctan2(f[0], -f[2]), np.arcsin(f[1])
    assert abs(cam.yaw - yaw) < 1e-6 and abs(cam.pitch - pitch) < 1e-6
    view = np.array(cam.view[:], np.float64).reshape(4, 4).T
    assert np.allclose(view[:3, :3], _rx(pitch) @ _ry(yaw), atol=1e-6)


# ctypes mirror in swr.py -> C struct of include/swr.h.
MIRRORS = {"TextureDesc": "swr_texture_desc", "TexRef": "swr_texref", "MaterialDesc": "swr_material_desc",
           "PrimitiveDesc": "swr_primitive_desc", "MeshDesc": "swr_mesh_desc", "NodeDesc": "swr_node_desc",
           "SceneDesc": "swr_scene_desc", "GltfOpts": "swr_gltf_opts", "SceneInfo": "swr_scene_info",
           "TextureView": "swr_texture_view", "PrimitiveView": "swr_primitive_view", "MeshView": "swr_mesh_view",
           "NodeView": "swr_node_view", "MaterialView": "swr_material_view", "SceneHostView": "swr_scene_host_view",
           "Camera": "swr_camera", "RendererOpts": "swr_renderer_opts", "FrameStats": "swr_frame_stats",
           "ViewDesc": "swr_view_desc", "BatchOpts": "swr_batch_opts", "ServerOpts": "swr_server_opts",
           "Request": "swr_request", "Completion": "swr_completion", "ServerStats": "swr_server_stats",
           "BatchTuning": "swr_batch_tuning"}


def test_struct_layouts_match_header(tmp_path):
    """Every ctypes structure of the binding has the size and field offsets
    the C compiler gives the header's struct (a field added on one side only
    shifts what the other reads)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "swr.h"', "int main(void) {"]
    for py, cn in MIRRORS.items():
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (py, cn))
        for f in getattr(swr, py)._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (py, f[0], cn, f[0]))
    lines.append("return 0; }")
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    declared = set(re.findall(r"\}\s*(swr_[a-z0-9_]+)\s*;", open(os.path.join(ROOT, "include", "swr.h")).read()))
    assert set(MIRRORS.values()) <= declared
    checked = 0
    for line in filter(None, out):
        key, value = line.split()
        if "." in key:
            cls, field = key.split(".")
            got = getattr(getattr(swr, cls), field).offset
        else:
            got = C.sizeof(getattr(swr, key))
        assert got == int(value), (key, got, int(value))
        checked += 1
    assert checked > len(MIRRORS)
