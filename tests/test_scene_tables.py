"""Load-time tables: every table the product's scene admission exports
(swr_scene_export) against the oracle's own build of the same input, bit for
bit. The oracle restates the reference's load path (mips, BRDF LUT, SH4,
GGX prefilter, generated normals and tangents, bounding spheres, scene
bounds, materials, light, voxel sun visibility) and its render camera from
the reference's sources; both sides run on the same host libm, so the
tables must be identical. CPU only (host-only scenes)."""
import copy
import ctypes as C

import numpy as np
import pytest

import gltf_reference
import oracle
import scenes
import swr
from test_gltf import build_doc, cube_faces, load, FACE


def _arr(ptr, n, dt):
    if n == 0:
        return np.zeros(0, dt)
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), shape=(n,)).copy()


def _bits(x):
    return np.ascontiguousarray(x).view(np.uint32)


def _tex(t):
    m = t.mip_count
    return {"head": (t.width, t.height, t.type, t.mip_count, t.data_len, tuple(_bits(np.array(t.width_height_vec[:],
                                                                                            np.float32)))),
            "offs": _arr(t.mip_offsets, m, np.uint32).tolist(), "ws": _arr(t.mip_widths, m, np.uint32).tolist(),
            "hs": _arr(t.mip_heights, m, np.uint32).tolist(), "stride": _arr(t.array_stride, m, np.uint32).tolist(),
            "data": _arr(t.data, t.data_len, np.uint32)}


def table_differences(pv, ov):
    """Names of the exported tables that differ between two host views."""
    out = []
    for f in ("primitive_count", "mesh_count", "node_count", "material_count", "texture_count", "voxel_size"):
        if getattr(pv, f) != getattr(ov, f):
            out.append(f)
    if out:
        return out
    for i in range(pv.primitive_count):
        a, b = pv.primitives[i], ov.primitives[i]
        nv = a.vertex_count
        for f, n, dt in (("positions", 4 * nv, np.float32), ("normals", 4 * nv, np.float32),
                         ("tangents", 4 * nv, np.float32), ("texcoords", 2 * nv, np.float32),
                         ("indices", a.index_count, np.uint32)):
            if not np.array_equal(_bits(_arr(getattr(a, f), n, dt)), _bits(_arr(getattr(b, f), n, dt))):
                out.append("primitive %d %s" % (i, f))
        if (a.vertex_count, a.index_count, a.material, a.triangle_id_base) != \
                (b.vertex_count, b.index_count, b.material, b.triangle_id_base):
            out.append("primitive %d header" % i)
        if not np.array_equal(_bits(np.array(a.sphere[:], np.float32)), _bits(np.array(b.sphere[:], np.float32))):
            out.append("primitive %d sphere" % i)
    for i in range(pv.mesh_count):
        a, b = pv.meshes[i], ov.meshes[i]
        for f, n in (("primitives", a.primitive_count), ("opaque", a.opaque_count),
                     ("translucent", a.translucent_count)):
            if _arr(getattr(a, f), n, np.uint32).tolist() != _arr(getattr(b, f), n, np.uint32).tolist():
                out.append("mesh %d %s" % (i, f))
    for i in range(pv.node_count):
        if bytes(pv.nodes[i]) != bytes(ov.nodes[i]):
            out.append("node %d" % i)
    for i in range(pv.material_count):
        if bytes(pv.materials[i]) != bytes(ov.materials[i]):
            out.append("material %d" % i)
    pairs = [("texture %d" % i, pv.textures[i], ov.textures[i]) for i in range(pv.texture_count)]
    pairs += [(n, getattr(pv, n), getattr(ov, n)) for n in ("cubemap", "cubemap_specular", "brdf_lut")]
    for name, a, b in pairs:
        ta, tb = _tex(a), _tex(b)
        for k in ta:
            if k == "data":
                if ta[k].shape != tb[k].shape or not np.array_equal(ta[k], tb[k]):
                    out.append("%s texels" % name)
            elif ta[k] != tb[k]:
                out.append("%s %s" % (name, k))
    for f in ("irradiance_sh", "light_direction", "light_color", "voxel_world_min", "voxel_world_max",
              "voxel_gi_sh4_const"):
        if np.ctypeslib.as_array(getattr(pv, f)).tobytes() != np.ctypeslib.as_array(getattr(ov, f)).tobytes():
            out.append(f)
    n = pv.voxel_size ** 3
    if not np.array_equal(_bits(_arr(pv.voxel_light_intensity, n, np.float32)),
                          _bits(_arr(ov.voxel_light_intensity, n, np.float32))):
        out.append("voxel_light_intensity")
    return out


def bounds_differ(info, obounds):
    mn, mx, c, diag = obounds
    return (tuple(info.bounds_min) != mn or tuple(info.bounds_max) != mx or tuple(info.bounds_center) != c
            or np.float32(info.bounds_diagonal) != np.float32(diag))


def mixed_scene():
    """Every texture type and odd texture sizes, generated normals and
    tangents, missing texcoords, given tangents, scaled and rotated nodes, a
    node without a mesh, a material with texture slots the reference drops
    (transmission texture without the extension, occlusion strength without
    an occlusion texture)."""
    rng = np.random.default_rng(5)

    def tex(w, h, t):
        return {"width": w, "height": h, "type": t, "rgba8": rng.integers(0, 2 ** 32, w * h, dtype=np.uint64)
                .astype(np.uint32)}

    P, F = scenes.icosphere(2)
    UV = scenes.spherical_uv(P)
    P2, UV2, F2 = scenes.grid(7, 5)

    def rot(a, s, t):
        c, sn = np.cos(a), np.sin(a)
        M = np.array([[c * s, 0, sn * s, t[0]], [0, s * 1.3, 0, t[1]], [-sn * s, 0, c * s, t[2]], [0, 0, 0, 1]],
                     np.float32)
        return M.T.reshape(16)

    n2 = len(P2)
    return {"meshes": [[{"positions": P * 1.5, "normals": None, "texcoords": UV, "indices": F, "material": 0},
                        {"positions": P + np.float32(2), "normals": None, "texcoords": None, "indices": F,
                         "material": 2}],
                       [{"positions": P2, "normals": None, "tangents": None, "texcoords": UV2, "indices": F2,
                         "material": 1}],
                       [{"positions": P2, "normals": np.tile(np.float32([0, 0, 1]), (n2, 1)),
                         "tangents": np.tile(np.float32([1, 0, 0, -1]), (n2, 1)), "texcoords": UV2 * 3,
                         "indices": F2, "material": -1}]],
            "nodes": [{"world": rot(0.3, 1.0, (0, 0, 0)), "local": rot(0.1, 1.0, (1, 0, 0)), "mesh": 0},
                      {"world": rot(1.3, 2.0, (3, 1, -2)), "mesh": 1}, {"world": rot(-0.7, 0.5, (-3, 2, 1)), "mesh": 2},
                      {"world": rot(0.0, 1.0, (5, 5, 5)), "mesh": -1}],
            "materials": [{"metallic": 0.3, "roughness": 0.6, "base_color": (0, 0, 1), "metallic_roughness": (1, 1, 2),
                           "normal": (2, 0, 0), "emissive": (3, 2, 1), "emissive_factor": (1, 0.5, 0.25),
                           "occlusion": (4, 0, 0), "occlusion_strength": 0.7, "alpha_mask": True,
                           "alpha_cutoff": 0.3},
                          {"metallic": 0.9, "roughness": 0.2, "base_color": (5, 0, 0), "has_transmission": True,
                           "transmission": 0.6, "transmission_texture": (4, 0, 0)},
                          {"metallic": 0.1, "roughness": 0.9, "occlusion_strength": 0.4, "transmission": 0.5,
                           "transmission_texture": (4, 0, 0)}],
            "textures": [tex(64, 32, 0), tex(33, 17, 2), tex(16, 64, 1), tex(5, 3, 0), tex(8, 8, 4), tex(1, 1, 0)],
            "cubemap": scenes.cubemap_faces(rng, 16), "cubemap_face_size": 16, "voxel_grid_size": 16,
            "specular_samples": 8, "brdf_lut_size": 16}


SCENES = {
    "small": lambda: scenes.small_scene(seed=3),
    "translucent": lambda: scenes.translucent_scene(),
    "mixed": mixed_scene,
    "textured": lambda: scenes.textured_scene(),
    "c1_spheres": lambda: scenes.spheres_scene(),
    "c2_reduced": lambda: scenes.stress_scene(seed=2, triangles=200_000, n_textures=2, tex_size=512)[0],
}


@pytest.mark.parametrize("name", list(SCENES))
def test_exported_tables_equal_the_oracle_build(name):
    sd = SCENES[name]()
    p = swr.Scene(sd, host_only=True)
    o = oracle.Scene(sd)
    assert table_differences(p.export(), o.view) == []
    assert not bounds_differ(p.info(), o.bounds)


def test_planted_texel_change_is_detected():
    sd = scenes.small_scene(seed=3)
    p = swr.Scene(sd, host_only=True)
    sd2 = copy.deepcopy(sd)
    sd2["textures"][0]["rgba8"] = sd2["textures"][0]["rgba8"] ^ np.uint32(1 << 8)
    diff = table_differences(p.export(), oracle.Scene(sd2).view)
    assert "texture 0 texels" in diff


def test_loaded_document_tables_equal_the_oracle_build(tmp_path):
    # The oracle builds the document's scene from the document itself
    # (gltf_reference), not through the product's loader.
    rng = np.random.default_rng(1)
    b, img, mr = build_doc(str(tmp_path), rng)
    s = load(b.write(str(tmp_path / "d"), "glb"))
    sd = gltf_reference.scene_dict(b, {"base.png": img, "orm.png": mr}, cube_faces(), FACE, voxel_grid_size=8,
                                   specular_samples=4, brdf_lut_size=8)
    o = oracle.Scene(sd)
    assert table_differences(s.export(), o.view) == []
    assert not bounds_differ(s.info(), o.bounds)


def test_cameras_equal_the_oracle_camera():
    rng = np.random.default_rng(1)
    for _ in range(3000):
        p = tuple(map(float, rng.normal(0, 50, 3).astype(np.float32)))
        t = tuple(map(float, rng.normal(0, 50, 3).astype(np.float32)))
        fov = float(np.float32(rng.uniform(0.2, 2.5)))
        w, h = int(rng.integers(1, 4000)), int(rng.integers(1, 3000))
        far = float(np.float32(rng.uniform(1, 1000)))
        assert bytes(swr.make_camera(p, t, fov, w, h, far)) == bytes(oracle.camera(p, t, fov, w, h, far))


@pytest.mark.parametrize("name", ["translucent", "mixed"])
def test_oracle_bvh_sun_visibility_equals_brute_force(name):
    o = oracle.Scene(SCENES[name]())
    np.testing.assert_array_equal(oracle.sun_visibility(o.view, threads=4, brute=True),
                                  oracle.sun_visibility(o.view, threads=4))
