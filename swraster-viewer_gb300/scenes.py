"""Seeded synthetic scenes with the shapes of the benchmark configurations.

No glTF sample assets are available, so scenes are generated: icospheres and
displaced grids with f32 positions/normals/UVs and u32 indices, seeded
value-noise textures and a seeded RGBA8 cubemap (fed as raw faces instead of
the reference's JPEG cross, because JPEG decoding is not bit-reproducible).

A scene is a plain dict consumed by swr.Scene:
  meshes:    [[{positions (V,3), normals (V,3)|None, texcoords (V,2)|None,
                indices (3T,), material}]]
  nodes:     [{world (16,) column-major, local, mesh}]
  materials: [{base_color_factor, metallic, roughness, base_color: (tex, wrap_s, wrap_t), ...}]
  textures:  [{width, height, type, rgba8 (H*W,) uint32 R-in-MSB}]
  cubemap, cubemap_face_size, voxel_grid_size, specular_samples, brdf_lut_size
"""
import math

import numpy as np

TEX_SRGB, TEX_NORMAL, TEX_METALLIC_ROUGHNESS, TEX_CUBEMAP, TEX_LINEAR = 0, 1, 2, 3, 4
WRAP_REPEAT, WRAP_MIRRORED = 0, 1


def icosphere(subdiv):
    """Unit icosphere, counter-clockwise outward faces (glTF front faces)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    verts = [np.array(p, np.float64) / np.linalg.norm(p) for p in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        faces = nf
    P = np.array(verts, np.float32)
    F = np.array(faces, np.uint32).reshape(-1)
    return P, F


def spherical_uv(P):
    u = 0.5 + np.arctan2(P[:, 2], P[:, 0]) / (2.0 * math.pi)
    v = 0.5 - np.arcsin(np.clip(P[:, 1], -1.0, 1.0)) / math.pi
    return np.stack([u, v], 1).astype(np.float32)


def grid(n, m):
    """Unit grid in the xy plane, z = 0, facing +z (counter-clockwise)."""
    xs = np.linspace(-0.5, 0.5, n + 1, dtype=np.float32)
    ys = np.linspace(-0.5, 0.5, m + 1, dtype=np.float32)
    X, Y = np.meshgrid(xs, ys)
    P = np.stack([X.ravel(), Y.ravel(), np.zeros(X.size, np.float32)], 1).astype(np.float32)
    UV = np.stack([(X.ravel() + 0.5), (0.5 - Y.ravel())], 1).astype(np.float32)
    i = np.arange(n)[None, :] + (n + 1) * np.arange(m)[:, None]
    a, b, c, d = i, i + 1, i + n + 1, i + n + 2
    F = np.stack([a, b, d, a, d, c], -1).reshape(-1).astype(np.uint32)
    return P, UV, F


def value_noise(rng, size, cells, channels=3):
    """Bilinear value noise in [0, 1]: (size, size, channels) float32."""
    lat = rng.random((cells + 1, cells + 1, channels), dtype=np.float32)
    x = np.linspace(0, cells, size, endpoint=False, dtype=np.float32)
    i = np.floor(x).astype(np.int64)
    f = (x - i)[:, None]
    f = f * f * (3 - 2 * f)
    row0 = lat[i] * (1 - f[:, :, None]) + lat[i + 1] * f[:, :, None]
    out = row0[:, i] * (1 - f[None, :, :]) + row0[:, i + 1] * f[None, :, :]
    return out.astype(np.float32)


def pack_rgba8(rgb, alpha=255):
    c = np.clip(np.round(rgb * 255.0), 0, 255).astype(np.uint32)
    a = np.full(c.shape[:-1], alpha, np.uint32)
    return ((c[..., 0] << 24) | (c[..., 1] << 16) | (c[..., 2] << 8) | a).reshape(-1).astype(np.uint32)


def noise_texture(rng, size, cells=16, tint=None):
    n = value_noise(rng, size, cells)
    if tint is not None:
        n = 0.35 + 0.65 * n * np.asarray(tint, np.float32)
    return {"width": size, "height": size, "type": TEX_SRGB, "rgba8": pack_rgba8(n)}


def normal_map_texture(rng, size, cells=8, strength=0.6):
    """Tangent-space normal map of seeded value noise, (n + 1) / 2 in RGB."""
    n = value_noise(rng, size, cells, channels=2)
    x = (n[..., 0] - 0.5) * (2.0 * strength)
    y = (n[..., 1] - 0.5) * (2.0 * strength)
    z = np.sqrt(np.clip(1.0 - x * x - y * y, 0.05, 1.0))
    inv = 1.0 / np.sqrt(x * x + y * y + z * z)
    nm = np.stack([x * inv, y * inv, z * inv], -1)
    return {"width": size, "height": size, "type": TEX_NORMAL, "rgba8": pack_rgba8(nm * 0.5 + 0.5)}


def metallic_roughness_texture(rng, size, cells=8):
    """glTF metallic-roughness layout: G roughness, B metallic (R unused)."""
    n = value_noise(rng, size, cells)
    return {"width": size, "height": size, "type": TEX_METALLIC_ROUGHNESS, "rgba8": pack_rgba8(n)}


def occlusion_texture(rng, size, cells=8):
    """Ambient occlusion in R, in [0.3, 1]."""
    n = 0.3 + 0.7 * value_noise(rng, size, cells)
    return {"width": size, "height": size, "type": TEX_LINEAR, "rgba8": pack_rgba8(n)}


def emissive_texture(rng, size, cells=8):
    n = value_noise(rng, size, cells) * rng.uniform(0.2, 1.0, 3).astype(np.float32)
    return {"width": size, "height": size, "type": TEX_SRGB, "rgba8": pack_rgba8(n)}


def cubemap_faces(rng, size):
    """Six seeded faces (+X,-X,+Y,-Y,+Z,-Z): a vertical sky gradient plus noise."""
    faces = []
    for face in range(6):
        n = value_noise(rng, size, 8)
        base = np.array([0.45, 0.6, 0.85], np.float32) if face != 3 else np.array([0.25, 0.22, 0.2], np.float32)
        if face == 2:
            base = np.array([0.7, 0.8, 1.0], np.float32)
        ramp = np.linspace(1.1, 0.7, size, dtype=np.float32)[:, None, None]
        img = np.clip(base[None, None, :] * ramp + 0.35 * (n - 0.5), 0.0, 1.0)
        faces.append(pack_rgba8(img))
    return np.concatenate(faces)


def translate_scale(center, s):
    m = np.eye(4, dtype=np.float32)
    m[0, 0] = m[1, 1] = m[2, 2] = s
    m[:3, 3] = center
    return m.T.reshape(16).copy()  # column-major


def spheres_scene(seed=1, count=64, subdiv=3, box=10.0, radius=(0.5, 2.0), tex_size=256, cube_size=128,
                  voxel=128, specular_samples=64, brdf_lut_size=128):
    """Plain method, small: `count` icospheres (subdivision `subdiv`) with
    centres uniform in [-box, box]^3, radii uniform in `radius` (node scale),
    one shared value-noise base-colour texture, per-mesh metallic/roughness
    uniform in [0, 1], a seeded cubemap."""
    rng = np.random.default_rng(seed)
    P, F = icosphere(subdiv)
    UV = spherical_uv(P)
    tex = noise_texture(rng, tex_size)
    meshes, nodes, mats = [], [], []
    centers = rng.uniform(-box, box, (count, 3)).astype(np.float32)
    radii = rng.uniform(radius[0], radius[1], count).astype(np.float32)
    for i in range(count):
        mats.append({"base_color_factor": (1.0, 1.0, 1.0, 1.0), "metallic": float(rng.random()),
                     "roughness": float(rng.random()), "base_color": (0, WRAP_REPEAT, WRAP_REPEAT)})
        meshes.append([{"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": i}])
        w = translate_scale(centers[i], radii[i])
        nodes.append({"world": w, "local": w, "mesh": i})
    return {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": [tex],
            "cubemap": cubemap_faces(rng, cube_size), "cubemap_face_size": cube_size, "voxel_grid_size": voxel,
            "specular_samples": specular_samples, "brdf_lut_size": brdf_lut_size}


def textured_scene(seed=13, count=12, subdiv=2, box=4.0, tex_size=64, cube_size=16, voxel=24):
    """Opaque materials with every texture slot of pbrMetallicRoughness in
    play: base colour, metallic-roughness, normal map (generated tangents),
    emissive texture and occlusion texture, each present or absent per
    material, with mixed wrap modes; icospheres (normals given) and displaced
    grids (normals generated)."""
    rng = np.random.default_rng(seed)
    P, F = icosphere(subdiv)
    UV = spherical_uv(P)
    GP, GUV, GF = grid(6, 6)
    GP = GP.copy()
    GP[:, 2] = 0.1 * np.sin(GP[:, 0] * 9.0) * np.cos(GP[:, 1] * 7.0)
    textures = [noise_texture(rng, tex_size), metallic_roughness_texture(rng, tex_size),
                normal_map_texture(rng, tex_size), emissive_texture(rng, tex_size // 2),
                occlusion_texture(rng, tex_size), normal_map_texture(rng, tex_size * 2, strength=0.9)]
    wraps = (WRAP_REPEAT, WRAP_MIRRORED, 2)

    def ref(t):
        return (t, int(rng.choice(wraps)), int(rng.choice(wraps)))

    meshes, nodes, mats = [], [], []
    centers = rng.uniform(-box, box, (count, 3)).astype(np.float32)
    radii = rng.uniform(0.8, 2.0, count).astype(np.float32)
    for i in range(count):
        m = {"base_color_factor": tuple(float(x) for x in rng.uniform(0.4, 1.0, 3)) + (1.0,),
             "metallic": float(rng.uniform(0.2, 1.0)), "roughness": float(rng.uniform(0.2, 1.0)),
             "base_color": ref(0)}
        if i % 3 != 2:
            m["metallic_roughness"] = ref(1)
        if i % 4 != 3:
            m["normal"] = ref(2 if i % 2 == 0 else 5)
        if i % 2 == 1:
            m["emissive"] = ref(3)
            m["emissive_factor"] = tuple(float(x) for x in rng.uniform(0.2, 1.5, 3))
        elif i % 4 == 0:
            m["emissive_factor"] = (0.3, 0.2, 0.1)
        if i % 3 != 1:
            m["occlusion"] = ref(4)
            m["occlusion_strength"] = float(rng.uniform(0.3, 1.0))
        mats.append(m)
        if i % 3 == 0:
            prim = {"positions": GP, "normals": None, "texcoords": GUV * np.float32(3.0), "indices": GF,
                    "material": i}
            w = translate_scale(centers[i], 2.5 * radii[i])
        else:
            prim = {"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": i}
            w = translate_scale(centers[i], radii[i])
        meshes.append([prim])
        nodes.append({"world": w, "local": w, "mesh": i})
    return {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": textures,
            "cubemap": cubemap_faces(rng, cube_size), "cubemap_face_size": cube_size, "voxel_grid_size": voxel,
            "specular_samples": 16, "brdf_lut_size": 32}


def translucent_scene(seed=11, count=8, subdiv=2, box=4.0, tex_size=64, cube_size=16, voxel=32):
    """Opaque and translucent (KHR_materials_transmission) spheres, one mesh
    with an opaque and a translucent primitive, a large translucent plane
    through the scene and a translucent sphere instanced twice at the same
    place (equal sort keys)."""
    rng = np.random.default_rng(seed)
    P, F = icosphere(subdiv)
    UV = spherical_uv(P)
    tex = noise_texture(rng, tex_size)
    meshes, nodes, mats = [], [], []

    def mat(translucent, textured_transmission=False):
        m = {"base_color_factor": tuple(float(x) for x in rng.uniform(0.3, 1.0, 3)) + (1.0,),
             "metallic": float(rng.random()), "roughness": float(rng.uniform(0.1, 1.0)),
             "base_color": (0, WRAP_REPEAT, WRAP_REPEAT)}
        if translucent:
            m["has_transmission"] = 1
            m["transmission"] = float(rng.uniform(0.2, 0.95))
            if textured_transmission:
                m["transmission_texture"] = (0, WRAP_MIRRORED, WRAP_REPEAT)
        mats.append(m)
        return len(mats) - 1

    centers = rng.uniform(-box, box, (count, 3)).astype(np.float32)
    radii = rng.uniform(0.8, 2.0, count).astype(np.float32)
    for i in range(count):
        mi = mat(translucent=(i % 2 == 1), textured_transmission=(i % 4 == 3))
        meshes.append([{"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": mi}])
        w = translate_scale(centers[i], radii[i])
        nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
    # One mesh, two primitives: translucent outer shell listed first, opaque core second.
    shell, core = mat(True), mat(False)
    meshes.append([{"positions": P * np.float32(1.6), "normals": P.copy(), "texcoords": UV, "indices": F,
                    "material": shell},
                   {"positions": P * np.float32(0.7), "normals": P.copy(), "texcoords": UV, "indices": F,
                    "material": core}])
    w = translate_scale(np.zeros(3, np.float32), 1.0)
    nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
    # Large translucent plane facing the camera (+z), through the scene.
    GP, GUV, GF = grid(6, 6)
    gm = mat(True, textured_transmission=True)
    meshes.append([{"positions": GP, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (len(GP), 1)),
                    "texcoords": GUV, "indices": GF, "material": gm}])
    w = translate_scale(np.array([0.0, 0.0, 1.0], np.float32), 3.0 * box)
    nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
    # The same translucent sphere twice at one place.
    tm = mat(True)
    meshes.append([{"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": tm}])
    w = translate_scale(np.array([1.0, -0.5, 2.0], np.float32), 1.2)
    nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
    nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
    return {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": [tex],
            "cubemap": cubemap_faces(rng, cube_size), "cubemap_face_size": cube_size, "voxel_grid_size": voxel,
            "specular_samples": 16, "brdf_lut_size": 32}


class Bounds:
    """Scene bounds in the shape default_camera_params and sphere_camera read
    (bounds_center, bounds_diagonal), for bounds that do not come from
    swr_scene_get_info."""

    def __init__(self, center, diagonal):
        self.bounds_center = tuple(center)
        self.bounds_diagonal = diagonal


def default_camera_params(info, width, height, fov=math.pi / 3.0):
    """load_scene's default camera (src/main.rs:210-225): distance = scene
    diagonal along +z from the bounds centre, far = 2 * diagonal."""
    c = np.array(info.bounds_center[:], np.float32)
    d = float(info.bounds_diagonal)
    pos = (float(c[0]), float(c[1]), float(c[2] + np.float32(d)))
    return pos, (float(c[0]), float(c[1]), float(c[2])), fov, width, height, float(np.float32(d) * np.float32(2.0))


def small_scene(seed=7, count=6, subdiv=2, tex_size=64, cube_size=16, voxel=32):
    """A quick scene for tests: few spheres, small textures and grids."""
    return spheres_scene(seed=seed, count=count, subdiv=subdiv, box=4.0, radius=(0.5, 2.0), tex_size=tex_size,
                         cube_size=cube_size, voxel=voxel, specular_samples=16, brdf_lut_size=32)


_ICO_CACHE = {}


def _ico(subdiv):
    if subdiv not in _ICO_CACHE:
        P, F = icosphere(subdiv)
        _ICO_CACHE[subdiv] = (P, spherical_uv(P), F)
    return _ICO_CACHE[subdiv]


def _look_rotation(forward, up=(0.0, 1.0, 0.0)):
    f = forward / np.linalg.norm(forward)
    r = np.cross(f, up)
    if np.linalg.norm(r) < 1e-6:
        r = np.cross(f, (1.0, 0.0, 0.0))
    r /= np.linalg.norm(r)
    u = np.cross(r, f)
    return np.stack([r, u, -f], 1)  # columns: local x, y, z (z toward -forward)


def stress_scene(seed=2, triangles=2_000_000, width=3840, height=2160, fov=math.pi / 3.0, far=400.0,
                 n_textures=8, tex_size=2048, cube_size=128, voxel=128, area=(0.5, 5000.0), side_fraction=0.15,
                 specular_samples=64, brdf_lut_size=128, all_slots=False):
    """Plain method, large: `triangles` triangles in icospheres and displaced
    grids seen by a camera at the origin looking down -z.

    Each object draws its mean front-facing triangle screen area A
    log-uniformly from `area` px and gets about c / sqrt(A) triangles, so the
    per-object triangle area is log-uniform over 0.5-5000 px while the total
    coverage stays near 8x the screen. Objects centred on a frustum side
    hold about `side_fraction` of the triangles (all of them take the clip
    path); about 3% of the others cross the near plane. `n_textures` value-noise
    textures of `tex_size`^2 (full mip chains) are shared by the materials. With
    `all_slots` every material also carries a metallic-roughness, normal,
    emissive and occlusion texture (four more shared textures of each kind).
    Returns (scene dict, camera params)."""
    rng = np.random.default_rng(seed)
    near = far * 0.01
    fpx = (height / 2.0) / math.tan(fov / 2.0)
    aspect = width / height
    textures = [noise_texture(rng, tex_size, cells=32, tint=rng.uniform(0.4, 1.0, 3)) for _ in range(n_textures)]
    slot_base = len(textures)
    if all_slots:
        ssz = max(16, tex_size // 2)
        for make in (metallic_roughness_texture, normal_map_texture, emissive_texture, occlusion_texture):
            textures += [make(np.random.default_rng(seed * 7 + k), ssz) for k in range(4)]
    meshes, nodes, mats = [], [], []
    total = edge_tris = 0
    tan_y = math.tan(fov / 2.0)
    tan_x = tan_y * aspect
    side_planes = [np.array(p) / np.linalg.norm(p) for p in
                   ((1.0, 0.0, tan_x), (-1.0, 0.0, tan_x), (0.0, 1.0, tan_y), (0.0, -1.0, tan_y))]
    # c such that E[c / sqrt(A)] * objects ~= triangles with ~1000 tris per object.
    lo, hi = math.log(area[0]), math.log(area[1])
    e_inv_sqrt = (area[0] ** -0.5 - area[1] ** -0.5) / (0.5 * (hi - lo))
    c = 1000.0 / e_inv_sqrt
    while total < triangles:
        A = math.exp(rng.uniform(lo, hi))
        T = int(max(8, min(8192, round(c / math.sqrt(A)))))
        if total + T > triangles:
            T = max(8, triangles - total)
        # Objects centred on a frustum side plane are chosen so that they hold
        # about `side_fraction` of all triangles: their bounding spheres
        # intersect the frustum, so all their triangles take the reference's
        # clip path (src/renderer.rs:423-468). A few more objects cross the
        # near plane; the reference's view-space near plane (0, 0, -1, near)
        # is positive for every point in front of the camera
        # (src/rendercamera.rs:141), so those stay off the clip path.
        edge = edge_tris < side_fraction * (total + T)
        near_obj = not edge and rng.random() < 0.03
        z = math.exp(rng.uniform(math.log(near * 3.0), math.log(far * 0.8)))
        if edge:
            side = rng.integers(4)
            nx, ny = rng.uniform(-1.0, 1.0), rng.uniform(-1.0, 1.0)
            if side == 0: nx = 1.0
            elif side == 1: nx = -1.0
            elif side == 2: ny = 1.0
            else: ny = -1.0
        elif near_obj:
            z = near * rng.uniform(0.6, 2.0)  # crosses the near plane
            nx, ny = rng.uniform(-0.8, 0.8), rng.uniform(-0.8, 0.8)
        else:
            nx, ny = rng.uniform(-0.95, 0.95), rng.uniform(-0.95, 0.95)
        center = np.array([nx * z * aspect * math.tan(fov / 2), ny * z * math.tan(fov / 2), -z], np.float32)
        sphere = rng.random() < 0.5
        ti = int(rng.integers(n_textures))
        mats.append({"base_color_factor": (1.0, 1.0, 1.0, 1.0), "metallic": float(rng.random()),
                     "roughness": float(rng.random()), "base_color": (ti, WRAP_REPEAT, WRAP_REPEAT)})
        if all_slots:
            k = len(mats) % 4
            mats[-1].update({"metallic_roughness": (slot_base + k, WRAP_REPEAT, WRAP_REPEAT),
                             "normal": (slot_base + 4 + k, WRAP_REPEAT, WRAP_REPEAT),
                             "emissive": (slot_base + 8 + k, WRAP_MIRRORED, WRAP_REPEAT),
                             "emissive_factor": (0.4, 0.3, 0.2),
                             "occlusion": (slot_base + 12 + k, WRAP_REPEAT, WRAP_MIRRORED),
                             "occlusion_strength": 0.8})
        if sphere:
            sub = int(np.clip(round(math.log(max(T, 20) / 20.0, 4)), 0, 5))
            P, UV, F = _ico(sub)
            T = F.size // 3
            r_px = math.sqrt(A * T / (2.0 * math.pi))
            r = r_px * z / fpx
            bound = r * math.sqrt(3.0)  # bounding sphere of the unit icosphere's box, scaled
            M = np.eye(4, dtype=np.float32)
            M[:3, :3] *= r
            M[:3, 3] = center
            prim = {"positions": P, "normals": P.copy(), "texcoords": UV, "indices": F, "material": len(mats) - 1}
        else:
            n = max(2, int(round(math.sqrt(T / 2.0))))
            P, UV, F = grid(n, n)
            T = F.size // 3
            L_px = math.sqrt(A * T)
            L = L_px * z / fpx
            bound = L * math.sqrt(0.5 + 0.08 * 0.08)
            P = P.copy()
            P[:, 2] = 0.08 * np.sin(P[:, 0] * rng.uniform(4, 12)) * np.cos(P[:, 1] * rng.uniform(4, 12))
            UV = UV * np.float32(rng.integers(1, 6))
            to_cam = -center / np.linalg.norm(center)
            tilt = rng.normal(0, 0.5, 3)
            R = _look_rotation(-(to_cam + 0.6 * tilt))
            M = np.eye(4, dtype=np.float32)
            M[:3, :3] = R * L
            M[:3, 3] = center
            prim = {"positions": P, "normals": None, "texcoords": UV, "indices": F, "material": len(mats) - 1}
        meshes.append([prim])
        w = M.T.reshape(16).astype(np.float32).copy()
        nodes.append({"world": w, "local": w, "mesh": len(meshes) - 1})
        total += T
        # Triangles on the clip path: the object's bounding sphere crosses a
        # side plane (view space = world space for this camera).
        if any(abs(float(np.dot(pn, center))) < bound for pn in side_planes):
            edge_tris += T
    sd = {"meshes": meshes, "nodes": nodes, "materials": mats, "textures": textures,
          "cubemap": cubemap_faces(rng, cube_size), "cubemap_face_size": cube_size, "voxel_grid_size": voxel,
          "specular_samples": specular_samples, "brdf_lut_size": brdf_lut_size}
    cam = ((0.0, 0.0, 0.0), (0.0, 0.0, -1.0), fov, width, height, far)
    return sd, cam


def hetero_scenes(seed=21, count=16, tri_range=(10_000, 4_000_000), res_range=((640, 480), (3840, 2160)),
                  max_triangles=None):
    """Batched heterogeneous scenes: `count` seeded scenes with triangle counts
    log-uniform in `tri_range`, 1-8 textures of 512-2048 px each, one view per
    scene at a resolution between 640x480 and 3840x2160. Returns a list of
    (scene dict, camera params)."""
    rng = np.random.default_rng(seed)
    out = []
    widths = [640, 960, 1280, 1600, 1920, 2560, 3200, 3840]
    for i in range(count):
        t = int(math.exp(rng.uniform(math.log(tri_range[0]), math.log(tri_range[1]))))
        if max_triangles:
            t = min(t, max_triangles)
        w = int(rng.choice(widths))
        h = int(round(w * 9 / 16 / 2)) * 2 if w > 640 else 480
        ntex = int(rng.integers(1, 9))
        tsz = int(rng.choice([512, 1024, 2048]))
        sd, cam = stress_scene(seed=seed * 100 + i, triangles=t, width=w, height=h, n_textures=ntex, tex_size=tsz,
                               voxel=128)
        out.append((sd, cam))
    return out


def sphere_camera(rng, info, width, height, rmin=15.0, rmax=40.0, fov=math.pi / 3.0):
    """A camera on a sphere of radius in [rmin, rmax] around the scene centre,
    looking at the centre (far plane beyond the scene)."""
    c = np.array(info.bounds_center[:], np.float64)
    u = rng.normal(size=3)
    u /= np.linalg.norm(u)
    r = rng.uniform(rmin, rmax)
    pos = c + u * r
    far = float(r + info.bounds_diagonal)
    return (tuple(map(float, pos)), tuple(map(float, c)), fov, width, height, far)
