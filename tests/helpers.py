"""Tiny hand-made scenes for known-answer tests."""
import numpy as np

import scenes


def tri_scene(triangles, normals=True):
    """One mesh per triangle (3 vertices each, world = identity)."""
    rng = np.random.default_rng(0)
    tex = scenes.noise_texture(rng, 8)
    meshes, nodes = [], []
    eye = np.eye(4, dtype=np.float32).reshape(16)
    for i, t in enumerate(triangles):
        P = np.asarray(t, np.float32).reshape(3, 3)
        n = np.cross(P[1] - P[0], P[2] - P[0])
        n = n / (np.linalg.norm(n) or 1.0)
        prim = {"positions": P, "normals": np.tile(n, (3, 1)).astype(np.float32) if normals else None,
                "texcoords": np.array([[0, 0], [1, 0], [0, 1]], np.float32),
                "indices": np.array([0, 1, 2], np.uint32), "material": 0}
        meshes.append([prim])
        nodes.append({"world": eye, "local": eye, "mesh": i})
    return {"meshes": meshes, "nodes": nodes,
            "materials": [{"metallic": 0.2, "roughness": 0.7, "base_color": (0, 0, 0)}], "textures": [tex],
            "cubemap": scenes.cubemap_faces(rng, 8), "cubemap_face_size": 8, "voxel_grid_size": 8,
            "specular_samples": 4, "brdf_lut_size": 8}


BACKGROUND = np.uint64(2 ** 64 - 1)
