"""The oracle's side of the glTF path (test infrastructure): a scene dict
(see scenes.py) for a document the tests wrote with DocBuilder, restating
what the reference's loader makes of it, so the oracle builds the scene
without the product's loader.

Restated from Scene::from_gltf (src/scene.rs:145-351): every document node
is kept in document order, its local transform is Node::get_local_transform
(src/scene.rs:396-419) and its world transform is composed from the roots
with the identity as the roots' parent (compute_final_transform_recursive,
src/scene.rs:356-381) using the oracle's glam restatement; primitives read
positions and indices, optional normals, tangents and texcoords
(src/scene.rs:439-495); materials follow Material::from_gltf
(src/scene.rs:690-780) and get_texture_and_sampler (src/scene.rs:637-688):
one texture per image URI, typed by the first material slot that asks for it
(materials in document order, slots base colour, metallic-roughness, normal,
emissive, occlusion, transmission), buffer-view images skipped, the sampler's
wrap modes or Repeat.

Accessor decoding is the gltf 1.4.1 crate's, restated from the glTF 2.0
specification: little-endian components at byteOffset + i * byteStride,
sparse substitutions applied, normalized integer texcoords divided by the
type's maximum in f32 (into_f32), indices widened to u32. Texels are the
images' RGBA8 samples (PNG is lossless, so decoding is exact)."""
import ctypes as C

import numpy as np

import oracle

COMP = {5120: "<i1", 5121: "<u1", 5122: "<i2", 5123: "<u2", 5125: "<u4", 5126: "<f4"}
NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
WRAP = {33071: 2, 33648: 1, 10497: 0}
TEX_SRGB, TEX_NORMAL, TEX_MR, TEX_LINEAR = 0, 1, 2, 4


def read_accessor(doc, binary, index):
    a = doc["accessors"][index]
    dt = np.dtype(COMP[a["componentType"]])
    n, count = NCOMP[a["type"]], a["count"]
    out = np.zeros((count, n), dt)
    if "bufferView" in a:
        v = doc["bufferViews"][a["bufferView"]]
        off = v.get("byteOffset", 0) + a.get("byteOffset", 0)
        stride = v.get("byteStride", 0) or dt.itemsize * n
        for k in range(count):
            out[k] = np.frombuffer(binary, dt, n, off + k * stride)
    sp = a.get("sparse")
    if sp:
        iv = doc["bufferViews"][sp["indices"]["bufferView"]]
        idt = np.dtype(COMP[sp["indices"]["componentType"]])
        idx = np.frombuffer(binary, idt, sp["count"], iv.get("byteOffset", 0) + sp["indices"].get("byteOffset", 0))
        vv = doc["bufferViews"][sp["values"]["bufferView"]]
        vals = np.frombuffer(binary, dt, sp["count"] * n, vv.get("byteOffset", 0) + sp["values"].get("byteOffset", 0))
        out[idx.astype(np.int64)] = vals.reshape(-1, n)
    return out, a.get("normalized", False)


def to_f32(arr, normalized):
    if arr.dtype == np.float32:
        return arr.astype(np.float32)
    if not normalized:
        return arr.astype(np.float32)
    mx = np.float32(np.iinfo(arr.dtype).max)
    f = arr.astype(np.float32) / mx
    if np.issubdtype(arr.dtype, np.signedinteger):
        f = np.maximum(f, np.float32(-1.0))
    return f.astype(np.float32)


def _mat_local(node):
    L = oracle.lib()
    out = (C.c_float * 16)()
    if "matrix" in node:
        m = (C.c_float * 16)(*node["matrix"])
        L.oracle_node_local(None, None, None, m, out)
    else:
        t = (C.c_float * 3)(*node.get("translation", (0.0, 0.0, 0.0)))
        r = (C.c_float * 4)(*node.get("rotation", (0.0, 0.0, 0.0, 1.0)))
        s = (C.c_float * 3)(*node.get("scale", (1.0, 1.0, 1.0)))
        L.oracle_node_local(t, r, s, None, out)
    return np.array(out[:], np.float32)


def _mat_mul(a, b):
    out = (C.c_float * 16)()
    oracle.lib().oracle_mat4_mul((C.c_float * 16)(*a), (C.c_float * 16)(*b), out)
    return np.array(out[:], np.float32)


def scene_dict(builder, images, cubemap_faces, cubemap_face_size, voxel_grid_size=128, specular_samples=64,
               brdf_lut_size=128):
    """builder: the DocBuilder whose document the product loads; images:
    {uri: (h, w, 4) uint8 RGBA samples}."""
    doc, binary = builder.doc, bytes(builder.bin)
    # Materials and their textures.
    textures, by_uri, mats = [], {}, []

    def texref(info, ttype):
        if info is None:
            return None
        t = doc["textures"][info["index"]]
        img = doc["images"][t["source"]]
        if "uri" not in img:
            return None
        uri = img["uri"]
        if uri not in by_uri:
            rgba = np.asarray(images[uri], np.uint32)
            h, w = rgba.shape[:2]
            packed = (rgba[..., 0] << 24) | (rgba[..., 1] << 16) | (rgba[..., 2] << 8) | rgba[..., 3]
            by_uri[uri] = len(textures)
            textures.append({"width": w, "height": h, "type": ttype, "rgba8": packed.reshape(-1).astype(np.uint32)})
        ws = wt = 0
        if "sampler" in t:
            smp = doc["samplers"][t["sampler"]]
            ws, wt = WRAP[smp.get("wrapS", 10497)], WRAP[smp.get("wrapT", 10497)]
        return (by_uri[uri], ws, wt)

    for m in doc.get("materials", []):
        pbr = m.get("pbrMetallicRoughness", {})
        tr = m.get("extensions", {}).get("KHR_materials_transmission")
        d = {"base_color_factor": tuple(pbr.get("baseColorFactor", (1.0, 1.0, 1.0, 1.0))),
             "metallic": pbr.get("metallicFactor", 1.0), "roughness": pbr.get("roughnessFactor", 1.0),
             "emissive_factor": tuple(m.get("emissiveFactor", (0.0, 0.0, 0.0))),
             "alpha_mask": m.get("alphaMode") == "MASK", "alpha_cutoff": m.get("alphaCutoff", 0.5)}
        d["base_color"] = texref(pbr.get("baseColorTexture"), TEX_SRGB)
        d["metallic_roughness"] = texref(pbr.get("metallicRoughnessTexture"), TEX_MR)
        d["normal"] = texref(m.get("normalTexture"), TEX_NORMAL)
        d["emissive"] = texref(m.get("emissiveTexture"), TEX_SRGB)
        d["occlusion"] = texref(m.get("occlusionTexture"), TEX_LINEAR)
        d["occlusion_strength"] = m["occlusionTexture"].get("strength", 1.0) if "occlusionTexture" in m else 1.0
        if tr is not None:
            d["has_transmission"] = True
            d["transmission"] = tr.get("transmissionFactor", 0.0)
            d["transmission_texture"] = texref(tr.get("transmissionTexture"), TEX_LINEAR)
        mats.append(d)
    if not mats:
        # glTF's default material (the reference would index its empty list).
        mats.append({"metallic": 1.0, "roughness": 1.0})
    meshes = []
    for mesh in doc["meshes"]:
        prims = []
        for p in mesh["primitives"]:
            at = p["attributes"]
            pos, _ = read_accessor(doc, binary, at["POSITION"])
            idx, _ = read_accessor(doc, binary, p["indices"])
            q = {"positions": pos.astype(np.float32), "indices": idx.reshape(-1).astype(np.uint32),
                 "material": p.get("material", -1), "normals": None, "tangents": None, "texcoords": None}
            if "NORMAL" in at:
                q["normals"] = read_accessor(doc, binary, at["NORMAL"])[0].astype(np.float32)
            if "TANGENT" in at:
                q["tangents"] = read_accessor(doc, binary, at["TANGENT"])[0].astype(np.float32)
            if "TEXCOORD_0" in at:
                q["texcoords"] = to_f32(*read_accessor(doc, binary, at["TEXCOORD_0"]))
            prims.append(q)
        meshes.append(prims)
    nodes = doc.get("nodes", [])
    local = [_mat_local(n) for n in nodes]
    world = [l.copy() for l in local]
    children = {c for n in nodes for c in n.get("children", [])}
    ident = np.eye(4, dtype=np.float32).reshape(16)

    def walk(i, parent):
        world[i] = _mat_mul(parent, local[i])
        for c in nodes[i].get("children", []):
            walk(c, world[i])

    for i in range(len(nodes)):
        if i not in children:
            walk(i, ident)
    out_nodes = [{"world": world[i], "local": local[i], "mesh": n.get("mesh", -1)} for i, n in enumerate(nodes)]
    return {"meshes": meshes, "nodes": out_nodes, "materials": mats, "textures": textures, "cubemap": cubemap_faces,
            "cubemap_face_size": cubemap_face_size, "voxel_grid_size": voxel_grid_size,
            "specular_samples": specular_samples, "brdf_lut_size": brdf_lut_size}
