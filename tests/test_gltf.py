"""glTF loader (swr_scene_load_gltf): documents written by the test in the
three container forms, node hierarchy and TRS/matrix transforms, accessor
types (normalized texcoords, u8/u16 indices, strides, sparse), materials and
samplers, image decoding (PNG of every colour type and bit depth, Adam7;
baseline JPEG), and the loader's error reporting. CPU only (host-only scenes)."""
import os

import numpy as np
import pytest

import scenes
import swr
from gltf_helpers import DocBuilder, pack_rgba, write_jpeg, write_png

FACE = 8


def cube_faces():
    return scenes.cubemap_faces(np.random.default_rng(3), FACE)


def load(path, **kw):
    return swr.Scene.load_gltf(path, cubemap_faces=cube_faces(), cubemap_face_size=FACE, voxel_grid_size=8,
                               specular_samples=4, brdf_lut_size=8, host_only=True, **kw)


def tex_mip0(view, i):
    t = view.textures[i]
    return np.ctypeslib.as_array(t.data, (t.width * t.height,)).copy(), t.width, t.height, t.type


def rgba_image(rng, h, w):
    return rng.integers(0, 256, (h, w, 4), dtype=np.uint8)


def build_doc(tmp, rng):
    """Three meshes, four nodes (hierarchy, TRS and matrix), two materials, textures."""
    b = DocBuilder()
    img = rgba_image(rng, 6, 5)
    write_png(os.path.join(tmp, "base.png"), img, 6, 8)
    mr = rgba_image(rng, 4, 4)
    write_png(os.path.join(tmp, "orm.png"), mr, 6, 8, interlace=True)
    quad_p = np.array([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, 1, 0]], np.float32)
    quad_n = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))
    quad_uv = np.array([[0, 65535], [65535, 65535], [65535, 0], [0, 0]], np.uint16)
    quad_i = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    m0 = {"attributes": {"POSITION": b.accessor(quad_p, 5126, "VEC3", stride=16),
                         "NORMAL": b.accessor(quad_n, 5126, "VEC3"),
                         "TEXCOORD_0": b.accessor(quad_uv, 5123, "VEC2", normalized=True)},
          "indices": b.accessor(quad_i, 5123, "SCALAR"), "material": 0}
    P, F = scenes.icosphere(1)
    m1 = {"attributes": {"POSITION": b.accessor(P, 5126, "VEC3")},
          "indices": b.accessor(F.astype(np.uint8), 5121, "SCALAR"), "material": 1}
    # Sparse: a quad whose vertex 2 is moved by the sparse substitution.
    sp_base = b.accessor(quad_p, 5126, "VEC3")
    si = b.accessor(np.array([2], np.uint8), 5121, "SCALAR")
    sv = b.accessor(np.array([[3, 3, 0]], np.float32), 5126, "VEC3")
    acc = b.doc["accessors"][sp_base]
    acc["sparse"] = {"count": 1, "indices": {"bufferView": b.doc["accessors"][si]["bufferView"], "componentType": 5121},
                     "values": {"bufferView": b.doc["accessors"][sv]["bufferView"]}}
    m2 = {"attributes": {"POSITION": sp_base}, "indices": b.accessor(np.array([0, 1, 2], np.uint32), 5125, "SCALAR")}
    b.doc["meshes"] = [{"primitives": [m0]}, {"primitives": [m1]}, {"primitives": [m2]}]
    b.doc["images"] = [{"uri": "base.png"}, {"uri": "orm.png"}]
    b.doc["samplers"] = [{"wrapS": 33071, "wrapT": 33648}]
    b.doc["textures"] = [{"source": 0}, {"source": 1, "sampler": 0}]
    b.doc["materials"] = [
        {"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}, "baseColorFactor": [0.5, 0.25, 1.0, 1.0],
                                  "metallicFactor": 0.25},
         "alphaMode": "MASK", "alphaCutoff": 0.3, "emissiveFactor": [0.1, 0.2, 0.3]},
        {"pbrMetallicRoughness": {"metallicRoughnessTexture": {"index": 1}, "roughnessFactor": 0.5},
         "occlusionTexture": {"index": 1, "strength": 0.75},
         "extensions": {"KHR_materials_transmission": {"transmissionFactor": 0.6}}},
    ]
    b.doc["nodes"] = [
        {"translation": [1, 2, 3], "rotation": [0, 1, 0, 0], "scale": [2, 2, 2], "children": [1]},
        {"matrix": [1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, -5, 1], "mesh": 0},
        {"scale": [0.5, 0.5, 0.5], "mesh": 1},
        {"mesh": 2},
    ]
    b.doc["scenes"] = [{"nodes": [0, 2, 3]}]
    return b, img, mr


def snapshot(scene):
    """Comparable content of an exported host view."""
    v = scene.export()
    out = {"nodes": [], "prims": [], "mats": [], "texs": []}
    for i in range(v.node_count):
        n = v.nodes[i]
        out["nodes"].append((tuple(n.transform), n.mesh))
    for i in range(v.primitive_count):
        p = v.primitives[i]
        pos = np.ctypeslib.as_array(p.positions, (p.vertex_count * 4,)).copy()
        uv = np.ctypeslib.as_array(p.texcoords, (p.vertex_count * 2,)).copy()
        idx = np.ctypeslib.as_array(p.indices, (p.index_count,)).copy()
        out["prims"].append((pos.tobytes(), uv.tobytes(), idx.tobytes(), p.material))
    for i in range(v.material_count):
        m = v.materials[i]
        out["mats"].append((tuple(m.base_color_factor), m.metallic_factor, m.roughness_factor,
                            tuple(m.emissive_factor), m.occlusion_strength, m.alpha_cutoff, m.transmission,
                            m.is_alpha_tested, m.is_translucent, tuple(m.tex), tuple(m.wrap_s), tuple(m.wrap_t)))
    for i in range(v.texture_count):
        d, w, h, t = tex_mip0(v, i)
        out["texs"].append((d.tobytes(), w, h, t))
    return out


def test_document_forms_agree_and_match_the_source(tmp_path):
    rng = np.random.default_rng(1)
    b, img, mr = build_doc(str(tmp_path), rng)
    snaps = []
    for form in ("bin", "data", "glb"):
        s = load(b.write(str(tmp_path / ("doc_" + form)), form))
        snaps.append(snapshot(s))
        s.close()
    assert snaps[0] == snaps[1] == snaps[2]
    sn = snaps[0]
    # World transforms: node 0 = T * R(180 deg about y) * S(2); node 1 = node 0 * translate(0, 0, -5).
    w0 = np.array([[-2, 0, 0, 1], [0, 2, 0, 2], [0, 0, -2, 3], [0, 0, 0, 1]], np.float32)
    w1 = w0 @ np.array([[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, -5], [0, 0, 0, 1]], np.float32)
    assert np.array_equal(np.array(sn["nodes"][0][0], np.float32), w0.T.reshape(16))
    assert np.array_equal(np.array(sn["nodes"][1][0], np.float32), w1.T.reshape(16))
    assert [n[1] for n in sn["nodes"]] == [-1, 0, 1, 2]
    # Quad texcoords: normalized u16 read as v / 65535.
    uv = np.frombuffer(sn["prims"][0][1], np.float32).reshape(-1, 2)
    assert np.array_equal(uv, np.array([[0, 1], [1, 1], [1, 0], [0, 0]], np.float32))
    # Icosphere: generated texcoords are zero; u8 indices widened.
    assert not np.frombuffer(sn["prims"][1][1], np.float32).any()
    assert np.array_equal(np.frombuffer(sn["prims"][1][2], np.uint32), scenes.icosphere(1)[1])
    # Sparse substitution moved vertex 2 to (3, 3, 0).
    pos = np.frombuffer(sn["prims"][2][0], np.float32).reshape(-1, 4)
    assert np.array_equal(pos[2, :3], np.array([3, 3, 0], np.float32))
    # Materials: factors, alpha mask with a base texture, transmission, shared image typed by first use.
    m0, m1 = sn["mats"]
    assert m0[0] == (0.5, 0.25, 1.0, 1.0) and m0[1] == 0.25 and m0[2] == 1.0 and m0[7] == 1 and m0[8] == 0
    assert abs(m0[5] - 0.3) < 1e-7
    assert m1[8] == 1 and abs(m1[6] - 0.6) < 1e-7 and abs(m1[4] - 0.75) < 1e-7
    assert m1[9][1] == m1[9][4] == 1  # metallic-roughness and occlusion share texture 1
    assert m1[10][1] == swr.WRAP_CLAMP_TO_EDGE and m1[11][1] == swr.WRAP_MIRRORED_REPEAT
    assert sn["texs"][1][3] == 2  # SWR_TEX_METALLIC_ROUGHNESS: the first use decides
    # Texels: PNG pixels packed with R in the most significant byte.
    assert np.array_equal(np.frombuffer(sn["texs"][0][0], np.uint32), pack_rgba(img))
    assert np.array_equal(np.frombuffer(sn["texs"][1][0], np.uint32), pack_rgba(mr))


PNG_CASES = [  # (colour type, bit depth, interlace)
    (0, 1, False), (0, 2, True), (0, 4, False), (0, 8, False), (0, 16, True), (2, 8, False), (2, 16, False),
    (3, 1, False), (3, 4, True), (3, 8, False), (4, 8, True), (4, 16, False), (6, 8, False), (6, 16, True)]


def expected_rgba(samples, ctype, depth, palette=None, trns_vals=None):
    h, w, _ = samples.shape
    s = samples.astype(np.int64)
    to8 = (lambda v: (v + 128) // 257) if depth == 16 else (lambda v: v * 255 // ((1 << depth) - 1))
    out = np.zeros((h, w, 4), np.int64)
    out[..., 3] = 255
    if ctype == 3:
        out[..., :3] = palette[s[..., 0]]
        out[..., 3] = trns_vals[s[..., 0]]
    elif ctype == 0:
        out[..., :3] = to8(s[..., :1])
        if trns_vals is not None:
            out[..., 3] = np.where(s[..., 0] == trns_vals, 0, 255)
    elif ctype == 4:
        out[..., :3] = to8(s[..., :1])
        out[..., 3] = to8(s[..., 1])
    elif ctype == 2:
        out[..., :3] = to8(s)
    else:
        out[...] = to8(s)
    return out.astype(np.uint8)


def test_png_colour_types_and_depths(tmp_path):
    rng = np.random.default_rng(7)
    b = DocBuilder()
    quad = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    prim = {"attributes": {"POSITION": b.accessor(quad, 5126, "VEC3")},
            "indices": b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR"), "material": 0}
    b.doc["meshes"] = [{"primitives": [prim]}]
    b.doc["nodes"] = [{"mesh": 0}]
    b.doc["scenes"] = [{"nodes": [0]}]
    b.doc["images"], b.doc["textures"], b.doc["materials"] = [], [], []
    expect = []
    for k, (ct, depth, il) in enumerate(PNG_CASES):
        h, w = 7 + k % 3, 9 + k % 4
        ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ct]
        hi = (1 << depth) if ct != 3 else min(1 << depth, 13)
        s = rng.integers(0, hi, (h, w, ch))
        palette = trns = trns_vals = None
        if ct == 3:
            palette = rng.integers(0, 256, (hi, 3))
            trns_vals = np.full(hi, 255)
            trns_vals[: hi // 2] = rng.integers(0, 256, hi // 2)
            trns = bytes(trns_vals[: hi // 2].astype(np.uint8))
        elif ct == 0:
            trns_vals = int(s[0, 0, 0])
            trns = int(trns_vals).to_bytes(2, "big")
        name = "img%02d.png" % k
        write_png(str(tmp_path / name), s, ct, depth, palette=palette, trns=trns, interlace=il)
        expect.append(expected_rgba(s, ct, depth, palette, trns_vals))
        b.doc["images"].append({"uri": name})
        b.doc["textures"].append({"source": k})
        b.doc["materials"].append({"pbrMetallicRoughness": {"baseColorTexture": {"index": k}}})
    sc = load(b.write(str(tmp_path / "pngs"), "bin"))
    v = sc.export()
    assert v.texture_count == len(PNG_CASES)
    for k, e in enumerate(expect):
        d, w, h, _ = tex_mip0(v, k)
        assert (w, h) == (e.shape[1], e.shape[0])
        assert np.array_equal(d, pack_rgba(e)), "PNG case %s" % (PNG_CASES[k],)
    sc.close()


def subsampled_reconstruction(rgb):
    """What a 4:2:0 round trip gives at best: chroma averaged over 2x2 by the
    encoder, replicated by the decoder (JFIF colour transforms)."""
    h, w = rgb.shape[:2]
    x = rgb.astype(np.float64)
    r, g, b = x[..., 0], x[..., 1], x[..., 2]
    y = 0.299 * r + 0.587 * g + 0.114 * b
    cb = -0.168736 * r - 0.331264 * g + 0.5 * b + 128
    cr = 0.5 * r - 0.418688 * g - 0.081312 * b + 128

    def sub(p):
        pad = np.pad(p, ((0, -h % 16), (0, -w % 16)), mode="edge")
        q = pad.reshape(pad.shape[0] // 2, 2, pad.shape[1] // 2, 2).mean(axis=(1, 3))
        return np.repeat(np.repeat(q, 2, 0), 2, 1)[:h, :w] - 128

    cb, cr = sub(cb), sub(cr)
    out = np.stack([y + 1.402 * cr, y - 0.344136 * cb - 0.714136 * cr, y + 1.772 * cb], -1)
    return np.clip(np.rint(out), 0, 255)


@pytest.mark.parametrize("subsample,restart,grey", [(False, 0, False), (True, 3, False), (False, 2, True)])
def test_baseline_jpeg(tmp_path, subsample, restart, grey):
    rng = np.random.default_rng(5)
    n = scenes.value_noise(rng, 24, 3)[:21, :19]
    rgb = np.clip(np.rint(n * 255), 0, 255).astype(np.uint8)
    src = rgb[..., 0] if grey else rgb
    write_jpeg(str(tmp_path / "t.jpg"), src, subsample=subsample, restart=restart)
    b = DocBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b.doc["meshes"] = [{"primitives": [{"attributes": {"POSITION": b.accessor(tri, 5126, "VEC3")},
                                        "indices": b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR")}]}]
    b.doc["nodes"] = [{"mesh": 0}]
    b.doc["images"] = [{"uri": "t.jpg"}]
    b.doc["textures"] = [{"source": 0}]
    b.doc["materials"] = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}]
    sc = load(b.write(str(tmp_path / "j"), "bin"))
    d, w, h, _ = tex_mip0(sc.export(), 0)
    assert (w, h) == (19, 21)
    got = np.stack([(d >> 24) & 255, (d >> 16) & 255, (d >> 8) & 255, d & 255], -1).reshape(21, 19, 4).astype(int)
    want = np.repeat(src[..., None], 3, -1) if grey else src
    if subsample:
        want = subsampled_reconstruction(src)
    err = np.abs(got[..., :3] - want.astype(int)).max()
    assert (got[..., 3] == 255).all()
    assert err <= 3, err
    sc.close()


def test_cubemap_from_cross_image(tmp_path):
    faces = cube_faces().reshape(6, FACE, FACE)
    cross = np.zeros((3 * FACE, 4 * FACE), np.uint32)
    for f, (cx, cy) in enumerate([(2, 1), (0, 1), (1, 0), (1, 2), (1, 1), (3, 1)]):
        cross[cy * FACE:(cy + 1) * FACE, cx * FACE:(cx + 1) * FACE] = faces[f]
    rgba = np.stack([(cross >> 24) & 255, (cross >> 16) & 255, (cross >> 8) & 255, cross & 255], -1)
    write_png(str(tmp_path / "cube.png"), rgba, 6, 8)
    rng = np.random.default_rng(2)
    b, _, _ = build_doc(str(tmp_path), rng)
    path = b.write(str(tmp_path / "c"), "glb")
    s1 = swr.Scene.load_gltf(path, cubemap_path=str(tmp_path / "cube.png"), voxel_grid_size=8, specular_samples=4,
                             brdf_lut_size=8, host_only=True)
    s2 = load(path)
    c1, c2 = s1.export().cubemap, s2.export().cubemap
    a1 = np.ctypeslib.as_array(c1.data, (c1.data_len,))
    a2 = np.ctypeslib.as_array(c2.data, (c2.data_len,))
    assert np.array_equal(a1, a2)
    s1.close()
    s2.close()


def expect_error(path, status, words, **kw):
    with pytest.raises(swr.SwrError) as e:
        load(path, **kw)
    assert e.value.status == status, str(e.value)
    assert words.lower() in str(e.value).lower()


def test_loader_errors(tmp_path):
    expect_error(str(tmp_path / "missing.gltf"), swr.SWR_IO_ERROR, "failed to load gltf")
    (tmp_path / "bad.gltf").write_text("{ not json")
    expect_error(str(tmp_path / "bad.gltf"), swr.SWR_IO_ERROR, "failed to load gltf")
    rng = np.random.default_rng(4)
    b, _, _ = build_doc(str(tmp_path), rng)
    del b.doc["meshes"][0]["primitives"][0]["indices"]
    expect_error(b.write(str(tmp_path / "noidx"), "bin"), swr.SWR_BAD_SCENE, "no indices")
    b, _, _ = build_doc(str(tmp_path), rng)
    b.doc["scenes"] = []
    expect_error(b.write(str(tmp_path / "noscene"), "data"), swr.SWR_BAD_SCENE, "no scenes")
    b, _, _ = build_doc(str(tmp_path), rng)
    b.doc["images"][0]["uri"] = "absent.png"
    expect_error(b.write(str(tmp_path / "noimg"), "bin"), swr.SWR_IO_ERROR, "absent.png")
    with pytest.raises(swr.SwrError) as e:
        swr.Scene.load_gltf(b.write(str(tmp_path / "nocube"), "glb"), host_only=True)
    assert e.value.status == swr.SWR_INVALID_ARG


def test_malformed_documents_are_rejected(tmp_path):
    """Malformed inputs found by fuzzing the loader under AddressSanitizer:
    each is an error, never an out-of-bounds read or a runaway allocation."""
    rng = np.random.default_rng(6)
    # A bufferView offset below zero (its sum with the length used to wrap).
    b, _, _ = build_doc(str(tmp_path), rng)
    b.doc["bufferViews"][0]["byteOffset"] = -8
    expect_error(b.write(str(tmp_path / "negoff"), "glb"), swr.SWR_BAD_SCENE, "past its buffer")
    # A stride so large the last element's offset would wrap.
    b, _, _ = build_doc(str(tmp_path), rng)
    b.doc["bufferViews"][0]["byteStride"] = 2 ** 62
    expect_error(b.write(str(tmp_path / "stride"), "glb"), swr.SWR_BAD_SCENE, "past its buffer")
    # Counts beyond the document's bytes, and numbers beyond int64.
    for count in (10 ** 12, 1e300):
        b, _, _ = build_doc(str(tmp_path), rng)
        b.doc["accessors"][0]["count"] = count
        with pytest.raises(swr.SwrError):
            load(b.write(str(tmp_path / "count"), "data"))
    # A buffer URI naming a directory.
    (tmp_path / "dir.bin").mkdir()
    b, _, _ = build_doc(str(tmp_path), rng)
    doc = b.write(str(tmp_path / "dirbuf"), "bin")
    text = open(doc).read().replace("geom%20data.bin", "dir.bin")
    open(doc, "w").write(text)
    expect_error(doc, swr.SWR_IO_ERROR, "cannot open")
    # A JPEG scan naming Huffman table 15 (tables are 0-3).
    rgb = rng.integers(0, 256, (16, 16, 3)).astype(np.uint8)
    write_jpeg(str(tmp_path / "t.jpg"), rgb)
    data = bytearray((tmp_path / "t.jpg").read_bytes())
    sos = data.index(b"\xff\xda")
    data[sos + 6] = 0xF0  # first component: DC table 15
    (tmp_path / "t.jpg").write_bytes(bytes(data))
    b = DocBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b.doc["meshes"] = [{"primitives": [{"attributes": {"POSITION": b.accessor(tri, 5126, "VEC3")},
                                        "indices": b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR")}]}]
    b.doc["nodes"] = [{"mesh": 0}]
    b.doc["images"] = [{"uri": "t.jpg"}]
    b.doc["textures"] = [{"source": 0}]
    b.doc["materials"] = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}]
    expect_error(b.write(str(tmp_path / "j"), "bin"), swr.SWR_IO_ERROR, "huffman table id")


@pytest.mark.gpu
def test_loaded_scene_renders_like_the_oracle(tmp_path):
    # A loaded document (alpha-masked textured quad, translucent sphere,
    # sparse-accessor triangle) through the kernels and the oracle.
    # The oracle builds the scene from the document itself (gltf_reference).
    import gltf_reference
    from test_gpu_parity import compare
    rng = np.random.default_rng(9)
    b, img, mr = build_doc(str(tmp_path), rng)
    s = swr.Scene.load_gltf(b.write(str(tmp_path / "r"), "glb"), cubemap_faces=cube_faces(), cubemap_face_size=FACE,
                            voxel_grid_size=16, specular_samples=8, brdf_lut_size=16)
    s.source = gltf_reference.scene_dict(b, {"base.png": img, "orm.png": mr}, cube_faces(), FACE, voxel_grid_size=16,
                                         specular_samples=8, brdf_lut_size=16)
    cam = swr.make_camera(*scenes.default_camera_params(s.info(), 200, 150))
    compare(s, cam, 200, 150)
    s.close()


def test_zero_accessor_larger_than_the_buffers_loads(tmp_path):
    # A POSITION accessor without a bufferView starts as zeros (glTF 2.0
    # 3.6.2); sparse substitutions set three of its 100 vertices. Its count
    # exceeds the buffer's bytes, which is valid for such an accessor.
    b = DocBuilder()
    si = b.accessor(np.array([0, 1, 2], np.uint8), 5121, "SCALAR")
    sv = b.accessor(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), 5126, "VEC3")
    idx = b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR")
    b.doc["accessors"].append({"componentType": 5126, "count": 100, "type": "VEC3",
                               "sparse": {"count": 3,
                                          "indices": {"bufferView": b.doc["accessors"][si]["bufferView"],
                                                      "componentType": 5121},
                                          "values": {"bufferView": b.doc["accessors"][sv]["bufferView"]}}})
    pos = len(b.doc["accessors"]) - 1
    b.doc["meshes"] = [{"primitives": [{"attributes": {"POSITION": pos}, "indices": idx}]}]
    b.doc["nodes"] = [{"mesh": 0}]
    assert len(b.bin) < 100
    s = load(b.write(str(tmp_path / "z"), "glb"))
    p = s.export().primitives[0]
    assert p.vertex_count == 100
    P = np.ctypeslib.as_array(p.positions, (400,)).reshape(100, 4)
    np.testing.assert_array_equal(P[:3, :3], [[0, 0, 0], [1, 0, 0], [0, 1, 0]])
    assert not P[3:, :3].any()
    s.close()


def _jpeg_texels(tmp_path, name):
    b = DocBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    b.doc["meshes"] = [{"primitives": [{"attributes": {"POSITION": b.accessor(tri, 5126, "VEC3")},
                                        "indices": b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR")}]}]
    b.doc["nodes"] = [{"mesh": 0}]
    b.doc["images"] = [{"uri": name}]
    b.doc["textures"] = [{"source": 0}]
    b.doc["materials"] = [{"pbrMetallicRoughness": {"baseColorTexture": {"index": 0}}}]
    sc = load(b.write(str(tmp_path / (name + "_doc")), "bin"))
    d, w, h, _ = tex_mip0(sc.export(), 0)
    sc.close()
    return d, w, h


@pytest.mark.parametrize("shape,subsample,restart", [((21, 19, 3), False, 0), ((40, 37, 3), True, 0),
                                                     ((33, 50, 3), True, 4), ((21, 19), False, 3),
                                                     ((64, 48, 3), False, 7)])
def test_progressive_jpeg_equals_baseline(tmp_path, shape, subsample, restart):
    # A progressive file (DC first and refinement scans, luma AC split into
    # two spectral bands, successive approximation from bit 2 to bit 0, end-
    # of-band runs, restart intervals) carries the coefficients of the
    # baseline file written from the same image: the decoder must give
    # identical texels for both.
    rng = np.random.default_rng(sum(shape) + restart)
    img = rng.integers(0, 256, shape).astype(np.uint8)
    if len(shape) == 3:
        img[::3] = (scenes.value_noise(rng, max(shape[:2]), 4)[:shape[0], :shape[1]] * 255).astype(np.uint8)[::3]
    write_jpeg(str(tmp_path / "b.jpg"), img, subsample=subsample, restart=restart)
    write_jpeg(str(tmp_path / "p.jpg"), img, subsample=subsample, restart=restart, progressive=True)
    assert (tmp_path / "p.jpg").read_bytes()[2:].find(b"\xff\xc2") >= 0
    db, w, h = _jpeg_texels(tmp_path, "b.jpg")
    dp, w2, h2 = _jpeg_texels(tmp_path, "p.jpg")
    assert (w, h) == (w2, h2) == (shape[1], shape[0])
    np.testing.assert_array_equal(dp, db)
