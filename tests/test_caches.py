"""Cache files of the reference's scene load: the GGX-prefiltered environment
(assets/cubemap.ggx: "GGX0", version 1, face width, face height, mip count,
then a brotli stream of the u32 texels; src/texture.rs:425-554) and the baked
voxel GI (<scene>.gi: "VGI0", version 8, grid dimensions, then a brotli
stream of n^3 x 4 x (r, g, b, w) f32; src/gi.rs:30-117). The library writes
and reads them through the system's brotli; pyarrow's brotli codec is the
independent encoder and decoder these tests check the files with. As in the
reference, a file with another magic, version, size or payload length, or a
corrupt stream, is ignored: the table is computed and the file rewritten."""
import struct

import numpy as np
import pytest

import scenes
import swr

pa = pytest.importorskip("pyarrow")


def texture_arrays(t):
    data = np.ctypeslib.as_array(t.data, (t.data_len,)).copy()
    meta = {k: np.ctypeslib.as_array(getattr(t, k), (t.mip_count,)).copy()
            for k in ("mip_offsets", "mip_widths", "mip_heights", "array_stride")}
    return data, meta, (t.width, t.height, t.type, t.mip_count, tuple(t.width_height_vec))


def brotli(payload, level=6):
    return pa.Codec("brotli", compression_level=level).compress(payload, asbytes=True)


def unbrotli(stream, size):
    return pa.decompress(stream, decompressed_size=size, codec="brotli", asbytes=True)


def scene_or_skip(sd, **kw):
    s = swr.Scene(sd, host_only=True, **kw)
    info = s.info()
    if swr.CACHE_NO_CODEC in (info.gi_cache, info.ggx_cache):
        pytest.skip("no brotli library on this system")
    return s


def test_ggx_cache_written_then_loaded(tmp_path):
    path = tmp_path / "cubemap.ggx"
    sd = scenes.small_scene()
    a = scene_or_skip(sd, ggx_cache=path)
    assert a.info().ggx_cache == swr.CACHE_WRITTEN
    data, meta, shape = texture_arrays(a.export().cubemap_specular)
    raw = path.read_bytes()
    w, h, mips = shape[0], shape[1], shape[3]
    assert struct.unpack("<4sIIII", raw[:20]) == (b"GGX0", 1, w, h, mips)
    assert np.array_equal(np.frombuffer(unbrotli(raw[20:], data.nbytes), "<u4"), data)
    b = scene_or_skip(sd, ggx_cache=path)
    assert b.info().ggx_cache == swr.CACHE_LOADED
    data_b, meta_b, shape_b = texture_arrays(b.export().cubemap_specular)
    assert np.array_equal(data_b, data) and shape_b == shape
    for k in meta:
        assert np.array_equal(meta_b[k], meta[k]), k
    # Everything else is computed as without a cache.
    c = swr.Scene(sd, host_only=True)
    assert c.info().ggx_cache == swr.CACHE_NONE
    assert np.array_equal(texture_arrays(c.export().cubemap_specular)[0], data)
    for s in (a, b, c):
        s.close()


def test_ggx_cache_from_another_encoder_is_used(tmp_path):
    """A file whose stream another brotli encoder wrote (pyarrow, quality 6
    and 11) is read, and its texels are what the scene shades with (the
    reference trusts a cache whose header and size match)."""
    sd = scenes.small_scene()
    ref = swr.Scene(sd, host_only=True)
    _, meta, shape = texture_arrays(ref.export().cubemap_specular)
    w, h, mips = shape[0], shape[1], shape[3]
    texels = np.random.default_rng(3).integers(0, 2 ** 32, w * h * 6 * mips, dtype=np.uint64).astype("<u4")
    for level in (6, 11):
        path = tmp_path / ("q%d.ggx" % level)
        path.write_bytes(struct.pack("<4sIIII", b"GGX0", 1, w, h, mips) + brotli(texels.tobytes(), level))
        s = scene_or_skip(sd, ggx_cache=path)
        assert s.info().ggx_cache == swr.CACHE_LOADED
        data, meta_s, shape_s = texture_arrays(s.export().cubemap_specular)
        assert np.array_equal(data, texels) and shape_s == shape
        for k in meta:
            assert np.array_equal(meta_s[k], meta[k]), k
        s.close()
    ref.close()


@pytest.mark.parametrize("defect", ["magic", "version", "width", "mips", "short_payload", "long_payload",
                                    "corrupt", "truncated", "header_only"])
def test_stale_ggx_cache_is_recomputed(tmp_path, defect):
    sd = scenes.small_scene()
    ref = swr.Scene(sd, host_only=True)
    good, _, shape = texture_arrays(ref.export().cubemap_specular)
    w, h, mips = shape[0], shape[1], shape[3]
    head = [b"GGX0", 1, w, h, mips]
    payload = np.full(good.size, 0x11223344, "<u4").tobytes()
    if defect == "magic":
        head[0] = b"GGX1"
    elif defect == "version":
        head[1] = 2
    elif defect == "width":
        head[2] = w * 2
    elif defect == "mips":
        head[4] = mips - 1
    elif defect == "short_payload":
        payload = payload[:-4]
    elif defect == "long_payload":
        payload = payload + b"\0\0\0\0"
    stream = brotli(payload)
    if defect == "corrupt":
        stream = bytes([stream[0] ^ 0xFF]) + stream[1:]
    elif defect == "truncated":
        stream = stream[: len(stream) // 2]
    elif defect == "header_only":
        stream = b""
    path = tmp_path / "cubemap.ggx"
    path.write_bytes(struct.pack("<4sIIII", *head) + stream)
    s = scene_or_skip(sd, ggx_cache=path)
    assert s.info().ggx_cache == swr.CACHE_WRITTEN
    assert np.array_equal(texture_arrays(s.export().cubemap_specular)[0], good)
    # The file now holds the computed table.
    raw = path.read_bytes()
    assert struct.unpack("<4sIIII", raw[:20]) == (b"GGX0", 1, w, h, mips)
    assert np.array_equal(np.frombuffer(unbrotli(raw[20:], good.nbytes), "<u4"), good)
    s.close()
    ref.close()


def gi_file(n, coeffs):
    return struct.pack("<4sIIII", b"VGI0", 8, n, n, n) + brotli(coeffs.astype("<f4").tobytes())


def test_gi_cache_gives_a_host_only_scene_its_grid(tmp_path):
    sd = scenes.small_scene(voxel=8)
    n = 8
    coeffs = np.random.default_rng(5).standard_normal(n ** 3 * 16).astype(np.float32)
    path = tmp_path / "scene.gi"
    path.write_bytes(gi_file(n, coeffs))
    s = scene_or_skip(sd, gi=True, gi_cache=path)
    assert s.info().gi_cache == swr.CACHE_LOADED
    v = s.export()
    assert v.voxel_size == n
    grid = np.ctypeslib.as_array(v.voxel_gi_sh4, (n ** 3 * 16,))
    assert np.array_equal(grid.view(np.uint32), coeffs.view(np.uint32))
    # save_gi_cache writes the same payload back (another encoder, same bytes
    # after decoding).
    out = tmp_path / "again.gi"
    s.save_gi_cache(out)
    raw = out.read_bytes()
    assert struct.unpack("<4sIIII", raw[:20]) == (b"VGI0", 8, n, n, n)
    assert unbrotli(raw[20:], coeffs.nbytes) == coeffs.astype("<f4").tobytes()
    s.close()


@pytest.mark.parametrize("defect", ["dims", "version", "payload"])
def test_stale_gi_cache_needs_the_bake(tmp_path, defect):
    """Without a usable file a host-only scene cannot bake (the bake runs on
    the device): the scene is refused."""
    n = 8
    sd = scenes.small_scene(voxel=n)
    coeffs = np.zeros(n ** 3 * 16, np.float32)
    raw = gi_file(n, coeffs)
    if defect == "dims":
        raw = struct.pack("<4sIIII", b"VGI0", 8, n, n, n + 1) + raw[20:]
    elif defect == "version":
        raw = struct.pack("<4sIIII", b"VGI0", 7, n, n, n) + raw[20:]
    else:
        raw = raw[:20] + brotli(coeffs[:-1].tobytes())
    path = tmp_path / "scene.gi"
    path.write_bytes(raw)
    with pytest.raises(swr.SwrError) as e:
        swr.Scene(sd, host_only=True, gi=True, gi_cache=path)
    assert e.value.status == swr.SWR_INVALID_ARG
    assert b"GI cache" in swr.lib().swr_last_error()


def test_save_errors(tmp_path):
    s = swr.Scene(scenes.small_scene(), host_only=True)
    with pytest.raises(swr.SwrError) as e:
        s.save_gi_cache(tmp_path / "x.gi")
    assert e.value.status == swr.SWR_INVALID_ARG
    with pytest.raises(swr.SwrError) as e:
        s.save_ggx_cache(tmp_path / "missing_dir" / "cubemap.ggx")
    assert e.value.status == swr.SWR_IO_ERROR
    s.close()


def test_gltf_gi_cache_path_follows_the_reference(tmp_path):
    """gi_cache=True: the glTF file's path with extension .gi
    (Path::with_extension, src/main.rs:249)."""
    from gltf_helpers import DocBuilder
    n = 8
    b = DocBuilder()
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    prim = {"attributes": {"POSITION": b.accessor(tri, 5126, "VEC3")},
            "indices": b.accessor(np.array([0, 1, 2], np.uint16), 5123, "SCALAR")}
    b.doc["meshes"] = [{"primitives": [prim]}]
    b.doc["nodes"] = [{"mesh": 0}]
    b.doc["scenes"] = [{"nodes": [0]}]
    gl = b.write(str(tmp_path / "tri"), "glb")
    coeffs = np.random.default_rng(6).standard_normal(n ** 3 * 16).astype(np.float32)
    (tmp_path / "tri.gi").write_bytes(gi_file(n, coeffs))
    rng = np.random.default_rng(1)
    s = swr.Scene.load_gltf(gl, cubemap_faces=scenes.cubemap_faces(rng, 8), cubemap_face_size=8, voxel_grid_size=n,
                            host_only=True, gi=True, gi_cache=True)
    info = s.info()
    if info.gi_cache == swr.CACHE_NO_CODEC:
        pytest.skip("no brotli library on this system")
    assert info.gi_cache == swr.CACHE_LOADED
    grid = np.ctypeslib.as_array(s.export().voxel_gi_sh4, (n ** 3 * 16,))
    assert np.array_equal(grid.view(np.uint32), coeffs.view(np.uint32))
    s.close()
