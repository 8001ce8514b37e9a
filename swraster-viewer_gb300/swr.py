"""ctypes binding of libswr (include/swr.h).

The binding is thin: it mirrors the C structures and wraps the handles in
small classes that free them. It has no fallback: if libswr.so is missing the
import of `lib()` raises.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.environ.get("SWR_LIBRARY") or os.path.join(HERE, "libswr.so")

SWR_OK, SWR_INVALID_ARG, SWR_NO_MEMORY, SWR_OVERFLOW, SWR_TIMEOUT = 0, 1, 2, 3, 4
SWR_CUDA_ERROR, SWR_IO_ERROR, SWR_BAD_SCENE, SWR_UNSUPPORTED, SWR_BUSY = 5, 6, 7, 8, 9
TEX_SRGB, TEX_NORMAL, TEX_METALLIC_ROUGHNESS, TEX_CUBEMAP, TEX_LINEAR = 0, 1, 2, 3, 4
WRAP_REPEAT, WRAP_MIRRORED_REPEAT, WRAP_CLAMP_TO_EDGE = 0, 1, 2
RSQRT_IEEE, RSQRT_AARCH64 = 0, 1
SCENE_HOST_ONLY = 1
SCENE_GI = 2
# swr_scene_info.gi_cache / ggx_cache
CACHE_NONE, CACHE_LOADED, CACHE_WRITTEN, CACHE_WRITE_FAILED, CACHE_NO_CODEC = 0, 1, 2, 3, 4

u32p = C.POINTER(C.c_uint32)
f32p = C.POINTER(C.c_float)


class TextureDesc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("type", C.c_uint32), ("reserved", C.c_uint32),
                ("rgba8", u32p)]


class TexRef(C.Structure):
    _fields_ = [("texture", C.c_int32), ("wrap_s", C.c_uint32), ("wrap_t", C.c_uint32), ("reserved", C.c_uint32)]


class MaterialDesc(C.Structure):
    _fields_ = [("base_color_factor", C.c_float * 4), ("metallic_factor", C.c_float),
                ("roughness_factor", C.c_float), ("emissive_factor", C.c_float * 3),
                ("occlusion_strength", C.c_float), ("alpha_cutoff", C.c_float), ("transmission", C.c_float),
                ("alpha_mask", C.c_uint32), ("has_transmission", C.c_uint32), ("base_color", TexRef),
                ("metallic_roughness", TexRef), ("normal", TexRef), ("emissive", TexRef), ("occlusion", TexRef),
                ("transmission_texture", TexRef)]


class PrimitiveDesc(C.Structure):
    _fields_ = [("vertex_count", C.c_uint32), ("index_count", C.c_uint32), ("positions", f32p), ("normals", f32p),
                ("tangents", f32p), ("texcoords", f32p), ("indices", u32p), ("material", C.c_int32),
                ("reserved", C.c_uint32)]


class MeshDesc(C.Structure):
    _fields_ = [("primitive_count", C.c_uint32), ("reserved", C.c_uint32),
                ("primitives", C.POINTER(PrimitiveDesc))]


class NodeDesc(C.Structure):
    _fields_ = [("world", C.c_float * 16), ("local", C.c_float * 16), ("mesh", C.c_int32), ("reserved", C.c_uint32)]


class SceneDesc(C.Structure):
    _fields_ = [("mesh_count", C.c_uint32), ("node_count", C.c_uint32), ("material_count", C.c_uint32),
                ("texture_count", C.c_uint32), ("meshes", C.POINTER(MeshDesc)), ("nodes", C.POINTER(NodeDesc)),
                ("materials", C.POINTER(MaterialDesc)), ("textures", C.POINTER(TextureDesc)),
                ("cubemap_face_size", C.c_uint32), ("voxel_grid_size", C.c_uint32), ("cubemap_faces", u32p),
                ("specular_samples", C.c_uint32), ("brdf_lut_size", C.c_uint32), ("gi_sh_scale", C.c_float),
                ("sky_visibility", C.c_float), ("host_threads", C.c_uint32), ("flags", C.c_uint32),
                ("gi_cache_path", C.c_char_p), ("ggx_cache_path", C.c_char_p)]


class GltfOpts(C.Structure):
    _fields_ = [("cubemap_faces", u32p), ("cubemap_face_size", C.c_uint32), ("voxel_grid_size", C.c_uint32),
                ("cubemap_path", C.c_char_p), ("specular_samples", C.c_uint32), ("brdf_lut_size", C.c_uint32),
                ("host_threads", C.c_uint32), ("flags", C.c_uint32), ("gi_cache_path", C.c_char_p),
                ("ggx_cache_path", C.c_char_p)]


class SceneInfo(C.Structure):
    _fields_ = [("triangle_count", C.c_uint64), ("vertex_count", C.c_uint64), ("device_bytes", C.c_uint64),
                ("node_count", C.c_uint32), ("draw_count", C.c_uint32), ("bounds_min", C.c_float * 3),
                ("bounds_max", C.c_float * 3), ("bounds_center", C.c_float * 3), ("bounds_diagonal", C.c_float),
                ("gi_cache", C.c_uint32), ("ggx_cache", C.c_uint32), ("precompute_host_texels", C.c_uint64)]


class TextureView(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("type", C.c_uint32), ("mip_count", C.c_uint32),
                ("data", u32p), ("data_len", C.c_uint64), ("mip_offsets", u32p), ("mip_widths", u32p),
                ("mip_heights", u32p), ("array_stride", u32p), ("width_height_vec", C.c_float * 4)]


class PrimitiveView(C.Structure):
    _fields_ = [("vertex_count", C.c_uint32), ("index_count", C.c_uint32), ("positions", f32p), ("normals", f32p),
                ("tangents", f32p), ("texcoords", f32p), ("indices", u32p), ("material", C.c_uint32),
                ("triangle_id_base", C.c_uint32), ("sphere", C.c_float * 4)]


class MeshView(C.Structure):
    _fields_ = [("primitive_count", C.c_uint32), ("opaque_count", C.c_uint32), ("translucent_count", C.c_uint32),
                ("reserved", C.c_uint32), ("primitives", u32p), ("opaque", u32p), ("translucent", u32p)]


class NodeView(C.Structure):
    _fields_ = [("transform", C.c_float * 16), ("sphere", C.c_float * 4), ("mesh", C.c_int32),
                ("triangle_id_base", C.c_uint32)]


class MaterialView(C.Structure):
    _fields_ = [("base_color_factor", C.c_float * 4), ("metallic_factor", C.c_float),
                ("roughness_factor", C.c_float), ("emissive_factor", C.c_float * 3),
                ("occlusion_strength", C.c_float), ("alpha_cutoff", C.c_float), ("transmission", C.c_float),
                ("is_alpha_tested", C.c_uint32), ("is_translucent", C.c_uint32), ("tex", C.c_int32 * 6),
                ("wrap_s", C.c_uint32 * 6), ("wrap_t", C.c_uint32 * 6)]


class SceneHostView(C.Structure):
    _fields_ = [("primitive_count", C.c_uint32), ("mesh_count", C.c_uint32), ("node_count", C.c_uint32),
                ("material_count", C.c_uint32), ("texture_count", C.c_uint32), ("voxel_size", C.c_uint32),
                ("primitives", C.POINTER(PrimitiveView)), ("meshes", C.POINTER(MeshView)),
                ("nodes", C.POINTER(NodeView)), ("materials", C.POINTER(MaterialView)),
                ("textures", C.POINTER(TextureView)), ("cubemap", TextureView), ("cubemap_specular", TextureView),
                ("brdf_lut", TextureView), ("irradiance_sh", (C.c_float * 3) * 4), ("light_direction", C.c_float * 3),
                ("light_color", C.c_float * 3), ("voxel_world_min", C.c_float * 3),
                ("voxel_world_max", C.c_float * 3), ("voxel_light_intensity", f32p),
                ("voxel_gi_sh4_const", (C.c_float * 4) * 4), ("voxel_gi_sh4", f32p)]


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("fov", C.c_float), ("width", C.c_float), ("height", C.c_float),
                ("one_over_width", C.c_float), ("one_over_height", C.c_float), ("near_plane", C.c_float),
                ("far_plane", C.c_float), ("yaw", C.c_float), ("pitch", C.c_float), ("roll", C.c_float),
                ("view_normal", C.c_float * 3), ("view", C.c_float * 16), ("projection", C.c_float * 16),
                ("view_project", C.c_float * 16), ("inverse_view_project", C.c_float * 16),
                ("skybox_transposed", C.c_float * 16), ("view_clip_planes", (C.c_float * 4) * 6)]


class RendererOpts(C.Structure):
    _fields_ = [("rsqrt_mode", C.c_uint32), ("sched_tile", C.c_uint32), ("bin_capacity", C.c_uint64),
                ("raster_warps", C.c_uint32), ("flags", C.c_uint32)]


class FrameStats(C.Structure):
    _fields_ = [("triangles_in", C.c_uint64), ("triangles_clipped", C.c_uint64), ("setup_triangles", C.c_uint64),
                ("bin_pairs", C.c_uint64), ("bin_capacity", C.c_uint64), ("tiles", C.c_uint32),
                ("overflow_retries", C.c_uint32), ("tile_luminance_mean", C.c_float), ("exposure", C.c_float),
                ("sched_tile", C.c_uint32), ("staged_bytes", C.c_uint64), ("culled_pairs", C.c_uint64),
                ("kernel_launches", C.c_uint64), ("triangles_clip_path", C.c_uint64)]


class BatchTuning(C.Structure):
    _fields_ = [("batch_class", C.c_uint32), ("tuned", C.c_uint32), ("sched_tile", C.c_uint32),
                ("fused_shade", C.c_uint32), ("raster_ctas_per_sm", C.c_uint32), ("reserved", C.c_uint32),
                ("bin_capacity", C.c_uint64)]


class ViewDesc(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("camera", C.POINTER(Camera)), ("width", C.c_int32), ("height", C.c_int32),
                ("exposure", C.c_float), ("rsqrt_mode", C.c_uint32), ("rgba8", C.c_void_p), ("vis", C.c_void_p)]


class BatchOpts(C.Structure):
    _fields_ = [("sched_tile", C.c_uint32), ("use_graph", C.c_uint32), ("bin_capacity", C.c_uint64),
                ("flags", C.c_uint32), ("raster_ctas_per_sm", C.c_uint32)]


class ServerOpts(C.Structure):
    _fields_ = [("memory_budget", C.c_uint64), ("max_batch_views", C.c_uint32), ("max_queue", C.c_uint32),
                ("inflight", C.c_uint32), ("sched_tile", C.c_uint32), ("rsqrt_mode", C.c_uint32),
                ("use_graph", C.c_uint32), ("flags", C.c_uint32)]


class Request(C.Structure):
    _fields_ = [("scene", C.c_int32), ("width", C.c_int32), ("height", C.c_int32), ("exposure", C.c_float),
                ("camera", Camera), ("tag", C.c_uint64)]


class Completion(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("tag", C.c_uint64), ("status", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("batch_views", C.c_int32), ("rgba8", C.c_void_p), ("vis", C.c_void_p),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("batches", C.c_uint64), ("device_bytes", C.c_uint64), ("budget", C.c_uint64)]


EXPORTS = [
    "swr_scene_create", "swr_scene_destroy", "swr_scene_get_info", "swr_scene_export", "swr_camera_init",
    "swr_camera_update", "swr_renderer_create", "swr_renderer_destroy", "swr_render_frame", "swr_renderer_sync",
    "swr_blit", "swr_renderer_set_blit_target", "swr_read_visbuffer", "swr_renderer_device_outputs", "swr_renderer_get_exposure",
    "swr_renderer_set_exposure", "swr_renderer_get_stats", "swr_renderer_get_tile_luminance", "swr_last_error",
    "swr_abi_version", "swr_renderer_set_profiling", "swr_renderer_get_profile", "swr_render_frame_noalloc",
    "swr_batch_create", "swr_batch_destroy", "swr_batch_render", "swr_batch_sync", "swr_batch_output",
    "swr_batch_autotune", "swr_batch_last_ms", "swr_batch_get_tuning", "swr_server_create", "swr_server_destroy", "swr_server_add_scene",
    "swr_server_submit", "swr_server_poll", "swr_server_release", "swr_server_get_stats", "swr_copy_to_host",
    "swr_selftest_rsqrt", "swr_scene_load_gltf", "swr_selftest_depth_floor", "swr_scene_save_gi_cache",
    "swr_scene_save_ggx_cache", "swr_selftest_srgb_pow",
]
STAGES = ["draws", "frontend", "clip", "scan", "scatter", "raster", "shade", "resolve"]

_lib = None


def lib():
    """Loads libswr.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise RuntimeError("libswr.so not built: run __graft_entry__.build()")
    L = C.CDLL(LIBPATH)
    vp = C.c_void_p
    sig = {
        "swr_scene_create": ([C.POINTER(SceneDesc), C.POINTER(vp)], C.c_int),
        "swr_scene_destroy": ([vp], None),
        "swr_scene_get_info": ([vp, C.POINTER(SceneInfo)], C.c_int),
        "swr_scene_export": ([vp, C.POINTER(SceneHostView)], C.c_int),
        "swr_camera_init": ([C.POINTER(Camera), f32p, f32p, C.c_float, C.c_float, C.c_float, C.c_float], C.c_int),
        "swr_camera_update": ([C.POINTER(Camera)], C.c_int),
        "swr_renderer_create": ([C.c_int32, C.c_int32, C.POINTER(RendererOpts), C.POINTER(vp)], C.c_int),
        "swr_renderer_destroy": ([vp], None),
        "swr_render_frame": ([vp, vp, C.POINTER(Camera), C.c_float, vp], C.c_int),
        "swr_renderer_sync": ([vp], C.c_int),
        "swr_blit": ([vp, vp, C.c_size_t, vp], C.c_int),
        "swr_renderer_set_blit_target": ([vp, vp, C.c_size_t], C.c_int),
        "swr_read_visbuffer": ([vp, vp, vp], C.c_int),
        "swr_renderer_device_outputs": ([vp, C.POINTER(vp), C.POINTER(vp)], C.c_int),
        "swr_renderer_get_exposure": ([vp, f32p], C.c_int),
        "swr_renderer_set_exposure": ([vp, C.c_float], C.c_int),
        "swr_renderer_get_stats": ([vp, C.POINTER(FrameStats)], C.c_int),
        "swr_renderer_get_tile_luminance": ([vp, f32p, C.c_uint32], C.c_int),
        "swr_renderer_set_profiling": ([vp, C.c_int32], C.c_int),
        "swr_renderer_get_profile": ([vp, f32p, C.c_int32, C.POINTER(C.c_uint32)], C.c_int),
        "swr_selftest_rsqrt": ([f32p, f32p, C.c_uint64, C.c_uint32], C.c_int),
        "swr_selftest_depth_floor": ([C.c_void_p, f32p, f32p, C.c_int32, C.c_int32, f32p], C.c_int),
        "swr_scene_load_gltf": ([C.c_char_p, C.POINTER(GltfOpts), C.POINTER(vp)], C.c_int),
        "swr_render_frame_noalloc": ([vp, C.POINTER(Camera), C.c_int32, C.c_int32, C.c_float, C.c_uint32, vp, vp, vp],
                                     C.c_int),
        "swr_batch_create": ([C.POINTER(BatchOpts), C.POINTER(vp)], C.c_int),
        "swr_batch_destroy": ([vp], None),
        "swr_batch_render": ([vp, C.POINTER(ViewDesc), C.c_int32, vp], C.c_int),
        "swr_batch_sync": ([vp], C.c_int),
        "swr_batch_output": ([vp, C.c_int32, C.POINTER(vp), C.POINTER(vp)], C.c_int),
        "swr_batch_autotune": ([vp, C.POINTER(ViewDesc), C.c_int32, vp, C.POINTER(C.c_uint32), f32p], C.c_int),
        "swr_batch_last_ms": ([vp, f32p], C.c_int),
        "swr_batch_get_tuning": ([vp, C.POINTER(ViewDesc), C.c_int32, C.POINTER(BatchTuning)], C.c_int),
        "swr_server_create": ([C.POINTER(ServerOpts), C.POINTER(vp)], C.c_int),
        "swr_server_destroy": ([vp], None),
        "swr_server_add_scene": ([vp, vp, C.POINTER(C.c_int32)], C.c_int),
        "swr_server_submit": ([vp, C.POINTER(Request), C.POINTER(C.c_uint64)], C.c_int),
        "swr_server_poll": ([vp, C.POINTER(Completion), C.c_int32, C.POINTER(C.c_int32), C.c_int32], C.c_int),
        "swr_server_release": ([vp, C.c_uint64], C.c_int),
        "swr_server_get_stats": ([vp, C.POINTER(ServerStats)], C.c_int),
        "swr_copy_to_host": ([vp, vp, C.c_size_t, vp], C.c_int),
        "swr_last_error": ([], C.c_char_p),
        "swr_abi_version": ([], C.c_int32),
        "swr_scene_save_gi_cache": ([vp, C.c_char_p], C.c_int),
        "swr_scene_save_ggx_cache": ([vp, C.c_char_p], C.c_int),
        "swr_selftest_srgb_pow": ([f32p, f32p, C.c_uint64, C.c_uint32], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


class SwrError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("swr status %d: %s" % (status, msg))
        self.status = status


def check(st):
    if st != SWR_OK:
        raise SwrError(st, lib().swr_last_error().decode(errors="replace"))


def _fp(a):
    return a.ctypes.data_as(f32p) if a is not None else None


def _up(a):
    return a.ctypes.data_as(u32p) if a is not None else None


def texref(index=-1, wrap_s=WRAP_REPEAT, wrap_t=WRAP_REPEAT):
    return TexRef(index, wrap_s, wrap_t, 0)


def scene_desc(sd, flags=0, host_threads=0, gi_cache=None, ggx_cache=None):
    """swr_scene_desc of a scene dict (see scenes.py), and the arrays it points
    into (keep them alive while the descriptor is used). Builds structures
    only: the library is not loaded. gi_cache / ggx_cache: cache file paths."""
    keep = []
    meshes = (MeshDesc * len(sd["meshes"]))()
    for mi, prims in enumerate(sd["meshes"]):
        arr = (PrimitiveDesc * len(prims))()
        for pi, p in enumerate(prims):
            pos = np.ascontiguousarray(p["positions"], np.float32)
            idx = np.ascontiguousarray(p["indices"], np.uint32)
            nrm = None if p.get("normals") is None else np.ascontiguousarray(p["normals"], np.float32)
            tan = None if p.get("tangents") is None else np.ascontiguousarray(p["tangents"], np.float32)
            uv = None if p.get("texcoords") is None else np.ascontiguousarray(p["texcoords"], np.float32)
            keep += [pos, idx, nrm, tan, uv]
            arr[pi] = PrimitiveDesc(pos.shape[0], idx.size, _fp(pos), _fp(nrm), _fp(tan), _fp(uv), _up(idx),
                                    p.get("material", -1), 0)
        keep.append(arr)
        meshes[mi] = MeshDesc(len(prims), 0, C.cast(arr, C.POINTER(PrimitiveDesc)))
    nodes = (NodeDesc * len(sd["nodes"]))()
    for ni, n in enumerate(sd["nodes"]):
        w = np.asarray(n["world"], np.float32).reshape(16)
        loc = np.asarray(n.get("local", n["world"]), np.float32).reshape(16)
        nodes[ni] = NodeDesc((C.c_float * 16)(*w), (C.c_float * 16)(*loc), n["mesh"], 0)
    mats = (MaterialDesc * len(sd["materials"]))()
    for i, m in enumerate(sd["materials"]):
        md = MaterialDesc()
        md.base_color_factor = (C.c_float * 4)(*m.get("base_color_factor", (1, 1, 1, 1)))
        md.metallic_factor = m.get("metallic", 1.0)
        md.roughness_factor = m.get("roughness", 1.0)
        md.emissive_factor = (C.c_float * 3)(*m.get("emissive_factor", (0, 0, 0)))
        md.occlusion_strength = m.get("occlusion_strength", 1.0)
        md.alpha_cutoff = m.get("alpha_cutoff", 0.5)
        md.transmission = m.get("transmission", 0.0)
        md.alpha_mask = 1 if m.get("alpha_mask") else 0
        md.has_transmission = 1 if m.get("has_transmission") else 0
        for slot in ("base_color", "metallic_roughness", "normal", "emissive", "occlusion",
                     "transmission_texture"):
            t = m.get(slot)
            setattr(md, slot, texref(*t) if t is not None else texref())
        mats[i] = md
    texs = (TextureDesc * max(1, len(sd["textures"])))()
    for i, t in enumerate(sd["textures"]):
        data = np.ascontiguousarray(t["rgba8"], np.uint32)
        keep.append(data)
        texs[i] = TextureDesc(t["width"], t["height"], t["type"], 0, _up(data))
    cube = np.ascontiguousarray(sd["cubemap"], np.uint32)
    keep += [meshes, nodes, mats, texs, cube]
    desc = SceneDesc()
    desc.mesh_count = len(sd["meshes"])
    desc.node_count = len(sd["nodes"])
    desc.material_count = len(sd["materials"])
    desc.texture_count = len(sd["textures"])
    desc.meshes = C.cast(meshes, C.POINTER(MeshDesc))
    desc.nodes = C.cast(nodes, C.POINTER(NodeDesc))
    desc.materials = C.cast(mats, C.POINTER(MaterialDesc))
    desc.textures = C.cast(texs, C.POINTER(TextureDesc))
    desc.cubemap_face_size = sd["cubemap_face_size"]
    desc.voxel_grid_size = sd.get("voxel_grid_size", 128)
    desc.cubemap_faces = _up(cube)
    desc.specular_samples = sd.get("specular_samples", 64)
    desc.brdf_lut_size = sd.get("brdf_lut_size", 128)
    desc.gi_sh_scale = sd.get("gi_sh_scale", 0.25)
    desc.sky_visibility = sd.get("sky_visibility", 1.0)
    desc.host_threads = host_threads
    desc.flags = flags
    desc.gi_cache_path = None if gi_cache is None else os.fsencode(gi_cache)
    desc.ggx_cache_path = None if ggx_cache is None else os.fsencode(ggx_cache)
    return desc, keep


class Scene:
    """Owns a swr_scene built from a scene dict (see scenes.py)."""

    def __init__(self, sd, host_only=False, host_threads=0, gi=False, gi_cache=None, ggx_cache=None):
        flags = (SCENE_HOST_ONLY if host_only else 0) | (SCENE_GI if gi else 0)
        desc, keep = scene_desc(sd, flags, host_threads, gi_cache, ggx_cache)
        h = C.c_void_p()
        check(lib().swr_scene_create(C.byref(desc), C.byref(h)))
        self.handle = h
        # The scene dict and flags the scene was made from; the library
        # copied everything it needs.
        self.source, self.flags = sd, flags

    @classmethod
    def load_gltf(cls, path, cubemap_faces=None, cubemap_face_size=0, cubemap_path=None, voxel_grid_size=0,
                  specular_samples=0, brdf_lut_size=0, host_only=False, host_threads=0, gi=False, gi_cache=None,
                  ggx_cache=None):
        """swr_scene_load_gltf: a .gltf/.glb file; the cubemap as raw faces or a cross image path.
        gi_cache: a path, or True for the reference's (the file's path with
        extension .gi, Path::with_extension); ggx_cache: a path."""
        o = GltfOpts()
        faces = None
        if cubemap_faces is not None:
            faces = np.ascontiguousarray(cubemap_faces, np.uint32)
            o.cubemap_faces = _up(faces)
            o.cubemap_face_size = cubemap_face_size
        if cubemap_path is not None:
            o.cubemap_path = os.fsencode(cubemap_path)
        o.voxel_grid_size = voxel_grid_size
        o.specular_samples = specular_samples
        o.brdf_lut_size = brdf_lut_size
        o.host_threads = host_threads
        o.flags = (SCENE_HOST_ONLY if host_only else 0) | (SCENE_GI if gi else 0)
        if gi_cache is True:
            gi_cache = os.path.splitext(os.fspath(path))[0] + ".gi"
        if gi_cache is not None:
            o.gi_cache_path = os.fsencode(gi_cache)
        if ggx_cache is not None:
            o.ggx_cache_path = os.fsencode(ggx_cache)
        h = C.c_void_p()
        check(lib().swr_scene_load_gltf(os.fsencode(path), C.byref(o), C.byref(h)))
        self = cls.__new__(cls)
        self.handle = h
        self.source, self.flags = None, o.flags
        return self

    def save_gi_cache(self, path):
        check(lib().swr_scene_save_gi_cache(self.handle, os.fsencode(path)))

    def save_ggx_cache(self, path):
        check(lib().swr_scene_save_ggx_cache(self.handle, os.fsencode(path)))

    def info(self):
        i = SceneInfo()
        check(lib().swr_scene_get_info(self.handle, C.byref(i)))
        return i

    def export(self):
        v = SceneHostView()
        check(lib().swr_scene_export(self.handle, C.byref(v)))
        return v

    def close(self):
        if getattr(self, "handle", None):
            lib().swr_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_camera(position, look_at, fov, width, height, far_plane):
    cam = Camera()
    p = (C.c_float * 3)(*position)
    t = (C.c_float * 3)(*look_at)
    check(lib().swr_camera_init(C.byref(cam), p, t, fov, float(width), float(height), far_plane))
    check(lib().swr_camera_update(C.byref(cam)))
    cam.args = (tuple(position), tuple(look_at), fov, width, height, far_plane)
    return cam


class Renderer:
    def __init__(self, width, height, rsqrt_mode=RSQRT_AARCH64, sched_tile=0, bin_capacity=0):
        o = RendererOpts(rsqrt_mode, sched_tile, bin_capacity, 0, 0)
        h = C.c_void_p()
        check(lib().swr_renderer_create(width, height, C.byref(o), C.byref(h)))
        self.handle = h
        self.width, self.height = width, height

    def render(self, scene, cam, dt=0.0, stream=None):
        check(lib().swr_render_frame(self.handle, scene.handle, C.byref(cam), dt, stream))

    def sync(self):
        check(lib().swr_renderer_sync(self.handle))

    def blit(self, out=None, stream=None):
        if out is None:
            out = np.zeros((self.height, self.width), np.uint32)
        check(lib().swr_blit(self.handle, out.ctypes.data_as(C.c_void_p), out.shape[1], stream))
        return out

    def set_blit_target(self, ptr, row_stride=0, keep=None):
        """Host framebuffer (address as int, or None to detach) that each
        following frame's shading pass writes directly; `keep` holds the
        object that owns the memory alive while it is the target."""
        check(lib().swr_renderer_set_blit_target(self.handle, C.c_void_p(ptr) if ptr else None, row_stride))
        self._blit_keep = keep if ptr else None

    def visbuffer(self, out=None, stream=None):
        if out is None:
            out = np.zeros((self.height, self.width), np.uint64)
        check(lib().swr_read_visbuffer(self.handle, out.ctypes.data_as(C.c_void_p), stream))
        return out

    def device_outputs(self):
        a, b = C.c_void_p(), C.c_void_p()
        check(lib().swr_renderer_device_outputs(self.handle, C.byref(a), C.byref(b)))
        return a.value, b.value

    def exposure(self):
        e = C.c_float()
        check(lib().swr_renderer_get_exposure(self.handle, C.byref(e)))
        return e.value

    def set_exposure(self, e):
        check(lib().swr_renderer_set_exposure(self.handle, e))

    def stats(self):
        s = FrameStats()
        check(lib().swr_renderer_get_stats(self.handle, C.byref(s)))
        return s

    def tile_luminance(self):
        tx = (self.width + 63) // 64
        ty = (self.height + 63) // 64
        out = np.zeros(tx * ty, np.float32)
        check(lib().swr_renderer_get_tile_luminance(self.handle, _fp(out), out.size))
        return out

    def set_profiling(self, on=True):
        check(lib().swr_renderer_set_profiling(self.handle, 1 if on else 0))

    def profile(self):
        """Mean ms per stage since profiling was enabled, and the frame count."""
        out = np.zeros(8, np.float32)
        n = C.c_uint32()
        check(lib().swr_renderer_get_profile(self.handle, _fp(out), 8, C.byref(n)))
        return dict(zip(STAGES, out.tolist())), n.value

    def close(self):
        if getattr(self, "handle", None):
            lib().swr_renderer_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def selftest_rsqrt(values, mode=RSQRT_AARCH64):
    """Device reciprocal square root of `values` (float32) in the given mode."""
    x = np.ascontiguousarray(values, np.float32)
    out = np.empty_like(x)
    check(lib().swr_selftest_rsqrt(x.ctypes.data_as(f32p), out.ctypes.data_as(f32p), x.size, mode))
    return out


def selftest_depth_floor(p, zow, oow, xe, ye):
    """Occlusion-culling depth floor of one packet, evaluated on the host by
    the raster's own source; -inf when no floor is taken."""
    p = np.ascontiguousarray(p, np.int32)
    zow = np.ascontiguousarray(zow, np.float32)
    oow = np.ascontiguousarray(oow, np.float32)
    z = np.zeros(1, np.float32)
    check(lib().swr_selftest_depth_floor(p.ctypes.data, zow.ctypes.data_as(f32p), oow.ctypes.data_as(f32p), xe, ye,
                                         z.ctypes.data_as(f32p)))
    return float(z[0])


def copy_device_to_host(dev_ptr, nbytes, out, stream=None):
    """Copies device memory (batch/server outputs) into a numpy array."""
    check(lib().swr_copy_to_host(out.ctypes.data_as(C.c_void_p), C.c_void_p(dev_ptr), nbytes, stream))
    return out


class Batch:
    """Many views per launch sequence (swr_batch_*)."""

    def __init__(self, sched_tile=0, use_graph=False, bin_capacity=0, fused_shade=False, raster_ctas_per_sm=0):
        h = C.c_void_p()
        o = BatchOpts(sched_tile, 1 if use_graph else 0, bin_capacity, 1 if fused_shade else 0, raster_ctas_per_sm)
        check(lib().swr_batch_create(C.byref(o), C.byref(h)))
        self.handle = h

    @staticmethod
    def views(items):
        """items: [(scene, camera, width, height, exposure, rsqrt_mode)]"""
        arr = (ViewDesc * len(items))()
        for i, (scene, cam, w, h, e, m) in enumerate(items):
            arr[i] = ViewDesc(scene.handle.value, C.pointer(cam), w, h, e, m, None, None)
        return arr

    def render(self, arr, stream=None):
        check(lib().swr_batch_render(self.handle, arr, len(arr), stream))

    def sync(self):
        check(lib().swr_batch_sync(self.handle))

    def output(self, i, w, h):
        a, b = C.c_void_p(), C.c_void_p()
        check(lib().swr_batch_output(self.handle, i, C.byref(a), C.byref(b)))
        rgba = copy_device_to_host(a.value, w * h * 4, np.zeros((h, w), np.uint32))
        vis = copy_device_to_host(b.value, w * h * 8, np.zeros((h, w), np.uint64))
        return rgba, vis

    def autotune(self, arr, stream=None):
        t = C.c_uint32()
        ms = C.c_float()
        check(lib().swr_batch_autotune(self.handle, arr, len(arr), stream, C.byref(t), C.byref(ms)))
        return t.value, ms.value

    def tuning(self, arr):
        """swr_batch_get_tuning: the configuration the batch uses for these views."""
        t = BatchTuning()
        check(lib().swr_batch_get_tuning(self.handle, arr, len(arr), C.byref(t)))
        return {f: getattr(t, f) for f, _ in BatchTuning._fields_ if f != "reserved"}

    def last_ms(self):
        ms = C.c_float()
        check(lib().swr_batch_last_ms(self.handle, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "handle", None):
            lib().swr_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Request loop with continuous batching (swr_server_*)."""

    def __init__(self, memory_budget=40 << 30, max_batch_views=64, max_queue=4096, inflight=2, sched_tile=0,
                 rsqrt_mode=RSQRT_AARCH64, use_graph=False, fused_shade=False):
        h = C.c_void_p()
        o = ServerOpts(memory_budget, max_batch_views, max_queue, inflight, sched_tile, rsqrt_mode,
                       1 if use_graph else 0, 1 if fused_shade else 0)
        check(lib().swr_server_create(C.byref(o), C.byref(h)))
        self.handle = h

    def add_scene(self, scene):
        i = C.c_int32()
        check(lib().swr_server_add_scene(self.handle, scene.handle, C.byref(i)))
        return i.value

    def submit(self, scene_id, cam, w, h, exposure=2.0, tag=0):
        r = Request(scene_id, w, h, exposure, cam, tag)
        t = C.c_uint64()
        st = lib().swr_server_submit(self.handle, C.byref(r), C.byref(t))
        if st == SWR_BUSY:
            return None
        check(st)
        return t.value

    def poll(self, max_n=256, wait_ms=10):
        out = (Completion * max_n)()
        n = C.c_int32()
        check(lib().swr_server_poll(self.handle, out, max_n, C.byref(n), wait_ms))
        return [out[i] for i in range(n.value)]

    def release(self, ticket):
        check(lib().swr_server_release(self.handle, ticket))

    def stats(self):
        s = ServerStats()
        check(lib().swr_server_get_stats(self.handle, C.byref(s)))
        return s

    def close(self):
        if getattr(self, "handle", None):
            lib().swr_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
