/*
 * swr.h — C ABI of the GB300 per-frame rasterization pipeline.
 *
 * This library replaces the per-frame render path of swraster-viewer
 * (Rust) with hand-written sm_103a CUDA kernels. Every entry point is plain C:
 * opaque handles, plain pointers and sizes, a status code, no exceptions, no
 * aborts. A Rust crate (or ctypes, cgo, JNI) binds to it verbatim.
 *
 * Reference interface each entry point replaces (paths inside the reference
 * project):
 *   swr_scene_create       Scene::from_gltf                   src/scene.rs:145-354
 *                          (+ load-time precompute driven by load_scene,
 *                           src/main.rs:100-291)
 *   swr_camera_init        RenderCamera::new                  src/rendercamera.rs:28-63
 *   swr_camera_update      RenderCamera::update_matrices      src/rendercamera.rs:78-86
 *   swr_renderer_create    Renderer::new                      src/renderer.rs:165-198
 *   swr_render_frame       Renderer::render_scene             src/renderer.rs:201-256
 *                        + Renderer::update_auto_exposure     src/renderer.rs:258-290
 *   swr_blit               Renderer::blit_to_buffer           src/renderer.rs:293-355
 *   swr_renderer_set_blit_target  (blit_to_buffer's destination, given once
 *                           so the shading pass writes it directly)
 *   swr_read_visbuffer     (no reference counterpart: the reference keeps a
 *                           per-tile packet index, src/tilerasterizer.rs:33-36;
 *                           this exports primitive + triangle ID per pixel)
 *
 * Conventions
 *   - Every call returns swr_status; swr_last_error() gives a message for the
 *     calling thread's last failure.
 *   - A scene is immutable after creation and may be shared by any number of
 *     renderers and streams. A renderer is single-threaded: one per
 *     thread/stream (the reference wraps its renderer in a Mutex,
 *     src/main.rs:312).
 *   - `stream` arguments are cudaStream_t values passed as void* (NULL = the
 *     legacy default stream).
 *   - Matrices are column-major float[16] (glam's layout).
 *   - RGBA8 pixels pack R in the most significant byte:
 *     r<<24 | g<<16 | b<<8 | a  (src/util.rs:98-100).
 */
#ifndef SWR_H
#define SWR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SWR_ABI_VERSION 2

typedef enum swr_status {
    SWR_OK = 0,
    SWR_INVALID_ARG = 1,
    SWR_NO_MEMORY = 2,
    SWR_OVERFLOW = 3,     /* a device capacity (bins, clip output) was exceeded */
    SWR_TIMEOUT = 4,      /* a bounded device wait gave up */
    SWR_CUDA_ERROR = 5,
    SWR_IO_ERROR = 6,
    SWR_BAD_SCENE = 7,
    SWR_UNSUPPORTED = 8,
    SWR_BUSY = 9          /* admission refused: memory budget or slots exhausted */
} swr_status;

/* Texture types, src/texture.rs:19-26. They select the mip filter. */
enum {
    SWR_TEX_SRGB = 0,
    SWR_TEX_NORMAL = 1,
    SWR_TEX_METALLIC_ROUGHNESS = 2,
    SWR_TEX_CUBEMAP = 3,
    SWR_TEX_LINEAR = 4
};

/* Wrap modes, src/texture.rs:554-558. */
enum {
    SWR_WRAP_REPEAT = 0,
    SWR_WRAP_MIRRORED_REPEAT = 1,
    SWR_WRAP_CLAMP_TO_EDGE = 2
};

/* Reciprocal square root used by Vec3x4::normalize (src/math.rs:10-49).
 * AARCH64 reproduces FRSQRTE + one FRSQRTS step (the reference as built on
 * Arm hosts such as Grace); IEEE is 1/sqrt(x) with two correctly rounded
 * operations (the reference's portable fallback). */
enum {
    SWR_RSQRT_IEEE = 0,
    SWR_RSQRT_AARCH64 = 1
};

/* ------------------------------------------------------------------ */
/* Scene description (in-memory; the synthetic-scene and glTF loaders  */
/* both produce this).                                                 */
/* ------------------------------------------------------------------ */

typedef struct swr_texture_desc {
    uint32_t width;
    uint32_t height;
    uint32_t type;            /* SWR_TEX_* */
    uint32_t reserved;
    const uint32_t* rgba8;    /* width*height texels, R in MSB */
} swr_texture_desc;

typedef struct swr_texref {
    int32_t texture;          /* index into swr_scene_desc.textures, -1 = none */
    uint32_t wrap_s;          /* SWR_WRAP_* */
    uint32_t wrap_t;
    uint32_t reserved;
} swr_texref;

/* glTF pbrMetallicRoughness material as read by Material::from_gltf,
 * src/scene.rs:690-780. */
typedef struct swr_material_desc {
    float base_color_factor[4];
    float metallic_factor;
    float roughness_factor;
    float emissive_factor[3];
    float occlusion_strength;   /* default 1 */
    float alpha_cutoff;         /* default 0.5 */
    float transmission;         /* KHR_materials_transmission factor */
    uint32_t alpha_mask;        /* glTF alphaMode == MASK */
    uint32_t has_transmission;  /* KHR_materials_transmission present -> translucent */
    swr_texref base_color;
    swr_texref metallic_roughness;
    swr_texref normal;
    swr_texref emissive;
    swr_texref occlusion;
    swr_texref transmission_texture;
} swr_material_desc;

/* One glTF primitive (src/scene.rs:439-495). normals/tangents/texcoords
 * may be NULL: normals are then generated (compute_smooth_normals), tangents
 * generated (compute_tangents) and texcoords zero-filled, as the reference
 * loader does. */
typedef struct swr_primitive_desc {
    uint32_t vertex_count;
    uint32_t index_count;       /* multiple of 3 */
    const float* positions;     /* vertex_count * 3 */
    const float* normals;       /* vertex_count * 3, or NULL */
    const float* tangents;      /* vertex_count * 4, or NULL */
    const float* texcoords;     /* vertex_count * 2, or NULL */
    const uint32_t* indices;    /* index_count */
    int32_t material;           /* -1 = material 0, as src/scene.rs:493 */
    uint32_t reserved;
} swr_primitive_desc;

typedef struct swr_mesh_desc {
    uint32_t primitive_count;
    uint32_t reserved;
    const swr_primitive_desc* primitives;
} swr_mesh_desc;

/* A flattened node. `world` is the final (parent-composed) transform;
 * `local` is the node's own transform, which the reference uses as the
 * initial bounding-sphere centre (src/scene.rs:384-394). For root nodes
 * both are equal. */
typedef struct swr_node_desc {
    float world[16];
    float local[16];
    int32_t mesh;               /* -1 = no mesh */
    uint32_t reserved;
} swr_node_desc;

typedef struct swr_scene_desc {
    uint32_t mesh_count;
    uint32_t node_count;
    uint32_t material_count;
    uint32_t texture_count;
    const swr_mesh_desc* meshes;
    const swr_node_desc* nodes;
    const swr_material_desc* materials;
    const swr_texture_desc* textures;
    /* Environment cubemap faces in +X,-X,+Y,-Y,+Z,-Z order, each
     * size*size RGBA8 (the unpacked cross of src/texture.rs:922-971). */
    uint32_t cubemap_face_size;
    uint32_t voxel_grid_size;   /* 128 in the reference (src/main.rs:228); at most 1024 */
    const uint32_t* cubemap_faces;
    uint32_t specular_samples;  /* GGX prefilter samples, 64 (src/scene.rs:179); at most 65536 */
    uint32_t brdf_lut_size;     /* 128 (src/scene.rs:221); at most 4096 */
    float gi_sh_scale;          /* 0.25 (src/main.rs:54) */
    float sky_visibility;       /* 1.0 (src/main.rs:280) */
    uint32_t host_threads;      /* precompute threads, 0 = all cores */
    uint32_t flags;             /* SWR_SCENE_* */
    /* Cache files (NULL = none), read when valid and written after the
     * table is computed, as load_scene does. ggx_cache_path: the
     * GGX-prefiltered environment (the reference's assets/cubemap.ggx,
     * "GGX0" v1, src/texture.rs:425-554, src/scene.rs:164-205; keyed on the
     * face size only, as there). gi_cache_path: with SWR_SCENE_GI, the baked
     * grid (the reference's <scene>.gi, "VGI0" v8, src/gi.rs:30-117,
     * src/main.rs:248-279); a valid file replaces the bake, which also lets
     * SWR_SCENE_HOST_ONLY scenes carry a baked grid. Both are brotli
     * streams, through the system's libbrotlienc/libbrotlidec; without
     * them the tables are computed (swr_scene_info reports
     * SWR_CACHE_NO_CODEC). */
    const char* gi_cache_path;
    const char* ggx_cache_path;
} swr_scene_desc;

/* swr_scene_info.gi_cache / ggx_cache */
#define SWR_CACHE_NONE 0u          /* no path given */
#define SWR_CACHE_LOADED 1u        /* the table was read from the file */
#define SWR_CACHE_WRITTEN 2u       /* absent, stale or unreadable: computed, then written */
#define SWR_CACHE_WRITE_FAILED 3u  /* computed; writing the file failed */
#define SWR_CACHE_NO_CODEC 4u      /* computed; no brotli library to read or write it */

/* swr_scene_desc.flags */
#define SWR_SCENE_HOST_ONLY 1u  /* build and precompute only; no device copy
                                   (swr_scene_export works, rendering does not) */
#define SWR_SCENE_GI 2u         /* bake the voxel GI (the reference's --gi: bake_voxel_gi,
                                   src/gi.rs:316-408) on the device and shade with
                                   the full SH4 grid; not with SWR_SCENE_HOST_ONLY */

typedef struct swr_scene swr_scene;

swr_status swr_scene_create(const swr_scene_desc* desc, swr_scene** out);

/* glTF 2.0 file loading: replaces load_gltf + Scene::from_gltf
 * (src/main.rs:86-98, src/scene.rs:145-354) followed by the voxel-grid setup
 * of load_scene (src/main.rs:226-287, non-GI path). Reads .gltf (external or
 * base64 data: buffers) and .glb files; every document node is kept
 * (compute_final_transform_recursive), primitives need positions and
 * indices, texture images are loaded from their URI relative to the file's
 * directory (PNG, or sequential or progressive JPEG) and images embedded in buffer views are
 * skipped, as the reference does. The environment cubemap is given as raw
 * faces or as the path of a cross-layout image (the reference's
 * assets/cubemap.jpg). Errors: SWR_IO_ERROR (file, buffer or image),
 * SWR_BAD_SCENE (missing positions/indices, out-of-range references),
 * SWR_INVALID_ARG (no cubemap). */
typedef struct swr_gltf_opts {
    const uint32_t* cubemap_faces;  /* 6 faces +X,-X,+Y,-Y,+Z,-Z of face_size^2 RGBA8 (R in MSB), or NULL */
    uint32_t cubemap_face_size;
    uint32_t voxel_grid_size;       /* 0 = 128 (src/main.rs:228) */
    const char* cubemap_path;       /* used when cubemap_faces is NULL */
    uint32_t specular_samples;      /* 0 = 64 */
    uint32_t brdf_lut_size;         /* 0 = 128 */
    uint32_t host_threads;          /* precompute threads, 0 = all cores */
    uint32_t flags;                 /* SWR_SCENE_* */
    const char* gi_cache_path;      /* as swr_scene_desc; the reference's is the
                                       file's path with extension .gi */
    const char* ggx_cache_path;     /* as swr_scene_desc (assets/cubemap.ggx there) */
} swr_gltf_opts;

swr_status swr_scene_load_gltf(const char* path, const swr_gltf_opts* opts, swr_scene** out);
void swr_scene_destroy(swr_scene* scene);

typedef struct swr_scene_info {
    uint64_t triangle_count;    /* sum over nodes of their mesh's triangles */
    uint64_t vertex_count;
    uint64_t device_bytes;      /* HBM held by the scene */
    uint32_t node_count;
    uint32_t draw_count;        /* (node, primitive) pairs */
    float bounds_min[3];
    float bounds_max[3];
    float bounds_center[3];
    float bounds_diagonal;
    uint32_t gi_cache;          /* SWR_CACHE_* */
    uint32_t ggx_cache;         /* SWR_CACHE_* */
    /* Scenes built on the device compute mip chains, the BRDF LUT and the
     * GGX-prefiltered environment there, bit-exact with the host: where
     * the device's powf leaves a texel's byte open, the texel is computed
     * again on the host. This counts those texels (0 for host-only scenes). */
    uint64_t precompute_host_texels;
} swr_scene_info;

swr_status swr_scene_get_info(const swr_scene* scene, swr_scene_info* out);

/* save_gi_cache (src/gi.rs:82-113) and save_prefiltered_specular_cubemap_cache
 * (src/texture.rs:520-554): write the scene's baked GI grid / prefiltered
 * environment to a cache file. SWR_INVALID_ARG when the scene has no baked
 * grid; SWR_IO_ERROR when the file cannot be written or no brotli library
 * is present. */
swr_status swr_scene_save_gi_cache(const swr_scene* scene, const char* path);
swr_status swr_scene_save_ggx_cache(const swr_scene* scene, const char* path);

/* Read-only host view of the processed scene (generated normals and
 * tangents, mip chains, prefiltered cubemap, BRDF LUT, voxel grid). Test
 * infrastructure uses it to feed a CPU implementation the same inputs the
 * kernels consume. Pointers stay valid until swr_scene_destroy. */
typedef struct swr_texture_view {
    uint32_t width;
    uint32_t height;
    uint32_t type;
    uint32_t mip_count;         /* max_mip_level + 1 */
    const uint32_t* data;       /* all mips and faces */
    uint64_t data_len;          /* texels */
    const uint32_t* mip_offsets;
    const uint32_t* mip_widths;
    const uint32_t* mip_heights;
    const uint32_t* array_stride;
    float width_height_vec[4];
} swr_texture_view;

typedef struct swr_primitive_view {
    uint32_t vertex_count;
    uint32_t index_count;
    const float* positions;     /* vertex_count * 4 (x, y, z, 1) */
    const float* normals;       /* vertex_count * 4 (x, y, z, 0) */
    const float* tangents;      /* vertex_count * 4 */
    const float* texcoords;     /* vertex_count * 2 */
    const uint32_t* indices;
    uint32_t material;
    uint32_t triangle_id_base;  /* static ID of triangle 0 (per mesh) */
    float sphere[4];            /* bounding sphere centre xyz, radius */
} swr_primitive_view;

typedef struct swr_mesh_view {
    uint32_t primitive_count;
    uint32_t opaque_count;
    uint32_t translucent_count;
    uint32_t reserved;
    const uint32_t* primitives;       /* index into swr_scene_host_view.primitives */
    const uint32_t* opaque;           /* local primitive indices, src/scene.rs:276-284 */
    const uint32_t* translucent;
} swr_mesh_view;

typedef struct swr_node_view {
    float transform[16];
    float sphere[4];            /* bounding_sphere_world */
    int32_t mesh;
    uint32_t triangle_id_base;  /* static ID of this node's first triangle */
} swr_node_view;

typedef struct swr_material_view {
    float base_color_factor[4];
    float metallic_factor;
    float roughness_factor;
    float emissive_factor[3];
    float occlusion_strength;
    float alpha_cutoff;
    float transmission;
    uint32_t is_alpha_tested;
    uint32_t is_translucent;
    int32_t tex[6];             /* base, metallic-roughness, normal, emissive, occlusion, transmission; -1 = none */
    uint32_t wrap_s[6];
    uint32_t wrap_t[6];
} swr_material_view;

typedef struct swr_scene_host_view {
    uint32_t primitive_count;
    uint32_t mesh_count;
    uint32_t node_count;
    uint32_t material_count;
    uint32_t texture_count;
    uint32_t voxel_size;        /* grid is voxel_size^3 */
    const swr_primitive_view* primitives;
    const swr_mesh_view* meshes;
    const swr_node_view* nodes;
    const swr_material_view* materials;
    const swr_texture_view* textures;
    swr_texture_view cubemap;
    swr_texture_view cubemap_specular;
    swr_texture_view brdf_lut;
    float irradiance_sh[4][3];
    float light_direction[3];
    float light_color[3];
    float voxel_world_min[3];
    float voxel_world_max[3];
    const float* voxel_light_intensity;   /* voxel_size^3 (sun visibility, blurred) */
    float voxel_gi_sh4_const[4][4];       /* per-voxel SH4 rgb (+w filled per voxel) */
    const float* voxel_gi_sh4;            /* SWR_SCENE_GI: voxel_size^3 x 4 (r, g, b, w), else NULL */
} swr_scene_host_view;

swr_status swr_scene_export(const swr_scene* scene, swr_scene_host_view* out);

/* ------------------------------------------------------------------ */
/* Camera (src/rendercamera.rs). Host maths, same operation order as  */
/* glam 0.30.                                                          */
/* ------------------------------------------------------------------ */

typedef struct swr_camera {
    float position[3];
    float fov;
    float width;
    float height;
    float one_over_width;
    float one_over_height;
    float near_plane;
    float far_plane;
    float yaw;
    float pitch;
    float roll;
    float view_normal[3];
    float view[16];
    float projection[16];
    float view_project[16];
    float inverse_view_project[16];
    float skybox_transposed[16];
    float view_clip_planes[6][4];
} swr_camera;

swr_status swr_camera_init(swr_camera* cam, const float position[3], const float look_at[3],
                           float fov, float width, float height, float far_plane);
swr_status swr_camera_update(swr_camera* cam);

/* ------------------------------------------------------------------ */
/* Plain per-frame renderer                                            */
/* ------------------------------------------------------------------ */

typedef struct swr_renderer_opts {
    uint32_t rsqrt_mode;        /* SWR_RSQRT_*, default AARCH64 */
    uint32_t sched_tile;        /* raster scheduling tile: 8, 16, 32 or 64; 0 = chosen from the frame size */
    uint64_t bin_capacity;      /* initial (triangle, tile) pair capacity, 0 = auto */
    uint32_t raster_warps;      /* warps per raster CTA, 0 = default */
    uint32_t flags;             /* reserved, 0 */
} swr_renderer_opts;

typedef struct swr_renderer swr_renderer;

swr_status swr_renderer_create(int32_t width, int32_t height, const swr_renderer_opts* opts,
                               swr_renderer** out);
void swr_renderer_destroy(swr_renderer* r);

/* render_scene + update_auto_exposure(dt). Enqueued on `stream`; returns
 * once the frame is enqueued (and, when dt > 0, after the exposure step's
 * host callback is enqueued). Bin overflow is detected on the device and
 * the frame is re-rendered with a larger capacity on the next call to
 * swr_renderer_sync, swr_blit or swr_read_visbuffer. */
swr_status swr_render_frame(swr_renderer* r, const swr_scene* scene, const swr_camera* camera,
                            float dt, void* stream);

/* Waits for the frame and reports device-side errors (overflow retries
 * happen here). */
swr_status swr_renderer_sync(swr_renderer* r);

/* Copies the tonemapped RGBA8 frame into `pixels` (host or device memory),
 * row_stride in pixels (0 = width). For an odd height the last row is left
 * untouched, as blit_to_buffer's chunks_exact drops it (src/renderer.rs:298). */
swr_status swr_blit(swr_renderer* r, uint32_t* pixels, size_t row_stride, void* stream);

/* Host framebuffer that every following frame's shading pass writes its
 * RGBA8 pixels into directly, over the host link, while it shades (the
 * renderer's device copy is written as well). A swr_blit to the same
 * pointer and row_stride then only waits for the frame; a blit anywhere
 * else copies as before. `pixels` must be device-writable: pinned or
 * registered host memory, device or managed memory, or any host memory on
 * systems whose GPU reads the host page tables (Grace); SWR_INVALID_ARG
 * otherwise. It must hold (height & ~1) rows of row_stride pixels (0 =
 * width) and stay valid while frames render into it. NULL detaches. The
 * reference blits into one of two backbuffers that alternate per frame
 * (src/main.rs:522-543): set the frame's backbuffer before its
 * swr_render_frame (a cheap call), then swr_blit into it. */
swr_status swr_renderer_set_blit_target(swr_renderer* r, uint32_t* pixels, size_t row_stride);

/* Visibility buffer, width*height entries: (static triangle ID << 3) | fan
 * index for covered pixels, UINT64_MAX where depth stayed +inf. Static
 * triangle IDs number triangles in scene order (node, primitive, triangle);
 * see swr_node_view.triangle_id_base. */
swr_status swr_read_visbuffer(swr_renderer* r, uint64_t* ids, void* stream);

/* Device pointers to the renderer's own outputs (valid until the next
 * frame or destroy). */
swr_status swr_renderer_device_outputs(swr_renderer* r, const uint32_t** rgba8,
                                       const uint64_t** vis);

swr_status swr_renderer_get_exposure(const swr_renderer* r, float* exposure);
swr_status swr_renderer_set_exposure(swr_renderer* r, float exposure);

typedef struct swr_frame_stats {
    uint64_t triangles_in;      /* triangles entering the front end */
    uint64_t triangles_clipped; /* triangles that went through the clipper */
    uint64_t setup_triangles;   /* triangles after clip/cull with >= 1 tile */
    uint64_t bin_pairs;         /* (triangle, tile) pairs */
    uint64_t bin_capacity;
    uint32_t tiles;
    uint32_t overflow_retries;
    float tile_luminance_mean;
    float exposure;
    uint32_t sched_tile;        /* scheduling tile the renderer uses */
    uint64_t staged_bytes;      /* host-to-device bytes per frame (frame, scene and view headers, node order) */
    uint64_t culled_pairs;      /* bin pairs the raster dropped as hidden behind depths already written */
    uint64_t kernel_launches;   /* kernels the renderer has enqueued since it was created (re-renders after
                                   an overflow included) */
    uint64_t triangles_clip_path; /* triangles of primitives whose bounding sphere intersects the frustum:
                                     the ones the reference sends through clip_against_frustum */
} swr_frame_stats;

swr_status swr_renderer_get_stats(swr_renderer* r, swr_frame_stats* out);

/* Per-tile centre luminance of the last frame (tiles_x * tiles_y floats,
 * 64-pixel reference tiles), the auto-exposure meter input
 * (src/tilerasterizer.rs:103-106). */
swr_status swr_renderer_get_tile_luminance(swr_renderer* r, float* out, uint32_t count);

/* Stage timing with CUDA events recorded on the frame's stream between the
 * kernels: draws (counter reset and the draw-list build), frontend, clip,
 * scan, scatter, raster, shade, resolve.
 * swr_renderer_get_profile waits for outstanding frames and returns the mean
 * milliseconds per stage over the frames since profiling was enabled. */
#define SWR_STAGES 8
swr_status swr_renderer_set_profiling(swr_renderer* r, int32_t enable);
swr_status swr_renderer_get_profile(swr_renderer* r, float* stage_ms, int32_t n, uint32_t* frames);

/* ------------------------------------------------------------------ */
/* Batched form: many views of one or more resident scenes rendered by */
/* one launch sequence (no reference counterpart; the reference renders */
/* one view per frame).                                                 */
/* ------------------------------------------------------------------ */

typedef struct swr_view_desc {
    const swr_scene* scene;
    const swr_camera* camera;
    int32_t width;
    int32_t height;
    float exposure;             /* 2.0 = a fresh renderer's exposure */
    uint32_t rsqrt_mode;        /* SWR_RSQRT_* */
    uint32_t* rgba8;            /* device output (width*height) or NULL: batch-owned */
    uint64_t* vis;              /* device output (width*height) or NULL: batch-owned */
} swr_view_desc;

typedef struct swr_batch_opts {
    uint32_t sched_tile;        /* 8, 16, 32, 64; 0 = autotuned choice for the batch's class, else chosen
                                   from the view sizes (several views: 32 px with fused shading) */
    uint32_t use_graph;         /* replay the frame as a CUDA graph */
    uint64_t bin_capacity;      /* initial pair capacity, 0 = auto */
    uint32_t flags;             /* SWR_BATCH_* */
    uint32_t raster_ctas_per_sm;/* with sched_tile set: persistent raster CTAs per SM, 0 = as many as fit */
} swr_batch_opts;

/* swr_batch_opts.flags */
#define SWR_BATCH_FUSED_SHADE 1u  /* with sched_tile 32: shade inside the raster kernel
                                     (8- and 16-px tiles always do, 64-px never) */

typedef struct swr_batch swr_batch;

swr_status swr_batch_create(const swr_batch_opts* opts, swr_batch** out);
void swr_batch_destroy(swr_batch* b);
/* Enqueues all views on `stream` (the tables are uploaded with one copy and
 * the seven kernels run once for the whole batch; the raster kernel is
 * persistent and pulls (view, tile) items from a device work counter). */
swr_status swr_batch_render(swr_batch* b, const swr_view_desc* views, int32_t n, void* stream);
/* Waits for the last batch; re-renders it after growing capacities if bins
 * overflowed. */
swr_status swr_batch_sync(swr_batch* b);
swr_status swr_batch_output(swr_batch* b, int32_t view, const uint32_t** rgba8, const uint64_t** vis);
/* Times every scheduling tile size (and, for 32-px tiles, shading fused
 * into the raster kernel or run after it; 8- and 16-px tiles always fuse,
 * 64-px tiles never), each with the persistent raster at 1, 2 or as many
 * CTAs per SM as fit, on these views and keeps the fastest for the batch's
 * class (pixel count, triangle count, view count), with the bin capacity it
 * needed (swr_batch_get_tuning reports the choice). */
swr_status swr_batch_autotune(swr_batch* b, const swr_view_desc* views, int32_t n, void* stream,
                              uint32_t* best_tile, float* best_ms);
/* Milliseconds of the last synced batch on the device (CUDA events). */
swr_status swr_batch_last_ms(swr_batch* b, float* ms);

/* What the batch would use for these views: the autotuner's choice for
 * their class (log2 pixels, log2 triangles, log2 views) when it has one,
 * else the default choice. The autotuner sweeps the scheduling tile (8, 16,
 * 32, 32 with shading fused into the raster kernel, 64) by the persistent
 * raster's CTAs per SM (all that fit, 1, 2) and keeps, besides the fastest,
 * the (triangle, tile) pair capacity that configuration needed, with which
 * later batches of the class start. No counterpart in the reference. */
typedef struct swr_batch_tuning {
    uint32_t batch_class;
    uint32_t tuned;               /* 1 when the autotuner measured this class */
    uint32_t sched_tile;
    uint32_t fused_shade;
    uint32_t raster_ctas_per_sm;  /* 0 = as many as the registers allow */
    uint32_t reserved;
    uint64_t bin_capacity;        /* 0 = grown from overflow counters */
} swr_batch_tuning;

swr_status swr_batch_get_tuning(const swr_batch* b, const swr_view_desc* views, int32_t n, swr_batch_tuning* out);

/* ------------------------------------------------------------------ */
/* Served form: a request loop over resident scenes with memory-budget */
/* admission and continuous batching (no reference counterpart).        */
/* ------------------------------------------------------------------ */

typedef struct swr_server_opts {
    uint64_t memory_budget;     /* HBM bytes for resident scenes + pooled framebuffers */
    uint32_t max_batch_views;   /* views per batch (default 64) */
    uint32_t max_queue;         /* pending requests before submit returns SWR_BUSY (default 4096) */
    uint32_t inflight;          /* batches in flight on separate streams (default 2) */
    uint32_t sched_tile;        /* 0 = chosen per batch (several views: 32 px with fused shading) */
    uint32_t rsqrt_mode;
    uint32_t use_graph;
    uint32_t flags;             /* SWR_BATCH_* for every batch (SWR_BATCH_FUSED_SHADE) */
} swr_server_opts;

typedef struct swr_request {
    int32_t scene;              /* id from swr_server_add_scene */
    int32_t width;
    int32_t height;
    float exposure;
    swr_camera camera;
    uint64_t tag;
} swr_request;

typedef struct swr_completion {
    uint64_t ticket;
    uint64_t tag;
    int32_t status;
    int32_t width;
    int32_t height;
    int32_t batch_views;        /* size of the batch this request ran in */
    const uint32_t* rgba8;      /* device; valid until swr_server_release(ticket) */
    const uint64_t* vis;
    double queue_ms;            /* submit -> batch launch */
    double latency_ms;          /* submit -> completion */
} swr_completion;

typedef struct swr_server_stats {
    uint64_t submitted, completed, rejected, batches;
    uint64_t device_bytes;      /* scenes + framebuffers + engines */
    uint64_t budget;
} swr_server_stats;

typedef struct swr_server swr_server;

swr_status swr_server_create(const swr_server_opts* opts, swr_server** out);
void swr_server_destroy(swr_server* s);
/* Makes a scene resident for the server; SWR_BUSY if it does not fit the
 * budget. The scene must outlive the server. */
swr_status swr_server_add_scene(swr_server* s, const swr_scene* scene, int32_t* id);
swr_status swr_server_submit(swr_server* s, const swr_request* req, uint64_t* ticket);
/* Up to `max` completions; waits up to wait_ms for the first one. */
swr_status swr_server_poll(swr_server* s, swr_completion* out, int32_t max, int32_t* n, int32_t wait_ms);
/* Returns a completed request's framebuffers to the pool. */
swr_status swr_server_release(swr_server* s, uint64_t ticket);
swr_status swr_server_get_stats(swr_server* s, swr_server_stats* out);

/* Copies `bytes` from device memory (batch or server outputs) into host
 * memory `dst`, ordered on `stream`; returns when the copy is done. */
swr_status swr_copy_to_host(void* dst, const void* src_device, size_t bytes, void* stream);

/* Numerics self-test: the device reciprocal square root of `n` host values
 * in the given SWR_RSQRT_* mode (the arithmetic every normalize of the
 * shading pass uses, src/math.rs:17-49), written to host `out`. */
swr_status swr_selftest_rsqrt(const float* in, float* out, uint64_t n, uint32_t rsqrt_mode);

/* Numerics self-test: the device powf of the load-time tables on `n` host
 * values, powf(x, 2.4) (mode 0, srgb_to_linear_scalar, src/util.rs:49-55) or
 * powf(x, 1/2.4) (mode 1, linear_to_srgb_scalar, src/util.rs:66-72), written
 * to host `out`. */
swr_status swr_selftest_srgb_pow(const float* in, float* out, uint64_t n, uint32_t mode);

/* Numerics self-test, host only: the lower bound the raster's occlusion
 * culling takes on the depths of a packet (subpixel vertices p[6] = x0, y0,
 * x1, y1, x2, y2; depth and 1/w interpolants zow[3], oow[3] as value at
 * vertex 0 then differences; xe, ye the end of the packet's rect clipped to
 * its 64-pixel tile, in subpixels), evaluated by the same source the device
 * runs; -infinity when the raster takes no bound for the packet. No
 * counterpart in the reference, whose raster tests every packet. */
swr_status swr_selftest_depth_floor(const int32_t* p, const float* zow, const float* oow, int32_t xe, int32_t ye,
                                    float* zlo);

/* Allocation-free frame. No counterpart in the reference: an addition for
 * callers that cannot allocate device memory while they render (processes
 * whose device memory belongs to another allocator or a fixed budget,
 * real-time loops that cannot afford a cudaMalloc that may synchronize the
 * device). Renders `scene` (already resident) from `camera` into the
 * caller's device buffers rgba8 (width*height, row pitch width; an odd last
 * row is left untouched) and vis (width*height), with a fixed `exposure`
 * (2.0 is a fresh renderer's) and without allocating anything: all per-frame
 * work buffers live in one fixed __device__ array of about 9 MB that every
 * GPU loading the library holds until exit. Limits: width, height <= 512, at
 * most 16384 triangles passing the frustum test, 4096 nodes, 4096 draws,
 * 65536 (triangle, tile) pairs, no translucent primitives; larger inputs
 * return SWR_INVALID_ARG, capacity overflow on the device returns
 * SWR_OVERFLOW. The first call on a device looks up the array's address.
 * Returns after the frame has finished; a per-device lock held until then
 * serializes calls on one device (they share its array, and would race on
 * it if their GPU work overlapped). */
swr_status swr_render_frame_noalloc(const swr_scene* scene, const swr_camera* camera, int32_t width,
                                    int32_t height, float exposure, uint32_t rsqrt_mode, uint32_t* rgba8,
                                    uint64_t* vis, void* stream);

const char* swr_last_error(void);
int32_t swr_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* SWR_H */
