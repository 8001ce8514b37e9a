// Internal data layout shared by the host runtime and the CUDA kernels.
//
// HBM layout (one scene):
//   vertices   DVertex[V]   48 B/vertex  {pos.xyz, u} {normal.xyz, v} {tangent.xyzw}
//   indices    u32[3T]      primitive-local, rebased by DPrimitive.vtx_base
//   prims      DPrimitive[] nodes DNode[] materials DMaterial[] textures DTexture[]
//   texels     u32 pool     RGBA8, R in MSB, every mip of every texture
//   voxel      f32[N^3]     blurred sun visibility (the only per-voxel data the
//                           non-GI shading path reads; the SH part is constant)
//
// Per frame (renderer-owned):
//   draws      DDraw[D]     (node, primitive) pairs in canonical order, + MVP
//   chunks     DChunk[]     256-triangle slices of draws, one CTA each
//   tri_state  u8[T]        0 none, 1 record in slot g, 2 clipped
//   rec_r      RecRaster[T + extra]   80 B: screen vertices, bbox, z/w, 1/w, depth floor
//   rec_s      RecShade [T + extra]  176 B: shading interpolators
//   fan_base   u32[T]       first extra slot of a clipped triangle's fans 1..6
//   bins       u32[cap]     record indices grouped by scheduling tile
//   keys       u64[pitch*rows] per view: orderable(z) << 32 | ~(seq8 + 1)
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace swr {

constexpr int kRefTile = 64;          // reference tile size, src/renderer.rs:14
constexpr int kSubpixelScale = 16;    // src/tilerasterizer.rs:10
constexpr int kSubpixelShift = 4;
constexpr int kChunkTris = 256;       // triangles per front-end CTA
constexpr uint64_t kEmptyKey = 0xFF800000FFFFFFFFull;  // orderable(+inf) << 32 | 0xFFFFFFFF

struct alignas(16) DVertex {
    float px, py, pz, u;
    float nx, ny, nz, v;
    float tx, ty, tz, tw;
};

struct alignas(16) DPrimitive {
    uint32_t vtx_base;
    uint32_t idx_base;
    uint32_t tri_count;
    uint32_t material;
};

struct alignas(16) DTexture {
    const uint32_t* data;      // device pointer to mip 0 of this texture
    uint32_t width, height;
    uint32_t max_mip;
    uint32_t pad0;
    float whv[4];              // width_height_vec
    uint32_t mip_offset[16];   // relative to data
    uint32_t mip_w[16];
    uint32_t mip_h[16];
    uint32_t array_stride[16];
    float mip_wf[16];
    float mip_hf[16];
    // 1 / mip_wf (1 / mip_hf) when that size is a power of two, else 0: a
    // division by 2^k and a multiplication by 2^-k round the same exact value.
    float mip_rwf[16];
    float mip_rhf[16];
};

enum : uint32_t {
    MAT_ALPHA_TESTED = 1u,
    MAT_TRANSLUCENT = 2u,
};

// Texture slots inside DMaterial.tex.
enum { TS_BASE = 0, TS_MR = 1, TS_NORMAL = 2, TS_EMISSIVE = 3, TS_OCCLUSION = 4, TS_TRANSMISSION = 5 };

struct alignas(16) DMaterial {
    float base_color[4];
    float metallic, roughness, occlusion_strength, alpha_cutoff;
    float emissive[3];
    uint32_t flags;
    int32_t tex[6];            // index into scene texture table, -1 none
    uint32_t wrap_s[6];
    uint32_t wrap_t[6];
    float transmission;
    uint32_t pad[1];
};

// Draw-list inputs (render_node / render_mesh, src/renderer.rs:357-420),
// laid out so one node needs two dependent reads: per node its world
// transform, static triangle base and its mesh's entry range; per mesh entry
// (opaque primitives, then translucent ones) the primitive, its local
// bounding sphere, triangle count and static triangle base within the mesh.
struct alignas(16) DNodeInfo {
    float xform[16];
    uint32_t tri_id_base;
    uint32_t entry_begin;      // into DScene.mesh_entries
    uint32_t n_opaque;
    uint32_t n_total;          // 0 for a node without a mesh
};
struct alignas(16) DMeshEntry {
    float sphere[4];
    uint32_t prim;             // global primitive index
    uint32_t tri_count;
    uint32_t tri_id_base;
    uint32_t pad;
};

// Scene-wide device constants. The per-voxel SH4 of the non-GI path is
// the same for every voxel (src/gi.rs:123-149): rgb = irradiance_sh * scale,
// w0 = light intensity (per voxel), w1 = sky visibility, w2 = w3 = 0.
struct alignas(16) DScene {
    const DVertex* vertices;
    const uint32_t* indices;
    const DPrimitive* prims;
    const float* node_xform;   // 16 floats per node
    const DMaterial* materials;
    const DTexture* textures;  // scene textures, then cubemap, specular, brdf lut
    const float* voxel_light;  // voxel_n^3
    const DNodeInfo* node_info;
    const DMeshEntry* mesh_entries;
    const float4* voxel_sh4;   // baked GI: voxel_n^3 x 4 (r, g, b, w), or null (constant SH form)
    uint32_t tex_cubemap, tex_specular, tex_brdf_lut, voxel_n;
    float voxel_min[3];
    float voxel_size_f[3];     // (max - min) / n per axis
    float gi_rgb[4][3];
    float sky_visibility;
    float light_dir[3];
    float light_color[3];
    float pad[3];
};

// One view (camera + resolution + outputs).
struct alignas(16) DView {
    float skybox_t[16];        // RenderCamera::skybox_matrix_transposed
    float cam_pos[3];
    float one_over_width, one_over_height;
    float width_f, height_f;
    float exposure;
    int32_t width, height;
    int32_t tiles_x, tiles_y;  // 64-px reference tiles
    int32_t stiles_x, stiles_y;// scheduling tiles
    uint32_t stile_base;       // first bin of this view
    uint32_t scene;            // index into the DScene table
    uint32_t quad_base;        // first shading quad of this view
    uint32_t quad_pitch;       // tiles_x * 32
    uint32_t rsqrt_mode;
    uint32_t flags;            // kViewLinear / kViewTranslucent: linear colour instead of RGBA8
    uint64_t key_offset;       // into the key buffer (u64 elements)
    uint64_t key_pitch;        // tiles_x * 64
    uint32_t* rgba8;           // width*height, row pitch out_pitch
    uint64_t* vis;             // width*height
    float* color;              // key_pitch * tiles_y * 64 * 3 (padded tile grid) when flags != 0
    float* tile_lum;           // tiles_x*tiles_y
    uint32_t out_pitch;
    uint32_t host_pitch;       // row pitch of rgba8_host
    uint32_t* rgba8_host;      // device-writable host copy of rgba8 (rows below height & ~1), or null
    // Camera of the device draw-list build (RenderCamera, src/rendercamera.rs).
    float cam_view[16];
    float cam_view_project[16];
    float cam_planes[24];      // view_clip_planes, view space
    uint32_t order_base;       // this view's sorted nodes in FrameArgs.node_order
    uint32_t n_order;
    uint32_t tiles_x_magic;    // ceil(2^32 / tiles_x), 0 when tiles_x == 1 (quad row = (q >> 5) * magic >> 32)
    uint32_t pad3;
};

// DView.flags
constexpr uint32_t kViewLinear = 1u;       // caller wants linear colour (exposure applied later)
constexpr uint32_t kViewTranslucent = 2u;  // view has translucent draws: shade, blend, then resolve
                                           // (set on the device by the draw-list build)

struct alignas(16) DDraw {
    float mvp[16];
    uint32_t node;
    uint32_t prim;
    uint32_t view;
    uint32_t clip;             // primitive's sphere intersects the frustum
    uint32_t tri_begin;        // global triangle index of this draw's triangle 0
    uint32_t tri_count;
    uint32_t static_base;      // static triangle ID of triangle 0
    uint32_t scene;
    uint32_t translucent;      // primitive of a translucent material (mesh.primitives_translucent)
    uint32_t pad[3];
};

struct DChunk {
    uint32_t draw;
    uint32_t tri_start;        // local to the draw
};

// RecRaster.material carries the alpha-test flag in its top bit and the
// translucent flag below it; RecShade.pad[0] holds a translucent record's
// average clip-space z (the sort key).
constexpr uint32_t kRecAlphaBit = 0x80000000u;
constexpr uint32_t kRecTransBit = 0x40000000u;
constexpr uint32_t kRecMaterialMask = 0x3FFFFFFFu;

// Raster-side triangle record (one per emitted, non-culled triangle).
struct alignas(16) RecRaster {
    int32_t p[6];              // screen subpixel positions p0, p1, p2
    uint16_t bb[4];            // screen_min_pixels.xy, screen_max_pixels.xy (0..32769)
    float ooa;                 // one_over_area
    float zow[3];              // z_over_w interpolator (a, da, db)
    float oow[3];              // one_over_w interpolator
    uint32_t seq8;             // (global triangle index << 3) | fan
    uint32_t material;
    uint32_t view;
    uint32_t zfloor;           // orderable depth floor of the whole triangle (occlusion culling), 0 = none
    uint32_t pad;
};
static_assert(sizeof(RecRaster) == 80, "RecRaster layout");

// Shading-side record.
struct alignas(16) RecShade {
    float nrm[9];              // normals a.xyz, da.xyz, db.xyz
    float tan[9];
    float tsign[3];
    float uow[3];
    float vow[3];
    float pww[9];              // pos_world_over_w
    float du_dv[4];
    uint32_t static_id;
    uint32_t pad[3];
};
static_assert(sizeof(RecShade) == 176, "RecShade layout");

// Device status word bits.
enum : uint32_t {
    ST_BIN_OVERFLOW = 1u,
    ST_CLIP_OVERFLOW = 2u,
    ST_QUEUE_OVERFLOW = 4u,
    ST_TIMEOUT = 8u,
    ST_TRANS_OVERFLOW = 16u,   // a scheduling tile has more translucent packets than one sort holds
    ST_DRAW_OVERFLOW = 32u,    // the frame's draws have more triangles (or draws, chunks) than allocated
};
// Status bits after which a frame is incomplete and is rendered again.
constexpr uint32_t kStRetry =
    ST_BIN_OVERFLOW | ST_CLIP_OVERFLOW | ST_QUEUE_OVERFLOW | ST_TRANS_OVERFLOW | ST_DRAW_OVERFLOW;

// Frame-level counters (device).
struct alignas(16) DCounters {
    uint32_t status;
    uint32_t clip_queue;       // triangles queued for clipping
    uint32_t extra_used;       // extra record slots taken by fans 1..6
    uint32_t setup_tris;       // records written
    unsigned long long pairs;  // (triangle, tile) pairs counted
    uint32_t work_next;        // persistent raster work cursor
    uint32_t trans_next;       // translucent pass work cursor
    uint32_t trans_packets;    // translucent (packet, tile) pairs
    uint32_t draw_tris;        // triangles of the frame's draws (the draw-list build's T)
    uint32_t draw_done;        // CTAs done counting draws (zero between frames)
    uint32_t draw_chunks;      // chunks and draws of the frame's draw list
    uint32_t draw_count;
    uint32_t culled;           // (triangle, tile) pairs the raster dropped as hidden
    uint32_t clip_path;        // triangles of draws whose sphere intersects the frustum (the clip path)
};

// Per-frame counts, uploaded with the tables: kernels read them from device
// memory so a launch sequence captured once (grids sized by capacity)
// serves any batch that fits the capacities.
struct alignas(16) DFrameDyn {
    uint32_t n_views;
    uint32_t n_chunks;
    uint32_t tri_total;        // T: main record slots used this frame
    uint32_t n_stiles;         // bins over all views
    uint32_t total_quads;      // shading work over all views
    uint32_t max_view_pixels;  // largest width * (height & ~1)
    uint32_t n_bins;           // n_stiles, or 2 * n_stiles with translucent bins after the opaque ones
    uint32_t n_slots;          // node slots of all views (device draw-list build)
};

// Everything a frame's kernels need, passed by value: pointers and
// capacities only (they change only when buffers grow).
struct FrameArgs {
    DFrameDyn* dyn;            // n_chunks and tri_total written by the draw-list build
    const DScene* scenes;
    DView* views;              // flags gain kViewTranslucent in the draw-list build
    DDraw* draws;
    DChunk* chunks;
    uint32_t chunk_cap;        // grid of k_frontend
    uint32_t tri_cap;          // main record slots allocated
    uint32_t extra_cap;        // extra record slots
    uint32_t clip_cap;         // clip queue capacity
    uint32_t stile_cap;        // bins allocated
    uint32_t quad_cap;         // shading quads allocated (grid bound)
    uint32_t pixel_cap;        // largest view's pixels (resolve grid)
    uint32_t view_cap;
    uint64_t bin_cap;
    uint32_t sched_tile;       // S
    uint32_t pad0;
    uint8_t* tri_state;
    RecRaster* rec_r;
    RecShade* rec_s;
    uint32_t* fan_base;
    uint2* clip_queue;         // (g, draw)
    uint32_t* tile_count;      // n_bins; after k_scan, the raster tile order
    uint32_t* tile_offset;     // n_bins + 1
    uint32_t* tile_cursor;     // n_bins
    uint32_t* bins;
    unsigned long long* keys;
    DCounters* counters;
    const uint8_t* rsqrt_table;// 512 entries, FRSQRTE estimates
    const float* exposure_dev; // exposure computed by the host step (dt > 0)
    uint32_t raster_grid;      // persistent raster CTAs
    uint32_t shade_grid;       // grid-stride shading CTAs
    uint32_t has_translucent;  // some view's scene has translucent primitives: run the translucent pass
    uint32_t defer_resolve;    // the caller launches the resolve (exposure from the host step)
    const uint32_t* node_order;// node slots: per view, node indices nearest first (device draw-list build)
    uint4* slot_blocks;        // per 256 node slots: draws, triangles, chunks; then their exclusive offsets
    uint32_t draw_cap;
    uint32_t slot_cap;
    uint32_t fused_shade;      // 32-px tiles: shade inside the raster kernel (8 and 16 px always do)
    uint32_t has_gi;           // some scene of the frame has a baked voxel grid
    uint32_t gpu_draws;        // build draws and chunks on the device (else the host staged them)
    uint32_t rsqrt_uniform;    // 1 + the rsqrt mode all views share, 0 = per view
};

// Launch wrappers (kernels.cu). `ev`, when given, holds 8 events recorded
// before reset, frontend, clip, scan, scatter, raster, shade and after shade.
// Enqueues one frame's kernels; returns how many it launched.
uint32_t launch_frame(const FrameArgs& a, void* stream, int num_sms, cudaEvent_t* ev = nullptr);
void launch_reset(const FrameArgs& a, void* stream);
void launch_resolve(const FrameArgs& a, void* stream);
// rsqrt of n device values in the given mode (table: the 512-byte FRSQRTE table).
cudaError_t launch_rsqrt_selftest(const float* in, float* out, uint64_t n, uint32_t mode, const uint8_t* table);
// The raster's occlusion-culling depth floor evaluated on the host (the
// device code's source compiled for the host).
bool depth_floor_host(const int32_t p[6], const float zow[3], const float oow[3], int32_t xe, int32_t ye, float& zlo);
// Per-device constant tables; call once per device outside stream capture.
cudaError_t init_kernel_constants();
// Persistent raster / grid-stride shading grid sizes for this device.
void frame_grids(int num_sms, uint32_t sched_tile, bool fuse32, uint32_t* raster_grid, uint32_t* shade_grid);
// Whether frames with this scheduling tile shade inside the raster kernel.
bool shade_fused(uint32_t sched_tile, bool fuse32);

}  // namespace swr
