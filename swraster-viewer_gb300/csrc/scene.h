// Host-side scene representation (the reference's Scene after load,
// src/scene.rs:65-121) and its HBM copy.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/swr.h"
#include "hostmath.h"
#include "internal.h"

namespace swr {

// Texture with mip chain (src/texture.rs:28-42).
struct HTexture {
    uint32_t width = 0, height = 0, type = SWR_TEX_LINEAR;
    std::vector<uint32_t> data;
    uint32_t max_mip = 0;
    std::vector<uint32_t> mip_offsets, mip_widths, mip_heights, array_stride;
    std::vector<float> mip_widths_f, mip_heights_f;
    float whv[4] = {0, 0, 0, 0};
    void generate_mipmaps();
    // Appends the mip levels' metadata generate_mipmaps would (offsets,
    // sizes, strides); data keeps level 0.
    void mip_layout();
    swr_texture_view view() const;
};

struct HPrimitive {
    std::vector<float> pos4, nrm4, tan4, uv2;
    std::vector<uint32_t> idx;
    uint32_t material = 0;
    uint32_t tri_id_base = 0;  // within the mesh
    float sphere[4] = {0, 0, 0, 0};
};

struct HMesh {
    std::vector<uint32_t> prims;  // global primitive indices
    std::vector<uint32_t> opaque, translucent;  // local indices
    uint32_t tri_count = 0;
};

struct HNode {
    M4 transform;
    float sphere[4] = {0, 0, 0, 0};
    int32_t mesh = -1;
    uint32_t tri_id_base = 0;
};

struct SceneImpl {
    std::vector<HPrimitive> prims;
    std::vector<HMesh> meshes;
    std::vector<HNode> nodes;
    std::vector<swr_material_view> materials;
    std::vector<HTexture> textures;
    HTexture cubemap, specular, brdf_lut;
    float irradiance_sh[4][3] = {};
    V3 light_dir{}, light_color{};
    V3 bounds_min{}, bounds_max{}, bounds_center{};
    float bounds_diagonal = 0;
    uint32_t voxel_n = 0;
    V3 voxel_min{}, voxel_max{};
    std::vector<float> voxel_light;
    std::vector<float> voxel_sh4;  // SWR_SCENE_GI: n^3 x 4 (r, g, b, w), blurred; empty otherwise
    float gi_sh_scale = 0.25f, sky_visibility = 1.0f;
    float gi_const[4][4] = {};
    uint64_t tri_total = 0, vtx_total = 0;
    // Draw-list bounds of one view (every primitive in the frustum).
    uint32_t max_draws = 0, max_chunks = 0;
    bool any_translucent = false;  // some node's mesh has translucent primitives
    uint32_t gi_cache = 0, ggx_cache = 0;  // SWR_CACHE_*
    uint64_t precompute_host_texels = 0;   // device precompute texels recomputed on the host

    // Export views.
    std::vector<swr_primitive_view> prim_views;
    std::vector<swr_mesh_view> mesh_views;
    std::vector<swr_node_view> node_views;
    std::vector<swr_texture_view> tex_views;

    // Device copy.
    void* d_block = nullptr;   // one allocation for everything
    uint64_t d_bytes = 0;
    DScene dscene{};
    DScene* d_scene = nullptr; // device copy of dscene
};

swr_status build_scene(const swr_scene_desc* desc, SceneImpl* s, std::string& err);
swr_status upload_scene(SceneImpl* s, std::string& err, bool to_device);
void free_scene_device(SceneImpl* s);
void export_scene(const SceneImpl* s, swr_scene_host_view* out);

// FRSQRTE estimate table (RecipSqrtEstimate, 9-bit operand -> estimate<7:0>).
void build_rsqrt_table(uint8_t out[512]);

}  // namespace swr

struct swr_scene {
    swr::SceneImpl impl;
};
