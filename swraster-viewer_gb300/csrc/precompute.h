// Load-time scene precompute on the device: the voxel grid's sun visibility
// (compute_sun_visibility + blur_grid, src/gi.rs:267-314 and
// src/voxelgrid.rs:370-419, with RayTracer::trace_transmittance,
// src/raytracer.rs:172-207).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/swr.h"

namespace swr {

// A world-space triangle of the ray tracer (RayTracer::new drops degenerate
// ones, src/raytracer.rs:71-133).
struct LightTri {
    float p0[3], p1[3], p2[3];
    uint32_t material;
};

// Transmittance toward the sun from every active voxel centre (1 for inactive
// voxels), then the 3x3x3 mean squared, into `out` (n^3 floats, x fastest).
// Equal to the host restatement bit for bit: the same float operations in the
// same order, and translucent hits multiplied in (t, triangle index) order.
// `cmin` is the first voxel centre, `ld` the normalised light direction.
swr_status sun_visibility_device(const LightTri* tris, size_t ntris, const uint8_t* translucent,
                                 const float* transmission, uint32_t nmat, const uint8_t* active, uint32_t n,
                                 const float bounds_min[3], const float bounds_max[3], const float cmin[3],
                                 const float vsz[3], const float ld[3], float bias, float* out, std::string& err);

// --- Voxel GI bake (bake_voxel_gi, src/gi.rs:316-408) --------------------
// RayTracer triangle with what a bounce needs (src/raytracer.rs:35-45).
struct BakeTri {
    float p0[3], p1[3], p2[3], n[3];
    float uv0[2], uv1[2], uv2[2];
    uint32_t material;
};
// BVH node over BakeTri indices (leaves: triangles order[left .. left+count)).
struct BakeNode {
    float mn[3], mx[3];
    uint32_t left, count;
};
struct BakeMaterial {
    float base[3], emissive[3];
    int32_t base_tex, emissive_tex;  // into BakeInput.textures, -1 none
    uint32_t base_wrap_s, base_wrap_t, emissive_wrap_s, emissive_wrap_t;
    uint32_t translucent;
    float transmission;
};
struct BakeTexture {
    uint32_t offset, width, height;  // mip 0 in the texel pool
};
struct BakeInput {
    const BakeTri* tris = nullptr;
    size_t ntris = 0;
    const BakeNode* nodes = nullptr;
    size_t nnodes = 0;
    const uint32_t* order = nullptr;
    const BakeMaterial* mats = nullptr;
    uint32_t nmat = 0;
    const uint32_t* texels = nullptr;  // RGBA8, R in the MSB
    size_t ntexels = 0;
    const BakeTexture* textures = nullptr;
    uint32_t ntex = 0;
    const uint32_t* cubemap = nullptr;  // mip 0, six faces
    uint32_t cube_size = 0;
    const float* sky_lut = nullptr;     // srgb_to_linear_scalar(b / 255) for every byte b
    const float* dirs = nullptr;        // direction sets, 9 x 64 x 3
    float irradiance_sh[4][3] = {};
    float light_dir[3] = {}, light_color[3] = {};
    uint32_t n = 0;
    float bounds_min[3] = {}, vsz[3] = {}, cmin[3] = {};
    const uint8_t* active = nullptr;    // n^3
    const float* sun = nullptr;         // n^3, blurred sun visibility
};
constexpr uint32_t kGiSamples = 64, kGiSets = 9;

// bake_voxel_gi + blur_gi_sh4 on the device: `out` gets n^3 voxels of four
// (r, g, b, w) SH4 coefficients, equal to the host restatement bit for bit.
// Surface textures are sampled bilinearly on the device and converted to
// linear on the host (srgb_to_linear_scalar with the host's powf), between
// the two kernels of each chunk of voxels.
swr_status gi_bake_device(const BakeInput& in, float* out, std::string& err);
float srgb_to_linear_host(float s);

}  // namespace swr
