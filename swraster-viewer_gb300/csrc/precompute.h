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

}  // namespace swr
