// Load-time texture precompute on the device: mip chains
// (Texture::generate_mipmaps, src/texture.rs:45-128), the BRDF LUT
// (generate_brdf_lut, src/texture.rs:199-243) and the GGX-prefiltered
// environment (generate_prefiltered_specular_cubemap, src/texture.rs:330-420).
//
// Results equal the host restatement bit for bit. Everything but powf is
// IEEE single-precision arithmetic in the host's order, and powf appears
// only on the way to an 8-bit texel:
//   - sRGB mips: both conversions go through host-made tables (the 256
//     linear values of the bytes, and for the way back the smallest float
//     that packs to each byte), so the device calls no powf;
//   - GGX prefilter: for each powf of an interpolated sample the device takes
//     the interval [p - W ulp, p + W ulp] around its own powf p, which holds
//     the host libm's value (tests/test_ibl_device.py measures the two
//     functions over every input the samples can pass), and carries both ends
//     through the monotone arithmetic that follows (sums of positive terms, a
//     division by a positive total, the scale to 0..255 and the truncation).
//     Where both ends give the same byte, it is the host's; the few texels
//     where they differ are computed again on the host.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "scene.h"

namespace swr {

// The host's per-texel functions (scene.cpp), used for the recomputed texels.
uint32_t mip_texel(uint32_t type, uint32_t p00, uint32_t p10, uint32_t p01, uint32_t p11);
uint32_t prefilter_texel(const HTexture& cube, uint32_t mip, uint32_t max_mip, uint32_t face, uint32_t x, uint32_t y,
                         uint32_t sample_count, const float* xi_x, const float* xi_y);
float srgb_to_linear_host(float s);
// For k = 1..255, out[k - 1] = the smallest float above 0.0031308 (the powf
// branch of linear_to_srgb_scalar) whose packed byte is at least k, or
// +infinity where no value up to 1 reaches k.
void srgb_byte_thresholds(float out[255]);
// hammersley(i, n) and cos / sin of its angle 2*pi*x (either may be null).
void hammersley_table(uint32_t n, float* xi_x, float* xi_y, float* cos_phi, float* sin_phi);
HTexture prefiltered_layout(uint32_t width, uint32_t height);

// Fills the mip levels of every texture (level 0 given, metadata for level 0
// only, as make_texture leaves it).
swr_status mipmaps_device(const std::vector<HTexture*>& textures, std::string& err);
// generate_brdf_lut(size), mips included.
swr_status brdf_lut_device(uint32_t size, HTexture& out, std::string& err);
// generate_prefiltered_specular_cubemap(cube, samples): mip 0 of `cube` is
// read; adds to `host_texels` the texels computed again on the host.
swr_status prefiltered_specular_device(const HTexture& cube, uint32_t samples, HTexture& out, uint64_t& host_texels,
                                       std::string& err);

// powf(x, 2.4) (mode 0) or powf(x, 1/2.4) (mode 1) as the device tables
// compute them, over n device values (test entry point).
swr_status srgb_pow_selftest(const float* in, float* out, uint64_t n, uint32_t mode, std::string& err);

}  // namespace swr
