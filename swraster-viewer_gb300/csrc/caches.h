// Cache files of the reference's scene load (caches.cpp): the GGX-prefiltered
// environment (src/texture.rs:425-554) and the baked voxel GI
// (src/gi.rs:30-117).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "scene.h"

namespace swr {

// Outcome of reading a cache file, as the reference's loaders return it:
// Loaded (Ok(Some)/Ok(true)); Miss (Ok(None)/Ok(false): no file, another
// magic, version or size); Error (Err: unreadable file or corrupt stream;
// the caller recomputes); NoCodec (no brotli library on this system).
enum class CacheRead { Loaded, Miss, Error, NoCodec };

bool cache_codec_available();

// assets/cubemap.ggx for a cubemap of width x height faces.
CacheRead read_ggx_cache(const char* path, uint32_t width, uint32_t height, HTexture& out, std::string& msg);
bool write_ggx_cache(const char* path, const HTexture& prefiltered, std::string& err);

// <scene>.gi for an n^3 grid; sh4: n^3 x 4 coefficients x (r, g, b, w).
CacheRead read_gi_cache(const char* path, uint32_t n, std::vector<float>& sh4, std::string& msg);
bool write_gi_cache(const char* path, uint32_t n, const std::vector<float>& sh4, std::string& err);

}  // namespace swr
