// Image decoding for the glTF loader: PNG (every colour type and bit depth,
// Adam7 interlacing) and baseline/extended-sequential JPEG, to 8-bit RGBA
// rows (R, G, B, A bytes per pixel), the layout the reference gets from
// image::open(..).to_rgba8() (src/texture.rs:913-917).
//
// PNG is lossless, so decoded texels equal the reference's. JPEG decoders
// differ in IDCT and chroma upsampling rounding; this one (float IDCT,
// replicated chroma, JFIF colour conversion) is not bit-identical to the
// reference's zune-jpeg, and textures decoded from JPEG can differ by a few
// levels per channel.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

namespace swr {

// Inflates a zlib stream (RFC 1950 header + RFC 1951 deflate data). At most
// `limit` bytes are produced; more is an error.
bool zlib_inflate(const uint8_t* src, size_t n, size_t limit, std::vector<uint8_t>& out, std::string& err);

bool decode_png(const uint8_t* data, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba,
                std::string& err);
bool decode_jpeg(const uint8_t* data, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba,
                 std::string& err);
// Chooses the decoder from the file signature.
bool decode_image(const uint8_t* data, size_t n, uint32_t& w, uint32_t& h, std::vector<uint8_t>& rgba,
                  std::string& err);

}  // namespace swr
