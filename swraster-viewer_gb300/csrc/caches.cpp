// Load-time cache files of the reference's scene load:
//   - the GGX-prefiltered environment, assets/cubemap.ggx: magic "GGX0",
//     version 1, face width, face height, mip count (src/texture.rs:12-17,
//     425-554);
//   - the baked voxel GI of a scene, <scene>.gi: magic "VGI0", version 8,
//     grid width, height, depth (src/gi.rs:14-117).
// Each file is a 20-byte little-endian header followed by one brotli stream
// of the payload (little-endian u32 texels / f32 SH4 coefficients, in the
// tables' own order). The reference compresses at quality 6 with a 2^22-byte
// window; any conforming brotli stream of the same payload reads the same.
// The codec is the system's libbrotlienc / libbrotlidec, opened on first use:
// without them no cache is read or written and the tables are computed as if
// the file were absent.
#include <dlfcn.h>

#include <cstdio>
#include <cstring>
#include <mutex>

#include "caches.h"

namespace swr {

namespace {

constexpr uint32_t kHeaderBytes = 20;
constexpr int kQuality = 6;   // GGX_CACHE_BROTLI_QUALITY, GI_CACHE_BROTLI_QUALITY
constexpr int kLgWin = 22;    // GGX_CACHE_BROTLI_LGWIN, GI_CACHE_BROTLI_LGWIN
constexpr uint32_t kGgxVersion = 1;
constexpr uint32_t kGiVersion = 8;

// The brotli C API (brotli/encode.h, brotli/decode.h): names and signatures.
using EncCompress = int (*)(int quality, int lgwin, int mode, size_t input_size, const uint8_t* input,
                            size_t* encoded_size, uint8_t* encoded);
using EncMaxSize = size_t (*)(size_t input_size);
using DecCreate = void* (*)(void* alloc_func, void* free_func, void* opaque);
using DecStream = int (*)(void* state, size_t* available_in, const uint8_t** next_in, size_t* available_out,
                          uint8_t** next_out, size_t* total_out);
using DecDestroy = void (*)(void* state);
enum { kDecError = 0, kDecSuccess = 1, kDecNeedsInput = 2, kDecNeedsOutput = 3 };
constexpr int kModeGeneric = 0;

struct Codec {
    EncCompress compress = nullptr;
    EncMaxSize max_size = nullptr;
    DecCreate create = nullptr;
    DecStream stream = nullptr;
    DecDestroy destroy = nullptr;
    bool ok = false;
};

void* open_first(const char* a, const char* b) {
    void* h = dlopen(a, RTLD_NOW | RTLD_LOCAL);
    return h ? h : dlopen(b, RTLD_NOW | RTLD_LOCAL);
}

const Codec& codec() {
    static Codec c;
    static std::once_flag once;
    std::call_once(once, [] {
        void* enc = open_first("libbrotlienc.so.1", "libbrotlienc.so");
        void* dec = open_first("libbrotlidec.so.1", "libbrotlidec.so");
        if (!enc || !dec) return;
        c.compress = reinterpret_cast<EncCompress>(dlsym(enc, "BrotliEncoderCompress"));
        c.max_size = reinterpret_cast<EncMaxSize>(dlsym(enc, "BrotliEncoderMaxCompressedSize"));
        c.create = reinterpret_cast<DecCreate>(dlsym(dec, "BrotliDecoderCreateInstance"));
        c.stream = reinterpret_cast<DecStream>(dlsym(dec, "BrotliDecoderDecompressStream"));
        c.destroy = reinterpret_cast<DecDestroy>(dlsym(dec, "BrotliDecoderDestroyInstance"));
        c.ok = c.compress && c.max_size && c.create && c.stream && c.destroy;
    });
    return c;
}

uint32_t le32(const uint8_t* p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}
void put32(std::vector<uint8_t>& b, uint32_t v) {
    for (int k = 0; k < 4; ++k) b.push_back((uint8_t)(v >> (8 * k)));
}

// fs::read: Err when the file exists but cannot be read.
bool read_file(const char* path, std::vector<uint8_t>& out, bool& exists) {
    exists = false;
    FILE* f = std::fopen(path, "rb");
    if (!f) return true;
    exists = true;
    bool ok = std::fseek(f, 0, SEEK_END) == 0;
    const long n = ok ? std::ftell(f) : -1;
    ok = ok && n >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
    if (ok) {
        out.resize((size_t)n);
        ok = n == 0 || std::fread(out.data(), 1, (size_t)n, f) == (size_t)n;
    }
    std::fclose(f);
    return ok;
}

// The whole brotli stream after the header, into `out` (exactly `expected`
// bytes kept; the decoded size is returned in `total`). false: the stream is
// corrupt or ends early (the reference's read_to_end fails).
bool decompress(const uint8_t* in, size_t in_len, size_t expected, std::vector<uint8_t>& out, size_t& total) {
    const Codec& c = codec();
    void* st = c.create(nullptr, nullptr, nullptr);
    if (!st) return false;
    out.assign(expected, 0);
    std::vector<uint8_t> spill(1 << 16);
    size_t avail_in = in_len;
    const uint8_t* next_in = in;
    total = 0;
    int r = kDecNeedsOutput;
    while (r == kDecNeedsOutput) {
        // Decoded bytes past `expected` go to a scratch buffer and are only
        // counted: the size check below rejects such a payload.
        uint8_t* next_out;
        size_t avail_out;
        if (total < expected) {
            next_out = out.data() + total;
            avail_out = expected - total;
        } else {
            next_out = spill.data();
            avail_out = spill.size();
        }
        size_t t = 0;
        r = c.stream(st, &avail_in, &next_in, &avail_out, &next_out, &t);
        total = t;
    }
    c.destroy(st);
    return r == kDecSuccess;
}

bool write_file(const char* path, const uint8_t* head, size_t head_len, const std::vector<uint8_t>& payload,
                std::string& err) {
    const Codec& c = codec();
    std::vector<uint8_t> enc(c.max_size(payload.size()) + 16);
    size_t enc_len = enc.size();
    if (!c.compress(kQuality, kLgWin, kModeGeneric, payload.size(), payload.data(), &enc_len, enc.data())) {
        err = "brotli compression failed";
        return false;
    }
    FILE* f = std::fopen(path, "wb");
    if (!f) {
        err = std::string("cannot create ") + path;
        return false;
    }
    bool ok = std::fwrite(head, 1, head_len, f) == head_len && std::fwrite(enc.data(), 1, enc_len, f) == enc_len;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) err = std::string("write failed: ") + path;
    return ok;
}

// Reads a cache file: header check, then the payload of `payload_len` bytes.
CacheRead read_cache(const char* path, const char magic[4], uint32_t version, const uint32_t dims[3],
                     size_t payload_len, std::vector<uint8_t>& payload, std::string& msg) {
    if (!codec().ok) return CacheRead::NoCodec;
    std::vector<uint8_t> bytes;
    bool exists = false;
    if (!read_file(path, bytes, exists)) {
        msg = std::string("cannot read ") + path;
        return CacheRead::Error;
    }
    if (!exists || bytes.size() < kHeaderBytes || std::memcmp(bytes.data(), magic, 4) != 0 ||
        le32(&bytes[4]) != version)
        return CacheRead::Miss;
    for (int k = 0; k < 3; ++k)
        if (le32(&bytes[8 + 4 * k]) != dims[k]) return CacheRead::Miss;
    size_t total = 0;
    if (!decompress(bytes.data() + kHeaderBytes, bytes.size() - kHeaderBytes, payload_len, payload, total)) {
        msg = std::string("corrupt brotli stream in ") + path;
        return CacheRead::Error;
    }
    return total == payload_len ? CacheRead::Loaded : CacheRead::Miss;
}

std::vector<uint8_t> header(const char magic[4], uint32_t version, const uint32_t dims[3]) {
    std::vector<uint8_t> h(magic, magic + 4);
    put32(h, version);
    for (int k = 0; k < 3; ++k) put32(h, dims[k]);
    return h;
}

uint32_t ggx_mips(uint32_t w, uint32_t h) { return 1u + (31u - (uint32_t)__builtin_clz(w > h ? w : h)); }

}  // namespace

bool cache_codec_available() { return codec().ok; }

CacheRead read_ggx_cache(const char* path, uint32_t width, uint32_t height, HTexture& out, std::string& msg) {
    const uint32_t mips = ggx_mips(width, height);
    const uint32_t dims[3] = {width, height, mips};
    const size_t face = (size_t)width * height;
    const size_t texels = face * 6 * mips;
    std::vector<uint8_t> payload;
    const CacheRead r = read_cache(path, "GGX0", kGgxVersion, dims, texels * 4, payload, msg);
    if (r != CacheRead::Loaded) return r;
    // The texture the reference rebuilds from the file: every mip at full
    // face resolution, six faces each, Linear (src/texture.rs:475-518).
    HTexture t;
    t.width = width;
    t.height = height;
    t.type = SWR_TEX_LINEAR;
    t.data.resize(texels);
    for (size_t i = 0; i < texels; ++i) t.data[i] = le32(&payload[4 * i]);
    t.max_mip = mips - 1;
    for (uint32_t m = 0; m < mips; ++m) {
        t.mip_offsets.push_back((uint32_t)(face * 6 * m));
        t.mip_widths.push_back(width);
        t.mip_heights.push_back(height);
        t.mip_widths_f.push_back((float)width);
        t.mip_heights_f.push_back((float)height);
        t.array_stride.push_back((uint32_t)face);
    }
    t.whv[0] = t.whv[1] = (float)width;
    t.whv[2] = t.whv[3] = (float)height;
    out = std::move(t);
    return CacheRead::Loaded;
}

bool write_ggx_cache(const char* path, const HTexture& t, std::string& err) {
    if (!codec().ok) {
        err = "no brotli codec (libbrotlienc/libbrotlidec) on this system";
        return false;
    }
    const uint32_t mips = t.max_mip + 1;
    if (t.data.size() != (size_t)t.width * t.height * 6 * mips) {
        // save_prefiltered_specular_cubemap_cache's size check.
        err = "prefiltered cubemap texture has unexpected data size";
        return false;
    }
    const uint32_t dims[3] = {t.width, t.height, mips};
    const std::vector<uint8_t> head = header("GGX0", kGgxVersion, dims);
    std::vector<uint8_t> payload;
    payload.reserve(t.data.size() * 4);
    for (uint32_t v : t.data) put32(payload, v);
    return write_file(path, head.data(), head.size(), payload, err);
}

CacheRead read_gi_cache(const char* path, uint32_t n, std::vector<float>& sh4, std::string& msg) {
    const uint32_t dims[3] = {n, n, n};
    const size_t floats = (size_t)n * n * n * 16;
    std::vector<uint8_t> payload;
    const CacheRead r = read_cache(path, "VGI0", kGiVersion, dims, floats * 4, payload, msg);
    if (r != CacheRead::Loaded) return r;
    sh4.resize(floats);
    for (size_t i = 0; i < floats; ++i) {
        const uint32_t u = le32(&payload[4 * i]);
        std::memcpy(&sh4[i], &u, 4);
    }
    return CacheRead::Loaded;
}

bool write_gi_cache(const char* path, uint32_t n, const std::vector<float>& sh4, std::string& err) {
    if (!codec().ok) {
        err = "no brotli codec (libbrotlienc/libbrotlidec) on this system";
        return false;
    }
    if (sh4.size() != (size_t)n * n * n * 16) {
        err = "the scene has no baked GI grid";
        return false;
    }
    const uint32_t dims[3] = {n, n, n};
    const std::vector<uint8_t> head = header("VGI0", kGiVersion, dims);
    std::vector<uint8_t> payload;
    payload.reserve(sh4.size() * 4);
    for (float f : sh4) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        put32(payload, u);
    }
    return write_file(path, head.data(), head.size(), payload, err);
}

}  // namespace swr
