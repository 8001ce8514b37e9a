// glTF 2.0 loader: .gltf (external or data: buffers) and .glb files to a
// swr_scene_desc, then the in-memory scene build. Follows the reference's
// load path: load_gltf / import_buffers (src/main.rs:86-98), Scene::from_gltf
// (src/scene.rs:145-354), Primitive::from_gltf (src/scene.rs:439-495),
// Material::from_gltf and get_texture_and_sampler (src/scene.rs:637-780) and
// TextureCache::load_texture (src/texture.rs:896-1015).
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <new>
#include <set>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "../../include/swr.h"
#include "hostmath.h"
#include "imagedec.h"
#include "json.h"
#include "renderer.h"
#include "scene.h"

namespace swr {
namespace {

using json::Value;

bool read_file(const std::string& path, std::vector<uint8_t>& out, std::string& err) {
    // Regular files only: a directory opens for reading on Linux and reports
    // a size of LONG_MAX.
    struct stat st;
    if (::stat(path.c_str(), &st) != 0 || !S_ISREG(st.st_mode)) {
        err = "cannot open '" + path + "'";
        return false;
    }
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) {
        err = "cannot open '" + path + "'";
        return false;
    }
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (n < 0) {
        std::fclose(f);
        err = "cannot read '" + path + "'";
        return false;
    }
    out.resize((size_t)n);
    const size_t got = n ? std::fread(out.data(), 1, (size_t)n, f) : 0;
    std::fclose(f);
    if (got != (size_t)n) {
        err = "short read of '" + path + "'";
        return false;
    }
    return true;
}

bool base64_decode(const std::string& s, size_t from, std::vector<uint8_t>& out) {
    out.clear();
    uint32_t acc = 0;
    int bits = 0;
    for (size_t i = from; i < s.size(); ++i) {
        const char c = s[i];
        int v;
        if (c >= 'A' && c <= 'Z') v = c - 'A';
        else if (c >= 'a' && c <= 'z') v = c - 'a' + 26;
        else if (c >= '0' && c <= '9') v = c - '0' + 52;
        else if (c == '+' || c == '-') v = 62;
        else if (c == '/' || c == '_') v = 63;
        else if (c == '=') break;
        else if (c == ' ' || c == '\n' || c == '\r' || c == '\t') continue;
        else return false;
        acc = (acc << 6) | (uint32_t)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((uint8_t)(acc >> bits));
        }
    }
    return true;
}

std::string percent_decode(const std::string& s) {
    std::string o;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] == '%' && i + 2 < s.size() && std::isxdigit((unsigned char)s[i + 1]) &&
            std::isxdigit((unsigned char)s[i + 2])) {
            o += (char)std::stoi(s.substr(i + 1, 2), nullptr, 16);
            i += 2;
        } else {
            o += s[i];
        }
    }
    return o;
}

struct Doc {
    Value root;
    std::string base_dir;
    std::vector<std::vector<uint8_t>> buffers;
};

// --- accessors --------------------------------------------------------------

size_t comp_size(int64_t t) {
    switch (t) {
        case 5120: case 5121: return 1;
        case 5122: case 5123: return 2;
        case 5125: case 5126: return 4;
        default: return 0;
    }
}
int type_count(const std::string& t) {
    if (t == "SCALAR") return 1;
    if (t == "VEC2") return 2;
    if (t == "VEC3") return 3;
    if (t == "VEC4") return 4;
    if (t == "MAT2") return 4;
    if (t == "MAT3") return 9;
    if (t == "MAT4") return 16;
    return 0;
}

// One component as a double: floats as stored, integers normalized or not.
double read_comp(const uint8_t* p, int64_t type, bool normalized) {
    switch (type) {
        case 5126: {
            float f;
            std::memcpy(&f, p, 4);
            return f;
        }
        case 5121: return normalized ? (double)((float)p[0] / 255.0f) : (double)p[0];
        case 5123: {
            uint16_t v;
            std::memcpy(&v, p, 2);
            return normalized ? (double)((float)v / 65535.0f) : (double)v;
        }
        case 5125: {
            uint32_t v;
            std::memcpy(&v, p, 4);
            return (double)v;
        }
        case 5120: {
            const int8_t v = (int8_t)p[0];
            return normalized ? (double)std::fmax((float)v / 127.0f, -1.0f) : (double)v;
        }
        case 5122: {
            int16_t v;
            std::memcpy(&v, p, 2);
            return normalized ? (double)std::fmax((float)v / 32767.0f, -1.0f) : (double)v;
        }
        default: return 0.0;
    }
}

// Reads accessor `idx` as count x ncomp doubles (sparse substitution applied).
// force_norm: integer components are normalized whatever the accessor's
// `normalized` flag says (the reader's into_f32 for texture coordinates).
bool read_accessor(const Doc& d, int64_t idx, int want_comps, std::vector<double>& out, int64_t& comp_type,
                   std::string& err, bool force_norm = false) {
    const Value* acc = json::get(&d.root, "accessors");
    const Value* a = acc ? acc->at((size_t)idx) : nullptr;
    if (!a) {
        err = "accessor index out of range";
        return false;
    }
    comp_type = json::integer(a->get("componentType"), 0);
    const int64_t count = json::integer(a->get("count"), -1);
    const int nc = type_count(json::string(a->get("type")));
    const bool normalized =
        force_norm || (a->get("normalized") && a->get("normalized")->kind == Value::Bool && a->get("normalized")->b);
    const size_t cs = comp_size(comp_type);
    if (count < 0 || nc == 0 || cs == 0 || (want_comps && nc != want_comps)) {
        err = "unsupported accessor layout";
        return false;
    }
    // An accessor with a bufferView reads every element from the document's
    // buffers, so it cannot hold more elements than they have bytes. One
    // without a bufferView starts as zeros (glTF 2.0, 3.6.2) and may take
    // sparse substitutions: its count is capped by a fixed element limit.
    constexpr int64_t kMaxZeroElements = int64_t(1) << 24;
    size_t total_bytes = 0;
    for (const std::vector<uint8_t>& b : d.buffers) total_bytes += b.size();
    if (a->get("bufferView") ? (uint64_t)count > (uint64_t)total_bytes : count > kMaxZeroElements) {
        err = a->get("bufferView") ? "accessor count beyond the document's buffers"
                                   : "accessor without a bufferView has more than 2^24 elements";
        return false;
    }
    out.assign((size_t)count * nc, 0.0);
    auto read_view = [&](int64_t view_idx, size_t byte_off, size_t n, int ncomp, int64_t ctype, bool norm,
                         const std::function<void(size_t, int, double)>& put) -> bool {
        const Value* views = json::get(&d.root, "bufferViews");
        const Value* v = views ? views->at((size_t)view_idx) : nullptr;
        if (!v) {
            err = "bufferView index out of range";
            return false;
        }
        const int64_t bi = json::integer(v->get("buffer"), -1);
        if (bi < 0 || (size_t)bi >= d.buffers.size()) {
            err = "buffer index out of range";
            return false;
        }
        const std::vector<uint8_t>& buf = d.buffers[(size_t)bi];
        const int64_t voff_i = json::integer(v->get("byteOffset"), 0);
        const int64_t vlen_i = json::integer(v->get("byteLength"), 0);
        const int64_t stride_i = json::integer(v->get("byteStride"), 0);
        const size_t elem = comp_size(ctype) * (size_t)ncomp;
        // Every term checked against the buffer before it is combined, so no
        // sum or product below can wrap.
        if (elem == 0 || voff_i < 0 || vlen_i < 0 || stride_i < 0 || (uint64_t)voff_i > buf.size() ||
            (uint64_t)vlen_i > buf.size() - (size_t)voff_i || (uint64_t)stride_i > buf.size()) {
            err = "accessor reads past its buffer";
            return false;
        }
        const size_t voff = (size_t)voff_i, vlen = (size_t)vlen_i;
        const size_t stride = stride_i ? (size_t)stride_i : elem;
        if (n && (byte_off > vlen || elem > vlen - byte_off ||
                  (n - 1 > 0 && (n - 1) > (vlen - byte_off - elem) / stride))) {
            err = "accessor reads past its buffer";
            return false;
        }
        const uint8_t* base = buf.data() + voff + byte_off;
        for (size_t i = 0; i < n; ++i)
            for (int c = 0; c < ncomp; ++c)
                put(i, c, read_comp(base + i * stride + (size_t)c * comp_size(ctype), ctype, norm));
        return true;
    };
    if (a->get("bufferView")) {
        if (!read_view(json::integer(a->get("bufferView"), -1), (size_t)json::integer(a->get("byteOffset"), 0),
                       (size_t)count, nc, comp_type, normalized, [&](size_t i, int c, double x) { out[i * nc + c] = x; }))
            return false;
    }
    if (const Value* sp = a->get("sparse")) {
        const int64_t sc = json::integer(sp->get("count"), 0);
        const Value* si = sp->get("indices");
        const Value* sv = sp->get("values");
        if (!si || !sv || sc < 0 || sc > count) {
            err = "bad sparse accessor";
            return false;
        }
        std::vector<uint32_t> where((size_t)sc);
        const int64_t itype = json::integer(si->get("componentType"), 0);
        if (!read_view(json::integer(si->get("bufferView"), -1), (size_t)json::integer(si->get("byteOffset"), 0),
                       (size_t)sc, 1, itype, false, [&](size_t i, int, double x) { where[i] = (uint32_t)x; }))
            return false;
        std::vector<double> vals((size_t)sc * nc);
        if (!read_view(json::integer(sv->get("bufferView"), -1), (size_t)json::integer(sv->get("byteOffset"), 0),
                       (size_t)sc, nc, comp_type, normalized, [&](size_t i, int c, double x) { vals[i * nc + c] = x; }))
            return false;
        for (size_t i = 0; i < (size_t)sc; ++i) {
            if (where[i] >= (uint32_t)count) {
                err = "sparse index out of range";
                return false;
            }
            for (int c = 0; c < nc; ++c) out[(size_t)where[i] * nc + c] = vals[i * nc + c];
        }
    }
    return true;
}

// --- buffers ---------------------------------------------------------------

bool load_buffers(Doc& d, const std::vector<uint8_t>* glb_bin, std::string& err) {
    const Value* bufs = json::get(&d.root, "buffers");
    const size_t n = bufs ? bufs->size() : 0;
    d.buffers.resize(n);
    for (size_t i = 0; i < n; ++i) {
        const Value* b = bufs->at(i);
        const Value* uri = b ? b->get("uri") : nullptr;
        if (!uri) {
            if (!glb_bin) {
                err = "buffer without uri outside a .glb file";
                return false;
            }
            d.buffers[i] = *glb_bin;
        } else {
            const std::string u = json::string(uri);
            if (u.rfind("data:", 0) == 0) {
                const size_t comma = u.find(',');
                if (comma == std::string::npos || u.find(";base64") == std::string::npos ||
                    !base64_decode(u, comma + 1, d.buffers[i])) {
                    err = "bad data: URI in buffer " + std::to_string(i);
                    return false;
                }
            } else if (!read_file(d.base_dir + "/" + percent_decode(u), d.buffers[i], err)) {
                return false;
            }
        }
        const size_t want = (size_t)json::integer(b ? b->get("byteLength") : nullptr, 0);
        if (d.buffers[i].size() < want) {
            err = "buffer " + std::to_string(i) + " shorter than its byteLength";
            return false;
        }
    }
    return true;
}

// --- textures -----------------------------------------------------------------

struct LoadedImage {
    uint32_t w = 0, h = 0;
    std::vector<uint32_t> texels;  // R in MSB (rgba8_pack_u8, src/util.rs:98-100)
};

bool load_image_file(const std::string& path, LoadedImage& img, std::string& err) {
    std::vector<uint8_t> bytes, rgba;
    if (!read_file(path, bytes, err)) return false;
    if (!decode_image(bytes.data(), bytes.size(), img.w, img.h, rgba, err)) {
        err = "'" + path + "': " + err;
        return false;
    }
    img.texels.resize((size_t)img.w * img.h);
    for (size_t i = 0; i < img.texels.size(); ++i)
        img.texels[i] = (uint32_t)rgba[4 * i] << 24 | (uint32_t)rgba[4 * i + 1] << 16 |
                        (uint32_t)rgba[4 * i + 2] << 8 | rgba[4 * i + 3];
    return true;
}

uint32_t wrap_mode(int64_t gl) {
    switch (gl) {
        case 33071: return SWR_WRAP_CLAMP_TO_EDGE;
        case 33648: return SWR_WRAP_MIRRORED_REPEAT;
        default: return SWR_WRAP_REPEAT;
    }
}

struct Builder {
    Doc& d;
    std::vector<LoadedImage> images;
    std::vector<swr_texture_desc> textures;
    std::map<std::string, int32_t> by_uri;  // TextureCache: keyed by URI, first type wins

    // get_texture_and_sampler (src/scene.rs:590-653): URI images only.
    bool texref(const Value* info, uint32_t type, swr_texref& out, std::string& err) {
        out = {-1, SWR_WRAP_REPEAT, SWR_WRAP_REPEAT, 0};
        if (!info) return true;
        const Value* texs = json::get(&d.root, "textures");
        const Value* t = texs ? texs->at((size_t)json::integer(info->get("index"), -1)) : nullptr;
        if (!t) {
            err = "texture index out of range";
            return false;
        }
        const Value* imgs = json::get(&d.root, "images");
        const Value* img = imgs ? imgs->at((size_t)json::integer(t->get("source"), -1)) : nullptr;
        if (!img) return true;  // no source image: no texture
        const Value* uri = img->get("uri");
        if (!uri) return true;  // bufferView images are not loaded (src/scene.rs:652)
        const std::string u = json::string(uri);
        auto it = by_uri.find(u);
        int32_t ti;
        if (it != by_uri.end()) {
            ti = it->second;
        } else {
            const bool absolute = u.rfind("http://", 0) == 0 || u.rfind("https://", 0) == 0 || u.rfind("file://", 0) == 0;
            const std::string path = absolute ? u : d.base_dir + "/" + u;
            LoadedImage li;
            if (!load_image_file(path, li, err)) {
                err = "Failed to load texture '" + u + "': " + err;
                return false;
            }
            images.push_back(std::move(li));
            textures.push_back({images.back().w, images.back().h, type, 0, nullptr});
            ti = (int32_t)textures.size() - 1;
            by_uri[u] = ti;
        }
        out.texture = ti;
        if (t->get("sampler")) {
            const Value* samplers = json::get(&d.root, "samplers");
            const Value* s = samplers ? samplers->at((size_t)json::integer(t->get("sampler"), -1)) : nullptr;
            if (!s) {
                err = "sampler index out of range";
                return false;
            }
            out.wrap_s = wrap_mode(json::integer(s->get("wrapS"), 10497));
            out.wrap_t = wrap_mode(json::integer(s->get("wrapT"), 10497));
        }
        return true;
    }
};

}  // namespace
}  // namespace swr

using namespace swr;

extern "C" swr_status swr_scene_load_gltf(const char* path, const swr_gltf_opts* opts, swr_scene** out) {
    if (!path || !out) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    *out = nullptr;
    swr_gltf_opts o{};
    if (opts) o = *opts;
    std::string err;
    auto fail = [&](swr_status st, const std::string& m) {
        set_last_error(m.c_str());
        return st;
    };
    if (!o.cubemap_faces && !o.cubemap_path)
        return fail(SWR_INVALID_ARG, "a cubemap (faces or cross image path) is required");
    if (o.cubemap_faces && o.cubemap_face_size == 0) return fail(SWR_INVALID_ARG, "cubemap_face_size is 0");
    try {
        Doc d;
        const std::string p(path);
        const size_t slash = p.find_last_of('/');
        d.base_dir = slash == std::string::npos ? "." : p.substr(0, slash);
        if (d.base_dir.empty()) d.base_dir = "/";
        std::vector<uint8_t> file, bin;
        if (!read_file(p, file, err)) return fail(SWR_IO_ERROR, "Failed to load GLTF file: " + err);
        const char* json_text = reinterpret_cast<const char*>(file.data());
        size_t json_len = file.size();
        bool is_glb = false;
        if (file.size() >= 12 && std::memcmp(file.data(), "glTF", 4) == 0) {
            // GLB: 12-byte header, JSON chunk, optional BIN chunk.
            is_glb = true;
            size_t pos = 12;
            json_len = 0;
            while (pos + 8 <= file.size()) {
                uint32_t clen, ctype;
                std::memcpy(&clen, &file[pos], 4);
                std::memcpy(&ctype, &file[pos + 4], 4);
                if (pos + 8 + (size_t)clen > file.size())
                    return fail(SWR_IO_ERROR, "Failed to load GLTF file: truncated GLB chunk");
                if (ctype == 0x4E4F534Au && json_len == 0) {  // "JSON"
                    json_text = reinterpret_cast<const char*>(&file[pos + 8]);
                    json_len = clen;
                } else if (ctype == 0x004E4942u && bin.empty()) {  // "BIN\0"
                    bin.assign(file.begin() + (long)pos + 8, file.begin() + (long)(pos + 8 + clen));
                }
                pos += 8 + (size_t)clen;
            }
            if (json_len == 0) return fail(SWR_IO_ERROR, "Failed to load GLTF file: GLB without a JSON chunk");
        }
        json::Parser jp(json_text, json_len);
        if (!jp.parse(d.root, err)) return fail(SWR_IO_ERROR, "Failed to load GLTF file: " + err);
        if (d.root.kind != Value::Object) return fail(SWR_IO_ERROR, "Failed to load GLTF file: not a JSON object");
        if (!load_buffers(d, is_glb ? &bin : nullptr, err)) return fail(SWR_IO_ERROR, "Failed to load GLTF file: " + err);
        const Value* scenes = d.root.get("scenes");
        if (!scenes || scenes->size() == 0) return fail(SWR_BAD_SCENE, "No scenes found in GLTF file");

        Builder B{d};
        // Materials (Material::from_gltf); a document without materials gets
        // the glTF default material as material 0.
        std::vector<swr_material_desc> mats;
        const Value* jm = d.root.get("materials");
        for (size_t i = 0; i < (jm ? jm->size() : 0); ++i) {
            const Value* m = jm->at(i);
            swr_material_desc md{};
            const Value* pbr = m->get("pbrMetallicRoughness");
            const Value* bcf = json::get(pbr, "baseColorFactor");
            for (int k = 0; k < 4; ++k) md.base_color_factor[k] = (float)json::num(bcf ? bcf->at((size_t)k) : nullptr, 1.0);
            md.metallic_factor = (float)json::num(json::get(pbr, "metallicFactor"), 1.0);
            md.roughness_factor = (float)json::num(json::get(pbr, "roughnessFactor"), 1.0);
            const Value* ef = m->get("emissiveFactor");
            for (int k = 0; k < 3; ++k) md.emissive_factor[k] = (float)json::num(ef ? ef->at((size_t)k) : nullptr, 0.0);
            const Value* occ = m->get("occlusionTexture");
            md.occlusion_strength = (float)json::num(json::get(occ, "strength"), 1.0);
            md.alpha_cutoff = (float)json::num(m->get("alphaCutoff"), 0.5);
            md.alpha_mask = json::string(m->get("alphaMode"), "OPAQUE") == "MASK" ? 1u : 0u;
            const Value* tr = json::get(json::get(m, "extensions"), "KHR_materials_transmission");
            md.has_transmission = tr ? 1u : 0u;
            md.transmission = (float)json::num(json::get(tr, "transmissionFactor"), 0.0);
            // Texture lookups in the reference's field order (the first use of
            // an image decides its texture type).
            if (!B.texref(json::get(pbr, "baseColorTexture"), SWR_TEX_SRGB, md.base_color, err) ||
                !B.texref(json::get(pbr, "metallicRoughnessTexture"), SWR_TEX_METALLIC_ROUGHNESS,
                          md.metallic_roughness, err) ||
                !B.texref(m->get("normalTexture"), SWR_TEX_NORMAL, md.normal, err) ||
                !B.texref(m->get("emissiveTexture"), SWR_TEX_SRGB, md.emissive, err) ||
                !B.texref(occ, SWR_TEX_LINEAR, md.occlusion, err) ||
                !B.texref(json::get(tr, "transmissionTexture"), SWR_TEX_LINEAR, md.transmission_texture, err))
                return fail(SWR_IO_ERROR, err);
            mats.push_back(md);
        }
        if (mats.empty()) {
            swr_material_desc md{};
            for (float& c : md.base_color_factor) c = 1.0f;
            md.metallic_factor = md.roughness_factor = 1.0f;
            md.occlusion_strength = 1.0f;
            md.alpha_cutoff = 0.5f;
            md.base_color = md.metallic_roughness = md.normal = md.emissive = md.occlusion = md.transmission_texture =
                swr_texref{-1, 0, 0, 0};
            mats.push_back(md);
        }
        for (size_t i = 0; i < B.textures.size(); ++i) B.textures[i].rgba8 = B.images[i].texels.data();

        // Meshes (Mesh::from_gltf / Primitive::from_gltf).
        struct PrimData {
            std::vector<float> pos, nrm, tan, uv;
            std::vector<uint32_t> idx;
        };
        std::vector<std::vector<PrimData>> pdata;
        std::vector<std::vector<swr_primitive_desc>> pdesc;
        std::vector<swr_mesh_desc> meshes;
        const Value* jms = d.root.get("meshes");
        const size_t nmesh = jms ? jms->size() : 0;
        pdata.resize(nmesh);
        pdesc.resize(nmesh);
        for (size_t mi = 0; mi < nmesh; ++mi) {
            const Value* prims = jms->at(mi)->get("primitives");
            const size_t np = prims ? prims->size() : 0;
            pdata[mi].resize(np);
            pdesc[mi].resize(np);
            for (size_t k = 0; k < np; ++k) {
                const Value* pr = prims->at(k);
                const Value* at = pr->get("attributes");
                PrimData& P = pdata[mi][k];
                std::vector<double> tmp;
                int64_t ct;
                if (!json::get(at, "POSITION"))
                    return fail(SWR_BAD_SCENE, "Missing data: No positions in primitive");
                if (!read_accessor(d, json::integer(json::get(at, "POSITION"), -1), 3, tmp, ct, err) || ct != 5126)
                    return fail(SWR_BAD_SCENE, "POSITION: " + (err.empty() ? std::string("must be float") : err));
                P.pos.assign(tmp.begin(), tmp.end());
                const size_t nv = P.pos.size() / 3;
                if (!pr->get("indices")) return fail(SWR_BAD_SCENE, "Missing data: No indices in primitive");
                if (!read_accessor(d, json::integer(pr->get("indices"), -1), 1, tmp, ct, err) ||
                    !(ct == 5121 || ct == 5123 || ct == 5125))
                    return fail(SWR_BAD_SCENE, "indices: " + (err.empty() ? std::string("bad component type") : err));
                P.idx.resize(tmp.size() - tmp.size() % 3);  // triangles, indices.len() / 3
                for (size_t i = 0; i < P.idx.size(); ++i) {
                    P.idx[i] = (uint32_t)tmp[i];
                    if (P.idx[i] >= nv) return fail(SWR_BAD_SCENE, "index out of range in primitive");
                }
                if (json::get(at, "TEXCOORD_0")) {
                    if (!read_accessor(d, json::integer(json::get(at, "TEXCOORD_0"), -1), 2, tmp, ct, err, true) ||
                        !(ct == 5126 || ct == 5121 || ct == 5123) || tmp.size() != nv * 2)
                        return fail(SWR_BAD_SCENE, "TEXCOORD_0: " + (err.empty() ? std::string("bad layout") : err));
                    P.uv.assign(tmp.begin(), tmp.end());
                }
                if (json::get(at, "NORMAL")) {
                    if (!read_accessor(d, json::integer(json::get(at, "NORMAL"), -1), 3, tmp, ct, err) || ct != 5126 ||
                        tmp.size() != nv * 3)
                        return fail(SWR_BAD_SCENE, "NORMAL: " + (err.empty() ? std::string("bad layout") : err));
                    P.nrm.assign(tmp.begin(), tmp.end());
                }
                if (json::get(at, "TANGENT")) {
                    if (!read_accessor(d, json::integer(json::get(at, "TANGENT"), -1), 4, tmp, ct, err) || ct != 5126 ||
                        tmp.size() != nv * 4)
                        return fail(SWR_BAD_SCENE, "TANGENT: " + (err.empty() ? std::string("bad layout") : err));
                    P.tan.assign(tmp.begin(), tmp.end());
                }
                swr_primitive_desc& D = pdesc[mi][k];
                D = swr_primitive_desc{};
                D.vertex_count = (uint32_t)nv;
                D.index_count = (uint32_t)P.idx.size();
                D.positions = P.pos.data();
                D.normals = P.nrm.empty() ? nullptr : P.nrm.data();
                D.tangents = P.tan.empty() ? nullptr : P.tan.data();
                D.texcoords = P.uv.empty() ? nullptr : P.uv.data();
                D.indices = P.idx.data();
                const int64_t mat = json::integer(pr->get("material"), 0);  // unwrap_or(0)
                if (mat < 0 || (size_t)mat >= mats.size()) return fail(SWR_BAD_SCENE, "material index out of range");
                D.material = (int32_t)mat;
            }
            meshes.push_back({(uint32_t)np, 0, pdesc[mi].data()});
        }

        // Nodes: every document node, world = parent * local from the roots
        // (compute_final_transform_recursive, src/scene.rs:356-382).
        const Value* jn = d.root.get("nodes");
        const size_t nn = jn ? jn->size() : 0;
        std::vector<swr_node_desc> nodes(nn);
        std::vector<M4> local(nn);
        std::set<int64_t> children;
        for (size_t i = 0; i < nn; ++i) {
            const Value* n = jn->at(i);
            M4 m;
            if (const Value* mat = n->get("matrix")) {
                float a[16];
                for (int k = 0; k < 16; ++k) a[k] = (float)json::num(mat->at((size_t)k), (k % 5 == 0) ? 1.0 : 0.0);
                m = from_array(a);
            } else {
                const Value* t = n->get("translation");
                const Value* r = n->get("rotation");
                const Value* s = n->get("scale");
                const V3 tv = {(float)json::num(t ? t->at(0) : nullptr, 0.0), (float)json::num(t ? t->at(1) : nullptr, 0.0),
                               (float)json::num(t ? t->at(2) : nullptr, 0.0)};
                const Quat q = {(float)json::num(r ? r->at(0) : nullptr, 0.0), (float)json::num(r ? r->at(1) : nullptr, 0.0),
                                (float)json::num(r ? r->at(2) : nullptr, 0.0), (float)json::num(r ? r->at(3) : nullptr, 1.0)};
                const V3 sv = {(float)json::num(s ? s->at(0) : nullptr, 1.0), (float)json::num(s ? s->at(1) : nullptr, 1.0),
                               (float)json::num(s ? s->at(2) : nullptr, 1.0)};
                m = mulmm(mulmm(mat_translation(tv), mat_from_quat(q)), mat_scale(sv));
            }
            local[i] = m;
            to_array(m, nodes[i].local);
            to_array(m, nodes[i].world);
            const int64_t mesh = json::integer(n->get("mesh"), -1);
            if (mesh >= (int64_t)nmesh) return fail(SWR_BAD_SCENE, "node mesh index out of range");
            nodes[i].mesh = (int32_t)mesh;
            if (const Value* ch = n->get("children"))
                for (size_t k = 0; k < ch->size(); ++k) children.insert(json::integer(ch->at(k), -1));
        }
        std::function<void(size_t, const M4&, int)> walk = [&](size_t i, const M4& parent, int depth) {
            if (depth > 1024) return;
            const M4 w = mulmm(parent, local[i]);
            to_array(w, nodes[i].world);
            if (const Value* ch = jn->at(i)->get("children"))
                for (size_t k = 0; k < ch->size(); ++k) {
                    const int64_t c = json::integer(ch->at(k), -1);
                    if (c >= 0 && (size_t)c < nn) walk((size_t)c, w, depth + 1);
                }
        };
        for (size_t i = 0; i < nn; ++i)
            if (!children.count((int64_t)i)) walk(i, identity4(), 0);

        // Environment cubemap.
        std::vector<uint32_t> faces;
        const uint32_t* face_ptr = o.cubemap_faces;
        uint32_t face = o.cubemap_face_size;
        if (!face_ptr) {
            LoadedImage cross;
            if (!load_image_file(o.cubemap_path, cross, err)) return fail(SWR_IO_ERROR, "cubemap: " + err);
            // Cross layout (src/texture.rs:922-945): +Y on row 0; -X +Z +X -Z on row 1; -Y on row 2.
            const uint32_t fw = cross.w / 4, fh = cross.h / 3;
            if (fw == 0 || fw != fh) return fail(SWR_BAD_SCENE, "cubemap cross must hold square faces");
            static const uint32_t pos[6][2] = {{2, 1}, {0, 1}, {1, 0}, {1, 2}, {1, 1}, {3, 1}};
            faces.resize((size_t)6 * fw * fh);
            size_t k = 0;
            for (const auto& fp : pos)
                for (uint32_t y = 0; y < fh; ++y)
                    for (uint32_t x = 0; x < fw; ++x) faces[k++] = cross.texels[(size_t)(fp[1] * fh + y) * cross.w + fp[0] * fw + x];
            face_ptr = faces.data();
            face = fw;
        }

        swr_scene_desc sd{};
        sd.mesh_count = (uint32_t)meshes.size();
        sd.node_count = (uint32_t)nodes.size();
        sd.material_count = (uint32_t)mats.size();
        sd.texture_count = (uint32_t)B.textures.size();
        sd.meshes = meshes.data();
        sd.nodes = nodes.data();
        sd.materials = mats.data();
        sd.textures = B.textures.data();
        sd.cubemap_face_size = face;
        sd.cubemap_faces = face_ptr;
        sd.voxel_grid_size = o.voxel_grid_size ? o.voxel_grid_size : 128u;
        sd.specular_samples = o.specular_samples ? o.specular_samples : 64u;
        sd.brdf_lut_size = o.brdf_lut_size ? o.brdf_lut_size : 128u;
        sd.gi_sh_scale = 0.25f;
        sd.sky_visibility = 1.0f;
        sd.host_threads = o.host_threads;
        sd.flags = o.flags;
        sd.gi_cache_path = o.gi_cache_path;
        sd.ggx_cache_path = o.ggx_cache_path;
        return swr_scene_create(&sd, out);
    } catch (const std::bad_alloc&) {
        return fail(SWR_NO_MEMORY, "out of host memory");
    } catch (...) {
        return fail(SWR_BAD_SCENE, "glTF load failed");
    }
}
