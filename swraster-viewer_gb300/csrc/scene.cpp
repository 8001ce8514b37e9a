// Scene admission: the reference's load path (Scene::from_gltf,
// src/scene.rs:145-354, and the voxel/IBL precompute driven by load_scene,
// src/main.rs:100-291) restated in C++, then one upload into HBM.
//
// All floating point follows the reference's operation order and is compiled
// with -ffp-contract=off. Transcendentals (powf, sinf, cosf, sqrtf) come from
// the host libm, the same functions a Rust build links.
#include "scene.h"

#include "caches.h"
#include "ibl.h"
#include "precompute.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>

namespace swr {

namespace {

constexpr float kPi = 3.14159265358979f;

unsigned hw_threads(uint32_t req) {
    if (req) return req;
    unsigned n = std::thread::hardware_concurrency();
    return n ? n : 1u;
}

template <typename F>
void parallel_for(size_t n, unsigned threads, F f) {
    if (threads <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::atomic<size_t> next{0};
    const size_t grain = std::max<size_t>(1, n / (threads * 16));
    auto worker = [&]() {
        for (;;) {
            size_t b = next.fetch_add(grain);
            if (b >= n) break;
            size_t e = std::min(n, b + grain);
            for (size_t i = b; i < e; ++i) f(i);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < threads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
}

// --- RGBA8 / colour helpers (src/util.rs:49-100) ------------------------
inline uint32_t f2u_sat(float x) {
    if (!(x > 0.0f)) return 0u;  // NaN and negatives
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}
inline V4 unpack4(uint32_t c) {
    return {(float)((c >> 24) & 0xFFu) / 255.0f, (float)((c >> 16) & 0xFFu) / 255.0f,
            (float)((c >> 8) & 0xFFu) / 255.0f, (float)(c & 0xFFu) / 255.0f};
}
inline uint32_t pack4(V4 c) {
    return (f2u_sat(c.x * 255.0f) << 24) | (f2u_sat(c.y * 255.0f) << 16) | (f2u_sat(c.z * 255.0f) << 8) |
           f2u_sat(c.w * 255.0f);
}
inline float srgb_to_linear_scalar(float s) {
    if (s <= 0.04045f) return s / 12.92f;
    return std::pow((s + 0.055f) / 1.055f, 2.4f);
}
inline float linear_to_srgb_scalar(float s) {
    if (s <= 0.0031308f) return s * 12.92f;
    return std::pow(s, 1.0f / 2.4f) * 1.055f - 0.055f;
}
inline uint32_t ilog2u(uint32_t v) { return 31u - (uint32_t)__builtin_clz(v); }

}  // namespace

// One texel of the next mip from its 2x2 parents (src/texture.rs:82-113).
uint32_t mip_texel(uint32_t type, uint32_t q00, uint32_t q10, uint32_t q01, uint32_t q11) {
    const V4 p00 = unpack4(q00), p10 = unpack4(q10), p01 = unpack4(q01), p11 = unpack4(q11);
    V4 avg;
    if (type == SWR_TEX_SRGB) {
        auto lin = [](V4 c) {
            return V4{srgb_to_linear_scalar(c.x), srgb_to_linear_scalar(c.y), srgb_to_linear_scalar(c.z), c.w};
        };
        const V4 l00 = lin(p00), l10 = lin(p10), l01 = lin(p01), l11 = lin(p11);
        V4 s = add4(add4(add4(l00, l10), l01), l11);
        s = {s.x / 4.0f, s.y / 4.0f, s.z / 4.0f, s.w / 4.0f};
        avg = {linear_to_srgb_scalar(s.x), linear_to_srgb_scalar(s.y), linear_to_srgb_scalar(s.z), s.w};
    } else if (type == SWR_TEX_METALLIC_ROUGHNESS) {
        const float r = (((p00.y * p00.y + p10.y * p10.y) + p01.y * p01.y) + p11.y * p11.y) / 4.0f;
        const float m = (((p00.z + p10.z) + p01.z) + p11.z) / 4.0f;
        avg = {p00.x, std::sqrt(r), m, p00.w};
    } else if (type == SWR_TEX_NORMAL) {
        auto n = [](V4 c) { return V4{c.x * 2.0f - 1.0f, c.y * 2.0f - 1.0f, c.z * 2.0f - 1.0f, c.w * 2.0f - 1.0f}; };
        V4 s = add4(add4(add4(n(p00), n(p10)), n(p01)), n(p11));
        s = {s.x / 4.0f, s.y / 4.0f, s.z / 4.0f, s.w / 4.0f};
        avg = {(s.x + 1.0f) / 2.0f, (s.y + 1.0f) / 2.0f, (s.z + 1.0f) / 2.0f, (s.w + 1.0f) / 2.0f};
    } else {
        V4 s = add4(add4(add4(p00, p10), p01), p11);
        avg = {s.x / 4.0f, s.y / 4.0f, s.z / 4.0f, s.w / 4.0f};
    }
    return pack4(avg);
}

float srgb_to_linear_host(float s) { return srgb_to_linear_scalar(s); }

void srgb_byte_thresholds(float out[255]) {
    auto byte = [](uint32_t bits) {
        float s;
        std::memcpy(&s, &bits, 4);
        return f2u_sat(linear_to_srgb_scalar(s) * 255.0f);
    };
    auto as_bits = [](float f) {
        uint32_t u;
        std::memcpy(&u, &f, 4);
        return u;
    };
    const uint32_t first = as_bits(0.0031308f) + 1u, last = as_bits(1.0f);
    for (uint32_t k = 1; k <= 255; ++k) {
        if (byte(last) < k) {
            out[k - 1] = INFINITY;
            continue;
        }
        uint32_t lo = first, hi = last;  // the first bits in [lo, hi] whose byte is >= k
        while (lo < hi) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (byte(mid) >= k) hi = mid;
            else lo = mid + 1;
        }
        std::memcpy(&out[k - 1], &lo, 4);
    }
}

void HTexture::mip_layout() {
    const uint32_t num_mips = 1u + ilog2u(std::max(width, height));
    const uint32_t array_size = type == SWR_TEX_CUBEMAP ? 6u : 1u;
    size_t size = data.size();
    for (uint32_t mip = 1; mip < num_mips; ++mip) {
        mip_offsets.push_back((uint32_t)size);
        const uint32_t mw = std::max(width >> mip, 1u), mh = std::max(height >> mip, 1u);
        array_stride.push_back(mw * mh);
        size += (size_t)mw * mh * array_size;
        mip_widths.push_back(mw);
        mip_heights.push_back(mh);
        mip_widths_f.push_back((float)mw);
        mip_heights_f.push_back((float)mh);
        max_mip += 1;
    }
}

// Texture::generate_mipmaps (src/texture.rs:45-128).
void HTexture::generate_mipmaps() {
    const uint32_t num_mips = 1u + ilog2u(std::max(width, height));
    const uint32_t array_size = type == SWR_TEX_CUBEMAP ? 6u : 1u;
    for (uint32_t mip = 1; mip < num_mips; ++mip) {
        mip_offsets.push_back((uint32_t)data.size());
        const uint32_t mw = std::max(width >> mip, 1u), mh = std::max(height >> mip, 1u);
        array_stride.push_back(mw * mh);
        const uint32_t prev_offset = mip_offsets[mip - 1];
        const uint32_t pw = mip_widths[mip - 1], ph = mip_heights[mip - 1];
        const uint32_t pstride = array_stride[mip - 1];
        for (uint32_t slice = 0; slice < array_size; ++slice) {
            const uint32_t so = prev_offset + slice * pstride;
            for (uint32_t y = 0; y < mh; ++y) {
                for (uint32_t x = 0; x < mw; ++x) {
                    const uint32_t x0 = x * 2, y0 = y * 2;
                    const uint32_t x1 = std::min(x0 + 1, pw - 1), y1 = std::min(y0 + 1, ph - 1);
                    data.push_back(mip_texel(type, data[so + y0 * pw + x0], data[so + y0 * pw + x1],
                                             data[so + y1 * pw + x0], data[so + y1 * pw + x1]));
                }
            }
        }
        mip_widths.push_back(mw);
        mip_heights.push_back(mh);
        mip_widths_f.push_back((float)mw);
        mip_heights_f.push_back((float)mh);
        max_mip += 1;
    }
}

swr_texture_view HTexture::view() const {
    swr_texture_view v{};
    v.width = width;
    v.height = height;
    v.type = type;
    v.mip_count = max_mip + 1;
    v.data = data.data();
    v.data_len = data.size();
    v.mip_offsets = mip_offsets.data();
    v.mip_widths = mip_widths.data();
    v.mip_heights = mip_heights.data();
    v.array_stride = array_stride.data();
    for (int i = 0; i < 4; ++i) v.width_height_vec[i] = whv[i];
    return v;
}

namespace {

HTexture make_texture(uint32_t w, uint32_t h, uint32_t type, const uint32_t* rgba, bool cubemap) {
    HTexture t;
    t.width = w;
    t.height = h;
    t.type = type;
    const size_t n = (size_t)w * h * (cubemap ? 6u : 1u);
    t.data.assign(rgba, rgba + n);
    t.mip_offsets = {0};
    t.mip_widths = {w};
    t.mip_heights = {h};
    t.mip_widths_f = {(float)w};
    t.mip_heights_f = {(float)h};
    t.array_stride = {cubemap ? w * h : 0u};
    t.whv[0] = (float)w;
    t.whv[1] = (float)w;
    t.whv[2] = (float)h;
    t.whv[3] = (float)h;
    return t;
}

// --- IBL precompute (src/texture.rs:135-420) ---------------------------
float radical_inverse_vdc(uint32_t bits) {
    bits = (bits << 16) | (bits >> 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    return (float)bits * 2.3283064e-10f;
}
inline void hammersley(uint32_t i, uint32_t n, float& x, float& y) {
    x = (float)i / (float)n;
    y = radical_inverse_vdc(i);
}
V3 importance_sample_ggx(float xi_x, float xi_y, V3 n, float roughness) {
    const float a = roughness * roughness;
    const float phi = (2.0f * kPi) * xi_x;
    const float cos_theta = std::sqrt((1.0f - xi_y) / (1.0f + (a * a - 1.0f) * xi_y));
    const float sin_theta = std::sqrt(std::fmax(1.0f - cos_theta * cos_theta, 0.0f));
    const V3 h = {std::cos(phi) * sin_theta, std::sin(phi) * sin_theta, cos_theta};
    const V3 up = std::fabs(n.z) < 0.999f ? V3{0, 0, 1} : V3{1, 0, 0};
    const V3 tangent = normalize3(cross3(n, up));
    const V3 bitangent = cross3(n, tangent);
    return normalize3(add(add(mul(tangent, h.x), mul(bitangent, h.y)), mul(n, h.z)));
}
inline float powi5(float x) {
    const float x2 = x * x;
    return x * (x2 * x2);
}
void integrate_brdf(float ndotv, float roughness, float& ra, float& rb) {
    const V3 v = {std::sqrt(std::fmax(1.0f - ndotv * ndotv, 0.0f)), 0.0f, ndotv};
    const V3 n = {0, 0, 1};
    const uint32_t sample_count = 128;
    float a = 0.0f, b = 0.0f;
    for (uint32_t i = 0; i < sample_count; ++i) {
        float xx, xy;
        hammersley(i, sample_count, xx, xy);
        const V3 h = importance_sample_ggx(xx, xy, n, roughness);
        const V3 l = normalize3(sub(mul(h, 2.0f * dot3(v, h)), v));
        const float ndotl = std::fmax(l.z, 0.0f);
        const float ndoth = std::fmax(h.z, 0.0f);
        const float vdoth = std::fmax(dot3(v, h), 0.0f);
        if (ndotl > 0.0f) {
            const float alpha = roughness * roughness;
            const float k = ((alpha + 1.0f) * (alpha + 1.0f)) * 0.125f;
            const float g_v = ndotv / (ndotv * (1.0f - k) + k);
            const float g_l = ndotl / (ndotl * (1.0f - k) + k);
            const float g_vis = std::fmax(((g_v * g_l) * vdoth) / (ndoth * std::fmax(ndotv, 1.0e-5f)), 0.0f);
            const float fc = powi5(1.0f - vdoth);
            a += (1.0f - fc) * g_vis;
            b += fc * g_vis;
        }
    }
    ra = a / (float)sample_count;
    rb = b / (float)sample_count;
}
HTexture generate_brdf_lut(uint32_t size, unsigned threads) {
    std::vector<uint32_t> data((size_t)size * size);
    const float size_f = (float)size;
    parallel_for(size, threads, [&](size_t y) {
        const float roughness = std::fmin(std::fmax(((float)y + 0.5f) / size_f, 0.0f), 1.0f);
        for (uint32_t x = 0; x < size; ++x) {
            const float ndotv = std::fmin(std::fmax(((float)x + 0.5f) / size_f, 0.0f), 1.0f);
            float ia, ib;
            integrate_brdf(std::fmax(ndotv, 1.0e-4f), std::fmax(roughness, 1.0e-4f), ia, ib);
            const V4 texel = {std::fmin(std::fmax(ia, 0.0f), 1.0f), std::fmin(std::fmax(ib, 0.0f), 1.0f), 0.0f, 1.0f};
            data[(size_t)y * size + x] = pack4(texel);
        }
    });
    HTexture t = make_texture(size, size, SWR_TEX_LINEAR, data.data(), false);
    t.generate_mipmaps();
    return t;
}
V3 face_uv_to_direction(uint32_t face, float u, float v) {
    V3 d;
    switch (face) {
        case 0: d = {1.0f, -v, -u}; break;
        case 1: d = {-1.0f, -v, u}; break;
        case 2: d = {u, 1.0f, v}; break;
        case 3: d = {u, -1.0f, -v}; break;
        case 4: d = {u, -v, 1.0f}; break;
        default: d = {-u, -v, -1.0f}; break;
    }
    return normalize3(d);
}
void direction_to_face_uv(V3 n, uint32_t& face, float& u, float& v) {
    const float ax = std::fabs(n.x), ay = std::fabs(n.y), az = std::fabs(n.z);
    if (ax >= ay && ax >= az) {
        if (n.x >= 0.0f) { face = 0; u = (-n.z / ax) * 0.5f + 0.5f; v = (-n.y / ax) * 0.5f + 0.5f; }
        else { face = 1; u = (n.z / ax) * 0.5f + 0.5f; v = (-n.y / ax) * 0.5f + 0.5f; }
    } else if (ay > ax && ay >= az) {
        if (n.y >= 0.0f) { face = 2; u = (n.x / ay) * 0.5f + 0.5f; v = (n.z / ay) * 0.5f + 0.5f; }
        else { face = 3; u = (n.x / ay) * 0.5f + 0.5f; v = (-n.z / ay) * 0.5f + 0.5f; }
    } else if (n.z >= 0.0f) {
        face = 4; u = (n.x / az) * 0.5f + 0.5f; v = (-n.y / az) * 0.5f + 0.5f;
    } else {
        face = 5; u = (-n.x / az) * 0.5f + 0.5f; v = (-n.y / az) * 0.5f + 0.5f;
    }
}
// sample_bilinear_rgb lane 0 with ClampToEdge (src/texture.rs:730-790).
V3 bilinear_slice(const HTexture& t, float u, float v, uint32_t slice) {
    const uint32_t wi = t.mip_widths[0];
    const float wf = t.mip_widths_f[0], hf = t.mip_heights_f[0];
    const uint32_t off = t.mip_offsets[0] + slice * t.array_stride[0];
    const float xf = u * wf - 0.5f, yf = v * hf - 0.5f;
    const float x0 = std::floor(xf), y0 = std::floor(yf);
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const float fx = xf - x0, fy = yf - y0;
    const float ofx = 1.0f - fx, ofy = 1.0f - fy;
    const uint32_t x0i = f2u_sat(std::fmin(x0, wf - 1.0f)), y0i = f2u_sat(std::fmin(y0, hf - 1.0f));
    const uint32_t x1i = f2u_sat(std::fmin(x1, wf - 1.0f)), y1i = f2u_sat(std::fmin(y1, hf - 1.0f));
    const V4 p00 = unpack4(t.data[off + y0i * wi + x0i]);
    const V4 p10 = unpack4(t.data[off + y0i * wi + x1i]);
    const V4 p01 = unpack4(t.data[off + y1i * wi + x0i]);
    const V4 p11 = unpack4(t.data[off + y1i * wi + x1i]);
    const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
    return {((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11,
            ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11,
            ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11};
}
// sample_cubemap_direction_linear (src/texture.rs:273-287).
V3 sample_dir_linear(const HTexture& cube, V3 dir) {
    uint32_t face;
    float u, v;
    direction_to_face_uv(dir, face, u, v);
    const V3 s = bilinear_slice(cube, std::fmin(std::fmax(u, 0.0f), 1.0f), std::fmin(std::fmax(v, 0.0f), 1.0f), face);
    return {srgb_to_linear_scalar(s.x), srgb_to_linear_scalar(s.y), srgb_to_linear_scalar(s.z)};
}
void compute_irradiance_sh4(const HTexture& cube, float out[4][3]) {
    V3 sh[4] = {};
    const float width = (float)cube.width, height = (float)cube.height;
    const float texel_omega = (2.0f / width) * (2.0f / height);
    for (uint32_t face = 0; face < 6; ++face) {
        for (uint32_t y = 0; y < cube.height; ++y) {
            const float v = (((float)y + 0.5f) / height) * 2.0f - 1.0f;
            for (uint32_t x = 0; x < cube.width; ++x) {
                const float u = (((float)x + 0.5f) / width) * 2.0f - 1.0f;
                const V3 dir = face_uv_to_direction(face, u, v);
                const float weight = texel_omega / std::pow((1.0f + u * u) + v * v, 1.5f);
                const V3 color = sample_dir_linear(cube, dir);
                const float basis[4] = {0.282095f, 0.488603f * dir.y, 0.488603f * dir.z, 0.488603f * dir.x};
                for (int i = 0; i < 4; ++i) sh[i] = add(sh[i], mul(color, basis[i] * weight));
            }
        }
    }
    sh[0] = mul(sh[0], kPi);
    for (int i = 1; i < 4; ++i) sh[i] = mul(sh[i], (2.0f * kPi) / 3.0f);
    sh[0] = mul(sh[0], 0.282095f);
    for (int i = 1; i < 4; ++i) sh[i] = mul(sh[i], 0.488603f);
    for (int i = 0; i < 4; ++i) {
        out[i][0] = sh[i].x;
        out[i][1] = sh[i].y;
        out[i][2] = sh[i].z;
    }
}
}  // namespace

// One texel of the GGX-prefiltered environment (the loop body of
// generate_prefiltered_specular_cubemap, src/texture.rs:357-393).
uint32_t prefilter_texel(const HTexture& cube, uint32_t mip, uint32_t max_mip, uint32_t face, uint32_t x, uint32_t y,
                         uint32_t sample_count, const float* xi_x, const float* xi_y) {
    const uint32_t bw = cube.width, bh = cube.height;
    const float roughness = max_mip > 0 ? (float)mip / (float)max_mip : 0.0f;
    const float v = (((float)y + 0.5f) / (float)bh) * 2.0f - 1.0f;
    const float u = (((float)x + 0.5f) / (float)bw) * 2.0f - 1.0f;
    const V3 r = face_uv_to_direction(face, u, v);
    V3 color;
    if (mip == 0) {
        color = sample_dir_linear(cube, r);
    } else {
        V3 accum = {0, 0, 0};
        float total = 0.0f;
        for (uint32_t i = 0; i < sample_count; ++i) {
            const V3 h = importance_sample_ggx(xi_x[i], xi_y[i], r, std::fmax(roughness, 0.045f));
            const V3 l = normalize3(sub(mul(h, 2.0f * dot3(r, h)), r));
            const float ndotl = std::fmax(dot3(r, l), 0.0f);
            if (ndotl > 0.0f) {
                accum = add(accum, mul(sample_dir_linear(cube, l), ndotl));
                total += ndotl;
            }
        }
        color = total > 0.0f ? V3{accum.x / total, accum.y / total, accum.z / total} : sample_dir_linear(cube, r);
    }
    return pack4({color.x, color.y, color.z, 1.0f});
}

void hammersley_table(uint32_t n, float* xi_x, float* xi_y, float* cos_phi, float* sin_phi) {
    for (uint32_t i = 0; i < n; ++i) {
        hammersley(i, n, xi_x[i], xi_y[i]);
        const float phi = (2.0f * kPi) * xi_x[i];
        if (cos_phi) cos_phi[i] = std::cos(phi);
        if (sin_phi) sin_phi[i] = std::sin(phi);
    }
}

// The prefiltered texture's layout: every mip at full face resolution, six
// faces each (src/texture.rs:335-356).
HTexture prefiltered_layout(uint32_t bw, uint32_t bh) {
    const uint32_t num_mips = 1u + ilog2u(std::max(bw, bh));
    HTexture t;
    t.width = bw;
    t.height = bh;
    t.type = SWR_TEX_LINEAR;
    const size_t face_texels = (size_t)bw * bh;
    t.data.resize(face_texels * 6 * num_mips);
    for (uint32_t mip = 0; mip < num_mips; ++mip) {
        t.mip_offsets.push_back((uint32_t)(face_texels * 6 * mip));
        t.mip_widths.push_back(bw);
        t.mip_heights.push_back(bh);
        t.mip_widths_f.push_back((float)bw);
        t.mip_heights_f.push_back((float)bh);
        t.array_stride.push_back(bw * bh);
    }
    t.max_mip = num_mips - 1;
    t.whv[0] = (float)bw;
    t.whv[1] = (float)bw;
    t.whv[2] = (float)bh;
    t.whv[3] = (float)bh;
    return t;
}

namespace {

HTexture generate_prefiltered_specular(const HTexture& cube, uint32_t sample_count, unsigned threads) {
    const uint32_t bw = cube.width, bh = cube.height;
    HTexture t = prefiltered_layout(bw, bh);
    const uint32_t num_mips = t.max_mip + 1;
    const size_t face_texels = (size_t)bw * bh;
    std::vector<float> xi_x(sample_count), xi_y(sample_count);
    hammersley_table(sample_count, xi_x.data(), xi_y.data(), nullptr, nullptr);
    const size_t rows = (size_t)num_mips * 6 * bh;
    parallel_for(rows, threads, [&](size_t row) {
        const uint32_t mip = (uint32_t)(row / (6 * bh));
        const uint32_t face = (uint32_t)((row / bh) % 6);
        const uint32_t y = (uint32_t)(row % bh);
        for (uint32_t x = 0; x < bw; ++x)
            t.data[t.mip_offsets[mip] + face * face_texels + (size_t)y * bw + x] =
                prefilter_texel(cube, mip, t.max_mip, face, x, y, sample_count, xi_x.data(), xi_y.data());
    });
    return t;
}

// --- Mesh processing (src/scene.rs:498-635) ----------------------------
void compute_smooth_normals(const std::vector<float>& pos4, const std::vector<uint32_t>& idx, std::vector<float>& nrm4) {
    const size_t nv = pos4.size() / 4;
    std::vector<V3> acc(nv, V3{0, 0, 0});
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const float* a = &pos4[4 * (size_t)idx[t]];
        const float* b = &pos4[4 * (size_t)idx[t + 1]];
        const float* c = &pos4[4 * (size_t)idx[t + 2]];
        const V3 e1 = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
        const V3 e2 = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const V3 f = cross3(e1, e2);
        for (int k = 0; k < 3; ++k) acc[idx[t + k]] = add(acc[idx[t + k]], f);
    }
    nrm4.assign(nv * 4, 0.0f);
    for (size_t i = 0; i < nv; ++i) {
        V3 n = acc[i];
        if (dot3(n, n) > 0.0f) n = normalize3(n); else n = {0, 0, 1};
        nrm4[4 * i] = n.x;
        nrm4[4 * i + 1] = n.y;
        nrm4[4 * i + 2] = n.z;
    }
}
// Vec3 (scalar glam) dot: sequential.
inline float dot3s(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline V3 normalize3s(V3 a) {
    const float r = 1.0f / std::sqrt(dot3s(a, a));
    return mul(a, r);
}
void compute_tangents(const std::vector<float>& pos4, const std::vector<float>& uv2, const std::vector<float>& nrm4,
                      const std::vector<uint32_t>& idx, std::vector<float>& tan4) {
    const size_t nv = pos4.size() / 4;
    std::vector<V3> tacc(nv, V3{0, 0, 0}), bacc(nv, V3{0, 0, 0});
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const uint32_t i0 = idx[t], i1 = idx[t + 1], i2 = idx[t + 2];
        const V3 p0 = {pos4[4 * i0], pos4[4 * i0 + 1], pos4[4 * i0 + 2]};
        const V3 p1 = {pos4[4 * i1], pos4[4 * i1 + 1], pos4[4 * i1 + 2]};
        const V3 p2 = {pos4[4 * i2], pos4[4 * i2 + 1], pos4[4 * i2 + 2]};
        const float u0 = uv2[2 * i0], v0 = uv2[2 * i0 + 1];
        const float u1 = uv2[2 * i1], v1 = uv2[2 * i1 + 1];
        const float u2 = uv2[2 * i2], v2 = uv2[2 * i2 + 1];
        const V3 e1 = sub(p1, p0), e2 = sub(p2, p0);
        const float d1x = u1 - u0, d1y = v1 - v0, d2x = u2 - u0, d2y = v2 - v0;
        const float det = d1x * d2y - d2x * d1y;
        if (std::fabs(det) < 1e-6f) continue;
        const V3 tn = sub(mul(e1, d2y), mul(e2, d1y));
        const V3 bn = sub(mul(e2, d1x), mul(e1, d2x));
        const V3 tangent = {tn.x / det, tn.y / det, tn.z / det};
        const V3 bitangent = {bn.x / det, bn.y / det, bn.z / det};
        tacc[i0] = add(tacc[i0], tangent); tacc[i1] = add(tacc[i1], tangent); tacc[i2] = add(tacc[i2], tangent);
        bacc[i0] = add(bacc[i0], bitangent); bacc[i1] = add(bacc[i1], bitangent); bacc[i2] = add(bacc[i2], bitangent);
    }
    tan4.assign(nv * 4, 0.0f);
    for (size_t i = 0; i < nv; ++i) {
        const V3 n = {nrm4[4 * i], nrm4[4 * i + 1], nrm4[4 * i + 2]};
        const V3 t = tacc[i];
        float* o = &tan4[4 * i];
        if (dot3s(t, t) < 1e-6f) {
            const V3 helper = std::fabs(n.x) > 0.9f ? V3{0, 1, 0} : V3{1, 0, 0};
            const V3 tg = normalize3s(cross3(n, helper));
            o[0] = tg.x; o[1] = tg.y; o[2] = tg.z; o[3] = 1.0f;
            continue;
        }
        const V3 tg = normalize3s(sub(t, mul(n, dot3s(n, t))));
        const V3 cnt = cross3(n, tg);
        const float hand = dot3s(cnt, bacc[i]) < 0.0f ? -1.0f : 1.0f;
        o[0] = tg.x; o[1] = tg.y; o[2] = tg.z; o[3] = hand;
    }
}
void compute_bounding_sphere(const std::vector<float>& pos4, float out[4]) {
    V3 mn = {INFINITY, INFINITY, INFINITY}, mx = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i + 3 < pos4.size() + 1 && i < pos4.size(); i += 4) {
        const V3 p = {pos4[i], pos4[i + 1], pos4[i + 2]};
        mn = v3min(mn, p);
        mx = v3max(mx, p);
    }
    const V3 c = mul(add(mn, mx), 0.5f);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    out[3] = length3(sub(mx, mn)) / 2.0f;
}

// Mat4 * &BoundingSphere (src/scene.rs:53-63).
void transform_sphere(const M4& m, const float in[4], float out[4]) {
    const float max_scale = ((length4(m.c[0]) + length4(m.c[1])) + length4(m.c[2])) / 3.0f;
    const V3 c = transform_point3(m, {in[0], in[1], in[2]});
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    out[3] = in[3] * max_scale;
}

// --- Ray tracer for sun visibility (src/raytracer.rs, src/gi.rs:151-314) ---
struct RtTri {
    V3 p0, p1, p2, n;
    uint32_t material;
};
struct BvhNode {
    float mn[3], mx[3];
    uint32_t left;   // child index, or first triangle for leaves
    uint32_t count;  // 0 for inner nodes
};
struct Bvh {
    std::vector<BvhNode> nodes;
    std::vector<uint32_t> order;
};
void bvh_build(const std::vector<RtTri>& tris, Bvh& b) {
    const size_t n = tris.size();
    b.order.resize(n);
    std::vector<float> cen(n * 3), bmn(n * 3), bmx(n * 3);
    for (size_t i = 0; i < n; ++i) {
        b.order[i] = (uint32_t)i;
        const RtTri& t = tris[i];
        const float e = 1.0e-5f;
        bmn[3 * i] = std::fmin(std::fmin(t.p0.x, t.p1.x), t.p2.x) - e;
        bmn[3 * i + 1] = std::fmin(std::fmin(t.p0.y, t.p1.y), t.p2.y) - e;
        bmn[3 * i + 2] = std::fmin(std::fmin(t.p0.z, t.p1.z), t.p2.z) - e;
        bmx[3 * i] = std::fmax(std::fmax(t.p0.x, t.p1.x), t.p2.x) + e;
        bmx[3 * i + 1] = std::fmax(std::fmax(t.p0.y, t.p1.y), t.p2.y) + e;
        bmx[3 * i + 2] = std::fmax(std::fmax(t.p0.z, t.p1.z), t.p2.z) + e;
        for (int k = 0; k < 3; ++k) cen[3 * i + k] = 0.5f * (bmn[3 * i + k] + bmx[3 * i + k]);
    }
    b.nodes.clear();
    b.nodes.reserve(2 * n / 2 + 16);
    struct Item { uint32_t node, begin, end; };
    std::vector<Item> stack;
    b.nodes.push_back({});
    stack.push_back({0, 0, (uint32_t)n});
    while (!stack.empty()) {
        Item it = stack.back();
        stack.pop_back();
        BvhNode nd;
        for (int k = 0; k < 3; ++k) { nd.mn[k] = INFINITY; nd.mx[k] = -INFINITY; }
        float cmn[3] = {INFINITY, INFINITY, INFINITY}, cmx[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = it.begin; i < it.end; ++i) {
            const uint32_t t = b.order[i];
            for (int k = 0; k < 3; ++k) {
                nd.mn[k] = std::fmin(nd.mn[k], bmn[3 * t + k]);
                nd.mx[k] = std::fmax(nd.mx[k], bmx[3 * t + k]);
                cmn[k] = std::fmin(cmn[k], cen[3 * t + k]);
                cmx[k] = std::fmax(cmx[k], cen[3 * t + k]);
            }
        }
        const uint32_t cnt = it.end - it.begin;
        int axis = 0;
        float ext = cmx[0] - cmn[0];
        for (int k = 1; k < 3; ++k)
            if (cmx[k] - cmn[k] > ext) { ext = cmx[k] - cmn[k]; axis = k; }
        if (cnt <= 4 || !(ext > 0.0f)) {
            nd.left = it.begin;
            nd.count = cnt;
            b.nodes[it.node] = nd;
            continue;
        }
        const uint32_t mid = it.begin + cnt / 2;
        std::nth_element(b.order.begin() + it.begin, b.order.begin() + mid, b.order.begin() + it.end,
                         [&](uint32_t x, uint32_t y) { return cen[3 * x + axis] < cen[3 * y + axis]; });
        const uint32_t l = (uint32_t)b.nodes.size();
        b.nodes.push_back({});
        b.nodes.push_back({});
        nd.left = l;
        nd.count = 0;
        b.nodes[it.node] = nd;
        stack.push_back({l, it.begin, mid});
        stack.push_back({l + 1, mid, it.end});
    }
}
// ray_triangle_intersect (src/raytracer.rs:225-260), Moller-Trumbore.
bool ray_tri(V3 o, V3 d, const RtTri& t, float tmin, float tmax, float& th) {
    const V3 e1 = sub(t.p1, t.p0), e2 = sub(t.p2, t.p0);
    const V3 pv = cross3(d, e2);
    const float det = dot3(e1, pv);
    if (std::fabs(det) <= 1.0e-8f) return false;
    const float inv = 1.0f / det;
    const V3 tv = sub(o, t.p0);
    const float u = dot3(tv, pv) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const V3 qv = cross3(tv, e1);
    const float v = dot3(d, qv) * inv;
    if (v < 0.0f || (u + v) > 1.0f) return false;
    const float tt = dot3(e2, qv) * inv;
    if (tt < tmin || tt > tmax) return false;
    th = tt;
    return true;
}
// trace_transmittance (src/raytracer.rs:172-207). Translucent hits multiply
// in (t, triangle index) order: the reference sorts by t and keeps its BVH's
// visiting order for equal t, which no other traversal reproduces, so equal
// t is ordered by triangle (the device version uses the same rule).
float trace_transmittance(const Bvh& b, const std::vector<RtTri>& tris, const std::vector<swr_material_view>& mats,
                          V3 o, V3 d, float tmin, float tmax) {
    const float inv[3] = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    std::vector<std::pair<float, uint32_t>> hits;  // (t, triangle)
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const BvhNode& nd = b.nodes[stack[--sp]];
        float t0 = 0.0f, t1 = INFINITY;
        const float oo[3] = {o.x, o.y, o.z};
        bool miss = false;
        for (int k = 0; k < 3; ++k) {
            float ta = (nd.mn[k] - oo[k]) * inv[k];
            float tb = (nd.mx[k] - oo[k]) * inv[k];
            if (ta != ta) ta = -INFINITY;
            if (tb != tb) tb = INFINITY;
            if (ta > tb) std::swap(ta, tb);
            t0 = std::fmax(t0, ta);
            t1 = std::fmin(t1, tb);
            if (t0 > t1) { miss = true; break; }
        }
        if (miss) continue;
        if (nd.count == 0) {
            if (sp + 2 <= 128) {
                stack[sp++] = nd.left;
                stack[sp++] = nd.left + 1;
            }
            continue;
        }
        for (uint32_t i = 0; i < nd.count; ++i) {
            const RtTri& t = tris[b.order[nd.left + i]];
            float th;
            if (!ray_tri(o, d, t, tmin, tmax, th)) continue;
            if (!mats[t.material].is_translucent) return 0.0f;
            hits.push_back({th, b.order[nd.left + i]});
        }
    }
    // t ascending (a NaN t, possible only with non-finite vertices, last), then triangle.
    std::sort(hits.begin(), hits.end(), [](const std::pair<float, uint32_t>& x, const std::pair<float, uint32_t>& y) {
        const bool xn = x.first != x.first, yn = y.first != y.first;
        if (xn != yn) return yn;
        if (!xn && x.first != y.first) return x.first < y.first;
        return x.second < y.second;
    });
    float tr = 1.0f;
    for (const auto& h : hits) {
        tr *= mats[tris[h.second].material].transmission;
        if (tr <= 0.0001f) return 0.0f;
    }
    return tr;
}

// build_uniform_sphere_samples (src/gi.rs:416-434) for every direction set
// of bake_voxel_gi: Hammersley points with a Cranley-Patterson rotation per
// set, mapped to the unit sphere.
std::vector<float> gi_direction_sets() {
    std::vector<float> d;
    d.reserve((size_t)kGiSets * kGiSamples * 3);
    const float pi = 3.14159265358979323846f;
    for (uint32_t set = 0; set < kGiSets; ++set) {
        const float ox = radical_inverse_vdc(set + 1), oy = ((float)set + 0.5f) / (float)kGiSets;
        for (uint32_t i = 0; i < kGiSamples; ++i) {
            float hx, hy;
            hammersley(i, kGiSamples, hx, hy);
            float xx = hx + ox, xy = hy + oy;
            xx = xx - std::trunc(xx);  // f32::fract
            xy = xy - std::trunc(xy);
            const float z = 1.0f - 2.0f * xx;
            const float r = std::sqrt(std::fmax(1.0f - z * z, 0.0f));
            const float phi = 2.0f * pi * xy;
            const V3 v = normalize3({r * std::cos(phi), r * std::sin(phi), z});
            d.push_back(v.x);
            d.push_back(v.y);
            d.push_back(v.z);
        }
    }
    return d;
}

// The voxel GI bake's inputs (the ray tracer's triangles with normals and
// texture coordinates, its BVH, materials, mip-0 textures, the sky) and the
// device bake; s->voxel_sh4 receives the blurred SH4 grid.
swr_status bake_gi(SceneImpl* s, const std::vector<RtTri>& rt, const std::vector<uint8_t>& active, uint32_t n,
                   V3 bmn, V3 vsz, std::string& err) {
    std::vector<BakeTri> bt;
    bt.reserve(rt.size());
    for (const HNode& nd : s->nodes) {
        if (nd.mesh < 0) continue;
        for (uint32_t gp : s->meshes[nd.mesh].prims) {
            const HPrimitive& p = s->prims[gp];
            for (size_t t = 0; t + 2 < p.idx.size(); t += 3) {
                V3 pp[3];
                for (int k = 0; k < 3; ++k) {
                    const float* q = &p.pos4[4 * (size_t)p.idx[t + k]];
                    const V4 w = mulmv(nd.transform, {q[0], q[1], q[2], q[3]});
                    pp[k] = {w.x, w.y, w.z};
                }
                const V3 fn = cross3(sub(pp[1], pp[0]), sub(pp[2], pp[0]));
                if (dot3(fn, fn) <= 1.0e-12f) continue;
                const V3 nn = normalize3(fn);
                BakeTri b{};
                const V3* P[3] = {&pp[0], &pp[1], &pp[2]};
                float* dst[3] = {b.p0, b.p1, b.p2};
                float* uv[3] = {b.uv0, b.uv1, b.uv2};
                for (int k = 0; k < 3; ++k) {
                    dst[k][0] = P[k]->x;
                    dst[k][1] = P[k]->y;
                    dst[k][2] = P[k]->z;
                    uv[k][0] = p.uv2[2 * (size_t)p.idx[t + k]];
                    uv[k][1] = p.uv2[2 * (size_t)p.idx[t + k] + 1];
                }
                b.n[0] = nn.x;
                b.n[1] = nn.y;
                b.n[2] = nn.z;
                b.material = p.material;
                bt.push_back(b);
            }
        }
    }
    Bvh bvh;
    if (!rt.empty()) bvh_build(rt, bvh);
    std::vector<BakeNode> nodes(bvh.nodes.size());
    for (size_t i = 0; i < nodes.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            nodes[i].mn[k] = bvh.nodes[i].mn[k];
            nodes[i].mx[k] = bvh.nodes[i].mx[k];
        }
        nodes[i].left = bvh.nodes[i].left;
        nodes[i].count = bvh.nodes[i].count;
    }
    // Mip 0 of every scene texture in one pool.
    std::vector<uint32_t> texels;
    std::vector<BakeTexture> texs;
    for (const HTexture& t : s->textures) {
        texs.push_back({(uint32_t)texels.size(), t.width, t.height});
        texels.insert(texels.end(), t.data.begin(), t.data.begin() + (size_t)t.width * t.height);
    }
    std::vector<BakeMaterial> mats;
    for (const swr_material_view& m : s->materials) {
        BakeMaterial b{};
        for (int k = 0; k < 3; ++k) {
            b.base[k] = m.base_color_factor[k];
            b.emissive[k] = m.emissive_factor[k];
        }
        b.base_tex = m.tex[0];
        b.emissive_tex = m.tex[3];
        b.base_wrap_s = m.wrap_s[0];
        b.base_wrap_t = m.wrap_t[0];
        b.emissive_wrap_s = m.wrap_s[3];
        b.emissive_wrap_t = m.wrap_t[3];
        b.translucent = m.is_translucent;
        b.transmission = m.transmission;
        mats.push_back(b);
    }
    std::vector<float> lut(256);
    for (int i = 0; i < 256; ++i) lut[i] = srgb_to_linear_scalar((float)i / 255.0f);
    const std::vector<float> dirs = gi_direction_sets();
    BakeInput in;
    in.tris = bt.data();
    in.ntris = bt.size();
    in.nodes = nodes.data();
    in.nnodes = nodes.size();
    in.order = bvh.order.data();
    in.mats = mats.data();
    in.nmat = (uint32_t)mats.size();
    in.texels = texels.data();
    in.ntexels = texels.size();
    in.textures = texs.data();
    in.ntex = (uint32_t)texs.size();
    in.cubemap = s->cubemap.data.data();
    in.cube_size = s->cubemap.width;
    in.sky_lut = lut.data();
    in.dirs = dirs.data();
    for (int i = 0; i < 4; ++i)
        for (int c = 0; c < 3; ++c) in.irradiance_sh[i][c] = s->irradiance_sh[i][c];
    const V3 ld = normalize3(s->light_dir);
    const V3 cmin = add(bmn, mul(vsz, 0.5f));
    const float l3[3] = {ld.x, ld.y, ld.z}, lc[3] = {s->light_color.x, s->light_color.y, s->light_color.z};
    for (int k = 0; k < 3; ++k) {
        in.light_dir[k] = l3[k];
        in.light_color[k] = lc[k];
    }
    in.n = n;
    in.bounds_min[0] = bmn.x;
    in.bounds_min[1] = bmn.y;
    in.bounds_min[2] = bmn.z;
    in.vsz[0] = vsz.x;
    in.vsz[1] = vsz.y;
    in.vsz[2] = vsz.z;
    in.cmin[0] = cmin.x;
    in.cmin[1] = cmin.y;
    in.cmin[2] = cmin.z;
    in.active = active.data();
    in.sun = s->voxel_light.data();
    s->voxel_sh4.assign((size_t)n * n * n * 16, 0.0f);
    return gi_bake_device(in, s->voxel_sh4.data(), err);
}

}  // namespace

swr_status build_scene(const swr_scene_desc* desc, SceneImpl* s, std::string& err) {
    const unsigned threads = hw_threads(desc->host_threads);
    // Materials (src/scene.rs:690-780).
    if (desc->material_count == 0) {
        err = "scene has no materials";
        return SWR_BAD_SCENE;
    }
    for (uint32_t i = 0; i < desc->material_count; ++i) {
        const swr_material_desc& m = desc->materials[i];
        swr_material_view v{};
        for (int k = 0; k < 4; ++k) v.base_color_factor[k] = m.base_color_factor[k];
        v.metallic_factor = m.metallic_factor;
        v.roughness_factor = m.roughness_factor;
        for (int k = 0; k < 3; ++k) v.emissive_factor[k] = m.emissive_factor[k];
        v.alpha_cutoff = m.alpha_cutoff;
        v.transmission = m.has_transmission ? m.transmission : 0.0f;
        // The transmission texture belongs to KHR_materials_transmission: a
        // material without the extension has none (src/scene.rs:770-779).
        const swr_texref none = {-1, 0, 0, 0};
        const swr_texref refs[6] = {m.base_color, m.metallic_roughness, m.normal, m.emissive, m.occlusion,
                                    m.has_transmission ? m.transmission_texture : none};
        for (int k = 0; k < 6; ++k) {
            if (refs[k].texture >= (int32_t)desc->texture_count) {
                err = "material references a missing texture";
                return SWR_BAD_SCENE;
            }
            v.tex[k] = refs[k].texture < 0 ? -1 : refs[k].texture;
            v.wrap_s[k] = refs[k].wrap_s;
            v.wrap_t[k] = refs[k].wrap_t;
            if (refs[k].texture >= 0 && (refs[k].wrap_s > 2 || refs[k].wrap_t > 2)) {
                err = "invalid wrap mode";
                return SWR_INVALID_ARG;
            }
        }
        // The occlusion strength is read from the occlusion texture info: 1
        // without one (src/scene.rs:756-759).
        v.occlusion_strength = v.tex[4] >= 0 ? m.occlusion_strength : 1.0f;
        v.is_alpha_tested = (m.alpha_mask && v.tex[0] >= 0) ? 1u : 0u;
        v.is_translucent = m.has_transmission ? 1u : 0u;
        s->materials.push_back(v);
    }
    // Textures.
    for (uint32_t i = 0; i < desc->texture_count; ++i) {
        const swr_texture_desc& t = desc->textures[i];
        if (!t.rgba8 || t.width == 0 || t.height == 0 || t.type == SWR_TEX_CUBEMAP || t.type > SWR_TEX_LINEAR) {
            err = "invalid texture";
            return SWR_INVALID_ARG;
        }
        s->textures.push_back(make_texture(t.width, t.height, t.type, t.rgba8, false));
    }
    // Mip chains, the BRDF LUT and the GGX prefilter run on the device for
    // scenes that go there (ibl.cu, bit-exact with these host loops), on
    // host threads for host-only scenes.
    const bool on_device = !(desc->flags & SWR_SCENE_HOST_ONLY);
    if (on_device) {
        std::vector<HTexture*> texs;
        for (HTexture& t : s->textures) texs.push_back(&t);
        const swr_status mst = mipmaps_device(texs, err);
        if (mst != SWR_OK) return mst;
    } else {
        parallel_for(s->textures.size(), threads, [&](size_t i) { s->textures[i].generate_mipmaps(); });
    }
    // Meshes / primitives (src/scene.rs:422-495).
    for (uint32_t mi = 0; mi < desc->mesh_count; ++mi) {
        const swr_mesh_desc& md = desc->meshes[mi];
        HMesh hm;
        for (uint32_t pi = 0; pi < md.primitive_count; ++pi) {
            const swr_primitive_desc& pd = md.primitives[pi];
            if (!pd.positions || !pd.indices || pd.index_count % 3 != 0 || pd.vertex_count == 0) {
                err = "invalid primitive";
                return SWR_INVALID_ARG;
            }
            for (uint32_t k = 0; k < pd.index_count; ++k)
                if (pd.indices[k] >= pd.vertex_count) {
                    err = "index out of range";
                    return SWR_BAD_SCENE;
                }
            HPrimitive hp;
            const size_t nv = pd.vertex_count;
            hp.pos4.resize(nv * 4);
            for (size_t v = 0; v < nv; ++v) {
                hp.pos4[4 * v] = pd.positions[3 * v];
                hp.pos4[4 * v + 1] = pd.positions[3 * v + 1];
                hp.pos4[4 * v + 2] = pd.positions[3 * v + 2];
                hp.pos4[4 * v + 3] = 1.0f;
            }
            hp.idx.assign(pd.indices, pd.indices + pd.index_count);
            hp.uv2.assign(nv * 2, 0.0f);
            if (pd.texcoords) std::memcpy(hp.uv2.data(), pd.texcoords, nv * 2 * sizeof(float));
            if (pd.normals) {
                hp.nrm4.assign(nv * 4, 0.0f);
                for (size_t v = 0; v < nv; ++v)
                    for (int k = 0; k < 3; ++k) hp.nrm4[4 * v + k] = pd.normals[3 * v + k];
            } else {
                compute_smooth_normals(hp.pos4, hp.idx, hp.nrm4);
            }
            if (pd.tangents) {
                hp.tan4.assign(pd.tangents, pd.tangents + nv * 4);
            } else {
                compute_tangents(hp.pos4, hp.uv2, hp.nrm4, hp.idx, hp.tan4);
            }
            compute_bounding_sphere(hp.pos4, hp.sphere);
            const int32_t mat = pd.material < 0 ? 0 : pd.material;
            if ((uint32_t)mat >= desc->material_count) {
                err = "primitive references a missing material";
                return SWR_BAD_SCENE;
            }
            hp.material = (uint32_t)mat;
            hp.tri_id_base = hm.tri_count;
            hm.tri_count += pd.index_count / 3;
            hm.prims.push_back((uint32_t)s->prims.size());
            if (s->materials[hp.material].is_translucent) hm.translucent.push_back(pi);
            else hm.opaque.push_back(pi);
            s->vtx_total += nv;
            s->prims.push_back(std::move(hp));
        }
        s->meshes.push_back(std::move(hm));
    }
    // Nodes (src/scene.rs:286-331): bounding_sphere_world starts at the local
    // transform's origin with radius 0 and grows by each primitive's sphere.
    uint32_t tri_base = 0;
    for (uint32_t ni = 0; ni < desc->node_count; ++ni) {
        const swr_node_desc& nd = desc->nodes[ni];
        HNode hn;
        hn.transform = from_array(nd.world);
        const M4 local = from_array(nd.local);
        const V4 o = mulmv(local, {0.0f, 0.0f, 0.0f, 1.0f});
        hn.sphere[0] = o.x;
        hn.sphere[1] = o.y;
        hn.sphere[2] = o.z;
        hn.sphere[3] = 0.0f;
        hn.mesh = nd.mesh;
        if (nd.mesh >= (int32_t)desc->mesh_count) {
            err = "node references a missing mesh";
            return SWR_BAD_SCENE;
        }
        hn.tri_id_base = tri_base;
        if (nd.mesh >= 0) {
            const HMesh& hm = s->meshes[nd.mesh];
            for (uint32_t gp : hm.prims) {
                float ws[4];
                transform_sphere(hn.transform, s->prims[gp].sphere, ws);
                const float dist = length3(sub({hn.sphere[0], hn.sphere[1], hn.sphere[2]}, {ws[0], ws[1], ws[2]}));
                if (dist + ws[3] > hn.sphere[3]) hn.sphere[3] = dist + ws[3];
            }
            tri_base += hm.tri_count;
            s->tri_total += hm.tri_count;
        }
        s->nodes.push_back(hn);
    }
    // Scene bounds (src/scene.rs:333-351).
    V3 bmn = {INFINITY, INFINITY, INFINITY}, bmx = {-INFINITY, -INFINITY, -INFINITY};
    for (const HNode& n : s->nodes) {
        if (n.mesh < 0) continue;
        for (uint32_t gp : s->meshes[n.mesh].prims) {
            const HPrimitive& p = s->prims[gp];
            for (size_t v = 0; v < p.pos4.size(); v += 4) {
                const V4 t = mulmv(n.transform, {p.pos4[v], p.pos4[v + 1], p.pos4[v + 2], 1.0f});
                bmn = {std::fmin(bmn.x, t.x), std::fmin(bmn.y, t.y), std::fmin(bmn.z, t.z)};
                bmx = {std::fmax(bmx.x, t.x), std::fmax(bmx.y, t.y), std::fmax(bmx.z, t.z)};
            }
        }
    }
    s->bounds_min = bmn;
    s->bounds_max = bmx;
    s->bounds_center = mul(add(bmn, bmx), 0.5f);
    s->bounds_diagonal = length3(sub(bmx, bmn));
    // Light (src/scene.rs:236-239).
    s->light_dir = normalize3({-0.2f, 1.0f, 0.5f});
    s->light_color = mul(V3{1.0f, 1.0f, 0.95f}, 5.0f);
    // Environment (src/scene.rs:152-228).
    if (!desc->cubemap_faces || desc->cubemap_face_size == 0) {
        err = "cubemap faces missing";
        return SWR_INVALID_ARG;
    }
    // Load-time tables grow with the square or cube of these sizes; past
    // these limits a descriptor asks for more memory than any scene needs.
    if (desc->cubemap_face_size > 16384u || desc->brdf_lut_size > 4096u || desc->voxel_grid_size > 1024u ||
        desc->specular_samples > 65536u) {
        err = "cubemap_face_size, brdf_lut_size, voxel_grid_size or specular_samples out of range";
        return SWR_INVALID_ARG;
    }
    s->cubemap = make_texture(desc->cubemap_face_size, desc->cubemap_face_size, SWR_TEX_CUBEMAP, desc->cubemap_faces, true);
    if (on_device) {
        const swr_status cst = mipmaps_device({&s->cubemap}, err);
        if (cst != SWR_OK) return cst;
    } else {
        s->cubemap.generate_mipmaps();
    }
    // The GGX-prefiltered environment, read from its cache file when one is
    // given and valid, else computed and written there (src/scene.rs:164-205).
    bool specular_loaded = false;
    if (desc->ggx_cache_path) {
        std::string msg;
        const CacheRead r = read_ggx_cache(desc->ggx_cache_path, s->cubemap.width, s->cubemap.height, s->specular, msg);
        specular_loaded = r == CacheRead::Loaded;
        s->ggx_cache = specular_loaded ? SWR_CACHE_LOADED : (r == CacheRead::NoCodec ? SWR_CACHE_NO_CODEC : 0u);
    }
    if (!specular_loaded) {
        const uint32_t samples = desc->specular_samples ? desc->specular_samples : 64u;
        if (on_device) {
            const swr_status pst = prefiltered_specular_device(s->cubemap, samples, s->specular, s->precompute_host_texels, err);
            if (pst != SWR_OK) return pst;
        } else {
            s->specular = generate_prefiltered_specular(s->cubemap, samples, threads);
        }
        if (desc->ggx_cache_path && s->ggx_cache != SWR_CACHE_NO_CODEC) {
            std::string werr;
            s->ggx_cache = write_ggx_cache(desc->ggx_cache_path, s->specular, werr) ? SWR_CACHE_WRITTEN
                                                                                    : SWR_CACHE_WRITE_FAILED;
        }
    }
    compute_irradiance_sh4(s->cubemap, s->irradiance_sh);
    if (on_device) {
        const swr_status bst = brdf_lut_device(desc->brdf_lut_size ? desc->brdf_lut_size : 128u, s->brdf_lut, err);
        if (bst != SWR_OK) return bst;
    } else {
        s->brdf_lut = generate_brdf_lut(desc->brdf_lut_size ? desc->brdf_lut_size : 128u, threads);
    }
    // Voxel grid (src/main.rs:227-281).
    const uint32_t n = desc->voxel_grid_size ? desc->voxel_grid_size : 128u;
    s->voxel_n = n;
    s->voxel_min = bmn;
    s->voxel_max = bmx;
    s->gi_sh_scale = desc->gi_sh_scale;
    s->sky_visibility = desc->sky_visibility;
    const size_t nvox = (size_t)n * n * n;
    const V3 wsz = sub(bmx, bmn);
    const V3 vsz = {wsz.x / (float)n, wsz.y / (float)n, wsz.z / (float)n};
    // RayTracer::new (src/raytracer.rs:71-133).
    std::vector<RtTri> rt;
    for (const HNode& nd : s->nodes) {
        if (nd.mesh < 0) continue;
        for (uint32_t gp : s->meshes[nd.mesh].prims) {
            const HPrimitive& p = s->prims[gp];
            for (size_t t = 0; t + 2 < p.idx.size(); t += 3) {
                V3 pp[3];
                for (int k = 0; k < 3; ++k) {
                    const float* q = &p.pos4[4 * (size_t)p.idx[t + k]];
                    const V4 w = mulmv(nd.transform, {q[0], q[1], q[2], q[3]});
                    pp[k] = {w.x, w.y, w.z};
                }
                const V3 fn = cross3(sub(pp[1], pp[0]), sub(pp[2], pp[0]));
                if (dot3(fn, fn) <= 1.0e-12f) continue;
                rt.push_back({pp[0], pp[1], pp[2], normalize3(fn), p.material});
            }
        }
    }
    // build_active_voxel_mask (src/gi.rs:151-265), occupancy + dilation.
    std::vector<uint8_t> occupied(nvox, 0);
    {
        const float mine = std::fmax(std::fmin(vsz.x, std::fmin(vsz.y, vsz.z)), 1.0e-6f);
        const float area_ref = mine * mine;
        for (const RtTri& t : rt) {
            const V3 e1 = sub(t.p1, t.p0), e2 = sub(t.p2, t.p0);
            const float area = 0.5f * length3(cross3(e1, e2));
            float ts = std::ceil((area / area_ref) * 2.0f);
            size_t target = ts != ts || ts <= 0.0f ? 0 : (ts >= 1.8e19f ? SIZE_MAX : (size_t)ts);
            target = std::min<size_t>(std::max<size_t>(target, 1), 4096);
            const size_t ns = (size_t)std::ceil(std::sqrt((float)target));
            for (size_t iu = 0; iu < ns; ++iu) {
                for (size_t iv = 0; iv < ns - iu; ++iv) {
                    const float u = ((float)iu + 0.5f) / (float)ns;
                    const float v = ((float)iv + 0.5f) / (float)ns;
                    const float w = (1.0f - u) - v;
                    if (w < 0.0f) continue;
                    const V3 p = add(add(mul(t.p0, w), mul(t.p1, u)), mul(t.p2, v));
                    const float fx = (p.x - bmn.x) / vsz.x, fy = (p.y - bmn.y) / vsz.y, fz = (p.z - bmn.z) / vsz.z;
                    if (fx < 0.0f || fy < 0.0f || fz < 0.0f) continue;
                    const float flx = std::floor(fx), fly = std::floor(fy), flz = std::floor(fz);
                    if (!(flx < (float)n) || !(fly < (float)n) || !(flz < (float)n)) continue;
                    const size_t x = (size_t)flx, y = (size_t)fly, z = (size_t)flz;
                    occupied[z * n * n + y * n + x] = 1;
                }
            }
        }
    }
    std::vector<uint8_t> active = occupied;
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                if (!occupied[(size_t)z * n * n + y * n + x]) continue;
                const uint32_t z0 = z >= 2 ? z - 2 : 0, y0 = y >= 2 ? y - 2 : 0, x0 = x >= 2 ? x - 2 : 0;
                const uint32_t z1 = std::min(z + 2, n - 1), y1 = std::min(y + 2, n - 1), x1 = std::min(x + 2, n - 1);
                for (uint32_t a = z0; a <= z1; ++a)
                    for (uint32_t b = y0; b <= y1; ++b)
                        for (uint32_t c = x0; c <= x1; ++c) active[(size_t)a * n * n + b * n + c] = 1;
            }
    // compute_sun_visibility (src/gi.rs:267-314) and blur_grid: on the device
    // for scenes that go to the device, else (host-only scenes) here.
    if (!(desc->flags & SWR_SCENE_HOST_ONLY)) {
        std::vector<LightTri> lt(rt.size());
        for (size_t i = 0; i < rt.size(); ++i) {
            const RtTri& t = rt[i];
            lt[i] = LightTri{{t.p0.x, t.p0.y, t.p0.z}, {t.p1.x, t.p1.y, t.p1.z}, {t.p2.x, t.p2.y, t.p2.z}, t.material};
        }
        std::vector<uint8_t> trans(s->materials.size());
        std::vector<float> transm(s->materials.size());
        for (size_t i = 0; i < s->materials.size(); ++i) {
            trans[i] = s->materials[i].is_translucent ? 1 : 0;
            transm[i] = s->materials[i].transmission;
        }
        const V3 ld = normalize3(s->light_dir);
        const V3 cmin = add(bmn, mul(vsz, 0.5f));
        const float bmin3[3] = {bmn.x, bmn.y, bmn.z}, bmax3[3] = {bmx.x, bmx.y, bmx.z};
        const float cmin3[3] = {cmin.x, cmin.y, cmin.z}, vsz3[3] = {vsz.x, vsz.y, vsz.z}, ld3[3] = {ld.x, ld.y, ld.z};
        s->voxel_light.assign(nvox, 0.0f);
        const swr_status vst = sun_visibility_device(lt.data(), lt.size(), trans.data(), transm.data(),
                                                     (uint32_t)trans.size(), active.data(), n, bmin3, bmax3, cmin3,
                                                     vsz3, ld3, length3(vsz) * 3.0f, s->voxel_light.data(), err);
        if (vst != SWR_OK) return vst;
    } else {
        std::vector<float> light(nvox, 1.0f);
        {
            Bvh bvh;
            if (!rt.empty()) bvh_build(rt, bvh);
            const V3 ld = normalize3(s->light_dir);
            const V3 cmin = add(bmn, mul(vsz, 0.5f));
            const float bias = length3(vsz) * 3.0f;
            size_t active_total = 0;
            for (uint8_t a : active) active_total += a;
            if (active_total > 0 && !rt.empty()) {
                parallel_for(nvox, threads, [&](size_t idx) {
                    if (!active[idx]) return;
                    const size_t z = idx / ((size_t)n * n);
                    const size_t rem = idx % ((size_t)n * n);
                    const size_t y = rem / n, x = rem % n;
                    const V3 vc = add(cmin, mulv(V3{(float)x, (float)y, (float)z}, vsz));
                    const V3 o = add(vc, mul(ld, bias));
                    light[idx] = trace_transmittance(bvh, rt, s->materials, o, ld, 1.0e-4f, INFINITY);
                });
            }
            // blur_grid (src/voxelgrid.rs:370-419): 3x3x3 mean, then squared.
            std::vector<float> blurred(nvox, 0.0f);
            parallel_for(n, threads, [&](size_t z) {
                for (uint32_t y = 0; y < n; ++y)
                    for (uint32_t x = 0; x < n; ++x) {
                        float sum = 0.0f;
                        int count = 0;
                        for (int dz = -1; dz <= 1; ++dz)
                            for (int dy = -1; dy <= 1; ++dy)
                                for (int dx = -1; dx <= 1; ++dx) {
                                    const int nx = (int)x + dx, ny = (int)y + dy, nz = (int)z + dz;
                                    if (nx >= 0 && nx < (int)n && ny >= 0 && ny < (int)n && nz >= 0 && nz < (int)n) {
                                        sum += light[(size_t)nz * n * n + (size_t)ny * n + nx];
                                        count += 1;
                                    }
                                }
                        float m = count > 0 ? sum / (float)count : 0.0f;
                        blurred[z * n * n + (size_t)y * n + x] = count > 0 ? m * m : 0.0f;
                    }
            });
            s->voxel_light = std::move(blurred);
        }
    }
    // bake_voxel_gi (src/gi.rs:316-408) with the reference's --gi.
    // The grid comes from the scene's .gi cache when one is given and valid
    // (try_load_gi_cache, src/main.rs:248-279), else it is baked and written.
    if (desc->flags & SWR_SCENE_GI) {
        bool gi_loaded = false;
        if (desc->gi_cache_path) {
            std::string msg;
            const CacheRead r = read_gi_cache(desc->gi_cache_path, n, s->voxel_sh4, msg);
            gi_loaded = r == CacheRead::Loaded;
            s->gi_cache = gi_loaded ? SWR_CACHE_LOADED : (r == CacheRead::NoCodec ? SWR_CACHE_NO_CODEC : 0u);
        }
        if (!gi_loaded) {
            if (desc->flags & SWR_SCENE_HOST_ONLY) {
                err = "the GI bake runs on the device: SWR_SCENE_GI with SWR_SCENE_HOST_ONLY needs a valid GI cache file";
                return SWR_INVALID_ARG;
            }
            const swr_status gst = bake_gi(s, rt, active, n, bmn, vsz, err);
            if (gst != SWR_OK) return gst;
            if (desc->gi_cache_path && s->gi_cache != SWR_CACHE_NO_CODEC) {
                std::string werr;
                s->gi_cache = write_gi_cache(desc->gi_cache_path, n, s->voxel_sh4, werr) ? SWR_CACHE_WRITTEN
                                                                                          : SWR_CACHE_WRITE_FAILED;
            }
        }
    }
    // initialize_voxel_gi_from_scene (src/gi.rs:123-149).
    for (int i = 0; i < 4; ++i) {
        for (int c = 0; c < 3; ++c) s->gi_const[i][c] = s->irradiance_sh[i][c] * s->gi_sh_scale;
        s->gi_const[i][3] = 0.0f;
    }
    s->gi_const[1][3] = s->sky_visibility;
    // Export views.
    for (const HPrimitive& p : s->prims) {
        swr_primitive_view v{};
        v.vertex_count = (uint32_t)(p.pos4.size() / 4);
        v.index_count = (uint32_t)p.idx.size();
        v.positions = p.pos4.data();
        v.normals = p.nrm4.data();
        v.tangents = p.tan4.data();
        v.texcoords = p.uv2.data();
        v.indices = p.idx.data();
        v.material = p.material;
        v.triangle_id_base = p.tri_id_base;
        for (int k = 0; k < 4; ++k) v.sphere[k] = p.sphere[k];
        s->prim_views.push_back(v);
    }
    for (const HMesh& m : s->meshes) {
        swr_mesh_view v{};
        v.primitive_count = (uint32_t)m.prims.size();
        v.opaque_count = (uint32_t)m.opaque.size();
        v.translucent_count = (uint32_t)m.translucent.size();
        v.primitives = m.prims.data();
        v.opaque = m.opaque.data();
        v.translucent = m.translucent.data();
        s->mesh_views.push_back(v);
    }
    for (const HNode& nd : s->nodes) {
        swr_node_view v{};
        to_array(nd.transform, v.transform);
        for (int k = 0; k < 4; ++k) v.sphere[k] = nd.sphere[k];
        v.mesh = nd.mesh;
        v.triangle_id_base = nd.tri_id_base;
        s->node_views.push_back(v);
    }
    for (const HTexture& t : s->textures) s->tex_views.push_back(t.view());
    return SWR_OK;
}

void export_scene(const SceneImpl* s, swr_scene_host_view* o) {
    std::memset(o, 0, sizeof(*o));
    o->primitive_count = (uint32_t)s->prims.size();
    o->mesh_count = (uint32_t)s->meshes.size();
    o->node_count = (uint32_t)s->nodes.size();
    o->material_count = (uint32_t)s->materials.size();
    o->texture_count = (uint32_t)s->textures.size();
    o->voxel_size = s->voxel_n;
    o->primitives = s->prim_views.data();
    o->meshes = s->mesh_views.data();
    o->nodes = s->node_views.data();
    o->materials = s->materials.data();
    o->textures = s->tex_views.data();
    o->cubemap = s->cubemap.view();
    o->cubemap_specular = s->specular.view();
    o->brdf_lut = s->brdf_lut.view();
    for (int i = 0; i < 4; ++i)
        for (int c = 0; c < 3; ++c) o->irradiance_sh[i][c] = s->irradiance_sh[i][c];
    o->light_direction[0] = s->light_dir.x;
    o->light_direction[1] = s->light_dir.y;
    o->light_direction[2] = s->light_dir.z;
    o->light_color[0] = s->light_color.x;
    o->light_color[1] = s->light_color.y;
    o->light_color[2] = s->light_color.z;
    o->voxel_world_min[0] = s->voxel_min.x;
    o->voxel_world_min[1] = s->voxel_min.y;
    o->voxel_world_min[2] = s->voxel_min.z;
    o->voxel_world_max[0] = s->voxel_max.x;
    o->voxel_world_max[1] = s->voxel_max.y;
    o->voxel_world_max[2] = s->voxel_max.z;
    o->voxel_light_intensity = s->voxel_light.data();
    o->voxel_gi_sh4 = s->voxel_sh4.empty() ? nullptr : s->voxel_sh4.data();
    for (int i = 0; i < 4; ++i)
        for (int c = 0; c < 4; ++c) o->voxel_gi_sh4_const[i][c] = s->gi_const[i][c];
}

namespace {
struct Arena {
    std::vector<uint8_t> host;
    uint64_t add(const void* p, size_t bytes) {
        const uint64_t off = (host.size() + 255) & ~uint64_t(255);
        host.resize(off + bytes);
        if (bytes && p) std::memcpy(host.data() + off, p, bytes);
        return off;
    }
};
DTexture to_dtex(const HTexture& t, uintptr_t addr) {
    DTexture d{};
    d.data = reinterpret_cast<const uint32_t*>(addr);
    d.width = t.width;
    d.height = t.height;
    d.max_mip = t.max_mip;
    for (int k = 0; k < 4; ++k) d.whv[k] = t.whv[k];
    for (uint32_t m = 0; m <= t.max_mip && m < 16; ++m) {
        d.mip_offset[m] = t.mip_offsets[m];
        d.mip_w[m] = t.mip_widths[m];
        d.mip_h[m] = t.mip_heights[m];
        d.array_stride[m] = t.array_stride[m];
        d.mip_wf[m] = t.mip_widths_f[m];
        d.mip_hf[m] = t.mip_heights_f[m];
        const uint32_t w = t.mip_widths[m], h = t.mip_heights[m];
        d.mip_rwf[m] = (w > 0 && (w & (w - 1)) == 0 && (float)w == d.mip_wf[m]) ? 1.0f / (float)w : 0.0f;
        d.mip_rhf[m] = (h > 0 && (h & (h - 1)) == 0 && (float)h == d.mip_hf[m]) ? 1.0f / (float)h : 0.0f;
    }
    return d;
}
}  // namespace

swr_status upload_scene(SceneImpl* s, std::string& err, bool to_device) {
    Arena ar;
    // Vertices, indices, primitive table.
    std::vector<DVertex> verts;
    verts.reserve(s->vtx_total);
    std::vector<uint32_t> idx;
    std::vector<DPrimitive> prims;
    for (const HPrimitive& p : s->prims) {
        DPrimitive dp;
        dp.vtx_base = (uint32_t)verts.size();
        dp.idx_base = (uint32_t)idx.size();
        dp.tri_count = (uint32_t)(p.idx.size() / 3);
        dp.material = p.material;
        prims.push_back(dp);
        const size_t nv = p.pos4.size() / 4;
        for (size_t v = 0; v < nv; ++v) {
            DVertex d;
            d.px = p.pos4[4 * v]; d.py = p.pos4[4 * v + 1]; d.pz = p.pos4[4 * v + 2]; d.u = p.uv2[2 * v];
            d.nx = p.nrm4[4 * v]; d.ny = p.nrm4[4 * v + 1]; d.nz = p.nrm4[4 * v + 2]; d.v = p.uv2[2 * v + 1];
            d.tx = p.tan4[4 * v]; d.ty = p.tan4[4 * v + 1]; d.tz = p.tan4[4 * v + 2]; d.tw = p.tan4[4 * v + 3];
            verts.push_back(d);
        }
        idx.insert(idx.end(), p.idx.begin(), p.idx.end());
    }
    // Per mesh: its primitives in render_mesh's order (opaque, then translucent).
    std::vector<DMeshEntry> entries;
    std::vector<uint32_t> mesh_begin;
    for (const HMesh& m : s->meshes) {
        mesh_begin.push_back((uint32_t)entries.size());
        for (int pass = 0; pass < 2; ++pass)
            for (uint32_t lp : pass == 0 ? m.opaque : m.translucent) {
                const HPrimitive& p = s->prims[m.prims[lp]];
                DMeshEntry me{};
                for (int k = 0; k < 4; ++k) me.sphere[k] = p.sphere[k];
                me.prim = m.prims[lp];
                me.tri_count = (uint32_t)(p.idx.size() / 3);
                me.tri_id_base = p.tri_id_base;
                entries.push_back(me);
            }
    }
    std::vector<float> xf;
    std::vector<DNodeInfo> node_info;
    s->max_draws = 0;
    s->max_chunks = 0;
    s->any_translucent = false;
    for (const HNode& n : s->nodes) {
        float a[16];
        to_array(n.transform, a);
        xf.insert(xf.end(), a, a + 16);
        DNodeInfo ni{};
        std::memcpy(ni.xform, a, sizeof(a));
        ni.tri_id_base = n.tri_id_base;
        if (n.mesh >= 0) {
            const HMesh& m = s->meshes[n.mesh];
            ni.entry_begin = mesh_begin[n.mesh];
            ni.n_opaque = (uint32_t)m.opaque.size();
            ni.n_total = (uint32_t)(m.opaque.size() + m.translucent.size());
            // Upper bounds of one view's draw list: every primitive drawn.
            for (uint32_t gp : m.prims) {
                const uint32_t tc = (uint32_t)(s->prims[gp].idx.size() / 3);
                if (tc == 0) continue;
                s->max_draws += 1;
                s->max_chunks += (tc + kChunkTris - 1) / kChunkTris;
            }
            if (!m.translucent.empty()) s->any_translucent = true;
        }
        node_info.push_back(ni);
    }
    std::vector<DMaterial> mats;
    for (const swr_material_view& m : s->materials) {
        DMaterial d{};
        for (int k = 0; k < 4; ++k) d.base_color[k] = m.base_color_factor[k];
        d.metallic = m.metallic_factor;
        d.roughness = m.roughness_factor;
        d.occlusion_strength = m.occlusion_strength;
        d.alpha_cutoff = m.alpha_cutoff;
        for (int k = 0; k < 3; ++k) d.emissive[k] = m.emissive_factor[k];
        d.flags = (m.is_alpha_tested ? MAT_ALPHA_TESTED : 0u) | (m.is_translucent ? MAT_TRANSLUCENT : 0u);
        for (int k = 0; k < 6; ++k) {
            d.tex[k] = m.tex[k];
            d.wrap_s[k] = m.wrap_s[k];
            d.wrap_t[k] = m.wrap_t[k];
        }
        d.transmission = m.transmission;
        mats.push_back(d);
    }
    const uint64_t o_vert = ar.add(verts.data(), verts.size() * sizeof(DVertex));
    const uint64_t o_idx = ar.add(idx.data(), idx.size() * sizeof(uint32_t));
    const uint64_t o_prim = ar.add(prims.data(), prims.size() * sizeof(DPrimitive));
    const uint64_t o_xf = ar.add(xf.data(), xf.size() * sizeof(float));
    const uint64_t o_mat = ar.add(mats.data(), mats.size() * sizeof(DMaterial));
    const uint64_t o_ninfo = ar.add(node_info.data(), node_info.size() * sizeof(DNodeInfo));
    const uint64_t o_entries = ar.add(entries.data(), entries.size() * sizeof(DMeshEntry));
    std::vector<uint64_t> o_tex;
    std::vector<const HTexture*> all_tex;
    for (const HTexture& t : s->textures) all_tex.push_back(&t);
    all_tex.push_back(&s->cubemap);
    all_tex.push_back(&s->specular);
    all_tex.push_back(&s->brdf_lut);
    for (const HTexture* t : all_tex) o_tex.push_back(ar.add(t->data.data(), t->data.size() * sizeof(uint32_t)));
    const uint64_t o_vox = ar.add(s->voxel_light.data(), s->voxel_light.size() * sizeof(float));
    const uint64_t o_sh4 = ar.add(s->voxel_sh4.data(), s->voxel_sh4.size() * sizeof(float));
    const uint64_t o_dtex = ar.add(nullptr, all_tex.size() * sizeof(DTexture));
    const uint64_t o_dscene = ar.add(nullptr, sizeof(DScene));
    void* dblock = nullptr;
    cudaError_t e = cudaSuccess;
    if (to_device) {
        e = cudaMalloc(&dblock, ar.host.size());
        if (e != cudaSuccess) {
            err = std::string("cudaMalloc(scene): ") + cudaGetErrorString(e);
            cudaGetLastError();
            return e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR;
        }
    }
    // Host-only scenes are packed against a zero base so the layout code runs.
    const uintptr_t base = reinterpret_cast<uintptr_t>(dblock);
    auto at = [&](uint64_t off) { return base + (uintptr_t)off; };
    std::vector<DTexture> dtex;
    for (size_t i = 0; i < all_tex.size(); ++i) dtex.push_back(to_dtex(*all_tex[i], at(o_tex[i])));
    std::memcpy(ar.host.data() + o_dtex, dtex.data(), dtex.size() * sizeof(DTexture));
    DScene& ds = s->dscene;
    ds = DScene{};
    ds.vertices = reinterpret_cast<const DVertex*>(at(o_vert));
    ds.indices = reinterpret_cast<const uint32_t*>(at(o_idx));
    ds.prims = reinterpret_cast<const DPrimitive*>(at(o_prim));
    ds.node_xform = reinterpret_cast<const float*>(at(o_xf));
    ds.materials = reinterpret_cast<const DMaterial*>(at(o_mat));
    ds.textures = reinterpret_cast<const DTexture*>(at(o_dtex));
    ds.voxel_light = reinterpret_cast<const float*>(at(o_vox));
    ds.voxel_sh4 = s->voxel_sh4.empty() ? nullptr : reinterpret_cast<const float4*>(at(o_sh4));
    ds.node_info = reinterpret_cast<const DNodeInfo*>(at(o_ninfo));
    ds.mesh_entries = reinterpret_cast<const DMeshEntry*>(at(o_entries));
    ds.tex_cubemap = (uint32_t)s->textures.size();
    ds.tex_specular = ds.tex_cubemap + 1;
    ds.tex_brdf_lut = ds.tex_cubemap + 2;
    ds.voxel_n = s->voxel_n;
    const V3 wsz = sub(s->voxel_max, s->voxel_min);
    ds.voxel_min[0] = s->voxel_min.x;
    ds.voxel_min[1] = s->voxel_min.y;
    ds.voxel_min[2] = s->voxel_min.z;
    // VoxelGrid::voxel_size (src/voxelgrid.rs:154-161).
    ds.voxel_size_f[0] = wsz.x / (float)s->voxel_n;
    ds.voxel_size_f[1] = wsz.y / (float)s->voxel_n;
    ds.voxel_size_f[2] = wsz.z / (float)s->voxel_n;
    for (int i = 0; i < 4; ++i)
        for (int c = 0; c < 3; ++c) ds.gi_rgb[i][c] = s->gi_const[i][c];
    ds.sky_visibility = s->sky_visibility;
    ds.light_dir[0] = s->light_dir.x;
    ds.light_dir[1] = s->light_dir.y;
    ds.light_dir[2] = s->light_dir.z;
    ds.light_color[0] = s->light_color.x;
    ds.light_color[1] = s->light_color.y;
    ds.light_color[2] = s->light_color.z;
    std::memcpy(ar.host.data() + o_dscene, &ds, sizeof(DScene));
    s->d_bytes = ar.host.size();
    if (!to_device) return SWR_OK;
    e = cudaMemcpy(dblock, ar.host.data(), ar.host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        cudaFree(dblock);
        err = std::string("cudaMemcpy(scene): ") + cudaGetErrorString(e);
        return SWR_CUDA_ERROR;
    }
    s->d_block = dblock;
    s->d_bytes = ar.host.size();
    s->d_scene = reinterpret_cast<DScene*>(at(o_dscene));
    return SWR_OK;
}

void free_scene_device(SceneImpl* s) {
    if (s->d_block) cudaFree(s->d_block);
    s->d_block = nullptr;
    s->d_scene = nullptr;
}

// RecipSqrtEstimate (Arm ARM, FPRSqrtEstimate's helper): a is a 9-bit
// fixed-point operand in [128, 512) for 0.25 <= x < 1.0; returns the 9-bit
// estimate r in [256, 512) of 1/sqrt(x); the table keeps r<7:0>.
void build_rsqrt_table(uint8_t out[512]) {
    for (int a0 = 0; a0 < 512; ++a0) {
        if (a0 < 128) {
            out[a0] = 0;
            continue;
        }
        int64_t a = a0;
        if (a < 256) {
            a = a * 2 + 1;
        } else {
            a = (a >> 1) << 1;
            a = (a + 1) * 2;
        }
        int64_t b = 512;
        while (a * (b + 1) * (b + 1) < (int64_t(1) << 28)) b = b + 1;
        const int64_t r = (b + 1) / 2;
        out[a0] = (uint8_t)(r & 0xFF);
    }
}

}  // namespace swr
