// CPU oracle, part 2: the reference's load-time scene processing and its
// render camera.
//
// TEST INFRASTRUCTURE ONLY. From an in-memory scene descriptor this file
// builds the processed scene the per-frame path reads: primitives with
// generated normals and tangents, bounding spheres, node spheres, scene
// bounds, materials, texture mip chains, the environment cubemap and its
// GGX-prefiltered copy, the BRDF LUT, irradiance SH4, the light, the voxel
// grid's sun visibility and constant SH4 (and, with SWR_SCENE_GI, the baked
// SH4 grid); and it builds the render camera's matrices. Every function is
// restated from the reference's sources (file:line given at each), not from
// the product, so a test can hold the product's exported tables against
// these bit for bit. Nothing in the product links, imports or calls it; only
// tests/, the smoke check and bench.py's CPU legs do.
//
// Parity status: unpinned against the reference binary (Rust; no toolchain
// or vendored crates exist here). Third-party arithmetic the reference relies
// on is restated from the published algorithms of glam 0.30.10 (Cargo.lock),
// in the order its aarch64 NEON backend evaluates them, since the reference
// runs on the GB300 host's Grace CPU: Vec4 dot = (x*x'+y*y')+(z*z'+w*w')
// (pairwise vaddvq), Vec3A dot = (x*x'+y*y')+z*z', normalize = v * (1/|v|),
// Mat4*Vec4 = ((X*x+Y*y)+Z*z)+W*w, transform_point3a = ((X*x+Y*y)+Z*z)+W,
// Quat*Quat in the grouping of glam's SIMD quat_mul, Mat4::inverse by the
// GLM cofactor expansion with the determinant summed pairwise. Rust's
// f32::powi(5) is LLVM's powi expansion x * ((x*x)*(x*x)); powf, sinf,
// cosf, tanf, atan2f and asinf come from the host libm, as a Rust build
// links them. Compiled with -ffp-contract=off: nothing here is fused.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#include "../include/swr.h"

extern "C" int oracle_sun_visibility(const swr_scene_host_view* v, uint32_t threads, float* out);
extern "C" int oracle_gi_bake(const swr_scene_host_view* v, uint32_t threads, float* out);

namespace ors {

const float kPi = 3.14159265358979323846f;  // std::f32::consts::PI

template <class F>
void par(size_t n, unsigned threads, F f) {
    if (threads <= 1 || n < 2) {
        for (size_t i = 0; i < n; ++i) f(i);
        return;
    }
    std::vector<std::thread> pool;
    const size_t per = (n + threads - 1) / threads;
    for (unsigned t = 0; t < threads; ++t) {
        const size_t a = t * per, b = std::min(n, a + per);
        if (a >= b) break;
        pool.emplace_back([=] {
            for (size_t i = a; i < b; ++i) f(i);
        });
    }
    for (auto& th : pool) th.join();
}

// ---------------------------------------------------------------- glam
struct V3 {
    float x, y, z;
};
struct V4 {
    float x, y, z, w;
};
struct M4 {
    V4 c[4];  // x_axis, y_axis, z_axis, w_axis
};
struct Q {
    float x, y, z, w;
};

inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 operator/(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline V4 operator+(V4 a, V4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
inline V4 operator*(V4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline float dot4(V4 a, V4 b) { return (a.x * b.x + a.y * b.y) + (a.z * b.z + a.w * b.w); }
inline float length(V3 a) { return std::sqrt(dot(a, a)); }
inline float length4(V4 a) { return std::sqrt(dot4(a, a)); }
inline V3 normalize(V3 a) { return a * (1.0f / length(a)); }
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline V3 xyz(V4 a) { return {a.x, a.y, a.z}; }

inline M4 mat(const float* a) {
    M4 m;
    std::memcpy(&m, a, sizeof(m));
    return m;
}
inline V4 mulv(const M4& m, V4 v) { return ((m.c[0] * v.x + m.c[1] * v.y) + m.c[2] * v.z) + m.c[3] * v.w; }
inline M4 mulm(const M4& a, const M4& b) {
    M4 r;
    for (int i = 0; i < 4; ++i) r.c[i] = mulv(a, b.c[i]);
    return r;
}
inline V3 transform_point3a(const M4& m, V3 p) { return xyz(((m.c[0] * p.x + m.c[1] * p.y) + m.c[2] * p.z) + m.c[3]); }
inline M4 identity() {
    M4 m{};
    m.c[0].x = m.c[1].y = m.c[2].z = m.c[3].w = 1.0f;
    return m;
}
inline M4 transpose(const M4& m) {
    const float* a = &m.c[0].x;
    float t[16];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) t[4 * i + j] = a[4 * j + i];
    return mat(t);
}
// Mat4::inverse: GLM's cofactor expansion as glam writes it.
M4 inverse(const M4& s) {
    const float m00 = s.c[0].x, m01 = s.c[0].y, m02 = s.c[0].z, m03 = s.c[0].w;
    const float m10 = s.c[1].x, m11 = s.c[1].y, m12 = s.c[1].z, m13 = s.c[1].w;
    const float m20 = s.c[2].x, m21 = s.c[2].y, m22 = s.c[2].z, m23 = s.c[2].w;
    const float m30 = s.c[3].x, m31 = s.c[3].y, m32 = s.c[3].z, m33 = s.c[3].w;
    const float coef00 = m22 * m33 - m32 * m23, coef02 = m12 * m33 - m32 * m13, coef03 = m12 * m23 - m22 * m13;
    const float coef04 = m21 * m33 - m31 * m23, coef06 = m11 * m33 - m31 * m13, coef07 = m11 * m23 - m21 * m13;
    const float coef08 = m21 * m32 - m31 * m22, coef10 = m11 * m32 - m31 * m12, coef11 = m11 * m22 - m21 * m12;
    const float coef12 = m20 * m33 - m30 * m23, coef14 = m10 * m33 - m30 * m13, coef15 = m10 * m23 - m20 * m13;
    const float coef16 = m20 * m32 - m30 * m22, coef18 = m10 * m32 - m30 * m12, coef19 = m10 * m22 - m20 * m12;
    const float coef20 = m20 * m31 - m30 * m21, coef22 = m10 * m31 - m30 * m11, coef23 = m10 * m21 - m20 * m11;
    const V4 fac0{coef00, coef00, coef02, coef03}, fac1{coef04, coef04, coef06, coef07};
    const V4 fac2{coef08, coef08, coef10, coef11}, fac3{coef12, coef12, coef14, coef15};
    const V4 fac4{coef16, coef16, coef18, coef19}, fac5{coef20, coef20, coef22, coef23};
    const V4 vec0{m10, m00, m00, m00}, vec1{m11, m01, m01, m01}, vec2{m12, m02, m02, m02}, vec3{m13, m03, m03, m03};
    auto lane = [](V4 a, V4 b) { return V4{a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; };
    auto sub = [](V4 a, V4 b) { return V4{a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; };
    const V4 inv0 = sub(lane(vec1, fac0), lane(vec2, fac1)) + lane(vec3, fac2);
    const V4 inv1 = sub(lane(vec0, fac0), lane(vec2, fac3)) + lane(vec3, fac4);
    const V4 inv2 = sub(lane(vec0, fac1), lane(vec1, fac3)) + lane(vec3, fac5);
    const V4 inv3 = sub(lane(vec0, fac2), lane(vec1, fac4)) + lane(vec2, fac5);
    const V4 sa{1.0f, -1.0f, 1.0f, -1.0f}, sb{-1.0f, 1.0f, -1.0f, 1.0f};
    M4 r;
    r.c[0] = lane(inv0, sa);
    r.c[1] = lane(inv1, sb);
    r.c[2] = lane(inv2, sa);
    r.c[3] = lane(inv3, sb);
    const V4 col0{r.c[0].x, r.c[1].x, r.c[2].x, r.c[3].x};
    const float det = dot4(s.c[0], col0);
    const float rcp = 1.0f / det;
    for (int i = 0; i < 4; ++i) r.c[i] = r.c[i] * rcp;
    return r;
}
// Quat::from_rotation_{x,y,z}: (s, c) = sin_cos(angle * 0.5).
inline Q rot_x(float a) { return {std::sin(a * 0.5f), 0.0f, 0.0f, std::cos(a * 0.5f)}; }
inline Q rot_y(float a) { return {0.0f, std::sin(a * 0.5f), 0.0f, std::cos(a * 0.5f)}; }
inline Q rot_z(float a) { return {0.0f, 0.0f, std::sin(a * 0.5f), std::cos(a * 0.5f)}; }
// Quat * Quat, grouped as glam's SIMD backends add the four broadcast
// products: (a.w*b + a.x*(b.w,-b.z,b.y,-b.x)) + (a.y*(b.z,b.w,-b.x,-b.y) + a.z*(-b.y,b.x,b.w,-b.z)).
inline Q qmul(Q a, Q b) {
    Q r;
    r.x = (a.w * b.x + a.x * b.w) + (a.y * b.z + -(a.z * b.y));
    r.y = (a.w * b.y + -(a.x * b.z)) + (a.y * b.w + a.z * b.x);
    r.z = (a.w * b.z + a.x * b.y) + (-(a.y * b.x) + a.z * b.w);
    r.w = (a.w * b.w + -(a.x * b.x)) + (-(a.y * b.y) + -(a.z * b.z));
    return r;
}
// Quat * Vec3A: v*(w*w - b.b) + b*((b.v)*2) + (b x v)*(w*2).
inline V3 qrot(Q q, V3 v) {
    const V3 b{q.x, q.y, q.z};
    return (v * (q.w * q.w - dot(b, b)) + b * (dot(b, v) * 2.0f)) + cross(b, v) * (q.w * 2.0f);
}
// Mat4::from_quat.
M4 from_quat(Q q) {
    const float x2 = q.x + q.x, y2 = q.y + q.y, z2 = q.z + q.z;
    const float xx = q.x * x2, xy = q.x * y2, xz = q.x * z2;
    const float yy = q.y * y2, yz = q.y * z2, zz = q.z * z2;
    const float wx = q.w * x2, wy = q.w * y2, wz = q.w * z2;
    M4 m;
    m.c[0] = {1.0f - (yy + zz), xy + wz, xz - wy, 0.0f};
    m.c[1] = {xy - wz, 1.0f - (xx + zz), yz + wx, 0.0f};
    m.c[2] = {xz + wy, yz - wx, 1.0f - (xx + yy), 0.0f};
    m.c[3] = {0.0f, 0.0f, 0.0f, 1.0f};
    return m;
}
// Mat4::perspective_rh (depth in [0, 1]).
M4 perspective_rh(float fov, float aspect, float zn, float zf) {
    const float s = std::sin(0.5f * fov), c = std::cos(0.5f * fov);
    const float h = c / s, w = h / aspect, r = zf / (zn - zf);
    M4 m{};
    m.c[0] = {w, 0.0f, 0.0f, 0.0f};
    m.c[1] = {0.0f, h, 0.0f, 0.0f};
    m.c[2] = {0.0f, 0.0f, r, -1.0f};
    m.c[3] = {0.0f, 0.0f, r * zn, 0.0f};
    return m;
}
inline void store(const M4& m, float* out) { std::memcpy(out, &m, sizeof(m)); }

// ---------------------------------------------------------------- camera
// RenderCamera::new + update_matrices (src/rendercamera.rs:28-63, 78-150).
void camera_init(swr_camera* cam, V3 pos, V3 look_at, float fov, float width, float height, float far_plane) {
    std::memset(cam, 0, sizeof(*cam));
    const V3 fwd = normalize(look_at - pos);
    cam->position[0] = pos.x;
    cam->position[1] = pos.y;
    cam->position[2] = pos.z;
    cam->fov = fov;
    cam->width = width;
    cam->height = height;
    cam->one_over_width = 1.0f / width;
    cam->one_over_height = 1.0f / height;
    cam->near_plane = far_plane * 0.01f;
    cam->far_plane = far_plane;
    cam->yaw = std::atan2(fwd.x, -fwd.z);
    cam->pitch = std::asin(fwd.y);
    cam->roll = 0.0f;
    // get_rotation: roll * pitch * yaw.
    const Q rot = qmul(qmul(rot_z(cam->roll), rot_x(cam->pitch)), rot_y(cam->yaw));
    const M4 rm = from_quat(rot);
    M4 tr = identity();
    tr.c[3] = {-pos.x, -pos.y, -pos.z, 1.0f};
    const M4 view = mulm(rm, tr);
    const M4 proj = perspective_rh(fov, width / height, cam->near_plane, far_plane);
    const M4 vp = mulm(proj, view);
    store(view, cam->view);
    store(proj, cam->projection);
    store(vp, cam->view_project);
    store(inverse(vp), cam->inverse_view_project);
    store(transpose(inverse(mulm(proj, rm))), cam->skybox_transposed);
    // compute_view_clip_planes (src/rendercamera.rs:137-150).
    const float aspect = width / height;
    const float tan_y = std::tan(fov * 0.5f), tan_x = tan_y * aspect;
    const float planes[6][4] = {{0.0f, 0.0f, -1.0f, cam->near_plane}, {0.0f, 0.0f, 1.0f, far_plane}};
    std::memcpy(cam->view_clip_planes, planes, sizeof(planes));
    const V3 side[4] = {{1.0f, 0.0f, -tan_x}, {-1.0f, 0.0f, -tan_x}, {0.0f, 1.0f, -tan_y}, {0.0f, -1.0f, -tan_y}};
    for (int i = 0; i < 4; ++i) {
        const V3 n = normalize(side[i]);
        cam->view_clip_planes[2 + i][0] = n.x;
        cam->view_clip_planes[2 + i][1] = n.y;
        cam->view_clip_planes[2 + i][2] = n.z;
        cam->view_clip_planes[2 + i][3] = 0.0f;
    }
    const V3 vn = qrot(Q{-rot.x, -rot.y, -rot.z, rot.w}, V3{0.0f, 0.0f, 1.0f});
    cam->view_normal[0] = vn.x;
    cam->view_normal[1] = vn.y;
    cam->view_normal[2] = vn.z;
}

// ---------------------------------------------------------------- util.rs
// `as u32` of an f32: saturating, NaN -> 0.
inline uint32_t as_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}
// rgba8_unpack_vec4 / rgba8_pack_vec4 (src/util.rs:82-96). A channel whose
// value reaches 256 spills into the next channel's bits, as in the reference.
inline V4 unpack(uint32_t c) {
    return {(float)((c >> 24) & 0xFFu) / 255.0f, (float)((c >> 16) & 0xFFu) / 255.0f,
            (float)((c >> 8) & 0xFFu) / 255.0f, (float)(c & 0xFFu) / 255.0f};
}
inline uint32_t pack(V4 c) {
    return (as_u32(c.x * 255.0f) << 24) | (as_u32(c.y * 255.0f) << 16) | (as_u32(c.z * 255.0f) << 8) |
           as_u32(c.w * 255.0f);
}
// srgb_to_linear_scalar / linear_to_srgb_scalar (src/util.rs:49-78).
inline float srgb_to_linear(float s) {
    return s <= 0.04045f ? s / 12.92f : std::pow((s + 0.055f) / 1.055f, 2.4f);
}
inline float linear_to_srgb(float s) {
    return s <= 0.0031308f ? s * 12.92f : std::pow(s, 1.0f / 2.4f) * 1.055f - 0.055f;
}
inline float fmax0(float a) { return std::fmax(a, 0.0f); }
// f32::clamp: NaN passes through.
inline float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}


// ---------------------------------------------------------------- texture.rs
struct Tex {
    uint32_t width = 0, height = 0, type = 0, max_mip = 0;
    float whv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
    std::vector<uint32_t> data, offs, ws, hs, stride;
    swr_texture_view view() const {
        swr_texture_view v;
        std::memset(&v, 0, sizeof(v));
        v.width = width;
        v.height = height;
        v.type = type;
        v.mip_count = max_mip + 1;
        v.data = data.data();
        v.data_len = data.size();
        v.mip_offsets = offs.data();
        v.mip_widths = ws.data();
        v.mip_heights = hs.data();
        v.array_stride = stride.data();
        for (int i = 0; i < 4; ++i) v.width_height_vec[i] = whv[i];
        return v;
    }
};

// A texture as the loader creates it, before its mips (src/texture.rs:937-1005):
// width_height_vec = (w, w, h, h); cubemaps keep the six faces one after the
// other (array stride = face texels), 2D textures have array stride 0.
Tex make_tex(uint32_t w, uint32_t h, uint32_t type, const uint32_t* texels, uint32_t slices) {
    Tex t;
    t.width = w;
    t.height = h;
    t.type = type;
    t.whv[0] = (float)w;
    t.whv[1] = (float)w;
    t.whv[2] = (float)h;
    t.whv[3] = (float)h;
    t.data.assign(texels, texels + (size_t)w * h * slices);
    t.offs = {0u};
    t.ws = {w};
    t.hs = {h};
    t.stride = {slices > 1 ? w * h : 0u};
    return t;
}

inline uint32_t ilog2(uint32_t x) { return 31u - (uint32_t)__builtin_clz(x); }

// Texture::generate_mipmaps (src/texture.rs:45-128).
void generate_mipmaps(Tex& t) {
    const uint32_t num_mips = 1 + ilog2(std::max(t.width, t.height));
    const uint32_t slices = t.type == SWR_TEX_CUBEMAP ? 6u : 1u;
    for (uint32_t mip = 1; mip < num_mips; ++mip) {
        t.offs.push_back((uint32_t)t.data.size());
        const uint32_t mw = std::max(t.width >> mip, 1u), mh = std::max(t.height >> mip, 1u);
        t.stride.push_back(mw * mh);
        const uint32_t prev = t.offs[mip - 1], pw = t.ws[mip - 1], ph = t.hs[mip - 1], ps = t.stride[mip - 1];
        for (uint32_t slice = 0; slice < slices; ++slice) {
            const uint32_t so = prev + slice * ps;
            for (uint32_t y = 0; y < mh; ++y)
                for (uint32_t x = 0; x < mw; ++x) {
                    const uint32_t x0 = x * 2, y0 = y * 2;
                    const uint32_t x1 = std::min(x0 + 1, pw - 1), y1 = std::min(y0 + 1, ph - 1);
                    const V4 p00 = unpack(t.data[so + (y0 * pw + x0)]);
                    const V4 p10 = unpack(t.data[so + (y0 * pw + x1)]);
                    const V4 p01 = unpack(t.data[so + (y1 * pw + x0)]);
                    const V4 p11 = unpack(t.data[so + (y1 * pw + x1)]);
                    V4 avg;
                    if (t.type == SWR_TEX_SRGB) {
                        auto lin = [](V4 p) { return V4{srgb_to_linear(p.x), srgb_to_linear(p.y), srgb_to_linear(p.z), p.w}; };
                        const V4 l00 = lin(p00), l10 = lin(p10), l01 = lin(p01), l11 = lin(p11);
                        const V4 a = ((l00 + l10) + l01) + l11;
                        const V4 m{a.x / 4.0f, a.y / 4.0f, a.z / 4.0f, a.w / 4.0f};
                        avg = {linear_to_srgb(m.x), linear_to_srgb(m.y), linear_to_srgb(m.z), m.w};
                    } else if (t.type == SWR_TEX_METALLIC_ROUGHNESS) {
                        const float rough = (((p00.y * p00.y + p10.y * p10.y) + p01.y * p01.y) + p11.y * p11.y) / 4.0f;
                        const float metal = (((p00.z + p10.z) + p01.z) + p11.z) / 4.0f;
                        avg = {p00.x, std::sqrt(rough), metal, p00.w};
                    } else if (t.type == SWR_TEX_NORMAL) {
                        auto sn = [](V4 p) { return V4{p.x * 2.0f - 1.0f, p.y * 2.0f - 1.0f, p.z * 2.0f - 1.0f, p.w * 2.0f - 1.0f}; };
                        const V4 a = ((sn(p00) + sn(p10)) + sn(p01)) + sn(p11);
                        const V4 m{a.x / 4.0f, a.y / 4.0f, a.z / 4.0f, a.w / 4.0f};
                        avg = {(m.x + 1.0f) / 2.0f, (m.y + 1.0f) / 2.0f, (m.z + 1.0f) / 2.0f, (m.w + 1.0f) / 2.0f};
                    } else {
                        const V4 a = ((p00 + p10) + p01) + p11;
                        avg = {a.x / 4.0f, a.y / 4.0f, a.z / 4.0f, a.w / 4.0f};
                    }
                    t.data.push_back(pack(avg));
                }
        }
        t.ws.push_back(mw);
        t.hs.push_back(mh);
        t.max_mip += 1;
    }
}

// radical_inverse_vdc / hammersley (src/texture.rs:135-146).
inline float radical_inverse(uint32_t bits) {
    bits = (bits << 16) | (bits >> 16);
    bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
    bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
    bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
    bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
    return (float)bits * 2.3283064e-10f;
}
// importance_sample_ggx (src/texture.rs:148-165).
V3 sample_ggx(float xi_x, float xi_y, V3 n, float roughness) {
    const float a = roughness * roughness;
    const float phi = (2.0f * kPi) * xi_x;
    const float cos_t = std::sqrt((1.0f - xi_y) / (1.0f + (a * a - 1.0f) * xi_y));
    const float sin_t = std::sqrt(fmax0(1.0f - cos_t * cos_t));
    const V3 h{std::cos(phi) * sin_t, std::sin(phi) * sin_t, cos_t};
    const V3 up = std::fabs(n.z) < 0.999f ? V3{0.0f, 0.0f, 1.0f} : V3{1.0f, 0.0f, 0.0f};
    const V3 tangent = normalize(cross(n, up));
    const V3 bitangent = cross(n, tangent);
    return normalize((tangent * h.x + bitangent * h.y) + n * h.z);
}
// f32::powi(x, 5) as LLVM expands it: x * ((x*x)*(x*x)).
inline float powi5(float x) {
    const float x2 = x * x;
    return x * (x2 * x2);
}
// integrate_brdf (src/texture.rs:167-197).
void integrate_brdf(float ndotv, float roughness, float& ra, float& rb) {
    const V3 v{std::sqrt(fmax0(1.0f - ndotv * ndotv)), 0.0f, ndotv};
    const V3 n{0.0f, 0.0f, 1.0f};
    const uint32_t count = 128;
    float a = 0.0f, b = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        const V3 h = sample_ggx((float)i / (float)count, radical_inverse(i), n, roughness);
        const V3 l = normalize(h * (2.0f * dot(v, h)) - v);
        const float ndotl = fmax0(l.z), ndoth = fmax0(h.z), vdoth = fmax0(dot(v, h));
        if (ndotl > 0.0f) {
            const float alpha = roughness * roughness;
            const float k = ((alpha + 1.0f) * (alpha + 1.0f)) * 0.125f;
            const float gv = ndotv / (ndotv * (1.0f - k) + k);
            const float gl = ndotl / (ndotl * (1.0f - k) + k);
            const float gvis = fmax0(((gv * gl) * vdoth) / (ndoth * std::fmax(ndotv, 1.0e-5f)));
            const float fc = powi5(1.0f - vdoth);
            a += (1.0f - fc) * gvis;
            b += fc * gvis;
        }
    }
    ra = a / (float)count;
    rb = b / (float)count;
}
// generate_brdf_lut (src/texture.rs:199-238): width_height_vec = size x 4.
Tex brdf_lut(uint32_t size, unsigned threads) {
    std::vector<uint32_t> texels((size_t)size * size);
    const float sf = (float)size;
    par(size, threads, [&](size_t y) {
        const float rough = clampf(((float)y + 0.5f) / sf, 0.0f, 1.0f);
        for (uint32_t x = 0; x < size; ++x) {
            const float ndotv = clampf(((float)x + 0.5f) / sf, 0.0f, 1.0f);
            float a, b;
            integrate_brdf(std::fmax(ndotv, 1.0e-4f), std::fmax(rough, 1.0e-4f), a, b);
            texels[y * size + x] = pack(V4{clampf(a, 0.0f, 1.0f), clampf(b, 0.0f, 1.0f), 0.0f, 1.0f});
        }
    });
    Tex t = make_tex(size, size, SWR_TEX_LINEAR, texels.data(), 1);
    t.whv[1] = sf;
    t.whv[2] = sf;
    generate_mipmaps(t);
    return t;
}
// cubemap_face_uv_to_direction (src/texture.rs:240-250).
V3 face_dir(uint32_t face, float u, float v) {
    V3 d;
    switch (face) {
        case 0: d = {1.0f, -v, -u}; break;
        case 1: d = {-1.0f, -v, u}; break;
        case 2: d = {u, 1.0f, v}; break;
        case 3: d = {u, -1.0f, -v}; break;
        case 4: d = {u, -v, 1.0f}; break;
        default: d = {-u, -v, -1.0f}; break;
    }
    return normalize(d);
}
// cubemap_direction_to_face_uv (src/texture.rs:252-271).
void dir_face(V3 n, uint32_t& face, float& u, float& v) {
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
// TextureAndSampler::sample_bilinear_rgb (src/texture.rs:730-790), one lane,
// mip 0, ClampToEdge on both axes (min(texel, dim - 1), then the saturating
// `as u32` of a negative texel gives 0).
V3 bilinear(const Tex& t, float u, float v, uint32_t slice) {
    const uint32_t wi = t.ws[0];
    const float wf = (float)t.ws[0], hf = (float)t.hs[0];
    const uint32_t off = t.offs[0] + slice * t.stride[0];
    const float xf = u * wf - 0.5f, yf = v * hf - 0.5f;
    const float x0 = std::floor(xf), y0 = std::floor(yf);
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const float fx = xf - x0, fy = yf - y0, ofx = 1.0f - fx, ofy = 1.0f - fy;
    const uint32_t ix0 = as_u32(std::fmin(x0, wf - 1.0f)), iy0 = as_u32(std::fmin(y0, hf - 1.0f));
    const uint32_t ix1 = as_u32(std::fmin(x1, wf - 1.0f)), iy1 = as_u32(std::fmin(y1, hf - 1.0f));
    const V4 p00 = unpack(t.data[off + iy0 * wi + ix0]), p10 = unpack(t.data[off + iy0 * wi + ix1]);
    const V4 p01 = unpack(t.data[off + iy1 * wi + ix0]), p11 = unpack(t.data[off + iy1 * wi + ix1]);
    const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
    return {((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11,
            ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11,
            ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11};
}
// sample_cubemap_direction_linear (src/texture.rs:273-287).
V3 sample_dir(const Tex& cube, V3 d) {
    uint32_t face;
    float u, v;
    dir_face(d, face, u, v);
    const V3 s = bilinear(cube, clampf(u, 0.0f, 1.0f), clampf(v, 0.0f, 1.0f), face);
    return {srgb_to_linear(s.x), srgb_to_linear(s.y), srgb_to_linear(s.z)};
}
// compute_irradiance_sh4 (src/texture.rs:289-328).
void irradiance_sh4(const Tex& cube, float out[4][3]) {
    V3 sh[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    const float w = (float)cube.width, h = (float)cube.height;
    const float omega = (2.0f / w) * (2.0f / h);
    for (uint32_t face = 0; face < 6; ++face)
        for (uint32_t y = 0; y < cube.height; ++y) {
            const float v = (((float)y + 0.5f) / h) * 2.0f - 1.0f;
            for (uint32_t x = 0; x < cube.width; ++x) {
                const float u = (((float)x + 0.5f) / w) * 2.0f - 1.0f;
                const V3 d = face_dir(face, u, v);
                const float weight = omega / std::pow((1.0f + u * u) + v * v, 1.5f);
                const V3 c = sample_dir(cube, d);
                const float basis[4] = {0.282095f, 0.488603f * d.y, 0.488603f * d.z, 0.488603f * d.x};
                for (int i = 0; i < 4; ++i) sh[i] = sh[i] + c * (basis[i] * weight);
            }
        }
    sh[0] = sh[0] * kPi;
    const float band1 = (2.0f * kPi) / 3.0f;
    for (int i = 1; i < 4; ++i) sh[i] = sh[i] * band1;
    sh[0] = sh[0] * 0.282095f;
    for (int i = 1; i < 4; ++i) sh[i] = sh[i] * 0.488603f;
    for (int i = 0; i < 4; ++i) {
        out[i][0] = sh[i].x;
        out[i][1] = sh[i].y;
        out[i][2] = sh[i].z;
    }
}
// generate_prefiltered_specular_cubemap (src/texture.rs:330-420): every mip
// at full face size, roughness = mip / max_mip, width_height_vec (w, w, h, h).
Tex prefiltered_specular(const Tex& cube, uint32_t samples, unsigned threads) {
    const uint32_t bw = cube.width, bh = cube.height;
    const uint32_t num_mips = 1 + ilog2(std::max(bw, bh)), max_mip = num_mips - 1;
    Tex t;
    t.width = bw;
    t.height = bh;
    t.type = SWR_TEX_LINEAR;
    t.max_mip = max_mip;
    t.whv[0] = (float)bw;
    t.whv[1] = (float)bw;
    t.whv[2] = (float)bh;
    t.whv[3] = (float)bh;
    const size_t face_texels = (size_t)bw * bh;
    t.data.resize(face_texels * 6 * num_mips);
    for (uint32_t mip = 0; mip < num_mips; ++mip) {
        t.offs.push_back((uint32_t)(face_texels * 6 * mip));
        t.ws.push_back(bw);
        t.hs.push_back(bh);
        t.stride.push_back(bw * bh);
    }
    par((size_t)num_mips * 6 * bh, threads, [&](size_t row) {
        const uint32_t mip = (uint32_t)(row / (6 * (size_t)bh));
        const uint32_t face = (uint32_t)((row / bh) % 6), y = (uint32_t)(row % bh);
        const float rough = max_mip > 0 ? (float)mip / (float)max_mip : 0.0f;
        const float v = (((float)y + 0.5f) / (float)bh) * 2.0f - 1.0f;
        for (uint32_t x = 0; x < bw; ++x) {
            const float u = (((float)x + 0.5f) / (float)bw) * 2.0f - 1.0f;
            const V3 r = face_dir(face, u, v);
            V3 color;
            if (mip == 0) {
                color = sample_dir(cube, r);
            } else {
                V3 acc{0.0f, 0.0f, 0.0f};
                float total = 0.0f;
                for (uint32_t i = 0; i < samples; ++i) {
                    const V3 h = sample_ggx((float)i / (float)samples, radical_inverse(i), r, std::fmax(rough, 0.045f));
                    const V3 l = normalize(h * (2.0f * dot(r, h)) - r);
                    const float ndotl = fmax0(dot(r, l));
                    if (ndotl > 0.0f) {
                        acc = acc + sample_dir(cube, l) * ndotl;
                        total += ndotl;
                    }
                }
                color = total > 0.0f ? acc / total : sample_dir(cube, r);
            }
            t.data[face_texels * 6 * mip + face * face_texels + (size_t)y * bw + x] = pack(V4{color.x, color.y, color.z, 1.0f});
        }
    });
    return t;
}

// ---------------------------------------------------------------- scene.rs
struct Prim {
    std::vector<float> pos4, nrm4, tan4, uv2;
    std::vector<uint32_t> idx;
    uint32_t material = 0, tri_base = 0;
    float sphere[4] = {0, 0, 0, 0};
};
struct Mesh {
    std::vector<uint32_t> prims, opaque, translucent;
    uint32_t tris = 0;
};

// compute_bounding_sphere (src/scene.rs:513-525): midpoint = (min+max)*0.5.
void bounding_sphere(const std::vector<float>& pos4, float out[4]) {
    V3 mn{INFINITY, INFINITY, INFINITY}, mx{-INFINITY, -INFINITY, -INFINITY};
    for (size_t v = 0; v < pos4.size(); v += 4) {
        mn = {std::fmin(mn.x, pos4[v]), std::fmin(mn.y, pos4[v + 1]), std::fmin(mn.z, pos4[v + 2])};
        mx = {std::fmax(mx.x, pos4[v]), std::fmax(mx.y, pos4[v + 1]), std::fmax(mx.z, pos4[v + 2])};
    }
    const V3 c = (mn + mx) * 0.5f;
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    out[3] = length(mx - mn) / 2.0f;
}
// compute_smooth_normals (src/scene.rs:527-557).
void smooth_normals(const std::vector<float>& pos4, const std::vector<uint32_t>& idx, std::vector<float>& nrm4) {
    const size_t nv = pos4.size() / 4;
    std::vector<V3> acc(nv, V3{0.0f, 0.0f, 0.0f});
    auto p = [&](uint32_t i) { return V4{pos4[4 * (size_t)i], pos4[4 * (size_t)i + 1], pos4[4 * (size_t)i + 2], pos4[4 * (size_t)i + 3]}; };
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const V4 v0 = p(idx[t]), v1 = p(idx[t + 1]), v2 = p(idx[t + 2]);
        const V3 e1{v1.x - v0.x, v1.y - v0.y, v1.z - v0.z}, e2{v2.x - v0.x, v2.y - v0.y, v2.z - v0.z};
        const V3 fn = cross(e1, e2);
        for (int k = 0; k < 3; ++k) acc[idx[t + k]] = acc[idx[t + k]] + fn;
    }
    nrm4.assign(nv * 4, 0.0f);
    for (size_t v = 0; v < nv; ++v) {
        const V3 n = dot(acc[v], acc[v]) > 0.0f ? normalize(acc[v]) : V3{0.0f, 0.0f, 1.0f};
        nrm4[4 * v] = n.x;
        nrm4[4 * v + 1] = n.y;
        nrm4[4 * v + 2] = n.z;
    }
}
// compute_tangents (src/scene.rs:559-635), glam's scalar Vec3 throughout.
void tangents(const std::vector<float>& pos4, const std::vector<float>& uv2, const std::vector<float>& nrm4,
              const std::vector<uint32_t>& idx, std::vector<float>& tan4) {
    const size_t nv = pos4.size() / 4;
    std::vector<V3> ta(nv, V3{0.0f, 0.0f, 0.0f}), ba(nv, V3{0.0f, 0.0f, 0.0f});
    auto P = [&](uint32_t i) { return V3{pos4[4 * (size_t)i], pos4[4 * (size_t)i + 1], pos4[4 * (size_t)i + 2]}; };
    for (size_t t = 0; t + 2 < idx.size(); t += 3) {
        const uint32_t i0 = idx[t], i1 = idx[t + 1], i2 = idx[t + 2];
        const V3 e1 = P(i1) - P(i0), e2 = P(i2) - P(i0);
        const float du1 = uv2[2 * (size_t)i1] - uv2[2 * (size_t)i0], dv1 = uv2[2 * (size_t)i1 + 1] - uv2[2 * (size_t)i0 + 1];
        const float du2 = uv2[2 * (size_t)i2] - uv2[2 * (size_t)i0], dv2 = uv2[2 * (size_t)i2 + 1] - uv2[2 * (size_t)i0 + 1];
        const float det = du1 * dv2 - du2 * dv1;
        if (std::fabs(det) < 1e-6f) continue;
        const V3 tg = (e1 * dv2 - e2 * dv1) / det;
        const V3 bt = (e2 * du1 - e1 * du2) / det;
        ta[i0] = ta[i0] + tg;
        ta[i1] = ta[i1] + tg;
        ta[i2] = ta[i2] + tg;
        ba[i0] = ba[i0] + bt;
        ba[i1] = ba[i1] + bt;
        ba[i2] = ba[i2] + bt;
    }
    tan4.assign(nv * 4, 0.0f);
    for (size_t v = 0; v < nv; ++v) {
        const V3 n{nrm4[4 * v], nrm4[4 * v + 1], nrm4[4 * v + 2]};
        const V3 t = ta[v];
        float o[4];
        if (dot(t, t) < 1e-6f) {
            const V3 helper = std::fabs(n.x) > 0.9f ? V3{0.0f, 1.0f, 0.0f} : V3{1.0f, 0.0f, 0.0f};
            const V3 tg = normalize(cross(n, helper));
            o[0] = tg.x, o[1] = tg.y, o[2] = tg.z, o[3] = 1.0f;
        } else {
            const V3 tg = normalize(t - n * dot(n, t));
            const float hand = dot(cross(n, tg), ba[v]) < 0.0f ? -1.0f : 1.0f;
            o[0] = tg.x, o[1] = tg.y, o[2] = tg.z, o[3] = hand;
        }
        std::memcpy(&tan4[4 * v], o, sizeof(o));
    }
}

struct Scene {
    std::vector<Prim> prims;
    std::vector<Mesh> meshes;
    std::vector<swr_node_view> nodes;
    std::vector<swr_material_view> materials;
    std::vector<Tex> textures;
    Tex cubemap, specular, lut;
    std::vector<float> light, sh4;
    std::vector<swr_primitive_view> pv;
    std::vector<swr_mesh_view> mv;
    std::vector<swr_texture_view> tv;
    float bmin[3], bmax[3], center[3], diagonal;
    swr_scene_host_view view;
};

// Scene::from_gltf's processing of an already flattened descriptor
// (src/scene.rs:145-351), the light (src/scene.rs:236-239), and load_scene's
// voxel grid (src/main.rs:226-281: grid over the scene bounds, sun
// visibility, then initialize_voxel_gi_from_scene, src/gi.rs:123-149, or
// with the GI flag the bake). Returns 0, or 1 for a descriptor that indexes
// out of range.
int build(const swr_scene_desc* d, unsigned threads, Scene& s) {
    // Material::from_gltf (src/scene.rs:690-780): alpha test only with a
    // base-colour texture; a transmission extension makes the material
    // translucent and is the only source of the transmission factor and
    // texture; occlusion strength only with an occlusion texture.
    for (uint32_t i = 0; i < d->material_count; ++i) {
        const swr_material_desc& m = d->materials[i];
        swr_material_view v;
        std::memset(&v, 0, sizeof(v));
        std::memcpy(v.base_color_factor, m.base_color_factor, sizeof(v.base_color_factor));
        v.metallic_factor = m.metallic_factor;
        v.roughness_factor = m.roughness_factor;
        std::memcpy(v.emissive_factor, m.emissive_factor, sizeof(v.emissive_factor));
        v.alpha_cutoff = m.alpha_cutoff;
        const swr_texref refs[6] = {m.base_color, m.metallic_roughness, m.normal, m.emissive, m.occlusion,
                                    m.has_transmission ? m.transmission_texture : swr_texref{-1, 0, 0, 0}};
        for (int k = 0; k < 6; ++k) {
            if (refs[k].texture >= (int32_t)d->texture_count) return 1;
            v.tex[k] = refs[k].texture < 0 ? -1 : refs[k].texture;
            v.wrap_s[k] = refs[k].wrap_s;
            v.wrap_t[k] = refs[k].wrap_t;
        }
        v.occlusion_strength = v.tex[4] >= 0 ? m.occlusion_strength : 1.0f;
        v.transmission = m.has_transmission ? m.transmission : 0.0f;
        v.is_alpha_tested = (m.alpha_mask && v.tex[0] >= 0) ? 1u : 0u;
        v.is_translucent = m.has_transmission ? 1u : 0u;
        s.materials.push_back(v);
    }
    for (uint32_t i = 0; i < d->texture_count; ++i) {
        const swr_texture_desc& t = d->textures[i];
        s.textures.push_back(make_tex(t.width, t.height, t.type, t.rgba8, 1));
    }
    par(s.textures.size(), threads, [&](size_t i) { generate_mipmaps(s.textures[i]); });
    // Mesh::from_gltf / Primitive::from_gltf (src/scene.rs:422-495).
    for (uint32_t mi = 0; mi < d->mesh_count; ++mi) {
        const swr_mesh_desc& md = d->meshes[mi];
        Mesh mesh;
        for (uint32_t pi = 0; pi < md.primitive_count; ++pi) {
            const swr_primitive_desc& pd = md.primitives[pi];
            Prim p;
            const size_t nv = pd.vertex_count;
            p.pos4.resize(nv * 4);
            for (size_t v = 0; v < nv; ++v) {
                for (int k = 0; k < 3; ++k) p.pos4[4 * v + k] = pd.positions[3 * v + k];
                p.pos4[4 * v + 3] = 1.0f;
            }
            p.idx.assign(pd.indices, pd.indices + pd.index_count);
            for (uint32_t k : p.idx)
                if (k >= pd.vertex_count) return 1;
            p.uv2.assign(nv * 2, 0.0f);
            if (pd.texcoords) std::memcpy(p.uv2.data(), pd.texcoords, nv * 2 * sizeof(float));
            if (pd.normals) {
                p.nrm4.assign(nv * 4, 0.0f);
                for (size_t v = 0; v < nv; ++v)
                    for (int k = 0; k < 3; ++k) p.nrm4[4 * v + k] = pd.normals[3 * v + k];
            } else {
                smooth_normals(p.pos4, p.idx, p.nrm4);
            }
            if (pd.tangents) p.tan4.assign(pd.tangents, pd.tangents + nv * 4);
            else tangents(p.pos4, p.uv2, p.nrm4, p.idx, p.tan4);
            bounding_sphere(p.pos4, p.sphere);
            p.material = pd.material < 0 ? 0u : (uint32_t)pd.material;
            if (p.material >= d->material_count) return 1;
            // Static triangle IDs of the visibility buffer: within a mesh,
            // primitives number their triangles one after the other.
            p.tri_base = mesh.tris;
            mesh.tris += pd.index_count / 3;
            mesh.prims.push_back((uint32_t)s.prims.size());
            (s.materials[p.material].is_translucent ? mesh.translucent : mesh.opaque).push_back(pi);
            s.prims.push_back(std::move(p));
        }
        s.meshes.push_back(std::move(mesh));
    }
    // Nodes (src/scene.rs:286-331, 384-394): the sphere starts at the local
    // transform's origin with radius 0 and grows by every primitive's sphere
    // under the world transform (Mat4 * &BoundingSphere, src/scene.rs:53-63).
    uint32_t tri_base = 0;
    for (uint32_t ni = 0; ni < d->node_count; ++ni) {
        const swr_node_desc& nd = d->nodes[ni];
        if (nd.mesh >= (int32_t)d->mesh_count) return 1;
        swr_node_view v;
        std::memset(&v, 0, sizeof(v));
        std::memcpy(v.transform, nd.world, sizeof(v.transform));
        const M4 world = mat(nd.world);
        const V4 o = mulv(mat(nd.local), V4{0.0f, 0.0f, 0.0f, 1.0f});
        V3 c{o.x, o.y, o.z};
        float r = 0.0f;
        v.mesh = nd.mesh;
        v.triangle_id_base = tri_base;
        if (nd.mesh >= 0) {
            const Mesh& mesh = s.meshes[nd.mesh];
            const float scale = ((length4(world.c[0]) + length4(world.c[1])) + length4(world.c[2])) / 3.0f;
            for (uint32_t gp : mesh.prims) {
                const float* ps = s.prims[gp].sphere;
                const V3 wc = transform_point3a(world, V3{ps[0], ps[1], ps[2]});
                const float wr = ps[3] * scale;
                const float dist = length(c - wc);
                if (dist + wr > r) r = dist + wr;
            }
            tri_base += mesh.tris;
        }
        v.sphere[0] = c.x;
        v.sphere[1] = c.y;
        v.sphere[2] = c.z;
        v.sphere[3] = r;
        s.nodes.push_back(v);
    }
    // Scene bounds (src/scene.rs:333-351, SceneBounds::grow :835-846).
    V3 mn{INFINITY, INFINITY, INFINITY}, mx{-INFINITY, -INFINITY, -INFINITY};
    for (const swr_node_view& n : s.nodes) {
        if (n.mesh < 0) continue;
        const M4 w = mat(n.transform);
        for (uint32_t gp : s.meshes[n.mesh].prims) {
            const Prim& p = s.prims[gp];
            for (size_t v = 0; v < p.pos4.size(); v += 4) {
                const V4 t = mulv(w, V4{p.pos4[v], p.pos4[v + 1], p.pos4[v + 2], 1.0f});
                mn = {std::fmin(mn.x, t.x), std::fmin(mn.y, t.y), std::fmin(mn.z, t.z)};
                mx = {std::fmax(mx.x, t.x), std::fmax(mx.y, t.y), std::fmax(mx.z, t.z)};
            }
        }
    }
    const V3 ctr = (mn + mx) * 0.5f;
    s.bmin[0] = mn.x, s.bmin[1] = mn.y, s.bmin[2] = mn.z;
    s.bmax[0] = mx.x, s.bmax[1] = mx.y, s.bmax[2] = mx.z;
    s.center[0] = ctr.x, s.center[1] = ctr.y, s.center[2] = ctr.z;
    s.diagonal = length(mx - mn);
    // Environment (src/scene.rs:152-228): the cubemap with its mips, the
    // GGX-prefiltered copy, irradiance SH4, the BRDF LUT.
    s.cubemap = make_tex(d->cubemap_face_size, d->cubemap_face_size, SWR_TEX_CUBEMAP, d->cubemap_faces, 6);
    generate_mipmaps(s.cubemap);
    s.specular = prefiltered_specular(s.cubemap, d->specular_samples ? d->specular_samples : 64u, threads);
    s.lut = brdf_lut(d->brdf_lut_size ? d->brdf_lut_size : 128u, threads);
    // Views.
    for (const Prim& p : s.prims) {
        swr_primitive_view v;
        std::memset(&v, 0, sizeof(v));
        v.vertex_count = (uint32_t)(p.pos4.size() / 4);
        v.index_count = (uint32_t)p.idx.size();
        v.positions = p.pos4.data();
        v.normals = p.nrm4.data();
        v.tangents = p.tan4.data();
        v.texcoords = p.uv2.data();
        v.indices = p.idx.data();
        v.material = p.material;
        v.triangle_id_base = p.tri_base;
        std::memcpy(v.sphere, p.sphere, sizeof(v.sphere));
        s.pv.push_back(v);
    }
    for (const Mesh& m : s.meshes) {
        swr_mesh_view v;
        std::memset(&v, 0, sizeof(v));
        v.primitive_count = (uint32_t)m.prims.size();
        v.opaque_count = (uint32_t)m.opaque.size();
        v.translucent_count = (uint32_t)m.translucent.size();
        v.primitives = m.prims.data();
        v.opaque = m.opaque.data();
        v.translucent = m.translucent.data();
        s.mv.push_back(v);
    }
    for (const Tex& t : s.textures) s.tv.push_back(t.view());
    swr_scene_host_view& o = s.view;
    std::memset(&o, 0, sizeof(o));
    o.primitive_count = (uint32_t)s.prims.size();
    o.mesh_count = (uint32_t)s.meshes.size();
    o.node_count = (uint32_t)s.nodes.size();
    o.material_count = (uint32_t)s.materials.size();
    o.texture_count = (uint32_t)s.textures.size();
    o.primitives = s.pv.data();
    o.meshes = s.mv.data();
    o.nodes = s.nodes.data();
    o.materials = s.materials.data();
    o.textures = s.tv.data();
    o.cubemap = s.cubemap.view();
    o.cubemap_specular = s.specular.view();
    o.brdf_lut = s.lut.view();
    irradiance_sh4(s.cubemap, o.irradiance_sh);
    const V3 ld = normalize(V3{-0.2f, 1.0f, 0.5f});
    const V3 lc = V3{1.0f, 1.0f, 0.95f} * 5.0f;
    o.light_direction[0] = ld.x, o.light_direction[1] = ld.y, o.light_direction[2] = ld.z;
    o.light_color[0] = lc.x, o.light_color[1] = lc.y, o.light_color[2] = lc.z;
    const uint32_t n = d->voxel_grid_size ? d->voxel_grid_size : 128u;
    o.voxel_size = n;
    std::memcpy(o.voxel_world_min, s.bmin, sizeof(s.bmin));
    std::memcpy(o.voxel_world_max, s.bmax, sizeof(s.bmax));
    s.light.assign((size_t)n * n * n, 0.0f);
    if (oracle_sun_visibility(&o, threads, s.light.data()) != 0) return 1;
    o.voxel_light_intensity = s.light.data();
    for (int i = 0; i < 4; ++i) {
        for (int c = 0; c < 3; ++c) o.voxel_gi_sh4_const[i][c] = o.irradiance_sh[i][c] * d->gi_sh_scale;
        o.voxel_gi_sh4_const[i][3] = 0.0f;
    }
    o.voxel_gi_sh4_const[1][3] = d->sky_visibility;
    if (d->flags & SWR_SCENE_GI) {
        s.sh4.assign((size_t)n * n * n * 16, 0.0f);
        if (oracle_gi_bake(&o, threads, s.sh4.data()) != 0) return 1;
        o.voxel_gi_sh4 = s.sh4.data();
    }
    return 0;
}

}  // namespace ors

extern "C" {

// Builds the processed scene of a descriptor (see ors::build) with `threads`
// host threads (0 = all cores). *out receives a handle for
// oracle_scene_free; *view the host view, valid until then.
int oracle_scene_build(const swr_scene_desc* desc, uint32_t threads, swr_scene_host_view* view, void** out) {
    if (!desc || !view || !out || desc->material_count == 0 || !desc->cubemap_faces || desc->cubemap_face_size == 0)
        return 1;
    unsigned th = threads ? threads : std::max(1u, std::thread::hardware_concurrency());
    ors::Scene* s = new ors::Scene();
    if (ors::build(desc, th, *s) != 0) {
        delete s;
        return 1;
    }
    *view = s->view;
    *out = s;
    return 0;
}

// Scene bounds (min, max, centre, diagonal) of a built scene: what the
// reference's load_scene places its default camera from (src/main.rs:212-224).
void oracle_scene_bounds(const void* scene, float out[10]) {
    const ors::Scene* s = (const ors::Scene*)scene;
    std::memcpy(out, s->bmin, 3 * sizeof(float));
    std::memcpy(out + 3, s->bmax, 3 * sizeof(float));
    std::memcpy(out + 6, s->center, 3 * sizeof(float));
    out[9] = s->diagonal;
}

void oracle_scene_free(void* scene) { delete (ors::Scene*)scene; }

// Node::get_local_transform (src/scene.rs:396-419): the glTF matrix (column
// major) when `matrix` is not NULL, else Mat4::from_translation(t) *
// Mat4::from_quat(r) * Mat4::from_scale(s), multiplied left to right.
void oracle_node_local(const float t[3], const float r[4], const float s[3], const float* matrix, float out[16]) {
    using namespace ors;
    if (matrix) {
        std::memcpy(out, matrix, 16 * sizeof(float));
        return;
    }
    M4 tm = identity();
    tm.c[3] = {t[0], t[1], t[2], 1.0f};
    M4 sm{};
    sm.c[0].x = s[0];
    sm.c[1].y = s[1];
    sm.c[2].z = s[2];
    sm.c[3].w = 1.0f;
    store(mulm(mulm(tm, from_quat(Q{r[0], r[1], r[2], r[3]})), sm), out);
}

// Mat4 * Mat4 (compute_final_transform_recursive: parent * local, with the
// identity as the roots' parent, src/scene.rs:356-381).
void oracle_mat4_mul(const float a[16], const float b[16], float out[16]) {
    using namespace ors;
    store(mulm(mat(a), mat(b)), out);
}

// RenderCamera::new followed by update_matrices (src/rendercamera.rs:28-150).
int oracle_camera_init(swr_camera* cam, const float position[3], const float look_at[3], float fov, float width,
                       float height, float far_plane) {
    if (!cam || !position || !look_at) return 1;
    ors::camera_init(cam, ors::V3{position[0], position[1], position[2]}, ors::V3{look_at[0], look_at[1], look_at[2]},
                     fov, width, height, far_plane);
    return 0;
}

}  // extern "C"
