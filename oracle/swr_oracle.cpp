// CPU oracle for the per-frame rasterization path of swraster-viewer.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++, the reference's
// per-frame path (Renderer::render_scene + update_auto_exposure +
// blit_to_buffer) so tests can check the CUDA kernels against it. Nothing in
// the product links, imports or calls it; only tests/, the smoke check and
// bench.py's CPU-baseline leg do.
//
// Parity status: unpinned against the reference binary. The reference is
// Rust; no Rust toolchain or vendored crates exist here, so it cannot be run
// and it ships no tests or golden images. Fidelity is argued line by line
// (every function cites the reference file:line it follows) and pinned where
// possible by known-answer tests derived from the reference's formulas and by
// checking the Arm FRSQRTE/FRSQRTS emulation against the real instructions on
// an aarch64 host.
//
// Structure follows the reference: 4-wide "Vec4" lanes are float[4] with
// per-lane IEEE operations in the reference's order (glam never fuses a
// multiply and an add; this file must be compiled with -ffp-contract=off),
// tiles of 64x64 pixels hold 2x2-quad buffers (color, depth, packet index,
// barycentrics), packets are queued per tile in the canonical sequential order
// (node rank after the stable distance sort, primitive — a mesh's opaque
// primitives before its translucent ones — triangle, fan) when run
// single-threaded, and in rayon-like nondeterministic order when run
// multi-threaded (the timed CPU baseline). Translucent packets are sorted back
// to front per tile by average clip z, equal keys in queue order.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "../include/swr.h"

namespace orc {

// ---------------------------------------------------------------- lanes
struct F4 {
    float l[4];
};
static inline F4 splat(float v) { return {{v, v, v, v}}; }
static inline F4 mk(float a, float b, float c, float d) { return {{a, b, c, d}}; }
#define LANEWISE(op)                                                                           \
    static inline F4 operator op(F4 a, F4 b) {                                                 \
        return {{a.l[0] op b.l[0], a.l[1] op b.l[1], a.l[2] op b.l[2], a.l[3] op b.l[3]}};   \
    }
LANEWISE(+)
LANEWISE(-)
LANEWISE(*)
LANEWISE(/)
#undef LANEWISE
static inline F4 operator+(F4 a, float s) { return a + splat(s); }
static inline F4 operator-(F4 a, float s) { return a - splat(s); }
static inline F4 operator*(F4 a, float s) { return a * splat(s); }
static inline F4 operator+(float s, F4 a) { return splat(s) + a; }
static inline F4 operator-(float s, F4 a) { return splat(s) - a; }
static inline F4 operator/(float s, F4 a) { return splat(s) / a; }
// glam max/min/clamp with IEEE maxNum/minNum semantics (scalar f32::max).
static inline F4 vmax(F4 a, F4 b) {
    F4 r;
    for (int i = 0; i < 4; ++i) r.l[i] = std::fmax(a.l[i], b.l[i]);
    return r;
}
static inline F4 vmin(F4 a, F4 b) {
    F4 r;
    for (int i = 0; i < 4; ++i) r.l[i] = std::fmin(a.l[i], b.l[i]);
    return r;
}
static inline F4 vclamp(F4 v, F4 lo, F4 hi) { return vmin(vmax(v, lo), hi); }
static inline F4 vfloor(F4 a) {
    F4 r;
    for (int i = 0; i < 4; ++i) r.l[i] = std::floor(a.l[i]);
    return r;
}
static inline F4 vround(F4 a) {
    F4 r;
    for (int i = 0; i < 4; ++i) r.l[i] = std::round(a.l[i]);
    return r;
}
typedef bool B4[4];

struct V3x4 {
    F4 x, y, z;
};
static inline V3x4 operator+(V3x4 a, V3x4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3x4 operator-(V3x4 a, V3x4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3x4 operator*(V3x4 a, V3x4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
static inline V3x4 operator*(V3x4 a, F4 s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3x4 operator*(V3x4 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline V3x4 operator-(V3x4 a, float s) { return {a.x - s, a.y - s, a.z - s}; }
static inline V3x4 operator+(V3x4 a, float s) { return {a.x + s, a.y + s, a.z + s}; }
static inline V3x4 operator/(V3x4 a, V3x4 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
static inline V3x4 v3splat(float v) { return {splat(v), splat(v), splat(v)}; }
static inline V3x4 v3f(float x, float y, float z) { return {splat(x), splat(y), splat(z)}; }
// Vec3x4::dot (src/math.rs:88-90).
static inline F4 dot(V3x4 a, V3x4 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3x4 cross(V3x4 a, V3x4 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
static inline V3x4 v3select(const B4 m, V3x4 a, V3x4 b) {
    V3x4 r;
    for (int i = 0; i < 4; ++i) {
        r.x.l[i] = m[i] ? a.x.l[i] : b.x.l[i];
        r.y.l[i] = m[i] ? a.y.l[i] : b.y.l[i];
        r.z.l[i] = m[i] ? a.z.l[i] : b.z.l[i];
    }
    return r;
}

// ---------------------------------------------------------------- rsqrt
// Arm FRSQRTE (FPRSqrtEstimate, FPCR.AH = 0, no increased precision) and
// FRSQRTS (FPRSqrtStepFused), restated from the Arm Architecture Reference
// Manual pseudocode.
static int recip_sqrt_estimate(int a) {
    if (a < 256) {
        a = a * 2 + 1;
    } else {
        a = (a >> 1) << 1;
        a = (a + 1) * 2;
    }
    long long b = 512;
    while ((long long)a * (b + 1) * (b + 1) < (1LL << 28)) b++;
    return (int)((b + 1) / 2);
}
static uint8_t g_est[512];
static std::once_flag g_est_once;
static void init_est() {
    for (int a = 128; a < 512; ++a) g_est[a] = (uint8_t)(recip_sqrt_estimate(a) & 0xFF);
}
static float frsqrte(float x) {
    std::call_once(g_est_once, init_est);
    uint32_t b;
    std::memcpy(&b, &x, 4);
    if (std::isnan(x)) {
        b |= 0x00400000u;
        float r;
        std::memcpy(&r, &b, 4);
        return r;
    }
    if (x == 0.0f) return std::copysign(INFINITY, x);
    if (b >> 31) return NAN;
    if (std::isinf(x)) return 0.0f;
    int e = (int)((b >> 23) & 0xFF);
    uint64_t frac = (uint64_t)(b & 0x7FFFFF) << 29;
    if (e == 0) {
        while (!((frac >> 51) & 1)) {
            frac <<= 1;
            e -= 1;
        }
        frac = (frac << 1) & ((1ULL << 52) - 1);
    }
    const int scaled = (e & 1) == 0 ? (int)(256 | (frac >> 44)) : (int)(128 | (frac >> 45));
    const int rexp = (380 - e) / 2;
    const uint32_t out = ((uint32_t)(rexp & 0xFF) << 23) | ((uint32_t)g_est[scaled] << 15);
    float r;
    std::memcpy(&r, &out, 4);
    return r;
}
static float frsqrts(float a, float b) {
    if (std::isnan(a)) return a;
    if (std::isnan(b)) return b;
    if ((std::isinf(a) && b == 0.0f) || (a == 0.0f && std::isinf(b))) return 1.5f;
    if (std::isinf(a) || std::isinf(b)) return (std::signbit(a) != std::signbit(b)) ? INFINITY : -INFINITY;
    // (3 - a*b) / 2 with one rounding: the product is exact in double, the
    // sum is rounded once by fmaf, halving is exact.
    return std::fmaf(-a, b, 3.0f) * 0.5f;
}
static int g_rsqrt_mode = SWR_RSQRT_AARCH64;
// rsqrt_vec (src/math.rs:17-49).
static F4 rsqrt_vec(F4 v) {
    F4 r;
    for (int i = 0; i < 4; ++i) {
        const float x = v.l[i];
        if (g_rsqrt_mode == SWR_RSQRT_AARCH64) {
            const float y0 = frsqrte(x);
            r.l[i] = y0 * frsqrts(x * y0, y0);
        } else {
            r.l[i] = 1.0f / std::sqrt(x);
        }
    }
    return r;
}
// Vec3x4::normalize (src/math.rs:101-108).
static inline V3x4 normalize(V3x4 a) {
    const F4 ol = rsqrt_vec((a.x * a.x + a.y * a.y) + a.z * a.z);
    return {a.x * ol, a.y * ol, a.z * ol};
}

// ---------------------------------------------------------------- casts
static inline uint32_t as_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)x;
}
static inline int32_t as_i32(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
static inline uint8_t as_u8(float x) {
    if (!(x > 0.0f)) return 0;
    if (x >= 255.0f) return 255;
    return (uint8_t)x;
}
static inline int32_t wsub(int32_t a, int32_t b) { return (int32_t)((uint32_t)a - (uint32_t)b); }
static inline int32_t wadd(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }
static inline int32_t wmul(int32_t a, int32_t b) { return (int32_t)((uint32_t)a * (uint32_t)b); }

// ---------------------------------------------------------------- util.rs
static inline float unorm(uint32_t c, int shift) { return (float)((c >> shift) & 0xFFu) / 255.0f; }
// srgb_to_linear_fast (src/util.rs:111-113).
static inline V3x4 srgb_fast(V3x4 x) { return x * (x * (x * 0.305306011f + 0.682171111f) + 0.012522878f); }
// tonemap (src/util.rs:37-41).
static inline V3x4 tonemap(V3x4 c) {
    const float k = 0.2f;
    return (c / (c + k)) * (1.0f + k);
}

// ScalarInterpolator / Vec3Interpolator (src/util.rs:149-194).
struct SI {
    float a, da, db;
    static SI from3(float x, float y, float z) { return {x, y - x, z - x}; }
    F4 interp(F4 b1, F4 b2) const { return (a + b1 * da) + b2 * db; }
};
struct VI {
    SI c[3];
    V3x4 interp(F4 b1, F4 b2) const { return {c[0].interp(b1, b2), c[1].interp(b1, b2), c[2].interp(b1, b2)}; }
};

// ---------------------------------------------------------------- texture.rs
struct Tex {
    const swr_texture_view* t;
    uint32_t wrap_s, wrap_t;
};
static inline float mipw(const swr_texture_view* t, uint32_t m) { return (float)t->mip_widths[m]; }
static inline float miph(const swr_texture_view* t, uint32_t m) { return (float)t->mip_heights[m]; }
// apply_wrap_mode (src/texture.rs:578-589).
static F4 apply_wrap(F4 texel, F4 dim, uint32_t mode) {
    F4 t = texel;
    if (mode == SWR_WRAP_REPEAT) {
        t = texel - vfloor(texel / dim) * dim;
    } else if (mode == SWR_WRAP_MIRRORED_REPEAT) {
        const F4 two = dim * 2.0f;
        const F4 m = texel - vfloor(texel / two) * two;
        t = vmin(m, two - m);
    }
    return vmin(t, dim - 1.0f);
}
// compute_mip_level (src/texture.rs:851-863).
static uint32_t compute_mip_level(const swr_texture_view* t, F4 du_dv) {
    const F4 d = du_dv * mk(t->width_height_vec[0], t->width_height_vec[1], t->width_height_vec[2],
                            t->width_height_vec[3]);
    const float dx2 = d.l[0] * d.l[0] + d.l[2] * d.l[2];
    const float dy2 = d.l[1] * d.l[1] + d.l[3] * d.l[3];
    const float fp = (dx2 + dy2) * 0.5f;
    const uint32_t u = as_u32(std::fmax(fp, 1.0f));
    uint32_t lg = 0;
    while ((u >> (lg + 1)) != 0) ++lg;
    const uint32_t mip = lg >> 1;
    const uint32_t mx = t->mip_count - 1;
    return mip < mx ? mip : mx;
}
static V3x4 gather_rgb(const swr_texture_view* t, const uint32_t idx[4]) {
    V3x4 r;
    for (int i = 0; i < 4; ++i) {
        const uint32_t c = t->data[idx[i]];
        r.x.l[i] = unorm(c, 24);
        r.y.l[i] = unorm(c, 16);
        r.z.l[i] = unorm(c, 8);
    }
    return r;
}
// sample4_rgb / sample4_alpha (src/texture.rs:680-714).
static void sample4_index(const Tex& tx, F4 u, F4 v, F4 du_dv, uint32_t idx[4]) {
    const swr_texture_view* t = tx.t;
    const uint32_t m = compute_mip_level(t, du_dv);
    const F4 wf = splat(mipw(t, m)), hf = splat(miph(t, m));
    const F4 x = apply_wrap(vfloor(u * wf), wf, tx.wrap_s);
    const F4 y = apply_wrap(vfloor(v * hf), hf, tx.wrap_t);
    for (int i = 0; i < 4; ++i) idx[i] = t->mip_offsets[m] + as_u32(y.l[i]) * t->mip_widths[m] + as_u32(x.l[i]);
}
static V3x4 sample4_rgb(const Tex& tx, F4 u, F4 v, F4 du_dv) {
    uint32_t idx[4];
    sample4_index(tx, u, v, du_dv, idx);
    return gather_rgb(tx.t, idx);
}
static F4 sample4_alpha(const Tex& tx, F4 u, F4 v, F4 du_dv) {
    uint32_t idx[4];
    sample4_index(tx, u, v, du_dv, idx);
    F4 r;
    for (int i = 0; i < 4; ++i) r.l[i] = unorm(tx.t->data[idx[i]], 0);
    return r;
}
// cubemap_uv_from_normal (src/texture.rs:593-644).
static void cubemap_uv(V3x4 n, F4& uf, F4& vf, uint32_t slice[4]) {
    for (int i = 0; i < 4; ++i) {
        const float nx = n.x.l[i], ny = n.y.l[i], nz = n.z.l[i];
        const float ax = std::fabs(nx), ay = std::fabs(ny), az = std::fabs(nz);
        const bool mx = ax >= ay && ax >= az;
        const bool my = ay > ax && ay >= az;
        const float sx = nx >= 0.0f ? 1.0f : -1.0f;
        const float sy = ny >= 0.0f ? 1.0f : -1.0f;
        const float sz = nz >= 0.0f ? 1.0f : -1.0f;
        const float u = mx ? (-nz * sx) : (my ? nx : nx * sz);
        const float v = mx ? -ny : (my ? nz * sy : -ny);
        float den = mx ? ax : (my ? ay : az);
        den = std::fmax(den, 1.0e-19f);
        uf.l[i] = 0.5f * (u / den + 1.0f);
        vf.l[i] = 0.5f * (v / den + 1.0f);
        const float fx = nx >= 0.0f ? 0.0f : 1.0f;
        const float fy = ny >= 0.0f ? 2.0f : 3.0f;
        const float fz = nz >= 0.0f ? 4.0f : 5.0f;
        slice[i] = as_u32(mx ? fx : (my ? fy : fz));
    }
}
// sample_cubemap_rgb (src/texture.rs:646-663).
static V3x4 sample_cubemap_rgb(const swr_texture_view* t, V3x4 n, const uint32_t mip_in[4]) {
    F4 u, v;
    uint32_t slice[4];
    cubemap_uv(n, u, v, slice);
    uint32_t idx[4];
    for (int i = 0; i < 4; ++i) {
        const uint32_t mx = t->mip_count - 1;
        const uint32_t m = mip_in[i] < mx ? mip_in[i] : mx;
        const float wf = mipw(t, m), hf = miph(t, m);
        float x = std::round(u.l[i] * (wf - 1.0f));
        float y = std::round(v.l[i] * (hf - 1.0f));
        x = std::fmin(std::fmax(x, 0.0f), wf - 1.0f);
        y = std::fmin(std::fmax(y, 0.0f), hf - 1.0f);
        idx[i] = t->mip_offsets[m] + slice[i] * t->array_stride[m] + as_u32(y) * t->mip_widths[m] + as_u32(x);
    }
    return gather_rgb(t, idx);
}
// sample_cubemap_trilinear_rgb (src/texture.rs:665-678).
static V3x4 sample_cubemap_trilinear(const swr_texture_view* t, V3x4 n, F4 mip) {
    const F4 mxv = splat((float)(t->mip_count - 1));
    const F4 m = vclamp(mip, splat(0.0f), mxv);
    const F4 m0 = vfloor(m);
    const F4 m1 = vmin(m0 + 1.0f, mxv);
    const F4 tt = m - m0;
    uint32_t i0[4], i1[4];
    for (int i = 0; i < 4; ++i) {
        i0[i] = as_u32(m0.l[i]);
        i1[i] = as_u32(m1.l[i]);
    }
    const V3x4 c0 = sample_cubemap_rgb(t, n, i0);
    const V3x4 c1 = sample_cubemap_rgb(t, n, i1);
    return {c0.x + (c1.x - c0.x) * tt, c0.y + (c1.y - c0.y) * tt, c0.z + (c1.z - c0.z) * tt};
}
// sample_bilinear_rgb, mip 0, slice 0, ClampToEdge (src/texture.rs:730-790).
static V3x4 sample_bilinear_rgb(const swr_texture_view* t, F4 u, F4 v) {
    const F4 wf = splat(mipw(t, 0)), hf = splat(miph(t, 0));
    const F4 xf = u * wf - 0.5f, yf = v * hf - 0.5f;
    const F4 x0 = vfloor(xf), y0 = vfloor(yf);
    const F4 x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const F4 fx = xf - x0, fy = yf - y0;
    const F4 ofx = 1.0f - fx, ofy = 1.0f - fy;
    const F4 cx0 = apply_wrap(x0, wf, SWR_WRAP_CLAMP_TO_EDGE), cy0 = apply_wrap(y0, hf, SWR_WRAP_CLAMP_TO_EDGE);
    const F4 cx1 = apply_wrap(x1, wf, SWR_WRAP_CLAMP_TO_EDGE), cy1 = apply_wrap(y1, hf, SWR_WRAP_CLAMP_TO_EDGE);
    uint32_t i00[4], i10[4], i01[4], i11[4];
    const uint32_t w = t->mip_widths[0], off = t->mip_offsets[0];
    for (int i = 0; i < 4; ++i) {
        i00[i] = off + as_u32(cy0.l[i]) * w + as_u32(cx0.l[i]);
        i10[i] = off + as_u32(cy0.l[i]) * w + as_u32(cx1.l[i]);
        i01[i] = off + as_u32(cy1.l[i]) * w + as_u32(cx0.l[i]);
        i11[i] = off + as_u32(cy1.l[i]) * w + as_u32(cx1.l[i]);
    }
    const V3x4 p00 = gather_rgb(t, i00), p10 = gather_rgb(t, i10), p01 = gather_rgb(t, i01), p11 = gather_rgb(t, i11);
    const F4 w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
    return {((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11,
            ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11,
            ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11};
}

// ---------------------------------------------------------------- voxel
struct Voxel {
    uint32_t n;
    float min[3], vs[3];
    const float* light;
    float gi[4][4];
    const float* sh4;  // baked grid (n^3 x 16), or null
};
// get_filtered_gi_sh4_packed_vec (src/voxelgrid.rs:264-368) over the baked
// grid, or over a grid whose voxels all hold gi[c] except w of coefficient 0
// (light intensity).
static void voxel_gi(const Voxel& g, V3x4 p, V3x4 out_rgb[4], F4 out_w[4]) {
    const F4 vx = (p.x - g.min[0]) / splat(g.vs[0]);
    const F4 vy = (p.y - g.min[1]) / splat(g.vs[1]);
    const F4 vz = (p.z - g.min[2]) / splat(g.vs[2]);
    const F4 x0f = vfloor(vx), y0f = vfloor(vy), z0f = vfloor(vz);
    uint64_t x0[4], y0[4], z0[4], x1[4], y1[4], z1[4];
    const uint64_t nm1 = g.n - 1;
    for (int i = 0; i < 4; ++i) {
        auto us = [](float f) -> uint64_t {
            if (!(f > 0.0f)) return 0;
            if (f >= 1.8446744e19f) return UINT64_MAX;
            return (uint64_t)f;
        };
        x0[i] = std::min(us(x0f.l[i]), nm1);
        y0[i] = std::min(us(y0f.l[i]), nm1);
        z0[i] = std::min(us(z0f.l[i]), nm1);
        x1[i] = std::min(x0[i] + 1, nm1);
        y1[i] = std::min(y0[i] + 1, nm1);
        z1[i] = std::min(z0[i] + 1, nm1);
    }
    const F4 fx = vx - x0f, fy = vy - y0f, fz = vz - z0f;
    auto coeff = [&](int c, int comp, const uint64_t* X, const uint64_t* Y, const uint64_t* Z) {
        F4 r;
        for (int i = 0; i < 4; ++i) {
            if (g.sh4)
                r.l[i] = g.sh4[(Z[i] * g.n * g.n + Y[i] * g.n + X[i]) * 16 + (uint64_t)c * 4 + comp];
            else if (c == 0 && comp == 3)
                r.l[i] = g.light[Z[i] * g.n * g.n + Y[i] * g.n + X[i]];
            else
                r.l[i] = g.gi[c][comp];
        }
        return r;
    };
    auto tri = [&](int c, int comp) {
        const F4 v000 = coeff(c, comp, x0, y0, z0), v001 = coeff(c, comp, x0, y0, z1);
        const F4 v010 = coeff(c, comp, x0, y1, z0), v011 = coeff(c, comp, x0, y1, z1);
        const F4 v100 = coeff(c, comp, x1, y0, z0), v101 = coeff(c, comp, x1, y0, z1);
        const F4 v110 = coeff(c, comp, x1, y1, z0), v111 = coeff(c, comp, x1, y1, z1);
        const F4 v00 = v000 * (1.0f - fx) + v100 * fx;
        const F4 v01 = v001 * (1.0f - fx) + v101 * fx;
        const F4 v10 = v010 * (1.0f - fx) + v110 * fx;
        const F4 v11 = v011 * (1.0f - fx) + v111 * fx;
        const F4 v0 = v00 * (1.0f - fy) + v10 * fy;
        const F4 v1 = v01 * (1.0f - fy) + v11 * fy;
        return v0 * (1.0f - fz) + v1 * fz;
    };
    for (int c = 0; c < 4; ++c) {
        out_rgb[c] = {tri(c, 0), tri(c, 1), tri(c, 2)};
        out_w[c] = tri(c, 3);
    }
}

// ---------------------------------------------------------------- glam mats
struct M4 {
    float m[16];  // column-major
};
static inline void mat_vec(const float* m, const float v[4], float o[4]) {
    for (int r = 0; r < 4; ++r) o[r] = ((m[r] * v[0] + m[4 + r] * v[1]) + m[8 + r] * v[2]) + m[12 + r] * v[3];
}
static inline M4 mat_mul(const float* a, const float* b) {
    M4 r;
    for (int c = 0; c < 4; ++c) mat_vec(a, b + 4 * c, r.m + 4 * c);
    return r;
}
static inline float len4(const float* c) { return std::sqrt((c[0] * c[0] + c[1] * c[1]) + (c[2] * c[2] + c[3] * c[3])); }
static inline float dot4(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + (a[2] * b[2] + a[3] * b[3]); }

// ---------------------------------------------------------------- renderer.rs
struct IV2 {
    int32_t x, y;
};
struct Vertex {
    float pos_clip[4];
    float pos_world[3];
    float normal[3];
    float tangent[4];
    float uv[2];
};
// RasterPacket (src/renderer.rs:58-76) plus the triangle identity this build
// exports in its visibility buffer.
struct Packet {
    IV2 min, max;
    IV2 p[3];
    SI zow, oow;
    VI normals, tangents;
    SI tsign, uow, vow;
    VI pww;
    float ooa;
    uint32_t material;
    float du_dv[4];
    uint32_t static_id, fan;
    float avg_z;  // translucent packets: mean clip-space z of the three vertices
};

constexpr int TILE = 64;

// BumpQueue-like per-tile queue: lock-free slot allocation, 1024-packet blocks.
struct Queue {
    std::atomic<size_t> count{0};
    std::vector<Packet*> blocks;
    std::mutex lock;
    void push(const Packet& p) {
        const size_t i = count.fetch_add(1, std::memory_order_relaxed);
        const size_t b = i / 1024;
        Packet* blk;
        {
            std::lock_guard<std::mutex> g(lock);
            while (blocks.size() <= b) blocks.push_back(new Packet[1024]);
            blk = blocks[b];
        }
        blk[i % 1024] = p;
    }
    const Packet& get(size_t i) const { return blocks[i / 1024][i % 1024]; }
    size_t size() const { return count.load(std::memory_order_relaxed); }
    ~Queue() {
        for (Packet* b : blocks) delete[] b;
    }
};

struct Tile {
    IV2 smin, smax;
    uint64_t quads_tested = 0, fragments = 0, depth_passed = 0;
    Queue opaque, translucent;
    std::vector<V3x4> color;
    std::vector<F4> depth;
    std::vector<uint32_t> pidx;  // 4 per quad
    std::vector<F4> bary1, bary2;
    float center_luminance = 1.0f;
};

struct Frame {
    const swr_scene_host_view* s;
    const swr_camera* cam;
    int width, height, tiles_x, tiles_y;
    float width_f, height_f;
    std::vector<Tile*> tiles;
    Voxel vox;
};

static Tex texof(const Frame& f, const swr_material_view& m, int slot) {
    return {&f.s->textures[m.tex[slot]], m.wrap_s[slot], m.wrap_t[slot]};
}

// clip_to_screen_subpixels (src/renderer.rs:834-846).
static IV2 to_screen(const Frame& f, const float* v) {
    const float nx = v[0] / v[3], ny = v[1] / v[3];
    const float sx = ((nx + 1.0f) * f.width_f) / 2.0f;
    const float sy = ((1.0f - ny) * f.height_f) / 2.0f;
    return {as_i32(std::round(sx * 16.0f)), as_i32(std::round(sy * 16.0f))};
}

// bin_triangle (src/renderer.rs:668-831); MODE_OPAQUE selects the queue.
static void bin_triangle(Frame& f, const Vertex* v, uint32_t material, uint32_t static_id, uint32_t fan, bool opaque) {
    const IV2 p0 = to_screen(f, v[0].pos_clip), p1 = to_screen(f, v[1].pos_clip), p2 = to_screen(f, v[2].pos_clip);
    const int32_t area = wsub(wmul(wsub(p1.x, p0.x), wsub(p2.y, p0.y)), wmul(wsub(p2.x, p0.x), wsub(p1.y, p0.y)));
    if (area > 0) return;
    const int32_t wsp = f.width * 16, hsp = f.height * 16;
    const IV2 mns = {std::max(std::min(std::min(p0.x, p1.x), p2.x), 0), std::max(std::min(std::min(p0.y, p1.y), p2.y), 0)};
    const IV2 mxs = {std::min(std::max(std::max(p0.x, p1.x), p2.x), wsp),
                     std::min(std::max(std::max(p0.y, p1.y), p2.y), hsp)};
    const IV2 mnp = {mns.x >> 4, mns.y >> 4};
    const IV2 mxp = {wadd(mxs.x, 16) >> 4, wadd(mxs.y, 16) >> 4};
    const int32_t aa = area < 0 ? (int32_t)(0u - (uint32_t)area) : area;
    Packet pk;
    pk.ooa = 1.0f / (float)aa;
    float oow[3], zow[3], uow[3], vow[3];
    for (int k = 0; k < 3; ++k) {
        oow[k] = 1.0f / v[k].pos_clip[3];
        zow[k] = v[k].pos_clip[2] * oow[k];
        uow[k] = v[k].uv[0] * oow[k];
        vow[k] = v[k].uv[1] * oow[k];
    }
    pk.zow = SI::from3(zow[0], zow[1], zow[2]);
    pk.oow = SI::from3(oow[0], oow[1], oow[2]);
    for (int c = 0; c < 3; ++c) {
        pk.normals.c[c] = SI::from3(v[0].normal[c], v[1].normal[c], v[2].normal[c]);
        pk.tangents.c[c] = SI::from3(v[0].tangent[c], v[1].tangent[c], v[2].tangent[c]);
        pk.pww.c[c] = SI::from3(v[0].pos_world[c] * oow[0], v[1].pos_world[c] * oow[1], v[2].pos_world[c] * oow[2]);
    }
    pk.tsign = SI::from3(v[0].tangent[3], v[1].tangent[3], v[2].tangent[3]);
    pk.uow = SI::from3(uow[0], uow[1], uow[2]);
    pk.vow = SI::from3(vow[0], vow[1], vow[2]);
    const float dx1 = (float)wsub(p1.x, p0.x), dx2 = (float)wsub(p2.x, p0.x);
    const float dy1 = (float)wsub(p1.y, p0.y), dy2 = (float)wsub(p2.y, p0.y);
    const float du1 = uow[1] - uow[0], du2 = uow[2] - uow[0], dv1 = vow[1] - vow[0], dv2 = vow[2] - vow[0];
    const float sc = pk.ooa * 16.0f;
    pk.du_dv[0] = (du1 * dy2 - du2 * dy1) * sc;
    pk.du_dv[1] = (du2 * dx1 - du1 * dx2) * sc;
    pk.du_dv[2] = (dv1 * dy2 - dv2 * dy1) * sc;
    pk.du_dv[3] = (dv2 * dx1 - dv1 * dx2) * sc;
    pk.p[0] = p0;
    pk.p[1] = p1;
    pk.p[2] = p2;
    pk.material = material;
    pk.static_id = static_id;
    pk.fan = fan;
    // Average z for the per-tile translucency sort (src/renderer.rs:765-774).
    pk.avg_z = opaque ? 0.0f : ((v[0].pos_clip[2] + v[1].pos_clip[2]) + v[2].pos_clip[2]) / 3.0f;
    const int32_t bx0 = mnp.x / TILE, by0 = mnp.y / TILE;
    const int32_t bx1 = (mxp.x + TILE - 1) / TILE, by1 = (mxp.y + TILE - 1) / TILE;
    const int32_t ntiles = (int32_t)f.tiles.size();
    for (int32_t y = by0; y < by1; ++y) {
        for (int32_t x = bx0; x < bx1; ++x) {
            const int32_t bi = y * f.tiles_x + x;
            if (bi < 0 || bi >= ntiles) continue;
            Tile* t = f.tiles[bi];
            const IV2 cmin = {std::max(mnp.x, t->smin.x), std::max(mnp.y, t->smin.y)};
            const IV2 cmax = {std::min(mxp.x, t->smax.x), std::min(mxp.y, t->smax.y)};
            if (cmax.x - cmin.x < 1 || cmax.y - cmin.y < 1) continue;
            pk.min = cmin;
            pk.max = cmax;
            if (opaque)
                t->opaque.push(pk);
            else
                t->translucent.push(pk);
        }
    }
}

// clip_against_frustum (src/renderer.rs:579-665).
static void clip_triangle(Frame& f, const Vertex* tri, uint32_t material, uint32_t static_id, bool opaque) {
    static const float planes[6][4] = {{0, 0, 1, 1}, {0, 0, -1, 1}, {1, 0, 0, 1},
                                       {-1, 0, 0, 1}, {0, 1, 0, 1}, {0, -1, 0, 1}};
    Vertex poly[16], np[16];
    int len = 3;
    poly[0] = tri[0];
    poly[1] = tri[1];
    poly[2] = tri[2];
    auto lerp = [](const Vertex& a, const Vertex& b, float t) {
        Vertex o;
        for (int i = 0; i < 4; ++i) o.pos_clip[i] = a.pos_clip[i] + (b.pos_clip[i] - a.pos_clip[i]) * t;
        for (int i = 0; i < 3; ++i) o.pos_world[i] = a.pos_world[i] + (b.pos_world[i] - a.pos_world[i]) * t;
        for (int i = 0; i < 3; ++i) o.normal[i] = a.normal[i] + (b.normal[i] - a.normal[i]) * t;
        for (int i = 0; i < 4; ++i) o.tangent[i] = a.tangent[i] + (b.tangent[i] - a.tangent[i]) * t;
        for (int i = 0; i < 2; ++i) o.uv[i] = a.uv[i] + (b.uv[i] - a.uv[i]) * t;
        return o;
    };
    for (int p = 0; p < 6; ++p) {
        if (len == 0) return;
        int nl = 0;
        for (int i = 0; i < len; ++i) {
            const Vertex& cur = poly[i];
            const Vertex& prv = poly[(i + len - 1) % len];
            const float dc = dot4(planes[p], cur.pos_clip), dp = dot4(planes[p], prv.pos_clip);
            if (dc >= 0.0f) {
                if (!(dp >= 0.0f)) np[nl++] = lerp(prv, cur, dp / (dp - dc));
                np[nl++] = cur;
            } else if (dp >= 0.0f) {
                np[nl++] = lerp(prv, cur, dp / (dp - dc));
            }
        }
        for (int i = 0; i < nl; ++i) poly[i] = np[i];
        len = nl;
    }
    if (len < 3) return;
    for (int i = 1; i < len - 1; ++i) {
        const Vertex t3[3] = {poly[0], poly[i], poly[i + 1]};
        bin_triangle(f, t3, material, static_id, (uint32_t)(i - 1), opaque);
    }
}

// render_primitive_inner (src/renderer.rs:470-574) for one triangle.
static void process_triangle(Frame& f, const swr_primitive_view& p, const float* model, const float* mvp, bool clip,
                             uint32_t t, uint32_t static_base, bool opaque) {
    Vertex v[3];
    for (int k = 0; k < 3; ++k) {
        const uint32_t i = p.indices[3 * t + k];
        const float* pos = p.positions + 4 * (size_t)i;
        const float* n = p.normals + 4 * (size_t)i;
        const float* tg = p.tangents + 4 * (size_t)i;
        float world[4];
        mat_vec(model, pos, world);
        mat_vec(mvp, pos, v[k].pos_clip);
        for (int c = 0; c < 3; ++c) {
            v[k].pos_world[c] = world[c];
            v[k].normal[c] = (model[c] * n[0] + model[4 + c] * n[1]) + model[8 + c] * n[2];
            v[k].tangent[c] = (model[c] * tg[0] + model[4 + c] * tg[1]) + model[8 + c] * tg[2];
        }
        v[k].tangent[3] = tg[3];
        v[k].uv[0] = p.texcoords[2 * (size_t)i];
        v[k].uv[1] = p.texcoords[2 * (size_t)i + 1];
    }
    if (clip)
        clip_triangle(f, v, p.material, static_base + t, opaque);
    else
        bin_triangle(f, v, p.material, static_base + t, 0, opaque);
}

// ---------------------------------------------------------------- tilerasterizer.rs
static inline size_t qindex(const Tile& t, IV2 px) {
    const int32_t lx = (px.x - t.smin.x) / 2, ly = (px.y - t.smin.y) / 2;
    const int32_t wq = (t.smax.x - t.smin.x) / 2;
    return (size_t)(ly * wq + lx);
}

struct Edges {
    F4 a01, b01, c01, a12, b12, c12, a20, b20, c20;
    F4 sx01, sx12, sx20, sy01, sy12, sy20;
};

static V3x4 pbr_shader(const Frame& f, const Packet& pk, F4 b1, F4 b2, bool translucent, const V3x4* cur);

// fine_raster (src/tilerasterizer.rs:293-383) with VBufferOpaqueShader
// (src/shader.rs:32-63) or, for translucent packets, TranslucentForwardShader
// (src/shader.rs:66-76).
static void fine_raster(const Frame& f, Tile& t, const Packet& pk, const Edges& e, size_t packet_index, int32_t xs,
                        int32_t ys, int32_t xe, int32_t ye, bool translucent) {
    const swr_material_view& mat = f.s->materials[pk.material];
    const F4 x = mk((float)(xs + 8), (float)(xs + 24), (float)(xs + 8), (float)(xs + 24));
    const F4 y = mk((float)(ys + 8), (float)(ys + 8), (float)(ys + 24), (float)(ys + 24));
    F4 w0r = (e.a12 * x + e.b12 * y) + e.c12;
    F4 w1r = (e.a20 * x + e.b20 * y) + e.c20;
    F4 w2r = (e.a01 * x + e.b01 * y) + e.c01;
    const F4 ooa = splat(pk.ooa);
    for (int32_t py = ys; py < ye; py += 32) {
        F4 w0 = w0r, w1 = w1r, w2 = w2r;
        for (int32_t px = xs; px < xe; px += 32) {
            B4 mask;
            bool any = false;
            t.quads_tested++;
            for (int i = 0; i < 4; ++i) {
                mask[i] = w0.l[i] >= 0.0f && w1.l[i] >= 0.0f && w2.l[i] >= 0.0f;
                any |= mask[i];
                t.fragments += mask[i] ? 1 : 0;
            }
            if (any) {
                const F4 b1 = w1 * ooa, b2 = w2 * ooa;
                const F4 w = 1.0f / pk.oow.interp(b1, b2);
                const F4 z = pk.zow.interp(b1, b2) * w;
                const IV2 pix = {px >> 4, py >> 4};
                const size_t qi = qindex(t, pix);
                // depth_test (src/tilerasterizer.rs:511-523).
                const F4 cur = t.depth[qi];
                B4 fm;
                bool anyp = false;
                for (int i = 0; i < 4; ++i) {
                    fm[i] = mask[i] && (z.l[i] <= cur.l[i]);
                    anyp |= fm[i];
                    t.depth_passed += fm[i] ? 1 : 0;
                }
                if (anyp && translucent) {
                    // TranslucentForwardShader::shade: blend over the tile colour,
                    // no depth write.
                    const V3x4 cur = t.color[qi];
                    const V3x4 c = pbr_shader(f, pk, b1, b2, true, &cur);
                    t.color[qi] = v3select(fm, c, cur);
                } else if (anyp) {
                    // VBufferOpaqueShader::shade (src/shader.rs:32-63).
                    if (mat.is_alpha_tested) {
                        const Tex tx = texof(f, mat, 0);
                        const F4 u = pk.uow.interp(b1, b2) * w, v = pk.vow.interp(b1, b2) * w;
                        const F4 a = sample4_alpha(tx, u, v, mk(pk.du_dv[0], pk.du_dv[1], pk.du_dv[2], pk.du_dv[3]));
                        for (int i = 0; i < 4; ++i) fm[i] = fm[i] && (a.l[i] >= mat.alpha_cutoff);
                    }
                    for (int i = 0; i < 4; ++i) {
                        if (!fm[i]) continue;
                        t.pidx[4 * qi + i] = (uint32_t)packet_index;
                        t.bary1[qi].l[i] = b1.l[i];
                        t.bary2[qi].l[i] = b2.l[i];
                        t.depth[qi].l[i] = z.l[i];
                    }
                }
            }
            w0 = w0 + e.sx12;
            w1 = w1 + e.sx20;
            w2 = w2 + e.sx01;
        }
        w0r = w0r + e.sy12;
        w1r = w1r + e.sy20;
        w2r = w2r + e.sy01;
    }
}

// rasterize_packet + coarse_raster (src/tilerasterizer.rs:114-291).
static void rasterize_packet(const Frame& f, Tile& t, const Packet& pk, size_t packet_index, bool translucent) {
    const IV2 p0 = pk.p[0], p1 = pk.p[1], p2 = pk.p[2];
    auto bias = [](int32_t a, int32_t b) { return (a < 0 || (a == 0 && b > 0)) ? 0 : -1; };
    const int32_t a01 = wsub(p1.y, p0.y), b01 = wsub(p0.x, p1.x);
    const int32_t c01 = wadd(wsub(wmul(p1.x, p0.y), wmul(p0.x, p1.y)), bias(a01, b01));
    const int32_t a12 = wsub(p2.y, p1.y), b12 = wsub(p1.x, p2.x);
    const int32_t c12 = wadd(wsub(wmul(p2.x, p1.y), wmul(p1.x, p2.y)), bias(a12, b12));
    const int32_t a20 = wsub(p0.y, p2.y), b20 = wsub(p2.x, p0.x);
    const int32_t c20 = wadd(wsub(wmul(p0.x, p2.y), wmul(p2.x, p0.y)), bias(a20, b20));
    Edges e;
    e.a01 = splat((float)a01); e.b01 = splat((float)b01); e.c01 = splat((float)c01);
    e.a12 = splat((float)a12); e.b12 = splat((float)b12); e.c12 = splat((float)c12);
    e.a20 = splat((float)a20); e.b20 = splat((float)b20); e.c20 = splat((float)c20);
    e.sx01 = splat((float)wmul(a01, 32)); e.sx12 = splat((float)wmul(a12, 32)); e.sx20 = splat((float)wmul(a20, 32));
    e.sy01 = splat((float)wmul(b01, 32)); e.sy12 = splat((float)wmul(b12, 32)); e.sy20 = splat((float)wmul(b20, 32));
    const int32_t wp = pk.max.x - pk.min.x, hp = pk.max.y - pk.min.y;
    const int32_t xs = (pk.min.x & ~1) * 16, ys = (pk.min.y & ~1) * 16;
    const int32_t xe = pk.max.x * 16, ye = pk.max.y * 16;
    if (wp > 16 || hp > 16) {
        for (int32_t by = ys; by < ye; by += 256) {
            for (int32_t bx = xs; bx < xe; bx += 256) {
                const F4 cx = mk((float)(bx + 8), (float)(bx + 256 - 8), (float)(bx + 8), (float)(bx + 256 - 8));
                const F4 cy = mk((float)(by + 8), (float)(by + 8), (float)(by + 256 - 8), (float)(by + 256 - 8));
                const F4 w0c = (e.a12 * cx + e.b12 * cy) + e.c12;
                const F4 w1c = (e.a20 * cx + e.b20 * cy) + e.c20;
                const F4 w2c = (e.a01 * cx + e.b01 * cy) + e.c01;
                auto maxel = [](F4 v) { return std::fmax(std::fmax(v.l[0], v.l[1]), std::fmax(v.l[2], v.l[3])); };
                if (maxel(w0c) < 0.0f || maxel(w1c) < 0.0f || maxel(w2c) < 0.0f) continue;
                fine_raster(f, t, pk, e, packet_index, bx, by, std::min(bx + 256, xe), std::min(by + 256, ye),
                            translucent);
            }
        }
    } else {
        fine_raster(f, t, pk, e, packet_index, xs, ys, xe, ye, translucent);
    }
}

// pbr_shader<TRANSLUCENT> (src/shader.rs:110-309); cur is the tile colour
// under a translucent fragment.
static V3x4 pbr_shader(const Frame& f, const Packet& pk, F4 b1, F4 b2, bool translucent, const V3x4* cur) {
    const swr_material_view& m = f.s->materials[pk.material];
    const float PI = 3.14159265358979f;
    const F4 EPS = splat(1e-6f);
    const F4 w = 1.0f / pk.oow.interp(b1, b2);
    const V3x4 in_n = normalize(pk.normals.interp(b1, b2));
    const V3x4 in_t = normalize(pk.tangents.interp(b1, b2));
    const F4 tsign = pk.tsign.interp(b1, b2);
    const V3x4 pw = pk.pww.interp(b1, b2) * w;
    const F4 uvx = pk.uow.interp(b1, b2) * w;
    const F4 uvy = pk.vow.interp(b1, b2) * w;
    const F4 du_dv = mk(pk.du_dv[0], pk.du_dv[1], pk.du_dv[2], pk.du_dv[3]) * w;
    const V3x4 tw = normalize(in_t - in_n * dot(in_n, in_t));
    F4 hand;
    for (int i = 0; i < 4; ++i) hand.l[i] = tsign.l[i] >= 0.0f ? 1.0f : -1.0f;
    const V3x4 bw = cross(in_n, tw) * hand;
    V3x4 nw = normalize(in_n);
    if (m.tex[2] >= 0) {
        const V3x4 tsn = sample4_rgb(texof(f, m, 2), uvx, uvy, du_dv) * 2.0f - 1.0f;
        nw = (tw * tsn.x + bw * tsn.y) + in_n * tsn.z;
        nw = normalize(nw);
    }
    const V3x4 ld = v3f(f.s->light_direction[0], f.s->light_direction[1], f.s->light_direction[2]);
    const V3x4 lc = v3f(f.s->light_color[0], f.s->light_color[1], f.s->light_color[2]);
    const V3x4 vd = v3f(f.cam->position[0], f.cam->position[1], f.cam->position[2]) - pw;
    const V3x4 vn = normalize(vd);
    const F4 ndl = vmax(dot(nw, ld), splat(0.0f));
    const V3x4 hv = normalize(ld + vn);
    const F4 ndh = vmax(dot(nw, hv), splat(0.0f));
    const F4 ndv = vmax(dot(nw, vn), splat(1.0e-4f));
    const F4 vdh = vmax(dot(vn, hv), splat(0.0f));
    V3x4 gi_rgb[4];
    F4 gi_w[4];
    voxel_gi(f.vox, pw, gi_rgb, gi_w);
    const F4 vli = vclamp(gi_w[0], splat(0.0f), splat(1.0f));
    const F4 skyv = vclamp(gi_w[1], splat(0.0f), splat(1.0f));
    V3x4 bc = v3f(m.base_color_factor[0], m.base_color_factor[1], m.base_color_factor[2]);
    if (m.tex[0] >= 0) bc = bc * srgb_fast(sample4_rgb(texof(f, m, 0), uvx, uvy, du_dv));
    F4 rough = splat(m.roughness_factor), metal = splat(m.metallic_factor);
    if (m.tex[1] >= 0) {
        const V3x4 mr = sample4_rgb(texof(f, m, 1), uvx, uvy, du_dv);
        rough = rough * mr.y;
        metal = metal * mr.z;
    }
    rough = vclamp(rough, splat(0.045f), splat(1.0f));
    metal = vclamp(metal, splat(0.0f), splat(1.0f));
    F4 ao = splat(1.0f);
    if (m.tex[4] >= 0) {
        ao = sample4_rgb(texof(f, m, 4), uvx, uvy, du_dv).x;
        ao = 1.0f + (ao - 1.0f) * splat(m.occlusion_strength);
    }
    const V3x4 f0 = {0.04f + (bc.x - 0.04f) * metal, 0.04f + (bc.y - 0.04f) * metal, 0.04f + (bc.z - 0.04f) * metal};
    const F4 omvh = 1.0f - vdh;
    const F4 omvh2 = omvh * omvh;
    const F4 omvh4 = omvh2 * omvh2;
    const F4 omvh5 = omvh4 * omvh;
    const V3x4 fd = f0 + (v3splat(1.0f) - f0) * omvh5;
    const F4 alpha = rough * rough;
    const F4 alpha2 = alpha * alpha;
    const F4 ndh2 = ndh * ndh;
    const F4 den_d = ndh2 * (alpha2 - 1.0f) + 1.0f;
    const F4 brdf_d = alpha2 / (splat(PI) * (den_d * den_d) + EPS);
    F4 k = rough + 1.0f;
    k = (k * k) * 0.125f;
    const F4 gv = ndv / ((ndv * (1.0f - k) + k) + EPS);
    const F4 gl = ndl / ((ndl * (1.0f - k) + k) + EPS);
    const F4 brdf_g = gv * gl;
    const F4 spec_dg = (brdf_d * brdf_g) / ((splat(4.0f) * ndl) * ndv + EPS);
    const V3x4 kd = (v3splat(1.0f) - fd) * (1.0f - metal);
    const V3x4 lambert = bc * splat(1.0f / PI);
    const V3x4 cdd = (((lc * kd) * lambert) * ndl) * vli;
    const V3x4 cds = (((lc * fd) * spec_dg) * ndl) * vli;
    const V3x4 kdi = (v3splat(1.0f) - f0) * (1.0f - metal);
    // eval_irradiance_sh_vec (src/shader.rs:102-108).
    V3x4 irr = ((gi_rgb[0] + gi_rgb[1] * nw.y) + gi_rgb[2] * nw.z) + gi_rgb[3] * nw.x;
    irr = {vmax(irr.x, splat(0.0f)), vmax(irr.y, splat(0.0f)), vmax(irr.z, splat(0.0f))};
    const V3x4 cid = ((irr * bc) * kdi) * splat(1.0f / PI);
    // reflect (src/math.rs:118-120).
    const V3x4 iv = vn * -1.0f;
    const V3x4 rd = iv - (nw * dot(iv, nw)) * 2.0f;
    const F4 spec_mip = rough * splat((float)(f.s->cubemap_specular.mip_count - 1));
    const V3x4 env = sample_cubemap_trilinear(&f.s->cubemap_specular, rd, spec_mip);
    const V3x4 lut = sample_bilinear_rgb(&f.s->brdf_lut, vclamp(ndv, splat(0.0f), splat(1.0f)),
                                         vclamp(rough, splat(0.0f), splat(1.0f)));
    V3x4 bsf = f0 * lut.x;
    bsf = {bsf.x + lut.y, bsf.y + lut.y, bsf.z + lut.y};
    V3x4 cis = env * bsf;
    const F4 ao_spec = 1.0f + (ao - 1.0f) * 0.5f;
    cis = cis * (ao_spec * skyv);
    V3x4 color;
    if (translucent) {
        F4 tr = splat(m.transmission);
        if (m.tex[5] >= 0) tr = tr * sample4_rgb(texof(f, m, 5), uvx, uvy, du_dv).x;
        tr = vclamp(tr, splat(0.0f), splat(1.0f));
        const F4 inv = 1.0f - tr;
        color = ((((*cur) * bc) * tr + (cdd + cid) * inv) + cds) + cis;
    } else {
        color = ((cdd + cds) + cid) + cis;
    }
    V3x4 em = v3splat(1.0f);
    if (m.tex[3] >= 0) em = srgb_fast(sample4_rgb(texof(f, m, 3), uvx, uvy, du_dv));
    color = color + em * v3f(m.emissive_factor[0], m.emissive_factor[1], m.emissive_factor[2]);
    return color;
}

// compute_skybox (src/tilerasterizer.rs:478-508).
static V3x4 compute_skybox(const Frame& f, IV2 pixel) {
    const float sx = (float)pixel.x, sy = (float)pixel.y;
    const F4 px = mk(sx + 0.5f, sx + 1.5f, sx + 0.5f, sx + 1.5f);
    const F4 py = mk(sy + 0.5f, sy + 0.5f, sy + 1.5f, sy + 1.5f);
    const F4 ndc_x = (px * f.cam->one_over_width) * 2.0f - 1.0f;
    const F4 ndc_y = (1.0f - py * f.cam->one_over_height) * 2.0f - 1.0f;
    const float* m = f.cam->skybox_transposed;
    const F4 one = splat(1.0f);
    const V3x4 d = {((ndc_x * m[0] + ndc_y * m[1]) + one * m[2]) + m[3],
                    ((ndc_x * m[4] + ndc_y * m[5]) + one * m[6]) + m[7],
                    ((ndc_x * m[8] + ndc_y * m[9]) + one * m[10]) + m[11]};
    const uint32_t mip0[4] = {0, 0, 0, 0};
    return srgb_fast(sample_cubemap_rgb(&f.s->cubemap, normalize(d), mip0));
}

// shade_vbuffer (src/tilerasterizer.rs:386-476).
static void shade_vbuffer(const Frame& f, Tile& t, bool skybox_only) {
    const int32_t tw = t.smax.x - t.smin.x, th = t.smax.y - t.smin.y;
    const int32_t wq = tw / 2;
    for (int32_t y = 0; y < th / 2; ++y) {
        const int32_t sy = t.smin.y + y * 2;
        for (int32_t qx = 0; qx < wq; ++qx) {
            const IV2 pixel = {t.smin.x + qx * 2, sy};
            const size_t qi = qindex(t, pixel);
            if (skybox_only) {
                t.color[qi] = compute_skybox(f, pixel);
                continue;
            }
            const uint32_t* pi = &t.pidx[4 * qi];
            const F4 depth = t.depth[qi];
            B4 dm;
            bool anyd = false, alld = true;
            for (int i = 0; i < 4; ++i) {
                dm[i] = depth.l[i] != INFINITY;
                anyd |= dm[i];
                alld &= dm[i];
            }
            V3x4 out = v3splat(0.0f);
            if (anyd) {
                B4 rem = {dm[0], dm[1], dm[2], dm[3]};
                for (;;) {
                    int lane = -1;
                    for (int i = 0; i < 4; ++i)
                        if (rem[i]) {
                            lane = i;
                            break;
                        }
                    if (lane < 0) break;
                    const uint32_t p = pi[lane];
                    B4 mask;
                    for (int i = 0; i < 4; ++i) mask[i] = pi[i] == p;
                    const Packet& pk = t.opaque.get(p);
                    const V3x4 c = pbr_shader(f, pk, t.bary1[qi], t.bary2[qi], false, nullptr);
                    out = v3select(mask, c, out);
                    for (int i = 0; i < 4; ++i) rem[i] = rem[i] && !mask[i];
                }
            }
            if (!alld) out = v3select(dm, out, compute_skybox(f, pixel));
            t.color[qi] = out;
        }
    }
}

// The translucency sort's order (src/tilerasterizer.rs:92-95): OrderedFloat
// avg_z, back to front (NaN is the largest value, -0 equals +0). The
// reference's in-place quicksort is unstable over a rayon-ordered queue, so
// equal keys have no defined order there; here they keep submission order.
static bool translucent_before(float a, float b) {
    if (a != a) return !(b != b);
    if (b != b) return false;
    return a > b;
}

// render_tile (src/tilerasterizer.rs:72-111).
static void render_tile(const Frame& f, Tile& t) {
    for (F4& d : t.depth) d = splat(INFINITY);
    const size_t n = t.opaque.size();
    for (size_t i = 0; i < n; ++i) rasterize_packet(f, t, t.opaque.get(i), i, false);
    shade_vbuffer(f, t, n == 0);
    const size_t nt = t.translucent.size();
    if (nt > 0) {
        std::vector<size_t> order(nt);
        std::iota(order.begin(), order.end(), (size_t)0);
        std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
            return translucent_before(t.translucent.get(a).avg_z, t.translucent.get(b).avg_z);
        });
        for (size_t k = 0; k < nt; ++k) rasterize_packet(f, t, t.translucent.get(order[k]), order[k], true);
    }
    const V3x4 cq = t.color[t.color.size() / 2];
    const F4 lx = (cq.x * 0.2126f + cq.y * 0.7152f) + cq.z * 0.0722f;
    t.center_luminance = (((lx.l[0] + lx.l[1]) + lx.l[2]) + lx.l[3]) * 0.25f;
}

template <typename F>
static void par_for(size_t n, unsigned threads, F fn) {
    if (threads <= 1) {
        for (size_t i = 0; i < n; ++i) fn(i);
        return;
    }
    std::atomic<size_t> next{0};
    auto w = [&]() {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= n) break;
            fn(i);
        }
    };
    std::vector<std::thread> pool;
    for (unsigned k = 1; k < threads; ++k) pool.emplace_back(w);
    w();
    for (auto& th : pool) th.join();
}

}  // namespace orc

extern "C" {

typedef struct oracle_opts {
    uint32_t rsqrt_mode;
    uint32_t threads;     /* 1 = canonical sequential order */
    float dt;
    float ev;             /* exposure state in: log2 of the current exposure (1.0 fresh) */
} oracle_opts;

typedef struct oracle_result {
    float ev;             /* exposure state out */
    float exposure;       /* exposure the blit used */
    float target;
    uint32_t tiles;
    uint64_t packets;     /* (triangle, tile) pairs queued */
    uint64_t triangles_in;
    uint64_t quads_tested;   /* quad coverage tests in fine_raster */
    uint64_t fragments;      /* lanes inside a triangle */
    uint64_t depth_passed;   /* lanes passing the depth test in queue order */
} oracle_result;

// Renderer::render_scene + update_auto_exposure + blit_to_buffer for a fresh
// Renderer (its vbuffer bary/packet index start at zero). rgba8 (height rows
// of width; an odd last row is not written, as chunks_exact drops it), vis
// (width*height) and tile_lum (tiles_x*tiles_y) may be NULL.
int oracle_render(const swr_scene_host_view* s, const swr_camera* cam, int32_t width, int32_t height,
                  const oracle_opts* o, uint32_t* rgba8, uint64_t* vis, float* tile_lum, oracle_result* res) {
    using namespace orc;
    if (!s || !cam || width <= 0 || height <= 0 || !o) return 1;
    g_rsqrt_mode = (int)o->rsqrt_mode;
    const unsigned threads = o->threads ? o->threads : 1;
    Frame f;
    f.s = s;
    f.cam = cam;
    f.width = width;
    f.height = height;
    f.width_f = (float)width;
    f.height_f = (float)height;
    f.tiles_x = (width + TILE - 1) / TILE;
    f.tiles_y = (height + TILE - 1) / TILE;
    f.vox.n = s->voxel_size;
    for (int k = 0; k < 3; ++k) {
        f.vox.min[k] = s->voxel_world_min[k];
        f.vox.vs[k] = (s->voxel_world_max[k] - s->voxel_world_min[k]) / (float)s->voxel_size;
    }
    f.vox.light = s->voxel_light_intensity;
    std::memcpy(f.vox.gi, s->voxel_gi_sh4_const, sizeof(f.vox.gi));
    f.vox.sh4 = s->voxel_gi_sh4;
    for (int ty = 0; ty < f.tiles_y; ++ty)
        for (int tx = 0; tx < f.tiles_x; ++tx) {
            Tile* t = new Tile();
            t->smin = {tx * TILE, ty * TILE};
            t->smax = {(tx + 1) * TILE, (ty + 1) * TILE};
            const size_t nq = (TILE / 2) * (TILE / 2);
            t->color.assign(nq, v3splat(0.0f));
            t->depth.assign(nq, splat(INFINITY));
            t->pidx.assign(4 * nq, 0u);
            t->bary1.assign(nq, splat(0.0f));
            t->bary2.assign(nq, splat(0.0f));
            f.tiles.push_back(t);
        }
    // compute_nodes_by_distance (src/renderer.rs:357-367).
    std::vector<uint32_t> order(s->node_count);
    std::iota(order.begin(), order.end(), 0u);
    std::vector<float> key(s->node_count);
    for (uint32_t i = 0; i < s->node_count; ++i) {
        const float* c = s->nodes[i].sphere;
        const float dx = cam->position[0] - c[0], dy = cam->position[1] - c[1], dz = cam->position[2] - c[2];
        key[i] = (dx * dx + dy * dy) + dz * dz;
    }
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
        const float x = key[a], y = key[b];
        if (x != x) return false;
        if (y != y) return true;
        return x < y;
    });
    // Front end work items: (primitive, model, mvp, clip, 128-triangle batch).
    struct Item {
        const swr_primitive_view* p;
        M4 mvp;
        const float* model;
        bool clip;
        uint32_t t0, t1, static_base;
        bool opaque;
    };
    std::vector<Item> items;
    uint64_t tri_in = 0;
    for (uint32_t ni : order) {
        const swr_node_view& n = s->nodes[ni];
        if (n.mesh < 0) continue;
        // render_node: mvp = VP * model (src/renderer.rs:369-384).
        const M4 mvp = mat_mul(cam->view_project, n.transform);
        const swr_mesh_view& mesh = s->meshes[n.mesh];
        // render_mesh (src/renderer.rs:386-420): opaque primitives, then translucent.
        for (uint32_t k = 0; k < mesh.opaque_count + mesh.translucent_count; ++k) {
            const bool opaque = k < mesh.opaque_count;
            const uint32_t local = opaque ? mesh.opaque[k] : mesh.translucent[k - mesh.opaque_count];
            const swr_primitive_view& p = s->primitives[mesh.primitives[local]];
            // Mat4 * &BoundingSphere (src/scene.rs:53-63) and
            // test_sphere_frustum (src/renderer.rs:130-142).
            const float* M = n.transform;
            const float scale = ((len4(M) + len4(M + 4)) + len4(M + 8)) / 3.0f;
            float c[3];
            for (int r = 0; r < 3; ++r) c[r] = ((M[r] * p.sphere[0] + M[4 + r] * p.sphere[1]) + M[8 + r] * p.sphere[2]) + M[12 + r];
            const float radius = p.sphere[3] * scale;
            const float cw[4] = {c[0], c[1], c[2], 1.0f};
            float cv[4];
            mat_vec(cam->view, cw, cv);
            int result = 0;  // 0 inside, 1 intersecting, 2 outside
            for (int pl = 0; pl < 6; ++pl) {
                const float d = dot4(cam->view_clip_planes[pl], cv);
                if (d < -radius) {
                    result = 2;
                    break;
                } else if (d < radius) {
                    result = 1;
                }
            }
            if (result == 2) continue;
            const uint32_t nt = p.index_count / 3;
            tri_in += nt;
            for (uint32_t t0 = 0; t0 < nt; t0 += 128)
                items.push_back({&p, mvp, n.transform, result == 1, t0, std::min(nt, t0 + 128),
                                 n.triangle_id_base + p.triangle_id_base, opaque});
        }
    }
    par_for(items.size(), threads, [&](size_t i) {
        const Item& it = items[i];
        for (uint32_t t = it.t0; t < it.t1; ++t)
            process_triangle(f, *it.p, it.model, it.mvp.m, it.clip, t, it.static_base, it.opaque);
    });
    uint64_t packets = 0;
    for (Tile* t : f.tiles) packets += t->opaque.size() + t->translucent.size();
    par_for(f.tiles.size(), threads, [&](size_t i) { render_tile(f, *f.tiles[i]); });
    // update_auto_exposure (src/renderer.rs:258-290).
    float ev = o->ev;
    float exposure, target = 0.0f;
    {
        const size_t n = f.tiles.size();
        std::vector<float> smp(n);
        for (size_t i = 0; i < n; ++i) smp[i] = std::log2(std::fmax(f.tiles[i]->center_luminance, 1e-4f));
        std::sort(smp.begin(), smp.end());
        size_t trim = (size_t)std::floor((float)n * 0.10f);
        trim = std::min(trim, (n - 1) / 2);
        float sum = 0.0f;
        for (size_t i = trim; i < n - trim; ++i) sum += smp[i];
        const float mean = sum / (float)(n - 2 * trim);
        const float y = 0.45f;
        const float meter = std::fmax((y * 0.2f) / std::fmax((1.0f + 0.2f) - y, 1e-6f), 1e-4f);
        const float tev0 = std::log2(meter) - mean;
        target = std::fmin(std::fmax(std::exp2(tev0), 0.05f), 32.0f);
        const float tev = std::log2(target);
        const float alpha = 1.0f - std::exp(-(std::fmax(o->dt, 0.0f) / std::fmax(1.0f, 1e-4f)));
        ev += (tev - ev) * alpha;
        exposure = std::exp2(ev);
    }
    // blit_to_buffer (src/renderer.rs:293-355).
    if (rgba8) {
        const int rows2 = height / 2;
        par_for((size_t)rows2, threads, [&](size_t qy) {
            const int py = (int)qy * 2;
            const int ty = py / TILE;
            for (int tx = 0; tx < f.tiles_x; ++tx) {
                const Tile& t = *f.tiles[ty * f.tiles_x + tx];
                const int lq = (py - t.smin.y) / 2;
                const int wq = (t.smax.x - t.smin.x) / 2;
                for (int qx = 0; qx < wq; ++qx) {
                    const int bx = t.smin.x + qx * 2;
                    V3x4 c = t.color[(size_t)(lq * wq + qx)];
                    c = c * splat(exposure);
                    c = tonemap(c);
                    for (int sy = 0; sy < 2; ++sy)
                        for (int sx = 0; sx < 2; ++sx) {
                            const int x = bx + sx;
                            if (x >= width) continue;
                            const int ln = sy * 2 + sx;
                            const uint32_t r = as_u8(c.x.l[ln] * 255.0f), g = as_u8(c.y.l[ln] * 255.0f),
                                           b = as_u8(c.z.l[ln] * 255.0f);
                            rgba8[(size_t)(py + sy) * width + x] = (r << 24) | (g << 16) | (b << 8) | 0xFFu;
                        }
                }
            }
        });
    }
    if (vis) {
        for (int y = 0; y < height; ++y)
            for (int x = 0; x < width; ++x) {
                const Tile& t = *f.tiles[(y / TILE) * f.tiles_x + (x / TILE)];
                const size_t qi = qindex(t, {x & ~1, y & ~1});
                const int ln = (y & 1) * 2 + (x & 1);
                uint64_t v = ~0ull;
                if (t.depth[qi].l[ln] != INFINITY) {
                    const Packet& pk = t.opaque.get(t.pidx[4 * qi + ln]);
                    v = ((uint64_t)pk.static_id << 3) | pk.fan;
                }
                vis[(size_t)y * width + x] = v;
            }
    }
    if (tile_lum)
        for (size_t i = 0; i < f.tiles.size(); ++i) tile_lum[i] = f.tiles[i]->center_luminance;
    if (res) {
        res->ev = ev;
        res->exposure = exposure;
        res->target = target;
        res->tiles = (uint32_t)f.tiles.size();
        res->packets = packets;
        res->triangles_in = tri_in;
        res->quads_tested = res->fragments = res->depth_passed = 0;
        for (Tile* t : f.tiles) {
            res->quads_tested += t->quads_tested;
            res->fragments += t->fragments;
            res->depth_passed += t->depth_passed;
        }
    }
    for (Tile* t : f.tiles) delete t;
    return 0;
}

// Voxel sun visibility of the load-time precompute: RayTracer::new's
// triangles (src/raytracer.rs:71-133), build_active_voxel_mask's occupancy
// and dilation (src/gi.rs:151-265), compute_sun_visibility's
// trace_transmittance per active voxel centre (src/gi.rs:267-314,
// src/raytracer.rs:172-207) and blur_grid (src/voxelgrid.rs:370-419). Every
// ray tests every triangle (no acceleration structure: results depend only
// on ray_triangle_intersect, src/raytracer.rs:225-260, and the hit order,
// t ascending, equal t by triangle). With `brute` = 0 a bounding-volume
// hierarchy of its own prunes the candidates conservatively: boxes are
// padded by 1e-4 of the scene's extent (plus 1e-5), far more than the
// rounding of the slab test or the tolerance of the triangle test, so every
// triangle the exact test could accept is still tested and the hit set is
// that of the brute-force loop. Writes voxel_size^3 floats to `out`.
int oracle_sun_visibility_ex(const swr_scene_host_view* v, uint32_t threads, float* out, int brute) {
    struct P3 {
        float x, y, z;
    };
    auto sub = [](P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; };
    auto add = [](P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; };
    auto mul = [](P3 a, float s) { return P3{a.x * s, a.y * s, a.z * s}; };
    auto dot = [](P3 a, P3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; };
    auto cross = [](P3 a, P3 b) {
        return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    };
    auto length = [&](P3 a) { return std::sqrt(dot(a, a)); };
    auto normalize = [&](P3 a) { return mul(a, 1.0f / length(a)); };
    struct Tri {
        P3 p0, p1, p2;
        uint32_t material;
    };
    // RayTracer::new: world positions (Mat4 * Vec4, x_axis*x + y_axis*y + z_axis*z + w_axis*w).
    std::vector<Tri> tris;
    for (uint32_t ni = 0; ni < v->node_count; ++ni) {
        const swr_node_view& nd = v->nodes[ni];
        if (nd.mesh < 0) continue;
        const swr_mesh_view& m = v->meshes[nd.mesh];
        const float* T = nd.transform;
        for (uint32_t k = 0; k < m.primitive_count; ++k) {
            const swr_primitive_view& p = v->primitives[m.primitives[k]];
            for (uint32_t t = 0; t + 2 < p.index_count; t += 3) {
                P3 w[3];
                for (int c = 0; c < 3; ++c) {
                    const float* q = p.positions + 4 * (size_t)p.indices[t + c];
                    float r[4];
                    for (int j = 0; j < 4; ++j) r[j] = ((T[j] * q[0] + T[4 + j] * q[1]) + T[8 + j] * q[2]) + T[12 + j] * q[3];
                    w[c] = P3{r[0], r[1], r[2]};
                }
                const P3 fn = cross(sub(w[1], w[0]), sub(w[2], w[0]));
                if (dot(fn, fn) <= 1.0e-12f) continue;
                tris.push_back({w[0], w[1], w[2], p.material});
            }
        }
    }
    const uint32_t n = v->voxel_size;
    const size_t nvox = (size_t)n * n * n;
    const P3 bmn{v->voxel_world_min[0], v->voxel_world_min[1], v->voxel_world_min[2]};
    const P3 bmx{v->voxel_world_max[0], v->voxel_world_max[1], v->voxel_world_max[2]};
    const P3 wsz = sub(bmx, bmn);
    const P3 vsz{wsz.x / (float)n, wsz.y / (float)n, wsz.z / (float)n};
    // Occupancy from barycentric samples per triangle, then dilation by 2.
    std::vector<uint8_t> occ(nvox, 0);
    const float mine = std::fmax(std::fmin(vsz.x, std::fmin(vsz.y, vsz.z)), 1.0e-6f);
    const float area_ref = mine * mine;
    for (const Tri& t : tris) {
        const float area = 0.5f * length(cross(sub(t.p1, t.p0), sub(t.p2, t.p0)));
        const float ts = std::ceil((area / area_ref) * 2.0f);
        size_t target = (ts != ts || ts <= 0.0f) ? 0 : (ts >= 1.8e19f ? SIZE_MAX : (size_t)ts);
        target = std::min<size_t>(std::max<size_t>(target, 1), 4096);
        const size_t ns = (size_t)std::ceil(std::sqrt((float)target));
        for (size_t iu = 0; iu < ns; ++iu)
            for (size_t iv = 0; iv < ns - iu; ++iv) {
                const float u = ((float)iu + 0.5f) / (float)ns, w2 = ((float)iv + 0.5f) / (float)ns;
                const float w = (1.0f - u) - w2;
                if (w < 0.0f) continue;
                const P3 p = add(add(mul(t.p0, w), mul(t.p1, u)), mul(t.p2, w2));
                const float fx = (p.x - bmn.x) / vsz.x, fy = (p.y - bmn.y) / vsz.y, fz = (p.z - bmn.z) / vsz.z;
                if (fx < 0.0f || fy < 0.0f || fz < 0.0f) continue;
                const float x = std::floor(fx), y = std::floor(fy), z = std::floor(fz);
                if (!(x < (float)n) || !(y < (float)n) || !(z < (float)n)) continue;
                occ[(size_t)z * n * n + (size_t)y * n + (size_t)x] = 1;
            }
    }
    std::vector<uint8_t> act(nvox, 0);
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                if (!occ[(size_t)z * n * n + (size_t)y * n + x]) continue;
                for (uint32_t a = (z >= 2 ? z - 2 : 0); a <= std::min(z + 2, n - 1); ++a)
                    for (uint32_t b = (y >= 2 ? y - 2 : 0); b <= std::min(y + 2, n - 1); ++b)
                        for (uint32_t c = (x >= 2 ? x - 2 : 0); c <= std::min(x + 2, n - 1); ++c)
                            act[(size_t)a * n * n + (size_t)b * n + c] = 1;
            }
    // Transmittance toward the sun.
    const P3 ld = normalize(P3{v->light_direction[0], v->light_direction[1], v->light_direction[2]});
    const P3 cmin = add(bmn, mul(vsz, 0.5f));
    const float bias = length(vsz) * 3.0f;
    std::vector<float> light(nvox, 1.0f);
    // Conservative BVH over the triangles: median split of the centroids on
    // the longest axis, at most 4 triangles per leaf, padded boxes.
    struct BNode {
        float mn[3], mx[3];
        uint32_t left, first, count;  // count > 0: leaf over order[first, first + count)
    };
    std::vector<BNode> bvh;
    std::vector<uint32_t> order(tris.size());
    std::iota(order.begin(), order.end(), 0u);
    if (!brute && !tris.empty()) {
        const float pad = 1.0e-4f * length(wsz) + 1.0e-5f;
        auto tmin3 = [](const Tri& t, int k) { const float* a = &t.p0.x; const float* b = &t.p1.x; const float* c = &t.p2.x; return std::fmin(a[k], std::fmin(b[k], c[k])); };
        auto tmax3 = [](const Tri& t, int k) { const float* a = &t.p0.x; const float* b = &t.p1.x; const float* c = &t.p2.x; return std::fmax(a[k], std::fmax(b[k], c[k])); };
        std::vector<std::array<uint32_t, 3>> work{{0u, (uint32_t)tris.size(), 0u}};
        bvh.push_back(BNode{});
        while (!work.empty()) {
            const auto w = work.back();
            work.pop_back();
            const uint32_t a = w[0], b = w[1], ni = w[2];
            BNode nd{};
            float cmn[3] = {INFINITY, INFINITY, INFINITY}, cmx[3] = {-INFINITY, -INFINITY, -INFINITY};
            for (int k = 0; k < 3; ++k) nd.mn[k] = INFINITY, nd.mx[k] = -INFINITY;
            for (uint32_t i = a; i < b; ++i) {
                const Tri& t = tris[order[i]];
                for (int k = 0; k < 3; ++k) {
                    nd.mn[k] = std::fmin(nd.mn[k], tmin3(t, k));
                    nd.mx[k] = std::fmax(nd.mx[k], tmax3(t, k));
                    const float c = (tmin3(t, k) + tmax3(t, k)) * 0.5f;
                    cmn[k] = std::fmin(cmn[k], c);
                    cmx[k] = std::fmax(cmx[k], c);
                }
            }
            for (int k = 0; k < 3; ++k) nd.mn[k] -= pad, nd.mx[k] += pad;
            if (b - a <= 4) {
                nd.first = a;
                nd.count = b - a;
                bvh[ni] = nd;
                continue;
            }
            int ax = 0;
            for (int k = 1; k < 3; ++k)
                if (cmx[k] - cmn[k] > cmx[ax] - cmn[ax]) ax = k;
            const uint32_t mid = a + (b - a) / 2;
            std::nth_element(order.begin() + a, order.begin() + mid, order.begin() + b, [&](uint32_t x, uint32_t y) {
                return (tmin3(tris[x], ax) + tmax3(tris[x], ax)) < (tmin3(tris[y], ax) + tmax3(tris[y], ax));
            });
            nd.left = (uint32_t)bvh.size();
            nd.count = 0;
            bvh[ni] = nd;
            bvh.push_back(BNode{});
            bvh.push_back(BNode{});
            work.push_back({a, mid, nd.left});
            work.push_back({mid, b, nd.left + 1});
        }
    }
    auto slab = [&](const BNode& b, P3 o) {
        const float oo[3] = {o.x, o.y, o.z}, dd[3] = {ld.x, ld.y, ld.z};
        float tn = -INFINITY, tf = INFINITY;
        for (int k = 0; k < 3; ++k) {
            if (std::fabs(dd[k]) < 1.0e-30f) {
                if (oo[k] < b.mn[k] || oo[k] > b.mx[k]) return false;
                continue;
            }
            float t0 = (b.mn[k] - oo[k]) / dd[k], t1 = (b.mx[k] - oo[k]) / dd[k];
            if (t0 > t1) std::swap(t0, t1);
            tn = std::fmax(tn, t0);
            tf = std::fmin(tf, t1);
        }
        return tf >= std::fmax(tn, 0.0f);
    };
    std::atomic<bool> too_deep{false};
    auto trace = [&](P3 o) {
        std::vector<std::pair<float, uint32_t>> hits;
        std::vector<uint32_t> cand;
        if (brute || bvh.empty()) {
            cand = order;
        } else {
            uint32_t stack[128];
            int sp = 0;
            stack[sp++] = 0;
            while (sp > 0) {
                const BNode& b = bvh[stack[--sp]];
                if (!slab(b, o)) continue;
                if (b.count > 0) {
                    for (uint32_t i = 0; i < b.count; ++i) cand.push_back(order[b.first + i]);
                } else if (sp + 2 <= 128) {
                    stack[sp++] = b.left;
                    stack[sp++] = b.left + 1;
                } else {
                    too_deep = true;  // a median split of 2^32 triangles is 32 levels deep: never
                    return 0.0f;
                }
            }
        }
        for (uint32_t i : cand) {
            const Tri& t = tris[i];
            const P3 e1 = sub(t.p1, t.p0), e2 = sub(t.p2, t.p0);
            const P3 pv = cross(ld, e2);
            const float det = dot(e1, pv);
            if (std::fabs(det) <= 1.0e-8f) continue;
            const float inv = 1.0f / det;
            const P3 tv = sub(o, t.p0);
            const float u = dot(tv, pv) * inv;
            if (!(u >= 0.0f && u <= 1.0f)) continue;
            const P3 qv = cross(tv, e1);
            const float w = dot(ld, qv) * inv;
            if (w < 0.0f || (u + w) > 1.0f) continue;
            const float th = dot(e2, qv) * inv;
            if (th < 1.0e-4f || th > INFINITY) continue;
            if (!v->materials[t.material].is_translucent) return 0.0f;
            hits.push_back({th, i});
        }
        std::sort(hits.begin(), hits.end(), [](const std::pair<float, uint32_t>& a, const std::pair<float, uint32_t>& b) {
            const bool an = a.first != a.first, bn = b.first != b.first;
            if (an != bn) return bn;
            if (!an && a.first != b.first) return a.first < b.first;
            return a.second < b.second;
        });
        float tr = 1.0f;
        for (const auto& h : hits) {
            tr *= v->materials[tris[h.second].material].transmission;
            if (tr <= 0.0001f) return 0.0f;
        }
        return tr;
    };
    const uint32_t nt = std::max<uint32_t>(1, threads);
    std::vector<std::thread> pool;
    for (uint32_t w = 0; w < nt; ++w)
        pool.emplace_back([&, w] {
            for (size_t idx = w; idx < nvox; idx += nt) {
                if (!act[idx]) continue;
                const uint32_t z = (uint32_t)(idx / ((size_t)n * n)), rem = (uint32_t)(idx % ((size_t)n * n));
                const uint32_t y = rem / n, x = rem % n;
                const P3 vc = add(cmin, P3{(float)x * vsz.x, (float)y * vsz.y, (float)z * vsz.z});
                light[idx] = trace(add(vc, mul(ld, bias)));
            }
        });
    for (auto& t : pool) t.join();
    if (too_deep) return 1;
    // blur_grid: mean of the in-range 3x3x3 neighbours, squared.
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                float sum = 0.0f;
                int count = 0;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int a = (int)x + dx, b = (int)y + dy, c = (int)z + dz;
                            if (a < 0 || b < 0 || c < 0 || a >= (int)n || b >= (int)n || c >= (int)n) continue;
                            sum += light[(size_t)c * n * n + (size_t)b * n + a];
                            count += 1;
                        }
                const float m = count > 0 ? sum / (float)count : 0.0f;
                out[(size_t)z * n * n + (size_t)y * n + x] = count > 0 ? m * m : 0.0f;
            }
    return 0;
}

int oracle_sun_visibility(const swr_scene_host_view* v, uint32_t threads, float* out) {
    return oracle_sun_visibility_ex(v, threads, out, 0);
}

// bake_voxel_gi (src/gi.rs:316-408) + blur_gi_sh4 (src/voxelgrid.rs:422-472)
// for a scene view whose voxel_light_intensity holds the blurred sun
// visibility: per active voxel (occupancy + dilation as above) 64 rays from
// its direction set; trace_nearest keeps the hit of smallest (t, triangle),
// trace_transmittance multiplies translucent hits in that order; every ray
// tests every triangle. Writes voxel_size^3 x 16 floats (four r, g, b, w).
int oracle_gi_bake(const swr_scene_host_view* v, uint32_t threads, float* out) {
    struct P3 {
        float x, y, z;
    };
    auto sub = [](P3 a, P3 b) { return P3{a.x - b.x, a.y - b.y, a.z - b.z}; };
    auto add = [](P3 a, P3 b) { return P3{a.x + b.x, a.y + b.y, a.z + b.z}; };
    auto mul = [](P3 a, float s) { return P3{a.x * s, a.y * s, a.z * s}; };
    auto mulv = [](P3 a, P3 b) { return P3{a.x * b.x, a.y * b.y, a.z * b.z}; };
    auto dot = [](P3 a, P3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; };
    auto cross = [](P3 a, P3 b) {
        return P3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
    };
    auto length = [&](P3 a) { return std::sqrt(dot(a, a)); };
    auto normalize = [&](P3 a) { return mul(a, 1.0f / length(a)); };
    auto vmax0 = [](P3 a) { return P3{std::fmax(a.x, 0.0f), std::fmax(a.y, 0.0f), std::fmax(a.z, 0.0f)}; };
    auto srgb_lin = [](float s) { return s <= 0.04045f ? s / 12.92f : std::pow((s + 0.055f) / 1.055f, 2.4f); };
    const float pi = 3.14159265358979323846f;
    struct Tri {
        P3 p0, p1, p2, n;
        float uv[3][2];
        uint32_t material;
    };
    std::vector<Tri> tris;
    for (uint32_t ni = 0; ni < v->node_count; ++ni) {
        const swr_node_view& nd = v->nodes[ni];
        if (nd.mesh < 0) continue;
        const swr_mesh_view& m = v->meshes[nd.mesh];
        const float* T = nd.transform;
        for (uint32_t k = 0; k < m.primitive_count; ++k) {
            const swr_primitive_view& p = v->primitives[m.primitives[k]];
            for (uint32_t t = 0; t + 2 < p.index_count; t += 3) {
                P3 w[3];
                Tri tr{};
                for (int c = 0; c < 3; ++c) {
                    const uint32_t vi = p.indices[t + c];
                    const float* q = p.positions + 4 * (size_t)vi;
                    float r[4];
                    for (int j = 0; j < 4; ++j) r[j] = ((T[j] * q[0] + T[4 + j] * q[1]) + T[8 + j] * q[2]) + T[12 + j] * q[3];
                    w[c] = P3{r[0], r[1], r[2]};
                    tr.uv[c][0] = p.texcoords[2 * (size_t)vi];
                    tr.uv[c][1] = p.texcoords[2 * (size_t)vi + 1];
                }
                const P3 fn = cross(sub(w[1], w[0]), sub(w[2], w[0]));
                if (dot(fn, fn) <= 1.0e-12f) continue;
                tr.p0 = w[0];
                tr.p1 = w[1];
                tr.p2 = w[2];
                tr.n = normalize(fn);
                tr.material = p.material;
                tris.push_back(tr);
            }
        }
    }
    const uint32_t n = v->voxel_size;
    const size_t nvox = (size_t)n * n * n;
    const P3 bmn{v->voxel_world_min[0], v->voxel_world_min[1], v->voxel_world_min[2]};
    const P3 bmx{v->voxel_world_max[0], v->voxel_world_max[1], v->voxel_world_max[2]};
    const P3 wsz = sub(bmx, bmn);
    const P3 vsz{wsz.x / (float)n, wsz.y / (float)n, wsz.z / (float)n};
    // Active voxels: occupancy from barycentric samples, dilated by 2.
    std::vector<uint8_t> occ(nvox, 0), act(nvox, 0);
    {
        const float mine = std::fmax(std::fmin(vsz.x, std::fmin(vsz.y, vsz.z)), 1.0e-6f);
        const float area_ref = mine * mine;
        for (const Tri& t : tris) {
            const float area = 0.5f * length(cross(sub(t.p1, t.p0), sub(t.p2, t.p0)));
            const float ts = std::ceil((area / area_ref) * 2.0f);
            size_t target = (ts != ts || ts <= 0.0f) ? 0 : (ts >= 1.8e19f ? SIZE_MAX : (size_t)ts);
            target = std::min<size_t>(std::max<size_t>(target, 1), 4096);
            const size_t ns = (size_t)std::ceil(std::sqrt((float)target));
            for (size_t iu = 0; iu < ns; ++iu)
                for (size_t iv = 0; iv < ns - iu; ++iv) {
                    const float u = ((float)iu + 0.5f) / (float)ns, w2 = ((float)iv + 0.5f) / (float)ns;
                    const float w = (1.0f - u) - w2;
                    if (w < 0.0f) continue;
                    const P3 p = add(add(mul(t.p0, w), mul(t.p1, u)), mul(t.p2, w2));
                    const float fx = (p.x - bmn.x) / vsz.x, fy = (p.y - bmn.y) / vsz.y, fz = (p.z - bmn.z) / vsz.z;
                    if (fx < 0.0f || fy < 0.0f || fz < 0.0f) continue;
                    const float x = std::floor(fx), y = std::floor(fy), z = std::floor(fz);
                    if (!(x < (float)n) || !(y < (float)n) || !(z < (float)n)) continue;
                    occ[(size_t)z * n * n + (size_t)y * n + (size_t)x] = 1;
                }
        }
        for (uint32_t z = 0; z < n; ++z)
            for (uint32_t y = 0; y < n; ++y)
                for (uint32_t x = 0; x < n; ++x) {
                    if (!occ[(size_t)z * n * n + (size_t)y * n + x]) continue;
                    for (uint32_t a = (z >= 2 ? z - 2 : 0); a <= std::min(z + 2, n - 1); ++a)
                        for (uint32_t b = (y >= 2 ? y - 2 : 0); b <= std::min(y + 2, n - 1); ++b)
                            for (uint32_t c = (x >= 2 ? x - 2 : 0); c <= std::min(x + 2, n - 1); ++c)
                                act[(size_t)a * n * n + (size_t)b * n + c] = 1;
                }
    }
    auto ray_tri = [&](P3 o, P3 d, const Tri& t, float tmin, float& th, float& bu, float& bv) {
        const P3 e1 = sub(t.p1, t.p0), e2 = sub(t.p2, t.p0);
        const P3 pv = cross(d, e2);
        const float det = dot(e1, pv);
        if (std::fabs(det) <= 1.0e-8f) return false;
        const float inv = 1.0f / det;
        const P3 tv = sub(o, t.p0);
        const float u = dot(tv, pv) * inv;
        if (!(u >= 0.0f && u <= 1.0f)) return false;
        const P3 qv = cross(tv, e1);
        const float w = dot(d, qv) * inv;
        if (w < 0.0f || (u + w) > 1.0f) return false;
        const float tt = dot(e2, qv) * inv;
        if (tt < tmin || tt > INFINITY) return false;
        th = tt;
        bu = u;
        bv = w;
        return true;
    };
    auto before = [](float ta, uint32_t ia, float tb, uint32_t ib) {
        const bool an = ta != ta, bn = tb != tb;
        if (an != bn) return bn;
        if (!an && ta != tb) return ta < tb;
        return ia < ib;
    };
    auto nearest = [&](P3 o, P3 d, float tmin, uint32_t& bi, float& bt, float& bu, float& bv) {
        bool found = false;
        for (uint32_t i = 0; i < (uint32_t)tris.size(); ++i) {
            float t, u, w;
            if (!ray_tri(o, d, tris[i], tmin, t, u, w)) continue;
            if (!found || before(t, i, bt, bi)) {
                found = true;
                bi = i;
                bt = t;
                bu = u;
                bv = w;
            }
        }
        return found;
    };
    auto transmittance = [&](P3 o, P3 d, float tmin) {
        std::vector<std::pair<float, uint32_t>> hits;
        for (uint32_t i = 0; i < (uint32_t)tris.size(); ++i) {
            float t, u, w;
            if (!ray_tri(o, d, tris[i], tmin, t, u, w)) continue;
            if (!v->materials[tris[i].material].is_translucent) return 0.0f;
            hits.push_back({t, i});
        }
        std::sort(hits.begin(), hits.end(), [&](const std::pair<float, uint32_t>& a, const std::pair<float, uint32_t>& b) {
            return before(a.first, a.second, b.first, b.second);
        });
        float tr = 1.0f;
        for (const auto& h : hits) {
            tr *= v->materials[tris[h.second].material].transmission;
            if (tr <= 0.0001f) return 0.0f;
        }
        return tr;
    };
    // sample_bilinear_rgb at mip 0 with the slot's wrap modes, to linear.
    auto wrapf = [](float t, float dim, uint32_t mode) {
        if (mode == 0u) {
            t = t - std::floor(t / dim) * dim;
        } else if (mode == 1u) {
            const float two = dim * 2.0f;
            t = t - std::floor(t / two) * two;
            t = std::fmin(t, two - t);
        }
        return std::fmin(t, dim - 1.0f);
    };
    auto to_u = [](float f) -> uint32_t {
        if (!(f > 0.0f)) return 0;
        if (f >= 4294967296.0f) return 0xFFFFFFFFu;
        return (uint32_t)f;
    };
    auto bilinear = [&](int32_t tex, float u, float w, uint32_t ws, uint32_t wt) {
        const swr_texture_view& T = v->textures[tex];
        const float wf = (float)T.width, hf = (float)T.height;
        const float xf = u * wf - 0.5f, yf = w * hf - 0.5f;
        const float x0 = std::floor(xf), y0 = std::floor(yf);
        const float fx = xf - x0, fy = yf - y0, ofx = 1.0f - fx, ofy = 1.0f - fy;
        const uint32_t ix0 = to_u(wrapf(x0, wf, ws)), iy0 = to_u(wrapf(y0, hf, wt));
        const uint32_t ix1 = to_u(wrapf(x0 + 1.0f, wf, ws)), iy1 = to_u(wrapf(y0 + 1.0f, hf, wt));
        const uint32_t p00 = T.data[iy0 * T.width + ix0], p10 = T.data[iy0 * T.width + ix1];
        const uint32_t p01 = T.data[iy1 * T.width + ix0], p11 = T.data[iy1 * T.width + ix1];
        const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
        float c[3];
        for (int k = 0; k < 3; ++k) {
            const int sh = 24 - 8 * k;
            auto un = [&](uint32_t p) { return (float)((p >> sh) & 0xFFu) / 255.0f; };
            c[k] = ((un(p00) * w00 + un(p10) * w10) + un(p01) * w01) + un(p11) * w11;
        }
        return P3{srgb_lin(c[0]), srgb_lin(c[1]), srgb_lin(c[2])};
    };
    // sample_sky_radiance: nearest texel of the cubemap's mip 0.
    auto sky = [&](P3 d) {
        const float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
        const bool mx = (ax >= ay) && (ax >= az), my = (ay > ax) && (ay >= az);
        const float sx = d.x >= 0.0f ? 1.0f : -1.0f, sy = d.y >= 0.0f ? 1.0f : -1.0f, sz = d.z >= 0.0f ? 1.0f : -1.0f;
        const float u = mx ? -d.z * sx : (my ? d.x : d.x * sz);
        const float w = mx ? -d.y : (my ? d.z * sy : -d.y);
        const float den = std::fmax(mx ? ax : (my ? ay : az), 1.0e-19f);
        const float uf = 0.5f * (u / den + 1.0f), vf = 0.5f * (w / den + 1.0f);
        const uint32_t slice = mx ? (d.x >= 0.0f ? 0u : 1u) : (my ? (d.y >= 0.0f ? 2u : 3u) : (d.z >= 0.0f ? 4u : 5u));
        const uint32_t cs = v->cubemap.width;
        const float wm1 = (float)cs - 1.0f;
        auto rnd = [](float x) {
            float t = std::trunc(x);
            if (std::fabs(x - t) >= 0.5f) t += std::copysign(1.0f, x);
            return t;
        };
        const uint32_t x = to_u(std::fmin(std::fmax(rnd(uf * wm1), 0.0f), wm1));
        const uint32_t y = to_u(std::fmin(std::fmax(rnd(vf * wm1), 0.0f), wm1));
        const uint32_t p = v->cubemap.data[slice * cs * cs + y * cs + x];
        auto un = [&](int sh) { return srgb_lin((float)((p >> sh) & 0xFFu) / 255.0f); };
        return P3{un(24), un(16), un(8)};
    };
    // Direction sets (build_uniform_sphere_samples, src/gi.rs:416-434).
    auto rad_inv = [](uint32_t bits) {
        bits = (bits << 16) | (bits >> 16);
        bits = ((bits & 0x55555555u) << 1) | ((bits & 0xAAAAAAAAu) >> 1);
        bits = ((bits & 0x33333333u) << 2) | ((bits & 0xCCCCCCCCu) >> 2);
        bits = ((bits & 0x0F0F0F0Fu) << 4) | ((bits & 0xF0F0F0F0u) >> 4);
        bits = ((bits & 0x00FF00FFu) << 8) | ((bits & 0xFF00FF00u) >> 8);
        return (float)bits * 2.3283064e-10f;
    };
    std::vector<P3> dirs;
    for (uint32_t set = 0; set < 9; ++set) {
        const float ox = rad_inv(set + 1), oy = ((float)set + 0.5f) / 9.0f;
        for (uint32_t i = 0; i < 64; ++i) {
            float xx = (float)i / 64.0f + ox, xy = rad_inv(i) + oy;
            xx = xx - std::trunc(xx);
            xy = xy - std::trunc(xy);
            const float z = 1.0f - 2.0f * xx;
            const float r = std::sqrt(std::fmax(1.0f - z * z, 0.0f));
            const float phi = 2.0f * pi * xy;
            dirs.push_back(normalize(P3{r * std::cos(phi), r * std::sin(phi), z}));
        }
    }
    const P3 ld = normalize(P3{v->light_direction[0], v->light_direction[1], v->light_direction[2]});
    const P3 lc{v->light_color[0], v->light_color[1], v->light_color[2]};
    P3 shc[4];
    for (int i = 0; i < 4; ++i) shc[i] = P3{v->irradiance_sh[i][0], v->irradiance_sh[i][1], v->irradiance_sh[i][2]};
    const float vlen = length(vsz);
    const float min_edge = std::fmax(std::fmin(std::fmin(vsz.x, vsz.y), vsz.z), 1.0e-6f);
    const float primary_weight = (4.0f * pi) / 64.0f;
    const float primary_bias = std::fmax(vlen * 0.35f, 1.0e-4f * 4.0f);
    const float hit_bias = std::fmax(vlen * 0.05f, 1.0e-4f * 8.0f);
    const float gi_tmin = std::fmax(min_edge * 0.15f, 1.0e-4f);
    const P3 cmin = add(bmn, mul(vsz, 0.5f));
    // estimate_surface_bounce_radiance (src/gi.rs:466-547).
    auto bounce = [&](uint32_t ti, float t, float bu, float bv, P3 o, P3 in_dir) {
        const Tri& tri = tris[ti];
        const swr_material_view& m = v->materials[tri.material];
        P3 nrm = tri.n;
        if (dot(nrm, mul(in_dir, -1.0f)) < 0.0f) nrm = mul(nrm, -1.0f);
        const float bw = (1.0f - bu) - bv;
        const float uvx = (tri.uv[0][0] * bw + tri.uv[1][0] * bu) + tri.uv[2][0] * bv;
        const float uvy = (tri.uv[0][1] * bw + tri.uv[1][1] * bu) + tri.uv[2][1] * bv;
        P3 em{m.emissive_factor[0], m.emissive_factor[1], m.emissive_factor[2]};
        if (m.tex[3] >= 0) em = mulv(em, bilinear(m.tex[3], uvx, uvy, m.wrap_s[3], m.wrap_t[3]));
        em = vmax0(em);
        P3 alb{m.base_color_factor[0], m.base_color_factor[1], m.base_color_factor[2]};
        if (m.tex[0] >= 0) alb = mulv(alb, bilinear(m.tex[0], uvx, uvy, m.wrap_s[0], m.wrap_t[0]));
        alb = mul(P3{std::fmin(std::fmax(alb.x, 0.0f), 1.0f), std::fmin(std::fmax(alb.y, 0.0f), 1.0f),
                     std::fmin(std::fmax(alb.z, 0.0f), 1.0f)}, 1.0f);
        if (dot(alb, alb) <= 0.0f && dot(em, em) <= 0.0f) return P3{0.0f, 0.0f, 0.0f};
        const float dir_bias = hit_bias * 0.5f;
        const P3 so = add(add(o, mul(in_dir, t)), mul(nrm, hit_bias));
        const float ndl = std::fmax(dot(nrm, ld), 0.0f);
        P3 e_sun{0.0f, 0.0f, 0.0f};
        if (ndl > 0.0f) e_sun = mul(lc, ndl * transmittance(add(so, mul(ld, dir_bias)), ld, gi_tmin));
        // sky_visibility_hemisphere4 + tangent_basis (src/gi.rs:549-578).
        const P3 up = std::fabs(nrm.z) < 0.999f ? P3{0.0f, 0.0f, 1.0f} : P3{1.0f, 0.0f, 0.0f};
        const P3 tg = normalize(cross(nrm, up));
        const P3 btg = cross(nrm, tg);
        const float dl[4][3] = {{0.0f, 0.0f, 1.0f}, {0.8660254f, 0.0f, 0.5f}, {-0.4330127f, 0.75f, 0.5f},
                                {-0.4330127f, -0.75f, 0.5f}};
        float vis = 0.0f;
        for (int i = 0; i < 4; ++i) {
            const P3 dir = normalize(add(add(mul(tg, dl[i][0]), mul(btg, dl[i][1])), mul(nrm, dl[i][2])));
            vis += transmittance(add(so, mul(dir, dir_bias)), dir, gi_tmin);
        }
        vis = vis * 0.25f;
        const P3 e_sky = mul(vmax0(add(add(add(shc[0], mul(shc[1], nrm.y)), mul(shc[2], nrm.z)), mul(shc[3], nrm.x))), vis);
        const P3 e_tot = vmax0(add(e_sun, e_sky));
        const P3 bnc = dot(e_tot, e_tot) > 0.0f ? mulv(alb, P3{e_tot.x / pi, e_tot.y / pi, e_tot.z / pi}) : P3{0, 0, 0};
        return add(bnc, em);
    };
    auto lum = [](P3 c) { return (0.2126f * c.x + 0.7152f * c.y) + 0.0722f * c.z; };
    std::vector<float> raw(nvox * 16);
    const uint32_t nt = std::max<uint32_t>(1, threads);
    std::vector<std::thread> pool;
    for (uint32_t wk = 0; wk < nt; ++wk)
        pool.emplace_back([&, wk] {
            for (size_t idx = wk; idx < nvox; idx += nt) {
                float* o = raw.data() + idx * 16;
                const float sun = v->voxel_light_intensity[idx];
                if (!act[idx]) {  // initialize_voxel_gi_from_scene(scale 1, sky 1)
                    for (int i = 0; i < 4; ++i) {
                        o[4 * i] = shc[i].x * 1.0f;
                        o[4 * i + 1] = shc[i].y * 1.0f;
                        o[4 * i + 2] = shc[i].z * 1.0f;
                        o[4 * i + 3] = 0.0f;
                    }
                    o[3] = sun;
                    o[7] = 1.0f;
                    continue;
                }
                const uint32_t z = (uint32_t)(idx / ((size_t)n * n)), rem = (uint32_t)(idx % ((size_t)n * n));
                const uint32_t y = rem / n, x = rem % n;
                const P3 vc = add(cmin, P3{(float)x * vsz.x, (float)y * vsz.y, (float)z * vsz.z});
                const uint32_t set = ((x % 3u) + 3u * (y % 3u) + (z % 3u)) % 9u;
                P3 rsh[4] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                uint32_t sky_hits = 0;
                for (uint32_t s = 0; s < 64; ++s) {
                    const P3 dir = dirs[set * 64 + s];
                    const P3 ro = add(vc, mul(dir, primary_bias));
                    uint32_t ti = 0;
                    float th = 0.0f, bu = 0.0f, bv = 0.0f;
                    P3 rad;
                    if (nearest(ro, dir, gi_tmin, ti, th, bu, bv)) {
                        rad = bounce(ti, th, bu, bv, ro, dir);
                    } else {
                        ++sky_hits;
                        rad = sky(dir);
                    }
                    if (dot(rad, rad) <= 0.0f) continue;
                    const float basis[4] = {0.282095f, 0.488603f * dir.y, 0.488603f * dir.z, 0.488603f * dir.x};
                    for (int i = 0; i < 4; ++i) rsh[i] = add(rsh[i], mul(rad, basis[i] * primary_weight));
                }
                rsh[0] = mul(rsh[0], pi * 0.282095f);
                const float k1 = ((2.0f * pi) / 3.0f) * 0.488603f;
                for (int i = 1; i < 4; ++i) rsh[i] = mul(rsh[i], k1);
                P3 rgb[4];
                for (int i = 0; i < 4; ++i) rgb[i] = vmax0(rsh[i]);
                const float floor_lum = lum(mul(shc[0], 0.005f));
                if (floor_lum > 0.0f) {
                    const float cur = lum(rgb[0]);
                    if (cur < floor_lum) {
                        const float t = std::fmin(std::fmax((floor_lum - cur) / floor_lum, 0.0f), 1.0f);
                        for (int i = 0; i < 4; ++i) rgb[i] = add(mul(rgb[i], 1.0f - t), mul(mul(shc[i], 0.005f), t));
                    }
                }
                for (int i = 0; i < 4; ++i) {
                    o[4 * i] = rgb[i].x;
                    o[4 * i + 1] = rgb[i].y;
                    o[4 * i + 2] = rgb[i].z;
                    o[4 * i + 3] = 0.0f;
                }
                o[3] = sun;
                o[7] = (float)sky_hits / 64.0f;
            }
        });
    for (auto& t : pool) t.join();
    // blur_gi_sh4.
    for (uint32_t z = 0; z < n; ++z)
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                float sum[16] = {};
                float count = 0.0f;
                for (int dz = -1; dz <= 1; ++dz)
                    for (int dy = -1; dy <= 1; ++dy)
                        for (int dx = -1; dx <= 1; ++dx) {
                            const int a = (int)x + dx, b = (int)y + dy, c = (int)z + dz;
                            if (a < 0 || b < 0 || c < 0 || a >= (int)n || b >= (int)n || c >= (int)n) continue;
                            const float* s = raw.data() + ((size_t)c * n * n + (size_t)b * n + a) * 16;
                            for (int k = 0; k < 16; ++k) sum[k] += s[k];
                            count += 1.0f;
                        }
                float* o = out + ((size_t)z * n * n + (size_t)y * n + x) * 16;
                for (int k = 0; k < 16; ++k) o[k] = sum[k] / count;
            }
    return 0;
}

// Depths of one packet's covered lanes as rasterize_packet + coarse_raster +
// fine_raster compute them (src/tilerasterizer.rs:114-383), without the depth
// test: the smallest depth and the number of covered lanes. p holds the
// subpixel vertices (x0, y0, x1, y1, x2, y2), zow and oow the interpolants
// (value at vertex 0, differences to vertices 1 and 2), rect the packet's
// pixel rect clipped to its 64-px tile (min x, min y, max x, max y). Checks
// the raster's occlusion-culling depth floor.
int oracle_packet_depths(const int32_t* p, float ooa, const float* zow, const float* oow, const int32_t* rect,
                         float* zmin, uint64_t* covered) {
    using namespace orc;
    auto bias = [](int32_t a, int32_t b) { return (a < 0 || (a == 0 && b > 0)) ? 0 : -1; };
    const int32_t a01 = wsub(p[3], p[1]), b01 = wsub(p[0], p[2]);
    const int32_t c01 = wadd(wsub(wmul(p[2], p[1]), wmul(p[0], p[3])), bias(a01, b01));
    const int32_t a12 = wsub(p[5], p[3]), b12 = wsub(p[2], p[4]);
    const int32_t c12 = wadd(wsub(wmul(p[4], p[3]), wmul(p[2], p[5])), bias(a12, b12));
    const int32_t a20 = wsub(p[1], p[5]), b20 = wsub(p[4], p[0]);
    const int32_t c20 = wadd(wsub(wmul(p[0], p[5]), wmul(p[4], p[1])), bias(a20, b20));
    const F4 A12 = splat((float)a12), B12 = splat((float)b12), C12 = splat((float)c12);
    const F4 A20 = splat((float)a20), B20 = splat((float)b20), C20 = splat((float)c20);
    const F4 A01 = splat((float)a01), B01 = splat((float)b01), C01 = splat((float)c01);
    const F4 sx12 = splat((float)wmul(a12, 32)), sx20 = splat((float)wmul(a20, 32)), sx01 = splat((float)wmul(a01, 32));
    const F4 sy12 = splat((float)wmul(b12, 32)), sy20 = splat((float)wmul(b20, 32)), sy01 = splat((float)wmul(b01, 32));
    const SI Z = {zow[0], zow[1], zow[2]}, O = {oow[0], oow[1], oow[2]};
    float zm = INFINITY;
    uint64_t n = 0;
    // fine_raster's walk over one region, depth of every covered lane.
    auto walk = [&](int32_t xs, int32_t ys, int32_t xe, int32_t ye) {
        const F4 x = mk((float)(xs + 8), (float)(xs + 24), (float)(xs + 8), (float)(xs + 24));
        const F4 y = mk((float)(ys + 8), (float)(ys + 8), (float)(ys + 24), (float)(ys + 24));
        F4 w0r = (A12 * x + B12 * y) + C12, w1r = (A20 * x + B20 * y) + C20, w2r = (A01 * x + B01 * y) + C01;
        for (int32_t py = ys; py < ye; py += 32) {
            F4 w0 = w0r, w1 = w1r, w2 = w2r;
            for (int32_t px = xs; px < xe; px += 32) {
                const F4 b1 = w1 * splat(ooa), b2 = w2 * splat(ooa);
                const F4 w = 1.0f / O.interp(b1, b2);
                const F4 z = Z.interp(b1, b2) * w;
                for (int i = 0; i < 4; ++i) {
                    if (!(w0.l[i] >= 0.0f && w1.l[i] >= 0.0f && w2.l[i] >= 0.0f)) continue;
                    ++n;
                    if (z.l[i] < zm) zm = z.l[i];  // a NaN depth never passes the depth test
                }
                w0 = w0 + sx12;
                w1 = w1 + sx20;
                w2 = w2 + sx01;
            }
            w0r = w0r + sy12;
            w1r = w1r + sy20;
            w2r = w2r + sy01;
        }
    };
    const int32_t wp = rect[2] - rect[0], hp = rect[3] - rect[1];
    const int32_t xs = (rect[0] & ~1) * 16, ys = (rect[1] & ~1) * 16, xe = rect[2] * 16, ye = rect[3] * 16;
    if (wp > 16 || hp > 16) {
        for (int32_t by = ys; by < ye; by += 256)
            for (int32_t bx = xs; bx < xe; bx += 256) {
                const F4 cx = mk((float)(bx + 8), (float)(bx + 256 - 8), (float)(bx + 8), (float)(bx + 256 - 8));
                const F4 cy = mk((float)(by + 8), (float)(by + 8), (float)(by + 256 - 8), (float)(by + 256 - 8));
                const F4 w0c = (A12 * cx + B12 * cy) + C12, w1c = (A20 * cx + B20 * cy) + C20;
                const F4 w2c = (A01 * cx + B01 * cy) + C01;
                auto maxel = [](F4 v) { return std::fmax(std::fmax(v.l[0], v.l[1]), std::fmax(v.l[2], v.l[3])); };
                if (maxel(w0c) < 0.0f || maxel(w1c) < 0.0f || maxel(w2c) < 0.0f) continue;
                walk(bx, by, std::min(bx + 256, xe), std::min(by + 256, ye));
            }
    } else {
        walk(xs, ys, xe, ye);
    }
    *zmin = zm;
    *covered = n;
    return 0;
}

// Arm FRSQRTE/FRSQRTS emulation, exposed for the known-answer tests.
float oracle_frsqrte(float x) { return orc::frsqrte(x); }

// The powf of srgb_to_linear_scalar (mode 0: powf(x, 2.4)) and of
// linear_to_srgb_scalar (mode 1: powf(x, 1 / 2.4)), src/util.rs:49-72, with
// the host libm, over n values on `threads` threads.
int oracle_srgb_pow(const float* x, uint64_t n, uint32_t mode, uint32_t threads, float* out) {
    if ((!x || !out) && n) return 1;
    const float y = mode == 0 ? 2.4f : 1.0f / 2.4f;
    const uint64_t t = threads ? threads : 1;
    std::vector<std::thread> pool;
    for (uint64_t k = 0; k < t; ++k)
        pool.emplace_back([=] {
            for (uint64_t i = n * k / t; i < n * (k + 1) / t; ++i) out[i] = std::pow(x[i], y);
        });
    for (auto& th : pool) th.join();
    return 0;
}
float oracle_frsqrts(float a, float b) { return orc::frsqrts(a, b); }
float oracle_rsqrt_aarch64(float x) {
    const float y0 = orc::frsqrte(x);
    return y0 * orc::frsqrts(x * y0, y0);
}

}  // extern "C"
