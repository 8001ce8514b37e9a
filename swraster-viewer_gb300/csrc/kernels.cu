// GB300 (sm_103a) kernels for the per-frame rasterization path.
//
// Frame = reset -> draw_emit -> frontend -> clip -> scan -> scatter -> raster
// -> shade (-> translucent -> resolve). All kernels are batched over views:
// the plain path is a batch of one.
//
//   k_reset     counters and bin counts cleared; per node slot (nodes sorted
//   k_draw_emit by the host) MVP, sphere/frustum test and draw counts
//               (render_node / render_mesh, src/renderer.rs:357-420), then
//               the draws and their 256-triangle chunks in the host loop's
//               order.
//   k_frontend  one thread per input triangle (256-triangle chunks of a draw):
//               vertex transform (src/renderer.rs:470-574), trivial clip
//               classification, triangle setup (bin_triangle,
//               src/renderer.rs:668-831), per-tile pair counts with
//               warp-aggregated atomics.
//   k_clip      Sutherland-Hodgman for triangles with a vertex outside a plane
//               (clip_against_frustum, src/renderer.rs:579-665), fan setup.
//   k_scan      exclusive scan of tile counts -> bin offsets, overflow check.
//   k_scatter   record indices into per-tile bins (warp-aggregated cursors);
//               replaces BumpQueue::push (src/bumpqueue.rs:96-112).
//   k_raster    one CTA per scheduling tile: the reference's coarse/fine
//               traversal and f32 edge stepping (src/tilerasterizer.rs:114-383)
//               with a 64-bit (depth, sequence) atomicMin per pixel in shared
//               memory; keys go to HBM (the visibility buffer).
//   k_shade     one thread per pixel, 4 per 2x2 quad: barycentrics rebuilt
//               from the winning record, quad-coupled mip selection,
//               pbr_shader / skybox (src/shader.rs:110-309,
//               src/tilerasterizer.rs:386-508), tile-centre luminance,
//               exposure + tonemap + RGBA8 pack (src/renderer.rs:293-355).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "depthfloor.cuh"
#include "devmath.cuh"
#include "internal.h"

// Raster variant: persistent CTAs pulling tiles from a device counter (needed
// for graph replay with a fixed grid) or one CTA per tile.
#ifndef SWR_RASTER_PERSISTENT
#define SWR_RASTER_PERSISTENT 1
#endif
// Raster: prefetch into L2 the record each thread will likely load in the next round.
// Shading fused into the raster kernel (k_raster<S, true>): each CTA shades
// its tile from the depth keys in shared memory right after rasterizing it,
// so raster and shading work of different tiles share the SMs and keys reach
// HBM only for the translucent pass. Always for tiles of 8 and 16 px, on
// request (FrameArgs.fused_shade, chosen by the batch autotuner) for 32;
// 64-px tiles keep the separate shading kernel (fused, a 4K frame was 18%
// slower: the two code bodies share the instruction cache and the shading
// part spills).
constexpr uint32_t kFusedShadeMaxTile = 16;
#ifndef SWR_RASTER_PREFETCH
#define SWR_RASTER_PREFETCH 1
#endif

namespace swr {

// --------------------------------------------------------------------------
// Small vector helpers (one lane of Vec3x4 / Vec4).
// --------------------------------------------------------------------------
struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return {x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ f3 normalize(f3 a, uint32_t mode, const uint8_t* tab) {
    const float l2 = (a.x * a.x + a.y * a.y) + a.z * a.z;
    const float r = rsqrt_mode(l2, mode, tab);
    return {a.x * r, a.y * r, a.z * r};
}
// glam Vec4::clamp = max(min).min(max); scalar IEEE max/min.
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }

// ScalarInterpolator::interpolate: (a + b1*da) + b2*db (src/util.rs:169-171).
__device__ __forceinline__ float interp(const float* s, float b1, float b2) { return (s[0] + b1 * s[1]) + b2 * s[2]; }
__device__ __forceinline__ f3 interp3(const float* s, float b1, float b2) {
    return {(s[0] + b1 * s[3]) + b2 * s[6], (s[1] + b1 * s[4]) + b2 * s[7], (s[2] + b1 * s[5]) + b2 * s[8]};
}

__constant__ float c_unorm8[256];  // i / 255.0 (src/util.rs:83-89)

__device__ __forceinline__ f3 unpack_rgb(uint32_t t) {
    return {c_unorm8[(t >> 24) & 0xFFu], c_unorm8[(t >> 16) & 0xFFu], c_unorm8[(t >> 8) & 0xFFu]};
}

// srgb_to_linear_fast (src/util.rs:111-113).
__device__ __forceinline__ float srgb_fast(float x) { return x * (x * (x * 0.305306011f + 0.682171111f) + 0.012522878f); }
__device__ __forceinline__ f3 srgb_fast3(f3 c) { return {srgb_fast(c.x), srgb_fast(c.y), srgb_fast(c.z)}; }

// --------------------------------------------------------------------------
// Texture sampling (src/texture.rs:578-863)
// --------------------------------------------------------------------------
// rdim: 1 / dim when dim is a power of two (texel / dim == texel * rdim
// exactly), else 0.
__device__ __forceinline__ float apply_wrap(float texel, float dim, float rdim, uint32_t mode) {
    float t = texel;
    if (mode == 0u) {  // Repeat
        const float q = rdim != 0.0f ? texel * rdim : texel / dim;
        t = texel - floorf(q) * dim;
    } else if (mode == 1u) {  // MirroredRepeat
        const float two = dim * 2.0f;
        const float q = rdim != 0.0f ? texel * (rdim * 0.5f) : texel / two;
        const float m = texel - floorf(q) * two;
        t = fminf(m, two - m);
    }
    return fminf(t, dim - 1.0f);
}

// compute_mip_level (src/texture.rs:851-863): one mip per quad.
__device__ __forceinline__ uint32_t mip_level(const DTexture& t, float d0, float d1, float d2, float d3) {
    const float tx = d0 * t.whv[0], ty = d1 * t.whv[1], tz = d2 * t.whv[2], tw = d3 * t.whv[3];
    const float dx2 = tx * tx + tz * tz;
    const float dy2 = ty * ty + tw * tw;
    const float fp = (dx2 + dy2) * 0.5f;
    const uint32_t u = f2u_sat(fmaxf(fp, 1.0f));
    const uint32_t mip = (31u - (uint32_t)__clz(u)) >> 1;
    return mip < t.max_mip ? mip : t.max_mip;
}

__device__ __forceinline__ uint32_t sample_texel(const DTexture& t, float u, float v, uint32_t mip, uint32_t ws,
                                                 uint32_t wt) {
    const float wf = t.mip_wf[mip], hf = t.mip_hf[mip];
    const uint32_t x = f2u_sat(apply_wrap(floorf(u * wf), wf, t.mip_rwf[mip], ws));
    const uint32_t y = f2u_sat(apply_wrap(floorf(v * hf), hf, t.mip_rhf[mip], wt));
    const uint32_t idx = t.mip_offset[mip] + y * t.mip_w[mip] + x;
    return __ldg(t.data + idx);
}

// cubemap_uv_from_normal (src/texture.rs:593-644).
__device__ __forceinline__ void cube_uv(f3 n, float& uf, float& vf, uint32_t& slice) {
    const float ax = fabsf(n.x), ay = fabsf(n.y), az = fabsf(n.z);
    const bool mx = (ax >= ay) && (ax >= az);
    const bool my = (ay > ax) && (ay >= az);
    const float sx = n.x >= 0.0f ? 1.0f : -1.0f;
    const float sy = n.y >= 0.0f ? 1.0f : -1.0f;
    const float sz = n.z >= 0.0f ? 1.0f : -1.0f;
    const float u_x = -n.z * sx, v_x = -n.y;
    const float u_y = n.x, v_y = n.z * sy;
    const float u_z = n.x * sz, v_z = -n.y;
    const float u = mx ? u_x : (my ? u_y : u_z);
    const float v = mx ? v_x : (my ? v_y : v_z);
    float den = mx ? ax : (my ? ay : az);
    den = fmaxf(den, 1.0e-19f);
    uf = 0.5f * (u / den + 1.0f);
    vf = 0.5f * (v / den + 1.0f);
    const uint32_t ix = n.x >= 0.0f ? 0u : 1u;
    const uint32_t iy = n.y >= 0.0f ? 2u : 3u;
    const uint32_t iz = n.z >= 0.0f ? 4u : 5u;
    slice = mx ? ix : (my ? iy : iz);
}

// sample_cubemap_rgb (src/texture.rs:646-663): nearest texel at one mip.
__device__ __forceinline__ f3 sample_cube(const DTexture& t, float uf, float vf, uint32_t slice, uint32_t mip) {
    if (mip > t.max_mip) mip = t.max_mip;
    const float wf = t.mip_wf[mip], hf = t.mip_hf[mip];
    const uint32_t off = t.mip_offset[mip] + slice * t.array_stride[mip];
    float x = round_away(uf * (wf - 1.0f));
    float y = round_away(vf * (hf - 1.0f));
    x = clampf(x, 0.0f, wf - 1.0f);
    y = clampf(y, 0.0f, hf - 1.0f);
    const uint32_t idx = off + f2u_sat(y) * t.mip_w[mip] + f2u_sat(x);
    return unpack_rgb(__ldg(t.data + idx));
}

// sample_bilinear_rgb at mip 0, slice 0 (src/texture.rs:730-790); ClampToEdge.
__device__ __forceinline__ f3 sample_bilinear(const DTexture& t, float u, float v) {
    const float wf = t.mip_wf[0], hf = t.mip_hf[0];
    const uint32_t wi = t.mip_w[0];
    const float xf = u * wf - 0.5f;
    const float yf = v * hf - 0.5f;
    const float x0 = floorf(xf), y0 = floorf(yf);
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const float fx = xf - x0, fy = yf - y0;
    const float ofx = 1.0f - fx, ofy = 1.0f - fy;
    const uint32_t x0i = f2u_sat(apply_wrap(x0, wf, 0.0f, 2u));
    const uint32_t y0i = f2u_sat(apply_wrap(y0, hf, 0.0f, 2u));
    const uint32_t x1i = f2u_sat(apply_wrap(x1, wf, 0.0f, 2u));
    const uint32_t y1i = f2u_sat(apply_wrap(y1, hf, 0.0f, 2u));
    const uint32_t off = t.mip_offset[0];
    const f3 p00 = unpack_rgb(__ldg(t.data + off + y0i * wi + x0i));
    const f3 p10 = unpack_rgb(__ldg(t.data + off + y0i * wi + x1i));
    const f3 p01 = unpack_rgb(__ldg(t.data + off + y1i * wi + x0i));
    const f3 p11 = unpack_rgb(__ldg(t.data + off + y1i * wi + x1i));
    const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
    return {((p00.x * w00 + p10.x * w10) + p01.x * w01) + p11.x * w11,
            ((p00.y * w00 + p10.y * w10) + p01.y * w01) + p11.y * w11,
            ((p00.z * w00 + p10.z * w10) + p01.z * w01) + p11.z * w11};
}

// --------------------------------------------------------------------------
// Edge functions (src/tilerasterizer.rs:136-164)
// --------------------------------------------------------------------------
__device__ __forceinline__ int32_t top_left_bias(int32_t a, int32_t b) { return (a < 0 || (a == 0 && b > 0)) ? 0 : -1; }

struct Edge {
    float a, b, c, sx, sy;
};
// Edge (xi, yi) -> (xj, yj): a = yj - yi, b = xi - xj, c = xj*yi - xi*yj + bias.
__device__ __forceinline__ Edge make_edge(int32_t xi, int32_t yi, int32_t xj, int32_t yj) {
    const int32_t a = wsub(yj, yi);
    const int32_t b = wsub(xi, xj);
    const int32_t c = wadd(wsub(wmul(xj, yi), wmul(xi, yj)), top_left_bias(a, b));
    Edge e;
    e.a = i2f(a);
    e.b = i2f(b);
    e.c = i2f(c);
    e.sx = i2f(wmul(a, 32));
    e.sy = i2f(wmul(b, 32));
    return e;
}
__device__ __forceinline__ float edge_eval(const Edge& e, float x, float y) { return (e.a * x + e.b * y) + e.c; }

// Traversal origin of a (record, 64-px reference tile) packet for one pixel:
// the quad-aligned clipped bbox min (fine path) or the 16-px block holding
// the pixel (coarse path), src/tilerasterizer.rs:191-291.
struct Origin {
    int32_t ox, oy;  // subpixels
};
__device__ __forceinline__ void clipped_rect(const RecRaster& r, int32_t tx0, int32_t ty0, int32_t& x0, int32_t& y0,
                                             int32_t& x1, int32_t& y1) {
    x0 = max(r.bb[0], tx0);
    y0 = max(r.bb[1], ty0);
    x1 = min(r.bb[2], tx0 + kRefTile);
    y1 = min(r.bb[3], ty0 + kRefTile);
}

// Rebuild bary1/bary2 of pixel (px, py) exactly as fine_raster produced them.
__device__ __forceinline__ void rebuild_bary(const RecRaster& r, int32_t px, int32_t py, float& b1, float& b2) {
    const int32_t tx0 = (px >> 6) << 6, ty0 = (py >> 6) << 6;
    int32_t x0, y0, x1, y1;
    clipped_rect(r, tx0, ty0, x0, y0, x1, y1);
    const bool coarse = (x1 - x0 > 16) || (y1 - y0 > 16);
    const int32_t xs = (x0 & ~1) * kSubpixelScale, ys = (y0 & ~1) * kSubpixelScale;
    int32_t ox = xs, oy = ys;
    if (coarse) {
        ox = xs + ((px * kSubpixelScale - xs) >> 8) * 256;
        oy = ys + ((py * kSubpixelScale - ys) >> 8) * 256;
    }
    const int32_t qi = (px * kSubpixelScale - ox) >> 5;
    const int32_t qj = (py * kSubpixelScale - oy) >> 5;
    const float lx = i2f(ox + ((px & 1) ? 24 : 8));
    const float ly = i2f(oy + ((py & 1) ? 24 : 8));
    const Edge e20 = make_edge(r.p[4], r.p[5], r.p[0], r.p[1]);
    const Edge e01 = make_edge(r.p[0], r.p[1], r.p[2], r.p[3]);
    float w1 = edge_eval(e20, lx, ly);
    float w2 = edge_eval(e01, lx, ly);
    for (int j = 0; j < qj; ++j) {
        w1 += e20.sy;
        w2 += e01.sy;
    }
    for (int i = 0; i < qi; ++i) {
        w1 += e20.sx;
        w2 += e01.sx;
    }
    b1 = w1 * r.ooa;
    b2 = w2 * r.ooa;
}

// --------------------------------------------------------------------------
// Front end
// --------------------------------------------------------------------------
struct Vtx {
    float cx, cy, cz, cw;  // pos_clip
    float wx, wy, wz;      // pos_world
    float nx, ny, nz;      // normal
    float tx, ty, tz, tw;  // tangent
    float u, v;
};

__device__ __forceinline__ Vtx transform_vertex(const DVertex* __restrict__ vb, uint32_t vi, const float* model,
                                                const float* mvp) {
    const float4 a = __ldg(reinterpret_cast<const float4*>(vb + vi));
    const float4 b = __ldg(reinterpret_cast<const float4*>(vb + vi) + 1);
    const float4 c = __ldg(reinterpret_cast<const float4*>(vb + vi) + 2);
    Vtx o;
    // Mat4 * Vec4 with w = 1: ((c0*x + c1*y) + c2*z) + c3*1 (src/renderer.rs:504-511).
    o.cx = ((mvp[0] * a.x + mvp[4] * a.y) + mvp[8] * a.z) + mvp[12];
    o.cy = ((mvp[1] * a.x + mvp[5] * a.y) + mvp[9] * a.z) + mvp[13];
    o.cz = ((mvp[2] * a.x + mvp[6] * a.y) + mvp[10] * a.z) + mvp[14];
    o.cw = ((mvp[3] * a.x + mvp[7] * a.y) + mvp[11] * a.z) + mvp[15];
    o.wx = ((model[0] * a.x + model[4] * a.y) + model[8] * a.z) + model[12];
    o.wy = ((model[1] * a.x + model[5] * a.y) + model[9] * a.z) + model[13];
    o.wz = ((model[2] * a.x + model[6] * a.y) + model[10] * a.z) + model[14];
    // Mat3A * Vec3A: (c0*x + c1*y) + c2*z (src/renderer.rs:514-521).
    o.nx = (model[0] * b.x + model[4] * b.y) + model[8] * b.z;
    o.ny = (model[1] * b.x + model[5] * b.y) + model[9] * b.z;
    o.nz = (model[2] * b.x + model[6] * b.y) + model[10] * b.z;
    o.tx = (model[0] * c.x + model[4] * c.y) + model[8] * c.z;
    o.ty = (model[1] * c.x + model[5] * c.y) + model[9] * c.z;
    o.tz = (model[2] * c.x + model[6] * c.y) + model[10] * c.z;
    o.tw = c.w;
    o.u = a.w;
    o.v = b.w;
    return o;
}

// clip_to_screen_subpixels (src/renderer.rs:834-846).
__device__ __forceinline__ void to_screen(const Vtx& v, float wf, float hf, int32_t& sx, int32_t& sy) {
    const float nx = v.cx / v.cw;
    const float ny = v.cy / v.cw;
    const float fx = ((nx + 1.0f) * wf) / 2.0f;
    const float fy = ((1.0f - ny) * hf) / 2.0f;
    sx = f2i_sat(round_away(fx * 16.0f));
    sy = f2i_sat(round_away(fy * 16.0f));
}

// One atomic per warp: returns a distinct slot of *counter to every active lane.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter) {
    const uint32_t active = __activemask();
    const int leader = __ffs(active) - 1;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if ((int)lane == leader) base = atomicAdd(counter, (uint32_t)__popc(active));
    base = __shfl_sync(active, base, leader);
    return base + (uint32_t)__popc(active & ((1u << lane) - 1u));
}
// One atomic per warp: adds the number of active lanes with `pred` set.
__device__ __forceinline__ void warp_count(uint32_t* counter, bool pred) {
    const uint32_t active = __activemask();
    const uint32_t b = __ballot_sync(active, pred);
    if ((int)(threadIdx.x & 31u) == __ffs(active) - 1 && b) atomicAdd(counter, (uint32_t)__popc(b));
}

// Warp-aggregated atomicAdd of 1 on counter[idx].
__device__ __forceinline__ void agg_inc(uint32_t* counter, uint32_t idx) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, idx);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(counter + idx, (uint32_t)__popc(peers));
}

// Iterate the scheduling tiles a setup triangle touches. f(stile) is called
// once per (triangle, scheduling tile) pair. Mirrors the bin loop of
// bin_triangle (src/renderer.rs:756-830) restricted to real tiles (the
// reference's x == tiles_x column aliases into the next row's tile 0 and only
// ever yields an empty rect or an exact duplicate packet).
template <typename F>
__device__ __forceinline__ void for_each_stile(const DView& v, int32_t S, int32_t mnx, int32_t mny, int32_t mxx,
                                               int32_t mxy, F f) {
    const int32_t bx0 = mnx / kRefTile, by0 = mny / kRefTile;
    const int32_t bx1 = min((mxx + kRefTile - 1) / kRefTile, v.tiles_x);
    const int32_t by1 = min((mxy + kRefTile - 1) / kRefTile, v.tiles_y);
    for (int32_t ty = by0; ty < by1; ++ty) {
        for (int32_t tx = bx0; tx < bx1; ++tx) {
            const int32_t x0 = max(mnx, tx * kRefTile), y0 = max(mny, ty * kRefTile);
            const int32_t x1 = min(mxx, tx * kRefTile + kRefTile), y1 = min(mxy, ty * kRefTile + kRefTile);
            if (x1 - x0 < 1 || y1 - y0 < 1) continue;
            const int32_t sx0 = x0 / S, sx1 = (x1 - 1) / S;
            const int32_t sy0 = y0 / S, sy1 = (y1 - 1) / S;
            for (int32_t sy = sy0; sy <= sy1; ++sy)
                for (int32_t sx = sx0; sx <= sx1; ++sx) f(v.stile_base + (uint32_t)(sy * v.stiles_x + sx));
        }
    }
}

// Occlusion culling runs for scheduling tiles of at least this many pixels
// (the raster drops packets hidden behind the depths of earlier rounds).
#ifndef SWR_CULL_MIN_TILE
#define SWR_CULL_MIN_TILE 64
#endif

// bin_triangle (src/renderer.rs:668-831): setup + count. Returns true when
// the triangle covers at least one tile; its records are then in r and q.
__device__ bool setup_triangle(const FrameArgs& a, const DView& view, const Vtx& v0, const Vtx& v1, const Vtx& v2,
                               uint32_t seq8, uint32_t static_id, uint32_t material, uint32_t view_idx,
                               RecRaster& r, RecShade& q) {
    int32_t p0x, p0y, p1x, p1y, p2x, p2y;
    to_screen(v0, view.width_f, view.height_f, p0x, p0y);
    to_screen(v1, view.width_f, view.height_f, p1x, p1y);
    to_screen(v2, view.width_f, view.height_f, p2x, p2y);
    const int32_t area = wsub(wmul(wsub(p1x, p0x), wsub(p2y, p0y)), wmul(wsub(p2x, p0x), wsub(p1y, p0y)));
    if (area > 0) return false;  // back-facing (CW front faces after the y flip)
    const int32_t wsub_px = view.width * kSubpixelScale, hsub_px = view.height * kSubpixelScale;
    const int32_t mns_x = max(min(min(p0x, p1x), p2x), 0);
    const int32_t mns_y = max(min(min(p0y, p1y), p2y), 0);
    const int32_t mxs_x = min(max(max(p0x, p1x), p2x), wsub_px);
    const int32_t mxs_y = min(max(max(p0y, p1y), p2y), hsub_px);
    const int32_t mnx = mns_x >> kSubpixelShift, mny = mns_y >> kSubpixelShift;
    const int32_t mxx = wadd(mxs_x, kSubpixelScale) >> kSubpixelShift;
    const int32_t mxy = wadd(mxs_y, kSubpixelScale) >> kSubpixelShift;

    uint32_t n = 0;
    const int32_t S = (int32_t)a.sched_tile;
    for_each_stile(view, S, mnx, mny, mxx, mxy, [&](uint32_t) { ++n; });
    if (n == 0) return false;

    // Interpolator setup (src/renderer.rs:699-754).
    const float ooa = 1.0f / i2f(wabs(area));
    const float oow0 = 1.0f / v0.cw, oow1 = 1.0f / v1.cw, oow2 = 1.0f / v2.cw;
    const float zow0 = v0.cz * oow0, zow1 = v1.cz * oow1, zow2 = v2.cz * oow2;
    const float u0 = v0.u * oow0, u1 = v1.u * oow1, u2 = v2.u * oow2;
    const float w0 = v0.v * oow0, w1 = v1.v * oow1, w2 = v2.v * oow2;
    const float dx1 = i2f(wsub(p1x, p0x)), dx2 = i2f(wsub(p2x, p0x));
    const float dy1 = i2f(wsub(p1y, p0y)), dy2 = i2f(wsub(p2y, p0y));
    const float du1 = u1 - u0, du2 = u2 - u0, dv1 = w1 - w0, dv2 = w2 - w0;
    const float du_dx = du1 * dy2 - du2 * dy1;
    const float du_dy = du2 * dx1 - du1 * dx2;
    const float dv_dx = dv1 * dy2 - dv2 * dy1;
    const float dv_dy = dv2 * dx1 - dv1 * dx2;
    const float s = ooa * 16.0f;

    r.p[0] = p0x; r.p[1] = p0y; r.p[2] = p1x; r.p[3] = p1y; r.p[4] = p2x; r.p[5] = p2y;
    r.bb[0] = (uint16_t)mnx; r.bb[1] = (uint16_t)mny; r.bb[2] = (uint16_t)mxx; r.bb[3] = (uint16_t)mxy;
    r.ooa = ooa;
    r.zow[0] = zow0; r.zow[1] = zow1 - zow0; r.zow[2] = zow2 - zow0;
    r.oow[0] = oow0; r.oow[1] = oow1 - oow0; r.oow[2] = oow2 - oow0;
    r.seq8 = seq8;
    r.material = material;
    r.view = view_idx;
    r.zfloor = 0u;  // taken by k_scatter when the frame culls
    r.pad = 0u;
    q.nrm[0] = v0.nx; q.nrm[1] = v0.ny; q.nrm[2] = v0.nz;
    q.nrm[3] = v1.nx - v0.nx; q.nrm[4] = v1.ny - v0.ny; q.nrm[5] = v1.nz - v0.nz;
    q.nrm[6] = v2.nx - v0.nx; q.nrm[7] = v2.ny - v0.ny; q.nrm[8] = v2.nz - v0.nz;
    q.tan[0] = v0.tx; q.tan[1] = v0.ty; q.tan[2] = v0.tz;
    q.tan[3] = v1.tx - v0.tx; q.tan[4] = v1.ty - v0.ty; q.tan[5] = v1.tz - v0.tz;
    q.tan[6] = v2.tx - v0.tx; q.tan[7] = v2.ty - v0.ty; q.tan[8] = v2.tz - v0.tz;
    q.tsign[0] = v0.tw; q.tsign[1] = v1.tw - v0.tw; q.tsign[2] = v2.tw - v0.tw;
    q.uow[0] = u0; q.uow[1] = u1 - u0; q.uow[2] = u2 - u0;
    q.vow[0] = w0; q.vow[1] = w1 - w0; q.vow[2] = w2 - w0;
    const float px0 = v0.wx * oow0, py0 = v0.wy * oow0, pz0 = v0.wz * oow0;
    const float px1 = v1.wx * oow1, py1 = v1.wy * oow1, pz1 = v1.wz * oow1;
    const float px2 = v2.wx * oow2, py2 = v2.wy * oow2, pz2 = v2.wz * oow2;
    q.pww[0] = px0; q.pww[1] = py0; q.pww[2] = pz0;
    q.pww[3] = px1 - px0; q.pww[4] = py1 - py0; q.pww[5] = pz1 - pz0;
    q.pww[6] = px2 - px0; q.pww[7] = py2 - py0; q.pww[8] = pz2 - pz0;
    q.du_dv[0] = du_dx * s; q.du_dv[1] = du_dy * s; q.du_dv[2] = dv_dx * s; q.du_dv[3] = dv_dy * s;
    q.static_id = static_id;
    // Average z for the per-tile translucency sort (src/renderer.rs:765-774).
    const bool translucent = (material & kRecTransBit) != 0u;
    q.pad[0] = translucent ? __float_as_uint(((v0.cz + v1.cz) + v2.cz) / 3.0f) : 0u;
    q.pad[1] = q.pad[2] = 0;
    const uint32_t bin_off = translucent ? a.dyn->n_stiles : 0u;
    for_each_stile(view, S, mnx, mny, mxx, mxy, [&](uint32_t st) { agg_inc(a.tile_count, bin_off + st); });
    return true;
}

__device__ __forceinline__ void store_records(const FrameArgs& a, uint32_t slot, const RecRaster& r,
                                              const RecShade& q) {
    const float4* sr = reinterpret_cast<const float4*>(&r);
    float4* dr = reinterpret_cast<float4*>(a.rec_r + slot);
#pragma unroll
    for (int i = 0; i < 5; ++i) dr[i] = sr[i];
    const float4* sq = reinterpret_cast<const float4*>(&q);
    float4* dq = reinterpret_cast<float4*>(a.rec_s + slot);
#pragma unroll
    for (int i = 0; i < 11; ++i) dq[i] = sq[i];
}

// --------------------------------------------------------------------------
// Draw list: render_scene's front half (src/renderer.rs:201-210, 357-420).
// The host sorts each view's nodes nearest first (compute_nodes_by_distance)
// into node slots, view after view. Per slot the device forms the node's MVP,
// tests every primitive's world bounding sphere against the view frustum and
// emits a draw, with its 256-triangle chunks, for each primitive not
// outside. k_reset's CTAs count per block of 256 slots and the last of them
// turns the block totals into offsets (so draws keep the host loop's order);
// k_draw_emit scans within each block and writes the draws.
// --------------------------------------------------------------------------
struct DrawCount {
    uint32_t draws, tris, chunks;
};

// Vec4::length with the pairwise dot (x*x + y*y) + (z*z + w*w).
__device__ __forceinline__ float len4(const float* c) {
    return __fsqrt_rn((c[0] * c[0] + c[1] * c[1]) + (c[2] * c[2] + c[3] * c[3]));
}

// Frustum class of a world-space sphere (test_sphere_frustum,
// src/renderer.rs:130-142): 0 outside, 1 inside, 2 intersecting.
__device__ __forceinline__ uint32_t sphere_class(const DView& v, const float ws[4]) {
    const float* m = v.cam_view;
    float cv[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) cv[r] = ((m[r] * ws[0] + m[4 + r] * ws[1]) + m[8 + r] * ws[2]) + m[12 + r] * 1.0f;
    uint32_t res = 1u;
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const float* pl = v.cam_planes + 4 * i;
        const float d = (pl[0] * cv[0] + pl[1] * cv[1]) + (pl[2] * cv[2] + pl[3] * cv[3]);
        if (d < -ws[3]) return 0u;
        if (d < ws[3]) res = 2u;
    }
    return res;
}

__device__ __forceinline__ uint32_t find_view_by_slot(const FrameArgs& a, uint32_t i) {
    uint32_t lo = 0, hi = a.dyn->n_views - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (a.views[mid].order_base <= i) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Draws of one node (render_node + render_mesh): counted, and with EMIT
// written from the given bases; `trans` is set when a translucent draw is
// written.
template <bool EMIT>
__device__ DrawCount node_draws(const FrameArgs& a, uint32_t vi, const DView& v, const DScene& sc, uint32_t node,
                                DrawCount base, bool& trans) {
    DrawCount c{0u, 0u, 0u};
    const DNodeInfo* np = sc.node_info + node;
    const uint32_t n_total = np->n_total;
    if (n_total == 0u) return c;
    float t[16];
    {
        const float4* x = reinterpret_cast<const float4*>(np->xform);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float4 q = __ldg(x + i);
            t[4 * i] = q.x;
            t[4 * i + 1] = q.y;
            t[4 * i + 2] = q.z;
            t[4 * i + 3] = q.w;
        }
    }
    const uint32_t entry_begin = np->entry_begin, n_opaque = np->n_opaque, node_tri_base = np->tri_id_base;
    const float max_scale = ((len4(t) + len4(t + 4)) + len4(t + 8)) / 3.0f;
    float mvp[16];
    if (EMIT) {
        const float* p = v.cam_view_project;
#pragma unroll
        for (int col = 0; col < 4; ++col) {
            const float* b = t + 4 * col;
#pragma unroll
            for (int r = 0; r < 4; ++r) mvp[4 * col + r] = ((p[r] * b[0] + p[4 + r] * b[1]) + p[8 + r] * b[2]) + p[12 + r] * b[3];
        }
    }
    for (uint32_t k = 0; k < n_total; ++k) {
        const DMeshEntry me = sc.mesh_entries[entry_begin + k];
        float ws[4];
        // transform_point3: ((c0*x + c1*y) + c2*z) + c3.
#pragma unroll
        for (int r = 0; r < 3; ++r) ws[r] = ((t[r] * me.sphere[0] + t[4 + r] * me.sphere[1]) + t[8 + r] * me.sphere[2]) + t[12 + r];
        ws[3] = me.sphere[3] * max_scale;
        const uint32_t cls = sphere_class(v, ws);
        if (cls == 0u) continue;
        const uint32_t tc = me.tri_count;
        if (tc == 0u) continue;
        const uint32_t nch = (tc + (uint32_t)kChunkTris - 1u) / (uint32_t)kChunkTris;
        if (EMIT) {
            const uint32_t di = base.draws + c.draws, ci = base.chunks + c.chunks;
            const bool translucent = k >= n_opaque;
            if (di < a.draw_cap && (uint64_t)ci + nch <= a.chunk_cap &&
                (uint64_t)base.tris + c.tris + tc <= a.tri_cap) {
                DDraw d;
#pragma unroll
                for (int i = 0; i < 16; ++i) d.mvp[i] = mvp[i];
                d.node = node;
                d.prim = me.prim;
                d.view = vi;
                d.clip = cls == 2u ? 1u : 0u;
                d.tri_begin = base.tris + c.tris;
                d.tri_count = tc;
                d.static_base = node_tri_base + me.tri_id_base;
                d.scene = v.scene;
                d.translucent = translucent ? 1u : 0u;
                d.pad[0] = d.pad[1] = d.pad[2] = 0u;
                a.draws[di] = d;
                for (uint32_t j = 0; j < nch; ++j) a.chunks[ci + j] = DChunk{di, j * (uint32_t)kChunkTris};
                trans |= translucent;
            } else {
                atomicOr(&a.counters->status, ST_DRAW_OVERFLOW);
            }
        }
        c.draws += 1u;
        c.tris += tc;
        c.chunks += nch;
    }
    return c;
}

// Block-wide sum (SUM) or exclusive scan of three counters over NT threads;
// `total` gets the block's sums.
template <int NT>
__device__ DrawCount block_scan3(DrawCount x, DrawCount& total, uint32_t* sm) {
    constexpr int NW = NT / 32;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    DrawCount inc = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t d = __shfl_up_sync(0xFFFFFFFFu, inc.draws, o);
        const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, inc.tris, o);
        const uint32_t c = __shfl_up_sync(0xFFFFFFFFu, inc.chunks, o);
        if (lane >= (uint32_t)o) {
            inc.draws += d;
            inc.tris += t;
            inc.chunks += c;
        }
    }
    __syncthreads();
    if (lane == 31u) {
        sm[warp] = inc.draws;
        sm[NW + warp] = inc.tris;
        sm[2 * NW + warp] = inc.chunks;
    }
    __syncthreads();
    DrawCount before{0u, 0u, 0u};
    total = DrawCount{0u, 0u, 0u};
#pragma unroll
    for (int w = 0; w < NW; ++w) {
        if ((uint32_t)w < warp) {
            before.draws += sm[w];
            before.tris += sm[NW + w];
            before.chunks += sm[2 * NW + w];
        }
        total.draws += sm[w];
        total.tris += sm[NW + w];
        total.chunks += sm[2 * NW + w];
    }
    return DrawCount{before.draws + inc.draws - x.draws, before.tris + inc.tris - x.tris,
                     before.chunks + inc.chunks - x.chunks};
}

constexpr int kSlotBlock = 256;  // node slots per draw-list block

__device__ __forceinline__ DrawCount slot_count(const FrameArgs& a, uint32_t i, uint32_t n) {
    if (i >= n) return DrawCount{0u, 0u, 0u};
    const uint32_t vi = find_view_by_slot(a, i);
    const DView& v = a.views[vi];
    bool unused = false;
    return node_draws<false>(a, vi, v, a.scenes[v.scene], a.node_order[i], DrawCount{0u, 0u, 0u}, unused);
}

// Frame totals from the draw-list sums; a frame past the capacities draws
// nothing and reports its totals, and the host renders it again with grown
// buffers.
__device__ __forceinline__ void set_draw_totals(const FrameArgs& a, const DrawCount& total) {
    if (total.tris > a.tri_cap || total.chunks > a.chunk_cap || total.draws > a.draw_cap) {
        atomicOr(&a.counters->status, ST_DRAW_OVERFLOW);
        a.dyn->n_chunks = 0u;
        a.dyn->tri_total = 0u;
    } else {
        a.dyn->n_chunks = total.chunks;
        a.dyn->tri_total = total.tris;
    }
    a.counters->draw_tris = total.tris;
    a.counters->draw_chunks = total.chunks;
    a.counters->draw_count = total.draws;
}

// Counts per block of 256 node slots (run by k_reset's CTAs); the last CTA
// to finish turns the block totals into exclusive offsets and sets the
// frame totals. No CTA waits for another. A frame of at most 256 slots is
// counted, scanned and emitted by CTA 0 alone (k_draw_emit then has nothing
// to do).
__device__ void draw_count_blocks(const FrameArgs& a) {
    __shared__ uint32_t sm[3 * (kSlotBlock / 32)];
    __shared__ bool last;
    const uint32_t n = a.dyn->n_slots;
    const uint32_t nb = (n + kSlotBlock - 1) / kSlotBlock;
    if (nb <= 1u) {
        if (blockIdx.x != 0) return;
        const uint32_t i = threadIdx.x;
        const DrawCount mine = slot_count(a, i, n);
        DrawCount total;
        const DrawCount ex = block_scan3<kSlotBlock>(mine, total, sm);
        if (threadIdx.x == 0) set_draw_totals(a, total);
        if (mine.draws == 0u || total.tris > a.tri_cap || total.chunks > a.chunk_cap || total.draws > a.draw_cap)
            return;
        const uint32_t vi = find_view_by_slot(a, i);
        const DView& v = a.views[vi];
        bool trans = false;
        node_draws<true>(a, vi, v, a.scenes[v.scene], a.node_order[i], ex, trans);
        if (trans) atomicOr(&a.views[vi].flags, kViewTranslucent);
        return;
    }
    for (uint32_t b = blockIdx.x; b < nb; b += gridDim.x) {
        DrawCount t;
        block_scan3<kSlotBlock>(slot_count(a, b * kSlotBlock + threadIdx.x, n), t, sm);
        if (threadIdx.x == 0) a.slot_blocks[b] = make_uint4(t.draws, t.tris, t.chunks, 0u);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&a.counters->draw_done, 1u) == gridDim.x - 1u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    const uint32_t per = (nb + kSlotBlock - 1) / kSlotBlock;
    const uint32_t b0 = threadIdx.x * per, b1 = min(b0 + per, nb);
    DrawCount mine{0u, 0u, 0u};
    for (uint32_t b = b0; b < b1; ++b) {
        const uint4 t = __ldcg(a.slot_blocks + b);
        mine.draws += t.x;
        mine.tris += t.y;
        mine.chunks += t.z;
    }
    DrawCount total;
    DrawCount run = block_scan3<kSlotBlock>(mine, total, sm);
    for (uint32_t b = b0; b < b1; ++b) {
        const uint4 t = __ldcg(a.slot_blocks + b);
        a.slot_blocks[b] = make_uint4(run.draws, run.tris, run.chunks, 0u);
        run.draws += t.x;
        run.tris += t.y;
        run.chunks += t.z;
    }
    if (threadIdx.x == 0) set_draw_totals(a, total);
}

__global__ void __launch_bounds__(kSlotBlock) k_draw_emit(FrameArgs a) {
    __shared__ uint32_t sm[3 * (kSlotBlock / 32)];
    if (blockIdx.x == 0 && threadIdx.x == 0) a.counters->draw_done = 0u;  // for the next frame
    const uint32_t n = a.dyn->n_slots;
    const uint32_t i = blockIdx.x * kSlotBlock + threadIdx.x;
    if (n <= (uint32_t)kSlotBlock || blockIdx.x * kSlotBlock >= n || a.dyn->n_chunks == 0u) return;
    const DrawCount mine = slot_count(a, i, n);
    DrawCount t;
    const DrawCount ex = block_scan3<kSlotBlock>(mine, t, sm);
    if (mine.draws == 0u) return;
    const uint4 base = a.slot_blocks[blockIdx.x];
    const uint32_t vi = find_view_by_slot(a, i);
    const DView& v = a.views[vi];
    bool trans = false;
    node_draws<true>(a, vi, v, a.scenes[v.scene], a.node_order[i],
                     DrawCount{base.x + ex.draws, base.y + ex.tris, base.z + ex.chunks}, trans);
    if (trans) atomicOr(&a.views[vi].flags, kViewTranslucent);
}

__global__ void __launch_bounds__(256) k_reset(FrameArgs a) {
    const uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t n = a.dyn->n_bins;
    for (uint32_t i = i0; i < n; i += gridDim.x * blockDim.x) a.tile_count[i] = 0u;
    if (i0 == 0) {
        a.counters->status = 0u;
        a.counters->clip_queue = 0u;
        a.counters->extra_used = 0u;
        a.counters->setup_tris = 0u;
        a.counters->pairs = 0ull;
        a.counters->work_next = 0u;
        a.counters->trans_next = 0u;
        a.counters->trans_packets = 0u;
        a.counters->culled = 0u;
        a.counters->clip_path = 0u;
        a.counters->draw_tris = a.gpu_draws ? 0u : a.dyn->tri_total;
    }
    if (a.gpu_draws) draw_count_blocks(a);
}

// True when clip_against_frustum (src/renderer.rs:579-665) returns nothing
// for this triangle without producing any intersection: at the first plane
// (near, far, right, left, top, bottom) that some vertex is outside of, all
// three are outside. Earlier planes then left the triangle untouched, so the
// clipper's polygon becomes empty at exactly that plane.
__device__ __forceinline__ bool clip_rejects_all(const Vtx& a, const Vtx& b, const Vtx& c) {
    const float da[6] = {a.cz + a.cw, -a.cz + a.cw, a.cx + a.cw, -a.cx + a.cw, a.cy + a.cw, -a.cy + a.cw};
    const float db[6] = {b.cz + b.cw, -b.cz + b.cw, b.cx + b.cw, -b.cx + b.cw, b.cy + b.cw, -b.cy + b.cw};
    const float dc[6] = {c.cz + c.cw, -c.cz + c.cw, c.cx + c.cw, -c.cx + c.cw, c.cy + c.cw, -c.cy + c.cw};
#pragma unroll
    for (int p = 0; p < 6; ++p) {
        const bool ia = da[p] >= 0.0f, ib = db[p] >= 0.0f, ic = dc[p] >= 0.0f;
        if (ia && ib && ic) continue;
        return !ia && !ib && !ic;
    }
    return false;
}

// Record material word: translucent primitives (no alpha test on their path,
// src/shader.rs:66-76) or opaque ones with the alpha-test flag.
__device__ __forceinline__ uint32_t record_material(const DScene& sc, const DDraw& d, uint32_t material) {
    if (d.translucent) return material | kRecTransBit;
    return material | ((sc.materials[material].flags & MAT_ALPHA_TESTED) ? kRecAlphaBit : 0u);
}

__device__ __forceinline__ bool vtx_inside_all(const Vtx& v) {
    // plane.dot(pos_clip) >= 0 for the six planes of src/renderer.rs:581-588;
    // every product is by 0 or +-1, so the dot is exactly +-c + w.
    return (v.cz + v.cw >= 0.0f) && (-v.cz + v.cw >= 0.0f) && (v.cx + v.cw >= 0.0f) && (-v.cx + v.cw >= 0.0f) &&
           (v.cy + v.cw >= 0.0f) && (-v.cy + v.cw >= 0.0f);
}

// Thread per triangle of a 256-triangle chunk of one draw.
__device__ __forceinline__ void frontend_triangle(const FrameArgs& a, uint32_t chunk) {
    const DChunk ch = a.chunks[chunk];
    const DDraw& d = a.draws[ch.draw];
    // The CTA's triangles are one draw's: count the chunk once for the
    // reference's clip path (every triangle of an intersecting primitive).
    if (threadIdx.x == 0 && d.clip) atomicAdd(&a.counters->clip_path, min((uint32_t)kChunkTris, d.tri_count - ch.tri_start));
    const uint32_t local = ch.tri_start + threadIdx.x;
    if (local >= d.tri_count) return;
    const uint32_t g = d.tri_begin + local;
    const DScene& sc = a.scenes[d.scene];
    const DView& view = a.views[d.view];
    const DPrimitive pr = sc.prims[d.prim];
    const float* model = sc.node_xform + 16u * d.node;
    const uint32_t* ib = sc.indices + pr.idx_base + 3u * local;
    const uint32_t i0 = __ldg(ib), i1 = __ldg(ib + 1), i2 = __ldg(ib + 2);
    const Vtx v0 = transform_vertex(sc.vertices, pr.vtx_base + i0, model, d.mvp);
    const Vtx v1 = transform_vertex(sc.vertices, pr.vtx_base + i1, model, d.mvp);
    const Vtx v2 = transform_vertex(sc.vertices, pr.vtx_base + i2, model, d.mvp);
    if (d.clip && !(vtx_inside_all(v0) && vtx_inside_all(v1) && vtx_inside_all(v2))) {
        if (clip_rejects_all(v0, v1, v2)) {  // the clipper would return an empty polygon
            a.tri_state[g] = 3;
            return;
        }
        const uint32_t q = warp_append(&a.counters->clip_queue);
        if (q < a.clip_cap) {
            a.clip_queue[q] = make_uint2(g, ch.draw);
        } else {
            atomicOr(&a.counters->status, ST_QUEUE_OVERFLOW);
        }
        a.tri_state[g] = 2;
        return;
    }
    // All three vertices inside: the clipper would return the triangle unchanged.
    const uint32_t mword = record_material(sc, d, pr.material);
    RecRaster r;
    RecShade q;
    const bool ok = setup_triangle(a, view, v0, v1, v2, g << 3, d.static_base + local, mword, d.view, r, q);
    if (ok) store_records(a, g, r, q);
    a.tri_state[g] = ok ? 1 : 0;
    warp_count(&a.counters->setup_tris, ok);
}

// Thread per triangle of a 256-triangle chunk, CTA per chunk (a loop over
// chunks per CTA made the kernel spill).
// Four CTAs per SM (64 registers, a few spilled): 4K front end 0.161 ms,
// against 0.164 at three (80 registers) and 0.204 at two (108 registers).
#ifndef SWR_FRONTEND_MIN_BLOCKS
#define SWR_FRONTEND_MIN_BLOCKS 4
#endif
__global__ void __launch_bounds__(kChunkTris, SWR_FRONTEND_MIN_BLOCKS) k_frontend(FrameArgs a) {
    if (blockIdx.x < a.dyn->n_chunks) frontend_triangle(a, blockIdx.x);
}

// intersect (src/renderer.rs:598-609).
__device__ __forceinline__ Vtx lerp_vtx(const Vtx& a, const Vtx& b, float t) {
    Vtx o;
    o.cx = a.cx + (b.cx - a.cx) * t; o.cy = a.cy + (b.cy - a.cy) * t;
    o.cz = a.cz + (b.cz - a.cz) * t; o.cw = a.cw + (b.cw - a.cw) * t;
    o.wx = a.wx + (b.wx - a.wx) * t; o.wy = a.wy + (b.wy - a.wy) * t; o.wz = a.wz + (b.wz - a.wz) * t;
    o.nx = a.nx + (b.nx - a.nx) * t; o.ny = a.ny + (b.ny - a.ny) * t; o.nz = a.nz + (b.nz - a.nz) * t;
    o.tx = a.tx + (b.tx - a.tx) * t; o.ty = a.ty + (b.ty - a.ty) * t;
    o.tz = a.tz + (b.tz - a.tz) * t; o.tw = a.tw + (b.tw - a.tw) * t;
    o.u = a.u + (b.u - a.u) * t; o.v = a.v + (b.v - a.v) * t;
    return o;
}
__device__ __forceinline__ float plane_dist(const Vtx& v, int p) {
    switch (p) {
        case 0: return v.cz + v.cw;   // near:   z + w
        case 1: return -v.cz + v.cw;  // far:   -z + w
        case 2: return v.cx + v.cw;   // right:  x + w
        case 3: return -v.cx + v.cw;  // left:  -x + w
        case 4: return v.cy + v.cw;   // top:    y + w
        default: return -v.cy + v.cw; // bottom: -y + w
    }
}

__global__ void __launch_bounds__(128) k_clip(FrameArgs a) {
    const uint32_t nq = min(a.counters->clip_queue, a.clip_cap);
    const uint32_t tri_total = a.dyn->tri_total;
    for (uint32_t q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
        const uint2 e = a.clip_queue[q];
        const uint32_t g = e.x;
        const DDraw& d = a.draws[e.y];
        const uint32_t local = g - d.tri_begin;
        const DScene& sc = a.scenes[d.scene];
        const DView& view = a.views[d.view];
        const DPrimitive pr = sc.prims[d.prim];
        const uint32_t mword = record_material(sc, d, pr.material);
        const float* model = sc.node_xform + 16u * d.node;
        const uint32_t* ib = sc.indices + pr.idx_base + 3u * local;
        Vtx poly[16], np[16];
        poly[0] = transform_vertex(sc.vertices, pr.vtx_base + __ldg(ib), model, d.mvp);
        poly[1] = transform_vertex(sc.vertices, pr.vtx_base + __ldg(ib + 1), model, d.mvp);
        poly[2] = transform_vertex(sc.vertices, pr.vtx_base + __ldg(ib + 2), model, d.mvp);
        int len = 3;
        for (int p = 0; p < 6 && len > 0; ++p) {
            int nl = 0;
            for (int i = 0; i < len; ++i) {
                const Vtx& cur = poly[i];
                const Vtx& prv = poly[(i + len - 1) % len];
                const float dc = plane_dist(cur, p), dp = plane_dist(prv, p);
                const bool cin = dc >= 0.0f, pin = dp >= 0.0f;
                if (cin) {
                    if (!pin) np[nl++] = lerp_vtx(prv, cur, dp / (dp - dc));
                    np[nl++] = cur;
                } else if (pin) {
                    np[nl++] = lerp_vtx(prv, cur, dp / (dp - dc));
                }
            }
            for (int i = 0; i < nl; ++i) poly[i] = np[i];
            len = nl;
        }
        uint32_t any = 0;
        if (len >= 3) {
            const int fans = len - 2;
            uint32_t base = 0;
            if (fans > 1) {
                base = atomicAdd(&a.counters->extra_used, (uint32_t)(fans - 1));
                if (base + (uint32_t)(fans - 1) > a.extra_cap) {
                    atomicOr(&a.counters->status, ST_CLIP_OVERFLOW);
                    a.tri_state[g] = 0;
                    continue;
                }
                a.fan_base[g] = tri_total + base;
            }
            for (int f = 0; f < fans; ++f) {
                const uint32_t slot = f == 0 ? g : tri_total + base + (uint32_t)(f - 1);
                RecRaster r;
                RecShade q;
                const bool ok = setup_triangle(a, view, poly[0], poly[f + 1], poly[f + 2], (g << 3) | (uint32_t)f,
                                               d.static_base + local, mword, d.view, r, q);
                if (ok) store_records(a, slot, r, q);
                if (ok) {
                    atomicAdd(&a.counters->setup_tris, 1u);
                    if (f == 0) any = 1;
                } else if (f > 0) {
                    // Mark the unused extra slot so the scatter skips it.
                    a.rec_r[slot].view = 0xFFFFFFFFu;
                }
            }
        }
        a.tri_state[g] = any ? 1 : 3;
    }
}

// Bucket of a bin of c packets for the raster visiting order: 0 for an empty
// bin, else two buckets per octave of c. Scheduling tiles below kOrderMinTile
// px are cheap enough that the raster visits them in screen order.
constexpr int kOrderBuckets = 66;
constexpr uint32_t kOrderMinTile = 32;
__device__ __forceinline__ uint32_t order_bucket(uint32_t c) {
    if (c == 0u) return 0u;
    const uint32_t bits = 32u - (uint32_t)__clz(c);
    const uint32_t half = bits >= 2u ? (c >> (bits - 2u)) & 1u : 0u;
    return 2u * bits - 1u + half;
}

// Exclusive scan of tile counts (single CTA). Also seeds the scatter cursors
// and writes the raster's tile visiting order. Each warp owns a contiguous
// run of 32-bin chunks and reads kScanUnroll chunks at once, so the loads of
// a batch of many views (10^5 bins) overlap instead of following one another.
constexpr int kScanUnroll = 8;
__global__ void __launch_bounds__(1024) k_scan(FrameArgs a) {
    __shared__ uint32_t wsum[32];
    __shared__ uint32_t bucket[kOrderBuckets];
    const uint32_t n = a.dyn->n_bins;
    const uint32_t n_st = a.dyn->n_stiles;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    // Raster visiting order: opaque scheduling tiles, heaviest bins first
    // (longest job first over the persistent CTAs, so the kernel does not end
    // on a late heavy tile). Bins are bucketed by half-octave of their size;
    // order within a bucket is arbitrary, since tiles are independent.
    const bool order = a.sched_tile >= kOrderMinTile;
    if (threadIdx.x < kOrderBuckets) bucket[threadIdx.x] = 0u;
    const uint32_t chunks = (n + 31u) >> 5;
    const uint32_t per = (chunks + 31u) >> 5;
    const uint32_t cb = min(warp * per, chunks), ce = min(cb + per, chunks);
    uint32_t s = 0;
    for (uint32_t c = cb; c < ce; c += kScanUnroll) {
        uint32_t v[kScanUnroll];
#pragma unroll
        for (int k = 0; k < kScanUnroll; ++k) {
            const uint32_t i = ((c + k) << 5) + lane;
            v[k] = (c + k < ce && i < n) ? a.tile_count[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kScanUnroll; ++k) s += v[k];
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, off);
    if (lane == 0) wsum[warp] = s;
    __syncthreads();
    uint32_t run, total;
    {
        const uint32_t x = wsum[lane];
        uint32_t incl = x;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= (uint32_t)off) incl += y;
        }
        run = __shfl_sync(0xFFFFFFFFu, incl - x, warp);
        total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    for (uint32_t c = cb; c < ce; c += kScanUnroll) {
        uint32_t v[kScanUnroll];
#pragma unroll
        for (int k = 0; k < kScanUnroll; ++k) {
            const uint32_t i = ((c + k) << 5) + lane;
            v[k] = (c + k < ce && i < n) ? a.tile_count[i] : 0u;
        }
#pragma unroll
        for (int k = 0; k < kScanUnroll; ++k) {
            uint32_t incl = v[k];
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, incl, off);
                if (lane >= (uint32_t)off) incl += y;
            }
            const uint32_t i = ((c + k) << 5) + lane;
            if (c + k < ce && i < n) {
                const uint32_t o = run + incl - v[k];
                a.tile_offset[i] = o;
                a.tile_cursor[i] = o;
            }
            if (order) {
                // Lanes of a warp that share a bucket add to it once (most
                // bins of a frame fall in a few buckets).
                const uint32_t key = (c + k < ce && i < n_st) ? order_bucket(v[k]) : (uint32_t)kOrderBuckets;
                const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key);
                if (key < (uint32_t)kOrderBuckets && lane == (uint32_t)(__ffs(peers) - 1))
                    atomicAdd(&bucket[key], (uint32_t)__popc(peers));
            }
            run += __shfl_sync(0xFFFFFFFFu, incl, 31);
        }
    }
    if (threadIdx.x == 0) {
        a.tile_offset[n] = total;
        a.counters->pairs = total;
        if ((uint64_t)total > a.bin_cap) atomicOr(&a.counters->status, ST_BIN_OVERFLOW);
    }
    if (!order) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int k = kOrderBuckets - 1; k >= 0; --k) {
            const uint32_t c = bucket[k];
            bucket[k] = acc;
            acc += c;
        }
    }
    __syncthreads();
    // The counts are no longer needed, so the order is written over them;
    // bin sizes come from the offsets.
    constexpr int kPlaceUnroll = 4;
    const uint32_t n_st_pad = (n_st + 1023u) & ~1023u;
    for (uint32_t i0 = threadIdx.x; i0 < n_st_pad; i0 += 1024u * kPlaceUnroll) {
        uint32_t key[kPlaceUnroll];
#pragma unroll
        for (int u = 0; u < kPlaceUnroll; ++u) {
            const uint32_t i = i0 + 1024u * u;
            key[u] = i < n_st ? order_bucket(a.tile_offset[i + 1] - a.tile_offset[i]) : (uint32_t)kOrderBuckets;
        }
#pragma unroll
        for (int u = 0; u < kPlaceUnroll; ++u) {
            const uint32_t peers = __match_any_sync(0xFFFFFFFFu, key[u]);
            const uint32_t leader = (uint32_t)(__ffs(peers) - 1);
            uint32_t base = 0;
            if (key[u] < (uint32_t)kOrderBuckets && lane == leader) base = atomicAdd(&bucket[key[u]], (uint32_t)__popc(peers));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (key[u] < (uint32_t)kOrderBuckets) a.tile_count[base + __popc(peers & ((1u << lane) - 1u))] = i0 + 1024u * u;
        }
    }
}

// Triangles whose bounding box spans fewer pixels than this take no depth
// floor, so their packets are never culled (0: every triangle takes one).
// Small triangles are most of what culling drops: on the 4K frame, raster +
// scatter took 0.394 + 0.075 ms with a floor for every triangle, 0.421 +
// 0.077 from 16 px, 0.467 + 0.061 from 64 px and 0.506 + 0.058 from 256 px.
#ifndef SWR_FLOOR_MIN_PX
#define SWR_FLOOR_MIN_PX 0
#endif

// Record slots are the frame's main slots [0, T) and the clipper's extra
// slots right after them.
__device__ __forceinline__ void scatter_slot(const FrameArgs& a, uint32_t slot, uint32_t tri_total) {
    if (slot < tri_total) {
        if (a.tri_state[slot] != 1) return;
    } else if (a.rec_r[slot].view == 0xFFFFFFFFu) {
        return;
    }
    const RecRaster& r = a.rec_r[slot];
    const DView& view = a.views[r.view];
    const uint32_t bin_off = (r.material & kRecTransBit) ? a.dyn->n_stiles : 0u;
    if ((int32_t)a.sched_tile >= SWR_CULL_MIN_TILE && !(r.material & kRecTransBit) &&
        (SWR_FLOOR_MIN_PX == 0 ||
         (uint32_t)(r.bb[2] - r.bb[0] + 1) * (uint32_t)(r.bb[3] - r.bb[1] + 1) >= (uint32_t)SWR_FLOOR_MIN_PX)) {
        // The depth floor of the whole triangle for the raster's occlusion
        // culling: every packet's sample coordinates lie below the bbox end,
        // so one floor bounds the depths of all its packets; taken once here
        // instead of per packet and round in the raster.
        float zl;
        if (depth_floor(r.p, r.zow, r.oow, (int32_t)r.bb[2] * kSubpixelScale, (int32_t)r.bb[3] * kSubpixelScale, zl))
            a.rec_r[slot].zfloor = float_to_ordered(zl);
    }
    for_each_stile(view, (int32_t)a.sched_tile, r.bb[0], r.bb[1], r.bb[2], r.bb[3], [&](uint32_t b) {
        const uint32_t st = bin_off + b;
        const uint32_t active = __activemask();
        const uint32_t peers = __match_any_sync(active, st);
        const int leader = __ffs(peers) - 1;
        const uint32_t lane = threadIdx.x & 31u;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(a.tile_cursor + st, (uint32_t)__popc(peers));
        base = __shfl_sync(peers, base, leader);
        const uint32_t rank = __popc(peers & ((1u << lane) - 1u));
        a.bins[base + rank] = slot;
    });
}

__global__ void k_scatter(FrameArgs a) {
    if (a.counters->status & (ST_BIN_OVERFLOW | ST_CLIP_OVERFLOW | ST_QUEUE_OVERFLOW)) return;
    const uint32_t tri_total = a.dyn->tri_total;
    const uint32_t n = tri_total + min(a.counters->extra_used, a.extra_cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        scatter_slot(a, i, tri_total);
}

// --------------------------------------------------------------------------
// Raster
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_view_by_stile(const FrameArgs& a, uint32_t st) {
    uint32_t lo = 0, hi = a.dyn->n_views - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (a.views[mid].stile_base <= st) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Alpha test of one lane (get_alpha_test_mask, src/shader.rs:311-329): the
// mip comes from the packet's du_dv without the per-lane w scale.
__device__ __forceinline__ bool alpha_pass(const DScene& sc, const DMaterial& m, const RecShade& q, float b1, float b2,
                                           float w, uint32_t mip) {
    const DTexture& t = sc.textures[m.tex[TS_BASE]];
    const float u = interp(q.uow, b1, b2) * w;
    const float v = interp(q.vow, b1, b2) * w;
    const uint32_t tx = sample_texel(t, u, v, mip, m.wrap_s[TS_BASE], m.wrap_t[TS_BASE]);
    return c_unorm8[tx & 0xFFu] >= m.alpha_cutoff;
}

// coarse_raster's block reject (src/tilerasterizer.rs:238-269): the block is
// skipped when any edge is negative at all four corner pixel centres.
__device__ __forceinline__ bool block_rejected(const Edge& e12, const Edge& e20, const Edge& e01, int32_t bx,
                                               int32_t by) {
    const float cx0 = i2f(bx + 8), cx1 = i2f(bx + 256 - 8);
    const float cy0 = i2f(by + 8), cy1 = i2f(by + 256 - 8);
    const float m0 = fmaxf(fmaxf(edge_eval(e12, cx0, cy0), edge_eval(e12, cx1, cy0)),
                           fmaxf(edge_eval(e12, cx0, cy1), edge_eval(e12, cx1, cy1)));
    const float m1 = fmaxf(fmaxf(edge_eval(e20, cx0, cy0), edge_eval(e20, cx1, cy0)),
                           fmaxf(edge_eval(e20, cx0, cy1), edge_eval(e20, cx1, cy1)));
    const float m2 = fmaxf(fmaxf(edge_eval(e01, cx0, cy0), edge_eval(e01, cx1, cy0)),
                           fmaxf(edge_eval(e01, cx0, cy1), edge_eval(e01, cx1, cy1)));
    return m0 < 0.0f || m1 < 0.0f || m2 < 0.0f;
}

struct PacketCtx {
    RecRaster r;
    Edge e01, e12, e20;
    int32_t xs, ys, xe, ye;
    bool coarse;
    uint32_t amip;
};

__device__ __forceinline__ void load_packet(const FrameArgs& a, const DScene& sc, uint32_t slot, int32_t tx0,
                                            int32_t ty0, PacketCtx& c) {
    const float4* src = reinterpret_cast<const float4*>(a.rec_r + slot);
    float4* dst = reinterpret_cast<float4*>(&c.r);
#pragma unroll
    for (int i = 0; i < 5; ++i) dst[i] = __ldg(src + i);
    c.e01 = make_edge(c.r.p[0], c.r.p[1], c.r.p[2], c.r.p[3]);
    c.e12 = make_edge(c.r.p[2], c.r.p[3], c.r.p[4], c.r.p[5]);
    c.e20 = make_edge(c.r.p[4], c.r.p[5], c.r.p[0], c.r.p[1]);
    int32_t x0, y0, x1, y1;
    clipped_rect(c.r, tx0, ty0, x0, y0, x1, y1);
    c.coarse = (x1 - x0 > 16) || (y1 - y0 > 16);
    c.xs = (x0 & ~1) * kSubpixelScale;
    c.ys = (y0 & ~1) * kSubpixelScale;
    c.xe = x1 * kSubpixelScale;
    c.ye = y1 * kSubpixelScale;
    c.amip = 0;
    if (c.r.material & kRecAlphaBit) {
        const DMaterial& m = sc.materials[c.r.material & kRecMaterialMask];
        const RecShade& q = a.rec_s[slot];
        c.amip = mip_level(sc.textures[m.tex[TS_BASE]], q.du_dv[0], q.du_dv[1], q.du_dv[2], q.du_dv[3]);
    }
}

// Block index ranges of a coarse packet's 16-px blocks that overlap the
// scheduling tile [s0, s0 + S).
__device__ __forceinline__ void block_range(int32_t start, int32_t end, int32_t s0, int32_t S, int32_t& lo,
                                            int32_t& hi) {
    const int32_t nb = (end - start + 255) >> 8;
    lo = 0;
    hi = nb;  // exclusive
    const int32_t t0 = s0 * 16, t1 = (s0 + S) * 16;
    while (lo < hi && start + 256 * lo + 256 <= t0) ++lo;
    while (hi > lo && start + 256 * (hi - 1) >= t1) --hi;
}

// ---- Regions -------------------------------------------------------------
//
// A region is what one fine_raster call walks (src/tilerasterizer.rs:293-384):
// a whole packet when its rect clipped to the 64-px reference tile is at most
// 16 px both ways, else one unrejected 16-px block of it. Its quads are
// (i, j) = (column, row) from the region origin; the reference reaches quad
// (i, j)'s edge values by adding step_y j times to the origin's values, then
// step_x i times. Origin values and steps are integers held in f32 (products
// and sums of integer-valued floats), so when |origin| + j_max |step_y| +
// i_max |step_x| <= 2^24 every partial sum is an exactly representable
// integer, and the value equals origin + j step_y + i step_x evaluated in any
// grouping. Such regions are "exact": any quad is evaluated directly, one
// quad per lane over all exact regions of a round. The others replay the
// sequential additions, one warp per region.

__device__ __forceinline__ float ru_add(float a, float b) { return __fadd_ru(a, b); }
__device__ __forceinline__ float ru_mul(float a, float b) { return __fmul_ru(a, b); }

// Quad range of a region clipped to the scheduling tile, packed as
// ilo | jlo << 4 | ihi << 8 | jhi << 12 (at most 9 quads a side); returns the
// quad count (0: nothing of the region is in the tile). Region origins and
// tile origins are even pixels, so a quad is either wholly in the tile or out.
__device__ __forceinline__ uint32_t clip_quads(int32_t ox, int32_t oy, int32_t ex, int32_t ey, int32_t sx0,
                                               int32_t sy0, int32_t S, uint32_t& ij) {
    const int32_t ncol = (ex - ox + 31) >> 5, nrow = (ey - oy + 31) >> 5;
    const int32_t px = ox >> kSubpixelShift, py = oy >> kSubpixelShift;
    const int32_t ilo = max(0, (sx0 - px) / 2), ihi = min(ncol, (sx0 + S - px) / 2);
    const int32_t jlo = max(0, (sy0 - py) / 2), jhi = min(nrow, (sy0 + S - py) / 2);
    if (ihi <= ilo || jhi <= jlo) return 0u;
    ij = (uint32_t)ilo | ((uint32_t)jlo << 4) | ((uint32_t)ihi << 8) | ((uint32_t)jhi << 12);
    return (uint32_t)((ihi - ilo) * (jhi - jlo));
}

// Edge values of the four quad lanes at a region origin, [edge * 4 + lane],
// edges in the order e12, e20, e01 (w0, w1, w2).
__device__ __forceinline__ void origin_values(const PacketCtx& c, int32_t ox, int32_t oy, float w[12]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float lx = i2f(ox + ((k & 1) ? 24 : 8));
        const float ly = i2f(oy + ((k >> 1) ? 24 : 8));
        w[k] = edge_eval(c.e12, lx, ly);
        w[4 + k] = edge_eval(c.e20, lx, ly);
        w[8 + k] = edge_eval(c.e01, lx, ly);
    }
}

__device__ __forceinline__ bool region_exact(const PacketCtx& c, const float w[12], uint32_t ij) {
    const float im = (float)((int32_t)((ij >> 8) & 0xFu) - 1), jm = (float)((int32_t)((ij >> 12) & 0xFu) - 1);
    const float sx[3] = {c.e12.sx, c.e20.sx, c.e01.sx}, sy[3] = {c.e12.sy, c.e20.sy, c.e01.sy};
    bool ok = true;
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const float m = fmaxf(fmaxf(fabsf(w[4 * e]), fabsf(w[4 * e + 1])), fmaxf(fabsf(w[4 * e + 2]), fabsf(w[4 * e + 3])));
        const float b = ru_add(ru_add(m, ru_mul(jm, fabsf(sy[e]))), ru_mul(im, fabsf(sx[e])));
        ok = ok && (b <= 16777216.0f);
    }
    return ok;
}

template <int S>
struct RasterShared {
    static constexpr int kThreads = S <= 16 ? 128 : 256;
    static constexpr int kMinBlocks = S <= 16 ? 6 : 3;         // CTAs per SM the register budget allows
    static constexpr int kRegions = kThreads + kThreads / 2;  // regions staged per round
    unsigned long long sk[S * S];                             // depth keys of the scheduling tile
    // Regions of the round, in packet order.
    float4 r_w[3][kRegions];   // origin edge values: edge e's four sample lanes in r_w[e]
    uint32_t r_geom[kRegions];  // quad range (16 b) | exact << 15 | origin x, y relative to the tile (int8 each)
    uint32_t r_pi[kRegions];    // packet index | kSlowRegion | ceil(2^15 / ni) << 16
    uint32_t r_qbeg[kRegions + 40];  // first flattened quad of each region, then end markers
    uint16_t slow[kRegions];    // regions that replay the sequential additions
    // Packets of the round, one per thread.
    // Per packet, packed for 16-byte loads: (sx12, sx20, sx01, sy12), (sy20, sy01),
    // (ooa, oow a, da, db), (zow a, da, db, seq8 bits).
    float4 p_s[kThreads];
    float2 p_s2[kThreads];
    float4 p_o[kThreads], p_z[kThreads];
    uint32_t p_mat[kThreads], p_amip[kThreads], p_slot[kThreads];
    uint32_t scan[kThreads / 32][2];
    uint32_t cell_far[(S / 8) * (S / 8)];  // farthest key depth of each 8x8-px cell (orderable bits)
    uint32_t n_regions, n_quads, n_slow, cur_tile;
    uint8_t tab[512];           // FRSQRTE table for the fused shading
};

constexpr uint32_t kSlowRegion = 0x8000u;  // region replays the sequential additions

// Interpolation constants of one packet.
struct PacketLanes {
    float ooa, oow[3], zow[3];
    uint32_t seq8, mat;
};

template <int S>
__device__ __forceinline__ PacketLanes packet_lanes(const RasterShared<S>& s, uint32_t pk) {
    PacketLanes L;
    const float4 o = s.p_o[pk], z = s.p_z[pk];
    L.ooa = o.x;
    L.oow[0] = o.y;
    L.oow[1] = o.z;
    L.oow[2] = o.w;
    L.zow[0] = z.x;
    L.zow[1] = z.y;
    L.zow[2] = z.z;
    L.seq8 = __float_as_uint(z.w);
    L.mat = s.p_mat[pk];
    return L;
}

// Depth test of one covered lane: bary, w, z as fine_raster computes them,
// then the canonical-order key (atomicMin keeps the lowest z, ties broken by
// submission order).
template <int S>
__device__ __forceinline__ void raster_lane(RasterShared<S>& s, const FrameArgs& a, const DScene& sc,
                                            const PacketLanes& L, uint32_t pk, float w1, float w2, int32_t lx,
                                            int32_t ly) {
    const float b1 = w1 * L.ooa, b2 = w2 * L.ooa;
    const float oi = interp(L.oow, b1, b2), zi = interp(L.zow, b1, b2);
    unsigned long long* slot = s.sk + ly * S + lx;
    const unsigned long long cur = *slot;
    const float w = 1.0f / oi;
    const float z = zi * w;
    bool pass = (z == z);
    if (pass && (L.mat & kRecAlphaBit))
        pass = alpha_pass(sc, sc.materials[L.mat & kRecMaterialMask], a.rec_s[s.p_slot[pk]], b1, b2, w, s.p_amip[pk]);
    if (pass) {
        const unsigned long long key = make_key(z, L.seq8);
        if (key < cur) atomicMin(slot, key);
    }
}

__device__ __forceinline__ int32_t geom_ox(uint32_t g) { return (int32_t)(int8_t)((g >> 16) & 0xFFu); }
__device__ __forceinline__ int32_t geom_oy(uint32_t g) { return (int32_t)(int8_t)(g >> 24); }

// Exact region quad: lane = one quad, evaluated in closed form.
template <int S>
__device__ __forceinline__ void raster_exact_quad(RasterShared<S>& s, const FrameArgs& a, const DScene& sc,
                                                  uint32_t r, uint32_t q, uint32_t g) {
    const uint32_t pi = s.r_pi[r];
    if (pi & kSlowRegion) return;
    const uint32_t pk = pi & 0x7FFFu;
    const int32_t ilo = (int32_t)(g & 0xFu), jlo = (int32_t)((g >> 4) & 0xFu);
    const int32_t ni = (int32_t)((g >> 8) & 0xFu) - ilo;
    const int32_t jj = (int32_t)((q * (pi >> 16)) >> 15);  // q / ni for q < 2^12
    const int32_t i = ilo + ((int32_t)q - jj * ni), j = jlo + jj;
    const float fi = (float)i, fj = (float)j;
    const float4 ps = s.p_s[pk];
    const float2 ps2 = s.p_s2[pk];
    const float sx[3] = {ps.x, ps.y, ps.z}, sy[3] = {ps.w, ps2.x, ps2.y};
    float w[12];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const float d = sy[e] * fj + sx[e] * fi;
        const float4 o = s.r_w[e][r];
        w[4 * e] = o.x + d;
        w[4 * e + 1] = o.y + d;
        w[4 * e + 2] = o.z + d;
        w[4 * e + 3] = o.w + d;
    }
    uint32_t cov = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) cov |= (w[k] >= 0.0f && w[4 + k] >= 0.0f && w[8 + k] >= 0.0f) ? (1u << k) : 0u;
    if (cov == 0u) return;
    const PacketLanes L = packet_lanes(s, pk);
    const int32_t lx0 = geom_ox(g) + 2 * i, ly0 = geom_oy(g) + 2 * j;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (cov & (1u << k)) raster_lane<S>(s, a, sc, L, pk, w[4 + k], w[8 + k], lx0 + (k & 1), ly0 + (k >> 1));
    }
}

// Sequential region: one warp, lane = (quad row, quad lane); each lane walks
// its row along x with the reference's additions.
template <int S>
__device__ __forceinline__ void raster_slow_region(RasterShared<S>& s, const FrameArgs& a, const DScene& sc,
                                                   uint32_t r) {
    const uint32_t lane = threadIdx.x & 31u;
    const int32_t k = (int32_t)(lane & 3u);
    const uint32_t pk = s.r_pi[r] & 0x7FFFu, g = s.r_geom[r];
    const int32_t ilo = (int32_t)(g & 0xFu), jlo = (int32_t)((g >> 4) & 0xFu);
    const int32_t ihi = (int32_t)((g >> 8) & 0xFu), jhi = (int32_t)((g >> 12) & 0xFu);
    const int32_t lx0 = geom_ox(g) + (k & 1), ly0 = geom_oy(g) + (k >> 1);
    const float4 ps = s.p_s[pk];
    const float2 ps2 = s.p_s2[pk];
    const float sx0 = ps.x, sx1 = ps.y, sx2 = ps.z;
    const float sy0 = ps.w, sy1 = ps2.x, sy2 = ps2.y;
    const PacketLanes L = packet_lanes(s, pk);
    for (int32_t j = jlo + (int32_t)(lane >> 2); j < jhi; j += 8) {
        const float* rw = reinterpret_cast<const float*>(&s.r_w[0][r]);
        float w0 = rw[k], w1 = reinterpret_cast<const float*>(&s.r_w[1][r])[k],
              w2 = reinterpret_cast<const float*>(&s.r_w[2][r])[k];
        for (int32_t t = 0; t < j; ++t) {
            w0 += sy0;
            w1 += sy1;
            w2 += sy2;
        }
        for (int32_t i = 0; i < ihi; ++i) {
            if (i >= ilo && w0 >= 0.0f && w1 >= 0.0f && w2 >= 0.0f)
                raster_lane<S>(s, a, sc, L, pk, w1, w2, lx0 + 2 * i, ly0 + 2 * j);
            w0 += sx0;
            w1 += sx1;
            w2 += sx2;
        }
    }
}

// ---- Occlusion culling ----------------------------------------------------
//
// Between rounds the raster records, per 8x8-px cell of the scheduling tile,
// the farthest depth its keys hold. A packet whose every depth lies beyond
// that of each cell it can touch cannot lower a key (keys only decrease, and
// winning a tie needs an equal depth), so it is dropped in pass 1: the keys
// come out as if it had been rasterized. (Testing each 16-px block of a
// coarse packet as well dropped 15% more pairs but made the 4K raster 6%
// slower.) The floor on a packet's depths, and the argument that it covers
// every rounding of the raster's arithmetic, are in depthfloor.cuh.

// Farthest key depth of each 8x8-px cell, then a barrier. Warp w takes cell
// row w: each load reads whole key rows (16 B a lane, consecutive lanes
// consecutive keys), so the warp's accesses cover distinct banks; four lanes
// hold a cell's part of a row and shuffles fold the lanes and rows.
template <int S>
__device__ __forceinline__ void cell_depths(RasterShared<S>& s) {
    constexpr int CW = S / 8;      // cells per side
    constexpr int LPR = S / 2;     // lanes per key row (two keys a lane)
    constexpr int RPW = 32 / LPR;  // key rows per warp load
    const int lane = (int)(threadIdx.x & 31u), warp = (int)(threadIdx.x >> 5);
    if (warp < CW) {
        uint32_t m = 0;
        const int col = (lane % LPR) * 2, sub = lane / LPR;
#pragma unroll
        for (int rr = 0; rr < 8; rr += RPW) {
            const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(s.sk + (warp * 8 + rr + sub) * S + col);
            m = max(m, max((uint32_t)(v.x >> 32), (uint32_t)(v.y >> 32)));
        }
        // The four lanes of a cell in a row, then the rows the warp's
        // lanes read side by side.
        m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, 1));
        m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, 2));
#pragma unroll
        for (int o = LPR; o < 32; o <<= 1) m = max(m, __shfl_xor_sync(0xFFFFFFFFu, m, o));
        if (lane < LPR && (lane & 3) == 0) s.cell_far[warp * CW + (lane >> 2)] = m;
    }
    __syncthreads();
}

// Farthest key depth over the cells holding pixels [xl, xh] x [yl, yh]
// clipped to the scheduling tile (all ones when none of them is in it).
template <int S>
__device__ __forceinline__ uint32_t cells_far(const RasterShared<S>& s, int32_t xl, int32_t xh, int32_t yl, int32_t yh,
                                              int32_t sx0, int32_t sy0) {
    xl = max(xl, sx0), xh = min(xh, sx0 + S - 1), yl = max(yl, sy0), yh = min(yh, sy0 + S - 1);
    if (xh < xl || yh < yl) return 0xFFFFFFFFu;
    const int32_t cx0 = (xl - sx0) >> 3, cx1 = (xh - sx0) >> 3, cy0 = (yl - sy0) >> 3, cy1 = (yh - sy0) >> 3;
    uint32_t far = 0;
    for (int32_t cy = cy0; cy <= cy1; ++cy)
        for (int32_t cx = cx0; cx <= cx1; ++cx) far = max(far, s.cell_far[cy * (S / 8) + cx]);
    return far;
}

// Orderable depth floor of the packet (its triangle's, taken by the front
// end); 0 (below every key) when none is taken. A packet is hidden when its
// floor is above the farthest depth of every cell its covered lanes can fall
// in: pixels [x0 & ~1, x1] of its clipped rect.
__device__ __forceinline__ uint32_t packet_floor(const PacketCtx& c) { return c.r.zfloor; }

// Pass 1 of a round for one packet: classify and split into regions, and
// either count them (regions, quads; the accepted 16-px blocks of a coarse
// packet go to bmask) or stage them from the given positions (bmask as the
// count left it).
template <int S>
__device__ __forceinline__ void packet_regions(RasterShared<S>& s, const PacketCtx& c, int32_t sx0, int32_t sy0,
                                               bool write, uint32_t pk, uint32_t& n_r, uint32_t& n_q,
                                               uint32_t& bmask) {
    auto region = [&](int32_t ox, int32_t oy, int32_t ex, int32_t ey) {
        uint32_t ij = 0;
        const uint32_t nq = clip_quads(ox, oy, ex, ey, sx0, sy0, S, ij);
        if (nq == 0) return false;
        if (write) {
            const uint32_t r = n_r;
            float w[12];
            origin_values(c, ox, oy, w);
            const bool exact = region_exact(c, w, ij);
#pragma unroll
            for (int e = 0; e < 3; ++e) s.r_w[e][r] = make_float4(w[4 * e], w[4 * e + 1], w[4 * e + 2], w[4 * e + 3]);
            const int32_t ox_rel = (ox >> kSubpixelShift) - sx0, oy_rel = (oy >> kSubpixelShift) - sy0;
            s.r_geom[r] = ij | ((uint32_t)(ox_rel & 0xFF) << 16) | ((uint32_t)(oy_rel & 0xFF) << 24);
            const uint32_t ni = ((ij >> 8) & 0xFu) - (ij & 0xFu);
            s.r_pi[r] = pk | (exact ? 0u : kSlowRegion) | (((32768u + ni - 1u) / ni) << 16);
            s.r_qbeg[r] = n_q;
            if (!exact) s.slow[atomicAdd(&s.n_slow, 1u)] = (uint16_t)r;
        }
        ++n_r;
        n_q += nq;
        return true;
    };
    if (!c.coarse) {
        region(c.xs, c.ys, c.xe, c.ye);
        return;
    }
    int32_t bxl, bxh, byl, byh;
    block_range(c.xs, c.xe, sx0, S, bxl, bxh);
    block_range(c.ys, c.ye, sy0, S, byl, byh);
    if (!write) bmask = 0;
    uint32_t bit = 1;  // at most 5 x 5 blocks of a 64-px reference tile
    for (int32_t by = byl; by < byh; ++by)
        for (int32_t bx = bxl; bx < bxh; ++bx, bit <<= 1) {
            const int32_t ox = c.xs + 256 * bx, oy = c.ys + 256 * by;
            if (write) {
                if (bmask & bit) region(ox, oy, min(ox + 256, c.xe), min(oy + 256, c.ye));
            } else if (!block_rejected(c.e12, c.e20, c.e01, ox, oy) &&
                       region(ox, oy, min(ox + 256, c.xe), min(oy + 256, c.ye))) {
                bmask |= bit;
            }
        }
}

__device__ __forceinline__ bool shade_needed(const DView& v, int32_t qx, int32_t qy);
// Shading variants by reciprocal square root: the values of SWR_RSQRT_IEEE and
// SWR_RSQRT_AARCH64, or any (read per view).
constexpr int kModeIeee = 0, kModeArm = 1, kModeAny = 2;
template <bool GI, int MODE>
__device__ __forceinline__ void shade_pixel(const FrameArgs& a, const uint8_t* tab, const DView& v,
                                            const DScene& sc, int32_t qx, int32_t qy, int32_t k, bool needed,
                                            unsigned long long key);

// Occlusion culling is on for 64-px scheduling tiles, the choice for large
// single views. It pays where many packets of a tile lie behind near
// geometry drawn first (the 2M-triangle 4K frame: 640 -> 728 frames/s) and
// costs where triangles are small and seldom hidden: on the served mix of
// orbiting cameras, culling in every tile size took the plain loop from
// 1,210 to 1,030 frames/s and the served batches (32-px tiles) from 4,980
// to 4,460; for the 16-px tiles of the 1280x720 small frame it cost 6%.
// A first round of 64 packets: 4K raster 0.444 ms, against 0.461 (32),
// 0.460 (128) and 0.477 (a full round of 256).
#ifndef SWR_CULL_FIRST
#define SWR_CULL_FIRST 64
#endif

// Persistent: each CTA pulls (view, scheduling tile) work items from a
// device-side counter until every tile of every view is done. Per tile, the
// bin's packets go through rounds of one packet per thread: pass 1 stages
// regions (a block-wide scan places them), pass 2 rasterizes the exact
// regions' quads flattened over all lanes, pass 3 the sequential regions.
template <int S, bool FUSE>
__global__ void __launch_bounds__(RasterShared<S>::kThreads, RasterShared<S>::kMinBlocks) k_raster(FrameArgs a) {
    using Sh = RasterShared<S>;
    constexpr int NT = Sh::kThreads, R = Sh::kRegions, NW = NT / 32;
    extern __shared__ __align__(16) unsigned char raster_smem[];
    Sh& s = *reinterpret_cast<Sh*>(raster_smem);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t n_tiles = a.dyn->n_stiles;
    constexpr bool kFuse = FUSE;
    // Occlusion culling for tiles of at least SWR_CULL_MIN_TILE px; the first
    // round of a tile takes at most kFirst packets, so that later rounds
    // meet the nearest depths sooner (taking light tiles, at most one round
    // of packets, whole instead: 4K 718 against 728 frames/s).
    constexpr bool kCull = S >= SWR_CULL_MIN_TILE;
    constexpr uint32_t kFirst = (kCull && SWR_CULL_FIRST > 0 && SWR_CULL_FIRST < NT) ? SWR_CULL_FIRST : NT;
    if (kFuse)
        for (int i = threadIdx.x; i < 512; i += NT) s.tab[i] = a.rsqrt_table[i];
    uint32_t n_culled = 0;
    for (uint32_t iter = 0;; ++iter) {
#if SWR_RASTER_PERSISTENT
        if (threadIdx.x == 0) {
            const uint32_t w = atomicAdd(&a.counters->work_next, 1u);
            s.cur_tile = w >= n_tiles ? n_tiles : a.sched_tile >= kOrderMinTile ? a.tile_count[w] : w;
        }
        __syncthreads();
        const uint32_t st = s.cur_tile;
#else
        if (iter > 0) break;
        const uint32_t st = blockIdx.x;
#endif
        if (st >= n_tiles) break;
        const uint32_t vi = find_view_by_stile(a, st);
        const DView& view = a.views[vi];
        const uint32_t local = st - view.stile_base;
        const int32_t sx0 = (int32_t)(local % (uint32_t)view.stiles_x) * S;
        const int32_t sy0 = (int32_t)(local / (uint32_t)view.stiles_x) * S;
        const int32_t tx0 = (sx0 / kRefTile) * kRefTile, ty0 = (sy0 / kRefTile) * kRefTile;
        for (int i = threadIdx.x; i < S * S; i += NT) s.sk[i] = kEmptyKey;
        const bool bad = (a.counters->status & (ST_BIN_OVERFLOW | ST_CLIP_OVERFLOW | ST_QUEUE_OVERFLOW)) != 0u;
        const uint32_t b0 = a.tile_offset[st], b1 = bad ? b0 : a.tile_offset[st + 1];
        const DScene& sc = a.scenes[view.scene];
        // Cell depths are valid once taken for this tile (until then they
        // hold another tile's, or nothing); they are taken again after a
        // round that had regions.
        bool keys_changed = false, cells_valid = false;
        for (uint32_t cursor = b0; cursor < b1;) {
            // The keys the previous rounds left, per cell, for occlusion culling.
            if (kCull && keys_changed) {
                cell_depths<S>(s);
                keys_changed = false;
                cells_valid = true;
            }
            const uint32_t lim = cursor == b0 ? kFirst : (uint32_t)NT;
            // Pass 1: count this thread's regions and quads.
            const uint32_t pidx = cursor + threadIdx.x;
            PacketCtx c;
            uint32_t slot = 0, n_r = 0, n_q = 0, bmask = 0;
            bool hidden = false;
            if (pidx < b1 && threadIdx.x < lim) {
                slot = a.bins[pidx];
                const uint32_t nidx = pidx + NT;  // this thread's likely packet next round
                const uint32_t nslot = nidx < b1 ? __ldg(a.bins + nidx) : 0xFFFFFFFFu;
                load_packet(a, sc, slot, tx0, ty0, c);
#if SWR_RASTER_PREFETCH
                if (nslot != 0xFFFFFFFFu) {
                    const char* np = reinterpret_cast<const char*>(a.rec_r + nslot);
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(np));
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(np + sizeof(RecRaster) - 1));
                }
#endif
                if (kCull && cells_valid) {
                    const uint32_t far = cells_far<S>(s, c.xs >> kSubpixelShift, c.xe >> kSubpixelShift,
                                                      c.ys >> kSubpixelShift, c.ye >> kSubpixelShift, sx0, sy0);
                    hidden = far < 0xFF800000u && packet_floor(c) > far;
                }
                if (!hidden) packet_regions<S>(s, c, sx0, sy0, false, threadIdx.x, n_r, n_q, bmask);
            }
            if (threadIdx.x == 0) s.n_slow = 0;
            // Block-wide exclusive scan of (regions, quads).
            uint32_t ir = n_r, iq = n_q;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t xr = __shfl_up_sync(0xFFFFFFFFu, ir, o);
                const uint32_t xq = __shfl_up_sync(0xFFFFFFFFu, iq, o);
                if (lane >= (uint32_t)o) {
                    ir += xr;
                    iq += xq;
                }
            }
            if (lane == 31u) {
                s.scan[warp][0] = ir;
                s.scan[warp][1] = iq;
            }
            __syncthreads();
            uint32_t pr = ir - n_r, pq = iq - n_q, all_r = 0;
            for (uint32_t w = 0; w < (uint32_t)NW; ++w) {
                if (w < warp) {
                    pr += s.scan[w][0];
                    pq += s.scan[w][1];
                }
                all_r += s.scan[w][0];
            }
            // Packets are taken in order while their regions fit.
            const bool taken = pr + n_r <= (uint32_t)R && threadIdx.x < lim;
            const uint32_t n_taken = (uint32_t)__syncthreads_count(taken);
            n_culled += (hidden && taken) ? 1u : 0u;
            // No packet of the round has a region (all culled or outside the
            // tile): no key changes, and the next round starts at once (every
            // thread has read the scan words before the barrier above).
            if (all_r == 0u) {
                cursor += n_taken;
                continue;
            }
            keys_changed = true;
            if (taken && threadIdx.x + 1u == n_taken) {
                s.n_regions = pr + n_r;
                s.n_quads = pq + n_q;
                s.r_qbeg[pr + n_r] = pq + n_q;
                for (int t = 1; t <= 33; ++t) s.r_qbeg[pr + n_r + t] = 0xFFFFFFFFu;
            }
            if (taken && n_r > 0u) {
                const uint32_t pk = threadIdx.x;
                s.p_s[pk] = make_float4(c.e12.sx, c.e20.sx, c.e01.sx, c.e12.sy);
                s.p_s2[pk] = make_float2(c.e20.sy, c.e01.sy);
                s.p_o[pk] = make_float4(c.r.ooa, c.r.oow[0], c.r.oow[1], c.r.oow[2]);
                s.p_z[pk] = make_float4(c.r.zow[0], c.r.zow[1], c.r.zow[2], __uint_as_float(c.r.seq8));
                s.p_mat[pk] = c.r.material;
                s.p_amip[pk] = c.amip;
                s.p_slot[pk] = slot;
                packet_regions<S>(s, c, sx0, sy0, true, pk, pr, pq, bmask);
            }
            cursor += n_taken;
            __syncthreads();
            // Pass 2: quads numbered 0..n_quads-1 region after region; each
            // warp takes one contiguous range, 32 quads per step.
            const uint32_t nq = s.n_quads, nr = s.n_regions;
            if (nq > 0u) {
                const uint32_t chunk = (nq + NW - 1u) / NW;
                const uint32_t f0 = warp * chunk, f1 = min(f0 + chunk, nq);
                if (f0 < f1) {
                    uint32_t lo = 0, hi = nr - 1u;  // last region starting at or before f0
                    while (lo < hi) {
                        const uint32_t mid = (lo + hi + 1u) >> 1;
                        if (s.r_qbeg[mid] <= f0) lo = mid; else hi = mid - 1u;
                    }
                    uint32_t rb = lo;
                    for (uint32_t f = f0; f < f1; f += 32u) {
                        // Region ends are strictly increasing (no empty region):
                        // lane l's region is rb + #{ends <= f + l}.
                        const uint32_t d = s.r_qbeg[rb + 1u + lane] - f;
                        const uint32_t mask = __reduce_or_sync(0xFFFFFFFFu, d <= 31u ? (1u << d) : 0u);
                        const uint32_t adv = __popc(__ballot_sync(0xFFFFFFFFu, d <= 32u));
                        const uint32_t r = rb + __popc(mask & ((2u << lane) - 1u));
                        const uint32_t g = f + lane;
                        if (g < f1) raster_exact_quad<S>(s, a, sc, r, g - s.r_qbeg[r], s.r_geom[r]);
                        rb += adv;
                    }
                }
            }
            // Pass 3: sequential regions, one warp each.
            const uint32_t nsl = s.n_slow;
            for (uint32_t m = warp; m < nsl; m += NW) raster_slow_region<S>(s, a, sc, s.slow[m]);
            __syncthreads();
        }
        unsigned long long* dst = a.keys + view.key_offset;
        // Fused: keys go to HBM only for the translucent pass; the tile is
        // shaded from shared memory, 4 lanes per quad, quads row by row.
        if (!kFuse || (view.flags & kViewTranslucent))
            for (int i = threadIdx.x; i < S * S; i += NT) {
                const int32_t ly = i / S, lx = i % S;
                dst[(uint64_t)(sy0 + ly) * view.key_pitch + (uint64_t)(sx0 + lx)] = s.sk[i];
            }
        constexpr int QS = S / 2;
        // Lanes read keys other threads initialised or wrote: a tile without
        // packets has had no barrier since the keys were reset.
        if (kFuse) __syncthreads();
        for (int base = 0; kFuse && base < S * S; base += NT) {
            const int t = base + (int)threadIdx.x;
            const bool live = t < S * S;
            const int ql = live ? (t >> 2) : 0;
            const int32_t k = t & 3;
            const int32_t qx = (sx0 >> 1) + ql % QS, qy = (sy0 >> 1) + ql / QS;
            const bool needed = live && shade_needed(view, qx, qy);
            unsigned long long key = kEmptyKey;
            if (needed) key = s.sk[(2 * (ql / QS) + (k >> 1)) * S + 2 * (ql % QS) + (k & 1)];
            shade_pixel<true, kModeAny>(a, s.tab, view, sc, qx, qy, k, needed, key);
        }
        __syncthreads();
    }
    n_culled = __reduce_add_sync(0xFFFFFFFFu, n_culled);
    if (lane == 0u && n_culled) atomicAdd(&a.counters->culled, n_culled);
}

// --------------------------------------------------------------------------
// Shading
// --------------------------------------------------------------------------
__device__ __forceinline__ uint32_t find_view_by_quad(const FrameArgs& a, uint32_t q) {
    uint32_t lo = 0, hi = a.dyn->n_views - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (a.views[mid].quad_base <= q) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// compute_skybox for one lane (src/tilerasterizer.rs:478-508).
__device__ __forceinline__ f3 skybox(const DView& v, const DScene& sc, int32_t qx_screen, int32_t qy_screen,
                                     int32_t kx, int32_t ky, uint32_t md, const uint8_t* tab) {
    const float pxf = i2f(qx_screen) + (kx ? 1.5f : 0.5f);
    const float pyf = i2f(qy_screen) + (ky ? 1.5f : 0.5f);
    const float ndc_x = ((pxf * v.one_over_width) * 2.0f) - 1.0f;
    const float ndc_y = ((1.0f - pyf * v.one_over_height) * 2.0f) - 1.0f;
    const float* m = v.skybox_t;
    f3 d;
    d.x = ((ndc_x * m[0] + ndc_y * m[1]) + 1.0f * m[2]) + m[3];
    d.y = ((ndc_x * m[4] + ndc_y * m[5]) + 1.0f * m[6]) + m[7];
    d.z = ((ndc_x * m[8] + ndc_y * m[9]) + 1.0f * m[10]) + m[11];
    const f3 n = normalize(d, md, tab);
    float uf, vf;
    uint32_t slice;
    cube_uv(n, uf, vf, slice);
    return srgb_fast3(sample_cube(sc.textures[sc.tex_cubemap], uf, vf, slice, 0u));
}

// get_filtered_gi_sh4_packed_vec over the baked grid: every coefficient's
// rgb and w trilinear.
__device__ __forceinline__ void voxel_gi_baked(const float4* G, uint32_t n, uint32_t x0, uint32_t y0, uint32_t z0,
                                            uint32_t x1, uint32_t y1, uint32_t z1, float fx, float fy, float fz,
                                            f3 sh[4], float& w0, float& w1) {
    const float ofx = 1.0f - fx, ofy = 1.0f - fy, ofz = 1.0f - fz;
    const uint32_t nn = n * n;
    const uint32_t c000 = z0 * nn + y0 * n + x0, c001 = z1 * nn + y0 * n + x0;
    const uint32_t c010 = z0 * nn + y1 * n + x0, c011 = z1 * nn + y1 * n + x0;
    const uint32_t c100 = z0 * nn + y0 * n + x1, c101 = z1 * nn + y0 * n + x1;
    const uint32_t c110 = z0 * nn + y1 * n + x1, c111 = z1 * nn + y1 * n + x1;
    for (int c = 0; c < 4; ++c) {
        const float4 a000 = __ldg(G + (size_t)c000 * 4 + c), a001 = __ldg(G + (size_t)c001 * 4 + c);
        const float4 a010 = __ldg(G + (size_t)c010 * 4 + c), a011 = __ldg(G + (size_t)c011 * 4 + c);
        const float4 a100 = __ldg(G + (size_t)c100 * 4 + c), a101 = __ldg(G + (size_t)c101 * 4 + c);
        const float4 a110 = __ldg(G + (size_t)c110 * 4 + c), a111 = __ldg(G + (size_t)c111 * 4 + c);
        auto tri = [&](float v000, float v001, float v010, float v011, float v100, float v101, float v110,
                       float v111) {
            const float v00 = v000 * ofx + v100 * fx, v01 = v001 * ofx + v101 * fx;
            const float v10 = v010 * ofx + v110 * fx, v11 = v011 * ofx + v111 * fx;
            const float v0 = v00 * ofy + v10 * fy, v1 = v01 * ofy + v11 * fy;
            return v0 * ofz + v1 * fz;
        };
        sh[c] = mk3(tri(a000.x, a001.x, a010.x, a011.x, a100.x, a101.x, a110.x, a111.x),
                    tri(a000.y, a001.y, a010.y, a011.y, a100.y, a101.y, a110.y, a111.y),
                    tri(a000.z, a001.z, a010.z, a011.z, a100.z, a101.z, a110.z, a111.z));
        const float w = tri(a000.w, a001.w, a010.w, a011.w, a100.w, a101.w, a110.w, a111.w);
        if (c == 0) w0 = w;
        if (c == 1) w1 = w;
    }
}

// get_filtered_gi_sh4_packed_vec (src/voxelgrid.rs:264-368) for the
// constant-SH voxel grid: w0 from the light grid, the rest constant; with
// GI, scenes with a baked grid read it instead (the variant without GI
// keeps the baked path's registers out of the common kernels).
template <bool GI>
__device__ void voxel_gi(const DScene& sc, f3 pos, f3 sh[4], float& w0, float& w1) {
    const uint32_t n = sc.voxel_n;
    const float vx = (pos.x - sc.voxel_min[0]) / sc.voxel_size_f[0];
    const float vy = (pos.y - sc.voxel_min[1]) / sc.voxel_size_f[1];
    const float vz = (pos.z - sc.voxel_min[2]) / sc.voxel_size_f[2];
    const float x0f = floorf(vx), y0f = floorf(vy), z0f = floorf(vz);
    uint32_t x0 = f2u_sat(x0f), y0 = f2u_sat(y0f), z0 = f2u_sat(z0f);
    x0 = min(x0, n - 1u); y0 = min(y0, n - 1u); z0 = min(z0, n - 1u);
    const uint32_t x1 = min(x0 + 1u, n - 1u), y1 = min(y0 + 1u, n - 1u), z1 = min(z0 + 1u, n - 1u);
    const float fx = vx - x0f, fy = vy - y0f, fz = vz - z0f;
    const float ofx = 1.0f - fx, ofy = 1.0f - fy, ofz = 1.0f - fz;
    const uint32_t nn = n * n;
    if (GI && sc.voxel_sh4) {
        voxel_gi_baked(sc.voxel_sh4, n, x0, y0, z0, x1, y1, z1, fx, fy, fz, sh, w0, w1);
        return;
    }
    const float* L = sc.voxel_light;
    const float w000 = __ldg(L + z0 * nn + y0 * n + x0), w001 = __ldg(L + z1 * nn + y0 * n + x0);
    const float w010 = __ldg(L + z0 * nn + y1 * n + x0), w011 = __ldg(L + z1 * nn + y1 * n + x0);
    const float w100 = __ldg(L + z0 * nn + y0 * n + x1), w101 = __ldg(L + z1 * nn + y0 * n + x1);
    const float w110 = __ldg(L + z0 * nn + y1 * n + x1), w111 = __ldg(L + z1 * nn + y1 * n + x1);
    {
        const float v00 = w000 * ofx + w100 * fx, v01 = w001 * ofx + w101 * fx;
        const float v10 = w010 * ofx + w110 * fx, v11 = w011 * ofx + w111 * fx;
        const float v0 = v00 * ofy + v10 * fy, v1 = v01 * ofy + v11 * fy;
        w0 = v0 * ofz + v1 * fz;
    }
    {
        const float c = sc.sky_visibility;
        const float v00 = c * ofx + c * fx;
        const float v0 = v00 * ofy + v00 * fy;
        w1 = v0 * ofz + v0 * fz;
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float o[3];
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) {
            const float c = sc.gi_rgb[i][ch];
            const float v00 = c * ofx + c * fx;
            const float v0 = v00 * ofy + v00 * fy;
            o[ch] = v0 * ofz + v0 * fz;
        }
        sh[i] = mk3(o[0], o[1], o[2]);
    }
}

// One material texture of a lane: quad mip (compute_mip_level) and point
// sample (sample4_rgb / sample4_alpha lane, src/texture.rs:680-727).
__device__ __forceinline__ uint32_t sample_slot(const DScene& sc, const DMaterial& m, int slot, float u, float v, const float* du_dv) {
    const DTexture& t = sc.textures[m.tex[slot]];
    const uint32_t mip = mip_level(t, du_dv[0], du_dv[1], du_dv[2], du_dv[3]);
    return sample_texel(t, u, v, mip, m.wrap_s[slot], m.wrap_t[slot]);
}

// pbr_shader<TRANS> for one lane (src/shader.rs:110-309). du_dv already holds
// packet.du_dv * w with component i scaled by lane i's w (Q6 quirk). `cur` is
// the colour under a translucent fragment. GI: read baked voxel grids.
template <bool TRANS, bool GI>
__device__ __forceinline__ f3 pbr_lane(const DScene& sc, const DView& v, const DMaterial& m, const RecShade& q,
                                       float w, float b1, float b2, const float du_dv[4], uint32_t md,
                                       const uint8_t* tab, f3 cur) {
    const float PI = 3.14159265358979f;
    const float EPS = 1e-6f;
    const float INV_PI = 1.0f / 3.14159265358979f;
    const f3 in_n = normalize(interp3(q.nrm, b1, b2), md, tab);
    const f3 in_t = normalize(interp3(q.tan, b1, b2), md, tab);
    const float tsign = interp(q.tsign, b1, b2);
    const f3 pw = interp3(q.pww, b1, b2) * w;
    const float uvx = interp(q.uow, b1, b2) * w;
    const float uvy = interp(q.vow, b1, b2) * w;
    const f3 tw = normalize(in_t - in_n * dot(in_n, in_t), md, tab);
    const float hand = tsign >= 0.0f ? 1.0f : -1.0f;
    const f3 bw = cross(in_n, tw) * hand;
    f3 nw = normalize(in_n, md, tab);
    if (m.tex[TS_NORMAL] >= 0) {
        const f3 s = unpack_rgb(sample_slot(sc, m, TS_NORMAL, uvx, uvy, du_dv));
        const f3 tsn = mk3(s.x * 2.0f - 1.0f, s.y * 2.0f - 1.0f, s.z * 2.0f - 1.0f);
        nw = (tw * tsn.x + bw * tsn.y) + in_n * tsn.z;
        nw = normalize(nw, md, tab);
    }
    const f3 ld = mk3(sc.light_dir[0], sc.light_dir[1], sc.light_dir[2]);
    const f3 lc = mk3(sc.light_color[0], sc.light_color[1], sc.light_color[2]);
    const f3 vd = mk3(v.cam_pos[0], v.cam_pos[1], v.cam_pos[2]) - pw;
    const f3 vn = normalize(vd, md, tab);
    const float ndl = fmaxf(dot(nw, ld), 0.0f);
    const f3 hv = normalize(ld + vn, md, tab);
    const float ndh = fmaxf(dot(nw, hv), 0.0f);
    const float ndv = fmaxf(dot(nw, vn), 1.0e-4f);
    const float vdh = fmaxf(dot(vn, hv), 0.0f);
    f3 sh[4];
    float gw0, gw1;
    voxel_gi<GI>(sc, pw, sh, gw0, gw1);
    const float vli = clampf(gw0, 0.0f, 1.0f);
    const float skyv = clampf(gw1, 0.0f, 1.0f);
    f3 bc = mk3(m.base_color[0], m.base_color[1], m.base_color[2]);
    if (m.tex[TS_BASE] >= 0) bc = bc * srgb_fast3(unpack_rgb(sample_slot(sc, m, TS_BASE, uvx, uvy, du_dv)));
    float rough = m.roughness, metal = m.metallic;
    if (m.tex[TS_MR] >= 0) {
        const f3 s = unpack_rgb(sample_slot(sc, m, TS_MR, uvx, uvy, du_dv));
        rough = rough * s.y;
        metal = metal * s.z;
    }
    rough = clampf(rough, 0.045f, 1.0f);
    metal = clampf(metal, 0.0f, 1.0f);
    float ao = 1.0f;
    if (m.tex[TS_OCCLUSION] >= 0) {
        ao = unpack_rgb(sample_slot(sc, m, TS_OCCLUSION, uvx, uvy, du_dv)).x;
        ao = 1.0f + (ao - 1.0f) * m.occlusion_strength;
    }
    const f3 c004 = mk3(0.04f, 0.04f, 0.04f);
    const f3 f0 = c004 + (bc - c004) * metal;
    const float omvh = 1.0f - vdh;
    const float omvh2 = omvh * omvh;
    const float omvh4 = omvh2 * omvh2;
    const float omvh5 = omvh4 * omvh;
    const f3 one = mk3(1.0f, 1.0f, 1.0f);
    const f3 fd = f0 + (one - f0) * omvh5;
    const float alpha = rough * rough;
    const float alpha2 = alpha * alpha;
    const float ndh2 = ndh * ndh;
    const float den_d = ndh2 * (alpha2 - 1.0f) + 1.0f;
    const float brdf_d = alpha2 / (PI * (den_d * den_d) + EPS);
    float k = rough + 1.0f;
    k = (k * k) * 0.125f;
    const float gv = ndv / ((ndv * (1.0f - k) + k) + EPS);
    const float gl = ndl / ((ndl * (1.0f - k) + k) + EPS);
    const float brdf_g = gv * gl;
    const float spec_dg = (brdf_d * brdf_g) / ((4.0f * ndl) * ndv + EPS);
    const f3 kd = (one - fd) * (1.0f - metal);
    const f3 lambert = bc * INV_PI;
    const f3 cdd = (((lc * kd) * lambert) * ndl) * vli;
    const f3 cds = (((lc * fd) * spec_dg) * ndl) * vli;
    const f3 kdi = (one - f0) * (1.0f - metal);
    f3 irr = ((sh[0] + sh[1] * nw.y) + sh[2] * nw.z) + sh[3] * nw.x;
    irr = mk3(fmaxf(irr.x, 0.0f), fmaxf(irr.y, 0.0f), fmaxf(irr.z, 0.0f));
    const f3 cid = ((irr * bc) * kdi) * INV_PI;
    // reflect: self - normal * self.dot(normal) * 2 (src/math.rs:118-120).
    const f3 iv = vn * -1.0f;
    const f3 rd = iv - (nw * dot(iv, nw)) * 2.0f;
    const DTexture& spec = sc.textures[sc.tex_specular];
    const float spec_mip = rough * (float)spec.max_mip;
    f3 env;
    {
        const float mx = (float)spec.max_mip;
        const float mp = clampf(spec_mip, 0.0f, mx);
        const float m0 = floorf(mp);
        const float m1 = fminf(m0 + 1.0f, mx);
        const float t = mp - m0;
        float uf, vf;
        uint32_t slice;
        cube_uv(rd, uf, vf, slice);
        const f3 c0 = sample_cube(spec, uf, vf, slice, f2u_sat(m0));
        const f3 c1 = sample_cube(spec, uf, vf, slice, f2u_sat(m1));
        env = c0 + (c1 - c0) * t;
    }
    const f3 lut = sample_bilinear(sc.textures[sc.tex_brdf_lut], clampf(ndv, 0.0f, 1.0f), clampf(rough, 0.0f, 1.0f));
    const f3 bsf = f0 * lut.x + mk3(lut.y, lut.y, lut.y);
    f3 cis = env * bsf;
    const float ao_spec = 1.0f + (ao - 1.0f) * 0.5f;
    cis = cis * (ao_spec * skyv);
    f3 col;
    if (TRANS) {
        float tr = m.transmission;
        if (m.tex[TS_TRANSMISSION] >= 0) tr = tr * unpack_rgb(sample_slot(sc, m, TS_TRANSMISSION, uvx, uvy, du_dv)).x;
        tr = clampf(tr, 0.0f, 1.0f);
        const float inv = 1.0f - tr;
        col = (((cur * bc) * tr + (cdd + cid) * inv) + cds) + cis;
    } else {
        col = ((cdd + cds) + cid) + cis;
    }
    f3 em = one;
    if (m.tex[TS_EMISSIVE] >= 0) em = srgb_fast3(unpack_rgb(sample_slot(sc, m, TS_EMISSIVE, uvx, uvy, du_dv)));
    col = col + em * mk3(m.emissive[0], m.emissive[1], m.emissive[2]);
    return col;
}

__device__ __forceinline__ uint32_t tonemap_pack(f3 c, float exposure) {
    // blit_to_buffer (src/renderer.rs:325-348) and tonemap (src/util.rs:37-41).
    const float k = 0.2f;
    const float kk = 1.0f + k;
    c = c * exposure;
    const f3 d = c + mk3(k, k, k);
    c = mk3(c.x / d.x, c.y / d.y, c.z / d.z) * kk;
    c = c * 255.0f;
    const uint32_t r = f2u8_sat(c.x), g = f2u8_sat(c.y), b = f2u8_sat(c.z);
    return (r << 24) | (g << 16) | (b << 8) | 0xFFu;
}

// One lane of the shading pass; all 32 lanes of a warp call it together
// (quad barycentrics and luminance are exchanged with warp shuffles).
// Whether pixel lane k of quad (qx, qy) of view v is shaded: inside the
// view, or in the centre quad of a reference tile (the luminance meter).
__device__ __forceinline__ bool shade_needed(const DView& v, int32_t qx, int32_t qy) {
    const bool centre = ((qx & 31) == 0) && ((qy & 31) == 16);
    return (2 * qx < v.width && 2 * qy < v.height) || centre;
}

// Shades lane k of quad (qx, qy) of view v given the pixel's depth key; all
// 32 lanes of a warp call it together, 4 consecutive lanes per quad. MODE:
// the reciprocal square root of every view of the launch, so only that one
// is compiled in, or kModeAny to read it from the view.
template <bool GI, int MODE>
__device__ __forceinline__ void shade_pixel(const FrameArgs& a, const uint8_t* tab, const DView& v,
                                            const DScene& sc, int32_t qx, int32_t qy, int32_t k, bool needed,
                                            unsigned long long key) {
    const uint32_t md = MODE == kModeAny ? v.rsqrt_mode : (uint32_t)MODE;
    const uint32_t lane = threadIdx.x & 31u;
    const int32_t kx = k & 1, ky = k >> 1;
    const int32_t px = 2 * qx + kx, py = 2 * qy + ky;
    const bool centre = ((qx & 31) == 0) && ((qy & 31) == 16);
    const bool writer = key != kEmptyKey;
    const float z = ordered_to_float((uint32_t)(key >> 32));
    const bool covered = writer && !(z == __int_as_float(0x7F800000));
    uint32_t slot = 0;
    RecRaster r;
    float b1 = 0.0f, b2 = 0.0f;
    if (writer) {
        const uint32_t s8 = key_seq8(key);
        const uint32_t g = s8 >> 3, f = s8 & 7u;
        slot = f == 0 ? g : a.fan_base[g] + f - 1u;
        const float4* src = reinterpret_cast<const float4*>(a.rec_r + slot);
        float4* dst = reinterpret_cast<float4*>(&r);
#pragma unroll
        for (int i = 0; i < 5; ++i) dst[i] = __ldg(src + i);
        rebuild_bary(r, px, py, b1, b2);
    }
    // bary1/bary2 of all four lanes of the quad (uncovered lanes hold 0, the
    // contents of a fresh renderer's vbuffer; src/tilerasterizer.rs:114-118).
    float qb1[4], qb2[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        qb1[i] = __shfl_sync(0xFFFFFFFFu, b1, (int)((lane & ~3u) + (uint32_t)i));
        qb2[i] = __shfl_sync(0xFFFFFFFFu, b2, (int)((lane & ~3u) + (uint32_t)i));
    }
    f3 col = mk3(0.0f, 0.0f, 0.0f);
    uint32_t vis_hi = 0xFFFFFFFFu, vis_fan = 0;
    if (needed) {
        if (covered) {
            RecShade q;
            {
                const float4* src = reinterpret_cast<const float4*>(a.rec_s + slot);
                float4* dst = reinterpret_cast<float4*>(&q);
#pragma unroll
                for (int i = 0; i < 11; ++i) dst[i] = __ldg(src + i);
            }
            // 1 / w at each quad lane's bary with this lane's triangle; this
            // lane's own entry is the w that shading uses (qb*[k] = b1, b2).
            float wq[4], dd[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                wq[i] = 1.0f / interp(r.oow, qb1[i], qb2[i]);
                dd[i] = q.du_dv[i] * wq[i];
            }
            const float w_own = k == 0 ? wq[0] : (k == 1 ? wq[1] : (k == 2 ? wq[2] : wq[3]));
            const DMaterial& m = sc.materials[r.material & kRecMaterialMask];
            col = pbr_lane<false, GI>(sc, v, m, q, w_own, b1, b2, dd, md, tab, col);
            vis_hi = q.static_id;
            vis_fan = r.seq8 & 7u;
        } else {
            col = skybox(v, sc, 2 * qx, 2 * qy, kx, ky, md, tab);
        }
    }
    // Tile-centre luminance (src/tilerasterizer.rs:103-106): quad (0, 16).
    const float lum = (col.x * 0.2126f + col.y * 0.7152f) + col.z * 0.0722f;
    const float l0 = __shfl_sync(0xFFFFFFFFu, lum, (int)(lane & ~3u));
    const float l1 = __shfl_sync(0xFFFFFFFFu, lum, (int)((lane & ~3u) + 1u));
    const float l2 = __shfl_sync(0xFFFFFFFFu, lum, (int)((lane & ~3u) + 2u));
    const float l3 = __shfl_sync(0xFFFFFFFFu, lum, (int)((lane & ~3u) + 3u));
    if (needed && centre && k == 0) {
        const uint32_t tile = (uint32_t)(qy >> 5) * (uint32_t)v.tiles_x + (uint32_t)(qx >> 5);
        v.tile_lum[tile] = (((l0 + l1) + l2) + l3) * 0.25f;
    }
    if (!needed) return;
    if (px < v.width && py < v.height) {
        v.vis[(uint64_t)py * (uint64_t)v.width + (uint64_t)px] =
            covered ? (((unsigned long long)vis_hi << 3) | vis_fan) : ~0ull;
    }
    if (v.flags) {
        // Linear colour over the padded tile grid (the translucent pass may
        // blend into the off-screen centre quad the luminance meter reads).
        float* c = v.color + ((uint64_t)py * v.key_pitch + (uint64_t)px) * 3u;
        c[0] = col.x;
        c[1] = col.y;
        c[2] = col.z;
    } else if (px < v.width && py < (v.height & ~1)) {
        const uint32_t c = tonemap_pack(col, v.exposure);
        v.rgba8[(uint64_t)py * v.out_pitch + (uint64_t)px] = c;
        if (v.rgba8_host) v.rgba8_host[(uint64_t)py * v.host_pitch + (uint64_t)px] = c;
    }
}

// Quad (qx, qy) of view-local quad index lq over the padded quad grid
// (quad_pitch = tiles_x * 32 quads wide, tiles_y * 32 rows). Each warp's
// eight quads form a 4x2 block (8x4 pixels), blocks row by row: a warp's
// pixels then fall on fewer triangles than in a 16x2 strip, so its record and
// texture loads hit more often (4K shade 0.604 -> 0.580 ms; 2x4 blocks and
// 8x4-quad blocks per CTA measured the same). The block row is
// (lq >> 6) / tiles_x by a multiply with the view's reciprocal (exact:
// lq >> 6 < 2^23, tiles_x <= 512).
__device__ __forceinline__ void quad_xy(const DView& v, uint32_t lq, int32_t& qx, int32_t& qy) {
    const uint32_t n = lq >> 6;
    const uint32_t brow = v.tiles_x_magic ? __umulhi(n, v.tiles_x_magic) : n;
    const uint32_t bcol = (lq >> 3) - brow * (v.quad_pitch >> 2);
    qx = (int32_t)(bcol * 4u + (lq & 3u));
    qy = (int32_t)(brow * 2u + ((lq >> 2) & 1u));
}

// One lane of the shading pass over the padded quad grid of every view.
template <bool GI, int MODE>
__device__ __forceinline__ void shade_thread(const FrameArgs& a, const uint8_t* tab, uint32_t gt, uint32_t total) {
    const uint32_t gq = gt >> 2;
    const bool live = gq < total;
    const uint32_t vi = find_view_by_quad(a, live ? gq : 0u);
    const DView& v = a.views[vi];
    int32_t qx, qy;
    quad_xy(v, gq - v.quad_base, qx, qy);
    const int32_t k = (int32_t)(gt & 3u);
    const bool needed = live && shade_needed(v, qx, qy);
    unsigned long long key = kEmptyKey;
    if (needed)
        key = a.keys[v.key_offset + (uint64_t)(2 * qy + (k >> 1)) * v.key_pitch + (uint64_t)(2 * qx + (k & 1))];
    shade_pixel<GI, MODE>(a, tab, v, a.scenes[v.scene], qx, qy, k, needed, key);
}

// CTA shape of the grid-stride shading kernel. Without voxel GI, seven
// 128-thread CTAs per SM (<= 72 registers): 4K frame shade 0.604 ms, against
// 0.612 ms at three 256-thread CTAs (80 registers), 0.741 ms at two (95) and
// 0.663 ms at four (64). The GI variant keeps three 256-thread CTAs: at 72
// registers its cone-tracing loop spills 216 B per thread.
template <bool GI> struct ShadeShape {
    static constexpr int kThreads = GI ? 256 : 128;
    static constexpr int kMinBlocks = GI ? 3 : 7;
};
// GI: the frame has scenes with a baked voxel grid. MODE: see shade_pixel.
template <bool GI, int MODE>
__global__ void __launch_bounds__(ShadeShape<GI>::kThreads, ShadeShape<GI>::kMinBlocks) k_shade(FrameArgs a) {
    __shared__ uint8_t tab[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) tab[i] = a.rsqrt_table[i];
    __syncthreads();
    // Every view's quad count is a multiple of 32, so each warp's lanes are
    // either all live or all past the end (warp-uniform loop).
    const uint32_t total = a.dyn->total_quads;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total * 4u; base += stride)
        shade_thread<GI, MODE>(a, tab, base + threadIdx.x, total);
}

__global__ void k_rsqrt_selftest(const float* in, float* out, uint64_t n, uint32_t mode, const uint8_t* table) {
    __shared__ uint8_t tab[512];
    for (int i = threadIdx.x; i < 512; i += blockDim.x) tab[i] = table[i];
    __syncthreads();
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = rsqrt_mode(in[i], mode, tab);
}

// --------------------------------------------------------------------------
// Translucent forward pass (render_tile, src/tilerasterizer.rs:92-101)
// --------------------------------------------------------------------------
constexpr int kTransCap = 2048;  // translucent packets one scheduling tile can sort
constexpr int kTransThreads = 256;

// Sort key of a translucent packet: OrderedFloat avg_z back to front (NaN is
// the largest value, -0 equals +0), then submission order. The reference's
// in-place quicksort (src/bumpqueue.rs:155-233) is unstable over a
// rayon-ordered queue, so it defines no order for equal keys; submission
// order is the one chosen here.
__device__ __forceinline__ unsigned long long trans_key(float avg_z, uint32_t seq8) {
    const uint32_t o = (avg_z != avg_z) ? 0xFFFFFFFFu : float_to_ordered(avg_z);
    return ((unsigned long long)(0xFFFFFFFFu - o) << 32) | (unsigned long long)seq8;
}

// Edge values of a quad's four lanes at quad (i, j) of a region with origin
// (ox, oy), as fine_raster reaches them: step_y added j times to the origin
// value, then step_x i times. Closed form where every partial sum is an
// integer below 2^24 (then exact), else the additions themselves.
__device__ __forceinline__ void quad_edge_values(const Edge& e, int32_t ox, int32_t oy, int32_t i, int32_t j,
                                                 float out[4]) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float v = edge_eval(e, i2f(ox + ((k & 1) ? 24 : 8)), i2f(oy + ((k >> 1) ? 24 : 8)));
        const float b = ru_add(ru_add(fabsf(v), ru_mul((float)j, fabsf(e.sy))), ru_mul((float)i, fabsf(e.sx)));
        if (b <= 16777216.0f) {
            v = v + (e.sy * (float)j + e.sx * (float)i);
        } else {
            for (int32_t t = 0; t < j; ++t) v += e.sy;
            for (int32_t t = 0; t < i; ++t) v += e.sx;
        }
        out[k] = v;
    }
}

// Per scheduling tile, after opaque shading: sort the tile's translucent
// packets back to front, then every thread walks its own quads through the
// sorted packets (fine_raster coverage, depth test against the opaque depth,
// TranslucentForwardShader blend over the current colour; no depth write).
// Quads are disjoint, so the per-pixel order is the sorted order.
template <int S>
__global__ void __launch_bounds__(kTransThreads) k_translucent(FrameArgs a) {
    __shared__ unsigned long long tkey[kTransCap];
    __shared__ uint32_t tslot[kTransCap];
    __shared__ uint32_t tsorted[kTransCap];
    __shared__ uint32_t tblk[kTransCap];
    __shared__ uint8_t tab[512];
    __shared__ uint32_t cur_tile;
    for (int i = threadIdx.x; i < 512; i += blockDim.x) tab[i] = a.rsqrt_table[i];
    const uint32_t n_st = a.dyn->n_stiles;
    const bool bad = (a.counters->status & (ST_BIN_OVERFLOW | ST_CLIP_OVERFLOW | ST_QUEUE_OVERFLOW)) != 0u;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) cur_tile = atomicAdd(&a.counters->trans_next, 1u);
        __syncthreads();
        const uint32_t st = cur_tile;
        if (st >= n_st || bad) break;
        const uint32_t b0 = a.tile_offset[n_st + st], n = a.tile_offset[n_st + st + 1] - b0;
        if (n == 0u) continue;
        if (n > (uint32_t)kTransCap) {
            if (threadIdx.x == 0) atomicOr(&a.counters->status, ST_TRANS_OVERFLOW);
            continue;
        }
        const uint32_t vi = find_view_by_stile(a, st);
        const DView& view = a.views[vi];
        const DScene& sc = a.scenes[view.scene];
        const uint32_t local = st - view.stile_base;
        const int32_t sx0 = (int32_t)(local % (uint32_t)view.stiles_x) * S;
        const int32_t sy0 = (int32_t)(local / (uint32_t)view.stiles_x) * S;
        const int32_t tx0 = (sx0 / kRefTile) * kRefTile, ty0 = (sy0 / kRefTile) * kRefTile;
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
            const uint32_t slot = a.bins[b0 + i];
            tslot[i] = slot;
            tkey[i] = trans_key(__uint_as_float(a.rec_s[slot].pad[0]), a.rec_r[slot].seq8);
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {  // keys are unique: rank = position
            const unsigned long long k = tkey[i];
            uint32_t rank = 0;
            for (uint32_t j = 0; j < n; ++j) rank += tkey[j] < k ? 1u : 0u;
            tsorted[rank] = tslot[i];
        }
        __syncthreads();
        // Coarse flag and accepted 16-px blocks (coarse_raster's reject) per packet.
        for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
            PacketCtx c;
            load_packet(a, sc, tsorted[k], tx0, ty0, c);
            uint32_t m = 0;
            if (c.coarse) {
                m = 0x80000000u;
                for (int32_t by = 0; by * 256 < c.ye - c.ys; ++by)
                    for (int32_t bx = 0; bx * 256 < c.xe - c.xs; ++bx)
                        if (!block_rejected(c.e12, c.e20, c.e01, c.xs + 256 * bx, c.ys + 256 * by))
                            m |= 1u << (by * 5 + bx);
            }
            tblk[k] = m;
        }
        __syncthreads();
        for (int32_t q = threadIdx.x; q < (S / 2) * (S / 2); q += blockDim.x) {
            const int32_t px0 = sx0 + 2 * (q % (S / 2)), py0 = sy0 + 2 * (q / (S / 2));
            float zop[4];
            f3 col[4];
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const uint64_t pi = (uint64_t)(py0 + (l >> 1)) * view.key_pitch + (uint64_t)(px0 + (l & 1));
                zop[l] = ordered_to_float((uint32_t)(a.keys[view.key_offset + pi] >> 32));
                const float* cp = view.color + pi * 3u;
                col[l] = mk3(cp[0], cp[1], cp[2]);
            }
            const int32_t X = px0 * kSubpixelScale, Y = py0 * kSubpixelScale;
            bool touched = false;
            for (uint32_t k = 0; k < n; ++k) {
                const uint32_t slot = tsorted[k];
                const RecRaster& rr = a.rec_r[slot];
                int32_t x0, y0, x1, y1;
                clipped_rect(rr, tx0, ty0, x0, y0, x1, y1);
                const int32_t xs = (x0 & ~1) * kSubpixelScale, ys = (y0 & ~1) * kSubpixelScale;
                if (X < xs || X >= x1 * kSubpixelScale || Y < ys || Y >= y1 * kSubpixelScale) continue;
                int32_t ox = xs, oy = ys;
                const uint32_t blk = tblk[k];
                if (blk >> 31) {
                    const int32_t bx = (X - xs) >> 8, by = (Y - ys) >> 8;
                    if (!((blk >> (by * 5 + bx)) & 1u)) continue;
                    ox = xs + 256 * bx;
                    oy = ys + 256 * by;
                }
                const int32_t i = (X - ox) >> 5, j = (Y - oy) >> 5;
                PacketCtx c;
                load_packet(a, sc, slot, tx0, ty0, c);
                float w0[4], w1[4], w2[4];
                quad_edge_values(c.e12, ox, oy, i, j, w0);
                quad_edge_values(c.e20, ox, oy, i, j, w1);
                quad_edge_values(c.e01, ox, oy, i, j, w2);
                float b1[4], b2[4], wl[4];
                uint32_t mask = 0;
#pragma unroll
                for (int l = 0; l < 4; ++l) {
                    b1[l] = w1[l] * c.r.ooa;
                    b2[l] = w2[l] * c.r.ooa;
                    wl[l] = 1.0f / interp(c.r.oow, b1[l], b2[l]);
                    const float z = interp(c.r.zow, b1[l], b2[l]) * wl[l];
                    if (w0[l] >= 0.0f && w1[l] >= 0.0f && w2[l] >= 0.0f && z <= zop[l]) mask |= 1u << l;
                }
                if (mask == 0u) continue;
                RecShade qs;
                {
                    const float4* src = reinterpret_cast<const float4*>(a.rec_s + slot);
                    float4* dst = reinterpret_cast<float4*>(&qs);
#pragma unroll
                    for (int t = 0; t < 11; ++t) dst[t] = __ldg(src + t);
                }
                float dd[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) dd[l] = qs.du_dv[l] * wl[l];
                const DMaterial& m = sc.materials[c.r.material & kRecMaterialMask];
#pragma unroll
                for (int l = 0; l < 4; ++l)
                    if (mask & (1u << l))
                        col[l] = pbr_lane<true, true>(sc, view, m, qs, wl[l], b1[l], b2[l], dd, view.rsqrt_mode,
                                                      tab, col[l]);
                touched = true;
            }
            if (!touched) continue;
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                const uint64_t pi = (uint64_t)(py0 + (l >> 1)) * view.key_pitch + (uint64_t)(px0 + (l & 1));
                float* cp = view.color + pi * 3u;
                cp[0] = col[l].x;
                cp[1] = col[l].y;
                cp[2] = col[l].z;
            }
            // Centre luminance of the reference tile (src/tilerasterizer.rs:103-106): quad (0, 16).
            if ((px0 & (kRefTile - 1)) == 0 && (py0 & (kRefTile - 1)) == kRefTile / 2) {
                float l4[4];
#pragma unroll
                for (int l = 0; l < 4; ++l) l4[l] = (col[l].x * 0.2126f + col[l].y * 0.7152f) + col[l].z * 0.0722f;
                const uint32_t tile = (uint32_t)(py0 / kRefTile) * (uint32_t)view.tiles_x + (uint32_t)(px0 / kRefTile);
                view.tile_lum[tile] = (((l4[0] + l4[1]) + l4[2]) + l4[3]) * 0.25f;
            }
        }
    }
}

// Exposure applied after the host's update_auto_exposure (dt > 0 path).
__global__ void k_resolve(FrameArgs a) {
    const uint32_t vi = blockIdx.y;
    if (vi >= a.dyn->n_views) return;
    const DView& v = a.views[vi];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t w = (uint32_t)v.width, h = (uint32_t)(v.height & ~1);
    if (i >= w * h || !v.flags) return;
    const uint32_t x = i % w, y = i / w;
    const float* c = v.color + ((uint64_t)y * v.key_pitch + x) * 3u;
    const float e = a.exposure_dev ? *a.exposure_dev : v.exposure;
    const uint32_t p = tonemap_pack(mk3(c[0], c[1], c[2]), e);
    v.rgba8[(uint64_t)y * v.out_pitch + x] = p;
    if (v.rgba8_host) v.rgba8_host[(uint64_t)y * v.host_pitch + x] = p;
}

// --------------------------------------------------------------------------
// Host launch wrappers
// --------------------------------------------------------------------------
static uint64_t g_const_init_mask = 0;  // one bit per device

template <int S, bool FUSE>
static cudaError_t raster_smem_attr() {
    return cudaFuncSetAttribute(k_raster<S, FUSE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sizeof(RasterShared<S>));
}

cudaError_t init_kernel_constants() {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 64 && (g_const_init_mask >> dev) & 1ull) return cudaSuccess;
    float t[256];
    for (int i = 0; i < 256; ++i) t[i] = (float)i / 255.0f;
    e = cudaMemcpyToSymbol(c_unorm8, t, sizeof(t));
    if (e == cudaSuccess) e = raster_smem_attr<8, true>();
    if (e == cudaSuccess) e = raster_smem_attr<16, true>();
    if (e == cudaSuccess) e = raster_smem_attr<32, false>();
    if (e == cudaSuccess) e = raster_smem_attr<32, true>();
    if (e == cudaSuccess) e = raster_smem_attr<64, false>();
    if (e == cudaSuccess && dev < 64) g_const_init_mask |= 1ull << dev;
    return e;
}

template <int S, bool FUSE>
static int raster_blocks_per_sm() {
    int rb = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rb, k_raster<S, FUSE>, RasterShared<S>::kThreads,
                                                  sizeof(RasterShared<S>));
    return rb;
}

bool shade_fused(uint32_t S, bool fuse32) { return S <= kFusedShadeMaxTile || (S == 32 && fuse32); }

void frame_grids(int num_sms, uint32_t S, bool fuse32, uint32_t* raster_grid, uint32_t* shade_grid) {
    int rb = 1, sb = 1;
    switch (S) {
        case 8: rb = raster_blocks_per_sm<8, true>(); break;
        case 16: rb = raster_blocks_per_sm<16, true>(); break;
        case 32: rb = fuse32 ? raster_blocks_per_sm<32, true>() : raster_blocks_per_sm<32, false>(); break;
        default: rb = raster_blocks_per_sm<64, false>(); break;
    }
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sb, k_shade<false, kModeArm>, ShadeShape<false>::kThreads, 0);
    cudaGetLastError();
    *raster_grid = (uint32_t)(num_sms * (rb > 0 ? rb : 1));
    *shade_grid = (uint32_t)(num_sms * (sb > 0 ? sb : 1));
}

void launch_reset(const FrameArgs& a, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t n = a.stile_cap > 0 ? a.stile_cap : 1u;
    // Enough CTAs for the bins and for the draw-list blocks (one per 256 node slots).
    const uint32_t slot_blocks = a.gpu_draws ? (a.slot_cap + kSlotBlock - 1u) / kSlotBlock : 0u;
    k_reset<<<min(max((n + 255) / 256, slot_blocks), 1024u), 256, 0, s>>>(a);
}

uint32_t launch_frame(const FrameArgs& a, void* stream, int num_sms, cudaEvent_t* ev) {
    cudaStream_t s = (cudaStream_t)stream;
    auto mark = [&](int i) {
        if (ev) cudaEventRecord(ev[i], s);
    };
    uint32_t launches = 0;
    mark(0);
    launch_reset(a, stream);
    launches++;
    // Frames of at most 256 node slots are emitted inside k_reset
    // (k_draw_emit returns at once); with a slot capacity of at most 256 it
    // is not launched.
    if (a.gpu_draws) {
        const uint32_t sg = (a.slot_cap + kSlotBlock - 1u) / kSlotBlock;
        if (sg > 1u) {
            k_draw_emit<<<sg, kSlotBlock, 0, s>>>(a);
            launches++;
        }
    }
    mark(1);
    // A frame's chunks number at most T / 256 + draws: the grid follows the
    // record slots, not the chunk capacity (sized from the scenes' bounds,
    // it can be far larger than what a frame draws).
    if (a.chunk_cap > 0) {
        // Host-built draw lists (no-alloc frames) size chunk_cap exactly.
        const uint64_t most = a.gpu_draws ? (uint64_t)a.tri_cap / kChunkTris + a.draw_cap + 1u : a.chunk_cap;
        k_frontend<<<(uint32_t)std::min<uint64_t>(a.chunk_cap, most), kChunkTris, 0, s>>>(a);
        launches++;
    }
    mark(2);
    k_clip<<<num_sms * 4, 128, 0, s>>>(a);
    mark(3);
    k_scan<<<1, 1024, 0, s>>>(a);
    launches += 2;
    mark(4);
    {
        // Thread per record slot over the capacity: blocks start in slot order,
        // so bins list records mostly in slot order and the raster's record
        // loads stay coalesced (a grid-stride loop here made k_raster 2% slower).
        const uint64_t n = (uint64_t)a.tri_cap + a.extra_cap;
        if (n > 0) {
            k_scatter<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
            launches++;
        }
    }
    mark(5);
    const uint32_t rg = SWR_RASTER_PERSISTENT ? (a.raster_grid > 0 ? a.raster_grid : (uint32_t)num_sms)
                                              : (a.stile_cap > 0 ? a.stile_cap : 1u);
    switch (a.sched_tile) {
        case 8: k_raster<8, true><<<rg, RasterShared<8>::kThreads, sizeof(RasterShared<8>), s>>>(a); break;
        case 16: k_raster<16, true><<<rg, RasterShared<16>::kThreads, sizeof(RasterShared<16>), s>>>(a); break;
        case 32:
            if (a.fused_shade)
                k_raster<32, true><<<rg, RasterShared<32>::kThreads, sizeof(RasterShared<32>), s>>>(a);
            else
                k_raster<32, false><<<rg, RasterShared<32>::kThreads, sizeof(RasterShared<32>), s>>>(a);
            break;
        default: k_raster<64, false><<<rg, RasterShared<64>::kThreads, sizeof(RasterShared<64>), s>>>(a); break;
    }
    launches++;
    mark(6);
    if (!shade_fused(a.sched_tile, a.fused_shade != 0)) {
        if (a.has_gi) {
            // a.shade_grid is sized for the variant without GI; this one's
            // CTAs per SM are taken once (the same on every GB300).
            static const uint32_t gi_blocks = [] {
                int b = 0;
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_shade<true, kModeArm>, ShadeShape<true>::kThreads, 0);
                cudaGetLastError();
                return (uint32_t)(b > 0 ? b : 1);
            }();
            const uint32_t sg = (uint32_t)num_sms * gi_blocks;
            const uint32_t T = ShadeShape<true>::kThreads;
            if (a.rsqrt_uniform == 1u + kModeArm) k_shade<true, kModeArm><<<sg, T, 0, s>>>(a);
            else if (a.rsqrt_uniform == 1u + kModeIeee) k_shade<true, kModeIeee><<<sg, T, 0, s>>>(a);
            else k_shade<true, kModeAny><<<sg, T, 0, s>>>(a);
        } else {
            const uint32_t sg = a.shade_grid > 0 ? a.shade_grid : (uint32_t)num_sms;
            const uint32_t T = ShadeShape<false>::kThreads;
            if (a.rsqrt_uniform == 1u + kModeArm) k_shade<false, kModeArm><<<sg, T, 0, s>>>(a);
            else if (a.rsqrt_uniform == 1u + kModeIeee) k_shade<false, kModeIeee><<<sg, T, 0, s>>>(a);
            else k_shade<false, kModeAny><<<sg, T, 0, s>>>(a);
        }
        launches++;
    }
    mark(7);
    if (a.has_translucent) {
        const uint32_t tg = (uint32_t)num_sms * 2u;
        switch (a.sched_tile) {
            case 8: k_translucent<8><<<tg, kTransThreads, 0, s>>>(a); break;
            case 16: k_translucent<16><<<tg, kTransThreads, 0, s>>>(a); break;
            case 32: k_translucent<32><<<tg, kTransThreads, 0, s>>>(a); break;
            default: k_translucent<64><<<tg, kTransThreads, 0, s>>>(a); break;
        }
        launches++;
        if (!a.defer_resolve) {
            launch_resolve(a, stream);
            launches++;
        }
    }
    return launches;
}

bool depth_floor_host(const int32_t p[6], const float zow[3], const float oow[3], int32_t xe, int32_t ye, float& zlo) {
    return depth_floor(p, zow, oow, xe, ye, zlo);
}

cudaError_t launch_rsqrt_selftest(const float* in, float* out, uint64_t n, uint32_t mode, const uint8_t* table) {
    const uint64_t blocks = std::min<uint64_t>((n + 255) / 256, 4096);
    if (blocks > 0) k_rsqrt_selftest<<<(unsigned)blocks, 256>>>(in, out, n, mode, table);
    return cudaGetLastError();
}

void launch_resolve(const FrameArgs& a, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    const uint32_t maxpx = a.pixel_cap > 0 ? a.pixel_cap : 1u;
    dim3 grid((maxpx + 255) / 256, a.view_cap > 0 ? a.view_cap : 1u);
    k_resolve<<<grid, 256, 0, s>>>(a);
}

}  // namespace swr
