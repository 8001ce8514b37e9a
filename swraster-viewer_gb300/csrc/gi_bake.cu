// Voxel GI bake on the device (bake_voxel_gi, src/gi.rs:316-408): per active
// voxel 64 primary rays from one of nine direction sets; a ray that hits a
// surface gathers its one-bounce radiance (sun through trace_transmittance,
// four hemisphere sky-visibility rays, albedo and emissive textures,
// estimate_surface_bounce_radiance, src/gi.rs:466-547), a ray that escapes
// samples the sky cubemap; the radiance is projected to SH4, convolved to
// irradiance, floored (apply_min_brightness_floor) and stored with the sun
// and sky visibility; then blur_gi_sh4 (src/voxelgrid.rs:422-472).
//
// Rays are traced through a BVH built on the host: trace_nearest keeps the
// hit of smallest (t, triangle index) and trace_transmittance multiplies the
// translucent hits in that order, so results do not depend on the traversal
// order (the reference keeps its BVH crate's visiting order for equal t).
#include "precompute.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "devmath.cuh"

namespace swr {

namespace {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kRayEps = 1.0e-4f;
// Active voxels baked per chunk (64 rays each, 6 texture values a ray).
constexpr uint32_t kBakeChunkVoxels = 16384;

struct V {
    float x, y, z;
};
__device__ __forceinline__ V mk(float x, float y, float z) { return V{x, y, z}; }
__device__ __forceinline__ V operator+(V a, V b) { return V{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V operator-(V a, V b) { return V{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V operator*(V a, float s) { return V{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V operator*(V a, V b) { return V{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ V operator/(V a, float s) { return V{a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ float dot(V a, V b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V cross(V a, V b) {
    return V{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// Vec3A::normalize: self * (1 / length).
__device__ __forceinline__ V normalize(V a) { return a * (1.0f / __fsqrt_rn(dot(a, a))); }
__device__ __forceinline__ V vmax0(V a) { return V{fmaxf(a.x, 0.0f), fmaxf(a.y, 0.0f), fmaxf(a.z, 0.0f)}; }
__device__ __forceinline__ V ld3(const float* p) { return V{p[0], p[1], p[2]}; }

struct Dev {
    const BakeTri* tris;
    const BakeNode* nodes;
    const uint32_t* order;
    const BakeMaterial* mats;
    const uint32_t* texels;
    const BakeTexture* textures;
    const uint32_t* cubemap;
    const float* sky_lut;
    const float* dirs;
    const uint8_t* active;
    const float* sun;
    const uint32_t* active_list;
    uint32_t n_active;
    uint32_t n_nodes;
    uint32_t cube_size;
    float sh[4][3];
    float light_dir[3], light_color[3];
    uint32_t n;
    float vsz[3], cmin[3];
    float* out;  // n^3 x 16 before the blur
};

// ray_triangle_intersect (src/raytracer.rs:225-260).
__device__ __forceinline__ bool ray_tri(V o, V d, const BakeTri& t, float tmin, float tmax, float& th, float& bu,
                                        float& bv) {
    const V p0 = ld3(t.p0);
    const V e1 = ld3(t.p1) - p0, e2 = ld3(t.p2) - p0;
    const V pv = cross(d, e2);
    const float det = dot(e1, pv);
    if (fabsf(det) <= 1.0e-8f) return false;
    const float inv = 1.0f / det;
    const V tv = o - p0;
    const float u = dot(tv, pv) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const V qv = cross(tv, e1);
    const float v = dot(d, qv) * inv;
    if (v < 0.0f || (u + v) > 1.0f) return false;
    const float tt = dot(e2, qv) * inv;
    if (tt < tmin || tt > tmax) return false;
    th = tt;
    bu = u;
    bv = v;
    return true;
}

__device__ __forceinline__ bool hit_before(float ta, uint32_t ia, float tb, uint32_t ib) {
    const bool an = ta != ta, bn = tb != tb;
    if (an != bn) return bn;
    if (!an && ta != tb) return ta < tb;
    return ia < ib;
}

// Ray / node box (slab test from t = 0); returns the entry distance or -1.
__device__ __forceinline__ float box_entry(const BakeNode& nd, V o, const float inv[3]) {
    const float oo[3] = {o.x, o.y, o.z};
    float t0 = 0.0f, t1 = INFINITY;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float ta = (nd.mn[k] - oo[k]) * inv[k];
        float tb = (nd.mx[k] - oo[k]) * inv[k];
        if (ta != ta) ta = -INFINITY;
        if (tb != tb) tb = INFINITY;
        if (ta > tb) {
            const float s = ta;
            ta = tb;
            tb = s;
        }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
        if (t0 > t1) return -1.0f;
    }
    return t0;
}

constexpr int kStack = 64;

// trace_nearest (src/raytracer.rs:134-170): the hit of smallest
// (t, triangle). Boxes entered well beyond the best hit are skipped.
__device__ bool trace_nearest(const Dev& D, V o, V d, float tmin, uint32_t& tri, float& th, float& bu, float& bv) {
    const float inv[3] = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    uint32_t stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    bool found = false;
    float best = INFINITY;
    if (D.n_nodes == 0) return false;
    while (sp > 0) {
        const BakeNode nd = D.nodes[stack[--sp]];
        const float t0 = box_entry(nd, o, inv);
        if (t0 < 0.0f) continue;
        if (found && t0 > best + (fabsf(best) * 1.0e-3f + 1.0e-5f)) continue;
        if (nd.count == 0) {
            if (sp + 2 <= kStack) {
                stack[sp++] = nd.left;
                stack[sp++] = nd.left + 1;
            }
            continue;
        }
        for (uint32_t i = 0; i < nd.count; ++i) {
            const uint32_t ti = D.order[nd.left + i];
            float t, u, v;
            if (!ray_tri(o, d, D.tris[ti], tmin, INFINITY, t, u, v)) continue;
            if (!found || hit_before(t, ti, th, tri)) {
                found = true;
                tri = ti;
                th = t;
                bu = u;
                bv = v;
                best = t;
            }
        }
    }
    return found;
}

// One traversal collecting the smallest translucent hit after (last_t,
// last_i) (all hits when first); returns false at an opaque hit.
__device__ bool next_translucent(const Dev& D, V o, V d, float tmin, bool first, float last_t, uint32_t last_i,
                                 bool& found, float& bt, uint32_t& bi, uint32_t& count) {
    const float inv[3] = {1.0f / d.x, 1.0f / d.y, 1.0f / d.z};
    uint32_t stack[kStack];
    int sp = 0;
    stack[sp++] = 0;
    found = false;
    count = 0;
    if (D.n_nodes == 0) return true;
    while (sp > 0) {
        const BakeNode nd = D.nodes[stack[--sp]];
        if (box_entry(nd, o, inv) < 0.0f) continue;
        if (nd.count == 0) {
            if (sp + 2 <= kStack) {
                stack[sp++] = nd.left;
                stack[sp++] = nd.left + 1;
            }
            continue;
        }
        for (uint32_t i = 0; i < nd.count; ++i) {
            const uint32_t ti = D.order[nd.left + i];
            const BakeTri& t = D.tris[ti];
            float th, u, v;
            if (!ray_tri(o, d, t, tmin, INFINITY, th, u, v)) continue;
            if (!D.mats[t.material].translucent) return false;
            ++count;
            if (!first && !hit_before(last_t, last_i, th, ti)) continue;
            if (!found || hit_before(th, ti, bt, bi)) {
                found = true;
                bt = th;
                bi = ti;
            }
        }
    }
    return true;
}

// trace_transmittance (src/raytracer.rs:172-207).
__device__ float trace_transmittance(const Dev& D, V o, V d, float tmin) {
    bool found;
    float bt = 0.0f;
    uint32_t bi = 0, count = 0;
    if (!next_translucent(D, o, d, tmin, true, 0.0f, 0u, found, bt, bi, count)) return 0.0f;
    float tr = 1.0f;
    for (uint32_t h = 0; h < count && found; ++h) {
        tr *= D.mats[D.tris[bi].material].transmission;
        if (tr <= 0.0001f) return 0.0f;
        if (h + 1 == count) break;
        uint32_t c2;
        next_translucent(D, o, d, tmin, false, bt, bi, found, bt, bi, c2);
    }
    return tr;
}

__device__ __forceinline__ float unorm8(uint32_t b) { return (float)b / 255.0f; }

// TextureAndSampler::apply_wrap_mode (src/texture.rs:578-589); WrapMode
// 0 repeat, 1 mirrored repeat, 2 clamp to edge.
__device__ __forceinline__ float wrap(float t, float dim, uint32_t mode) {
    if (mode == 0u) {
        t = t - floorf(t / dim) * dim;
    } else if (mode == 1u) {
        const float two = dim * 2.0f;
        t = t - floorf(t / two) * two;
        t = fminf(t, two - t);
    }
    return fminf(t, dim - 1.0f);
}

// sample_bilinear_rgb at mip 0 (src/texture.rs:730-790): the sRGB values
// before srgb_to_linear_scalar, which the host applies (its powf).
__device__ void sample_bilinear_srgb(const Dev& D, const BakeTexture& T, float u, float v, uint32_t ws, uint32_t wt,
                                     float* c) {
    const float wf = (float)T.width, hf = (float)T.height;
    const float xf = u * wf - 0.5f, yf = v * hf - 0.5f;
    const float x0 = floorf(xf), y0 = floorf(yf);
    const float x1 = x0 + 1.0f, y1 = y0 + 1.0f;
    const float fx = xf - x0, fy = yf - y0;
    const float ofx = 1.0f - fx, ofy = 1.0f - fy;
    const uint32_t ix0 = f2u_sat(wrap(x0, wf, ws)), iy0 = f2u_sat(wrap(y0, hf, wt));
    const uint32_t ix1 = f2u_sat(wrap(x1, wf, ws)), iy1 = f2u_sat(wrap(y1, hf, wt));
    const uint32_t p00 = D.texels[T.offset + iy0 * T.width + ix0], p10 = D.texels[T.offset + iy0 * T.width + ix1];
    const uint32_t p01 = D.texels[T.offset + iy1 * T.width + ix0], p11 = D.texels[T.offset + iy1 * T.width + ix1];
    const float w00 = ofx * ofy, w10 = fx * ofy, w01 = ofx * fy, w11 = fx * fy;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const int sh = 24 - 8 * k;
        c[k] = ((unorm8((p00 >> sh) & 0xFFu) * w00 + unorm8((p10 >> sh) & 0xFFu) * w10) +
                unorm8((p01 >> sh) & 0xFFu) * w01) +
               unorm8((p11 >> sh) & 0xFFu) * w11;
    }
}

// sample_sky_radiance (src/gi.rs:580-593): nearest texel of cubemap mip 0.
__device__ V sky_radiance(const Dev& D, V d) {
    const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    const bool mx = (ax >= ay) && (ax >= az);
    const bool my = (ay > ax) && (ay >= az);
    const float sx = d.x >= 0.0f ? 1.0f : -1.0f, sy = d.y >= 0.0f ? 1.0f : -1.0f, sz = d.z >= 0.0f ? 1.0f : -1.0f;
    const float u = mx ? -d.z * sx : (my ? d.x : d.x * sz);
    const float v = mx ? -d.y : (my ? d.z * sy : -d.y);
    const float den = fmaxf(mx ? ax : (my ? ay : az), 1.0e-19f);
    const float uf = 0.5f * (u / den + 1.0f), vf = 0.5f * (v / den + 1.0f);
    const uint32_t slice = mx ? (d.x >= 0.0f ? 0u : 1u) : (my ? (d.y >= 0.0f ? 2u : 3u) : (d.z >= 0.0f ? 4u : 5u));
    const float wm1 = (float)D.cube_size - 1.0f;
    const uint32_t x = f2u_sat(fminf(fmaxf(round_away(uf * wm1), 0.0f), wm1));
    const uint32_t y = f2u_sat(fminf(fmaxf(round_away(vf * wm1), 0.0f), wm1));
    const uint32_t p = D.cubemap[slice * D.cube_size * D.cube_size + y * D.cube_size + x];
    return V{D.sky_lut[(p >> 24) & 0xFFu], D.sky_lut[(p >> 16) & 0xFFu], D.sky_lut[(p >> 8) & 0xFFu]};
}

// sky_visibility_hemisphere4 + tangent_basis (src/gi.rs:549-578).
__device__ float sky_visibility4(const Dev& D, V origin, V n, float dir_bias, float tmin) {
    const V up = fabsf(n.z) < 0.999f ? mk(0.0f, 0.0f, 1.0f) : mk(1.0f, 0.0f, 0.0f);
    const V tg = normalize(cross(n, up));
    const V bt = cross(n, tg);
    const float dl[4][3] = {{0.0f, 0.0f, 1.0f}, {0.8660254f, 0.0f, 0.5f}, {-0.4330127f, 0.75f, 0.5f},
                            {-0.4330127f, -0.75f, 0.5f}};
    float sum = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const V dir = normalize((tg * dl[i][0] + bt * dl[i][1]) + n * dl[i][2]);
        sum += trace_transmittance(D, origin + dir * dir_bias, dir, tmin);
    }
    return sum * 0.25f;
}

// The hit's texture coordinates (src/gi.rs:480-486).
__device__ __forceinline__ void hit_uv(const BakeTri& tri, float bu, float bv, float& uvx, float& uvy) {
    const float bw = (1.0f - bu) - bv;
    uvx = (tri.uv0[0] * bw + tri.uv1[0] * bu) + tri.uv2[0] * bv;
    uvy = (tri.uv0[1] * bw + tri.uv1[1] * bu) + tri.uv2[1] * bv;
}

// estimate_surface_bounce_radiance (src/gi.rs:466-547). lin: the ray's base
// and emissive texture samples in linear (srgb_to_linear_scalar of the
// bilinear sample, computed on the host).
__device__ V bounce_radiance(const Dev& D, uint32_t ti, float t, float bu, float bv, V o, V in_dir, float hit_bias,
                             float tmin, const float* lin) {
    const BakeTri& tri = D.tris[ti];
    const BakeMaterial& m = D.mats[tri.material];
    V nrm = ld3(tri.n);
    if (dot(nrm, in_dir * -1.0f) < 0.0f) nrm = nrm * -1.0f;
    V emissive = ld3(m.emissive);
    if (m.emissive_tex >= 0) emissive = emissive * ld3(lin + 3);
    emissive = vmax0(emissive);
    V albedo = ld3(m.base);
    if (m.base_tex >= 0) albedo = albedo * ld3(lin);
    albedo = V{fminf(fmaxf(albedo.x, 0.0f), 1.0f), fminf(fmaxf(albedo.y, 0.0f), 1.0f),
               fminf(fmaxf(albedo.z, 0.0f), 1.0f)} * 1.0f;
    if (dot(albedo, albedo) <= 0.0f && dot(emissive, emissive) <= 0.0f) return mk(0.0f, 0.0f, 0.0f);
    const float dir_bias = hit_bias * 0.5f;
    const V pos = o + in_dir * t;
    const V so = pos + nrm * hit_bias;
    const V ldir = ld3(D.light_dir);
    const float ndl = fmaxf(dot(nrm, ldir), 0.0f);
    V e_sun = mk(0.0f, 0.0f, 0.0f);
    if (ndl > 0.0f) {
        const float vis = trace_transmittance(D, so + ldir * dir_bias, ldir, tmin);
        e_sun = ld3(D.light_color) * (ndl * vis);
    }
    const float skyv = sky_visibility4(D, so, nrm, dir_bias, tmin);
    // eval_sh4_irradiance: c0 + c1 * n.y + c2 * n.z + c3 * n.x.
    const V c0 = ld3(D.sh[0]), c1 = ld3(D.sh[1]), c2 = ld3(D.sh[2]), c3 = ld3(D.sh[3]);
    const V e_sky = vmax0(((c0 + c1 * nrm.y) + c2 * nrm.z) + c3 * nrm.x) * skyv;
    const V e_tot = vmax0(e_sun + e_sky);
    const V bounce = dot(e_tot, e_tot) > 0.0f ? albedo * (e_tot / kPi) : mk(0.0f, 0.0f, 0.0f);
    return bounce + emissive;
}

__device__ __forceinline__ float luminance(V c) { return (0.2126f * c.x + 0.7152f * c.y) + 0.0722f * c.z; }

// The bake's per-voxel constants and the primary rays of a voxel.
struct BakeConsts {
    V vsz, cmin;
    float primary_weight, primary_bias, hit_bias, gi_tmin;
};
__device__ __forceinline__ BakeConsts bake_consts(const Dev& D) {
    BakeConsts c;
    c.vsz = ld3(D.vsz);
    c.cmin = ld3(D.cmin);
    const float vlen = __fsqrt_rn(dot(c.vsz, c.vsz));
    const float min_edge = fmaxf(fminf(fminf(c.vsz.x, c.vsz.y), c.vsz.z), 1.0e-6f);
    c.primary_weight = (4.0f * kPi) / (float)kGiSamples;
    c.primary_bias = fmaxf(vlen * 0.35f, kRayEps * 4.0f);
    c.hit_bias = fmaxf(vlen * 0.05f, kRayEps * 8.0f);
    c.gi_tmin = fmaxf(min_edge * 0.15f, kRayEps);
    return c;
}
// Voxel idx's centre and its direction set.
__device__ __forceinline__ void voxel_rays(const Dev& D, const BakeConsts& c, uint32_t idx, V& vc, const float*& dirs) {
    const uint32_t n = D.n;
    const uint32_t z = idx / (n * n), rem = idx % (n * n);
    const uint32_t y = rem / n, x = rem % n;
    vc = c.cmin + mk((float)x, (float)y, (float)z) * c.vsz;
    const uint32_t set = ((x % 3u) + 3u * (y % 3u) + (z % 3u)) % kGiSets;
    dirs = D.dirs + (size_t)set * kGiSamples * 3;
}

// Rays of a chunk of active voxels [k0, k1) are numbered r = (k - k0) * 64 + s.
// First step, one thread per ray: trace the primary ray; `hit` gets the
// nearest hit (triangle, t, u, v; triangle 0xFFFFFFFF when the ray escapes)
// and `srgb` the bilinear sRGB samples of the hit's base and emissive
// textures (6 floats; NaN where the hit has no such texture). The host turns
// the samples into linear values with its powf.
__global__ void __launch_bounds__(128) k_gi_tex(Dev D, uint32_t k0, uint32_t k1, uint4* hit, float* srgb) {
    const BakeConsts bc = bake_consts(D);
    const uint64_t nr = (uint64_t)(k1 - k0) * kGiSamples;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < nr; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = k0 + (uint32_t)(r / kGiSamples), s = (uint32_t)(r % kGiSamples);
        V vc;
        const float* dirs;
        voxel_rays(D, bc, D.active_list[k], vc, dirs);
        const V dir = ld3(dirs + 3 * s);
        const V ro = vc + dir * bc.primary_bias;
        float* o = srgb + r * 6;
#pragma unroll
        for (int c = 0; c < 6; ++c) o[c] = __int_as_float(0x7FC00000);
        uint32_t ti = 0;
        float th = 0.0f, bu = 0.0f, bv = 0.0f;
        if (!trace_nearest(D, ro, dir, bc.gi_tmin, ti, th, bu, bv)) {
            hit[r] = make_uint4(0xFFFFFFFFu, 0u, 0u, 0u);
            continue;
        }
        hit[r] = make_uint4(ti, __float_as_uint(th), __float_as_uint(bu), __float_as_uint(bv));
        const BakeTri& tri = D.tris[ti];
        const BakeMaterial& m = D.mats[tri.material];
        float uvx, uvy;
        hit_uv(tri, bu, bv, uvx, uvy);
        if (m.base_tex >= 0) sample_bilinear_srgb(D, D.textures[m.base_tex], uvx, uvy, m.base_wrap_s, m.base_wrap_t, o);
        if (m.emissive_tex >= 0)
            sample_bilinear_srgb(D, D.textures[m.emissive_tex], uvx, uvy, m.emissive_wrap_s, m.emissive_wrap_t, o + 3);
    }
}

// Second step, one thread per ray: its radiance (the bounce at the hit, with
// the texture samples in linear from `lin`, or the sky) into `rad`.
__global__ void __launch_bounds__(128) k_gi_ray(Dev D, uint32_t k0, uint32_t k1, const uint4* hit, const float* lin,
                                                float* rad) {
    const BakeConsts bc = bake_consts(D);
    const uint64_t nr = (uint64_t)(k1 - k0) * kGiSamples;
    for (uint64_t r = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; r < nr; r += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t k = k0 + (uint32_t)(r / kGiSamples), s = (uint32_t)(r % kGiSamples);
        V vc;
        const float* dirs;
        voxel_rays(D, bc, D.active_list[k], vc, dirs);
        const V dir = ld3(dirs + 3 * s);
        const V ro = vc + dir * bc.primary_bias;
        const uint4 h = hit[r];
        const V radiance = h.x == 0xFFFFFFFFu
                               ? sky_radiance(D, dir)
                               : bounce_radiance(D, h.x, __uint_as_float(h.y), __uint_as_float(h.z),
                                                 __uint_as_float(h.w), ro, dir, bc.hit_bias, bc.gi_tmin, lin + r * 6);
        rad[3 * r] = radiance.x;
        rad[3 * r + 1] = radiance.y;
        rad[3 * r + 2] = radiance.z;
    }
}

// Third step, one thread per voxel: its 64 radiances projected to SH4 in ray
// order, convolved, floored, stored with the sun and sky visibility.
__global__ void __launch_bounds__(128) k_gi_accum(Dev D, uint32_t k0, uint32_t k1, const uint4* hit,
                                                  const float* rad) {
    const BakeConsts bc = bake_consts(D);
    const float primary_weight = bc.primary_weight;
    for (uint32_t k = k0 + blockIdx.x * blockDim.x + threadIdx.x; k < k1; k += gridDim.x * blockDim.x) {
        const uint32_t idx = D.active_list[k];
        V vc;
        const float* dirs;
        voxel_rays(D, bc, idx, vc, dirs);
        V rsh[4] = {mk(0, 0, 0), mk(0, 0, 0), mk(0, 0, 0), mk(0, 0, 0)};
        uint32_t sky_hits = 0;
        for (uint32_t s = 0; s < kGiSamples; ++s) {
            const uint64_t r = (uint64_t)(k - k0) * kGiSamples + s;
            const V dir = ld3(dirs + 3 * s);
            if (hit[r].x == 0xFFFFFFFFu) ++sky_hits;
            const V radiance = ld3(rad + 3 * r);
            if (dot(radiance, radiance) <= 0.0f) continue;
            // project_radiance_sh4 (src/gi.rs:437-452).
            const float basis[4] = {0.282095f, 0.488603f * dir.y, 0.488603f * dir.z, 0.488603f * dir.x};
#pragma unroll
            for (int i = 0; i < 4; ++i) rsh[i] = rsh[i] + radiance * (basis[i] * primary_weight);
        }
        // radiance_to_irradiance_sh4 (src/gi.rs:454-461).
        rsh[0] = rsh[0] * (kPi * 0.282095f);
        const float k1c = ((2.0f * kPi) / 3.0f) * 0.488603f;
        rsh[1] = rsh[1] * k1c;
        rsh[2] = rsh[2] * k1c;
        rsh[3] = rsh[3] * k1c;
        V rgb[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) rgb[i] = vmax0(rsh[i]);
        // apply_min_brightness_floor (src/gi.rs:631-660).
        const V floor0 = ld3(D.sh[0]) * 0.005f;
        const float floor_lum = luminance(floor0);
        if (floor_lum > 0.0f) {
            const float cur = luminance(rgb[0]);
            if (cur < floor_lum) {
                const float t = fminf(fmaxf((floor_lum - cur) / floor_lum, 0.0f), 1.0f);
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const V target = ld3(D.sh[i]) * 0.005f;
                    rgb[i] = rgb[i] * (1.0f - t) + target * t;
                }
            }
        }
        float* o = D.out + (size_t)idx * 16;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            o[4 * i] = rgb[i].x;
            o[4 * i + 1] = rgb[i].y;
            o[4 * i + 2] = rgb[i].z;
            o[4 * i + 3] = 0.0f;
        }
        o[3] = D.sun[idx];
        o[7] = (float)sky_hits / (float)kGiSamples;
    }
}

// initialize_voxel_gi_from_scene(scale 1, sky 1) for voxels the bake skips.
__global__ void k_gi_init(Dev D) {
    const uint64_t total = (uint64_t)D.n * D.n * D.n;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        if (D.active[idx]) continue;
        float* o = D.out + idx * 16;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            o[4 * i] = D.sh[i][0] * 1.0f;
            o[4 * i + 1] = D.sh[i][1] * 1.0f;
            o[4 * i + 2] = D.sh[i][2] * 1.0f;
            o[4 * i + 3] = 0.0f;
        }
        o[3] = D.sun[idx];
        o[7] = 1.0f;
    }
}

// blur_gi_sh4 (src/voxelgrid.rs:422-472): mean of the in-range 3x3x3
// neighbours, coefficient by coefficient.
__global__ void k_gi_blur(const float* in, float* out, uint32_t n) {
    const uint64_t total = (uint64_t)n * n * n;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t z = (int32_t)(idx / ((uint64_t)n * n));
        const int32_t rem = (int32_t)(idx % ((uint64_t)n * n));
        const int32_t y = rem / (int32_t)n, x = rem % (int32_t)n;
        float sum[16];
#pragma unroll
        for (int c = 0; c < 16; ++c) sum[c] = 0.0f;
        float count = 0.0f;
        for (int32_t dz = -1; dz <= 1; ++dz)
            for (int32_t dy = -1; dy <= 1; ++dy)
                for (int32_t dx = -1; dx <= 1; ++dx) {
                    const int32_t nx = x + dx, ny = y + dy, nz = z + dz;
                    if (nx < 0 || nx >= (int32_t)n || ny < 0 || ny >= (int32_t)n || nz < 0 || nz >= (int32_t)n)
                        continue;
                    const float* s = in + ((uint64_t)nz * n * n + (uint64_t)ny * n + (uint64_t)nx) * 16;
#pragma unroll
                    for (int c = 0; c < 16; ++c) sum[c] += s[c];
                    count += 1.0f;
                }
        float* o = out + idx * 16;
#pragma unroll
        for (int c = 0; c < 16; ++c) o[c] = count > 0.0f ? sum[c] / count : in[idx * 16 + c];
    }
}

struct Mem {
    std::vector<void*> ptrs;
    ~Mem() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t put(T** dst, const T* src, size_t count) {
        void* q = nullptr;
        cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e != cudaSuccess) return e;
        ptrs.push_back(q);
        *dst = static_cast<T*>(q);
        if (src && count) e = cudaMemcpy(q, src, count * sizeof(T), cudaMemcpyHostToDevice);
        return e;
    }
};

struct HostPinned {
    float* p = nullptr;
    ~HostPinned() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t alloc(size_t count) {
        void* q = nullptr;
        const cudaError_t e = cudaMallocHost(&q, count * sizeof(float));
        p = static_cast<float*>(q);
        return e;
    }
};

}  // namespace

swr_status gi_bake_device(const BakeInput& in, float* out, std::string& err) {
    const uint32_t n = in.n;
    const uint64_t nvox = (uint64_t)n * n * n;
    std::vector<uint32_t> active_list;
    for (uint64_t i = 0; i < nvox; ++i)
        if (in.active[i]) active_list.push_back((uint32_t)i);
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    Mem m;
    Dev D{};
    BakeTri* tris = nullptr;
    BakeNode* nodes = nullptr;
    uint32_t *order = nullptr, *texels = nullptr, *cube = nullptr, *alist = nullptr;
    BakeMaterial* mats = nullptr;
    BakeTexture* texs = nullptr;
    float *lut = nullptr, *dirs = nullptr, *sun = nullptr, *raw = nullptr, *blur = nullptr;
    uint8_t* active = nullptr;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (x != cudaSuccess && e == cudaSuccess) e = x;
    };
    chk(m.put(&tris, in.tris, in.ntris));
    chk(m.put(&nodes, in.nodes, in.nnodes));
    chk(m.put(&order, in.order, in.ntris));
    chk(m.put(&mats, in.mats, in.nmat));
    chk(m.put(&texels, in.texels, in.ntexels));
    chk(m.put(&texs, in.textures, in.ntex));
    chk(m.put(&cube, in.cubemap, (size_t)6 * in.cube_size * in.cube_size));
    chk(m.put(&lut, in.sky_lut, 256));
    chk(m.put(&dirs, in.dirs, (size_t)kGiSets * kGiSamples * 3));
    chk(m.put(&active, in.active, nvox));
    chk(m.put(&sun, in.sun, nvox));
    chk(m.put(&alist, active_list.data(), active_list.size()));
    chk(m.put(&raw, (const float*)nullptr, nvox * 16));
    chk(m.put(&blur, (const float*)nullptr, nvox * 16));
    if (e == cudaSuccess) {
        D.tris = tris;
        D.nodes = nodes;
        D.order = order;
        D.mats = mats;
        D.texels = texels;
        D.textures = texs;
        D.cubemap = cube;
        D.sky_lut = lut;
        D.dirs = dirs;
        D.active = active;
        D.sun = sun;
        D.active_list = alist;
        D.n_active = (uint32_t)active_list.size();
        D.n_nodes = (uint32_t)in.nnodes;
        D.cube_size = in.cube_size;
        for (int i = 0; i < 4; ++i)
            for (int c = 0; c < 3; ++c) D.sh[i][c] = in.irradiance_sh[i][c];
        for (int k = 0; k < 3; ++k) {
            D.light_dir[k] = in.light_dir[k];
            D.light_color[k] = in.light_color[k];
            D.vsz[k] = in.vsz[k];
            D.cmin[k] = in.cmin[k];
        }
        D.n = n;
        D.out = raw;
        const uint32_t vg = (uint32_t)std::min<uint64_t>((nvox + 255) / 256, (uint64_t)sms * 16);
        k_gi_init<<<vg, 256>>>(D);
        e = cudaGetLastError();
        // The active voxels in chunks: the texture samples of a chunk's rays
        // go to the host, which converts them to linear with its own powf
        // (bit for bit the reference's srgb_to_linear_scalar), then the
        // chunk is baked with them. Pipelined on one stream: the device
        // samples chunk i+1 and bakes chunk i-1 while the host converts
        // chunk i (two pinned buffers alternate).
        float *d_srgb = nullptr, *d_lin = nullptr, *d_rad = nullptr;
        uint4* d_hit[2] = {nullptr, nullptr};  // chunk i's hits in d_hit[i % 2]
        const uint32_t chunk = std::min<uint32_t>(std::max<uint32_t>(D.n_active, 1u), kBakeChunkVoxels);
        const size_t chunk_rays = (size_t)chunk * kGiSamples, chunk_vals = chunk_rays * 6;
        if (e == cudaSuccess) e = m.put(&d_srgb, (const float*)nullptr, chunk_vals);
        if (e == cudaSuccess) e = m.put(&d_lin, (const float*)nullptr, chunk_vals);
        if (e == cudaSuccess) e = m.put(&d_rad, (const float*)nullptr, chunk_rays * 3);
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) e = m.put(&d_hit[b], (const uint4*)nullptr, chunk_rays);
        HostPinned hp;
        cudaStream_t st = nullptr;
        cudaEvent_t ready[2] = {nullptr, nullptr};
        if (e == cudaSuccess && D.n_active) e = hp.alloc(2 * chunk_vals);
        if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        for (int b = 0; b < 2 && e == cudaSuccess; ++b) e = cudaEventCreateWithFlags(&ready[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);  // k_gi_init and the inputs
        const unsigned threads = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        const uint32_t n_chunks = (D.n_active + chunk - 1) / chunk;
        auto range = [&](uint32_t i, uint32_t& k0, uint32_t& k1) {
            k0 = i * chunk;
            k1 = std::min(D.n_active, k0 + chunk);
        };
        // Samples of chunk i into pinned buffer i % 2.
        auto sample = [&](uint32_t i) {
            uint32_t k0, k1;
            range(i, k0, k1);
            const size_t nv = (size_t)(k1 - k0) * kGiSamples * 6;
            k_gi_tex<<<(uint32_t)std::min<uint64_t>(((uint64_t)(k1 - k0) * kGiSamples + 127) / 128, (uint64_t)sms * 64),
                       128, 0, st>>>(D, k0, k1, d_hit[i % 2], d_srgb);
            cudaError_t x = cudaGetLastError();
            if (x == cudaSuccess)
                x = cudaMemcpyAsync(hp.p + (i % 2) * chunk_vals, d_srgb, nv * sizeof(float), cudaMemcpyDeviceToHost, st);
            if (x == cudaSuccess) x = cudaEventRecord(ready[i % 2], st);
            return x;
        };
        if (e == cudaSuccess && n_chunks) e = sample(0);
        for (uint32_t i = 0; i < n_chunks && e == cudaSuccess; ++i) {
            uint32_t k0, k1;
            range(i, k0, k1);
            const size_t nv = (size_t)(k1 - k0) * kGiSamples * 6;
            e = cudaEventSynchronize(ready[i % 2]);
            if (e == cudaSuccess && i + 1 < n_chunks) e = sample(i + 1);
            if (e != cudaSuccess) break;
            float* vals = hp.p + (i % 2) * chunk_vals;
            std::vector<std::thread> pool;
            for (unsigned t = 0; t < threads; ++t)
                pool.emplace_back([=] {
                    for (size_t j = nv * t / threads; j < nv * (t + 1) / threads; ++j)
                        if (vals[j] == vals[j]) vals[j] = srgb_to_linear_host(vals[j]);
                });
            for (auto& th : pool) th.join();
            // Stream order keeps this copy ahead of the next write to the
            // same pinned buffer (chunk i + 2's samples).
            e = cudaMemcpyAsync(d_lin, vals, nv * sizeof(float), cudaMemcpyHostToDevice, st);
            if (e != cudaSuccess) break;
            // Chunk i + 1 was sampled above into the other hit buffer; d_lin
            // and d_rad are next written after these two kernels in stream
            // order.
            k_gi_ray<<<(uint32_t)std::min<uint64_t>(((uint64_t)(k1 - k0) * kGiSamples + 127) / 128, (uint64_t)sms * 64),
                       128, 0, st>>>(D, k0, k1, d_hit[i % 2], d_lin, d_rad);
            k_gi_accum<<<(uint32_t)std::min<uint64_t>((k1 - k0 + 127) / 128, (uint64_t)sms * 64), 128, 0, st>>>(
                D, k0, k1, d_hit[i % 2], d_rad);
            e = cudaGetLastError();
        }
        if (st) {
            const cudaError_t x = cudaStreamSynchronize(st);
            if (e == cudaSuccess) e = x;
        }
        for (cudaEvent_t ev : ready)
            if (ev) cudaEventDestroy(ev);
        if (st) cudaStreamDestroy(st);
        if (e == cudaSuccess) {
            k_gi_blur<<<vg, 256>>>(raw, blur, n);
            e = cudaGetLastError();
        }
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, blur, nvox * 16 * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = std::string("device GI bake: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR;
    }
    return SWR_OK;
}

}  // namespace swr
