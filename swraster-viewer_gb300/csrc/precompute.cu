// Voxel sun visibility on the device (scene admission): every ray of
// compute_sun_visibility (src/gi.rs:267-314) starts at a voxel centre and
// runs along the one light direction, so instead of a BVH the triangles are
// binned into a 2D grid over the plane across the light: a ray meets a
// triangle's padded bounding box (the reference's BVH test, 1e-5 padding,
// src/raytracer.rs:113-121) only where its projection lies inside the box's
// projected silhouette, so it needs only the triangles binned in the one cell
// its origin projects to. Each candidate then gets the exact
// Moller-Trumbore test of ray_triangle_intersect (src/raytracer.rs:225-260).
//
//   k_lv_count / k_lv_scatter  triangle -> cells its padded box covers
//   k_lv_scan                  exclusive scan of cell counts (one CTA)
//   k_lv_trace                 thread per voxel: transmittance toward the sun
//   k_lv_blur                  blur_grid: 3x3x3 mean, squared
#include "precompute.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

namespace swr {

namespace {

struct LightGrid {
    float u[3], v[3];       // basis of the plane across the light
    float umin, vmin;       // grid origin in that plane
    float inv_cell;         // cells per unit
    float margin;           // widening of every projected box (rounding of the projections)
    uint32_t g;             // cells per side
};

__device__ __forceinline__ float dot3d(const float* a, float x, float y, float z) {
    return (a[0] * x + a[1] * y) + a[2] * z;
}

__device__ __forceinline__ int32_t cell_of(float p, float mn, float inv, uint32_t g) {
    const float c = floorf((p - mn) * inv);
    if (!(c >= 0.0f)) return 0;
    if (c >= (float)(g - 1)) return (int32_t)(g - 1);
    return (int32_t)c;
}

// Cell range of a triangle: the reference pads its bounding box by 1e-5 per
// axis; the 8 corners of that box are projected and the range widened by
// the projection's rounding margin.
__device__ void tri_cells(const LightTri& t, const LightGrid& G, int32_t& cu0, int32_t& cu1, int32_t& cv0,
                          int32_t& cv1) {
    const float e = 1.0e-5f;
    float mn[3], mx[3];
    for (int k = 0; k < 3; ++k) {
        mn[k] = fminf(fminf(t.p0[k], t.p1[k]), t.p2[k]) - e;
        mx[k] = fmaxf(fmaxf(t.p0[k], t.p1[k]), t.p2[k]) + e;
    }
    float u0 = INFINITY, u1 = -INFINITY, v0 = INFINITY, v1 = -INFINITY;
    for (int c = 0; c < 8; ++c) {
        const float x = (c & 1) ? mx[0] : mn[0], y = (c & 2) ? mx[1] : mn[1], z = (c & 4) ? mx[2] : mn[2];
        const float pu = dot3d(G.u, x, y, z), pv = dot3d(G.v, x, y, z);
        u0 = fminf(u0, pu);
        u1 = fmaxf(u1, pu);
        v0 = fminf(v0, pv);
        v1 = fmaxf(v1, pv);
    }
    cu0 = cell_of(u0 - G.margin, G.umin, G.inv_cell, G.g);
    cu1 = cell_of(u1 + G.margin, G.umin, G.inv_cell, G.g);
    cv0 = cell_of(v0 - G.margin, G.vmin, G.inv_cell, G.g);
    cv1 = cell_of(v1 + G.margin, G.vmin, G.inv_cell, G.g);
}

__global__ void k_lv_count(const LightTri* tris, uint32_t n, LightGrid G, uint32_t* count) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int32_t cu0, cu1, cv0, cv1;
        tri_cells(tris[i], G, cu0, cu1, cv0, cv1);
        for (int32_t cv = cv0; cv <= cv1; ++cv)
            for (int32_t cu = cu0; cu <= cu1; ++cu) atomicAdd(count + (uint32_t)cv * G.g + (uint32_t)cu, 1u);
    }
}

// Exclusive scan of n counts into off[0..n] (single CTA); cursor = off.
__global__ void __launch_bounds__(1024) k_lv_scan(const uint32_t* count, uint32_t n, uint32_t* off, uint32_t* cursor) {
    __shared__ uint32_t part[1024];
    const uint32_t per = (n + 1023u) / 1024u;
    const uint32_t b = threadIdx.x * per, e = min(b + per, n);
    uint32_t s = 0;
    for (uint32_t i = b; i < e; ++i) s += count[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (uint32_t o = 1; o < 1024u; o <<= 1) {
        const uint32_t v = threadIdx.x >= o ? part[threadIdx.x - o] : 0u;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    uint32_t run = part[threadIdx.x] - s;
    for (uint32_t i = b; i < e; ++i) {
        off[i] = run;
        cursor[i] = run;
        run += count[i];
    }
    if (threadIdx.x == 1023) off[n] = part[1023];
}

__global__ void k_lv_scatter(const LightTri* tris, uint32_t n, LightGrid G, uint32_t* cursor, uint32_t* list) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        int32_t cu0, cu1, cv0, cv1;
        tri_cells(tris[i], G, cu0, cu1, cv0, cv1);
        for (int32_t cv = cv0; cv <= cv1; ++cv)
            for (int32_t cu = cu0; cu <= cu1; ++cu) list[atomicAdd(cursor + (uint32_t)cv * G.g + (uint32_t)cu, 1u)] = i;
    }
}

// ray_triangle_intersect (src/raytracer.rs:225-260) in the host
// restatement's operation order.
__device__ __forceinline__ bool ray_tri(const float o[3], const float d[3], const LightTri& t, float tmin, float tmax,
                                        float& th) {
    const float e1[3] = {t.p1[0] - t.p0[0], t.p1[1] - t.p0[1], t.p1[2] - t.p0[2]};
    const float e2[3] = {t.p2[0] - t.p0[0], t.p2[1] - t.p0[1], t.p2[2] - t.p0[2]};
    const float pv[3] = {d[1] * e2[2] - d[2] * e2[1], d[2] * e2[0] - d[0] * e2[2], d[0] * e2[1] - d[1] * e2[0]};
    const float det = (e1[0] * pv[0] + e1[1] * pv[1]) + e1[2] * pv[2];
    if (fabsf(det) <= 1.0e-8f) return false;
    const float inv = 1.0f / det;
    const float tv[3] = {o[0] - t.p0[0], o[1] - t.p0[1], o[2] - t.p0[2]};
    const float u = ((tv[0] * pv[0] + tv[1] * pv[1]) + tv[2] * pv[2]) * inv;
    if (!(u >= 0.0f && u <= 1.0f)) return false;
    const float qv[3] = {tv[1] * e1[2] - tv[2] * e1[1], tv[2] * e1[0] - tv[0] * e1[2], tv[0] * e1[1] - tv[1] * e1[0]};
    const float v = ((d[0] * qv[0] + d[1] * qv[1]) + d[2] * qv[2]) * inv;
    if (v < 0.0f || (u + v) > 1.0f) return false;
    const float tt = ((e2[0] * qv[0] + e2[1] * qv[1]) + e2[2] * qv[2]) * inv;
    if (tt < tmin || tt > tmax) return false;
    th = tt;
    return true;
}

// (t, index) order with a NaN t after every number.
__device__ __forceinline__ bool hit_before(float ta, uint32_t ia, float tb, uint32_t ib) {
    const bool an = ta != ta, bn = tb != tb;
    if (an != bn) return bn;
    if (!an && ta != tb) return ta < tb;
    return ia < ib;
}

struct TraceArgs {
    const LightTri* tris;
    const uint32_t* off;
    const uint32_t* list;
    const uint8_t* translucent;
    const float* transmission;
    const uint8_t* active;
    float* light;
    uint32_t n;
    float cmin[3], vsz[3], ld[3];
    float bias;
    LightGrid G;
};

// trace_transmittance: 0 at any opaque hit, else the product of the
// translucent hits' transmissions in hit order, 0 once it reaches 1e-4.
__global__ void k_lv_trace(TraceArgs a) {
    const uint32_t n = a.n;
    const uint64_t total = (uint64_t)n * n * n;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        if (!a.active[idx]) {
            a.light[idx] = 1.0f;
            continue;
        }
        const uint32_t z = (uint32_t)(idx / ((uint64_t)n * n));
        const uint32_t rem = (uint32_t)(idx % ((uint64_t)n * n));
        const uint32_t y = rem / n, x = rem % n;
        float o[3];
        const float xyz[3] = {(float)x, (float)y, (float)z};
        for (int k = 0; k < 3; ++k) {
            const float vc = a.cmin[k] + xyz[k] * a.vsz[k];
            o[k] = vc + a.ld[k] * a.bias;
        }
        const LightGrid& G = a.G;
        const int32_t cu = cell_of(dot3d(G.u, o[0], o[1], o[2]), G.umin, G.inv_cell, G.g);
        const int32_t cv = cell_of(dot3d(G.v, o[0], o[1], o[2]), G.vmin, G.inv_cell, G.g);
        const uint32_t cell = (uint32_t)cv * G.g + (uint32_t)cu;
        const uint32_t b0 = a.off[cell], b1 = a.off[cell + 1];
        uint32_t n_trans = 0;
        bool opaque = false;
        for (uint32_t k = b0; k < b1 && !opaque; ++k) {
            const uint32_t ti = a.list[k];
            const LightTri t = a.tris[ti];
            float th;
            if (!ray_tri(o, a.ld, t, 1.0e-4f, INFINITY, th)) continue;
            if (!a.translucent[t.material]) opaque = true;
            else ++n_trans;
        }
        float tr = 1.0f;
        if (opaque) {
            tr = 0.0f;
        } else {
            // The translucent hits in order, one pass over the cell per hit.
            float last_t = -INFINITY;
            uint32_t last_i = 0;
            bool first = true;
            for (uint32_t h = 0; h < n_trans; ++h) {
                float best_t = 0.0f;
                uint32_t best_i = 0xFFFFFFFFu, best_m = 0;
                bool found = false;
                for (uint32_t k = b0; k < b1; ++k) {
                    const uint32_t ti = a.list[k];
                    const LightTri t = a.tris[ti];
                    float th;
                    if (!ray_tri(o, a.ld, t, 1.0e-4f, INFINITY, th)) continue;
                    if (!first && !hit_before(last_t, last_i, th, ti)) continue;
                    if (!found || hit_before(th, ti, best_t, best_i)) {
                        best_t = th;
                        best_i = ti;
                        best_m = t.material;
                        found = true;
                    }
                }
                if (!found) break;
                tr *= a.transmission[best_m];
                if (tr <= 0.0001f) {
                    tr = 0.0f;
                    break;
                }
                last_t = best_t;
                last_i = best_i;
                first = false;
            }
        }
        a.light[idx] = tr;
    }
}

// blur_grid (src/voxelgrid.rs:370-419): mean of the in-range 3x3x3
// neighbours (z, y, x loops in that order), squared.
__global__ void k_lv_blur(const float* in, float* out, uint32_t n) {
    const uint64_t total = (uint64_t)n * n * n;
    for (uint64_t idx = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; idx < total;
         idx += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t z = (int32_t)(idx / ((uint64_t)n * n));
        const int32_t rem = (int32_t)(idx % ((uint64_t)n * n));
        const int32_t y = rem / (int32_t)n, x = rem % (int32_t)n;
        float sum = 0.0f;
        int32_t count = 0;
        for (int32_t dz = -1; dz <= 1; ++dz)
            for (int32_t dy = -1; dy <= 1; ++dy)
                for (int32_t dx = -1; dx <= 1; ++dx) {
                    const int32_t nx = x + dx, ny = y + dy, nz = z + dz;
                    if (nx >= 0 && nx < (int32_t)n && ny >= 0 && ny < (int32_t)n && nz >= 0 && nz < (int32_t)n) {
                        sum += in[(uint64_t)nz * n * n + (uint64_t)ny * n + (uint64_t)nx];
                        count += 1;
                    }
                }
        const float m = count > 0 ? sum / (float)count : 0.0f;
        out[idx] = count > 0 ? m * m : 0.0f;
    }
}

struct DevMem {
    std::vector<void*> ptrs;
    ~DevMem() {
        for (void* p : ptrs) cudaFree(p);
    }
    template <class T>
    cudaError_t alloc(T** p, size_t count) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, std::max<size_t>(count, 1) * sizeof(T));
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
};

}  // namespace

swr_status sun_visibility_device(const LightTri* tris, size_t ntris, const uint8_t* translucent,
                                 const float* transmission, uint32_t nmat, const uint8_t* active, uint32_t n,
                                 const float bounds_min[3], const float bounds_max[3], const float cmin[3],
                                 const float vsz[3], const float ld[3], float bias, float* out, std::string& err) {
    if (ntris > 0xFFFFFFF0ull) {
        err = "too many triangles for the device sun visibility";
        return SWR_INVALID_ARG;
    }
    const uint64_t nvox = (uint64_t)n * n * n;
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // Grid over the plane across the light: basis, bounds of the projected
    // scene box, about 2 cells per triangle (at most 1024 per side).
    LightGrid G{};
    {
        const float up[3] = {std::fabs(ld[1]) < 0.9f ? 0.0f : 1.0f, std::fabs(ld[1]) < 0.9f ? 1.0f : 0.0f, 0.0f};
        float u[3] = {ld[1] * up[2] - ld[2] * up[1], ld[2] * up[0] - ld[0] * up[2], ld[0] * up[1] - ld[1] * up[0]};
        const float ul = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
        for (float& c : u) c /= ul;
        const float v[3] = {ld[1] * u[2] - ld[2] * u[1], ld[2] * u[0] - ld[0] * u[2], ld[0] * u[1] - ld[1] * u[0]};
        for (int k = 0; k < 3; ++k) {
            G.u[k] = u[k];
            G.v[k] = v[k];
        }
        float u0 = INFINITY, u1 = -INFINITY, v0 = INFINITY, v1 = -INFINITY, mag = 0.0f;
        for (int c = 0; c < 8; ++c) {
            const float x = (c & 1) ? bounds_max[0] : bounds_min[0];
            const float y = (c & 2) ? bounds_max[1] : bounds_min[1];
            const float z = (c & 4) ? bounds_max[2] : bounds_min[2];
            const float pu = (G.u[0] * x + G.u[1] * y) + G.u[2] * z, pv = (G.v[0] * x + G.v[1] * y) + G.v[2] * z;
            u0 = std::fmin(u0, pu);
            u1 = std::fmax(u1, pu);
            v0 = std::fmin(v0, pv);
            v1 = std::fmax(v1, pv);
            mag = std::fmax(mag, std::fabs(x) + std::fabs(y) + std::fabs(z));
        }
        const float ext = std::fmax(std::fmax(u1 - u0, v1 - v0), 1.0e-6f);
        // Rounding of a projection is below 3 ulp of the largest |coordinate| sum.
        G.margin = 8.0f * 1.1920929e-7f * (mag + ext) + 1.0e-6f * ext;
        const float pad = 4.0f * G.margin + 0.01f * ext;
        G.umin = u0 - pad;
        G.vmin = v0 - pad;
        const double side = std::sqrt(2.0 * (double)std::max<size_t>(ntris, 1));
        G.g = (uint32_t)std::min(1024.0, std::max(16.0, side));
        G.inv_cell = (float)G.g / (ext + 2.0f * pad);
    }
    const uint32_t cells = G.g * G.g;
    DevMem m;
    LightTri* d_tris = nullptr;
    uint32_t *d_count = nullptr, *d_off = nullptr, *d_cursor = nullptr, *d_list = nullptr;
    uint8_t *d_trans = nullptr, *d_active = nullptr;
    float *d_transm = nullptr, *d_light = nullptr, *d_blur = nullptr;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (x != cudaSuccess && e == cudaSuccess) e = x;
    };
    chk(m.alloc(&d_tris, ntris));
    chk(m.alloc(&d_count, cells));
    chk(m.alloc(&d_off, cells + 1));
    chk(m.alloc(&d_cursor, cells));
    chk(m.alloc(&d_trans, nmat));
    chk(m.alloc(&d_transm, nmat));
    chk(m.alloc(&d_active, nvox));
    chk(m.alloc(&d_light, nvox));
    chk(m.alloc(&d_blur, nvox));
    if (e == cudaSuccess && ntris) e = cudaMemcpy(d_tris, tris, ntris * sizeof(LightTri), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nmat) e = cudaMemcpy(d_trans, translucent, nmat, cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nmat) e = cudaMemcpy(d_transm, transmission, nmat * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_active, active, nvox, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_count, 0, cells * sizeof(uint32_t));
    const uint32_t tgrid = (uint32_t)std::min<uint64_t>((ntris + 255) / 256 + 1, (uint64_t)sms * 16);
    if (e == cudaSuccess) {
        k_lv_count<<<tgrid, 256>>>(d_tris, (uint32_t)ntris, G, d_count);
        k_lv_scan<<<1, 1024>>>(d_count, cells, d_off, d_cursor);
        e = cudaGetLastError();
    }
    uint32_t entries = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&entries, d_off + cells, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) chk(m.alloc(&d_list, entries));
    if (e == cudaSuccess) {
        k_lv_scatter<<<tgrid, 256>>>(d_tris, (uint32_t)ntris, G, d_cursor, d_list);
        TraceArgs a{};
        a.tris = d_tris;
        a.off = d_off;
        a.list = d_list;
        a.translucent = d_trans;
        a.transmission = d_transm;
        a.active = d_active;
        a.light = d_light;
        a.n = n;
        for (int k = 0; k < 3; ++k) {
            a.cmin[k] = cmin[k];
            a.vsz[k] = vsz[k];
            a.ld[k] = ld[k];
        }
        a.bias = bias;
        a.G = G;
        const uint32_t vgrid = (uint32_t)std::min<uint64_t>((nvox + 127) / 128, (uint64_t)sms * 32);
        k_lv_trace<<<vgrid, 128>>>(a);
        k_lv_blur<<<(uint32_t)std::min<uint64_t>((nvox + 255) / 256, (uint64_t)sms * 16), 256>>>(d_light, d_blur, n);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, d_blur, nvox * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        err = std::string("device sun visibility: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR;
    }
    return SWR_OK;
}

}  // namespace swr
