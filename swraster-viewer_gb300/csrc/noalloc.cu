// swr_render_frame_noalloc: one frame with no memory allocation at all.
//
// Who needs it: callers that cannot call cudaMalloc/cudaFree while they
// render: processes whose device memory is owned by another allocator (a
// framework's caching allocator, a fixed budget carved out at start-up), and
// real-time loops that cannot afford cudaMalloc/cudaFree, which may
// synchronize the whole device. The caller passes the scene (already
// resident), the camera and its own device output buffers; every per-frame
// work buffer lives in one file-scope __device__ array of fixed size.
//
// Limits: width, height <= 512; at most 16384 triangles pass the
// sphere/frustum test; at most 4096 nodes and 4096 draws; at most 65536
// (triangle, tile) pairs and 8192 extra clipped fan triangles. Larger frames
// are rejected before any GPU work; a frame whose (triangle, tile) pairs or
// clipped triangles exceed the fixed capacity on the device returns
// SWR_OVERFLOW.
//
// The array (about 9 MB) stays allocated on every GPU that loads the library
// until the process exits. Its device address is looked up with
// cudaGetSymbolAddress on the first call on each device. All calls on a
// device share that device's array and it keeps the last call's contents:
// the frame's counters and tile counts are cleared by the first kernel of
// every call. A call holds its device's lock until its frame has finished
// (it waits for its stream before returning), so calls in one process never
// overlap on a GPU; were that lock or that wait removed, calls whose work
// overlapped on the GPU would race on the array. Calls on different devices
// run concurrently; they share only the host staging buffers, under a
// separate lock held while the tables are staged.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/swr.h"
#include "internal.h"
#include "renderer.h"
#include "scene.h"

namespace swr {
namespace {

constexpr int kNaMaxDim = 512;
constexpr uint32_t kNaMaxTris = 16384;
constexpr uint32_t kNaExtra = 8192;
constexpr uint32_t kNaMaxNodes = 4096;
constexpr uint32_t kNaMaxDraws = 4096;
constexpr uint32_t kNaMaxChunks = kNaMaxTris / kChunkTris + kNaMaxDraws;
constexpr uint32_t kNaBinCap = 65536;
constexpr uint32_t kNaTiles = (kNaMaxDim / kRefTile) * (kNaMaxDim / kRefTile);

constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }
// Scratch layout (byte offsets).
constexpr size_t oDyn = 0;
constexpr size_t oScene = oDyn + al(sizeof(DFrameDyn));
constexpr size_t oView = oScene + al(sizeof(DScene));
constexpr size_t oDraws = oView + al(sizeof(DView));
constexpr size_t oChunks = oDraws + al(sizeof(DDraw) * kNaMaxDraws);
constexpr size_t oState = oChunks + al(sizeof(DChunk) * kNaMaxChunks);
constexpr size_t oRecR = oState + al(kNaMaxTris);
constexpr size_t oRecS = oRecR + al(sizeof(RecRaster) * (kNaMaxTris + kNaExtra));
constexpr size_t oFan = oRecS + al(sizeof(RecShade) * (kNaMaxTris + kNaExtra));
constexpr size_t oClipQ = oFan + al(sizeof(uint32_t) * kNaMaxTris);
constexpr size_t oCount = oClipQ + al(sizeof(uint2) * kNaMaxTris);
constexpr size_t oOffset = oCount + al(sizeof(uint32_t) * (kNaTiles + 1));
constexpr size_t oCursor = oOffset + al(sizeof(uint32_t) * (kNaTiles + 1));
constexpr size_t oBins = oCursor + al(sizeof(uint32_t) * (kNaTiles + 1));
constexpr size_t oKeys = oBins + al(sizeof(uint32_t) * kNaBinCap);
constexpr size_t oCounters = oKeys + al(sizeof(unsigned long long) * kNaMaxDim * kNaMaxDim);
constexpr size_t oTab = oCounters + al(sizeof(DCounters));
constexpr size_t oLum = oTab + al(512);
constexpr size_t kNaScratchBytes = oLum + al(sizeof(float) * kNaTiles);

__device__ __align__(256) unsigned char g_noalloc_scratch[kNaScratchBytes];

constexpr int kMaxDevices = 64;
unsigned char* g_dev_ptr[kMaxDevices] = {};
int g_dev_sms[kMaxDevices] = {};
std::mutex g_dev_mu[kMaxDevices];  // per device: its scratch array and set-up
std::mutex g_stage_mu;              // the host staging buffers below

// Host staging (static, no heap): scene, view, draws, chunks.
unsigned char g_stage[al(sizeof(DFrameDyn)) + al(sizeof(DScene)) + al(sizeof(DView)) + al(sizeof(DDraw) * kNaMaxDraws) +
                      al(sizeof(DChunk) * kNaMaxChunks)];
uint32_t g_raster_grid[64] = {}, g_shade_grid[64] = {};
uint32_t g_order[kNaMaxNodes], g_tmp[kNaMaxNodes];
float g_key[kNaMaxNodes];

bool less_key(uint32_t a, uint32_t b) {
    const float x = g_key[a], y = g_key[b];
    if (x != x) return false;
    if (y != y) return true;
    return x < y;
}

// Stable bottom-up merge sort of g_order[0..n) by g_key (OrderedFloat order),
// equivalent to the stable sort of compute_nodes_by_distance.
void stable_sort_nodes(uint32_t n) {
    uint32_t* src = g_order;
    uint32_t* dst = g_tmp;
    for (uint32_t w = 1; w < n; w *= 2) {
        for (uint32_t lo = 0; lo < n; lo += 2 * w) {
            const uint32_t mid = lo + w < n ? lo + w : n;
            const uint32_t hi = lo + 2 * w < n ? lo + 2 * w : n;
            uint32_t i = lo, j = mid, k = lo;
            while (i < mid && j < hi) dst[k++] = less_key(src[j], src[i]) ? src[j++] : src[i++];
            while (i < mid) dst[k++] = src[i++];
            while (j < hi) dst[k++] = src[j++];
        }
        uint32_t* t = src;
        src = dst;
        dst = t;
    }
    if (src != g_order) std::memcpy(g_order, src, n * sizeof(uint32_t));
}

swr_status na_fail(swr_status st, const char* msg) {
    set_last_error(msg);
    return st;
}

}  // namespace
}  // namespace swr

extern "C" swr_status swr_render_frame_noalloc(const swr_scene* scene, const swr_camera* cam, int32_t width,
                                                int32_t height, float exposure, uint32_t rsqrt_mode, uint32_t* rgba8,
                                                uint64_t* vis, void* stream_v) {
    using namespace swr;
    if (!scene || !cam || !rgba8 || !vis) return na_fail(SWR_INVALID_ARG, "null argument");
    if (width <= 0 || height <= 0 || width > kNaMaxDim || height > kNaMaxDim)
        return na_fail(SWR_INVALID_ARG, "swr_render_frame_noalloc: width and height must be in [1, 512]");
    if (rsqrt_mode > SWR_RSQRT_AARCH64) return na_fail(SWR_INVALID_ARG, "bad rsqrt_mode");
    if (!(exposure > 0.0f) || !std::isfinite(exposure)) return na_fail(SWR_INVALID_ARG, "exposure must be positive");
    const SceneImpl& s = scene->impl;
    if (!s.d_scene) return na_fail(SWR_INVALID_ARG, "scene was created host-only");
    if (s.nodes.size() > kNaMaxNodes)
        return na_fail(SWR_INVALID_ARG, "swr_render_frame_noalloc: the scene has more than 4096 nodes");
    cudaStream_t stream = (cudaStream_t)stream_v;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return na_fail(SWR_CUDA_ERROR, "cudaGetDevice failed");
    // Lock order: the device's lock, then (while staging) the staging lock.
    std::lock_guard<std::mutex> dev_lock(g_dev_mu[dev]);
    if (!g_dev_ptr[dev]) {
        // One-time set-up for this device.
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return na_fail(SWR_CUDA_ERROR, "cudaGetSymbolAddress(scratch) failed");
        }
        uint8_t tab[512];
        build_rsqrt_table(tab);
        e = cudaMemcpy(static_cast<unsigned char*>(p) + oTab, tab, 512, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return na_fail(SWR_CUDA_ERROR, "scratch set-up copy failed");
        }
        if (init_kernel_constants() != cudaSuccess) {
            cudaGetLastError();
            return na_fail(SWR_CUDA_ERROR, "kernel constant set-up failed");
        }
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        g_dev_sms[dev] = sms > 0 ? sms : 148;
        frame_grids(g_dev_sms[dev], 64, false, &g_raster_grid[dev], &g_shade_grid[dev]);
        g_dev_ptr[dev] = static_cast<unsigned char*>(p);
    }
    unsigned char* base = g_dev_ptr[dev];
    std::unique_lock<std::mutex> stage_lock(g_stage_mu);
    // Draws in canonical order (compute_nodes_by_distance + render_node +
    // render_mesh + test_sphere_frustum), into static host arrays.
    const uint32_t nn = (uint32_t)s.nodes.size();
    const V3 cp = {cam->position[0], cam->position[1], cam->position[2]};
    for (uint32_t i = 0; i < nn; ++i) {
        g_order[i] = i;
        const V3 d = sub(cp, {s.nodes[i].sphere[0], s.nodes[i].sphere[1], s.nodes[i].sphere[2]});
        g_key[i] = dot3(d, d);
    }
    stable_sort_nodes(nn);
    DDraw* draws = reinterpret_cast<DDraw*>(g_stage + oDraws);
    DChunk* chunks = reinterpret_cast<DChunk*>(g_stage + oDraws + al(sizeof(DDraw) * kNaMaxDraws));
    uint32_t nd = 0, nc = 0, tri = 0;
    const M4 vp = from_array(cam->view_project);
    const M4 view_m = from_array(cam->view);
    for (uint32_t oi = 0; oi < nn; ++oi) {
        const uint32_t ni = g_order[oi];
        const HNode& n = s.nodes[ni];
        if (n.mesh < 0) continue;
        const M4 mvp = mulmm(vp, n.transform);
        const HMesh& m = s.meshes[n.mesh];
        if (!m.translucent.empty())
            return na_fail(SWR_INVALID_ARG, "translucent primitives need a colour buffer: use swr_render_frame");
        for (uint32_t lp : m.opaque) {
            const uint32_t gp = m.prims[lp];
            const HPrimitive& p = s.prims[gp];
            const float scale =
                ((length4(n.transform.c[0]) + length4(n.transform.c[1])) + length4(n.transform.c[2])) / 3.0f;
            const V3 c = transform_point3(n.transform, {p.sphere[0], p.sphere[1], p.sphere[2]});
            const float radius = p.sphere[3] * scale;
            const V4 cv = mulmv(view_m, {c.x, c.y, c.z, 1.0f});
            int cls = 0;  // 0 inside, 1 intersecting, 2 outside
            for (int k = 0; k < 6; ++k) {
                const V4 pl = {cam->view_clip_planes[k][0], cam->view_clip_planes[k][1], cam->view_clip_planes[k][2],
                               cam->view_clip_planes[k][3]};
                const float d = dot4(pl, cv);
                if (d < -radius) {
                    cls = 2;
                    break;
                }
                if (d < radius) cls = 1;
            }
            if (cls == 2) continue;
            const uint32_t tc = (uint32_t)(p.idx.size() / 3);
            if (tc == 0) continue;
            if (nd >= kNaMaxDraws) return na_fail(SWR_INVALID_ARG, "swr_render_frame_noalloc: more than 4096 draws");
            if (tri + tc > kNaMaxTris)
                return na_fail(SWR_INVALID_ARG, "swr_render_frame_noalloc: more than 16384 visible triangles");
            DDraw& d = draws[nd];
            to_array(mvp, d.mvp);
            d.node = ni;
            d.prim = gp;
            d.view = 0;
            d.clip = cls == 1 ? 1u : 0u;
            d.tri_begin = tri;
            d.tri_count = tc;
            d.static_base = n.tri_id_base + p.tri_id_base;
            d.scene = 0;
            for (uint32_t t = 0; t < tc; t += kChunkTris) chunks[nc++] = {nd, t};
            ++nd;
            tri += tc;
        }
    }
    DView* v = reinterpret_cast<DView*>(g_stage + oView);
    std::memset(v, 0, sizeof(DView));
    init_view(*v, *cam, width, height, 64);
    v->scene = 0;
    v->rsqrt_mode = rsqrt_mode;
    v->exposure = exposure;
    v->rgba8 = rgba8;
    v->vis = vis;
    v->tile_lum = reinterpret_cast<float*>(base + oLum);
    v->out_pitch = (uint32_t)width;
    v->stile_base = 0;
    v->quad_base = 0;
    v->key_offset = 0;
    std::memcpy(g_stage + oScene, &s.dscene, sizeof(DScene));
    DFrameDyn* dyn = reinterpret_cast<DFrameDyn*>(g_stage + oDyn);
    std::memset(dyn, 0, sizeof(DFrameDyn));
    dyn->n_views = 1;
    dyn->n_chunks = nc;
    dyn->tri_total = tri;
    dyn->n_stiles = (uint32_t)(v->stiles_x * v->stiles_y);
    dyn->n_bins = dyn->n_stiles;
    dyn->total_quads = v->quad_pitch * (uint32_t)v->tiles_y * 32u;
    dyn->max_view_pixels = (uint32_t)width * (uint32_t)(height & ~1);
    // Tables to the scratch array (pageable source: the copy is staged
    // before cudaMemcpyAsync returns, so the static buffer can be reused).
    cudaError_t e = cudaMemcpyAsync(base + oDyn, g_stage, oDraws + sizeof(DDraw) * nd, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess && nc)
        e = cudaMemcpyAsync(base + oChunks, chunks, sizeof(DChunk) * nc, cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return na_fail(SWR_CUDA_ERROR, "table upload failed");
    }
    stage_lock.unlock();  // the copies above have taken the staged tables
    FrameArgs a{};
    a.dyn = reinterpret_cast<DFrameDyn*>(base + oDyn);
    a.scenes = reinterpret_cast<const DScene*>(base + oScene);
    a.views = reinterpret_cast<DView*>(base + oView);
    a.draws = reinterpret_cast<DDraw*>(base + oDraws);
    a.chunks = reinterpret_cast<DChunk*>(base + oChunks);
    a.chunk_cap = nc;
    a.tri_cap = tri > 0 ? tri : 1u;
    a.extra_cap = kNaExtra;
    a.clip_cap = tri > 0 ? tri : 1u;
    a.stile_cap = dyn->n_stiles;
    a.quad_cap = dyn->total_quads;
    a.pixel_cap = dyn->max_view_pixels;
    a.view_cap = 1;
    a.bin_cap = kNaBinCap;
    a.sched_tile = 64;
    a.tri_state = base + oState;
    a.rec_r = reinterpret_cast<RecRaster*>(base + oRecR);
    a.rec_s = reinterpret_cast<RecShade*>(base + oRecS);
    a.fan_base = reinterpret_cast<uint32_t*>(base + oFan);
    a.clip_queue = reinterpret_cast<uint2*>(base + oClipQ);
    a.tile_count = reinterpret_cast<uint32_t*>(base + oCount);
    a.tile_offset = reinterpret_cast<uint32_t*>(base + oOffset);
    a.tile_cursor = reinterpret_cast<uint32_t*>(base + oCursor);
    a.bins = reinterpret_cast<uint32_t*>(base + oBins);
    a.keys = reinterpret_cast<unsigned long long*>(base + oKeys);
    a.counters = reinterpret_cast<DCounters*>(base + oCounters);
    a.rsqrt_table = base + oTab;
    a.exposure_dev = nullptr;
    a.has_gi = s.voxel_sh4.empty() ? 0u : 1u;
    a.raster_grid = g_raster_grid[dev];
    a.shade_grid = g_shade_grid[dev];
    launch_frame(a, stream, g_dev_sms[dev]);
    e = cudaGetLastError();
    if (e != cudaSuccess) return na_fail(SWR_CUDA_ERROR, "kernel launch failed");
    // Report device-side capacity overflow: wait for the frame, read the
    // status word (a copy, not an allocation).
    uint32_t status = 0;
    e = cudaMemcpyAsync(&status, base + oCounters, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return na_fail(SWR_CUDA_ERROR, "frame execution failed");
    }
    if (status & kStRetry)
        return na_fail(SWR_OVERFLOW, "swr_render_frame_noalloc: fixed scratch capacity exceeded (bins or clip output)");
    return SWR_OK;
}
