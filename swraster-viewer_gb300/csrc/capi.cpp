// extern "C" entry points (include/swr.h). No exception crosses the ABI;
// every failure becomes a status plus a thread-local message.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <limits>
#include <new>
#include <string>

#include "../../include/swr.h"
#include "caches.h"
#include "ibl.h"
#include "renderer.h"
#include "scene.h"

using namespace swr;

namespace {

thread_local std::string g_err;

swr_status fail(swr_status st, const std::string& msg) {
    g_err = msg;
    return st;
}
swr_status cuda_fail(cudaError_t e, const char* what) {
    cudaGetLastError();
    return fail(e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

namespace swr {
// Lets entry points outside this file report through swr_last_error().
void set_last_error(const char* msg) { g_err = msg; }
}  // namespace swr

extern "C" {

const char* swr_last_error(void) { return g_err.c_str(); }
int32_t swr_abi_version(void) { return SWR_ABI_VERSION; }

// ---------------------------------------------------------------- scene

swr_status swr_scene_create(const swr_scene_desc* desc, swr_scene** out) {
    if (!desc || !out) return fail(SWR_INVALID_ARG, "null argument");
    *out = nullptr;
    swr_scene* s = new (std::nothrow) swr_scene();
    if (!s) return fail(SWR_NO_MEMORY, "out of host memory");
    std::string err;
    swr_status st;
    try {
        st = build_scene(desc, &s->impl, err);
        if (st == SWR_OK) st = upload_scene(&s->impl, err, !(desc->flags & SWR_SCENE_HOST_ONLY));
    } catch (const std::bad_alloc&) {
        st = SWR_NO_MEMORY;
        err = "out of host memory";
    } catch (...) {
        st = SWR_BAD_SCENE;
        err = "scene construction failed";
    }
    if (st != SWR_OK) {
        free_scene_device(&s->impl);
        delete s;
        return fail(st, err);
    }
    *out = s;
    return SWR_OK;
}

void swr_scene_destroy(swr_scene* s) {
    if (!s) return;
    free_scene_device(&s->impl);
    delete s;
}

swr_status swr_scene_get_info(const swr_scene* s, swr_scene_info* o) {
    if (!s || !o) return fail(SWR_INVALID_ARG, "null argument");
    const SceneImpl& m = s->impl;
    std::memset(o, 0, sizeof(*o));
    o->triangle_count = m.tri_total;
    o->vertex_count = m.vtx_total;
    o->device_bytes = m.d_bytes;
    o->node_count = (uint32_t)m.nodes.size();
    uint32_t draws = 0;
    for (const HNode& n : m.nodes)
        if (n.mesh >= 0) draws += (uint32_t)m.meshes[n.mesh].prims.size();
    o->draw_count = draws;
    o->bounds_min[0] = m.bounds_min.x; o->bounds_min[1] = m.bounds_min.y; o->bounds_min[2] = m.bounds_min.z;
    o->bounds_max[0] = m.bounds_max.x; o->bounds_max[1] = m.bounds_max.y; o->bounds_max[2] = m.bounds_max.z;
    o->bounds_center[0] = m.bounds_center.x; o->bounds_center[1] = m.bounds_center.y;
    o->bounds_center[2] = m.bounds_center.z;
    o->bounds_diagonal = m.bounds_diagonal;
    o->gi_cache = m.gi_cache;
    o->ggx_cache = m.ggx_cache;
    o->precompute_host_texels = m.precompute_host_texels;
    return SWR_OK;
}

swr_status swr_scene_save_gi_cache(const swr_scene* s, const char* path) {
    if (!s || !path) return fail(SWR_INVALID_ARG, "null argument");
    if (s->impl.voxel_sh4.empty()) return fail(SWR_INVALID_ARG, "the scene has no baked GI grid (SWR_SCENE_GI)");
    std::string err;
    try {
        if (!write_gi_cache(path, s->impl.voxel_n, s->impl.voxel_sh4, err)) return fail(SWR_IO_ERROR, err);
    } catch (const std::bad_alloc&) {
        return fail(SWR_NO_MEMORY, "out of host memory");
    }
    return SWR_OK;
}

swr_status swr_scene_save_ggx_cache(const swr_scene* s, const char* path) {
    if (!s || !path) return fail(SWR_INVALID_ARG, "null argument");
    std::string err;
    try {
        if (!write_ggx_cache(path, s->impl.specular, err)) return fail(SWR_IO_ERROR, err);
    } catch (const std::bad_alloc&) {
        return fail(SWR_NO_MEMORY, "out of host memory");
    }
    return SWR_OK;
}

swr_status swr_scene_export(const swr_scene* s, swr_scene_host_view* out) {
    if (!s || !out) return fail(SWR_INVALID_ARG, "null argument");
    export_scene(&s->impl, out);
    return SWR_OK;
}

// ---------------------------------------------------------------- camera

// RenderCamera::new (src/rendercamera.rs:28-63).
swr_status swr_camera_init(swr_camera* c, const float pos[3], const float look[3], float fov, float width,
                           float height, float far_plane) {
    if (!c || !pos || !look) return fail(SWR_INVALID_ARG, "null argument");
    if (!(width > 0.0f) || !(height > 0.0f)) return fail(SWR_INVALID_ARG, "camera size must be positive");
    std::memset(c, 0, sizeof(*c));
    const V3 p = {pos[0], pos[1], pos[2]};
    const V3 f = normalize3(sub({look[0], look[1], look[2]}, p));
    c->position[0] = p.x;
    c->position[1] = p.y;
    c->position[2] = p.z;
    c->fov = fov;
    c->width = width;
    c->height = height;
    c->one_over_width = 1.0f / width;
    c->one_over_height = 1.0f / height;
    c->near_plane = far_plane * 0.01f;
    c->far_plane = far_plane;
    c->yaw = std::atan2(f.x, -f.z);
    c->pitch = std::asin(f.y);
    c->roll = 0.0f;
    const M4 id = identity4();
    to_array(id, c->view);
    to_array(id, c->projection);
    to_array(id, c->view_project);
    to_array(id, c->inverse_view_project);
    to_array(id, c->skybox_transposed);
    return SWR_OK;
}

// RenderCamera::update_matrices (src/rendercamera.rs:78-150).
swr_status swr_camera_update(swr_camera* c) {
    if (!c) return fail(SWR_INVALID_ARG, "null argument");
    const Quat q = quat_mul(quat_mul(quat_rot_z(c->roll), quat_rot_x(c->pitch)), quat_rot_y(c->yaw));
    const M4 rot = mat_from_quat(q);
    const M4 view = mulmm(rot, mat_translation({-c->position[0], -c->position[1], -c->position[2]}));
    const M4 proj = perspective_rh(c->fov, c->width / c->height, c->near_plane, c->far_plane);
    const M4 vp = mulmm(proj, view);
    to_array(view, c->view);
    to_array(proj, c->projection);
    to_array(vp, c->view_project);
    to_array(inverse4(vp), c->inverse_view_project);
    to_array(transpose4(inverse4(mulmm(proj, rot))), c->skybox_transposed);
    const float aspect = c->width / c->height;
    const float tan_y = std::tan(c->fov * 0.5f);
    const float tan_x = tan_y * aspect;
    const V3 right = normalize3({1.0f, 0.0f, -tan_x});
    const V3 left = normalize3({-1.0f, 0.0f, -tan_x});
    const V3 top = normalize3({0.0f, 1.0f, -tan_y});
    const V3 bottom = normalize3({0.0f, -1.0f, -tan_y});
    const float planes[6][4] = {{0.0f, 0.0f, -1.0f, c->near_plane}, {0.0f, 0.0f, 1.0f, c->far_plane},
                                {right.x, right.y, right.z, 0.0f},   {left.x, left.y, left.z, 0.0f},
                                {top.x, top.y, top.z, 0.0f},         {bottom.x, bottom.y, bottom.z, 0.0f}};
    std::memcpy(c->view_clip_planes, planes, sizeof(planes));
    const V3 vn = quat_rotate(quat_conj(q), {0.0f, 0.0f, 1.0f});
    c->view_normal[0] = vn.x;
    c->view_normal[1] = vn.y;
    c->view_normal[2] = vn.z;
    return SWR_OK;
}

// ---------------------------------------------------------------- renderer

swr_status swr_renderer_create(int32_t width, int32_t height, const swr_renderer_opts* opts, swr_renderer** out) {
    if (!out) return fail(SWR_INVALID_ARG, "null argument");
    *out = nullptr;
    if (width <= 0 || height <= 0 || width > 32768 || height > 32768)
        return fail(SWR_INVALID_ARG, "renderer size out of range");
    swr_renderer_opts o{};
    o.rsqrt_mode = SWR_RSQRT_AARCH64;
    if (opts) o = *opts;
    if (o.rsqrt_mode > SWR_RSQRT_AARCH64) return fail(SWR_INVALID_ARG, "bad rsqrt_mode");
    if (o.sched_tile != 0 && o.sched_tile != 8 && o.sched_tile != 16 && o.sched_tile != 32 && o.sched_tile != 64)
        return fail(SWR_INVALID_ARG, "sched_tile must be 0, 8, 16, 32 or 64");
    swr_renderer* r = new (std::nothrow) swr_renderer();
    if (!r) return fail(SWR_NO_MEMORY, "out of host memory");
    r->width = width;
    r->height = height;
    r->opts = o;
    r->eng.bin_cap = o.bin_capacity;
    std::string err;
    swr_status st = r->eng.init(err);
    if (st != SWR_OK) {
        r->eng.release();
        delete r;
        return fail(st, err);
    }
    if (r->opts.sched_tile == 0) r->opts.sched_tile = auto_sched_tile(&width, &height, 1, r->eng.num_sms);
    r->eng.sched_tile = r->opts.sched_tile;
    r->tiles_x = (uint32_t)((width + 63) / 64);
    r->tiles_y = (uint32_t)((height + 63) / 64);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (x != cudaSuccess && e == cudaSuccess) e = x;
    };
    chk(r->rgba8.ensure((size_t)width * height * sizeof(uint32_t)));
    chk(r->vis.ensure((size_t)width * height * sizeof(uint64_t)));
    chk(r->tile_lum.ensure((size_t)r->tiles_x * r->tiles_y * sizeof(float)));
    chk(cudaHostAlloc((void**)&r->h_lum, (size_t)r->tiles_x * r->tiles_y * sizeof(float), cudaHostAllocDefault));
    chk(cudaHostAlloc((void**)&r->h_expo, sizeof(float), cudaHostAllocMapped));
    chk(cudaHostAlloc((void**)&r->h_status, sizeof(uint32_t), cudaHostAllocDefault));
    if (e == cudaSuccess) chk(cudaHostGetDevicePointer((void**)&r->d_expo, r->h_expo, 0));
    chk(cudaEventCreateWithFlags(&r->expo_done, cudaEventDisableTiming));
    chk(cudaHostAlloc((void**)&r->h_counters, sizeof(DCounters), cudaHostAllocDefault));
    chk(cudaEventCreateWithFlags(&r->status_ev, cudaEventDisableTiming));
    if (e != cudaSuccess) {
        swr_renderer_destroy(r);
        return cuda_fail(e, "renderer allocation");
    }
    *r->h_expo = r->expo.exposure;
    *out = r;
    return SWR_OK;
}

void swr_renderer_destroy(swr_renderer* r) {
    if (!r) return;
    cudaDeviceSynchronize();
    r->eng.release();
    r->rgba8.release();
    r->vis.release();
    r->tile_lum.release();
    if (r->h_lum) cudaFreeHost(r->h_lum);
    if (r->h_expo) cudaFreeHost(r->h_expo);
    if (r->h_status) cudaFreeHost(r->h_status);
    if (r->expo_done) cudaEventDestroy(r->expo_done);
    if (r->h_counters) cudaFreeHost(r->h_counters);
    if (r->status_ev) cudaEventDestroy(r->status_ev);
    for (auto& set : r->prof_ev)
        for (cudaEvent_t& e : set)
            if (e) cudaEventDestroy(e);
    delete r;
}

namespace {

void prof_collect(swr_renderer* r, int slot) {
    if (!r->prof_pending[slot]) return;
    cudaEvent_t* ev = r->prof_ev[slot];
    const int last = r->prof_resolve[slot] ? 9 : 7;
    cudaEventSynchronize(ev[last]);
    for (int i = 0; i < 7; ++i) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev[i], ev[i + 1]) == cudaSuccess) r->prof_ms[i] += ms;
    }
    if (r->prof_resolve[slot]) {
        float ms = 0.0f;
        if (cudaEventElapsedTime(&ms, ev[8], ev[9]) == cudaSuccess) r->prof_ms[7] += ms;
    }
    cudaGetLastError();
    r->prof_frames += 1;
    r->prof_pending[slot] = false;
}

void CUDART_CB exposure_callback(void* p) {
    swr_renderer* r = static_cast<swr_renderer*>(p);
    // A frame that overflowed its bins is re-rendered; it must not advance
    // the exposure state.
    if (*r->h_status & kStRetry) return;
    r->expo.update(r->h_lum, (size_t)r->tiles_x * r->tiles_y, r->pending_dt);
    *r->h_expo = r->expo.exposure;
}

swr_status enqueue_frame(swr_renderer* r, const swr_scene* scene, const swr_camera* cam, float dt,
                         cudaStream_t stream) {
    std::string err;
    if (r->expo_pending) {
        cudaEventSynchronize(r->expo_done);
        r->expo_pending = false;
    }
    std::vector<const SceneImpl*> scenes = {&scene->impl};
    std::vector<DView> views(1);
    DView& v = views[0];
    std::memset(&v, 0, sizeof(v));
    init_view(v, *cam, r->width, r->height, r->eng.sched_tile);
    v.scene = 0;
    v.rsqrt_mode = r->opts.rsqrt_mode;
    v.rgba8 = r->rgba8.as<uint32_t>();
    v.vis = r->vis.as<uint64_t>();
    v.tile_lum = r->tile_lum.as<float>();
    v.out_pitch = (uint32_t)r->width;
    v.rgba8_host = r->blit_target_dev;
    v.host_pitch = (uint32_t)r->blit_stride;
    r->frame_target = r->blit_target;
    r->frame_stride = r->blit_stride;
    const bool deferred = dt > 0.0f;
    r->eng.defer_resolve = deferred;
    if (deferred) {
        v.flags = kViewLinear;  // the engine provides the colour buffer
        v.exposure = 0.0f;
    } else {
        // update_auto_exposure with dt == 0 leaves ev unchanged: exposure = 2^ev.
        v.exposure = std::exp2(r->expo.ev);
        r->expo.exposure = v.exposure;
    }
    std::vector<const swr_camera*> cams = {cam};
    cudaEvent_t* ev = nullptr;
    int slot = -1;
    if (r->profiling) {
        slot = r->prof_next;
        r->prof_next = (r->prof_next + 1) % swr_renderer::kProfRing;
        prof_collect(r, slot);
        ev = r->prof_ev[slot];
        r->prof_pending[slot] = true;
        r->prof_resolve[slot] = deferred;
    }
    FrameArgs a{};
    swr_status st = r->eng.run(scenes, views, cams, stream, &a, err, ev);
    if (st != SWR_OK) return fail(st, err);
    if (deferred) {
        const size_t nt = (size_t)r->tiles_x * r->tiles_y;
        cudaMemcpyAsync(r->h_lum, r->tile_lum.p, nt * sizeof(float), cudaMemcpyDeviceToHost, stream);
        cudaMemcpyAsync(r->h_status, r->eng.counters.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream);
        r->pending_dt = dt;
        cudaLaunchHostFunc(stream, exposure_callback, r);
        a.exposure_dev = r->d_expo;
        if (ev) cudaEventRecord(ev[8], stream);
        launch_resolve(a, stream);
        r->eng.kernel_launches++;
        if (ev) cudaEventRecord(ev[9], stream);
        cudaEventRecord(r->expo_done, stream);
        r->expo_pending = true;
    }
    cudaMemcpyAsync(r->h_counters, r->eng.counters.p, sizeof(DCounters), cudaMemcpyDeviceToHost, stream);
    cudaEventRecord(r->status_ev, stream);
    r->status_pending = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
    r->last_args = a;
    return SWR_OK;
}

swr_status grow_for_overflow(swr_renderer* r, const DCounters& c) {
    std::string err;
    const swr_status st = r->eng.grow_for(c, err);
    r->opts.sched_tile = r->eng.sched_tile;
    if (st != SWR_OK) return fail(st, err);
    return SWR_OK;
}

// Before a new frame replaces the last one: if the last frame's counters are
// already back, grow what overflowed; never waits.
swr_status poll_frame(swr_renderer* r) {
    if (r->checked || !r->status_pending) return SWR_OK;
    const cudaError_t e = cudaEventQuery(r->status_ev);
    if (e == cudaErrorNotReady) {
        cudaGetLastError();
        return SWR_OK;
    }
    if (e != cudaSuccess) return cuda_fail(e, "frame execution");
    r->status_pending = false;
    const DCounters c = *r->h_counters;
    r->eng.last = c;
    if (c.status & kStRetry) return grow_for_overflow(r, c);
    return SWR_OK;
}

swr_status check_frame(swr_renderer* r) {
    if (r->checked) return SWR_OK;
    for (int attempt = 0; attempt < 6; ++attempt) {
        cudaError_t e = cudaStreamSynchronize(r->last_stream);
        if (e != cudaSuccess) return cuda_fail(e, "frame execution");
        DCounters c{};
        e = cudaMemcpy(&c, r->eng.counters.p, sizeof(c), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "counter readback");
        r->eng.last = c;
        if (!(c.status & kStRetry)) {
            r->checked = true;
            return SWR_OK;
        }
        swr_status gs = grow_for_overflow(r, c);
        if (gs != SWR_OK) return gs;
        // The overflowed frame's exposure step was skipped by the callback.
        swr_status st = enqueue_frame(r, r->last_scene, &r->last_cam, r->last_dt, r->last_stream);
        if (st != SWR_OK) return st;
    }
    return fail(SWR_OVERFLOW, "bin capacity could not be grown enough");
}

}  // namespace

swr_status swr_render_frame(swr_renderer* r, const swr_scene* scene, const swr_camera* cam, float dt, void* stream) {
    if (!r || !scene || !cam) return fail(SWR_INVALID_ARG, "null argument");
    if (!scene->impl.d_scene) return fail(SWR_INVALID_ARG, "scene was created host-only");
    if (!(dt >= 0.0f) && !(dt < 0.0f)) return fail(SWR_INVALID_ARG, "dt is NaN");
    // The previous frame is replaced, so it is not waited for: a frame is
    // checked (and re-rendered after an overflow) when its result is read.
    swr_status st = poll_frame(r);
    if (st != SWR_OK) return st;
    r->last_scene = scene;
    r->last_cam = *cam;
    r->last_dt = dt;
    r->last_stream = (cudaStream_t)stream;
    st = enqueue_frame(r, scene, cam, dt, (cudaStream_t)stream);
    if (st != SWR_OK) return st;
    r->checked = false;
    r->have_frame = true;
    return SWR_OK;
}

swr_status swr_renderer_sync(swr_renderer* r) {
    if (!r) return fail(SWR_INVALID_ARG, "null argument");
    return check_frame(r);
}

swr_status swr_blit(swr_renderer* r, uint32_t* pixels, size_t row_stride, void* stream) {
    if (!r || !pixels) return fail(SWR_INVALID_ARG, "null argument");
    if (!r->have_frame) return fail(SWR_INVALID_ARG, "no frame rendered");
    swr_status st = check_frame(r);
    if (st != SWR_OK) return st;
    if (row_stride == 0) row_stride = (size_t)r->width;
    if (row_stride < (size_t)r->width) return fail(SWR_INVALID_ARG, "row_stride smaller than width");
    if (pixels == r->frame_target && row_stride == r->frame_stride) {
        // The shading pass already wrote this frame into `pixels`.
        const cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
        if (e != cudaSuccess) return cuda_fail(e, "blit wait");
        return SWR_OK;
    }
    const size_t rows = (size_t)(r->height & ~1);
    cudaError_t e = cudaMemcpy2DAsync(pixels, row_stride * sizeof(uint32_t), r->rgba8.p, (size_t)r->width * 4,
                                      (size_t)r->width * 4, rows, cudaMemcpyDefault, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "blit copy");
    return SWR_OK;
}

swr_status swr_renderer_set_blit_target(swr_renderer* r, uint32_t* pixels, size_t row_stride) {
    if (!r) return fail(SWR_INVALID_ARG, "null argument");
    if (!pixels) {
        r->blit_target = r->blit_target_dev = nullptr;
        r->blit_stride = 0;
        return SWR_OK;
    }
    if (row_stride == 0) row_stride = (size_t)r->width;
    if (row_stride < (size_t)r->width || row_stride > 0xFFFFFFFFull)
        return fail(SWR_INVALID_ARG, "row_stride smaller than width or above 2^32-1");
    // The device must be able to store to the memory: pinned or registered
    // host memory (through its device address), device or managed memory,
    // or pageable host memory where the device reads the host page tables.
    cudaPointerAttributes at{};
    cudaError_t e = cudaPointerGetAttributes(&at, pixels);
    cudaGetLastError();
    uint32_t* dev = nullptr;
    if (e == cudaSuccess && (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeDevice ||
                             at.type == cudaMemoryTypeManaged)) {
        dev = static_cast<uint32_t*>(at.devicePointer);
    } else if (e == cudaSuccess && at.type == cudaMemoryTypeUnregistered) {
        int d = 0, pageable = 0;
        cudaGetDevice(&d);
        if (cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, d) == cudaSuccess && pageable)
            dev = pixels;
    }
    if (!dev)
        return fail(SWR_INVALID_ARG,
                    "blit target is not device-writable (use pinned or registered host memory)");
    r->blit_target = pixels;
    r->blit_target_dev = dev;
    r->blit_stride = row_stride;
    return SWR_OK;
}

swr_status swr_read_visbuffer(swr_renderer* r, uint64_t* ids, void* stream) {
    if (!r || !ids) return fail(SWR_INVALID_ARG, "null argument");
    if (!r->have_frame) return fail(SWR_INVALID_ARG, "no frame rendered");
    swr_status st = check_frame(r);
    if (st != SWR_OK) return st;
    cudaError_t e = cudaMemcpyAsync(ids, r->vis.p, (size_t)r->width * r->height * sizeof(uint64_t), cudaMemcpyDefault,
                                    (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "visbuffer copy");
    return SWR_OK;
}

swr_status swr_renderer_device_outputs(swr_renderer* r, const uint32_t** rgba8, const uint64_t** vis) {
    if (!r) return fail(SWR_INVALID_ARG, "null argument");
    if (rgba8) *rgba8 = r->rgba8.as<uint32_t>();
    if (vis) *vis = r->vis.as<uint64_t>();
    return SWR_OK;
}

swr_status swr_renderer_get_exposure(const swr_renderer* r, float* e) {
    if (!r || !e) return fail(SWR_INVALID_ARG, "null argument");
    if (r->expo_pending) cudaEventSynchronize(r->expo_done);
    *e = r->expo.exposure;
    return SWR_OK;
}

swr_status swr_renderer_set_exposure(swr_renderer* r, float e) {
    if (!r || !(e > 0.0f) || !std::isfinite(e)) return fail(SWR_INVALID_ARG, "exposure must be positive");
    if (r->expo_pending) {
        cudaEventSynchronize(r->expo_done);
        r->expo_pending = false;
    }
    r->expo.exposure = e;
    r->expo.ev = std::log2(e);
    return SWR_OK;
}

swr_status swr_renderer_get_stats(swr_renderer* r, swr_frame_stats* o) {
    if (!r || !o) return fail(SWR_INVALID_ARG, "null argument");
    swr_status st = check_frame(r);
    if (st != SWR_OK) return st;
    std::memset(o, 0, sizeof(*o));
    const DCounters& c = r->eng.last;
    o->triangles_in = c.draw_tris;
    o->triangles_clipped = c.clip_queue;
    o->setup_triangles = c.setup_tris;
    o->bin_pairs = c.pairs;
    o->bin_capacity = r->eng.bin_cap;
    o->tiles = r->tiles_x * r->tiles_y;
    o->overflow_retries = r->eng.retries;
    o->exposure = r->expo.exposure;
    o->sched_tile = r->opts.sched_tile;
    o->staged_bytes = r->eng.lay.staged;
    o->culled_pairs = c.culled;
    o->kernel_launches = r->eng.kernel_launches;
    o->triangles_clip_path = c.clip_path;
    return SWR_OK;
}

swr_status swr_renderer_set_profiling(swr_renderer* r, int32_t enable) {
    if (!r) return fail(SWR_INVALID_ARG, "null argument");
    if (enable && !r->prof_ev[0][0]) {
        for (auto& set : r->prof_ev)
            for (cudaEvent_t& e : set)
                if (cudaEventCreate(&e) != cudaSuccess) return cuda_fail(cudaGetLastError(), "profiling events");
    }
    for (int i = 0; i < swr_renderer::kProfRing; ++i) r->prof_pending[i] = false;
    for (double& m : r->prof_ms) m = 0.0;
    r->prof_frames = 0;
    r->profiling = enable != 0;
    return SWR_OK;
}

swr_status swr_renderer_get_profile(swr_renderer* r, float* stage_ms, int32_t n, uint32_t* frames) {
    if (!r || !stage_ms) return fail(SWR_INVALID_ARG, "null argument");
    for (int i = 0; i < swr_renderer::kProfRing; ++i) prof_collect(r, i);
    for (int i = 0; i < n && i < SWR_STAGES; ++i)
        stage_ms[i] = r->prof_frames ? (float)(r->prof_ms[i] / r->prof_frames) : 0.0f;
    if (frames) *frames = r->prof_frames;
    return SWR_OK;
}

swr_status swr_renderer_get_tile_luminance(swr_renderer* r, float* out, uint32_t count) {
    if (!r || !out) return fail(SWR_INVALID_ARG, "null argument");
    swr_status st = check_frame(r);
    if (st != SWR_OK) return st;
    const uint32_t n = r->tiles_x * r->tiles_y;
    if (count < n) return fail(SWR_INVALID_ARG, "count smaller than tile count");
    cudaError_t e = cudaMemcpy(out, r->tile_lum.p, n * sizeof(float), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "tile luminance copy");
    return SWR_OK;
}


swr_status swr_selftest_srgb_pow(const float* in, float* out, uint64_t n, uint32_t mode) {
    if ((!in || !out) && n > 0) return fail(SWR_INVALID_ARG, "null argument");
    if (mode > 1) return fail(SWR_INVALID_ARG, "bad mode");
    std::string err;
    const swr_status st = srgb_pow_selftest(in, out, n, mode, err);
    return st == SWR_OK ? SWR_OK : fail(st, err);
}

swr_status swr_selftest_rsqrt(const float* in, float* out, uint64_t n, uint32_t rsqrt_mode) {
    if ((!in || !out) && n > 0) return fail(SWR_INVALID_ARG, "null argument");
    if (rsqrt_mode > SWR_RSQRT_AARCH64) return fail(SWR_INVALID_ARG, "bad rsqrt_mode");
    if (n == 0) return SWR_OK;
    uint8_t tab[512];
    build_rsqrt_table(tab);
    void* d = nullptr;
    const size_t bytes = (size_t)n * sizeof(float);
    cudaError_t e = cudaMalloc(&d, 2 * bytes + 512);
    if (e != cudaSuccess) return cuda_fail(e, "self-test allocation");
    float* din = static_cast<float*>(d);
    float* dout = din + n;
    uint8_t* dtab = reinterpret_cast<uint8_t*>(dout + n);
    e = cudaMemcpy(din, in, bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(dtab, tab, 512, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_rsqrt_selftest(din, dout, n, rsqrt_mode, dtab);
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess) return cuda_fail(e, "self-test");
    return SWR_OK;
}

swr_status swr_selftest_depth_floor(const int32_t* p, const float* zow, const float* oow, int32_t xe, int32_t ye,
                                    float* zlo) {
    if (!p || !zow || !oow || !zlo) return fail(SWR_INVALID_ARG, "null argument");
    float z = 0.0f;
    *zlo = depth_floor_host(p, zow, oow, xe, ye, z) ? z : -std::numeric_limits<float>::infinity();
    return SWR_OK;
}

}  // extern "C"
