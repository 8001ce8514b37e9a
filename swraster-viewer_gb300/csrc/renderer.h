// Host runtime of the per-frame renderer: draw-list construction, device
// buffer management, exposure state (Renderer, src/renderer.rs:144-198).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/swr.h"
#include "internal.h"
#include "scene.h"

namespace swr {

// Grow-only device buffer.
struct DBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t want = n + n / 4;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
    }
    template <typename T>
    T* as() const { return static_cast<T*>(p); }
};

// Pinned host staging buffer.
struct HBuf {
    void* p = nullptr;
    size_t bytes = 0;
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        size_t want = n + n / 4 + 256;
        cudaError_t e = cudaHostAlloc(&p, want, cudaHostAllocDefault);
        if (e == cudaSuccess) bytes = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
    }
};

// Table region layout (host staging and device copy use the same offsets).
struct TableLayout {
    // Staged from the host each frame: [0, staged). Device-written after it:
    // per node slot counts and offsets, draws, chunks.
    size_t o_dyn = 0, o_scenes = 0, o_views = 0, o_order = 0, staged = 0;
    size_t o_slots = 0, o_draws = 0, o_chunks = 0, total = 0;
};
TableLayout table_layout(uint32_t scene_cap, uint32_t view_cap, uint32_t order_cap, uint32_t draw_cap,
                         uint32_t chunk_cap);

// Reusable frame engine: everything a batch of views needs on the device.
// prepare() builds the per-frame tables on the host and grows capacities;
// launch() uploads the tables with one copy and runs the frame, either as
// direct launches or by replaying a CUDA graph captured for the current
// capacities (every per-frame count is read from the device table header).
struct FrameEngine {
    int num_sms = 148;
    uint32_t sched_tile = 64;
    uint64_t bin_cap = 0, extra_cap = 0;
    uint32_t scene_cap = 0, view_cap = 0, order_cap = 0, draw_cap = 0, chunk_cap = 0, tri_cap = 0, stile_cap = 0,
             quad_cap = 0;
    uint32_t pixel_cap = 0;
    uint64_t key_cap = 0;
    uint32_t raster_grid = 0, shade_grid = 0, grid_tile = 0;
    uint32_t raster_cta_cap = 0, grid_cap = 0;  // raster CTAs per SM (0: as many as fit; batch autotuner's choice)
    bool fuse32 = false;        // 32-px tiles shade inside the raster kernel (batch autotuner's choice)
    bool grid_fused32 = false;
    DBuf tables, tri_state, rec_r, rec_s, fan_base, clip_queue;
    DBuf tile_count, tile_offset, tile_cursor, bins, keys, counters, rsqrt_tab;
    DBuf color;                // linear colour of views that need it (padded tile grids)
    bool defer_resolve = false;// the caller resolves (renderer frames with dt > 0)
    static constexpr int kStageRing = 4;
    static constexpr uint64_t kTriCapFromBound = 8u << 20;  // record slots sized from scene bounds, at most
    HBuf h_stage[kStageRing];  // pinned staging of the per-frame tables, one per frame in flight
    std::vector<uint32_t> h_order;  // per-frame node order of every view (capacity kept)
    TableLayout lay;
    cudaEvent_t stage_done[kStageRing] = {};
    bool stage_pending[kStageRing] = {};
    int stage_slot = 0;
    uint32_t retries = 0;
    uint64_t kernel_launches = 0;  // kernels enqueued (graph replays count the graph's kernels)
    uint32_t graph_kernels = 0;    // kernels in the captured graph
    DCounters last{};
    DFrameDyn dyn{};
    FrameArgs args{};
    // Graph replay.
    bool use_graph = false;
    cudaGraphExec_t graph_exec = nullptr;
    FrameArgs graph_args{};
    cudaStream_t graph_stream = nullptr;
    cudaStream_t capture_stream = nullptr;  // legacy default streams cannot be captured

    swr_status init(std::string& err);
    // Grows what a frame's counters report as overflowed (bins, clip slots)
    // or, when a tile held too many translucent packets, halves the
    // scheduling tile; SWR_OVERFLOW when nothing is left to grow.
    swr_status grow_for(const DCounters& c, std::string& err);
    void release();
    swr_status prepare(const std::vector<const SceneImpl*>& scenes, std::vector<DView>& views,
                       const std::vector<const swr_camera*>& cams, std::string& err);
    swr_status launch(cudaStream_t stream, cudaEvent_t* ev, std::string& err);
    // prepare + launch (the plain renderer's path).
    swr_status run(const std::vector<const SceneImpl*>& scenes, std::vector<DView>& views,
                   const std::vector<const swr_camera*>& cams, cudaStream_t stream, FrameArgs* out_args,
                   std::string& err, cudaEvent_t* ev = nullptr);
};

// compute_nodes_by_distance (src/renderer.rs:201-210): appends the scene's
// node indices, nearest first, to `out`.
void sort_nodes_by_distance(const SceneImpl& s, const swr_camera& cam, std::vector<uint32_t>& out);

// Fill the view-geometry fields of a DView (tiles, pitches, camera).
void init_view(DView& v, const swr_camera& cam, int32_t width, int32_t height, uint32_t sched_tile);

// Scheduling tile for views of the given sizes when the caller leaves it to
// the library: the largest of 64, 32, 16 that still gives the raster kernel
// at least 8 tiles per SM (16 when none does).
uint32_t auto_sched_tile(const int32_t* widths, const int32_t* heights, int32_t n, int num_sms);

// Sets the calling thread's swr_last_error() message.
void set_last_error(const char* msg);

// update_auto_exposure (src/renderer.rs:258-290).
struct ExposureState {
    float exposure = 2.0f;
    float target = 2.0f;
    float ev = 1.0f;  // log2(2.0)
    void update(const float* tile_lum, size_t n, float dt);
};

}  // namespace swr

struct swr_renderer {
    int32_t width = 0, height = 0;
    swr_renderer_opts opts{};
    swr::FrameEngine eng;
    swr::DBuf rgba8, vis, tile_lum;
    // Host memory the shading pass also writes RGBA8 into
    // (swr_renderer_set_blit_target): the caller's pointer, the address the
    // device uses for it, its row pitch in pixels; and the target the last
    // enqueued frame was rendered into.
    uint32_t* blit_target = nullptr;
    uint32_t* blit_target_dev = nullptr;
    size_t blit_stride = 0;
    uint32_t* frame_target = nullptr;
    size_t frame_stride = 0;
    swr::ExposureState expo;
    // Mapped pinned memory for the dt > 0 exposure step.
    float* h_lum = nullptr;
    uint32_t* h_status = nullptr;
    float* h_expo = nullptr;
    float* d_expo = nullptr;
    cudaEvent_t expo_done = nullptr;
    bool expo_pending = false;
    float pending_dt = 0.0f;
    // Last frame, kept for overflow re-runs.
    const swr_scene* last_scene = nullptr;
    swr_camera last_cam{};
    float last_dt = 0.0f;
    cudaStream_t last_stream = nullptr;
    bool have_frame = false;
    bool checked = true;
    // Counters of the last frame, copied back asynchronously so the next
    // frame can adapt capacities without waiting for this one.
    swr::DCounters* h_counters = nullptr;
    cudaEvent_t status_ev = nullptr;
    bool status_pending = false;
    swr::FrameArgs last_args{};
    uint32_t tiles_x = 0, tiles_y = 0;
    // Stage profiling: a ring of event sets, one per in-flight frame.
    static constexpr int kProfRing = 64;
    bool profiling = false;
    cudaEvent_t prof_ev[kProfRing][10] = {};
    bool prof_pending[kProfRing] = {};
    bool prof_resolve[kProfRing] = {};
    int prof_next = 0;
    double prof_ms[SWR_STAGES] = {};
    uint32_t prof_frames = 0;
};
