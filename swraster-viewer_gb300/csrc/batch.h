// Batched form internals (shared by the batch C ABI and the server).
#pragma once

#include <map>
#include <string>
#include <vector>

#include "renderer.h"

namespace swr {

// Autotuner class of a batch: log2 of total pixels, log2 of triangles,
// log2 of the view count.
uint32_t batch_class(const swr_view_desc* v, int32_t n);

struct OwnedOutput {
    DBuf rgba8, vis;
};

struct BatchImpl {
    swr_batch_opts opts{};
    FrameEngine eng;
    std::vector<OwnedOutput> owned;
    DBuf tile_lum;
    std::vector<swr_view_desc> saved;
    std::vector<swr_camera> saved_cams;
    // class -> scheduling tile | 0x100 when 32-px tiles shade fused | raster CTAs per SM << 12 (0: all that fit)
    std::map<uint32_t, uint32_t> tuned;
    std::map<uint32_t, uint64_t> tuned_bins;  // class -> (triangle, tile) pair capacity to start a batch with
    bool opt_fuse32 = false;             // with opts.sched_tile == 32: shade fused (autotuner trials)
    uint32_t opt_raster_cap = 0;         // with opts.sched_tile set: raster CTAs per SM (autotuner trials)
    bool base_fuse32 = false;            // SWR_BATCH_FUSED_SHADE
    cudaEvent_t ev_start = nullptr, ev_end = nullptr;
    cudaStream_t last_stream = nullptr;
    bool pending = false;

    swr_status render(const swr_view_desc* vd, int32_t n, cudaStream_t stream, std::string& err);
    swr_status enqueue(const swr_view_desc* vd, int32_t n, cudaStream_t stream, std::string& err);
    swr_status sync(std::string& err);
    uint32_t tuned_tile(const swr_view_desc* vd, int32_t n) const;
};

}  // namespace swr

struct swr_batch {
    swr::BatchImpl impl;
};
