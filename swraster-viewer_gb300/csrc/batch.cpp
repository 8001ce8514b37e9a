// Batched form: many views (any mix of resident scenes and resolutions) per
// launch sequence, optional CUDA-graph replay, and an autotuner that picks
// the raster scheduling tile per batch class.
#include "batch.h"

#include <algorithm>
#include <cmath>
#include <cstring>

using namespace swr;

namespace swr {

namespace {
inline uint32_t log2u(uint64_t v) {
    uint32_t r = 0;
    while (v > 1) {
        v >>= 1;
        ++r;
    }
    return r;
}
}  // namespace

uint32_t batch_class(const swr_view_desc* v, int32_t n) {
    uint64_t px = 0, tris = 0;
    for (int32_t i = 0; i < n; ++i) {
        px += (uint64_t)v[i].width * (uint64_t)v[i].height;
        tris += v[i].scene->impl.tri_total;
    }
    return (log2u(px) << 16) | (log2u(tris) << 8) | std::min<uint32_t>(log2u((uint64_t)n), 255u);
}

swr_status BatchImpl::enqueue(const swr_view_desc* vd, int32_t n, cudaStream_t stream, std::string& err) {
    // Unique scenes of this batch.
    std::vector<const SceneImpl*> scenes;
    std::vector<DView> views((size_t)n);
    std::vector<const swr_camera*> cams((size_t)n);
    size_t tiles_total = 0;
    for (int32_t i = 0; i < n; ++i) {
        const SceneImpl* sc = &vd[i].scene->impl;
        uint32_t si = 0;
        while (si < scenes.size() && scenes[si] != sc) ++si;
        if (si == scenes.size()) scenes.push_back(sc);
        DView& v = views[i];
        std::memset(&v, 0, sizeof(v));
        init_view(v, *vd[i].camera, vd[i].width, vd[i].height, eng.sched_tile);
        v.scene = si;
        v.rsqrt_mode = vd[i].rsqrt_mode;
        v.exposure = vd[i].exposure;
        v.out_pitch = (uint32_t)vd[i].width;
        cams[i] = vd[i].camera;
        tiles_total += (size_t)v.tiles_x * v.tiles_y;
    }
    // Batch-owned outputs and per-view tile luminance.
    if (owned.size() < (size_t)n) owned.resize((size_t)n);
    cudaError_t e = tile_lum.ensure(std::max<size_t>(1, tiles_total) * sizeof(float));
    size_t tl = 0;
    for (int32_t i = 0; i < n && e == cudaSuccess; ++i) {
        DView& v = views[i];
        const size_t px = (size_t)vd[i].width * vd[i].height;
        if (vd[i].rgba8) {
            v.rgba8 = vd[i].rgba8;
        } else {
            e = owned[i].rgba8.ensure(px * sizeof(uint32_t));
            v.rgba8 = owned[i].rgba8.as<uint32_t>();
        }
        if (e == cudaSuccess) {
            if (vd[i].vis) {
                v.vis = vd[i].vis;
            } else {
                e = owned[i].vis.ensure(px * sizeof(uint64_t));
                v.vis = owned[i].vis.as<uint64_t>();
            }
        }
        v.tile_lum = tile_lum.as<float>() + tl;
        tl += (size_t)v.tiles_x * v.tiles_y;
    }
    if (e != cudaSuccess) {
        err = std::string("output allocation failed: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return SWR_NO_MEMORY;
    }
    swr_status st = eng.prepare(scenes, views, cams, err);
    if (st != SWR_OK) return st;
    cudaEventRecord(ev_start, stream);
    st = eng.launch(stream, nullptr, err);
    cudaEventRecord(ev_end, stream);
    last_stream = stream;
    return st;
}

swr_status BatchImpl::sync(std::string& err) {
    if (!pending) return SWR_OK;
    for (int attempt = 0; attempt < 6; ++attempt) {
        cudaError_t e = cudaStreamSynchronize(last_stream);
        if (e != cudaSuccess) {
            err = std::string("batch execution: ") + cudaGetErrorString(e);
            cudaGetLastError();
            return SWR_CUDA_ERROR;
        }
        DCounters c{};
        e = cudaMemcpy(&c, eng.counters.p, sizeof(c), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            err = "counter readback failed";
            return SWR_CUDA_ERROR;
        }
        eng.last = c;
        if (!(c.status & kStRetry)) {
            pending = false;
            return SWR_OK;
        }
        swr_status gs = eng.grow_for(c, err);
        if (gs != SWR_OK) {
            pending = false;
            return gs;
        }
        std::vector<swr_view_desc> vd = saved;
        for (size_t i = 0; i < vd.size(); ++i) vd[i].camera = &saved_cams[i];
        swr_status st = enqueue(vd.data(), (int32_t)vd.size(), last_stream, err);
        if (st != SWR_OK) return st;
    }
    err = "bin capacity could not be grown enough";
    return SWR_OVERFLOW;
}

swr_status BatchImpl::render(const swr_view_desc* vd, int32_t n, cudaStream_t stream, std::string& err) {
    swr_status st = sync(err);
    if (st != SWR_OK) return st;
    // Tuned choices carry "32-px tiles shade inside the raster kernel" in bit 8
    // and the raster CTAs per SM in bits 12-15.
    const uint32_t cap = std::min<uint32_t>(opt_raster_cap ? opt_raster_cap : opts.raster_ctas_per_sm, 15u);
    const uint32_t want = opts.sched_tile ? opts.sched_tile | (opt_fuse32 ? 0x100u : 0u) | (cap << 12)
                                          : tuned_tile(vd, n);
    eng.sched_tile = want & 0xFFu;
    eng.fuse32 = (want & 0x100u) != 0u;
    eng.raster_cta_cap = (want >> 12) & 0xFu;
    if (!opts.sched_tile) {
        // A tuned class starts with the bin capacity it needed, so its first
        // batch is not rendered twice after a bin overflow.
        auto it = tuned_bins.find(batch_class(vd, n));
        if (it != tuned_bins.end() && eng.bin_cap < it->second) eng.bin_cap = it->second;
    }
    saved.assign(vd, vd + n);
    saved_cams.resize((size_t)n);
    for (int32_t i = 0; i < n; ++i) saved_cams[i] = *vd[i].camera;
    st = enqueue(vd, n, stream, err);
    if (st == SWR_OK) pending = true;
    return st;
}

uint32_t BatchImpl::tuned_tile(const swr_view_desc* vd, int32_t n) const {
    auto it = tuned.find(batch_class(vd, n));
    if (it != tuned.end()) return it->second;
    std::vector<int32_t> w((size_t)n), h((size_t)n);
    for (int32_t i = 0; i < n; ++i) {
        w[(size_t)i] = vd[i].width;
        h[(size_t)i] = vd[i].height;
    }
    const uint32_t S = auto_sched_tile(w.data(), h.data(), n, eng.num_sms);
    // Several views: at most 32-px tiles, shaded inside the raster kernel.
    // Tiles of uneven views balance better over the persistent CTAs, and the
    // keys stay in shared memory (served mix, 5,000 req/s: 3,900 frames/s
    // with 64-px tiles, 4,960 with fused 32-px tiles).
    if (n > 1 && S >= 32u) return 32u | 0x100u;
    return S;
}

}  // namespace swr

namespace {
bool valid_views(const swr_view_desc* v, int32_t n, std::string& err) {
    if (!v || n <= 0) {
        err = "no views";
        return false;
    }
    for (int32_t i = 0; i < n; ++i) {
        if (!v[i].scene || !v[i].camera || !v[i].scene->impl.d_scene) {
            err = "view without a resident scene or camera";
            return false;
        }
        if (v[i].width <= 0 || v[i].height <= 0 || v[i].width > 32768 || v[i].height > 32768) {
            err = "view size out of range";
            return false;
        }
        if (v[i].rsqrt_mode > SWR_RSQRT_AARCH64 || !(v[i].exposure > 0.0f)) {
            err = "bad rsqrt_mode or exposure";
            return false;
        }
    }
    return true;
}
}  // namespace

extern "C" {

swr_status swr_batch_create(const swr_batch_opts* opts, swr_batch** out) {
    if (!out) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    *out = nullptr;
    swr_batch_opts o{};
    if (opts) o = *opts;
    if (o.sched_tile != 0 && o.sched_tile != 8 && o.sched_tile != 16 && o.sched_tile != 32 && o.sched_tile != 64) {
        set_last_error("sched_tile must be 0, 8, 16, 32 or 64");
        return SWR_INVALID_ARG;
    }
    swr_batch* b = new (std::nothrow) swr_batch();
    if (!b) {
        set_last_error("out of host memory");
        return SWR_NO_MEMORY;
    }
    b->impl.opts = o;
    b->impl.opt_fuse32 = b->impl.base_fuse32 = (o.flags & SWR_BATCH_FUSED_SHADE) != 0u;
    b->impl.eng.bin_cap = o.bin_capacity;
    b->impl.eng.use_graph = o.use_graph != 0;
    std::string err;
    swr_status st = b->impl.eng.init(err);
    if (st == SWR_OK && (cudaEventCreate(&b->impl.ev_start) != cudaSuccess ||
                         cudaEventCreate(&b->impl.ev_end) != cudaSuccess)) {
        st = SWR_CUDA_ERROR;
        err = "cudaEventCreate failed";
    }
    if (st != SWR_OK) {
        swr_batch_destroy(b);
        set_last_error(err.c_str());
        return st;
    }
    *out = b;
    return SWR_OK;
}

void swr_batch_destroy(swr_batch* b) {
    if (!b) return;
    cudaDeviceSynchronize();
    b->impl.eng.release();
    for (auto& o : b->impl.owned) {
        o.rgba8.release();
        o.vis.release();
    }
    b->impl.tile_lum.release();
    if (b->impl.ev_start) cudaEventDestroy(b->impl.ev_start);
    if (b->impl.ev_end) cudaEventDestroy(b->impl.ev_end);
    delete b;
}

swr_status swr_batch_render(swr_batch* b, const swr_view_desc* views, int32_t n, void* stream) {
    std::string err;
    if (!b) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    if (!valid_views(views, n, err)) {
        set_last_error(err.c_str());
        return SWR_INVALID_ARG;
    }
    swr_status st = b->impl.render(views, n, (cudaStream_t)stream, err);
    if (st != SWR_OK) set_last_error(err.c_str());
    return st;
}

swr_status swr_batch_sync(swr_batch* b) {
    if (!b) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    std::string err;
    swr_status st = b->impl.sync(err);
    if (st != SWR_OK) set_last_error(err.c_str());
    return st;
}

swr_status swr_batch_output(swr_batch* b, int32_t view, const uint32_t** rgba8, const uint64_t** vis) {
    if (!b || view < 0 || (size_t)view >= b->impl.saved.size()) {
        set_last_error("bad view index");
        return SWR_INVALID_ARG;
    }
    std::string err;
    swr_status st = b->impl.sync(err);
    if (st != SWR_OK) {
        set_last_error(err.c_str());
        return st;
    }
    const swr_view_desc& d = b->impl.saved[view];
    if (rgba8) *rgba8 = d.rgba8 ? d.rgba8 : b->impl.owned[view].rgba8.as<uint32_t>();
    if (vis) *vis = d.vis ? d.vis : b->impl.owned[view].vis.as<uint64_t>();
    return SWR_OK;
}

swr_status swr_copy_to_host(void* dst, const void* src, size_t bytes, void* stream) {
    if (!dst || !src) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, (cudaStream_t)stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        cudaGetLastError();
        return SWR_CUDA_ERROR;
    }
    return SWR_OK;
}

swr_status swr_batch_last_ms(swr_batch* b, float* ms) {
    if (!b || !ms) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    std::string err;
    swr_status st = b->impl.sync(err);
    if (st != SWR_OK) {
        set_last_error(err.c_str());
        return st;
    }
    if (cudaEventElapsedTime(ms, b->impl.ev_start, b->impl.ev_end) != cudaSuccess) {
        cudaGetLastError();
        *ms = 0.0f;
    }
    return SWR_OK;
}

swr_status swr_batch_autotune(swr_batch* b, const swr_view_desc* views, int32_t n, void* stream,
                              uint32_t* best_tile, float* best_ms) {
    std::string err;
    if (!b) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    if (!valid_views(views, n, err)) {
        set_last_error(err.c_str());
        return SWR_INVALID_ARG;
    }
    BatchImpl& B = b->impl;
    const swr_batch_opts keep = B.opts;
    uint32_t best = 64;
    uint64_t best_pairs = 0;
    float bms = 1e30f;
    // Scheduling tiles (32-px tiles also with the shading fused into the
    // raster kernel) by raster CTAs per SM (0: as many as the registers
    // allow); the bin capacity the best one needed is kept for the class.
    for (uint32_t code : {64u, 32u, 32u | 0x100u, 16u, 8u}) {
        for (uint32_t cap : {0u, 1u, 2u}) {
            B.opts.sched_tile = code & 0xFFu;
            B.opt_fuse32 = (code & 0x100u) != 0u;
            B.opt_raster_cap = cap;
            float total = 0.0f;
            uint64_t pairs = 0;
            for (int rep = 0; rep < 4; ++rep) {
                swr_status st = B.render(views, n, (cudaStream_t)stream, err);
                if (st == SWR_OK) st = B.sync(err);
                if (st != SWR_OK) {
                    B.opts = keep;
                    B.opt_fuse32 = B.base_fuse32;
                    B.opt_raster_cap = 0;
                    set_last_error(err.c_str());
                    return st;
                }
                float ms = 0.0f;
                cudaEventElapsedTime(&ms, B.ev_start, B.ev_end);
                if (rep > 0) total += ms;  // first run warms capacities and graphs
                pairs = B.eng.last.pairs;
            }
            if (total < bms) {
                bms = total;
                best = code | (cap << 12);
                best_pairs = pairs;
            }
        }
    }
    B.opts = keep;
    B.opt_fuse32 = B.base_fuse32;
    B.opt_raster_cap = 0;
    const uint32_t cls = batch_class(views, n);
    B.tuned[cls] = best;
    B.tuned_bins[cls] = best_pairs + best_pairs / 8 + 1024;
    if (best_tile) *best_tile = best & 0xFFu;
    if (best_ms) *best_ms = bms / 3.0f;
    return SWR_OK;
}

swr_status swr_batch_get_tuning(const swr_batch* b, const swr_view_desc* views, int32_t n, swr_batch_tuning* out) {
    std::string err;
    if (!b || !out) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    if (!valid_views(views, n, err)) {
        set_last_error(err.c_str());
        return SWR_INVALID_ARG;
    }
    const BatchImpl& B = b->impl;
    std::memset(out, 0, sizeof(*out));
    out->batch_class = batch_class(views, n);
    auto it = B.tuned.find(out->batch_class);
    out->tuned = it != B.tuned.end() ? 1u : 0u;
    const uint32_t code = B.tuned_tile(views, n);
    out->sched_tile = code & 0xFFu;
    out->fused_shade = (code & 0x100u) ? 1u : 0u;
    out->raster_ctas_per_sm = (code >> 12) & 0xFu;
    auto bt = B.tuned_bins.find(out->batch_class);
    out->bin_capacity = bt != B.tuned_bins.end() ? bt->second : 0u;
    return SWR_OK;
}

}  // extern "C"
