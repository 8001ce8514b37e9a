// Per-frame host runtime: node sort, view tables, device capacities,
// kernel launch, exposure. The draw list itself (MVPs, sphere/frustum
// classification, draws and chunks) is built on the device.
#include "renderer.h"

#include <algorithm>
#include <cmath>
#include <cstring>

namespace swr {

namespace {

// OrderedFloat ordering as an unsigned key: monotonic in the float value,
// every NaN above +inf and equal to the others, -0 and +0 equal (they
// compare equal, so a stable sort keeps them in index order).
inline uint32_t ordered_bits(float f) {
    if (f != f) return 0xFFFFFFFFu;
    if (f == 0.0f) f = 0.0f;
    uint32_t b;
    std::memcpy(&b, &f, sizeof(b));
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

}  // namespace

void sort_nodes_by_distance(const SceneImpl& s, const swr_camera& cam, std::vector<uint32_t>& out) {
    // compute_nodes_by_distance: stable sort by squared distance, as one sort
    // of (distance key, node index) words.
    const size_t nn = s.nodes.size();
    thread_local std::vector<uint64_t> order;
    order.resize(nn);
    const V3 cp = {cam.position[0], cam.position[1], cam.position[2]};
    for (size_t i = 0; i < nn; ++i) {
        const V3 d = sub(cp, {s.nodes[i].sphere[0], s.nodes[i].sphere[1], s.nodes[i].sphere[2]});
        order[i] = ((uint64_t)ordered_bits(dot3(d, d)) << 32) | (uint64_t)i;
    }
    std::sort(order.begin(), order.end());
    for (const uint64_t o : order) out.push_back((uint32_t)o);
}

void init_view(DView& v, const swr_camera& cam, int32_t width, int32_t height, uint32_t S) {
    std::memcpy(v.skybox_t, cam.skybox_transposed, sizeof(v.skybox_t));
    v.cam_pos[0] = cam.position[0];
    v.cam_pos[1] = cam.position[1];
    v.cam_pos[2] = cam.position[2];
    v.one_over_width = cam.one_over_width;
    v.one_over_height = cam.one_over_height;
    v.width_f = (float)width;
    v.height_f = (float)height;
    v.width = width;
    v.height = height;
    v.tiles_x = (width + kRefTile - 1) / kRefTile;
    v.tiles_y = (height + kRefTile - 1) / kRefTile;
    v.stiles_x = v.tiles_x * (kRefTile / (int32_t)S);
    v.stiles_y = v.tiles_y * (kRefTile / (int32_t)S);
    v.quad_pitch = (uint32_t)v.tiles_x * 32u;
    v.tiles_x_magic = v.tiles_x > 1 ? (uint32_t)((0x100000000ull + (uint64_t)v.tiles_x - 1u) / (uint64_t)v.tiles_x) : 0u;
    v.key_pitch = (uint64_t)v.tiles_x * kRefTile;
}

uint32_t auto_sched_tile(const int32_t* widths, const int32_t* heights, int32_t n, int num_sms) {
    const uint64_t want = 8ull * (uint64_t)(num_sms > 0 ? num_sms : 1);
    for (uint32_t S : {64u, 32u}) {
        uint64_t tiles = 0;
        for (int32_t i = 0; i < n; ++i)
            tiles += (uint64_t)((widths[i] + S - 1) / S) * (uint64_t)((heights[i] + S - 1) / S);
        if (tiles >= want) return S;
    }
    return 16u;
}

void ExposureState::update(const float* lum, size_t n, float dt) {
    if (n == 0) return;
    std::vector<float> s(n);
    for (size_t i = 0; i < n; ++i) s[i] = std::log2(std::fmax(lum[i], 1e-4f));
    // total_cmp order (no NaN can appear after max with 1e-4).
    std::sort(s.begin(), s.end());
    size_t trim = (size_t)std::floor((float)n * 0.10f);
    trim = std::min(trim, (n - 1) / 2);
    float sum = 0.0f;
    for (size_t i = trim; i < n - trim; ++i) sum += s[i];
    const float mean = sum / (float)(n - 2 * trim);
    // tonemap_inverse_scalar(0.45) (src/util.rs:43-47).
    const float y = std::fmin(std::fmax(0.45f, 0.0f), 1.0f);
    const float den = std::fmax(1.0f + 0.2f - y, 1e-6f);
    const float meter_key = std::fmax((y * 0.2f) / den, 1e-4f);
    const float target_ev = std::log2(meter_key) - mean;
    const float t = std::exp2(target_ev);
    target = std::fmin(std::fmax(t, 0.05f), 32.0f);
    const float tev = std::log2(target);
    const float tau = std::fmax(1.0f, 1e-4f);
    const float alpha = 1.0f - std::exp(-(std::fmax(dt, 0.0f) / tau));
    ev += (tev - ev) * alpha;
    exposure = std::exp2(ev);
}

TableLayout table_layout(uint32_t scene_cap, uint32_t view_cap, uint32_t order_cap, uint32_t draw_cap,
                         uint32_t chunk_cap) {
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    TableLayout L;
    L.o_dyn = 0;
    L.o_scenes = al(sizeof(DFrameDyn));
    L.o_views = L.o_scenes + al(sizeof(DScene) * scene_cap);
    L.o_order = L.o_views + al(sizeof(DView) * view_cap);
    L.staged = L.o_order + al(sizeof(uint32_t) * order_cap);
    L.o_slots = L.staged;
    L.o_draws = L.o_slots + al(sizeof(uint4) * ((order_cap + 255) / 256));
    L.o_chunks = L.o_draws + al(sizeof(DDraw) * draw_cap);
    L.total = L.o_chunks + al(sizeof(DChunk) * chunk_cap);
    return L;
}

swr_status FrameEngine::init(std::string& err) {
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && sms > 0) num_sms = sms;
    if (init_kernel_constants() != cudaSuccess) {
        err = "kernel constant upload failed";
        cudaGetLastError();
        return SWR_CUDA_ERROR;
    }
    if (rsqrt_tab.ensure(512) != cudaSuccess || counters.ensure(sizeof(DCounters)) != cudaSuccess) {
        err = "cudaMalloc failed";
        return SWR_NO_MEMORY;
    }
    if (cudaMemset(counters.p, 0, sizeof(DCounters)) != cudaSuccess) {
        err = "cudaMemset failed";
        return SWR_CUDA_ERROR;
    }
    uint8_t tab[512];
    build_rsqrt_table(tab);
    if (cudaMemcpy(rsqrt_tab.p, tab, 512, cudaMemcpyHostToDevice) != cudaSuccess) {
        err = "cudaMemcpy failed";
        return SWR_CUDA_ERROR;
    }
    for (cudaEvent_t& ev : stage_done)
        if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
            err = "cudaEventCreate failed";
            return SWR_CUDA_ERROR;
        }
    return SWR_OK;
}

void FrameEngine::release() {
    if (graph_exec) cudaGraphExecDestroy(graph_exec);
    graph_exec = nullptr;
    if (capture_stream) cudaStreamDestroy(capture_stream);
    capture_stream = nullptr;
    for (DBuf* b : {&tables, &tri_state, &rec_r, &rec_s, &fan_base, &clip_queue, &tile_count, &tile_offset,
                    &tile_cursor, &bins, &keys, &counters, &rsqrt_tab, &color})
        b->release();
    for (int i = 0; i < kStageRing; ++i) {
        h_stage[i].release();
        if (stage_done[i]) cudaEventDestroy(stage_done[i]);
        stage_done[i] = nullptr;
        stage_pending[i] = false;
    }
}

namespace {
inline uint32_t grow(uint32_t cur, uint64_t need) {
    if (need <= cur) return cur;
    const uint64_t g = need + need / 4 + 16;
    return (uint32_t)std::min<uint64_t>(g, 0xFFFFFFF0ull);
}
}  // namespace

swr_status FrameEngine::prepare(const std::vector<const SceneImpl*>& scenes, std::vector<DView>& vws,
                                const std::vector<const swr_camera*>& cams, std::string& err) {
    // Per view: the node order (the host's part of the draw list) and the
    // camera the device builds the draws with; capacities from the scenes'
    // bounds (every primitive in the frustum), since the draw list itself is
    // only known on the device.
    h_order.clear();
    uint64_t tri_bound = 0, draw_bound = 0, chunk_bound = 0;
    uint32_t stile_cursor = 0, quad_cursor = 0, max_px = 0;
    uint64_t key_cursor = 0, color_floats = 0;
    bool any_translucent = false;
    for (size_t i = 0; i < vws.size(); ++i) {
        DView& v = vws[i];
        const SceneImpl& sc = *scenes[v.scene];
        const swr_camera& cam = *cams[i];
        std::memcpy(v.cam_view, cam.view, sizeof(v.cam_view));
        std::memcpy(v.cam_view_project, cam.view_project, sizeof(v.cam_view_project));
        std::memcpy(v.cam_planes, cam.view_clip_planes, sizeof(v.cam_planes));
        v.order_base = (uint32_t)h_order.size();
        v.n_order = (uint32_t)sc.nodes.size();
        sort_nodes_by_distance(sc, cam, h_order);
        tri_bound += sc.tri_total;
        draw_bound += sc.max_draws;
        chunk_bound += sc.max_chunks;
        // kViewTranslucent is set on the device when a translucent draw is
        // emitted; a view whose scene has translucent primitives gets the
        // colour buffer the translucent pass blends into.
        v.flags &= kViewLinear;
        any_translucent |= sc.any_translucent;
        // Linear colour over the padded tile grid (engine-owned), offset kept
        // in the pointer field until the buffer exists.
        v.color = nullptr;
        if (v.flags || sc.any_translucent) {
            v.color = reinterpret_cast<float*>((uintptr_t)(color_floats + 1));
            color_floats += v.key_pitch * (uint64_t)v.tiles_y * kRefTile * 3u;
        }
        v.stile_base = stile_cursor;
        stile_cursor += (uint32_t)(v.stiles_x * v.stiles_y);
        v.quad_base = quad_cursor;
        quad_cursor += v.quad_pitch * (uint32_t)v.tiles_y * 32u;
        v.key_offset = key_cursor;
        key_cursor += v.key_pitch * (uint64_t)v.tiles_y * kRefTile;
        max_px = std::max<uint32_t>(max_px, (uint32_t)v.width * (uint32_t)(v.height & ~1));
    }
    if (tri_bound > 0xFFFFFFF0ull || chunk_bound > 0xFFFFFFF0ull || h_order.size() > 0xFFFFFFF0ull) {
        err = "frame above 2^32 triangles, chunks or nodes";
        return SWR_INVALID_ARG;
    }
    // Capacities (grow-only, with headroom so small changes keep a captured graph valid).
    scene_cap = grow(scene_cap, scenes.size());
    view_cap = grow(view_cap, vws.size());
    order_cap = grow(order_cap, std::max<size_t>(1, h_order.size()));
    // Draws and chunks are small: their bounds are allocated. Record slots
    // (256 B per triangle) follow the bound up to kTriCapFromBound; past it
    // they grow to what frames actually draw (a frame that finds more
    // triangles than slots is rendered again with grown buffers), so
    // batches of large scenes hold what is visible, not every triangle.
    draw_cap = grow(draw_cap, std::max<uint64_t>(1, draw_bound));
    chunk_cap = grow(chunk_cap, std::max<uint64_t>(1, chunk_bound));
    tri_cap = grow(tri_cap, std::max<uint64_t>(1, std::min<uint64_t>(tri_bound, kTriCapFromBound)));
    // Bins: opaque per scheduling tile, then (frames with translucent draws)
    // translucent per scheduling tile.
    stile_cap = grow(stile_cap, 2ull * stile_cursor + 1);
    quad_cap = grow(quad_cap, quad_cursor);
    pixel_cap = grow(pixel_cap, max_px);
    if (key_cursor > key_cap) key_cap = key_cursor + key_cursor / 4;
    // Clip fan slots: a sixteenth of the triangles to start with (clipped
    // triangles are a few percent of a frame); a frame that needs more is
    // rendered again with them doubled.
    if (extra_cap < std::max<uint64_t>(4096, tri_cap / 16)) extra_cap = std::max<uint64_t>(4096, tri_cap / 16);
    if (bin_cap < std::max<uint64_t>(65536, (uint64_t)tri_cap * 2 + stile_cap * 4ull))
        bin_cap = std::max<uint64_t>(65536, (uint64_t)tri_cap * 2 + stile_cap * 4ull);
    lay = table_layout(scene_cap, view_cap, order_cap, draw_cap, chunk_cap);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (x != cudaSuccess && e == cudaSuccess) e = x;
    };
    const size_t slots = (size_t)tri_cap + extra_cap;
    chk(tables.ensure(lay.total));
    chk(tri_state.ensure(tri_cap));
    chk(rec_r.ensure(slots * sizeof(RecRaster)));
    chk(rec_s.ensure(slots * sizeof(RecShade)));
    chk(fan_base.ensure((size_t)tri_cap * sizeof(uint32_t)));
    chk(clip_queue.ensure((size_t)tri_cap * sizeof(uint2)));
    chk(tile_count.ensure((size_t)(stile_cap + 1) * sizeof(uint32_t)));
    chk(tile_offset.ensure((size_t)(stile_cap + 1) * sizeof(uint32_t)));
    chk(tile_cursor.ensure((size_t)(stile_cap + 1) * sizeof(uint32_t)));
    chk(bins.ensure(bin_cap * sizeof(uint32_t)));
    chk(keys.ensure(std::max<uint64_t>(1, key_cap) * sizeof(unsigned long long)));
    if (color_floats > 0) chk(color.ensure(color_floats * sizeof(float)));
    if (e != cudaSuccess) {
        err = std::string("device allocation failed: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SWR_NO_MEMORY : SWR_CUDA_ERROR;
    }
    // The staging buffer of this frame was last read by the copy of the
    // frame kStageRing frames back.
    if (stage_pending[stage_slot]) {
        cudaEventSynchronize(stage_done[stage_slot]);
        stage_pending[stage_slot] = false;
    }
    HBuf& h_stage_cur = h_stage[stage_slot];
    if (h_stage_cur.ensure(lay.staged) != cudaSuccess) {
        err = "pinned allocation failed";
        return SWR_NO_MEMORY;
    }
    dyn = DFrameDyn{};
    dyn.n_views = (uint32_t)vws.size();
    dyn.n_chunks = 0;    // written by the draw-list build
    dyn.tri_total = 0;
    dyn.n_stiles = stile_cursor;
    dyn.total_quads = quad_cursor;
    dyn.max_view_pixels = max_px;
    dyn.n_bins = any_translucent ? 2u * stile_cursor : stile_cursor;
    dyn.n_slots = (uint32_t)h_order.size();
    for (DView& v : vws)
        if (v.color) v.color = color.as<float>() + ((uintptr_t)v.color - 1u);
    uint8_t* hs = static_cast<uint8_t*>(h_stage_cur.p);
    std::memcpy(hs + lay.o_dyn, &dyn, sizeof(dyn));
    for (size_t i = 0; i < scenes.size(); ++i)
        std::memcpy(hs + lay.o_scenes + i * sizeof(DScene), &scenes[i]->dscene, sizeof(DScene));
    std::memcpy(hs + lay.o_views, vws.data(), vws.size() * sizeof(DView));
    if (!h_order.empty()) std::memcpy(hs + lay.o_order, h_order.data(), h_order.size() * sizeof(uint32_t));
    const bool fused32 = fuse32 && sched_tile == 32;
    if (grid_tile != sched_tile || grid_fused32 != fused32 || grid_cap != raster_cta_cap) {
        frame_grids(num_sms, sched_tile, fused32, &raster_grid, &shade_grid);
        if (raster_cta_cap) raster_grid = std::min<uint32_t>(raster_grid, (uint32_t)num_sms * raster_cta_cap);
        grid_tile = sched_tile;
        grid_fused32 = fused32;
        grid_cap = raster_cta_cap;
    }
    uint8_t* tb = static_cast<uint8_t*>(tables.p);
    FrameArgs a{};
    a.dyn = reinterpret_cast<DFrameDyn*>(tb + lay.o_dyn);
    a.scenes = reinterpret_cast<const DScene*>(tb + lay.o_scenes);
    a.views = reinterpret_cast<DView*>(tb + lay.o_views);
    a.draws = reinterpret_cast<DDraw*>(tb + lay.o_draws);
    a.chunks = reinterpret_cast<DChunk*>(tb + lay.o_chunks);
    a.node_order = reinterpret_cast<const uint32_t*>(tb + lay.o_order);
    a.slot_blocks = reinterpret_cast<uint4*>(tb + lay.o_slots);
    a.slot_cap = order_cap;
    a.draw_cap = draw_cap;
    a.gpu_draws = 1u;
    a.fused_shade = fused32 ? 1u : 0u;
    a.chunk_cap = chunk_cap;
    a.tri_cap = tri_cap;
    a.extra_cap = (uint32_t)extra_cap;
    a.clip_cap = tri_cap;
    a.stile_cap = stile_cap;
    a.quad_cap = quad_cap;
    a.pixel_cap = pixel_cap;
    a.view_cap = view_cap;
    a.bin_cap = bin_cap;
    a.sched_tile = sched_tile;
    a.tri_state = tri_state.as<uint8_t>();
    a.rec_r = rec_r.as<RecRaster>();
    a.rec_s = rec_s.as<RecShade>();
    a.fan_base = fan_base.as<uint32_t>();
    a.clip_queue = clip_queue.as<uint2>();
    a.tile_count = tile_count.as<uint32_t>();
    a.tile_offset = tile_offset.as<uint32_t>();
    a.tile_cursor = tile_cursor.as<uint32_t>();
    a.bins = bins.as<uint32_t>();
    a.keys = keys.as<unsigned long long>();
    a.counters = counters.as<DCounters>();
    a.rsqrt_table = rsqrt_tab.as<uint8_t>();
    a.exposure_dev = nullptr;
    a.raster_grid = raster_grid;
    a.shade_grid = shade_grid;
    a.has_translucent = any_translucent ? 1u : 0u;
    a.rsqrt_uniform = 0u;
    if (!vws.empty()) {
        bool same = true;
        for (const DView& v : vws) same = same && v.rsqrt_mode == vws[0].rsqrt_mode;
        if (same && vws[0].rsqrt_mode <= 1u) a.rsqrt_uniform = 1u + vws[0].rsqrt_mode;
    }
    a.has_gi = 0u;
    for (const SceneImpl* sc : scenes)
        if (!sc->voxel_sh4.empty()) a.has_gi = 1u;
    a.defer_resolve = defer_resolve ? 1u : 0u;
    args = a;
    return SWR_OK;
}

swr_status FrameEngine::launch(cudaStream_t stream, cudaEvent_t* ev, std::string& err) {
    // The staging copy runs ahead of the kernels (graph or not) and is the
    // only reader of its staging buffer; with a ring of them the host stages
    // up to kStageRing frames ahead of the device.
    const int slot = stage_slot;
    cudaError_t e = cudaMemcpyAsync(tables.p, h_stage[slot].p, lay.staged, cudaMemcpyHostToDevice, stream);
    if (e == cudaSuccess) e = cudaEventRecord(stage_done[slot], stream);
    if (e == cudaSuccess) {
        stage_pending[slot] = true;
        stage_slot = (slot + 1) % kStageRing;
    }
    if (e == cudaSuccess && use_graph && !ev) {
        const bool same = graph_exec && std::memcmp(&graph_args, &args, sizeof(args)) == 0;
        if (!same) {
            if (graph_exec) cudaGraphExecDestroy(graph_exec);
            graph_exec = nullptr;
            if (!capture_stream) e = cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking);
            cudaGraph_t g = nullptr;
            // Capture on the engine's own stream; the graph is then launched
            // into the caller's stream (which may be the legacy default one).
            if (e == cudaSuccess) e = cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                graph_kernels = launch_frame(args, capture_stream, num_sms, nullptr);
                e = cudaStreamEndCapture(capture_stream, &g);
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&graph_exec, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                err = std::string("graph capture failed: ") + cudaGetErrorString(e);
                cudaGetLastError();
                graph_exec = nullptr;
                return SWR_CUDA_ERROR;
            }
            graph_args = args;
            graph_stream = stream;
        }
        e = cudaGraphLaunch(graph_exec, stream);
        if (e == cudaSuccess) kernel_launches += graph_kernels;
    } else if (e == cudaSuccess) {
        kernel_launches += launch_frame(args, stream, num_sms, ev);
        e = cudaGetLastError();
    }
    if (e != cudaSuccess) {
        err = std::string("frame launch failed: ") + cudaGetErrorString(e);
        cudaGetLastError();
        return SWR_CUDA_ERROR;
    }
    return SWR_OK;
}

swr_status FrameEngine::grow_for(const DCounters& c, std::string& err) {
    if (c.status & ST_DRAW_OVERFLOW) {
        tri_cap = grow(tri_cap, c.draw_tris);
        chunk_cap = grow(chunk_cap, c.draw_chunks);
        draw_cap = grow(draw_cap, c.draw_count);
    }
    if (c.status & ST_BIN_OVERFLOW) bin_cap = std::max<uint64_t>(bin_cap * 2, c.pairs + c.pairs / 4);
    if (c.status & ST_CLIP_OVERFLOW)
        extra_cap = std::max<uint64_t>(extra_cap * 2, (uint64_t)c.extra_used + c.extra_used / 4);
    if (c.status & ST_TRANS_OVERFLOW) {
        if (sched_tile <= 8) {
            err = "more translucent packets overlap one 8-pixel tile than the translucent sort holds";
            return SWR_OVERFLOW;
        }
        sched_tile /= 2;
    }
    retries++;
    return SWR_OK;
}

swr_status FrameEngine::run(const std::vector<const SceneImpl*>& scenes, std::vector<DView>& vws,
                            const std::vector<const swr_camera*>& cams, cudaStream_t stream, FrameArgs* out,
                            std::string& err, cudaEvent_t* ev) {
    swr_status st = prepare(scenes, vws, cams, err);
    if (st != SWR_OK) return st;
    st = launch(stream, ev, err);
    if (out) *out = args;
    return st;
}

}  // namespace swr
