// Served form: a request loop over HBM-resident scenes.
//
// Requests (scene, camera, resolution) are queued by swr_server_submit. A
// worker thread forms batches continuously: whenever one of the `inflight`
// engines (each with its own stream) is free, every pending request that can
// get a framebuffer from the pool joins the next batch (FIFO, up to
// max_batch_views). Framebuffers are pooled per resolution and new ones are
// allocated only while resident scenes + framebuffers + engine buffers stay
// within the memory budget; otherwise requests wait for releases. Batches on
// different engines overlap on the device. A host callback on each batch's
// stream wakes the worker, which checks the batch's status word (re-running
// it on bin overflow) and publishes completions.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>

#include "batch.h"

using namespace swr;

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct FB {
    DBuf rgba8, vis;
    int32_t w = 0, h = 0;
};

struct Req {
    uint64_t ticket;
    swr_request r;
    double t_submit;
};

struct Engine {
    std::unique_ptr<BatchImpl> b;
    cudaStream_t stream = nullptr;
    bool busy = false;
    uint64_t bytes = 0;  // device bytes of the engine's buffers, refreshed by the worker under the lock
    uint64_t reserved = 0;  // bytes admitted for the batch in flight (its buffers may grow to it on a retry)
    std::atomic<bool> done{false};
    std::vector<Req> reqs;
    std::vector<FB*> fbs;
    double t_launch = 0.0;
};

struct Done {
    swr_completion c;
    FB* fb;
};

}  // namespace

struct swr_server {
    swr_server_opts opts{};
    std::vector<const swr_scene*> scenes;
    std::vector<bool> scene_translucent;  // the scene has translucent primitives (colour buffer per view)
    uint64_t scene_bytes = 0, fb_bytes = 0;
    std::vector<std::unique_ptr<Engine>> engines;
    std::map<uint64_t, std::vector<FB*>> free_fbs;  // key: w << 32 | h
    std::vector<std::unique_ptr<FB>> all_fbs;
    std::deque<Req> pending;
    std::deque<Done> done;
    std::map<uint64_t, FB*> held;
    std::mutex mu;
    std::condition_variable cv, cv_done;
    std::thread worker;
    bool stop = false;
    uint64_t next_ticket = 1;
    swr_server_stats stats{};

    // Read under the lock; the worker refreshes Engine::bytes after an
    // engine's buffers may have grown (never while another thread reads).
    uint64_t engine_bytes() {
        uint64_t t = 0;
        for (auto& e : engines) t += std::max(e->bytes, e->reserved);
        return t;
    }

    FB* get_fb(int32_t w, int32_t h) {
        const uint64_t key = ((uint64_t)(uint32_t)w << 32) | (uint32_t)h;
        auto& fl = free_fbs[key];
        if (!fl.empty()) {
            FB* f = fl.back();
            fl.pop_back();
            return f;
        }
        const uint64_t need = (uint64_t)w * h * (sizeof(uint32_t) + sizeof(uint64_t));
        if (scene_bytes + fb_bytes + engine_bytes() + need > opts.memory_budget) return nullptr;
        auto f = std::make_unique<FB>();
        f->w = w;
        f->h = h;
        if (f->rgba8.ensure((size_t)w * h * sizeof(uint32_t)) != cudaSuccess ||
            f->vis.ensure((size_t)w * h * sizeof(uint64_t)) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        fb_bytes += f->rgba8.bytes + f->vis.bytes;
        all_fbs.push_back(std::move(f));
        return all_fbs.back().get();
    }

    // Device bytes an engine needs for a batch, upper estimate: keys of the
    // padded tile grids (and linear colour for views of scenes with
    // translucent primitives), triangle records (raster + shade + clip
    // headroom) and bins for every triangle of every view's scene.
    static uint64_t batch_need(const std::vector<std::pair<int32_t, int32_t>>& dims,
                               const std::vector<uint64_t>& tris, const std::vector<bool>& trans) {
        uint64_t t = 0;
        for (size_t i = 0; i < dims.size(); ++i) {
            const uint64_t tx = (uint64_t)(dims[i].first + 63) / 64, ty = (uint64_t)(dims[i].second + 63) / 64;
            t += tx * ty * 64 * 64 * (trans[i] ? 8 + 12 : 8) * 5 / 4;  // with the keys' 25% headroom
            // Record slots as the engine sizes them at most: every triangle of
            // the view's scene plus the 25% growth headroom, clip fan slots
            // (a quarter more), per-slot state, fan bases, clip queue and two
            // bin entries per slot.
            const uint64_t T = tris[i] * 5 / 4 + 16;
            t += (T + T / 4) * (80 + 176) + T * (1 + 4 + 8) + T * 2 * 4;
        }
        return t + (1u << 20);
    }
    // Worker thread only (the engine's buffers are not being grown).
    static uint64_t one_engine_bytes(const Engine& e) {
        const FrameEngine& f = e.b->eng;
        uint64_t t = e.b->tile_lum.bytes;
        for (const DBuf* d : {&f.tables, &f.tri_state, &f.rec_r, &f.rec_s, &f.fan_base, &f.clip_queue,
                              &f.tile_count, &f.tile_offset, &f.tile_cursor, &f.bins, &f.keys, &f.counters,
                              &f.rsqrt_tab, &f.color})
            t += d->bytes;
        for (const OwnedOutput& o : e.b->owned) t += o.rgba8.bytes + o.vis.bytes;
        return t;
    }

    void put_fb(FB* f) { free_fbs[((uint64_t)(uint32_t)f->w << 32) | (uint32_t)f->h].push_back(f); }

    static void CUDART_CB on_done(void* p) {
        auto* pr = static_cast<std::pair<swr_server*, Engine*>*>(p);
        pr->second->done.store(true);
        pr->first->cv.notify_one();
    }

    std::vector<std::pair<swr_server*, Engine*>> cb_args;

    void run() {
        std::unique_lock<std::mutex> lk(mu);
        while (!stop) {
            cv.wait_for(lk, std::chrono::milliseconds(2), [&] {
                if (stop) return true;
                for (auto& e : engines)
                    if (e->busy && e->done.load()) return true;
                if (!pending.empty())
                    for (auto& e : engines)
                        if (!e->busy) return true;
                return false;
            });
            if (stop) break;
            // Completions.
            for (auto& e : engines) {
                if (!e->busy || !e->done.load()) continue;
                lk.unlock();
                std::string err;
                const swr_status st = e->b->sync(err);  // may re-render with grown buffers
                const double t = now_ms();
                const uint64_t eb = one_engine_bytes(*e);
                lk.lock();
                e->bytes = eb;
                for (size_t i = 0; i < e->reqs.size(); ++i) {
                    Done d{};
                    d.c.ticket = e->reqs[i].ticket;
                    d.c.tag = e->reqs[i].r.tag;
                    d.c.status = st;
                    d.c.width = e->reqs[i].r.width;
                    d.c.height = e->reqs[i].r.height;
                    d.c.batch_views = (int32_t)e->reqs.size();
                    d.c.rgba8 = e->fbs[i]->rgba8.as<uint32_t>();
                    d.c.vis = e->fbs[i]->vis.as<uint64_t>();
                    d.c.queue_ms = e->t_launch - e->reqs[i].t_submit;
                    d.c.latency_ms = t - e->reqs[i].t_submit;
                    d.fb = e->fbs[i];
                    done.push_back(d);
                    stats.completed++;
                }
                e->reqs.clear();
                e->fbs.clear();
                e->busy = false;
                e->reserved = 0;
                e->done.store(false);
                cv_done.notify_all();
            }
            // Launch new batches on free engines.
            for (size_t ei = 0; ei < engines.size() && !pending.empty(); ++ei) {
                Engine& e = *engines[ei];
                if (e.busy) continue;
                std::vector<Req> reqs;
                std::vector<FB*> fbs;
                std::vector<std::pair<int32_t, int32_t>> dims;
                std::vector<uint64_t> tris;
                std::vector<bool> trans;
                const uint64_t others = engine_bytes() - std::max(e.bytes, e.reserved);
                uint64_t admitted = 0;
                while (!pending.empty() && reqs.size() < opts.max_batch_views) {
                    const Req& q = pending.front();
                    // Admission: this engine's buffers for the grown batch must
                    // fit the budget next to the scenes, framebuffers and the
                    // other engines (a lone request is always tried).
                    dims.push_back({q.r.width, q.r.height});
                    tris.push_back(scenes[q.r.scene]->impl.tri_total);
                    trans.push_back(scene_translucent[q.r.scene]);
                    const uint64_t need = std::max(e.bytes, batch_need(dims, tris, trans));
                    if (!reqs.empty() && scene_bytes + fb_bytes + others + need +
                                                 (uint64_t)q.r.width * q.r.height * 12 > opts.memory_budget) {
                        break;
                    }
                    FB* f = get_fb(q.r.width, q.r.height);
                    if (!f) break;  // wait for framebuffers to be released
                    admitted = need;
                    reqs.push_back(q);
                    fbs.push_back(f);
                    pending.pop_front();
                }
                if (reqs.empty()) break;
                std::vector<swr_view_desc> vd(reqs.size());
                for (size_t i = 0; i < reqs.size(); ++i) {
                    vd[i].scene = scenes[reqs[i].r.scene];
                    vd[i].camera = &reqs[i].r.camera;
                    vd[i].width = reqs[i].r.width;
                    vd[i].height = reqs[i].r.height;
                    vd[i].exposure = reqs[i].r.exposure;
                    vd[i].rsqrt_mode = opts.rsqrt_mode;
                    vd[i].rgba8 = fbs[i]->rgba8.as<uint32_t>();
                    vd[i].vis = fbs[i]->vis.as<uint64_t>();
                }
                e.reqs = std::move(reqs);
                e.fbs = std::move(fbs);
                e.busy = true;
                e.reserved = admitted;
                e.done.store(false);
                e.t_launch = now_ms();
                stats.batches++;
                lk.unlock();
                std::string err;
                // vd's camera pointers refer to e.reqs, which the worker owns.
                for (size_t i = 0; i < vd.size(); ++i) vd[i].camera = &e.reqs[i].r.camera;
                swr_status st = e.b->render(vd.data(), (int32_t)vd.size(), e.stream, err);
                if (st == SWR_OK) {
                    if (cudaLaunchHostFunc(e.stream, on_done, &cb_args[ei]) != cudaSuccess) st = SWR_CUDA_ERROR;
                }
                const uint64_t eb = one_engine_bytes(e);
                lk.lock();
                e.bytes = eb;
                if (st != SWR_OK) {
                    // Report the failure for every request of the batch.
                    const double t = now_ms();
                    for (size_t i = 0; i < e.reqs.size(); ++i) {
                        Done d{};
                        d.c.ticket = e.reqs[i].ticket;
                        d.c.tag = e.reqs[i].r.tag;
                        d.c.status = st;
                        d.c.latency_ms = t - e.reqs[i].t_submit;
                        d.fb = e.fbs[i];
                        done.push_back(d);
                    }
                    e.reqs.clear();
                    e.fbs.clear();
                    e.busy = false;
                    e.reserved = 0;
                    cv_done.notify_all();
                }
            }
        }
    }
};

extern "C" {

swr_status swr_server_create(const swr_server_opts* opts, swr_server** out) {
    if (!out) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    *out = nullptr;
    swr_server_opts o{};
    if (opts) o = *opts;
    if (o.memory_budget == 0) o.memory_budget = 40ull << 30;
    if (o.max_batch_views == 0) o.max_batch_views = 64;
    if (o.max_queue == 0) o.max_queue = 4096;
    if (o.inflight == 0) o.inflight = 2;
    if (o.inflight > 8) o.inflight = 8;
    if (o.sched_tile != 0 && o.sched_tile != 8 && o.sched_tile != 16 && o.sched_tile != 32 && o.sched_tile != 64) {
        set_last_error("sched_tile must be 0, 8, 16, 32 or 64");
        return SWR_INVALID_ARG;
    }
    swr_server* s = new (std::nothrow) swr_server();
    if (!s) {
        set_last_error("out of host memory");
        return SWR_NO_MEMORY;
    }
    s->opts = o;
    s->stats.budget = o.memory_budget;
    s->cb_args.resize(o.inflight);
    for (uint32_t i = 0; i < o.inflight; ++i) {
        auto e = std::make_unique<Engine>();
        e->b = std::make_unique<BatchImpl>();
        e->b->opts.sched_tile = o.sched_tile;
        e->b->opt_fuse32 = e->b->base_fuse32 = (o.flags & SWR_BATCH_FUSED_SHADE) != 0u;
        e->b->eng.use_graph = o.use_graph != 0;
        std::string err;
        swr_status st = e->b->eng.init(err);
        if (st == SWR_OK && (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess ||
                             cudaEventCreate(&e->b->ev_start) != cudaSuccess ||
                             cudaEventCreate(&e->b->ev_end) != cudaSuccess)) {
            st = SWR_CUDA_ERROR;
            err = "stream/event creation failed";
        }
        if (st != SWR_OK) {
            s->engines.push_back(std::move(e));
            swr_server_destroy(s);
            set_last_error(err.c_str());
            return st;
        }
        s->cb_args[i] = {s, e.get()};
        e->bytes = swr_server::one_engine_bytes(*e);
        s->engines.push_back(std::move(e));
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return SWR_OK;
}

void swr_server_destroy(swr_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaDeviceSynchronize();
    for (auto& e : s->engines) {
        e->b->eng.release();
        e->b->tile_lum.release();
        for (auto& o : e->b->owned) {
            o.rgba8.release();
            o.vis.release();
        }
        if (e->b->ev_start) cudaEventDestroy(e->b->ev_start);
        if (e->b->ev_end) cudaEventDestroy(e->b->ev_end);
        if (e->stream) cudaStreamDestroy(e->stream);
    }
    for (auto& f : s->all_fbs) {
        f->rgba8.release();
        f->vis.release();
    }
    delete s;
}

swr_status swr_server_add_scene(swr_server* s, const swr_scene* scene, int32_t* id) {
    if (!s || !scene || !id) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    if (!scene->impl.d_scene) {
        set_last_error("scene was created host-only");
        return SWR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->scene_bytes + s->fb_bytes + s->engine_bytes() + scene->impl.d_bytes > s->opts.memory_budget) {
        set_last_error("scene does not fit the memory budget");
        return SWR_BUSY;
    }
    s->scene_bytes += scene->impl.d_bytes;
    s->scenes.push_back(scene);
    bool trans = false;
    for (const HMesh& m : scene->impl.meshes) trans |= !m.translucent.empty();
    s->scene_translucent.push_back(trans);
    *id = (int32_t)s->scenes.size() - 1;
    return SWR_OK;
}

swr_status swr_server_submit(swr_server* s, const swr_request* r, uint64_t* ticket) {
    if (!s || !r) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    if (r->width <= 0 || r->height <= 0 || r->width > 32768 || r->height > 32768 || !(r->exposure > 0.0f)) {
        set_last_error("bad request size or exposure");
        return SWR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (r->scene < 0 || (size_t)r->scene >= s->scenes.size()) {
        set_last_error("unknown scene id");
        return SWR_INVALID_ARG;
    }
    if (s->pending.size() >= s->opts.max_queue) {
        s->stats.rejected++;
        set_last_error("request queue full");
        return SWR_BUSY;
    }
    Req q{s->next_ticket++, *r, now_ms()};
    s->pending.push_back(q);
    s->stats.submitted++;
    if (ticket) *ticket = q.ticket;
    s->cv.notify_one();
    return SWR_OK;
}

swr_status swr_server_poll(swr_server* s, swr_completion* out, int32_t max, int32_t* n, int32_t wait_ms) {
    if (!s || !out || !n || max <= 0) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_ms > 0)
        s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !s->done.empty(); });
    int32_t k = 0;
    while (k < max && !s->done.empty()) {
        Done d = s->done.front();
        s->done.pop_front();
        out[k++] = d.c;
        if (d.c.status == SWR_OK)
            s->held[d.c.ticket] = d.fb;
        else if (d.fb)
            s->put_fb(d.fb);
    }
    *n = k;
    return SWR_OK;
}

swr_status swr_server_release(swr_server* s, uint64_t ticket) {
    if (!s) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->held.find(ticket);
    if (it == s->held.end()) {
        set_last_error("unknown or already released ticket");
        return SWR_INVALID_ARG;
    }
    s->put_fb(it->second);
    s->held.erase(it);
    s->cv.notify_one();
    return SWR_OK;
}

swr_status swr_server_get_stats(swr_server* s, swr_server_stats* out) {
    if (!s || !out) {
        set_last_error("null argument");
        return SWR_INVALID_ARG;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->device_bytes = s->scene_bytes + s->fb_bytes + s->engine_bytes();
    out->budget = s->opts.memory_budget;
    return SWR_OK;
}

}  // extern "C"
