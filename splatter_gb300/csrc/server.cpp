// Serving runtime of libsplatter_cuda.so (spl_server_*, include/splatter.h).  It has no counterpart
// in the reference, whose Renderer renders one frame per call (renderer.rs:355-466).
//
// Scenes: every scene has a page-locked host copy in the device layout (one block: rotations,
// scale+opacity, SH, x, y, z) and, while resident, one block from a stream-ordered device memory
// pool.  Residency is admitted against `scene_memory_budget`; the least recently used scene with no
// request in flight is evicted (its device block returned to the pool on the copy stream) and copied
// back for its next request, the request's stream waiting on the copy's event: at the request's
// admission, or earlier, while it still waits in the queue (up to two scenes of the next 2 x slots
// queued requests, evicting none that those requests want).
//
// Requests: a FIFO queue filled by spl_server_submit from any thread.  One scheduler thread admits
// the head request whenever a slot is free (continuous admission: no batch boundary), renders it on
// the slot's stream (a captured frame graph per viewport and scene-size class, launched with the
// request's scene and camera, or direct launches), copies the image and the frame's error word to the host, and
// queues a host callback that marks the slot done and wakes the scheduler.  Slots share nothing on the device but the
// scene arrays they read, so the frames of different slots overlap.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <tuple>
#include <vector>

#include "spl_internal.h"

namespace {

uint64_t now_ns() {
    return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
               std::chrono::steady_clock::now().time_since_epoch())
        .count();
}

// Device/host block layout of one scene of n splats: rot[n] float4, scale_alpha[n] float4, sh[48n],
// x[n], y[n], z[n] (every array 16-byte aligned when the block is).
constexpr uint64_t SPLAT_BYTES = 16 + 16 + 192 + 4 + 4 + 4;

struct ServerScene {
    uint32_t id = 0;
    spl_scene view;  // owns = false: its arrays point into `dev` while resident
    uint64_t n = 0, bytes = 0;
    unsigned char* host = nullptr;  // page-locked copy
    unsigned char* dev = nullptr;   // pool block while resident
    cudaEvent_t ready = nullptr;    // the block's last copy to the device
    uint64_t last_use = 0;
    uint32_t in_flight = 0;
    bool wanted = false;      // needed by one of the next queued requests (scheduler's lookahead window)
    bool prefetched = false;  // copied back ahead of its request; the request that uses it reports it

    void point_view() {
        unsigned char* b = dev;
        view.rot = reinterpret_cast<float4*>(b);
        view.scale_alpha = reinterpret_cast<float4*>(b + 16 * n);
        view.sh = reinterpret_cast<float*>(b + 32 * n);
        view.x = reinterpret_cast<float*>(b + 224 * n);
        view.y = reinterpret_cast<float*>(b + 228 * n);
        view.z = reinterpret_cast<float*>(b + 232 * n);
    }
};

using GraphKey = std::tuple<uint32_t, uint32_t, uint64_t>;  // viewport width, height, scene-size class

// Grids of a captured frame are sized for the size class: the next power of two of the scene's
// splat count (at least 2^16, at most the renderer's maximum), so a small scene does not launch the
// empty CTAs of the largest one.
uint64_t size_class(uint64_t n, uint64_t max_n) {
    uint64_t c = 1ull << 16;
    while (c < n) c <<= 1;
    return c < max_n ? c : max_n;
}

struct Slot {
    spl_server* owner = nullptr;
    uint32_t index = 0;
    spl_renderer* r = nullptr;
    cudaStream_t st = nullptr;
    void* d_out = nullptr;
    uint32_t* h_err = nullptr;  // page-locked: the frame's device error bits
    std::map<GraphKey, spl_frame_graph*> graphs;
    bool busy = false;
    std::atomic<bool> done{false};
    std::atomic<uint64_t> t_done{0};
    spl_request req{};
    uint64_t t_submit = 0, t_start = 0;
    ServerScene* scene = nullptr;
    bool restored = false;
    int launch_status = SPL_OK;
};

struct Pending {
    spl_request req;
    uint64_t t_submit;
};

constexpr int BLOCKED = -1;  // make_resident: every other resident scene is in use; retry after a completion

}  // namespace

struct spl_server {
    spl_config cfg{};
    spl_server_config scfg{};
    int device = 0;
    size_t pixel_bytes = 4;
    cudaMemPool_t pool = nullptr;
    cudaStream_t copy_st = nullptr;
    std::vector<std::unique_ptr<ServerScene>> scenes;
    std::atomic<uint32_t> scene_count{0};
    std::vector<std::unique_ptr<Slot>> slots;
    uint64_t resident_bytes = 0, use_tick = 0;
    std::mutex sched_mu;  // scenes, slots, residency: the scheduler loop and spl_server_add_scene
    std::mutex q_mu;
    std::deque<Pending> queue;
    std::mutex wake_mu;
    std::condition_variable wake_cv;
    bool wake = false, stop = false;
    std::mutex c_mu;
    std::condition_variable c_cv;
    std::deque<spl_completion> done;
    std::atomic<uint64_t> submitted{0}, completed{0}, failed{0}, evictions{0}, restores{0}, graphs_captured{0},
        graph_launches{0}, direct_launches{0}, max_in_flight{0};
    std::thread thread;
};

namespace {

void notify(spl_server* s) {
    {
        std::lock_guard<std::mutex> lk(s->wake_mu);
        s->wake = true;
    }
    s->wake_cv.notify_one();
}

void CUDART_CB on_slot_done(void* p) {
    Slot* slot = static_cast<Slot*>(p);
    slot->t_done.store(now_ns(), std::memory_order_relaxed);
    slot->done.store(true, std::memory_order_release);
    notify(slot->owner);
}

// Returns the scene's device block to the pool.  Only for scenes with no request in flight: their
// last frames have completed (the slot callbacks ran), so nothing on the device still reads them.
void evict(spl_server* s, ServerScene* sc) {
    cudaFreeAsync(sc->dev, s->copy_st);
    sc->dev = nullptr;
    sc->prefetched = false;
    s->resident_bytes -= sc->bytes;
    s->evictions.fetch_add(1);
}

// The least recently used resident scene with no request in flight, preferring scenes that none of
// the next queued requests wants; with `spare_wanted` the wanted ones are never chosen.
ServerScene* lru_victim(spl_server* s, const ServerScene* keep, bool spare_wanted) {
    ServerScene* v = nullptr;
    for (auto& c : s->scenes) {
        if (!c->dev || c.get() == keep || c->in_flight != 0 || (spare_wanted && c->wanted)) continue;
        if (!v || (v->wanted && !c->wanted) || (v->wanted == c->wanted && c->last_use < v->last_use)) v = c.get();
    }
    return v;
}

// Evicts until `need` more bytes fit the budget; BLOCKED when the scenes in use leave no room yet.
int make_room(spl_server* s, uint64_t need, const ServerScene* keep, bool spare_wanted) {
    const uint64_t budget = s->scfg.scene_memory_budget;
    if (!budget) return SPL_OK;
    if (need > budget) return spl::fail(SPL_ERR_CAPACITY, "scene of %llu bytes exceeds the scene memory budget",
                                        (unsigned long long)need);
    while (s->resident_bytes + need > budget) {
        ServerScene* v = lru_victim(s, keep, spare_wanted);
        if (!v) return BLOCKED;
        evict(s, v);
    }
    return SPL_OK;
}

int alloc_block(spl_server* s, ServerScene* sc, bool spare_wanted) {
    for (;;) {
        cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&sc->dev), sc->bytes, s->pool, s->copy_st);
        if (e == cudaSuccess) return SPL_OK;
        cudaGetLastError();
        sc->dev = nullptr;
        if (e != cudaErrorMemoryAllocation) return spl::fail(SPL_ERR_CUDA, "cudaMallocFromPoolAsync: %s",
                                                             cudaGetErrorString(e));
        ServerScene* v = lru_victim(s, sc, spare_wanted);  // out of device memory below the budget: evict further
        if (!v) return BLOCKED;
        evict(s, v);
    }
}

// Copies an evicted scene back to the device (asynchronously, on the copy stream).  With
// `spare_wanted` (a restore ahead of its request) no scene that a queued request wants is evicted.
int make_resident(spl_server* s, ServerScene* sc, bool spare_wanted = false) {
    int rc = make_room(s, sc->bytes, sc, spare_wanted);
    if (rc) return rc;
    rc = alloc_block(s, sc, spare_wanted);
    if (rc) return rc;
    CU(cudaMemcpyAsync(sc->dev, sc->host, sc->bytes, cudaMemcpyHostToDevice, s->copy_st));
    CU(cudaEventRecord(sc->ready, s->copy_st));
    sc->point_view();
    s->resident_bytes += sc->bytes;
    s->restores.fetch_add(1);
    return SPL_OK;
}

void complete(spl_server* s, const spl_completion& c) {
    if (c.status == SPL_OK)
        s->completed.fetch_add(1);
    else
        s->failed.fetch_add(1);
    {
        std::lock_guard<std::mutex> lk(s->c_mu);
        s->done.push_back(c);
    }
    s->c_cv.notify_all();
}

void retire(spl_server* s) {
    for (auto& slot : s->slots) {
        if (!slot->busy || !slot->done.load(std::memory_order_acquire)) continue;
        spl_completion c{};
        c.tag = slot->req.tag;
        c.slot = slot->index;
        c.t_submit_ns = slot->t_submit;
        c.t_start_ns = slot->t_start;
        c.t_done_ns = slot->t_done.load(std::memory_order_relaxed);
        c.restored = slot->restored ? 1u : 0u;
        c.status = slot->launch_status;
        if (c.status == SPL_OK && *slot->h_err) {
            const uint32_t err = *slot->h_err;
            c.status = (err & SPL_DEV_ERR_LOOKBACK) ? SPL_ERR_LOOKBACK_TIMEOUT : SPL_ERR_CAPACITY;
        }
        slot->scene->in_flight--;
        slot->scene = nullptr;
        slot->busy = false;
        complete(s, c);
    }
}

void launch(spl_server* s, Slot* slot, const Pending& p, ServerScene* sc, bool restored) {
    const spl_request& req = p.req;
    slot->busy = true;
    slot->done.store(false, std::memory_order_relaxed);
    slot->req = req;
    slot->t_submit = p.t_submit;
    slot->t_start = now_ns();
    slot->scene = sc;
    slot->restored = restored;
    sc->in_flight++;
    sc->last_use = ++s->use_tick;
    int rc = SPL_OK;
    if (cudaStreamWaitEvent(slot->st, sc->ready, 0) != cudaSuccess) {
        cudaGetLastError();
        rc = spl::fail(SPL_ERR_CUDA, "cudaStreamWaitEvent failed");
    }
    if (!rc && s->scfg.use_graphs) {
        const uint64_t cls = size_class(sc->n, s->cfg.max_splat_count);
        const GraphKey key{req.width, req.height, cls};
        auto it = slot->graphs.find(key);
        if (it == slot->graphs.end()) {
            spl_frame_graph* g = nullptr;
            rc = spl_frame_graph_create(slot->r, req.width, req.height, cls, slot->d_out, &g);
            if (!rc) {
                it = slot->graphs.emplace(key, g).first;
                s->graphs_captured.fetch_add(1);
            }
        }
        if (!rc) rc = spl_frame_graph_launch(it->second, &sc->view, req.camera_to_world, slot->st);
        if (!rc) s->graph_launches.fetch_add(1);
    } else if (!rc) {
        rc = spl_render_frame(slot->r, &sc->view, req.camera_to_world, req.width, req.height, slot->d_out, slot->st);
        if (!rc) s->direct_launches.fetch_add(1);
    }
    if (!rc) {
        cudaError_t e = cudaMemcpyAsync(slot->h_err, &slot->r->fc->err, 4, cudaMemcpyDeviceToHost, slot->st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(req.host_out, slot->d_out, (size_t)req.width * req.height * s->pixel_bytes,
                                cudaMemcpyDeviceToHost, slot->st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = spl::fail(SPL_ERR_CUDA, "result copy: %s", cudaGetErrorString(e));
        }
    }
    slot->launch_status = rc;
    if (cudaLaunchHostFunc(slot->st, on_slot_done, slot) != cudaSuccess) {
        // cannot happen on a valid stream; retire the slot at once
        cudaGetLastError();
        if (!slot->launch_status) slot->launch_status = SPL_ERR_CUDA;
        slot->t_done.store(now_ns());
        slot->done.store(true, std::memory_order_release);
    }
    uint64_t busy = 0;
    for (auto& o : s->slots) busy += o->busy ? 1 : 0;
    uint64_t m = s->max_in_flight.load();
    while (busy > m && !s->max_in_flight.compare_exchange_weak(m, busy)) {
    }
}

// Admits queue heads while slots are free.  A head whose scene cannot be made resident yet (every
// other resident scene in use) waits for a completion.
void admit(spl_server* s) {
    for (;;) {
        Slot* slot = nullptr;
        for (auto& o : s->slots)
            if (!o->busy) {
                slot = o.get();
                break;
            }
        if (!slot) return;
        Pending p;
        {
            std::lock_guard<std::mutex> lk(s->q_mu);
            if (s->queue.empty()) return;
            p = s->queue.front();
        }
        ServerScene* sc = s->scenes[p.req.scene_id].get();
        bool restored = false;
        int rc = SPL_OK;
        if (!sc->dev) {
            rc = make_resident(s, sc);
            if (rc == BLOCKED) return;
            restored = rc == SPL_OK;
        } else if (sc->prefetched) {  // copied back ahead of this request
            restored = true;
            sc->prefetched = false;
        }
        {
            std::lock_guard<std::mutex> lk(s->q_mu);
            s->queue.pop_front();
        }
        if (rc) {
            spl_completion c{};
            c.tag = p.req.tag;
            c.status = rc;
            c.t_submit_ns = c.t_start_ns = c.t_done_ns = now_ns();
            complete(s, c);
            continue;
        }
        launch(s, slot, p, sc, restored);
    }
}

// Marks the scenes of the next `window` queued requests as wanted (evicted last, never by a restore
// ahead of a request) and returns their ids in queue order.
std::vector<uint32_t> mark_wanted(spl_server* s, size_t window) {
    std::vector<uint32_t> ids;
    {
        std::lock_guard<std::mutex> lk(s->q_mu);
        for (size_t i = 0; i < s->queue.size() && ids.size() < window; ++i) ids.push_back(s->queue[i].req.scene_id);
    }
    for (auto& c : s->scenes) c->wanted = false;
    for (uint32_t id : ids)
        if (id < s->scenes.size()) s->scenes[id]->wanted = true;
    return ids;
}

// With a scene memory budget: copies the scenes of the next queued requests back before those
// requests are admitted, so that the copy engine works while the slots render (a restore at admission
// leaves it idle until a slot frees).  At most two such restores wait for their requests at a time,
// and none evicts a scene that a queued request in the window wants.
void prefetch(spl_server* s) {
    if (!s->scfg.scene_memory_budget) return;
    const std::vector<uint32_t> ids = mark_wanted(s, 2 * s->slots.size());
    int ahead = 0;
    for (auto& c : s->scenes) ahead += c->prefetched ? 1 : 0;
    for (uint32_t id : ids) {
        if (ahead >= 2) break;
        if (id >= s->scenes.size()) continue;
        ServerScene* sc = s->scenes[id].get();
        if (sc->dev) continue;
        if (make_resident(s, sc, true) != SPL_OK) break;  // no room yet (an error is reported at admission)
        sc->prefetched = true;
        sc->last_use = ++s->use_tick;
        ++ahead;
    }
}

void scheduler(spl_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        bool idle;
        {
            std::lock_guard<std::mutex> g(s->sched_mu);
            retire(s);
            if (s->scfg.scene_memory_budget) mark_wanted(s, 2 * s->slots.size());
            admit(s);
            prefetch(s);
            bool any_busy = false;
            for (auto& o : s->slots) any_busy = any_busy || o->busy;
            std::lock_guard<std::mutex> lk(s->q_mu);
            idle = !any_busy && s->queue.empty();
        }
        std::unique_lock<std::mutex> wl(s->wake_mu);
        if (s->stop && idle) return;
        s->wake_cv.wait(wl, [&] { return s->wake || s->stop; });
        s->wake = false;
    }
}

void release_server(spl_server* s) {
    for (auto& slot : s->slots) {
        for (auto& kv : slot->graphs) spl_frame_graph_destroy(kv.second);
        slot->graphs.clear();
        if (slot->r) spl_renderer_destroy(slot->r);
        if (slot->st) cudaStreamDestroy(slot->st);
        if (slot->d_out) cudaFree(slot->d_out);
        if (slot->h_err) cudaFreeHost(slot->h_err);
    }
    s->slots.clear();
    for (auto& sc : s->scenes) {
        if (sc->dev) cudaFreeAsync(sc->dev, s->copy_st);
        sc->dev = nullptr;
    }
    if (s->copy_st) cudaStreamSynchronize(s->copy_st);
    for (auto& sc : s->scenes) {
        if (sc->host) cudaFreeHost(sc->host);
        if (sc->ready) cudaEventDestroy(sc->ready);
    }
    s->scenes.clear();
    if (s->copy_st) cudaStreamDestroy(s->copy_st);
    if (s->pool) cudaMemPoolDestroy(s->pool);
    cudaGetLastError();
}

}  // namespace

extern "C" {

uint64_t spl_server_now_ns(void) { return now_ns(); }

int spl_server_create(const spl_config* cfg, const spl_server_config* scfg, spl_server** out) {
    if (!cfg || !scfg || !out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    *out = nullptr;
    if (scfg->slots == 0 || scfg->slots > 64) return spl::fail(SPL_ERR_INVALID, "slots %u outside [1, 64]", scfg->slots);
    if (scfg->max_width == 0 || scfg->max_height == 0 || scfg->max_width > 65535 || scfg->max_height > 65535)
        return spl::fail(SPL_ERR_INVALID, "max viewport %ux%u", scfg->max_width, scfg->max_height);
    spl_server* s = new (std::nothrow) spl_server();
    if (!s) return spl::fail(SPL_ERR_OOM, "host allocation failed");
    s->cfg = *cfg;
    s->scfg = *scfg;
    s->pixel_bytes = cfg->blend_mode == SPL_BLEND_FP32 ? 16 : 4;
    cudaGetDevice(&s->device);
    auto bail = [&](int rc) {
        release_server(s);
        delete s;
        return rc;
    };
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = s->device;
    cudaError_t e = cudaMemPoolCreate(&s->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = ~0ull;  // keep freed blocks mapped for the next restore
        e = cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->copy_st, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bail(spl::fail(SPL_ERR_CUDA, "server setup: %s", cudaGetErrorString(e)));
    }
    const size_t out_bytes = (size_t)scfg->max_width * scfg->max_height * s->pixel_bytes;
    for (uint32_t i = 0; i < scfg->slots; ++i) {
        auto slot = std::make_unique<Slot>();
        slot->owner = s;
        slot->index = i;
        int rc = spl_renderer_create(cfg, &slot->r);
        // several slots run frames at once: the cooperative sort assumes the whole device
        if (!rc && scfg->slots > 1) rc = spl_renderer_set_sort_mode(slot->r, SPL_SORT_ONESWEEP);
        // concurrent frames already fill the device at a frame's end: the tile order would only add work
        if (!rc && scfg->slots > 1) slot->r->order_tiles = false;
        // the slots capture their own graphs per viewport and size class (use_graphs); otherwise frames
        // are launched directly, whatever the order of scenes
        if (!rc) slot->r->frame_graphs = false;
        if (!rc) rc = spl_renderer_reserve(slot->r, scfg->max_width, scfg->max_height);
        if (!rc) {
            e = cudaStreamCreateWithFlags(&slot->st, cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaMalloc(&slot->d_out, out_bytes);
            if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&slot->h_err), 4);
            if (e != cudaSuccess) {
                cudaGetLastError();
                rc = spl::fail(e == cudaErrorMemoryAllocation ? SPL_ERR_OOM : SPL_ERR_CUDA, "slot setup: %s",
                               cudaGetErrorString(e));
            }
        }
        s->slots.push_back(std::move(slot));
        if (rc) return bail(rc);
    }
    s->thread = std::thread(scheduler, s);
    *out = s;
    return SPL_OK;
}

void spl_server_destroy(spl_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->wake_mu);
        s->stop = true;
        s->wake = true;
    }
    s->wake_cv.notify_one();
    if (s->thread.joinable()) s->thread.join();
    release_server(s);
    delete s;
}

int spl_server_add_scene(spl_server* s, const float* records62, uint64_t count, int records_on_device,
                         uint32_t* scene_id) {
    if (!s || !scene_id || (!records62 && count)) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    if (count == 0) return spl::fail(SPL_ERR_INVALID, "empty scene");
    std::lock_guard<std::mutex> g(s->sched_mu);
    auto sc = std::make_unique<ServerScene>();
    sc->id = (uint32_t)s->scenes.size();
    sc->n = count < s->cfg.max_splat_count ? count : s->cfg.max_splat_count;  // scene.rs:46
    sc->bytes = (sc->n * SPLAT_BYTES + 255) & ~255ull;
    sc->view.owns = false;
    sc->view.n = sc->n;
    sc->view.device = s->device;
    int rc = make_room(s, sc->bytes, nullptr, false);
    if (rc == BLOCKED) return spl::fail(SPL_ERR_CAPACITY, "scenes in use leave no room for a new scene");
    if (rc) return rc;
    cudaError_t e = cudaEventCreateWithFlags(&sc->ready, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaHostAlloc(reinterpret_cast<void**>(&sc->host), sc->bytes, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (sc->ready) cudaEventDestroy(sc->ready);
        if (sc->host) cudaFreeHost(sc->host);
        return spl::fail(SPL_ERR_OOM, "scene host copy: %s", cudaGetErrorString(e));
    }
    auto undo = [&](int code) {
        if (sc->dev) cudaFreeAsync(sc->dev, s->copy_st);
        cudaStreamSynchronize(s->copy_st);
        cudaFreeHost(sc->host);
        cudaEventDestroy(sc->ready);
        cudaGetLastError();
        return code;
    };
    rc = alloc_block(s, sc.get(), false);
    if (rc == BLOCKED) return undo(spl::fail(SPL_ERR_OOM, "no device memory for the scene"));
    if (rc) return undo(rc);
    sc->point_view();
    if (records_on_device) {
        rc = spl_scene_load_chunk_device(&sc->view, records62, 0, sc->n, s->copy_st);
    } else {
        // through a device staging piece (pageable source: each copy completes before it returns)
        const uint64_t piece = 1ull << 20;
        float* tmp = nullptr;
        const uint64_t tn = sc->n < piece ? sc->n : piece;
        e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&tmp), tn * 248, s->pool, s->copy_st);
        for (uint64_t first = 0; e == cudaSuccess && !rc && first < sc->n; first += piece) {
            const uint64_t cnt = sc->n - first < piece ? sc->n - first : piece;
            e = cudaMemcpyAsync(tmp, records62 + first * 62, cnt * 248, cudaMemcpyHostToDevice, s->copy_st);
            if (e == cudaSuccess) rc = spl_scene_load_chunk_device(&sc->view, tmp, first, cnt, s->copy_st);
        }
        if (tmp) cudaFreeAsync(tmp, s->copy_st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            rc = spl::fail(SPL_ERR_CUDA, "scene upload: %s", cudaGetErrorString(e));
        }
    }
    if (rc) return undo(rc);
    e = cudaMemcpyAsync(sc->host, sc->dev, sc->bytes, cudaMemcpyDeviceToHost, s->copy_st);
    if (e == cudaSuccess) e = cudaEventRecord(sc->ready, s->copy_st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->copy_st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return undo(spl::fail(SPL_ERR_CUDA, "scene host copy: %s", cudaGetErrorString(e)));
    }
    sc->last_use = ++s->use_tick;
    s->resident_bytes += sc->bytes;
    *scene_id = sc->id;
    s->scenes.push_back(std::move(sc));
    s->scene_count.store((uint32_t)s->scenes.size(), std::memory_order_release);
    return SPL_OK;
}

int spl_server_submit(spl_server* s, const spl_request* req) {
    if (!s || !req || !req->host_out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    if (req->scene_id >= s->scene_count.load(std::memory_order_acquire))
        return spl::fail(SPL_ERR_INVALID, "unknown scene %u", req->scene_id);
    if (req->width == 0 || req->height == 0 || req->width > s->scfg.max_width || req->height > s->scfg.max_height)
        return spl::fail(SPL_ERR_INVALID, "viewport %ux%u outside the server's %ux%u", req->width, req->height,
                         s->scfg.max_width, s->scfg.max_height);
    {
        std::lock_guard<std::mutex> lk(s->q_mu);
        s->queue.push_back(Pending{*req, now_ns()});
    }
    s->submitted.fetch_add(1);
    notify(s);
    return SPL_OK;
}

int spl_server_poll(spl_server* s, spl_completion* out, uint32_t capacity, uint32_t* count, int64_t timeout_us) {
    if (!s || !count || (!out && capacity)) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    *count = 0;
    std::unique_lock<std::mutex> lk(s->c_mu);
    auto ready = [&] { return !s->done.empty(); };
    if (timeout_us < 0)
        s->c_cv.wait(lk, ready);
    else if (timeout_us > 0)
        s->c_cv.wait_for(lk, std::chrono::microseconds(timeout_us), ready);
    uint32_t n = 0;
    while (n < capacity && !s->done.empty()) {
        out[n++] = s->done.front();
        s->done.pop_front();
    }
    *count = n;
    return SPL_OK;
}

int spl_server_get_stats(spl_server* s, spl_server_stats* out) {
    if (!s || !out) return spl::fail(SPL_ERR_INVALID, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    out->submitted = s->submitted.load();
    out->completed = s->completed.load();
    out->failed = s->failed.load();
    out->evictions = s->evictions.load();
    out->restores = s->restores.load();
    out->graphs_captured = s->graphs_captured.load();
    out->graph_launches = s->graph_launches.load();
    out->direct_launches = s->direct_launches.load();
    out->max_in_flight = s->max_in_flight.load();
    std::lock_guard<std::mutex> g(s->sched_mu);
    for (auto& sc : s->scenes)
        if (sc->dev) {
            out->resident_scenes++;
            out->resident_bytes += sc->bytes;
        }
    return SPL_OK;
}

}  // extern "C"
