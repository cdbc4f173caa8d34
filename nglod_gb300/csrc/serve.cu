// Continuous-batching request server (nglod_serve_*): host-side scheduler
// over the library's own render and query entry points.
//
// State machine of a request: pending (FIFO) -> running (in a slot, its
// region allocated in the pool, work queued on the slot's stream, an event
// recorded after it) -> finished (the event completed; waiting to be polled)
// -> held (polled; results readable in the pool) -> released (region back
// in the pool, after the caller's copy stream passed a recorded event).
// Nothing blocks on the device except nglod_serve_destroy.
#include <chrono>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include "common.cuh"

namespace nglod {
namespace {

constexpr int64_t kRegionAlign = 256;
constexpr int kMaxSlots = 64;

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int64_t align_up(int64_t v) { return (v + kRegionAlign - 1) & ~(kRegionAlign - 1); }

// Byte offsets of a request's arrays inside its region.
struct Layout {
    int64_t org = 0, dir = 0, x = 0, t = 0, normal = 0, hit = 0, counter = 0, status = 0, sdf = 0;
    int64_t total = 0;
};

bool request_valid(const nglod_serve_request &r) {
    if (r.kind == NGLOD_SERVE_RENDER)
        return r.width > 0 && r.height > 0 && (int64_t)r.width * r.height <= ((int64_t)1 << 31) - 1;
    if (r.kind == NGLOD_SERVE_QUERY) return r.n >= 0 && r.n <= ((int64_t)1 << 31) - 1 && (r.n == 0 || r.points);
    return false;
}

Layout layout_of(const nglod_serve_request &r) {
    Layout L;
    int64_t off = 0;
    auto take = [&](int64_t bytes) {
        const int64_t o = off;
        off += align_up(bytes > 0 ? bytes : 1);
        return o;
    };
    if (r.kind == NGLOD_SERVE_RENDER) {
        const int64_t n = (int64_t)r.width * r.height;
        L.org = take(12 * n);
        L.dir = take(12 * n);
        L.x = take(12 * n);
        L.t = take(4 * n);
        L.normal = take(12 * n);
        L.hit = take(n);
        L.counter = take(8);
        L.status = take(4);
    } else {
        L.sdf = take(4 * r.n);
        L.status = take(4);
    }
    L.total = off;
    return L;
}

// First-fit allocator over the byte range [0, size) with coalescing frees.
class Pool {
   public:
    void reset(int64_t size) {
        free_.clear();
        if (size > 0) free_[0] = size;
    }
    int64_t alloc(int64_t bytes) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            const int64_t off = it->first, rest = it->second - bytes;
            free_.erase(it);
            if (rest > 0) free_[off + bytes] = rest;
            return off;
        }
        return -1;
    }
    void release(int64_t off, int64_t bytes) {
        auto next = free_.lower_bound(off);
        if (next != free_.end() && next->first == off + bytes) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == off) {
                prev->second += bytes;
                return;
            }
        }
        free_[off] = bytes;
    }

   private:
    std::map<int64_t, int64_t> free_;
};

struct Ticket {
    int64_t id = 0;
    nglod_serve_request req{};
    Layout lay;
    int64_t region = -1;
    int slot = -1;
    int32_t status = NGLOD_OK;
    double t_submit = 0, t_admit = 0, t_done = 0;
    cudaEvent_t ready = nullptr;  // recorded on the request's ready stream at submit
};

struct Model {
    bool bf16 = false;
    nglod_dense_model f32{};
    nglod_bf16_model b16{};
};

struct Quarantined {
    int64_t region, bytes;
    cudaEvent_t ev;
};

}  // namespace
}  // namespace nglod

using namespace nglod;

struct nglod_server {
    std::mutex mu;
    int64_t budget = 0;
    int slots = 0;
    bool custom = false;
    nglod_serve_executor ex{};
    int device = 0;
    char *pool_base = nullptr;
    int32_t *host_status = nullptr;  // pinned, one per slot
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> done_events;
    std::vector<cudaEvent_t> spare_events;
    Pool pool;
    std::vector<Model> models;
    std::deque<Ticket *> pending;
    std::vector<Ticket *> running;  // per slot
    std::deque<Ticket *> unpolled;
    std::map<int64_t, Ticket *> held;
    std::vector<Quarantined> quarantine;
    int64_t next_id = 0, used = 0, peak = 0, submitted = 0, completed = 0;
    int n_running = 0, max_concurrent = 0;
    bool stopped = false;
};

namespace {

// Makes the server's device current for the scope of an API call.
struct DeviceScope {
    int prev = -1;
    bool active = false;
    explicit DeviceScope(const nglod_server *s) {
        if (s->custom) return;
        if (cudaGetDevice(&prev) == cudaSuccess && prev != s->device) active = cudaSetDevice(s->device) == cudaSuccess;
    }
    ~DeviceScope() {
        if (active) cudaSetDevice(prev);
    }
};

int take_event(nglod_server *s, cudaEvent_t *ev) {
    if (!s->spare_events.empty()) {
        *ev = s->spare_events.back();
        s->spare_events.pop_back();
        return NGLOD_OK;
    }
    return cuda_status(cudaEventCreateWithFlags(ev, cudaEventDisableTiming), "serve: event create");
}

void give_event(nglod_server *s, cudaEvent_t ev) {
    if (ev) s->spare_events.push_back(ev);
}

void free_region(nglod_server *s, int64_t region, int64_t bytes) {
    s->pool.release(region, bytes);
    s->used -= bytes;
}

// Queues one request's work on its slot's stream.
int launch_cuda(nglod_server *s, Ticket *tk) {
    const nglod_serve_request &r = tk->req;
    cudaStream_t st = s->streams[tk->slot];
    char *base = s->pool_base + tk->region;
    const Model &m = s->models[r.model];
    int32_t *status = reinterpret_cast<int32_t *>(base + tk->lay.status);
    if (tk->ready) {
        NGLOD_TRY(cuda_status(cudaStreamWaitEvent(st, tk->ready, 0), "serve: wait for inputs"));
        give_event(s, tk->ready);
        tk->ready = nullptr;
    }
    NGLOD_TRY(cuda_status(cudaMemsetAsync(status, 0, sizeof(int32_t), st), "serve: status reset"));
    nglod_stream_t ns = reinterpret_cast<nglod_stream_t>(st);
    if (r.kind == NGLOD_SERVE_RENDER) {
        const int64_t n = (int64_t)r.width * r.height;
        float *org = reinterpret_cast<float *>(base + tk->lay.org);
        float *dir = reinterpret_cast<float *>(base + tk->lay.dir);
        float *x = reinterpret_cast<float *>(base + tk->lay.x);
        float *t = reinterpret_cast<float *>(base + tk->lay.t);
        float *normal = reinterpret_cast<float *>(base + tk->lay.normal);
        uint8_t *hit = reinterpret_cast<uint8_t *>(base + tk->lay.hit);
        int64_t *counter = reinterpret_cast<int64_t *>(base + tk->lay.counter);
        NGLOD_TRY(nglod_camera_rays(r.eye, r.at, r.up, r.fov_deg, r.width, r.height, org, dir, ns));
        nglod_trace_params p = r.trace;
        p.lod = r.lod;
        if (m.bf16)
            NGLOD_TRY(nglod_trace_bf16(&m.b16, &p, org, dir, n, x, t, hit, normal, counter, status, ns));
        else
            NGLOD_TRY(nglod_trace(&m.f32, &p, org, dir, n, x, t, hit, normal, counter, ns));
    } else if (r.n > 0) {
        float *out = reinterpret_cast<float *>(base + tk->lay.sdf);
        if (m.bf16)
            NGLOD_TRY(nglod_sdf_fwd_bf16(&m.b16, r.points, r.n, r.lod, out, status, ns));
        else
            NGLOD_TRY(nglod_sdf_fwd(&m.f32, r.points, r.n, r.lod, 0, out, ns));
    }
    NGLOD_TRY(cuda_status(cudaMemcpyAsync(&s->host_status[tk->slot], status, sizeof(int32_t), cudaMemcpyDeviceToHost, st),
                          "serve: status copy"));
    return cuda_status(cudaEventRecord(s->done_events[tk->slot], st), "serve: event record");
}

// 1 finished, 0 running, < 0 failed.
int query_slot(nglod_server *s, Ticket *tk) {
    if (s->custom) return s->ex.query(s->ex.ctx, tk->id, tk->slot);
    const cudaError_t e = cudaEventQuery(s->done_events[tk->slot]);
    if (e == cudaErrorNotReady) return 0;
    if (e != cudaSuccess) return cuda_status(e, "serve: event query");
    if (s->host_status[tk->slot] != 0) {
        set_error("serve: request %lld: a bounded tensor-core wait timed out", (long long)tk->id);
        return NGLOD_ERR_TIMEOUT;
    }
    return 1;
}

void finish(nglod_server *s, Ticket *tk, int32_t status, double t) {
    tk->status = status;
    tk->t_done = t;
    s->unpolled.push_back(tk);
    ++s->completed;
}

void reclaim(nglod_server *s) {
    size_t k = 0;
    for (size_t i = 0; i < s->quarantine.size(); ++i) {
        Quarantined &q = s->quarantine[i];
        const cudaError_t e = cudaEventQuery(q.ev);
        if (e == cudaErrorNotReady) {
            s->quarantine[k++] = q;
            continue;
        }
        free_region(s, q.region, q.bytes);
        give_event(s, q.ev);
    }
    s->quarantine.resize(k);
}

void retire(nglod_server *s) {
    const double t = now_s();
    for (int i = 0; i < s->slots; ++i) {
        Ticket *tk = s->running[i];
        if (!tk) continue;
        const int q = query_slot(s, tk);
        if (q == 0) continue;
        s->running[i] = nullptr;
        --s->n_running;
        finish(s, tk, q == 1 ? tk->status : q, t);
    }
}

void admit(nglod_server *s) {
    while (!s->pending.empty()) {
        int slot = -1;
        for (int i = 0; i < s->slots; ++i)
            if (!s->running[i]) {
                slot = i;
                break;
            }
        if (slot < 0) return;
        Ticket *tk = s->pending.front();
        const int64_t region = s->pool.alloc(tk->lay.total);
        if (region < 0) return;
        s->pending.pop_front();
        s->used += tk->lay.total;
        if (s->used > s->peak) s->peak = s->used;
        tk->region = region;
        tk->slot = slot;
        tk->t_admit = now_s();
        if (!s->custom) s->host_status[slot] = 0;
        const int st = s->custom ? s->ex.launch(s->ex.ctx, tk->id, slot, &tk->req, region, tk->lay.total)
                                 : launch_cuda(s, tk);
        if (st != NGLOD_OK) {
            tk->status = st;
            // Work queued before the failing launch may still write the
            // region: the request keeps its slot until that work is done.
            if (s->custom || cudaEventRecord(s->done_events[slot], s->streams[slot]) != cudaSuccess) {
                finish(s, tk, st, now_s());
                continue;
            }
        }
        s->running[slot] = tk;
        ++s->n_running;
        if (s->n_running > s->max_concurrent) s->max_concurrent = s->n_running;
    }
}

void pump(nglod_server *s) {
    if (!s->custom) reclaim(s);
    retire(s);
    if (!s->stopped) admit(s);
}

void fill_result(const nglod_server *s, const Ticket *tk, nglod_serve_result *r) {
    *r = nglod_serve_result{};
    r->ticket = tk->id;
    r->kind = tk->req.kind;
    r->status = tk->status;
    r->t_submit = tk->t_submit;
    r->t_admit = tk->t_admit;
    r->t_done = tk->t_done;
    const bool render = tk->req.kind == NGLOD_SERVE_RENDER;
    r->units = render ? (int64_t)tk->req.width * tk->req.height : tk->req.n;
    if (tk->region < 0 || tk->status != NGLOD_OK) return;
    // byte offsets when the pool is not allocated (custom executors)
    char *base = reinterpret_cast<char *>(reinterpret_cast<uintptr_t>(s->pool_base) + (uintptr_t)tk->region);
    if (render) {
        r->x = reinterpret_cast<float *>(base + tk->lay.x);
        r->t = reinterpret_cast<float *>(base + tk->lay.t);
        r->hit = reinterpret_cast<uint8_t *>(base + tk->lay.hit);
        r->normal = reinterpret_cast<float *>(base + tk->lay.normal);
    } else {
        r->sdf = reinterpret_cast<float *>(base + tk->lay.sdf);
    }
}

int start_common(const nglod_serve_config *cfg, nglod_server **out) {
    NGLOD_REQUIRE(cfg && out, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(cfg->num_slots >= 1 && cfg->num_slots <= kMaxSlots, NGLOD_ERR_INVALID,
                  "num_slots=%d outside [1, %d]", cfg->num_slots, kMaxSlots);
    NGLOD_REQUIRE(cfg->hbm_budget_bytes >= kRegionAlign, NGLOD_ERR_INVALID, "hbm_budget_bytes=%lld is too small",
                  (long long)cfg->hbm_budget_bytes);
    *out = nullptr;
    return NGLOD_OK;
}

}  // namespace

extern "C" int64_t nglod_serve_request_bytes(const nglod_serve_request *request) {
    if (!request || !request_valid(*request)) return 0;
    return layout_of(*request).total;
}

extern "C" int nglod_serve_start(const nglod_serve_config *config, nglod_server **server) {
    NGLOD_TRY(start_common(config, server));
    nglod_server *s = new nglod_server();
    s->budget = config->hbm_budget_bytes;
    s->slots = config->num_slots;
    s->running.assign(s->slots, nullptr);
    s->pool.reset(s->budget);
    int st = cuda_status(cudaGetDevice(&s->device), "serve: device");
    if (st == NGLOD_OK) st = cuda_status(cudaMalloc(&s->pool_base, (size_t)s->budget), "serve: pool");
    if (st == NGLOD_OK)
        st = cuda_status(cudaHostAlloc(&s->host_status, sizeof(int32_t) * s->slots, cudaHostAllocDefault),
                         "serve: host status");
    for (int i = 0; st == NGLOD_OK && i < s->slots; ++i) {
        cudaStream_t q = nullptr;
        cudaEvent_t e = nullptr;
        st = cuda_status(cudaStreamCreateWithFlags(&q, cudaStreamNonBlocking), "serve: stream");
        if (st == NGLOD_OK) s->streams.push_back(q);
        if (st == NGLOD_OK) st = cuda_status(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "serve: event");
        if (st == NGLOD_OK) s->done_events.push_back(e);
    }
    if (st != NGLOD_OK) {
        nglod_serve_destroy(s);
        return st;
    }
    *server = s;
    return NGLOD_OK;
}

extern "C" int nglod_serve_start_custom(const nglod_serve_config *config, const nglod_serve_executor *executor,
                                        nglod_server **server) {
    NGLOD_TRY(start_common(config, server));
    NGLOD_REQUIRE(executor && executor->launch && executor->query, NGLOD_ERR_INVALID,
                  "executor needs launch and query callbacks");
    nglod_server *s = new nglod_server();
    s->budget = config->hbm_budget_bytes;
    s->slots = config->num_slots;
    s->running.assign(s->slots, nullptr);
    s->pool.reset(s->budget);
    s->custom = true;
    s->ex = *executor;
    *server = s;
    return NGLOD_OK;
}

extern "C" int nglod_serve_add_model_f32(nglod_server *server, const nglod_dense_model *model, int32_t *model_id) {
    NGLOD_REQUIRE(server && model && model_id, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(model->num_lods >= 1 && model->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID,
                  "num_lods=%d outside [1, %d]", model->num_lods, NGLOD_MAX_LODS);
    std::lock_guard<std::mutex> g(server->mu);
    Model m;
    m.f32 = *model;
    server->models.push_back(m);
    *model_id = (int32_t)server->models.size() - 1;
    return NGLOD_OK;
}

extern "C" int nglod_serve_add_model_bf16(nglod_server *server, const nglod_bf16_model *model, int32_t *model_id) {
    NGLOD_REQUIRE(server && model && model_id, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(model->num_lods >= 1 && model->num_lods <= NGLOD_MAX_LODS, NGLOD_ERR_INVALID,
                  "num_lods=%d outside [1, %d]", model->num_lods, NGLOD_MAX_LODS);
    std::lock_guard<std::mutex> g(server->mu);
    Model m;
    m.bf16 = true;
    m.b16 = *model;
    server->models.push_back(m);
    *model_id = (int32_t)server->models.size() - 1;
    return NGLOD_OK;
}

extern "C" int nglod_serve_submit(nglod_server *server, const nglod_serve_request *request, double t_arrival,
                                  int64_t *ticket) {
    NGLOD_REQUIRE(server && request && ticket, NGLOD_ERR_INVALID, "null pointer argument");
    NGLOD_REQUIRE(request_valid(*request), NGLOD_ERR_INVALID,
                  "invalid request (kind %d, %dx%d, n=%lld, points %s)", request->kind, request->width,
                  request->height, (long long)request->n, request->points ? "set" : "null");
    std::lock_guard<std::mutex> g(server->mu);
    DeviceScope dev(server);
    NGLOD_REQUIRE(!server->stopped, NGLOD_ERR_INVALID, "server is stopped");
    NGLOD_REQUIRE(server->custom || (request->model >= 0 && request->model < (int32_t)server->models.size()),
                  NGLOD_ERR_INVALID, "model id %d not registered (%d models)", request->model,
                  (int)server->models.size());
    const Layout lay = layout_of(*request);
    NGLOD_REQUIRE(lay.total <= server->budget, NGLOD_ERR_CAPACITY,
                  "request needs %lld bytes, more than the whole budget of %lld", (long long)lay.total,
                  (long long)server->budget);
    Ticket *tk = new Ticket();
    tk->id = server->next_id++;
    tk->req = *request;
    tk->lay = lay;
    tk->t_submit = t_arrival >= 0 ? t_arrival : now_s();
    if (!server->custom && request->has_ready_stream) {
        int st = take_event(server, &tk->ready);
        if (st == NGLOD_OK)
            st = cuda_status(cudaEventRecord(tk->ready, reinterpret_cast<cudaStream_t>(request->ready_stream)),
                             "serve: ready event");
        if (st != NGLOD_OK) {
            give_event(server, tk->ready);
            delete tk;
            return st;
        }
    }
    server->pending.push_back(tk);
    ++server->submitted;
    *ticket = tk->id;
    pump(server);
    return NGLOD_OK;
}

extern "C" int nglod_serve_poll(nglod_server *server, nglod_serve_result *results, int32_t max_results,
                                int32_t *count) {
    NGLOD_REQUIRE(server && count && (results || max_results == 0) && max_results >= 0, NGLOD_ERR_INVALID,
                  "null pointer argument");
    std::lock_guard<std::mutex> g(server->mu);
    DeviceScope dev(server);
    pump(server);
    int32_t k = 0;
    while (k < max_results && !server->unpolled.empty()) {
        Ticket *tk = server->unpolled.front();
        server->unpolled.pop_front();
        fill_result(server, tk, &results[k++]);
        server->held[tk->id] = tk;
    }
    *count = k;
    return NGLOD_OK;
}

extern "C" int nglod_serve_release(nglod_server *server, int64_t ticket, int32_t has_stream, nglod_stream_t stream) {
    NGLOD_REQUIRE(server, NGLOD_ERR_INVALID, "null pointer argument");
    std::lock_guard<std::mutex> g(server->mu);
    DeviceScope dev(server);
    auto it = server->held.find(ticket);
    NGLOD_REQUIRE(it != server->held.end(), NGLOD_ERR_INVALID, "ticket %lld is not a polled, unreleased request",
                  (long long)ticket);
    Ticket *tk = it->second;
    server->held.erase(it);
    if (tk->region >= 0) {
        if (!server->custom && has_stream) {
            cudaEvent_t ev = nullptr;
            int st = take_event(server, &ev);
            if (st == NGLOD_OK)
                st = cuda_status(cudaEventRecord(ev, reinterpret_cast<cudaStream_t>(stream)), "serve: release event");
            if (st != NGLOD_OK) {
                // the region cannot be proven idle: keep it out of the pool
                give_event(server, ev);
                delete tk;
                return st;
            }
            server->quarantine.push_back({tk->region, tk->lay.total, ev});
        } else {
            free_region(server, tk->region, tk->lay.total);
        }
    }
    delete tk;
    pump(server);
    return NGLOD_OK;
}

extern "C" int nglod_serve_get_info(nglod_server *server, nglod_serve_info *info) {
    NGLOD_REQUIRE(server && info, NGLOD_ERR_INVALID, "null pointer argument");
    std::lock_guard<std::mutex> g(server->mu);
    info->budget_bytes = server->budget;
    info->used_bytes = server->used;
    info->peak_used_bytes = server->peak;
    info->num_slots = server->slots;
    info->pending = (int32_t)server->pending.size();
    info->running = server->n_running;
    info->unpolled = (int32_t)server->unpolled.size();
    info->held = (int32_t)server->held.size();
    info->max_concurrent = server->max_concurrent;
    info->submitted = server->submitted;
    info->completed = server->completed;
    return NGLOD_OK;
}

extern "C" int nglod_serve_stop(nglod_server *server, double timeout_s, int32_t *unfinished, int32_t *dropped) {
    NGLOD_REQUIRE(server && unfinished && dropped, NGLOD_ERR_INVALID, "null pointer argument");
    const double t0 = now_s();
    {
        std::lock_guard<std::mutex> g(server->mu);
        DeviceScope dev(server);
        server->stopped = true;
        *dropped = (int32_t)server->pending.size();
        for (Ticket *tk : server->pending) {
            give_event(server, tk->ready);
            delete tk;
        }
        server->pending.clear();
    }
    for (;;) {
        {
            std::lock_guard<std::mutex> g(server->mu);
            DeviceScope dev(server);
            pump(server);
            if (server->n_running == 0 || now_s() - t0 >= timeout_s) {
                *unfinished = server->n_running;
                return NGLOD_OK;
            }
        }
        std::this_thread::sleep_for(std::chrono::microseconds(100));
    }
}

extern "C" int nglod_serve_destroy(nglod_server *server) {
    if (!server) return NGLOD_OK;
    int st = NGLOD_OK;
    {
        std::lock_guard<std::mutex> g(server->mu);
        DeviceScope dev(server);
        if (!server->custom) {
            for (cudaStream_t q : server->streams) {
                const int e = cuda_status(cudaStreamSynchronize(q), "serve: stream sync");
                if (st == NGLOD_OK) st = e;
            }
            for (Quarantined &q : server->quarantine) {
                cudaEventSynchronize(q.ev);
                cudaEventDestroy(q.ev);
            }
            for (cudaStream_t q : server->streams) cudaStreamDestroy(q);
            for (cudaEvent_t e : server->done_events) cudaEventDestroy(e);
            for (cudaEvent_t e : server->spare_events) cudaEventDestroy(e);
            for (Ticket *tk : server->pending)
                if (tk->ready) cudaEventDestroy(tk->ready);
            if (server->pool_base) cudaFree(server->pool_base);
            if (server->host_status) cudaFreeHost(server->host_status);
        }
        for (Ticket *tk : server->pending) delete tk;
        for (Ticket *tk : server->running) delete tk;
        for (Ticket *tk : server->unpolled) delete tk;
        for (auto &kv : server->held) delete kv.second;
    }
    delete server;
    return st;
}
