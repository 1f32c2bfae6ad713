// Serving loop: continuous batching of render / LiDAR / SRP requests over resident scenes.
//
// Each lane owns a context (stream, scratch, counters, error word), a wave engine and a host
// thread.  Between waves a lane admits queued requests in arrival order while their per-request
// state (pixel accumulators, staging, LiDAR tables) fits the engine's free memory, runs the SRP
// queries, then runs one wave over everything resident; a request leaves as soon as its last wave
// has run.  Requests that arrive while others are on the GPU therefore join the next wave, and
// with two or more lanes one lane plans and launches while the other's wave is on the GPU.
#include "common.cuh"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>
#include <unordered_set>

namespace {

double now_s() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Pending {
    uint64_t ticket = 0;
    crt_request req;                      // pointers below point into this record
    crt_camera_desc camera;
    crt_light_desc lights[16];
    crt_render_params params;
    crt_lidar_grid_desc lidar;
    bool srp = false;
    crt_srp_desc srp_desc;
    std::vector<double> quats;
    double* force = nullptr;
    double* torque = nullptr;
    double submit_s = 0;
    void fix_pointers() {
        req.camera = &camera;
        req.lights = lights;
        req.params = &params;
        req.lidar = &lidar;
    }
};

}  // namespace

struct crt_server {
    int device = 0;
    crt_server_config cfg;
    std::vector<crt_context*> lanes;
    std::vector<WaveEngine*> engines;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Pending*> queue;
    std::unordered_map<uint64_t, crt_server_result> done;
    std::unordered_set<uint64_t> outstanding;   // issued and not yet collected by crt_server_wait
    uint64_t next_ticket = 1;
    bool stop = false;
    crt_server_stats stats;
};

namespace {

void publish(crt_server* S, Pending* p, int status, double start_s, double end_s, uint32_t batch_size) {
    crt_server_result r;
    r.status = status;
    r.submit_s = p->submit_s;
    r.start_s = start_s;
    r.end_s = end_s;
    r.batch_size = batch_size;
    S->done[p->ticket] = r;
    S->stats.completed++;
    if (status != CRT_OK) S->stats.failed++;
    delete p;
}

// One lane: admits queued requests (renders, LiDAR scans, SRP queries) into its wave engine whenever
// their state fits (FIFO), and runs one wave per iteration; an SRP query's sun rays ride in the waves'
// primary traces, one range per wave.  Requests leave when their last wave is done.
void lane_loop(crt_server* S, size_t lane) {
    crt_context* ctx = S->lanes[lane];
    WaveEngine* E = S->engines[lane];
    cudaSetDevice(S->device);
    std::unordered_map<uint64_t, std::pair<Pending*, double>> resident;   // tag -> (request, admitted at)
    std::vector<uint64_t> finished;
    while (true) {
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty() || !resident.empty(); });
            if (S->stop && S->queue.empty() && resident.empty()) return;
            const double now = now_s();
            while (!S->queue.empty() && resident.size() < S->cfg.max_batch) {
                Pending* p = S->queue.front();
                bool ok = false;
                const int rc = crt_guard(ctx, [&] {
                    ok = p->srp ? engine_admit_srp(E, p->req.scene, p->srp_desc, p->quats.data(), p->quats.size() / 4,
                                                   p->force, p->torque, p->ticket)
                                : engine_admit(E, p->req, p->ticket);
                });
                if (rc != CRT_OK) {   // a CUDA failure, or an attitude quaternion of zero length
                    S->queue.pop_front();
                    publish(S, p, rc, now, now_s(), 0);
                    continue;
                }
                if (!ok) break;       // head of the queue waits for memory (FIFO admission)
                S->queue.pop_front();
                resident[p->ticket] = {p, now};
            }
        }
        S->cv_done.notify_all();
        crt_counters c0{}, c1{};
        if (S->cfg.count_rays) crt_context_get_counters(ctx, &c0);
        if (resident.empty()) continue;
        const double t0 = now_s();
        const size_t sharing = resident.size();
        finished.clear();
        std::vector<uint64_t> dropped;
        const int rc = crt_guard(ctx, [&] { engine_step(E, finished); });
        if (rc != CRT_OK) engine_abort(E, dropped);
        const double t1 = now_s();
        if (S->cfg.count_rays) crt_context_get_counters(ctx, &c1);
        {
            std::lock_guard<std::mutex> lk(S->mu);
            for (int pass = 0; pass < 2; ++pass) {
                for (uint64_t tag : pass ? dropped : finished) {
                    auto it = resident.find(tag);
                    if (it == resident.end()) continue;
                    publish(S, it->second.first, pass ? rc : CRT_OK, it->second.second, t1, (uint32_t)sharing);
                    resident.erase(it);
                }
            }
            S->stats.batches++;
            S->stats.busy_s += t1 - t0;
            if (S->cfg.count_rays) S->stats.rays += (c1.rays + c1.resolved) - (c0.rays + c0.resolved);
        }
        S->cv_done.notify_all();
    }
}

thread_local std::string t_submit_error;

// crt_guard for the submitting thread: the message goes to a per-thread string, not to a lane's
// context, whose thread may be writing its own error at the same time.
template <class F>
int submit_guard(F&& f) {
    try {
        f();
        return CRT_OK;
    } catch (const CrtError& e) {
        t_submit_error = e.msg;
        return e.status;
    } catch (const std::bad_alloc&) {
        t_submit_error = "host allocation failed";
        return CRT_ERR_OOM;
    } catch (const std::exception& e) {
        t_submit_error = e.what();
        return CRT_ERR_INVALID;
    }
}


}  // namespace

extern "C" {

int crt_server_create(int device, const crt_server_config* cfg, crt_server** out) {
    if (!out) return CRT_ERR_INVALID;
    *out = nullptr;
    crt_server_config c = cfg ? *cfg : crt_server_config{2, (size_t)4 << 30, 256, 0, 0};
    if (c.wave_paths == 0) c.wave_paths = 1u << 22;
    if (c.lanes < 1 || c.lanes > 8 || c.max_batch < 1 || c.wave_paths < (1u << 16)) return CRT_ERR_INVALID;
    crt_server* S = new crt_server();
    S->device = device;
    S->cfg = c;
    std::memset(&S->stats, 0, sizeof(S->stats));
    auto unwind = [&](int rc) {
        for (WaveEngine* e : S->engines) engine_destroy(e);
        for (crt_context* x : S->lanes) crt_context_destroy(x);
        delete S;
        return rc;
    };
    for (uint32_t l = 0; l < c.lanes; ++l) {
        crt_context* ctx = nullptr;
        int rc = crt_context_create(device, &ctx);
        if (rc != CRT_OK) return unwind(rc);
        S->lanes.push_back(ctx);
        ctx->wave_paths = c.wave_paths;
        if (c.count_rays) crt_context_set_counting(ctx, 1);   // per-wave ray counts
        WaveEngine* e = nullptr;
        rc = crt_guard(ctx, [&] { e = engine_create(ctx, c.lane_budget_bytes); });
        if (rc != CRT_OK) return unwind(rc);
        S->engines.push_back(e);
    }
    for (uint32_t l = 0; l < c.lanes; ++l) S->threads.emplace_back(lane_loop, S, (size_t)l);
    *out = S;
    return CRT_OK;
}

int crt_server_destroy(crt_server* S) {
    if (!S) return CRT_OK;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (std::thread& t : S->threads) t.join();
    for (WaveEngine* e : S->engines) engine_destroy(e);
    for (crt_context* c : S->lanes) crt_context_destroy(c);
    delete S;
    return CRT_OK;
}

const char* crt_server_last_error(void) { return t_submit_error.c_str(); }

int crt_server_submit(crt_server* S, const crt_server_request* r, uint64_t* ticket) {
    if (!S || !r || !ticket) return CRT_ERR_INVALID;
    Pending* p = new (std::nothrow) Pending();
    if (!p) return CRT_ERR_OOM;
    int rc = submit_guard([&] {
        const crt_request& q = r->base;
        CRT_CHECK(q.scene && q.scene->ctx && q.scene->ctx->device == S->device, CRT_ERR_INVALID,
                  "request scene must live on the server's device");
        std::memset(&p->req, 0, sizeof(p->req));
        p->req = q;
        if (q.kind == CRT_REQUEST_SRP) {
            CRT_CHECK(r->srp && r->quaternions && r->force && r->torque, CRT_ERR_INVALID, "incomplete SRP request");
            CRT_CHECK(r->n_att > 0 && r->n_att <= (1u << 20), CRT_ERR_INVALID, "bad attitude count");
            CRT_CHECK(r->srp->grid > 0 && r->srp->grid <= 32768, CRT_ERR_INVALID, "grid must be in [1, 32768]");
            p->srp = true;
            p->srp_desc = *r->srp;
            p->quats.assign(r->quaternions, r->quaternions + 4 * r->n_att);
            p->force = r->force;
            p->torque = r->torque;
        } else {
            batch_check_request(q);
            if (q.kind == CRT_REQUEST_RENDER) {
                p->camera = *q.camera;
                CRT_CHECK(q.n_lights <= 16, CRT_ERR_INVALID, "at most 16 lights per render");
                for (uint32_t l = 0; l < q.n_lights; ++l) p->lights[l] = q.lights[l];
                p->params = *q.params;
            } else {
                p->lidar = *q.lidar;
            }
            p->fix_pointers();
        }
    });
    if (rc != CRT_OK) {
        delete p;
        return rc;
    }
    {
        std::lock_guard<std::mutex> lk(S->mu);
        p->ticket = S->next_ticket++;
        p->submit_s = now_s();
        *ticket = p->ticket;
        S->outstanding.insert(p->ticket);
        S->queue.push_back(p);
        S->stats.submitted++;
    }
    S->cv_work.notify_one();
    return CRT_OK;
}

int crt_server_wait(crt_server* S, uint64_t ticket, double timeout_s, crt_server_result* out) {
    if (!S || !out) return CRT_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    if (!S->outstanding.count(ticket)) return CRT_ERR_INVALID;   // never issued, or already collected
    // ready also when another thread collected the ticket meanwhile (it notifies cv_done)
    auto ready = [&] { return S->done.count(ticket) != 0 || !S->outstanding.count(ticket); };
    if (timeout_s < 0) S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return CRT_ERR_TIMEOUT;
    auto it = S->done.find(ticket);
    if (it == S->done.end()) return CRT_ERR_INVALID;
    *out = it->second;
    S->done.erase(it);
    S->outstanding.erase(ticket);
    lk.unlock();
    S->cv_done.notify_all();
    return CRT_OK;
}

int crt_server_get_stats(crt_server* S, crt_server_stats* out) {
    if (!S || !out) return CRT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
    return CRT_OK;
}

}  // extern "C"
