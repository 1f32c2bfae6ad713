// Serving loop: continuous batching of render / LiDAR / SRP requests over resident scenes.
//
// Each lane owns a context (stream, scratch, counters, error word) and a host thread.  A lane takes
// the oldest queued requests while their estimated device footprint fits its budget (a request
// larger than the budget runs alone), runs the render and LiDAR requests as one crt_batch and the
// SRP requests one by one, then publishes per-request timings.  With two or more lanes, a batch is
// formed and launched while the previous one is still on the GPU, so their work overlaps.
#include "common.cuh"

#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <thread>
#include <unordered_map>

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
    size_t footprint = 0;
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
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Pending*> queue;
    std::unordered_map<uint64_t, crt_server_result> done;
    uint64_t next_ticket = 1;
    bool stop = false;
    crt_server_stats stats;
};

namespace {

void lane_loop(crt_server* S, size_t lane) {
    crt_context* ctx = S->lanes[lane];
    cudaSetDevice(S->device);
    while (true) {
        std::vector<Pending*> batch;
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] { return S->stop || !S->queue.empty(); });
            if (S->queue.empty()) return;   // stopping and drained
            size_t used = 0;
            while (!S->queue.empty() && batch.size() < S->cfg.max_batch) {
                Pending* p = S->queue.front();
                if (!batch.empty() && used + p->footprint > S->cfg.lane_budget_bytes) break;
                used += p->footprint;
                batch.push_back(p);
                S->queue.pop_front();
            }
        }
        const double t0 = now_s();
        int status = CRT_OK;
        std::vector<int> srp_status(batch.size(), CRT_OK);
        uint64_t rays = 0;
        {
            std::vector<crt_request> reqs;
            for (Pending* p : batch)
                if (!p->srp) reqs.push_back(p->req);
            crt_counters c0{}, c1{};
            crt_context_get_counters(ctx, &c0);
            if (!reqs.empty())
                status = crt_guard(ctx, [&] { batch_run(ctx, reqs.data(), reqs.size(), nullptr); });
            for (size_t k = 0; k < batch.size(); ++k) {
                Pending* p = batch[k];
                if (!p->srp) continue;
                srp_status[k] = crt_guard(ctx, [&] {
                    srp_run(ctx, p->req.scene, &p->srp_desc, p->quats.data(), p->quats.size() / 4, p->force,
                            p->torque, nullptr);
                });
            }
            const int sync = crt_context_synchronize(ctx);
            if (status == CRT_OK) status = sync;
            crt_context_get_counters(ctx, &c1);
            rays = c1.rays - c0.rays;
        }
        const double t1 = now_s();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            for (size_t k = 0; k < batch.size(); ++k) {
                Pending* p = batch[k];
                crt_server_result r;
                r.status = p->srp ? srp_status[k] : status;
                r.submit_s = p->submit_s;
                r.start_s = t0;
                r.end_s = t1;
                r.batch_size = (uint32_t)batch.size();
                S->done[p->ticket] = r;
                S->stats.completed++;
                if (r.status != CRT_OK) S->stats.failed++;
                delete p;
            }
            S->stats.batches++;
            S->stats.rays += rays;
            S->stats.busy_s += t1 - t0;
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

size_t srp_footprint(const crt_srp_desc& d, size_t n_att) {
    const size_t tiles = ((size_t)(d.grid + 7) / 8) * ((d.grid + 3) / 4);
    return (tiles / 16 + 1) * 48 * std::max<size_t>(n_att, 1) + n_att * 112;
}

}  // namespace

extern "C" {

int crt_server_create(int device, const crt_server_config* cfg, crt_server** out) {
    if (!out) return CRT_ERR_INVALID;
    *out = nullptr;
    crt_server_config c = cfg ? *cfg : crt_server_config{2, (size_t)4 << 30, 64};
    if (c.lanes < 1 || c.lanes > 8 || c.max_batch < 1) return CRT_ERR_INVALID;
    crt_server* S = new crt_server();
    S->device = device;
    S->cfg = c;
    std::memset(&S->stats, 0, sizeof(S->stats));
    for (uint32_t l = 0; l < c.lanes; ++l) {
        crt_context* ctx = nullptr;
        int rc = crt_context_create(device, &ctx);
        if (rc != CRT_OK) {
            for (crt_context* x : S->lanes) crt_context_destroy(x);
            delete S;
            return rc;
        }
        crt_context_set_counting(ctx, 1);   // per-batch ray counts (a few integer adds per node visit)
        S->lanes.push_back(ctx);
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
    for (crt_context* c : S->lanes) crt_context_destroy(c);
    delete S;
    return CRT_OK;
}

const char* crt_server_last_error(void) { return t_submit_error.c_str(); }

int crt_server_submit(crt_server* S, const crt_server_request* r, uint64_t* ticket) {
    if (!S || !r || !ticket) return CRT_ERR_INVALID;
    Pending* p = new (std::nothrow) Pending();
    if (!p) return CRT_ERR_OOM;
    const uint32_t wave_paths = S->lanes[0]->wave_paths;
    int rc = submit_guard([&] {
        const crt_request& q = r->base;
        CRT_CHECK(q.scene && q.scene->ctx && q.scene->ctx->device == S->device, CRT_ERR_INVALID,
                  "request scene must live on the server's device");
        std::memset(&p->req, 0, sizeof(p->req));
        p->req = q;
        if (q.kind == CRT_REQUEST_SRP) {
            CRT_CHECK(r->srp && r->quaternions && r->force && r->torque, CRT_ERR_INVALID, "incomplete SRP request");
            CRT_CHECK(r->n_att > 0 && r->n_att <= (1u << 20), CRT_ERR_INVALID, "bad attitude count");
            CRT_CHECK(r->srp->grid > 0 && r->srp->grid <= 65536, CRT_ERR_INVALID, "grid must be in [1, 65536]");
            p->srp = true;
            p->srp_desc = *r->srp;
            p->quats.assign(r->quaternions, r->quaternions + 4 * r->n_att);
            p->force = r->force;
            p->torque = r->torque;
            p->footprint = srp_footprint(p->srp_desc, r->n_att);
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
            p->footprint = batch_footprint(p->req, wave_paths);
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
        S->queue.push_back(p);
        S->stats.submitted++;
    }
    S->cv_work.notify_one();
    return CRT_OK;
}

int crt_server_wait(crt_server* S, uint64_t ticket, double timeout_s, crt_server_result* out) {
    if (!S || !out) return CRT_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    auto ready = [&] { return S->done.count(ticket) != 0; };
    if (timeout_s < 0) S->cv_done.wait(lk, ready);
    else if (!S->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) return CRT_ERR_TIMEOUT;
    *out = S->done[ticket];
    S->done.erase(ticket);
    return CRT_OK;
}

int crt_server_get_stats(crt_server* S, crt_server_stats* out) {
    if (!S || !out) return CRT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(S->mu);
    *out = S->stats;
    return CRT_OK;
}

}  // extern "C"
