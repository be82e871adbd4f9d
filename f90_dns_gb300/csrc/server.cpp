// Request-serving loop over the C-ABI: continuous batching of independent
// channel runs on one GPU.  No counterpart in the reference (one run per
// process, DNS_pressure_BC_3D.f90:184-428).
//
// A worker thread advances the runs.  Requests wait in FIFO order until their
// device footprint (dns3d_footprint_bytes) fits under the byte budget and a
// slot is free; a second thread then builds each admitted run's handle
// (operators, inverses, tuning) while the running ones go on, and the worker
// takes the built runs in as they come.  Work is queued in chunks of
// `steps_per_round` steps, and every unit gets its next chunk as soon as its
// previous one has completed (dns3d_query / dns3d_batch_query), so runs of
// different sizes do not wait for one another: the small runs with at least
// a full chunk left form a batch (dns3d_batch: every stage of a step is one
// ragged launch over all of them), re-formed only while it is idle and its
// membership has changed; large runs and a run's last, shorter chunk step on
// their own streams beside it.  A finished run's
// diagnostics (and, on request, its final u, v, w, p_total) are kept, and the
// batch and its handle are destroyed at once so its memory admits the next
// request.
//
// Built only on the public entry points of include/dns3d_capi.h.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "dns3d_capi.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    long long id = 0;
    dns3d_config cfg{};
    int nsteps = 0;
    int keep_state = 0;
    int status = DNS3D_REQ_QUEUED;
    int error = DNS3D_OK;
    int steps_done = 0;
    unsigned long long bytes = 0;
    Clock::time_point t_submit, t_start, t_finish;
    dns3d_handle* h = nullptr;
    dns3d_diag diag{};
    std::vector<double> state;  // u, v, w, p_total when keep_state
    int pending = 0;            // steps queued on the run's own stream, not yet counted
    bool in_batch = false;      // a member of the current batch (stepped only through it)
};

// Runs at or above this many grid points keep their own launches in a batch
// (the library's ragged stages take smaller runs only, dns3d_capi.h); the
// server steps them on their own streams, never inside a batch.
constexpr long long kLargeRunPoints = 1LL << 20;

bool large_run(const dns3d_config& c) { return (long long)c.nx * c.ny * c.nz >= kLargeRunPoints; }

double seconds(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double>(b - a).count();
}

}  // namespace

struct dns3d_server {
    dns3d_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Request>> queue;
    std::vector<std::shared_ptr<Request>> active;
    std::map<long long, std::shared_ptr<Request>> all;
    long long next_id = 1;
    bool stop = false;
    unsigned long long bytes_in_use = 0;
    unsigned long long point_steps = 0;
    Clock::time_point t0;
    std::thread worker;
    std::thread builder;
    std::condition_variable cv_build;
    std::deque<std::shared_ptr<Request>> to_build;   // admitted, handle not yet created
    std::vector<std::shared_ptr<Request>> built;     // handle created, not yet running
    int building = 0;                                 // handles being created now
    // worker-thread state: the batch of the runs taking full rounds
    dns3d_batch* batch = nullptr;
    std::vector<dns3d_handle*> batch_runs;
    int batch_pending = 0;  // steps queued on the batch, not yet counted
    bool use_batch = true;  // DNS3D_SERVER_BATCH=0: every run steps on its own stream

    void loop();
    void build_loop();
    void drop_batch();
    void admit_locked();
};

// Admission (under mu): the queue's head while its footprint fits the budget
// and a slot is free; admitted requests go to the builder thread.
void dns3d_server::admit_locked() {
    bool any = false;
    while (!queue.empty() && (int)(active.size() + to_build.size() + built.size()) < opts.max_runs) {
        auto r = queue.front();
        if (bytes_in_use + r->bytes > opts.max_bytes) break;  // FIFO: the head waits for memory
        queue.pop_front();
        bytes_in_use += r->bytes;
        to_build.push_back(r);
        any = true;
    }
    if (any) cv_build.notify_one();
}

// Builder thread: creates the admitted runs' handles one at a time.  A handle
// built after the server began to stop is destroyed and its request cancelled.
void dns3d_server::build_loop() {
    for (;;) {
        std::shared_ptr<Request> r;
        {
            std::unique_lock<std::mutex> lk(mu);
            cv_build.wait(lk, [&] { return stop || !to_build.empty(); });
            if (stop) return;
            r = to_build.front();
            to_build.pop_front();
            ++building;
        }
        dns3d_config c = r->cfg;
        c.device = opts.device;
        dns3d_handle* h = nullptr;
        const int rc = dns3d_create(&c, &h);
        std::lock_guard<std::mutex> lk(mu);
        --building;
        if (rc || stop) {
            if (h) dns3d_destroy(h);
            r->status = DNS3D_REQ_FAILED;
            r->error = rc ? rc : DNS3D_E_CANCELLED;
            r->t_finish = Clock::now();
            bytes_in_use -= r->bytes;
            cv_done.notify_all();
        } else {
            r->h = h;
            r->status = DNS3D_REQ_RUNNING;
            r->t_start = Clock::now();
            built.push_back(r);
        }
        cv_work.notify_all();
    }
}

void dns3d_server::drop_batch() {
    if (batch) {
        if (batch_pending > 0) dns3d_batch_synchronize(batch);
        dns3d_batch_destroy(batch);
    }
    batch = nullptr;
    batch_runs.clear();
    batch_pending = 0;
}

void dns3d_server::loop() {
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(mu);
            // with nothing running, wait for a request or a built run
            cv_work.wait(lk, [&] { return stop || !active.empty() || !queue.empty() || !built.empty(); });
            if (stop) {  // cancel everything: queued, built and running requests end as failed
                for (auto& r : queue) {
                    r->status = DNS3D_REQ_FAILED;
                    r->error = DNS3D_E_CANCELLED;
                }
                queue.clear();
                for (auto& r : to_build) {
                    r->status = DNS3D_REQ_FAILED;
                    r->error = DNS3D_E_CANCELLED;
                    bytes_in_use -= r->bytes;
                }
                to_build.clear();
                drop_batch();
                for (auto* list : {&active, &built}) {
                    for (auto& r : *list) {
                        dns3d_destroy(r->h);
                        r->h = nullptr;
                        r->status = DNS3D_REQ_FAILED;
                        r->error = DNS3D_E_CANCELLED;
                        r->t_finish = Clock::now();
                        bytes_in_use -= r->bytes;
                    }
                    list->clear();
                }
                cv_done.notify_all();
                return;
            }
            admit_locked();
            for (auto& r : built) active.push_back(r);
            built.clear();
            if (active.empty()) {
                // admitted runs are being built: wait for one (or a stop)
                cv_work.wait(lk, [&] { return stop || !built.empty() || (to_build.empty() && building == 0); });
                continue;
            }
        }
        bool progressed = false;
        // (1) count the steps of completed chunks
        if (batch && batch_pending > 0) {
            int fin = 0;
            if (dns3d_batch_query(batch, &fin) != DNS3D_OK) {
                fin = 1;
                for (auto& r : active)
                    if (r->in_batch) r->error = DNS3D_E_CUDA;
            }
            if (fin) {
                for (auto& r : active)
                    if (r->in_batch && !r->error) r->steps_done += batch_pending;
                batch_pending = 0;
                progressed = true;
            }
        }
        for (auto& r : active) {
            if (r->in_batch || r->pending == 0) continue;
            int fin = 0;
            if (dns3d_query(r->h, &fin) != DNS3D_OK) {
                fin = 1;
                r->error = DNS3D_E_CUDA;
            }
            if (fin) {
                if (!r->error) r->steps_done += r->pending;
                r->pending = 0;
                progressed = true;
            }
        }
        // (2) finished runs, once nothing of theirs is in flight
        std::vector<std::shared_ptr<Request>> done;
        for (auto& r : active)
            if ((r->error || r->steps_done >= r->nsteps) && r->pending == 0 && !(r->in_batch && batch_pending > 0))
                done.push_back(r);
        for (auto& r : done)
            if (r->in_batch) {  // the batch is idle here; drop it before its handle goes
                drop_batch();
                for (auto& a : active) a->in_batch = false;
                break;
            }
        for (auto& r : done) {
            if (!r->error) {
                const int rc = dns3d_diagnostics(r->h, &r->diag);
                if (rc && rc != DNS3D_E_NONFINITE) r->error = rc;
                if (!r->error && r->keep_state) {
                    const size_t n = (size_t)r->cfg.nx * r->cfg.ny * r->cfg.nz;
                    r->state.resize(4 * n);
                    const int rs = dns3d_get_state(r->h, r->state.data(), r->state.data() + n, r->state.data() + 2 * n,
                                                   r->state.data() + 3 * n, nullptr, nullptr, nullptr, nullptr, nullptr);
                    if (rs) r->error = rs;
                }
            }
            dns3d_destroy(r->h);
            r->h = nullptr;
            std::lock_guard<std::mutex> lk(mu);
            r->t_finish = Clock::now();
            r->status = r->error ? DNS3D_REQ_FAILED : DNS3D_REQ_DONE;
            bytes_in_use -= r->bytes;
            point_steps += (unsigned long long)r->steps_done * r->cfg.nx * r->cfg.ny * r->cfg.nz;
            active.erase(std::find(active.begin(), active.end(), r));
            cv_done.notify_all();
            progressed = true;
        }
        // (3) the batch, while idle: re-form it if its membership changed, and
        // queue its next chunk
        const int spr = opts.steps_per_round;
        if (batch_pending == 0) {
            std::vector<dns3d_handle*> full;
            if (use_batch)
                for (auto& r : active)
                    if (!r->error && !large_run(r->cfg) && r->pending == 0 && r->nsteps - r->steps_done >= spr)
                        full.push_back(r->h);
            if (full.size() < 2) full.clear();
            if (full != batch_runs) {
                drop_batch();
                for (auto& r : active) r->in_batch = false;
                if (!full.empty() && dns3d_batch_create(full.data(), (int)full.size(), 0, &batch) == DNS3D_OK) {
                    batch_runs = full;
                    for (auto& r : active)
                        r->in_batch = std::find(full.begin(), full.end(), r->h) != full.end();
                } else {
                    batch = nullptr;  // the runs step on their own streams instead
                }
            }
            if (batch) {
                if (dns3d_batch_step(batch, spr) == DNS3D_OK) {
                    batch_pending = spr;
                } else {
                    for (auto& r : active)
                        if (r->in_batch) r->error = DNS3D_E_CUDA;
                }
                progressed = true;
            }
        }
        // (4) every idle run outside the batch gets its next chunk
        for (auto& r : active) {
            if (r->in_batch || r->pending > 0 || r->error) continue;
            const int k = std::min(spr, r->nsteps - r->steps_done);
            if (k <= 0) continue;
            if (dns3d_step(r->h, k) == DNS3D_OK) r->pending = k;
            else r->error = DNS3D_E_CUDA;
            progressed = true;
        }
        // (5) all units busy: wait a little (or for a new request or built run)
        if (!progressed) {
            std::unique_lock<std::mutex> lk(mu);
            cv_work.wait_for(lk, std::chrono::microseconds(200), [&] { return stop || !built.empty(); });
        }
    }
}

namespace {

void fill_info(const Request& r, const Clock::time_point t0, dns3d_request_info* info) {
    std::memset(info, 0, sizeof(*info));
    info->status = r.status;
    info->error = r.error;
    info->steps_done = r.steps_done;
    info->nsteps = r.nsteps;
    info->bytes = r.bytes;
    info->t_submit = seconds(t0, r.t_submit);
    info->t_start = r.status >= DNS3D_REQ_RUNNING || r.t_start != Clock::time_point() ? seconds(t0, r.t_start) : -1.0;
    info->t_finish = (r.status == DNS3D_REQ_DONE || r.status == DNS3D_REQ_FAILED) ? seconds(t0, r.t_finish) : -1.0;
    info->diag = r.diag;
}

}  // namespace

extern "C" {

int dns3d_server_opts_defaults(dns3d_server_opts* o) {
    if (!o) return DNS3D_E_INVALID;
    std::memset(o, 0, sizeof(*o));
    o->max_bytes = 160ull << 30;
    o->max_runs = 256;
    o->steps_per_round = 10;
    o->device = 0;
    return DNS3D_OK;
}

int dns3d_server_create(const dns3d_server_opts* opts, dns3d_server** out) {
    if (!opts || !out || opts->max_runs < 1 || opts->steps_per_round < 1 || opts->max_bytes == 0)
        return DNS3D_E_INVALID;
    auto* s = new dns3d_server();
    s->opts = *opts;
    s->t0 = Clock::now();
    const char* env = std::getenv("DNS3D_SERVER_BATCH");
    s->use_batch = !(env && std::strcmp(env, "0") == 0);
    s->worker = std::thread([s] { s->loop(); });
    s->builder = std::thread([s] { s->build_loop(); });
    *out = s;
    return DNS3D_OK;
}

int dns3d_server_submit(dns3d_server* s, const dns3d_config* cfg, int nsteps, int keep_state, long long* id) {
    if (!s || !cfg || nsteps < 1 || !id) return DNS3D_E_INVALID;
    auto r = std::make_shared<Request>();
    r->cfg = *cfg;
    r->nsteps = nsteps;
    r->keep_state = keep_state;
    const int rc = dns3d_footprint_bytes(cfg, &r->bytes);
    if (rc) return rc;
    if (r->bytes > s->opts.max_bytes) return DNS3D_E_OOM;  // could never be admitted
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return DNS3D_E_INVALID;
    r->id = s->next_id++;
    r->t_submit = Clock::now();
    s->queue.push_back(r);
    s->all[r->id] = r;
    *id = r->id;
    s->cv_work.notify_one();
    return DNS3D_OK;
}

int dns3d_server_poll(dns3d_server* s, long long id, dns3d_request_info* info) {
    if (!s || !info) return DNS3D_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return DNS3D_E_INVALID;
    fill_info(*it->second, s->t0, info);
    return DNS3D_OK;
}

int dns3d_server_wait(dns3d_server* s, long long id, double timeout_s, dns3d_request_info* info) {
    if (!s || !info) return DNS3D_E_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return DNS3D_E_INVALID;
    auto r = it->second;
    const auto pred = [&] { return r->status == DNS3D_REQ_DONE || r->status == DNS3D_REQ_FAILED; };
    if (timeout_s < 0) s->cv_done.wait(lk, pred);
    else s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    fill_info(*r, s->t0, info);
    return pred() ? DNS3D_OK : DNS3D_E_TIMEOUT;
}

int dns3d_server_result_state(dns3d_server* s, long long id, double* u, double* v, double* w, double* p_total) {
    if (!s) return DNS3D_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return DNS3D_E_INVALID;
    const Request& r = *it->second;
    if (r.status != DNS3D_REQ_DONE || r.state.empty()) return DNS3D_E_INVALID;
    const size_t n = (size_t)r.cfg.nx * r.cfg.ny * r.cfg.nz;
    double* dst[4] = {u, v, w, p_total};
    for (int f = 0; f < 4; ++f)
        if (dst[f]) std::memcpy(dst[f], r.state.data() + f * n, n * sizeof(double));
    return DNS3D_OK;
}

int dns3d_server_release(dns3d_server* s, long long id) {
    if (!s) return DNS3D_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(id);
    if (it == s->all.end()) return DNS3D_E_INVALID;
    if (it->second->status != DNS3D_REQ_DONE && it->second->status != DNS3D_REQ_FAILED) return DNS3D_E_INVALID;
    s->all.erase(it);
    return DNS3D_OK;
}

int dns3d_server_get_stats(dns3d_server* s, dns3d_server_stats* st) {
    if (!s || !st) return DNS3D_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(st, 0, sizeof(*st));
    st->queued = (int)s->queue.size();
    st->running = (int)s->active.size();
    st->bytes_in_use = s->bytes_in_use;
    st->point_steps_done = s->point_steps;
    st->uptime_s = seconds(s->t0, Clock::now());
    return DNS3D_OK;
}

int dns3d_server_destroy(dns3d_server* s) {
    if (!s) return DNS3D_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_work.notify_all();
        s->cv_build.notify_all();
    }
    if (s->builder.joinable()) s->builder.join();
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return DNS3D_OK;
}

}  // extern "C"
