// The solve server (plb_server_*, include/plb.h): continuous batching of
// independent lattice-Boltzmann solves on one GPU.
//
// One scheduler thread owns every CUDA call.  Each loop it
//   1. admits queued requests in arrival order while their device bytes fit
//      the budget (a request larger than the whole budget fails),
//   2. advances every class of running solves (same lattice, storage and
//      arithmetic) by one tick -- min(tick_steps, fewest steps left in the
//      class) -- as one batch, all classes enqueued before any is waited for,
//   3. retires solves that have run all their steps: rho and u are copied to
//      host memory, the solve is destroyed, its bytes return to the budget.
// Clients submit from any thread and wait on a condition variable.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <tuple>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/plb.h"

namespace plb {
void record_error(const std::string& msg);   // capi.cu: the plb_last_error() slot
}

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    int64_t id = 0;
    plb_params p{};
    std::vector<uint8_t> mask;
    int64_t steps = 0, remaining = 0;
    int state = PLB_REQ_QUEUED;
    double t_sub = 0, t_adm = 0, t_done = 0;
    int64_t bytes = 0;
    plb_solve* s = nullptr;
    std::vector<float> rho, u;
    std::string err;
};

struct Class {
    std::vector<Req*> members;
    plb_batch* batch = nullptr;
    bool dirty = true;
};

using ClassKey = std::tuple<int, int, int>;   // q, storage, arith

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

}  // namespace

struct plb_server {
    int device = 0;
    int64_t budget = 0, used = 0, peak = 0;
    int tick = 100;
    Clock::time_point t0;
    std::thread th;
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    bool stop = false;
    std::deque<Req*> pending;
    std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
    int64_t next_id = 1;
    std::map<ClassKey, Class> classes;   // scheduler thread only

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
};

namespace {

void finish(plb_server* srv, Req* r, int state, const std::string& err) {
    std::lock_guard<std::mutex> lk(srv->mu);
    r->state = state;
    r->err = err;
    r->t_done = srv->now();
    if (r->bytes) {
        srv->used -= r->bytes;
        r->bytes = 0;
    }
    srv->done_cv.notify_all();
}

// Creates the request's solve (scheduler thread).  Returns an error message or "".
std::string start_solve(Req* r) {
    plb_solve* s = nullptr;
    if (plb_solve_create(&r->p, &s) != PLB_OK) return plb_last_error();
    if (!r->mask.empty() && plb_set_mask(s, r->mask.data()) != PLB_OK) {
        std::string e = plb_last_error();
        plb_solve_destroy(s);
        return e;
    }
    if (plb_initialize(s) != PLB_OK) {
        std::string e = plb_last_error();
        plb_solve_destroy(s);
        return e;
    }
    r->s = s;
    return "";
}

void retire(plb_server* srv, Req* r) {
    std::string err;
    r->rho.resize(plb_field_len(r->s, PLB_FIELD_RHO));
    r->u.resize(plb_field_len(r->s, PLB_FIELD_U));
    if (plb_get_field(r->s, PLB_FIELD_RHO, r->rho.data()) != PLB_OK ||
        plb_get_field(r->s, PLB_FIELD_U, r->u.data()) != PLB_OK)
        err = plb_last_error();
    plb_solve_destroy(r->s);
    r->s = nullptr;
    finish(srv, r, err.empty() ? PLB_REQ_DONE : PLB_REQ_FAILED, err);
}

void scheduler(plb_server* srv) {
    cudaSetDevice(srv->device);
    for (;;) {
        // 1. admission
        std::vector<Req*> admitted;
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            bool running = false;
            for (auto& kv : srv->classes) running |= !kv.second.members.empty();
            if (!running)
                srv->work_cv.wait(lk, [&] { return srv->stop || !srv->pending.empty(); });
            if (srv->stop) break;
            while (!srv->pending.empty()) {
                Req* r = srv->pending.front();
                const int64_t need = plb_solve_bytes(&r->p);
                if (need > srv->budget) {
                    srv->pending.pop_front();
                    r->state = PLB_REQ_FAILED;
                    r->err = "request needs more device memory than the whole budget";
                    r->t_done = srv->now();
                    srv->done_cv.notify_all();
                    continue;
                }
                if (srv->used + need > srv->budget) break;   // wait for room, keep arrival order
                srv->pending.pop_front();
                srv->used += need;
                if (srv->used > srv->peak) srv->peak = srv->used;
                r->bytes = need;
                r->state = PLB_REQ_RUNNING;
                r->t_adm = srv->now();
                admitted.push_back(r);
            }
        }
        for (Req* r : admitted) {
            const std::string e = start_solve(r);
            if (!e.empty()) {
                finish(srv, r, PLB_REQ_FAILED, e);
                continue;
            }
            Class& c = srv->classes[ClassKey(r->p.q, r->p.storage, r->p.arith)];
            c.members.push_back(r);
            c.dirty = true;
        }
        // 2. one tick for every class
        std::vector<std::pair<Class*, int64_t>> ticking;
        for (auto& kv : srv->classes) {
            Class& c = kv.second;
            if (c.members.empty()) continue;
            if (c.dirty) {
                if (c.batch) plb_batch_destroy(c.batch);
                c.batch = nullptr;
                std::vector<plb_solve*> ss;
                for (Req* r : c.members) ss.push_back(r->s);
                if (plb_batch_create((int32_t)ss.size(), ss.data(), &c.batch) != PLB_OK) {
                    const std::string e = plb_last_error();
                    for (Req* r : c.members) {
                        plb_solve_destroy(r->s);
                        r->s = nullptr;
                        finish(srv, r, PLB_REQ_FAILED, e);
                    }
                    c.members.clear();
                    continue;
                }
                c.dirty = false;
            }
            int64_t t = srv->tick;
            for (Req* r : c.members) t = r->remaining < t ? r->remaining : t;
            if (t < 1) t = 1;
            if (plb_batch_step_async(c.batch, t) != PLB_OK) {
                const std::string e = plb_last_error();
                for (Req* r : c.members) {
                    plb_solve_destroy(r->s);
                    r->s = nullptr;
                    finish(srv, r, PLB_REQ_FAILED, e);
                }
                c.members.clear();
                plb_batch_destroy(c.batch);
                c.batch = nullptr;
                continue;
            }
            ticking.emplace_back(&c, t);
        }
        // 3. retire
        for (auto& ct : ticking) {
            Class& c = *ct.first;
            plb_batch_synchronize(c.batch);
            std::vector<Req*> keep;
            for (Req* r : c.members) {
                r->remaining -= ct.second;
                if (r->remaining <= 0) {
                    retire(srv, r);
                    c.dirty = true;
                } else {
                    keep.push_back(r);
                }
            }
            c.members.swap(keep);
            if (c.members.empty() && c.batch) {
                plb_batch_destroy(c.batch);
                c.batch = nullptr;
            }
        }
    }
    // stop: drop everything
    for (auto& kv : srv->classes) {
        if (kv.second.batch) plb_batch_destroy(kv.second.batch);
        for (Req* r : kv.second.members)
            if (r->s) plb_solve_destroy(r->s);
    }
    srv->classes.clear();
}

}  // namespace

extern "C" {

int64_t plb_solve_bytes(const plb_params* p) {
    if (!p) return 0;
    const long long esize = p->storage == PLB_STORAGE_FP16_DEV ? 2 : p->storage == PLB_STORAGE_FP64 ? 8 : 4;
    long long ks, cells_box;
    const long long cells = (long long)p->nx * p->ny * p->nz;
    if (p->semantics == PLB_SEMANTICS_NATIVE) {
        const long long ys = round_up(p->nx, 32 / esize);
        ks = round_up(ys * p->ny * p->nz, 128);
    } else {
        const long long ys = round_up(8 + p->nx + 1, 8);
        ks = round_up(ys * (p->ny + 2) * (p->nz + 2), 64);
    }
    cells_box = (long long)(p->nx + 2) * (p->ny + 2) * (p->nz + 2);
    long long b = 2LL * p->q * ks * esize;        // two population buffers
    b += 4LL * ks * 4;                            // rho, u
    b += 2LL * 27 * 4 + 1024LL * 4 * 8 + 4 * 8;   // constants, reduction partials
    if (p->semantics == PLB_SEMANTICS_NATIVE) b += 2LL * ks + 4LL * ks + cells;   // types, links, mask
    b += 3LL * cells_box * 4;                     // transfer buffer for reading u back
    return (int64_t)b;
}

int plb_server_start(int32_t device, int64_t budget_bytes, int32_t tick_steps, plb_server** out) {
    if (!out || budget_bytes <= 0) return -1;
    plb_server* srv = new plb_server();
    srv->device = device;
    srv->budget = budget_bytes;
    srv->tick = tick_steps > 0 ? tick_steps : 100;
    srv->t0 = Clock::now();
    srv->th = std::thread(scheduler, srv);
    *out = srv;
    return PLB_OK;
}

int plb_server_submit(plb_server* srv, const plb_request* req, int64_t* id) {
    if (!srv || !req || !id) return PLB_EINVAL;
    if (req->params.semantics != PLB_SEMANTICS_NATIVE || req->steps < 1) {
        plb::record_error("served requests need NATIVE semantics and at least one step");
        return PLB_EINVAL;
    }
    auto r = std::make_unique<Req>();
    r->p = req->params;
    r->steps = r->remaining = req->steps;
    if (req->mask) r->mask.assign(req->mask, req->mask + req->params.nx * req->params.ny * req->params.nz);
    std::lock_guard<std::mutex> lk(srv->mu);
    r->id = srv->next_id++;
    r->t_sub = srv->now();
    *id = r->id;
    srv->pending.push_back(r.get());
    srv->reqs[r->id] = std::move(r);
    srv->work_cv.notify_all();
    return PLB_OK;
}

int plb_server_status(plb_server* srv, int64_t id, int32_t* state) {
    if (!srv || !state) return PLB_EINVAL;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return PLB_EINVAL;
    *state = it->second->state;
    return PLB_OK;
}

int plb_server_wait(plb_server* srv, int64_t id, double timeout_s) {
    if (!srv) return PLB_EINVAL;
    std::unique_lock<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return PLB_EINVAL;
    Req* r = it->second.get();
    const bool ok = srv->done_cv.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] {
        return r->state == PLB_REQ_DONE || r->state == PLB_REQ_FAILED;
    });
    if (!ok) return PLB_ETIMEOUT;
    if (r->state == PLB_REQ_FAILED) {
        plb::record_error(r->err);
        return PLB_ECUDA;
    }
    return PLB_OK;
}

int plb_server_result(plb_server* srv, int64_t id, float* rho, float* u, double* times3) {
    if (!srv) return PLB_EINVAL;
    std::unique_ptr<Req> r;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        auto it = srv->reqs.find(id);
        if (it == srv->reqs.end()) return PLB_EINVAL;
        if (it->second->state == PLB_REQ_FAILED) {
            plb::record_error(it->second->err);
            srv->reqs.erase(it);
            return PLB_ECUDA;
        }
        if (it->second->state != PLB_REQ_DONE) return PLB_ESTATE;
        r = std::move(it->second);
        srv->reqs.erase(it);
    }
    if (rho) std::memcpy(rho, r->rho.data(), r->rho.size() * sizeof(float));
    if (u) std::memcpy(u, r->u.data(), r->u.size() * sizeof(float));
    if (times3) { times3[0] = r->t_sub; times3[1] = r->t_adm; times3[2] = r->t_done; }
    return PLB_OK;
}

int plb_server_memory(plb_server* srv, int64_t* in_use, int64_t* peak) {
    if (!srv) return PLB_EINVAL;
    std::lock_guard<std::mutex> lk(srv->mu);
    if (in_use) *in_use = srv->used;
    if (peak) *peak = srv->peak;
    return PLB_OK;
}

int plb_server_stop(plb_server* srv) {
    if (!srv) return PLB_OK;
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        srv->stop = true;
        srv->work_cv.notify_all();
    }
    if (srv->th.joinable()) srv->th.join();
    delete srv;
    return PLB_OK;
}

}  // extern "C"
