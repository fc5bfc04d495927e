// The solve server (plb_server_*, include/plb.h): continuous batching of
// independent lattice-Boltzmann solves on one GPU.
//
// One scheduler thread owns every CUDA call.  Running work is a set of lanes,
// each on its own stream: a batch lane holds the small solves of one class
// (same lattice, storage and arithmetic) and advances them as one plb_batch;
// a solo lane holds one large solve and advances it with the solve's own
// kernels.  Each loop the scheduler
//   1. admits queued requests while their device bytes fit the budget (a
//      request larger than the whole budget fails), the one with the fewest
//      cell updates first unless the oldest has waited PLB_SERVER_MAX_WAIT
//      seconds (default 30; PLB_SERVER_ORDER=fifo: arrival order), while the
//      running requests hold fewer than PLB_SERVER_ACTIVE_CELLS cells
//      (default 2^23), and routes each to a new solo lane or to its class's
//      batch lane,
//   2. collects the lanes whose tick has ended (an event per lane, polled):
//      solves that have run all their steps retire -- rho and u are copied to
//      host memory, the solve is destroyed, its bytes return to the budget,
//   3. starts the next tick of every idle lane -- min(tick_steps, fewest
//      steps left in the lane) -- after rebuilding a batch whose members
//      changed,
// so one lane's tick never waits for another's.  Device memory is
// stream-ordered, so retiring a solve does not synchronize the device.
// Clients submit from any thread and wait on a condition variable.
#include <atomic>
#include <cmath>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
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
#include "admission.h"

namespace plb {
void record_error(const std::string& msg);   // capi.cu: the plb_last_error() slot
int check_params(const plb_params* p);       // capi.cu: plb_solve_create's validation
int set_solve_priority(plb_solve* s, int priority);   // capi.cu: move onto a stream of that priority
int set_batch_priority(plb_batch* b, int priority);
int read_moments(plb_solve* s, float* rho, float* u);   // capi.cu: rho and u with one wait
int set_batch_multi(plb_batch* b, bool multi);          // capi.cu: one launch a call
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
    std::atomic<bool> cancel{false};   // set by plb_server_cancel while it runs
};

// A unit of running work with its own stream: one batch of small solves of a
// class, or one large solve.
struct Lane {
    bool solo = false;
    std::vector<Req*> members;
    std::vector<Req*> joining;     // batch lanes: admitted while a tick was in flight
    plb_batch* batch = nullptr;
    bool dirty = true;             // batch membership changed since it was built
    cudaEvent_t done = nullptr;    // recorded after each tick
    int64_t inflight = 0;          // steps of the tick in flight; 0 when idle
};

using ClassKey = std::tuple<int, int, int, int>;   // q, storage, arith, collision

long long round_up(long long v, long long m) { return (v + m - 1) / m * m; }

// Solves of at least this many cells run in their own lane.
// Admission order.  Under overload the budget fills with admitted requests
// that share the device, and a request's latency is its wait for admission
// plus its share of the device; taking the smallest work first (with an age
// bound so large requests are not starved) shortens the median wait without
// changing the total work or its rate.
bool fifo_order() {
    static const bool v = [] {
        const char* e = std::getenv("PLB_SERVER_ORDER");
        return e && std::strcmp(e, "fifo") == 0;
    }();
    return v;
}

double max_wait_s() {
    static const double v = [] {
        const char* e = std::getenv("PLB_SERVER_MAX_WAIT");
        const double x = e ? std::atof(e) : 0.0;
        return x > 0.0 ? x : 30.0;
    }();
    return v;
}

double work_of(const Req* r) { return (double)r->p.nx * r->p.ny * r->p.nz * (double)r->steps; }

int64_t cells_of(const Req* r) { return (int64_t)r->p.nx * r->p.ny * r->p.nz; }

// Cells the running requests may hold together (PLB_SERVER_ACTIVE_CELLS).
// Enough to keep the device saturated; more only makes the admitted
// requests share it longer (every one finishes later) and costs the
// scheduler thread more lanes to service.  A request larger than the cap
// runs once nothing else is running.
int64_t active_cells_cap() {
    static const int64_t v = [] {
        const char* e = std::getenv("PLB_SERVER_ACTIVE_CELLS");
        const long long x = e ? std::atoll(e) : 0;
        return (int64_t)(x > 0 ? x : (1LL << 23));
    }();
    return v;
}

bool server_batch_multi() {
    static const bool v = [] {
        const char* e = std::getenv("PLB_SERVER_BATCH_MULTI");
        return e && std::strcmp(e, "1") == 0;
    }();
    return v;
}

long long solo_cells() {
    static const long long v = [] {
        const char* e = std::getenv("PLB_SERVER_SOLO_CELLS");
        const long long x = e ? std::atoll(e) : 0;
        return x > 0 ? x : (1LL << 19);
    }();
    return v;
}

}  // namespace

struct plb_server {
    int device = 0;
    int64_t budget = 0, used = 0, peak = 0;
    int64_t active_cells = 0;   // cells of the running requests (scheduler's admission cap)
    int tick = 100;
    Clock::time_point t0;
    std::thread th;
    std::mutex mu;
    std::condition_variable work_cv, done_cv;
    bool stop = false;
    std::deque<Req*> pending;
    std::unordered_map<int64_t, std::unique_ptr<Req>> reqs;
    int64_t next_id = 1;
    // scheduler thread only
    // seconds the scheduler spent creating solves, collecting finished ones,
    // rebuilding batches and launching ticks, and sleeping with every lane
    // busy (PLB_SERVER_STATS=1 prints them when the server stops)
    double t_create = 0, t_retire = 0, t_rebuild = 0, t_launch = 0, t_idle = 0;
    int64_t n_rebuild = 0, n_ticks = 0;
    std::map<ClassKey, std::unique_ptr<Lane>> batch_lanes;
    std::vector<std::unique_ptr<Lane>> solo_lanes;
    // retired solves whose streams may still be busy: destroyed once idle,
    // so retirement never waits for a destruction
    std::vector<plb_solve*> graveyard;
    int prio_least = 0, prio_greatest = 0;   // cudaDeviceGetStreamPriorityRange

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
        srv->active_cells -= cells_of(r);
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
    if (plb::read_moments(r->s, r->rho.data(), r->u.data()) != PLB_OK) err = plb_last_error();
    srv->graveyard.push_back(r->s);
    r->s = nullptr;
    finish(srv, r, err.empty() ? PLB_REQ_DONE : PLB_REQ_FAILED, err);
}

// Destroys the retired solves whose streams have no work left (all of them
// when `all`).
void bury(plb_server* srv, bool all) {
    for (size_t i = 0; i < srv->graveyard.size();) {
        plb_solve* s = srv->graveyard[i];
        if (all || cudaStreamQuery((cudaStream_t)plb_stream_handle(s)) != cudaErrorNotReady) {
            plb_solve_destroy(s);
            srv->graveyard[i] = srv->graveyard.back();
            srv->graveyard.pop_back();
        } else {
            ++i;
        }
    }
}

// A running request cancelled by its client: its solve is destroyed and
// its bytes return to the budget; there is no result.
void drop_cancelled(plb_server* srv, Req* r) {
    if (r->s) plb_solve_destroy(r->s);
    r->s = nullptr;
    finish(srv, r, PLB_REQ_CANCELLED, "request was cancelled");
}

void fail_lane(plb_server* srv, Lane& L, const std::string& e) {
    if (L.batch) plb_batch_destroy(L.batch);
    L.batch = nullptr;
    for (std::vector<Req*>* v : {&L.members, &L.joining})
        for (Req* r : *v) {
            if (r->s) plb_solve_destroy(r->s);
            r->s = nullptr;
            finish(srv, r, PLB_REQ_FAILED, e);
        }
    L.members.clear();
    L.joining.clear();
    L.inflight = 0;
    L.dirty = true;
}

// Starts the next tick of an idle lane with members.
// Lanes run on streams ranked by their work, so that small requests are not
// held up behind large ones when the device is oversubscribed: batch lanes
// (small requests) at the highest priority, solo lanes one level lower for
// each factor of ~3 of cell updates above 3e8.
int solo_priority(const plb_server* srv, const Req* r) {
    const double w = (double)r->p.nx * r->p.ny * r->p.nz * (double)r->steps;
    int level = w > 3e8 ? (int)(std::log10(w / 3e8) * 2.0) : 0;
    const int levels = srv->prio_least - srv->prio_greatest;   // >= 0; larger number = lower priority
    if (level > levels) level = levels;
    return srv->prio_greatest + level;
}

void launch_tick(plb_server* srv, Lane& L) {
    if (!L.done && cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming) != cudaSuccess) {
        fail_lane(srv, L, "cudaEventCreate failed");
        return;
    }
    int64_t t = srv->tick;
    for (Req* r : L.members) t = r->remaining < t ? r->remaining : t;
    if (t < 1) t = 1;
    void* stream = nullptr;
    if (L.solo) {
        if (plb_step_async(L.members[0]->s, t) != PLB_OK) return fail_lane(srv, L, plb_last_error());
        stream = plb_stream_handle(L.members[0]->s);
    } else {
        if (L.dirty) {
            const auto tr = Clock::now();
            ++srv->n_rebuild;
            if (L.batch) plb_batch_destroy(L.batch);
            L.batch = nullptr;
            std::vector<plb_solve*> ss;
            for (Req* r : L.members) ss.push_back(r->s);
            if (plb_batch_create((int32_t)ss.size(), ss.data(), &L.batch) != PLB_OK)
                return fail_lane(srv, L, plb_last_error());
            if (plb::set_batch_priority(L.batch, srv->prio_greatest) != PLB_OK)
                return fail_lane(srv, L, plb_last_error());
            // PLB_SERVER_BATCH_MULTI=1: one cooperative launch a tick, no
            // graph capture per membership (measured on 300 small requests
            // arriving at once: 214 solves/s against 231 with graph chunks;
            // the lanes are bound by the GPU, not by the scheduler)
            if (plb::set_batch_multi(L.batch, server_batch_multi()) != PLB_OK)
                return fail_lane(srv, L, plb_last_error());
            L.dirty = false;
            srv->t_rebuild += std::chrono::duration<double>(Clock::now() - tr).count();
        }
        if (plb_batch_step_async(L.batch, t) != PLB_OK) return fail_lane(srv, L, plb_last_error());
        stream = plb_batch_stream_handle(L.batch);
    }
    if (cudaEventRecord(L.done, (cudaStream_t)stream) != cudaSuccess) return fail_lane(srv, L, "cudaEventRecord failed");
    L.inflight = t;
}

// Collects a lane whose tick has ended; returns false while it still runs.
bool collect_tick(plb_server* srv, Lane& L) {
    const cudaError_t q = cudaEventQuery(L.done);
    if (q == cudaErrorNotReady) return false;
    if (q != cudaSuccess) {
        fail_lane(srv, L, std::string("tick failed: ") + cudaGetErrorString(q));
        return true;
    }
    // a batch tick's multi-step launch reports a grid barrier that timed out
    if (!L.solo && L.batch && plb_batch_synchronize(L.batch) != PLB_OK) {
        fail_lane(srv, L, plb_last_error());
        return true;
    }
    std::vector<Req*> keep;
    for (Req* r : L.members) {
        r->remaining -= L.inflight;
        if (r->cancel) {
            drop_cancelled(srv, r);
            L.dirty = true;
        } else if (r->remaining <= 0) {
            retire(srv, r);
            L.dirty = true;
        } else {
            keep.push_back(r);
        }
    }
    L.members.swap(keep);
    L.inflight = 0;
    return true;
}

void scheduler(plb_server* srv) {
    cudaSetDevice(srv->device);
    if (cudaDeviceGetStreamPriorityRange(&srv->prio_least, &srv->prio_greatest) != cudaSuccess)
        srv->prio_least = srv->prio_greatest = 0;
    for (;;) {
        // 1. admission
        std::vector<Req*> admitted;
        size_t waiting = 0;   // requests left queued (no room yet)
        {
            std::unique_lock<std::mutex> lk(srv->mu);
            bool busy = !srv->solo_lanes.empty();
            for (auto& kv : srv->batch_lanes)
                busy |= !kv.second->members.empty() || !kv.second->joining.empty();
            if (!busy)
                srv->work_cv.wait(lk, [&] { return srv->stop || !srv->pending.empty(); });
            if (srv->stop) break;
            plb::AdmissionState ast;
            ast.budget = srv->budget;
            ast.cap_cells = active_cells_cap();
            ast.max_wait = max_wait_s();
            ast.fifo = fifo_order();
            std::vector<plb::AdmissionView> view;
            for (const Req* q : srv->pending)
                view.push_back({q->t_sub, work_of(q), cells_of(q), plb_solve_bytes(&q->p)});
            while (!srv->pending.empty()) {
                ast.used = srv->used;
                ast.active_cells = srv->active_cells;
                const size_t pick = plb::admission_pick(view, ast, srv->now());
                Req* r = srv->pending[pick];
                const int64_t need = view[pick].bytes;
                const plb::Admit what = plb::admission_decide(view[pick], ast);
                if (what == plb::Admit::kReject) {
                    srv->pending.erase(srv->pending.begin() + (long)pick);
                    view.erase(view.begin() + (long)pick);
                    r->state = PLB_REQ_FAILED;
                    r->err = "request needs more device memory than the whole budget";
                    r->t_done = srv->now();
                    srv->done_cv.notify_all();
                    continue;
                }
                if (what == plb::Admit::kWait) break;   // wait for room
                srv->pending.erase(srv->pending.begin() + (long)pick);
                view.erase(view.begin() + (long)pick);
                srv->active_cells += cells_of(r);
                srv->used += need;
                if (srv->used > srv->peak) srv->peak = srv->used;
                r->bytes = need;
                r->state = PLB_REQ_RUNNING;
                r->t_adm = srv->now();
                admitted.push_back(r);
            }
            waiting = srv->pending.size();
        }
        for (Req* r : admitted) {
            const auto tc = Clock::now();
            const std::string e = start_solve(r);
            srv->t_create += std::chrono::duration<double>(Clock::now() - tc).count();
            if (!e.empty()) {
                finish(srv, r, PLB_REQ_FAILED, e);
                continue;
            }
            // large solves, and AA ones (batches are AB only), run alone
            if (r->p.nx * r->p.ny * r->p.nz >= solo_cells() || r->p.streaming == PLB_STREAMING_AA) {
                if (plb::set_solve_priority(r->s, solo_priority(srv, r)) != PLB_OK) {
                    const std::string e2 = plb_last_error();
                    plb_solve_destroy(r->s);
                    r->s = nullptr;
                    finish(srv, r, PLB_REQ_FAILED, e2);
                    continue;
                }
                auto L = std::make_unique<Lane>();
                L->solo = true;
                L->members.push_back(r);
                srv->solo_lanes.push_back(std::move(L));
            } else {
                // a batch member's own work (its read-back at retirement)
                // runs at the batch lanes' priority, between their kernels
                if (plb::set_solve_priority(r->s, srv->prio_greatest) != PLB_OK) {
                    const std::string e2 = plb_last_error();
                    plb_solve_destroy(r->s);
                    r->s = nullptr;
                    finish(srv, r, PLB_REQ_FAILED, e2);
                    continue;
                }
                auto& L = srv->batch_lanes[ClassKey(r->p.q, r->p.storage, r->p.arith, r->p.collision)];
                if (!L) L = std::make_unique<Lane>();
                L->joining.push_back(r);
            }
        }
        // 2. collect ended ticks, 3. start the next ones
        bool progressed = !admitted.empty();
        auto service = [&](Lane& L) {
            if (L.inflight) {
                const auto tr = Clock::now();
                const bool ended = collect_tick(srv, L);
                srv->t_retire += std::chrono::duration<double>(Clock::now() - tr).count();
                if (!ended) return;
            }
            if (!L.joining.empty()) {
                for (Req* r : L.joining) {
                    if (r->cancel) drop_cancelled(srv, r);
                    else L.members.push_back(r);
                }
                L.joining.clear();
                L.dirty = true;
            }
            if (L.members.empty()) {
                if (L.batch) plb_batch_destroy(L.batch);
                L.batch = nullptr;
                return;
            }
            const auto tl = Clock::now();
            launch_tick(srv, L);
            ++srv->n_ticks;
            srv->t_launch += std::chrono::duration<double>(Clock::now() - tl).count();
            progressed = true;
        };
        for (auto& kv : srv->batch_lanes) service(*kv.second);
        for (auto& L : srv->solo_lanes) service(*L);
        bury(srv, false);
        for (size_t i = 0; i < srv->solo_lanes.size();) {
            Lane& L = *srv->solo_lanes[i];
            if (L.members.empty() && !L.inflight) {
                if (L.done) cudaEventDestroy(L.done);
                srv->solo_lanes.erase(srv->solo_lanes.begin() + (long)i);
            } else {
                ++i;
            }
        }
        if (!progressed) {
            // every lane is mid-tick: sleep briefly, or until a new request arrives
            const auto ti = Clock::now();
            std::unique_lock<std::mutex> lk(srv->mu);
            srv->work_cv.wait_for(lk, std::chrono::microseconds(200),
                                  [&] { return srv->stop || srv->pending.size() > waiting; });
            srv->t_idle += std::chrono::duration<double>(Clock::now() - ti).count();
        }
    }
    // stop: wait for the ticks in flight, then drop everything
    auto drop = [&](Lane& L) {
        if (L.inflight) cudaEventSynchronize(L.done);
        if (L.batch) plb_batch_destroy(L.batch);
        for (std::vector<Req*>* v : {&L.members, &L.joining})
            for (Req* r : *v)
                if (r->s) plb_solve_destroy(r->s);
        if (L.done) cudaEventDestroy(L.done);
    };
    for (auto& kv : srv->batch_lanes) drop(*kv.second);
    for (auto& L : srv->solo_lanes) drop(*L);
    srv->batch_lanes.clear();
    srv->solo_lanes.clear();
    bury(srv, true);
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
    const long long nbuf = (p->semantics == PLB_SEMANTICS_NATIVE && p->streaming == PLB_STREAMING_AA) ? 1 : 2;
    long long b = nbuf * p->q * ks * esize;       // population buffers
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
    // malformed requests (a NaN viscosity, an unknown lattice, ...) are refused
    // here, on the caller's thread, with plb_solve_create's message
    const int v = plb::check_params(&req->params);
    if (v != PLB_OK) return v;
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
        return r->state == PLB_REQ_DONE || r->state == PLB_REQ_FAILED || r->state == PLB_REQ_CANCELLED;
    });
    if (!ok) return PLB_ETIMEOUT;
    if (r->state == PLB_REQ_FAILED) {
        plb::record_error(r->err);
        return PLB_ECUDA;
    }
    if (r->state == PLB_REQ_CANCELLED) {
        plb::record_error(r->err);
        return PLB_ESTATE;
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
        if (it->second->state == PLB_REQ_FAILED || it->second->state == PLB_REQ_CANCELLED) {
            plb::record_error(it->second->err);
            const int rc = it->second->state == PLB_REQ_FAILED ? PLB_ECUDA : PLB_ESTATE;
            srv->reqs.erase(it);
            return rc;
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

int plb_server_cancel(plb_server* srv, int64_t id) {
    if (!srv) return PLB_EINVAL;
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return PLB_EINVAL;
    Req* r = it->second.get();
    if (r->state == PLB_REQ_QUEUED) {
        for (auto q = srv->pending.begin(); q != srv->pending.end(); ++q)
            if (*q == r) {
                srv->pending.erase(q);
                break;
            }
        r->state = PLB_REQ_CANCELLED;
        r->err = "request was cancelled";
        r->t_done = srv->now();
        srv->done_cv.notify_all();
        return PLB_OK;
    }
    if (r->state == PLB_REQ_RUNNING) {
        r->cancel = true;   // the scheduler drops it when its current tick ends
        return PLB_OK;
    }
    plb::record_error("request already finished");
    return PLB_ESTATE;
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
    const char* st = std::getenv("PLB_SERVER_STATS");
    if (st && std::strcmp(st, "1") == 0)
        std::fprintf(stderr,
                     "plb_server: create %.3f s, collect/retire %.3f s, batch rebuilds %.3f s (%lld), "
                     "tick launches %.3f s (%lld), idle %.3f s\n",
                     srv->t_create, srv->t_retire, srv->t_rebuild, (long long)srv->n_rebuild, srv->t_launch,
                     (long long)srv->n_ticks, srv->t_idle);
    delete srv;
    return PLB_OK;
}

}  // extern "C"
