// Serving loop for the engine: requests of different L, phi, neel, channel
// and walker counts are admitted by device footprint and advanced
// concurrently (continuous batching).  Host-side C++ over the engine's C ABI;
// declared in include/gpvmc_gb300.h.
//
// A worker thread schedules every job.  Each pass over its state it
//   1. admits queued requests in arrival order while a slot is free and the
//      admitted jobs' gv_job_footprint bytes stay within the budget (a request
//      larger than the whole budget runs when the device is otherwise empty),
//      and creates the job and its walkers (vmc.cpp:140-263 for one request)
//      on a helper thread, since the FP64 start inversions take a while;
//   2. keeps two walk calls of chunk_sweeps sweeps in flight on every admitted
//      job's stream (thermalisation first, then the measured sweeps, whose
//      quantity sums accumulate across calls), so that work of all admitted
//      jobs overlaps on the device;
//   3. retires jobs whose calls have completed: a helper thread reads their
//      results (optionally re-measures the final configurations with fresh
//      FP64 inverses), frees the job and its bytes, and wakes waiting callers.
// A job is touched by one thread at a time (its helper, then the worker, then
// its helper); jobs run on their own streams.
// A job's chain depends only on its own request (seed, walkers, chunking), so
// its results do not depend on what else is running.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <future>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/gpvmc_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
    uint64_t ticket = 0;
    gv_request r{};
    gv_result res{};
    uint64_t footprint = 0;
    gv_job* job = nullptr;
    cudaEvent_t ev[2] = {nullptr, nullptr};
    uint64_t total = 0;      // walk calls to issue
    uint64_t issued = 0;     // walk calls issued
    int inflight = 0;        // issued calls not yet seen complete
    uint64_t therm_calls = 0;
    uint64_t chunk_len = 0;  // steps per call
    std::future<gv_status> start_f;   // job creation and walker start on a helper thread
    std::future<void> finish_f;       // result collection on a helper thread
};

}  // namespace

struct gv_server {
    gv_server_config cfg{};
    uint64_t budget = 0;
    int device = 0;
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Req*> pending;
    std::map<uint64_t, std::unique_ptr<Req>> reqs;
    std::vector<Req*> starting;  // worker thread only: jobs being created
    std::vector<Req*> running;   // worker thread only: jobs whose walks are being issued
    std::vector<Req*> finishing; // worker thread only: jobs whose results are being collected
    uint64_t next_ticket = 1;
    uint64_t used = 0;
    int n_running = 0;
    bool stop = false;
    Clock::time_point t0;
    std::thread worker;

    double now() const { return std::chrono::duration<double>(Clock::now() - t0).count(); }
    void run();
    gv_status start(Req* q);
    void finish(Req* q, gv_status st);
    bool advance(Req* q);
};

namespace {

// Mean over walkers of E/site (ground state) or Re tr H / (Ns Re tr O)
// (exciton), and of StagMagnZ, from the job's accumulators.
gv_status summarise(gv_job* j, int W, int Ns, int Nexc, double* e_site, double* stagmagn)
{
    std::vector<int32_t> n(W);
    gv_status st;
    double se = 0.0;
    int ne = 0;
    if (Nexc > 1) {
        std::vector<double> v(size_t(W) * 4 * Nexc * Nexc);
        if ((st = gv_job_read_projheis(j, v.data(), n.data()))) return st;
        for (int w = 0; w < W; ++w) {
            const double* H = v.data() + size_t(w) * 4 * Nexc * Nexc;
            const double* O = H + 2 * size_t(Nexc) * Nexc;
            double th = 0.0, to = 0.0;
            for (int k = 0; k < Nexc; ++k) { th += H[2 * (size_t(k) * Nexc + k)]; to += O[2 * (size_t(k) * Nexc + k)]; }
            if (n[w] > 0 && to != 0.0) { se += th / (double(Ns) * to); ++ne; }
        }
    } else {
        std::vector<double> v(size_t(W) * 4);
        if ((st = gv_job_read_projheis(j, v.data(), n.data()))) return st;
        for (int w = 0; w < W; ++w)
            if (n[w] > 0) { se += v[4 * w] / n[w]; ++ne; }
    }
    *e_site = ne ? se / ne : std::nan("");
    std::vector<double> m(size_t(W) * 2);
    if ((st = gv_job_read_stagmagn(j, m.data(), n.data()))) return st;
    double sm = 0.0;
    int nm = 0;
    for (int w = 0; w < W; ++w)
        if (n[w] > 0) { sm += m[2 * w] / n[w]; ++nm; }
    *stagmagn = nm ? sm / nm : std::nan("");
    return GV_OK;
}

// One ProjHeis measurement of the job's current configurations from its own
// inverses against one from fresh FP64 inverses of the same configurations.
gv_status validate(gv_job* j, const gv_job_config& c, int W, int Ns, int Nexc, double* err)
{
    std::vector<int8_t> cfg(size_t(W) * Ns);
    gv_status st;
    if ((st = gv_job_read_config(j, cfg.data()))) return st;
    gv_job_config c64 = c;
    c64.precision = GV_PREC_FP64;
    c64.reinv_every = 0;
    c64.flags = 0;
    c64.meas_mask = GV_MEAS_PROJHEIS;
    gv_job* r = nullptr;
    if ((st = gv_job_create(&c64, &r))) return st;
    const size_t per = Nexc > 1 ? size_t(4) * Nexc * Nexc : 4;
    std::vector<double> a(size_t(W) * per), b(size_t(W) * per);
    std::vector<int32_t> n(W);
    if (!(st = gv_job_init_walkers(r, cfg.data())) && !(st = gv_job_reset_quantities(r)) && !(st = gv_job_measure(r)) &&
        !(st = gv_job_read_projheis(r, b.data(), n.data())) && !(st = gv_job_set_meas_mask(j, GV_MEAS_PROJHEIS)) &&
        !(st = gv_job_reset_quantities(j)) && !(st = gv_job_measure(j)))
        st = gv_job_read_projheis(j, a.data(), n.data());
    gv_job_destroy(r);
    if (st) return st;
    double e = 0.0;
    for (int w = 0; w < W; ++w) {
        if (Nexc > 1) {
            double d = 0.0, mx = 0.0;
            for (size_t i = 0; i < per / 2; ++i) {
                const double dr = a[w * per + 2 * i] - b[w * per + 2 * i], di = a[w * per + 2 * i + 1] - b[w * per + 2 * i + 1];
                d = std::max(d, std::hypot(dr, di));
                mx = std::max(mx, std::hypot(b[w * per + 2 * i], b[w * per + 2 * i + 1]));
            }
            e = std::max(e, mx > 0.0 ? d / mx : d);
        } else {
            e = std::max(e, std::fabs(a[w * per] - b[w * per]));
        }
    }
    *err = e;
    return GV_OK;
}

}  // namespace

void gv_server::finish(Req* q, gv_status st)
{
    cudaSetDevice(device);
    const gv_job_config& c = q->r.job;
    gv_result res = q->res;
    res.validation_error = -1.0;
    if (q->job) {
        gv_status s2 = gv_job_synchronize(q->job);
        if (!st) st = s2;
        int32_t Ns = 0, Nexc = 1;
        gv_job_dims(q->job, &Ns, nullptr, nullptr, &Nexc);
        std::vector<uint64_t> cnt(size_t(c.n_walkers) * 5);
        if (!gv_job_read_counts(q->job, cnt.data()))
            for (int w = 0; w < c.n_walkers; ++w) { res.steps += cnt[5 * w]; res.accepted += cnt[5 * w + 1]; }
        if (!st && q->r.sweeps > 0) st = summarise(q->job, c.n_walkers, Ns, Nexc, &res.e_site, &res.stagmagn);
        if (!st && q->r.validate) st = validate(q->job, c, c.n_walkers, Ns, Nexc, &res.validation_error);
        gv_job_destroy(q->job);
        q->job = nullptr;
    }
    for (cudaEvent_t& e : q->ev)
        if (e) { cudaEventDestroy(e); e = nullptr; }
    std::lock_guard<std::mutex> lk(m);
    res.status = st;
    res.state = GV_REQ_DONE;
    res.t_done = now();
    q->res = res;
    used -= q->footprint;
    --n_running;
    cv_done.notify_all();
}

// Job creation and walker start (FP64 start inversions, the exciton's state
// pick): on a helper thread, so that the worker keeps issuing other jobs' walks.
gv_status gv_server::start(Req* q)
{
    cudaSetDevice(device);
    gv_job_config c = q->r.job;
    c.flags |= GV_FLAG_CUDA_GRAPHS;   // the job's walk calls repeat: one graph launch each
    gv_status st = gv_job_create(&c, &q->job);
    if (!st) st = gv_job_set_meas_mask(q->job, c.meas_mask);
    if (!st) st = gv_job_init_walkers(q->job, nullptr);
    if (!st && (cudaEventCreateWithFlags(&q->ev[0], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&q->ev[1], cudaEventDisableTiming) != cudaSuccess))
        st = GV_ERR_CUDA;
    const uint64_t sweep = uint64_t(c.L) * c.L;
    const uint64_t cs = uint64_t(std::max(1, cfg.chunk_sweeps));
    q->chunk_len = cs * sweep;
    q->therm_calls = (q->r.therm_sweeps + cs - 1) / cs;
    q->total = q->therm_calls + (q->r.sweeps + cs - 1) / cs;
    return st;
}

// Issue calls up to two in flight, retire completed ones; true if anything moved.
bool gv_server::advance(Req* q)
{
    bool moved = false;
    while (q->inflight > 0) {
        const cudaError_t e = cudaEventQuery(q->ev[(q->issued - q->inflight) & 1]);
        if (e == cudaErrorNotReady) break;
        if (e != cudaSuccess) return false;
        --q->inflight;
        moved = true;
    }
    while (q->inflight < 2 && q->issued < q->total) {
        const uint64_t i = q->issued;
        const bool meas = i >= q->therm_calls;
        const uint64_t left = meas ? q->r.sweeps - (i - q->therm_calls) * (q->chunk_len / (uint64_t(q->r.job.L) * q->r.job.L))
                                   : q->r.therm_sweeps - i * (q->chunk_len / (uint64_t(q->r.job.L) * q->r.job.L));
        const uint64_t len = std::min<uint64_t>(q->chunk_len, left * uint64_t(q->r.job.L) * q->r.job.L);
        gv_status st = GV_OK;
        if (meas && i == q->therm_calls) st = gv_job_reset_quantities(q->job);
        if (!st) st = gv_job_walk_continue(q->job, len, meas ? q->r.meas : 0);
        void* s = nullptr;
        if (!st) st = gv_job_stream(q->job, &s);
        if (!st && cudaEventRecord(q->ev[i & 1], static_cast<cudaStream_t>(s)) != cudaSuccess) st = GV_ERR_CUDA;
        if (st) { q->total = q->issued; q->res.status = st; break; }
        ++q->issued;
        ++q->inflight;
        moved = true;
    }
    return moved;
}

void gv_server::run()
{
    cudaSetDevice(device);
    for (;;) {
        std::vector<Req*> admit;
        {
            std::lock_guard<std::mutex> lk(m);
            if (stop && pending.empty() && n_running == 0 && starting.empty() && finishing.empty()) break;
            while (!pending.empty() && n_running < cfg.max_jobs) {
                Req* q = pending.front();
                if (used + q->footprint > budget && n_running > 0) break;
                pending.pop_front();
                used += q->footprint;
                ++n_running;
                q->res.state = GV_REQ_RUNNING;
                q->res.t_admit = now();
                admit.push_back(q);
            }
        }
        bool moved = !admit.empty();
        for (Req* q : admit) {
            q->start_f = std::async(std::launch::async, [this, q] { return start(q); });
            starting.push_back(q);
        }
        for (size_t i = 0; i < starting.size();) {
            Req* q = starting[i];
            if (q->start_f.wait_for(std::chrono::seconds(0)) != std::future_status::ready) { ++i; continue; }
            const gv_status st = q->start_f.get();
            {
                std::lock_guard<std::mutex> lk(m);   // poll() reads the result under the lock
                q->res.t_started = now();
            }
            starting.erase(starting.begin() + i);
            if (st) {
                q->finish_f = std::async(std::launch::async, [this, q, st] { finish(q, st); });
                finishing.push_back(q);
            } else {
                running.push_back(q);
            }
            moved = true;
        }
        for (size_t i = 0; i < running.size();) {
            Req* q = running[i];
            moved |= advance(q);
            if (q->issued == q->total && q->inflight == 0) {
                {
                    std::lock_guard<std::mutex> lk(m);
                    q->res.t_walked = now();
                }
                running.erase(running.begin() + i);
                const gv_status st = q->res.status;
                q->finish_f = std::async(std::launch::async, [this, q, st] { finish(q, st); });
                finishing.push_back(q);
                moved = true;
            } else {
                ++i;
            }
        }
        for (size_t i = 0; i < finishing.size();) {
            if (finishing[i]->finish_f.wait_for(std::chrono::seconds(0)) == std::future_status::ready) {
                finishing[i]->finish_f.get();
                finishing.erase(finishing.begin() + i);
                moved = true;
            } else {
                ++i;
            }
        }
        if (!moved) {
            std::unique_lock<std::mutex> lk(m);
            cv_work.wait_for(lk, std::chrono::microseconds(100));
        }
    }
}

extern "C" {

gv_status gv_server_create(const gv_server_config* cfg, gv_server** out)
{
    if (!cfg || !out || cfg->max_jobs < 1 || cfg->chunk_sweeps < 1) return GV_ERR_INVALID;
    *out = nullptr;
    auto* s = new gv_server;
    s->cfg = *cfg;
    if (cudaGetDevice(&s->device) != cudaSuccess) { delete s; return GV_ERR_CUDA; }
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { delete s; return GV_ERR_CUDA; }
    s->budget = cfg->hbm_budget ? cfg->hbm_budget : uint64_t(0.8 * double(fr));
    s->t0 = Clock::now();
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return GV_OK;
}

gv_status gv_server_submit(gv_server* s, const gv_request* r, uint64_t* ticket)
{
    if (!s || !r || !ticket) return GV_ERR_INVALID;
    const uint64_t sweep = uint64_t(r->job.L) * r->job.L;
    if (r->sweeps > 0 && (r->meas == 0 || sweep % r->meas)) return GV_ERR_INVALID;
    uint64_t fp = 0;
    if (gv_job_footprint(&r->job, &fp)) return GV_ERR_INVALID;
    auto q = std::make_unique<Req>();
    q->r = *r;
    q->footprint = fp;
    q->res.state = GV_REQ_PENDING;
    q->res.footprint = fp;
    q->res.validation_error = -1.0;
    std::lock_guard<std::mutex> lk(s->m);
    if (s->stop) return GV_ERR_INVALID;
    q->ticket = s->next_ticket++;
    q->res.t_submit = s->now();
    *ticket = q->ticket;
    s->pending.push_back(q.get());
    s->reqs[q->ticket] = std::move(q);
    s->cv_work.notify_all();
    return GV_OK;
}

gv_status gv_server_poll(gv_server* s, uint64_t ticket, gv_result* out)
{
    if (!s || !out) return GV_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return GV_ERR_INVALID;
    *out = it->second->res;
    return GV_OK;
}

gv_status gv_server_wait(gv_server* s, uint64_t ticket, double timeout_s, gv_result* out)
{
    if (!s) return GV_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->m);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return GV_ERR_INVALID;
    Req* q = it->second.get();
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s),
                                        [q] { return q->res.state == GV_REQ_DONE; });
    if (out) *out = q->res;
    return ok ? GV_OK : GV_ERR_TIMEOUT;
}

gv_status gv_server_drain(gv_server* s, double timeout_s)
{
    if (!s) return GV_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->m);
    const bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [s] {
        if (!s->pending.empty() || s->n_running) return false;
        for (auto& kv : s->reqs)
            if (kv.second->res.state != GV_REQ_DONE) return false;
        return true;
    });
    return ok ? GV_OK : GV_ERR_TIMEOUT;
}

gv_status gv_server_destroy(gv_server* s)
{
    if (!s) return GV_OK;
    {
        std::lock_guard<std::mutex> lk(s->m);
        s->stop = true;
        s->cv_work.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    delete s;
    return GV_OK;
}

}  // extern "C"
