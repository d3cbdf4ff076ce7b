// bsj_server.cpp -- continuous-batching request loop over the GB300 engine.
//
// The reference solves one instance per call, synchronously (gpu/v1/solver.cu:178-298);
// its drivers call it in a loop (gpu/v1/main.cu:62-71, gpu/v1/benchmark.cu:44-77).  Here
// solves arrive as requests and share the GPU:
//   - bsj_submit copies the request into a FIFO and returns a ticket at once;
//   - one worker thread admits queued requests while an in-flight slot (a CUDA stream)
//     is free and the device memory they would hold fits the budget, so requests that
//     arrive while others run join them on the device as slots and memory free up;
//   - each admitted request runs as a plan whose whole level loop is one CUDA-graph
//     launch on its slot's stream, so the levels of different requests overlap;
//   - finished plans go to an idle pool keyed by shape (n, m, K, mode) and the next
//     request of that shape reuses the plan and its graph (bsj_plan_update: new data, no
//     allocation, no re-capture); idle plans are freed, oldest first, when memory is short;
//   - bsj_poll / bsj_wait hand out the result with the request's queue and run times;
//   - bsj_server_prepare queues plan builds of a shape before its requests arrive.
// A request's result does not depend on what else runs: every plan owns its memory and
// the kernels of one request read nothing of another's.
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bsj.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    uint64_t ticket = 0;
    int32_t n = 0, m = 0;
    std::vector<int32_t> machine, duration;
    bsj_beam beam{};
    int64_t bytes = 0;  // device footprint of its plan
    std::string shape;
    Clock::time_point submitted, admitted;
    bool prepare = false;  // bsj_server_prepare: build and pool a plan, no result
    bool built = false;    // no idle plan was free: this request built its plan
};

struct Done {
    bsj_status status = BSJ_OK;
    bsj_result result{};
    std::vector<int32_t> seq;
    bsj_request_times times{};
};

struct Slot {
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    Request req;
    bsj_plan* plan = nullptr;
};

std::string shape_of(const Request& r)
{
    return std::to_string(r.n) + "x" + std::to_string(r.m) + ":" + std::to_string(r.beam.mode) + ":" +
           std::to_string(r.beam.beam_width);
}

}  // namespace

struct bsj_server {
    bsj_context* ctx = nullptr;      // the worker's: plans, captures, uploads
    bsj_context* est_ctx = nullptr;  // bsj_submit's footprint checks (under mu)
    int device = 0;
    int64_t budget = 0;
    int cluster_inflight = 0;   // others in flight up to which a request runs the cluster select
    std::vector<Slot> slots;

    std::mutex mu;
    std::condition_variable cv_work;   // the worker: new requests or stop
    std::condition_variable cv_done;   // waiters: a request finished
    std::deque<Request> pending;
    std::unordered_map<uint64_t, Done> finished;
    std::unordered_map<uint64_t, int> live;  // tickets submitted and not yet handed out
    uint64_t next_ticket = 1;
    bool stop = false;
    bsj_server_stats stats{};

    // worker-owned
    std::map<std::string, std::vector<bsj_plan*>> idle;
    std::list<std::pair<std::string, bsj_plan*>> idle_lru;  // oldest first
    int64_t bytes_inflight = 0, bytes_idle = 0;
    std::thread worker;

    void run();
    bool admit_one(Request& r, Slot& s, int busy);
    void finish(Slot& s);
    void evict_idle(int64_t need);
    bsj_plan* take_idle(const std::string& shape);
};

bsj_plan* bsj_server::take_idle(const std::string& shape)
{
    auto it = idle.find(shape);
    if (it == idle.end() || it->second.empty()) return nullptr;
    bsj_plan* p = it->second.back();
    it->second.pop_back();
    for (auto l = idle_lru.begin(); l != idle_lru.end(); ++l)
        if (l->second == p) { idle_lru.erase(l); break; }
    bytes_idle -= bsj_plan_device_bytes(p);
    return p;
}

// Frees idle plans, oldest first, until `need` more bytes fit the budget (or none is left).
void bsj_server::evict_idle(int64_t need)
{
    while (!idle_lru.empty() && bytes_inflight + bytes_idle + need > budget) {
        auto [shape, p] = idle_lru.front();
        idle_lru.pop_front();
        auto& v = idle[shape];
        for (size_t i = 0; i < v.size(); i++)
            if (v[i] == p) { v.erase(v.begin() + (long)i); break; }
        bytes_idle -= bsj_plan_device_bytes(p);
        bsj_plan_destroy(p);
    }
}

namespace bsj {
bsj_status plan_capture_forms(bsj_plan* p);   // bsj_engine.cu
}

bool bsj_server::admit_one(Request& r, Slot& s, int busy)
{
    bsj_instance inst{r.n, r.m, r.machine.data(), r.duration.data()};
    bsj_plan* p = r.prepare ? nullptr : take_idle(r.shape);
    bsj_status st = BSJ_OK;
    const Clock::time_point t0 = Clock::now();
    const bool reused = (p != nullptr);
    if (reused) {
        st = bsj_plan_update(p, 1, &inst, 1, &r.beam);
    } else {
        evict_idle(r.bytes);
        st = bsj_plan_create(ctx, 1, &inst, 1, &r.beam, &p);
    }
    // a prepared plan gets the graphs of both selection forms now, off the request path
    if (st == BSJ_OK && r.prepare) st = bsj::plan_capture_forms(p);
    const Clock::time_point t1 = Clock::now();
    // the cluster select halves a wide level's latency for about twice the SM time: worth it
    // while the device has SMs to spare, not when many requests already share it
    if (st == BSJ_OK) st = bsj_plan_set_select_cluster(p, busy <= cluster_inflight ? 1 : 0);
    if (st == BSJ_OK) st = bsj_plan_run(p, s.stream);
    if (st == BSJ_OK && cudaEventRecord(s.done, s.stream) != cudaSuccess) st = BSJ_ERR_CUDA;
    {
        // a new plan captures its graph on its first run: that counts as building
        const double prep = ms_between(t0, t1), run = ms_between(t1, Clock::now());
        std::lock_guard<std::mutex> lk(mu);
        if (reused) {
            stats.plans_reused++;
            stats.update_ms += prep;
            stats.launch_ms += run;
        } else {
            stats.plans_built++;
            stats.build_ms += prep + run;
        }
    }
    if (st != BSJ_OK && r.prepare) {
        if (p) bsj_plan_destroy(p);
        return false;
    }
    if (st != BSJ_OK) {
        if (p) bsj_plan_destroy(p);
        Done d;
        d.status = st;
        d.times.queue_ms = ms_between(r.submitted, Clock::now());
        std::lock_guard<std::mutex> lk(mu);
        finished[r.ticket] = std::move(d);
        stats.completed++;
        cv_done.notify_all();
        return false;
    }
    s.plan = p;
    s.req = std::move(r);
    s.req.built = !reused;
    s.busy = true;
    bytes_inflight += bsj_plan_device_bytes(p);
    return true;
}

void bsj_server::finish(Slot& s)
{
    Done d;
    const Clock::time_point now = Clock::now();
    d.seq.assign((size_t)s.req.n * s.req.m, 0);
    d.result.sequence = d.seq.data();
    d.status = bsj_plan_results(s.plan, &d.result);
    d.result.sequence = nullptr;
    const double collect = ms_between(now, Clock::now());
    d.times.queue_ms = ms_between(s.req.submitted, s.req.admitted);
    d.times.run_ms = ms_between(s.req.admitted, now);
    d.times.built_plan = s.req.built ? 1 : 0;
    bytes_inflight -= bsj_plan_device_bytes(s.plan);
    if (d.status == BSJ_OK) {
        idle[s.req.shape].push_back(s.plan);
        idle_lru.push_back({s.req.shape, s.plan});
        bytes_idle += bsj_plan_device_bytes(s.plan);
    } else {
        bsj_plan_destroy(s.plan);
    }
    s.plan = nullptr;
    s.busy = false;
    std::lock_guard<std::mutex> lk(mu);
    if (s.req.prepare) {
        // a prepared plan: pooled above (counted once it is there), nobody waits for it
        if (d.status == BSJ_OK) stats.plans_prepared++;
        return;
    }
    finished[s.req.ticket] = std::move(d);
    stats.completed++;
    stats.collect_ms += collect;
    cv_done.notify_all();
}

void bsj_server::run()
{
    cudaSetDevice(device);
    for (;;) {
        // retire finished slots
        int busy = 0;
        for (Slot& s : slots) {
            if (!s.busy) continue;
            cudaError_t q = cudaEventQuery(s.done);
            if (q == cudaSuccess) finish(s);
            else if (q == cudaErrorNotReady) busy++;
            else finish(s);  // the error surfaces through bsj_plan_results
        }
        // admit queued requests, in order, while a slot and the memory are free
        for (Slot& s : slots) {
            if (s.busy) continue;
            Request r;
            {
                std::lock_guard<std::mutex> lk(mu);
                if (stop || pending.empty()) break;
                const Request& head = pending.front();
                const bool reusable = !head.prepare && idle.count(head.shape) && !idle[head.shape].empty();
                // a request whose plan would exceed the budget waits for running ones,
                // unless nothing runs (it was checked against the budget at submit)
                if (!reusable && busy > 0 && bytes_inflight + head.bytes > budget) break;
                r = std::move(pending.front());
                pending.pop_front();
            }
            r.admitted = Clock::now();
            if (admit_one(r, s, busy)) {
                busy++;
                std::lock_guard<std::mutex> lk(mu);
                if (busy > stats.peak_inflight) stats.peak_inflight = busy;
                const int64_t held = bytes_inflight + bytes_idle;
                if (held > stats.peak_device_bytes) stats.peak_device_bytes = held;
            }
        }
        std::unique_lock<std::mutex> lk(mu);
        if (stop && busy == 0) break;
        if (busy == 0 && pending.empty()) {
            cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        } else if (busy > 0) {
            // device work in flight: look again shortly (event queries are cheap)
            cv_work.wait_for(lk, std::chrono::microseconds(20));
        }
    }
}

extern "C" {

bsj_status bsj_server_create(bsj_server** out, int device, const bsj_server_config* cfg)
{
    if (!out) return BSJ_ERR_INVALID;
    *out = nullptr;
    bsj_server_config c{};
    if (cfg) c = *cfg;
    if (c.max_inflight <= 0) c.max_inflight = 32;
    if (c.max_inflight > 256) return BSJ_ERR_LIMIT;
    bsj_server* s = new bsj_server();
    bsj_status st = bsj_create(&s->ctx, device);
    if (st == BSJ_OK) st = bsj_create(&s->est_ctx, device);
    if (st != BSJ_OK) {
        if (s->ctx) bsj_destroy(s->ctx);
        delete s;
        return st;
    }
    s->device = device < 0 ? 0 : device;
    cudaGetDevice(&s->device);
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        bsj_destroy(s->est_ctx);
        bsj_destroy(s->ctx);
        delete s;
        return BSJ_ERR_CUDA;
    }
    s->budget = c.memory_budget > 0 ? c.memory_budget : (int64_t)(free_b / 4 * 3);
    if (c.cluster_inflight > 0) {
        s->cluster_inflight = c.cluster_inflight;
    } else if (c.cluster_inflight == 0) {
        int sms = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
        s->cluster_inflight = sms / 8;
    } else {
        s->cluster_inflight = -1;
    }
    s->slots.resize((size_t)c.max_inflight);
    for (Slot& sl : s->slots) {
        if (cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) {
            bsj_server_destroy(s);
            return BSJ_ERR_CUDA;
        }
    }
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return BSJ_OK;
}

void bsj_server_destroy(bsj_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->pending.clear();
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    cudaSetDevice(s->device);
    for (auto& kv : s->idle)
        for (bsj_plan* p : kv.second) bsj_plan_destroy(p);
    for (Slot& sl : s->slots) {
        if (sl.plan) bsj_plan_destroy(sl.plan);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (s->ctx) bsj_destroy(s->ctx);
    if (s->est_ctx) bsj_destroy(s->est_ctx);
    delete s;
}

static bsj_status intake(bsj_server* s, const bsj_instance* inst, const bsj_beam* beam, uint64_t* ticket,
                         int32_t prepare_copies)
{
    if (!s || !inst || !beam || !inst->machine || !inst->duration) return BSJ_ERR_INVALID;
    if (inst->n < 1 || inst->m < 1 || inst->n > BSJ_MAX_JOBS || inst->m > BSJ_MAX_MACHINES ||
        (int64_t)inst->n * inst->m > BSJ_MAX_OPS)
        return BSJ_ERR_LIMIT;
    Request r;
    r.n = inst->n;
    r.m = inst->m;
    const size_t N = (size_t)inst->n * inst->m;
    r.machine.assign(inst->machine, inst->machine + N);
    r.duration.assign(inst->duration, inst->duration + N);
    r.beam = *beam;
    r.beam.instance = 0;
    r.beam.bound_group = -1;
    r.shape = shape_of(r);
    bsj_instance view{r.n, r.m, r.machine.data(), r.duration.data()};
    {
        // footprint check and input validation, without allocating
        std::lock_guard<std::mutex> lk(s->mu);
        bsj_status st = bsj_plan_estimate(s->est_ctx, 1, &view, 1, &r.beam, &r.bytes);
        if (st != BSJ_OK) return st;
        if (r.bytes > s->budget) return BSJ_ERR_LIMIT;
        r.submitted = Clock::now();
        if (prepare_copies > 0) {
            r.prepare = true;
            for (int32_t k = 0; k < prepare_copies; k++) s->pending.push_back(r);
        } else {
            r.ticket = s->next_ticket++;
            *ticket = r.ticket;
            s->live[r.ticket] = 1;
            s->stats.submitted++;
            s->pending.push_back(std::move(r));
        }
    }
    s->cv_work.notify_one();
    return BSJ_OK;
}

bsj_status bsj_submit(bsj_server* s, const bsj_instance* inst, const bsj_beam* beam, uint64_t* ticket)
{
    if (!ticket) return BSJ_ERR_INVALID;
    return intake(s, inst, beam, ticket, 0);
}

bsj_status bsj_server_prepare(bsj_server* s, const bsj_instance* inst, const bsj_beam* beam, int32_t copies)
{
    if (copies < 1 || copies > 256) return BSJ_ERR_INVALID;
    return intake(s, inst, beam, nullptr, copies);
}

static void hand_out(Done& d, bsj_result* result, bsj_request_times* times)
{
    if (result) {
        int32_t* keep = result->sequence;
        *result = d.result;
        result->sequence = keep;
        if (keep) std::memcpy(keep, d.seq.data(), d.seq.size() * sizeof(int32_t));
    }
    if (times) *times = d.times;
}

bsj_status bsj_poll(bsj_server* s, uint64_t ticket, bsj_result* result, bsj_request_times* times, int32_t* done)
{
    if (!s || !done) return BSJ_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->live.count(ticket)) return BSJ_ERR_INVALID;
    auto it = s->finished.find(ticket);
    if (it == s->finished.end()) {
        *done = 0;
        return BSJ_OK;
    }
    *done = 1;
    const bsj_status st = it->second.status;
    hand_out(it->second, result, times);
    s->finished.erase(it);
    s->live.erase(ticket);
    return st;
}

bsj_status bsj_wait(bsj_server* s, uint64_t ticket, bsj_result* result, bsj_request_times* times)
{
    if (!s) return BSJ_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->live.count(ticket)) return BSJ_ERR_INVALID;
    s->cv_done.wait(lk, [&] { return s->finished.count(ticket) > 0; });
    auto it = s->finished.find(ticket);
    const bsj_status st = it->second.status;
    hand_out(it->second, result, times);
    s->finished.erase(it);
    s->live.erase(ticket);
    return st;
}

bsj_status bsj_server_get_stats(bsj_server* s, bsj_server_stats* out)
{
    if (!s || !out) return BSJ_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->stats;
    out->budget_bytes = s->budget;
    out->pending = (int64_t)s->pending.size();
    return BSJ_OK;
}

}  // extern "C"
