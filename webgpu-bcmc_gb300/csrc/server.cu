// server.cu -- continuous-batching isosurface server over a batched engine
// (bcmc_server_* in include/bcmc.h).  Host code only: a worker thread owns the
// engine; clients submit (volume, isovalue) requests from any thread.
//
// The worker keeps up to two batches on the device.  Whenever a lane of batch
// buffers is free it takes every request that has arrived (up to max_batch;
// with nothing in flight, after an optional short wait for company) and
// launches them as one batch without waiting for it.  So requests that arrive
// while a batch is on the GPU go out at once in the next one: its active test,
// cache claims and decode run while the first batch's marching cubes do, and
// its marching cubes follow on the device.  A batch's completion (a host
// callback after its results reach the host) wakes the worker, which hands the
// results to their waiters.  Admission by memory: a batch whose active blocks
// do not fit the slot pool, or whose vertex count (known after the count
// pass) does not fit the vertex budget, is run again on its own; the longest
// prefix that fits is answered and the rest goes back to the front of the
// queue.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <random>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "bcmc_impl.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t ticket;
    uint32_t volume;
    float iso;
    void* host;
    uint64_t host_capacity;
    Clock::time_point arrive;
};

struct Done {
    bcmc_status status;
    bcmc_query_result result;
    double latency_ms;
};

}  // namespace

struct bcmc_server {
    bcmc_engine* eng = nullptr;
    bcmc_server_opts opts{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request> pending;
    std::unordered_map<uint64_t, Done> done;
    std::unordered_set<uint64_t> unclaimed;  // submitted, not yet waited for
    uint64_t next_ticket = 1;
    bool stop = false;
    bool lane_done[2] = {false, false};  // set by the completion callback
    std::thread worker;
    uint64_t batches = 0, batched_requests = 0, overlapped = 0;
    double avg_verts = 0.0;  // worker only
};

namespace {

struct LaneDone {
    bcmc_server* s;
    int lane;
};

// Runs on a CUDA host thread once a batch's results are on the host.
void on_lane_done(void* p)
{
    LaneDone* d = static_cast<LaneDone*>(p);
    {
        std::lock_guard<std::mutex> lk(d->s->mu);
        d->s->lane_done[d->lane] = true;
    }
    d->s->cv_work.notify_all();
}

struct InFlight {
    int lane;
    std::vector<Request> batch;
};

// Hands a batch's outcome to its waiters (under the lock).
void finish_batch(bcmc_server* s, std::vector<Request>& batch, const std::vector<bcmc_query_result>& res,
                  bcmc_status st)
{
    const Clock::time_point t = Clock::now();
    ++s->batches;
    s->batched_requests += batch.size();
    if (st == BCMC_OK)
        for (size_t i = 0; i < batch.size(); ++i)  // running mean of vertices per request
            s->avg_verts = s->avg_verts == 0.0 ? (double)res[i].num_vertices + 1.0
                                               : 0.98 * s->avg_verts + 0.02 * (double)res[i].num_vertices;
    for (size_t i = 0; i < batch.size(); ++i) {
        Done d;
        d.status = st;
        d.result = st == BCMC_OK ? res[i] : bcmc_query_result{};
        d.result.vertex_offset = 0;
        d.latency_ms = std::chrono::duration<double, std::milli>(t - batch[i].arrive).count();
        s->done[batch[i].ticket] = d;
    }
}

void worker_loop(bcmc_server* s)
{
    cudaSetDevice(bcmc::engine_device(s->eng));
    std::deque<InFlight> inflight;  // oldest first, at most two
    LaneDone cb[2] = {{s, 0}, {s, 1}};
    std::vector<bcmc_query> qs;
    std::vector<bcmc_query_result> res;
    for (;;) {
        std::vector<Request> batch;
        int lane = -1;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] {
                const bool can_launch = !s->pending.empty() && inflight.size() < 2;
                const bool oldest_done = !inflight.empty() && s->lane_done[inflight.front().lane];
                return can_launch || oldest_done || (s->stop && inflight.empty());
            });
            if (s->pending.empty() && inflight.empty()) return;  // stop requested and nothing left
            if (!s->pending.empty() && inflight.size() < 2) {
                if (inflight.empty() && s->opts.max_wait_us && s->pending.size() < s->opts.max_batch && !s->stop) {
                    s->cv_work.wait_for(lk, std::chrono::microseconds(s->opts.max_wait_us),
                                        [&] { return s->stop || s->pending.size() >= s->opts.max_batch; });
                }
                // size the batch so that its expected vertex count stays within the
                // engine's vertex budget: an over-full batch would pay a count pass
                // for requests the engine then refuses
                size_t cap_n = std::min<size_t>(s->opts.max_batch, bcmc::engine_max_batch(s->eng));
                const uint64_t budget = bcmc::engine_vertex_budget(s->eng);
                if (budget && s->avg_verts > 0.0)
                    cap_n = std::max<size_t>(1, std::min<size_t>(cap_n, (size_t)(0.8 * (double)budget / s->avg_verts)));
                const size_t n = std::min<size_t>(s->pending.size(), cap_n);
                batch.assign(s->pending.begin(), s->pending.begin() + n);
                s->pending.erase(s->pending.begin(), s->pending.begin() + n);
                lane = inflight.empty() ? 0 : 1 - inflight.front().lane;
                s->lane_done[lane] = false;
                if (!inflight.empty()) ++s->overlapped;
            }
        }
        if (lane >= 0) {  // launch, do not wait
            qs.resize(batch.size());
            for (size_t i = 0; i < batch.size(); ++i) qs[i] = bcmc_query{batch[i].volume, batch[i].iso};
            const bcmc_status st =
                bcmc::engine_submit(s->eng, lane, qs.data(), (uint32_t)qs.size(), on_lane_done, &cb[lane]);
            if (st == BCMC_OK) {
                inflight.push_back(InFlight{lane, std::move(batch)});
            } else {
                std::lock_guard<std::mutex> lk(s->mu);
                finish_batch(s, batch, res, st);
                s->cv_done.notify_all();
            }
            continue;
        }
        // the oldest batch is done: its results to their waiters
        InFlight f = std::move(inflight.front());
        inflight.pop_front();
        res.assign(f.batch.size(), bcmc_query_result{});
        uint32_t admitted = 0;
        bcmc_status st = bcmc::engine_complete(s->eng, f.lane, res.data(), &admitted);
        std::vector<Request> rest;
        if (st == BCMC_OK && admitted < f.batch.size()) {
            rest.assign(f.batch.begin() + admitted, f.batch.end());
            f.batch.resize(admitted);
        }
        if (st == BCMC_OK) {
            for (size_t i = 0; i < f.batch.size() && st == BCMC_OK; ++i) {
                if (!f.batch[i].host || !res[i].num_vertices) continue;
                const uint64_t n = std::min<uint64_t>(res[i].num_vertices, f.batch[i].host_capacity);
                st = bcmc::engine_copy_lane_vertices(s->eng, f.lane, res[i].vertex_offset, n, f.batch[i].host);
            }
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            // the rest did not fit this batch's memory: back to the front of the queue
            if (!rest.empty()) s->pending.insert(s->pending.begin(), rest.begin(), rest.end());
            s->lane_done[f.lane] = false;
            finish_batch(s, f.batch, res, st);
        }
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" bcmc_status bcmc_server_create(bcmc_engine* eng, const bcmc_server_opts* opts, bcmc_server** out)
{
    if (!eng || !out) return BCMC_E_ARG;
    *out = nullptr;
    bcmc_server* s = new (std::nothrow) bcmc_server();
    if (!s) return BCMC_E_OOM;
    s->eng = eng;
    if (opts) s->opts = *opts;
    if (!s->opts.max_batch) s->opts.max_batch = 256;
    try {
        s->worker = std::thread(worker_loop, s);
    } catch (...) {
        delete s;
        return BCMC_E_OOM;
    }
    *out = s;
    return BCMC_OK;
}

extern "C" void bcmc_server_destroy(bcmc_server* s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    bcmc::engine_drain(s->eng);  // the last completion callback has returned
    delete s;
}

extern "C" bcmc_status bcmc_server_submit(bcmc_server* s, uint32_t volume, float isovalue, void* host_vertices,
                                          uint64_t host_capacity, uint64_t* ticket)
{
    if (!s || !ticket || (host_vertices && !host_capacity)) return BCMC_E_ARG;
    // an unknown volume is refused here: in a batch it would fail its batch-mates too
    if (volume >= bcmc::engine_num_volumes(s->eng)) return BCMC_E_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return BCMC_E_STATE;
        *ticket = s->next_ticket++;
        s->unclaimed.insert(*ticket);
        s->pending.push_back(Request{*ticket, volume, isovalue, host_vertices, host_capacity, Clock::now()});
    }
    s->cv_work.notify_one();
    return BCMC_OK;
}

extern "C" bcmc_status bcmc_server_wait(bcmc_server* s, uint64_t ticket, bcmc_query_result* result,
                                        double* latency_ms)
{
    if (!s || !ticket) return BCMC_E_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    // each ticket is waited for once: one never issued or already claimed
    // (whose result is gone) would otherwise block for ever
    if (s->unclaimed.erase(ticket) == 0) return BCMC_E_ARG;
    s->cv_done.wait(lk, [&] { return s->done.count(ticket) != 0; });
    const Done d = s->done[ticket];
    s->done.erase(ticket);
    if (result) *result = d.result;
    if (latency_ms) *latency_ms = d.latency_ms;
    return d.status;
}

extern "C" bcmc_status bcmc_server_run_load(bcmc_server* s, const bcmc_load_spec* spec, bcmc_load_report* out)
{
    if (!s || !spec || !out || !(spec->rate_qps > 0.0) || !spec->requests || !spec->num_volumes || !spec->volumes ||
        !spec->weights || !spec->iso_lo || !spec->iso_hi)
        return BCMC_E_ARG;
    std::mt19937_64 rng(spec->seed);
    std::exponential_distribution<double> gap(spec->rate_qps);
    std::vector<double> w(spec->weights, spec->weights + spec->num_volumes);
    std::discrete_distribution<uint32_t> pick(w.begin(), w.end());
    std::uniform_real_distribution<float> unit(0.0f, 1.0f);
    std::vector<uint64_t> tickets(spec->requests);
    uint64_t batches0, overlapped0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        batches0 = s->batches;
        overlapped0 = s->overlapped;
    }
    const Clock::time_point t0 = Clock::now();
    double at = 0.0;
    for (uint32_t i = 0; i < spec->requests; ++i) {  // open loop: arrivals do not wait for completions
        at += gap(rng);
        const uint32_t k = pick(rng);
        const float iso = spec->iso_lo[k] + unit(rng) * (spec->iso_hi[k] - spec->iso_lo[k]);
        std::this_thread::sleep_until(t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(at)));
        const bcmc_status st = bcmc_server_submit(s, spec->volumes[k], iso, nullptr, 0, &tickets[i]);
        if (st != BCMC_OK) return st;
    }
    std::vector<double> lat(spec->requests);
    uint64_t verts = 0;
    bcmc_status worst = BCMC_OK;
    for (uint32_t i = 0; i < spec->requests; ++i) {
        bcmc_query_result r{};
        const bcmc_status st = bcmc_server_wait(s, tickets[i], &r, &lat[i]);
        if (st != BCMC_OK) worst = st;
        verts += r.num_vertices;
    }
    const double dur = std::chrono::duration<double>(Clock::now() - t0).count();
    std::vector<double> sorted = lat;
    std::sort(sorted.begin(), sorted.end());
    auto pct = [&](double p) {
        const double pos = p / 100.0 * (double)(sorted.size() - 1);
        const size_t lo = (size_t)pos, hi = std::min(lo + 1, sorted.size() - 1);
        return sorted[lo] + (sorted[hi] - sorted[lo]) * (pos - (double)lo);
    };
    double sum = 0.0;
    for (double v : sorted) sum += v;
    bcmc_load_report r{};
    r.offered_qps = spec->rate_qps;
    r.achieved_qps = spec->requests / dur;
    r.p50_ms = pct(50.0);
    r.p95_ms = pct(95.0);
    r.p99_ms = pct(99.0);
    r.mean_ms = sum / sorted.size();
    r.max_ms = sorted.back();
    r.duration_s = dur;
    r.completed = spec->requests;
    r.vertices = verts;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r.batches = s->batches - batches0;
        r.overlapped_batches = s->overlapped - overlapped0;
    }
    r.mean_batch = r.batches ? (double)spec->requests / (double)r.batches : 0.0;
    *out = r;
    return worst;
}
