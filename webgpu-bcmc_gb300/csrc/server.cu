// server.cu -- continuous-batching isosurface server over a batched engine
// (bcmc_server_* in include/bcmc.h).  Host code only: a worker thread owns the
// engine; clients submit (volume, isovalue) requests from any thread.
//
// Whenever the device is free the worker takes every request that has arrived
// (up to max_batch, after an optional short wait for company) and runs them as
// one engine batch; requests arriving meanwhile queue for the next batch.
// Admission by memory: the engine runs the longest prefix of the batch whose
// active blocks fit the slot pool and whose vertex count (known after the
// count pass) fits the vertex budget; the rest goes back to the front of the
// queue for the next batch.
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
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread worker;
    uint64_t batches = 0, batched_requests = 0;
    double avg_verts = 0.0;  // worker only
};

namespace {

void worker_loop(bcmc_server* s)
{
    cudaSetDevice(bcmc::engine_device(s->eng));
    std::vector<Request> batch;
    std::vector<bcmc_query> qs;
    std::vector<bcmc_query_result> res;
    for (;;) {
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->pending.empty(); });
            if (s->pending.empty()) return;  // stop requested and nothing left
            if (s->opts.max_wait_us && s->pending.size() < s->opts.max_batch && !s->stop) {
                s->cv_work.wait_for(lk, std::chrono::microseconds(s->opts.max_wait_us),
                                    [&] { return s->stop || s->pending.size() >= s->opts.max_batch; });
            }
            // size the batch so that its expected vertex count stays within the
            // engine's vertex budget: an over-full batch would pay a count pass
            // for requests the engine then refuses
            size_t cap_n = s->opts.max_batch;
            const uint64_t budget = bcmc::engine_vertex_budget(s->eng);
            if (budget && s->avg_verts > 0.0)
                cap_n = std::max<size_t>(1, std::min<size_t>(cap_n, (size_t)(0.8 * (double)budget / s->avg_verts)));
            const size_t n = std::min<size_t>(s->pending.size(), cap_n);
            batch.assign(s->pending.begin(), s->pending.begin() + n);
            s->pending.erase(s->pending.begin(), s->pending.begin() + n);
        }
        qs.resize(batch.size());
        res.assign(batch.size(), bcmc_query_result{});
        for (size_t i = 0; i < batch.size(); ++i) qs[i] = bcmc_query{batch[i].volume, batch[i].iso};
        uint32_t admitted = 0;
        bcmc_status st = bcmc_engine_run_admit(s->eng, qs.data(), (uint32_t)qs.size(), res.data(), &admitted);
        if (st == BCMC_OK && admitted < batch.size()) {
            // the rest did not fit this batch's memory: back to the front of the queue
            std::lock_guard<std::mutex> lk(s->mu);
            s->pending.insert(s->pending.begin(), batch.begin() + admitted, batch.end());
            batch.resize(admitted);
        }
        if (st == BCMC_OK) {
            for (size_t i = 0; i < batch.size() && st == BCMC_OK; ++i) {
                if (!batch[i].host || !res[i].num_vertices) continue;
                const uint64_t n = std::min<uint64_t>(res[i].num_vertices, batch[i].host_capacity);
                st = bcmc_engine_copy_vertices(s->eng, res[i].vertex_offset, n, batch[i].host);
            }
        }
        const Clock::time_point t = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            ++s->batches;
            s->batched_requests += batch.size();
            if (st == BCMC_OK)
                for (size_t i = 0; i < batch.size(); ++i)  // running mean of vertices per request
                    s->avg_verts = s->avg_verts == 0.0 ? (double)res[i].num_vertices + 1.0
                                                       : 0.98 * s->avg_verts + 0.02 * (double)res[i].num_vertices;
            for (size_t i = 0; i < batch.size(); ++i) {
                Done d;
                d.status = st;
                d.result = res[i];
                d.result.vertex_offset = 0;
                d.latency_ms = std::chrono::duration<double, std::milli>(t - batch[i].arrive).count();
                s->done[batch[i].ticket] = d;
            }
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
    delete s;
}

extern "C" bcmc_status bcmc_server_submit(bcmc_server* s, uint32_t volume, float isovalue, void* host_vertices,
                                          uint64_t host_capacity, uint64_t* ticket)
{
    if (!s || !ticket || (host_vertices && !host_capacity)) return BCMC_E_ARG;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return BCMC_E_STATE;
        *ticket = s->next_ticket++;
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
    if (ticket >= s->next_ticket) return BCMC_E_ARG;
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
    uint64_t batches0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        batches0 = s->batches;
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
    }
    r.mean_batch = r.batches ? (double)spec->requests / (double)r.batches : 0.0;
    *out = r;
    return worst;
}
