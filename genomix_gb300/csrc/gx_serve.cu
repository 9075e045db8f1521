// gx_serve.cu — graph builds served as they arrive (gx_serve_*).
//
// A server owns `lanes` contexts on one device, each with its own stream and one worker
// thread.  Submitted jobs wait in one FIFO queue.  Whenever a lane is idle it admits, in
// arrival order, every waiting job whose estimated device memory still fits the server's
// budget and the pass's own cap (`pass_bytes`; the oldest job is always admitted when nothing
// else is in flight, so a job larger than the budget still runs, alone), up to `max_batch`
// jobs, and runs them as one gx_batch_run pass.  Every job of a pass finishes when the pass
// does, so the cap keeps small jobs out of a large job's pass: the large one runs on a lane of
// its own while the other lanes keep serving the small ones, and large jobs (above a quarter
// of the cap) never hold every lane at once.  Jobs that arrive while lanes
// are busy are picked up by the next lane to free up: batches form continuously, and the
// passes of different lanes overlap on the device.  Results stay device-resident in their jobs until the caller emits and destroys
// them.  While the server runs a job, the job belongs to it: call nothing on that job until
// gx_serve_poll reports it done.
#include <algorithm>
#include <chrono>
#include <cstddef>
#include <condition_variable>
#include <cstdio>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gxgpu.h"
#include "gx_job_internal.h"

using namespace gxi;

namespace {

double now_ms() {
    using namespace std::chrono;
    return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

// Device bytes a job needs while it runs, from its input size: occurrences ~ text bytes,
// two copies of (key + edge bits), node offsets and counts, read heads, the record stream.
size_t estimate_bytes(const gx_job *j) {
    size_t text = j->text_len;
    for (int m = 0; m < 2; m++)
        for (const std::string &f : j->fastq[m]) text += f.size() / 2;  // a FASTQ record holds its read twice
    const size_t per_byte = j->k > 32 ? 64 : 44;
    return text * per_byte + (64u << 20);
}

struct Ticket {
    gx_job *job = nullptr;
    gx_ctx *home = nullptr;
    size_t est = 0;
    bool large = false;  // estimated above a quarter of pass_bytes
    double t_submit = 0, t_start = 0, t_done = 0;
    gx_status st = GX_OK;
    bool done = false;
};

}  // namespace

struct gx_server {
    int device = 0;
    std::vector<gx_ctx *> lanes;
    std::vector<std::thread> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, Ticket> tickets;
    uint64_t next_id = 1;
    size_t budget = 0, in_use = 0, pass_bytes = 0;
    int max_batch = 64;
    int running = 0;
    int large_passes = 0;  // passes in flight that hold a large job
    bool stop = false;
    gx_serve_stats stats{};
};

static void lane_loop_impl(gx_server *sv, gx_ctx *lane);

// a lane thread must never end the process: report, fail what it holds, stop the lane
static void lane_loop(gx_server *sv, gx_ctx *lane) {
    try {
        lane_loop_impl(sv, lane);
    } catch (const std::exception &e) {
        fprintf(stderr, "gxgpu: serving lane stopped: %s\n", e.what());
    } catch (...) {
        fprintf(stderr, "gxgpu: serving lane stopped: unexpected exception\n");
    }
}

static void lane_loop_impl(gx_server *sv, gx_ctx *lane) {
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        // admit in arrival order while memory lasts
        // Large jobs hold at most lanes - 1 lanes: while they do, an idle lane passes over them
        // (they keep their order among themselves) and admits the small jobs behind them.
        std::vector<uint64_t> take;
        std::vector<size_t> take_pos;
        size_t est = 0;
        bool large = false;
        const int lanes = (int)sv->lanes.size();
        for (;;) {
            take.clear();
            take_pos.clear();
            est = 0;
            large = false;
            size_t pos = 0;
            for (auto it = sv->pending.begin(); it != sv->pending.end(); ++it, ++pos) {
                const uint64_t id = *it;
                if ((int)take.size() >= sv->max_batch) break;
                const Ticket &t = sv->tickets[id];
                if (t.large && lanes > 1 && sv->large_passes >= lanes - 1) continue;
                const size_t e = t.est;
                const bool alone = take.empty() && sv->in_use == 0;
                if (!alone && sv->in_use + est + e > sv->budget) break;  // keep arrival order
                if (!take.empty() && est + e > sv->pass_bytes) break;   // the pass is full
                take.push_back(id);
                take_pos.push_back(pos);
                est += e;
                large = large || t.large;
            }
            if (!take.empty() || (sv->stop && sv->pending.empty())) break;
            sv->cv_work.wait(lk);
        }
        if (take.empty()) return;  // stopping, nothing left
        for (size_t q = take_pos.size(); q-- > 0;) sv->pending.erase(sv->pending.begin() + (long)take_pos[q]);
        if (large) sv->large_passes++;
        sv->in_use += est;
        sv->running += (int)take.size();
        std::vector<gx_job *> jobs;
        const double t0 = now_ms();
        for (uint64_t id : take) {
            Ticket &t = sv->tickets[id];
            t.t_start = t0;
            t.job->ctx = lane;  // the lane's stream runs it
            jobs.push_back(t.job);
        }
        sv->stats.batches++;
        if (take.size() > sv->stats.max_batch_jobs) sv->stats.max_batch_jobs = take.size();
        lk.unlock();
        std::vector<gx_status> st(jobs.size(), GX_ECUDA);
        gx_batch_run(lane, jobs.data(), (int)jobs.size(), st.data());  // exception-safe
        const double t1 = now_ms();
        lk.lock();
        for (size_t q = 0; q < take.size(); q++) {
            Ticket &t = sv->tickets[take[q]];
            t.job->ctx = t.home;  // every result is complete on the device: the lane synchronized
            t.st = st[q];
            t.t_done = t1;
            t.done = true;
        }
        sv->in_use -= est;
        if (large) sv->large_passes--;
        sv->running -= (int)take.size();
        sv->stats.jobs_done += take.size();
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
}

extern "C" {

static gx_status serve_create_impl(gx_ctx *ctx, const gx_serve_opts *opts, gx_server **out);

gx_status gx_serve_create(gx_ctx *ctx, const gx_serve_opts *opts, gx_server **out) {
    return guarded("gx_serve_create", [&] { return serve_create_impl(ctx, opts, out); });
}

static gx_status serve_create_impl(gx_ctx *ctx, const gx_serve_opts *opts, gx_server **out) {
    if (!ctx || !out) return GX_EINVAL;
    // callers built against the struct before pass_bytes existed pass the shorter size
    if (opts && opts->struct_size < offsetof(gx_serve_opts, pass_bytes)) return GX_EINVAL;
    const bool has_pass = opts && opts->struct_size >= offsetof(gx_serve_opts, pass_bytes) + sizeof(size_t);
    *out = nullptr;
    gx_server *sv = new (std::nothrow) gx_server();
    if (!sv) return GX_ENOMEM;
    sv->device = ctx->device;
    const int lanes = opts && opts->lanes > 0 ? opts->lanes : 4;
    sv->max_batch = opts && opts->max_batch > 0 ? opts->max_batch : 64;
    sv->budget = opts && opts->mem_budget ? opts->mem_budget : ctx->mem_limit;
    sv->pass_bytes = has_pass && opts->pass_bytes ? opts->pass_bytes : (2ull << 30);
    for (int i = 0; i < lanes; i++) {
        gx_ctx_opts co{sizeof(gx_ctx_opts), ctx->mem_limit, 0, ctx->test_alloc_fail_above};
        gx_ctx *c = nullptr;
        const gx_status st = gx_ctx_create(ctx->device, &co, &c);
        if (st != GX_OK) {
            for (gx_ctx *l : sv->lanes) gx_ctx_destroy(l);
            delete sv;
            return st;
        }
        sv->lanes.push_back(c);
    }
    for (gx_ctx *l : sv->lanes) sv->workers.emplace_back(lane_loop, sv, l);
    *out = sv;
    return GX_OK;
}

static gx_status serve_submit_impl(gx_server *sv, gx_job *j, uint64_t *ticket);

gx_status gx_serve_submit(gx_server *sv, gx_job *j, uint64_t *ticket) {
    return guarded("gx_serve_submit", [&] { return serve_submit_impl(sv, j, ticket); });
}

static gx_status serve_submit_impl(gx_server *sv, gx_job *j, uint64_t *ticket) {
    if (!sv || !j || !ticket) return GX_EINVAL;
    if (j->ctx->device != sv->device) return GX_EINVAL;
    if (j->state != JS_INPUT) return GX_ESTATE;
    {
        // the job's inputs were queued on its own context's stream: they must have landed
        std::lock_guard<std::mutex> lk(j->ctx->mu);
        cudaSetDevice(j->ctx->device);
        if (cudaStreamSynchronize(j->ctx->stream) != cudaSuccess) return GX_ECUDA;
    }
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->stop) return GX_EBUSY;
    const uint64_t id = sv->next_id++;
    Ticket t;
    t.job = j;
    t.home = j->ctx;
    t.est = estimate_bytes(j);
    t.large = t.est > sv->pass_bytes / 4;
    t.t_submit = now_ms();
    sv->tickets[id] = t;
    sv->pending.push_back(id);
    sv->stats.jobs_submitted++;
    *ticket = id;
    sv->cv_work.notify_one();
    return GX_OK;
}

static gx_status serve_poll_impl(gx_server *sv, uint64_t ticket, int timeout_ms, gx_status *job_status,
                        double *latency_ms);

gx_status gx_serve_poll(gx_server *sv, uint64_t ticket, int timeout_ms, gx_status *job_status,
                        double *latency_ms) {
    return guarded("gx_serve_poll", [&] { return serve_poll_impl(sv, ticket, timeout_ms, job_status, latency_ms); });
}

static gx_status serve_poll_impl(gx_server *sv, uint64_t ticket, int timeout_ms, gx_status *job_status,
                        double *latency_ms) {
    if (!sv) return GX_EINVAL;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return GX_EINVAL;
    auto ready = [&] { return sv->tickets[ticket].done; };
    if (!ready()) {
        if (timeout_ms == 0) return GX_EAGAIN;
        if (timeout_ms < 0)
            sv->cv_done.wait(lk, ready);
        else if (!sv->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready))
            return GX_EAGAIN;
    }
    const Ticket t = sv->tickets[ticket];
    sv->tickets.erase(ticket);
    if (job_status) *job_status = t.st;
    if (latency_ms) *latency_ms = t.t_done - t.t_submit;
    return GX_OK;
}

gx_status gx_serve_cancel(gx_server *sv, uint64_t ticket) {
    if (!sv) return GX_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return GX_EINVAL;
    Ticket &t = it->second;
    if (t.done) return GX_ESTATE;
    auto q = std::find(sv->pending.begin(), sv->pending.end(), ticket);
    if (q == sv->pending.end()) return GX_EBUSY;  // admitted: it runs to the end
    sv->pending.erase(q);
    t.st = GX_ECANCELLED;
    t.t_done = now_ms();
    t.done = true;
    sv->stats.jobs_cancelled++;
    sv->cv_done.notify_all();
    return GX_OK;
}

gx_status gx_serve_stats_get(gx_server *sv, gx_serve_stats *out) {
    if (!sv || !out) return GX_EINVAL;
    std::lock_guard<std::mutex> lk(sv->mu);
    *out = sv->stats;
    out->jobs_waiting = sv->pending.size();
    out->jobs_running = (uint64_t)sv->running;
    out->bytes_in_use = sv->in_use;
    return GX_OK;
}

void gx_serve_destroy(gx_server *sv) {
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;  // queued jobs still run
        sv->cv_work.notify_all();
    }
    for (std::thread &t : sv->workers) t.join();
    for (gx_ctx *l : sv->lanes) gx_ctx_destroy(l);
    delete sv;
}

}  // extern "C"
