// Many independent k-Shape jobs on one GPU: a worker pool for batches and a
// continuous-batching request loop.  No counterpart in the reference (one job per
// process, Code/test/test_kshape.cu).
//
// Each worker is a context (its own stream and workspace) driven by its own host
// thread; the loop of each job replays its iteration stages from CUDA graphs, so
// jobs of different sizes overlap on the device: a small job's stages fill the
// SMs a large job's stages leave idle, and no job waits for another's host
// synchronisations.
//
// Admission keeps the bytes held by the workers' workspaces (grow-only device
// buffers) within the budget.  A running job may grow its worker's buffers by up
// to its footprint, so while it runs that much is reserved on top of what the
// worker held; when it ends the reservation is replaced by the bytes actually
// held.  A worker may take the oldest queued job with held + reserved +
// footprint <= budget; a job that has waited at the head of the queue for more
// than TIMESC_POOL_HEAD_WAIT_S seconds (default 2) is the only one that may
// start, so small jobs cannot overtake a large one forever.  Idle workers hand
// their workspaces back when that lets a job start (pool_sched.h); a job larger
// than the whole budget is rejected at submission.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "pool_sched.h"
#include "tc_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    const tc_job* job = nullptr;
    tc_result* result = nullptr;
    uint64_t footprint = 0;
    int status = TC_OK;
    bool done = false;
    Clock::time_point submitted, started, finished;
};

// Estimated work of a job (for largest-first batch order): assignment pairs times
// the FFT cost per pair, plus the Gram.
double job_work(const tc_job& j) {
    const int F = tc::fft_size(j.m, j.mode);
    int lg = 0;
    while ((1 << lg) < F) ++lg;
    return (double)j.n * j.k * F * (lg + 1) + (double)j.n * j.m * j.m;
}

}  // namespace

struct tc_pool {
    int device = 0;
    uint64_t budget = 0;
    std::vector<tc_ctx*> ctx;
    std::vector<uint64_t> held;   // workspace bytes per worker
    std::vector<uint64_t> resv;   // growth reserved for the job a worker runs
    std::vector<bool> busy;
    std::vector<std::thread> threads;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<uint64_t> queue;   // tickets in submission order
    std::unordered_map<uint64_t, Request> reqs;
    uint64_t next_ticket = 1;
    int running = 0;
    bool stopping = false;
    double head_wait_s = 2.0;     // after this long at the head of the queue a job has priority

    uint64_t held_total() const {
        uint64_t t = 0;
        for (size_t w = 0; w < held.size(); ++w) t += held[w] + resv[w];
        return t;
    }

    // Under mu: the queued ticket worker w may start (its footprint is then
    // reserved), releasing idle workspaces where that lets a job start (the rules
    // of sched_pick).  0 if none.
    uint64_t pick(int w) {
        for (int pass = 0; pass < 2; ++pass) {
            std::vector<tc::SchedJob> q;
            q.reserve(queue.size());
            const Clock::time_point now = Clock::now();
            for (uint64_t t : queue) {
                const Request& r = reqs[t];
                q.push_back(tc::SchedJob{r.footprint, std::chrono::duration<double>(now - r.submitted).count()});
            }
            tc::SchedWorkers ws;
            ws.budget = budget;
            ws.held = held;
            ws.resv = resv;
            ws.busy = busy;
            const tc::SchedChoice c = tc::sched_pick(q, ws, head_wait_s);
            if (c.index >= 0) {
                auto it = queue.begin() + c.index;
                const uint64_t t = *it;
                resv[w] = reqs[t].footprint;
                queue.erase(it);
                return t;
            }
            if (!c.release_idle || pass == 1) break;
            for (size_t v = 0; v < ctx.size(); ++v)  // idle workers (this one included) hand back their buffers
                if (!busy[v] && held[v] > 0) {
                    cudaSetDevice(device);
                    cudaStreamSynchronize(ctx[v]->own_stream);
                    tc::release_workspace(ctx[v]);
                    held[v] = 0;
                }
        }
        return 0;
    }

    void worker(int w) {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        for (;;) {
            uint64_t t = 0;
            cv_work.wait(lk, [&] { return stopping || (!queue.empty() && (t = pick(w)) != 0); });
            if (t == 0) return;  // stopping with nothing this worker can take
            busy[w] = true;
            ++running;
            Request& r = reqs[t];
            r.started = Clock::now();
            const tc_job* job = r.job;
            tc_result* res = r.result;
            lk.unlock();
            const int st = tc_kshape_run(ctx[w], job, res);
            if (st != TC_OK && std::getenv("TIMESC_TRACE"))
                std::fprintf(stderr, "timesc pool: job failed (%d): %s\n", st, tc_last_error(ctx[w]));
            lk.lock();
            held[w] = tc::workspace_bytes(ctx[w]);
            resv[w] = 0;
            busy[w] = false;
            --running;
            Request& r2 = reqs[t];
            r2.status = st;
            r2.finished = Clock::now();
            r2.done = true;
            cv_done.notify_all();
            cv_work.notify_all();  // memory or a worker came free
        }
    }

    int submit(const tc_job* job, tc_result* result, uint64_t* ticket) {
        Request r;
        r.job = job;
        r.result = result;
        r.footprint = tc_job_footprint(job);
        r.submitted = Clock::now();
        std::lock_guard<std::mutex> lk(mu);
        if (r.footprint > budget) return TC_ERR_REJECTED;
        const uint64_t t = next_ticket++;
        reqs[t] = r;
        queue.push_back(t);
        *ticket = t;
        cv_work.notify_all();
        return TC_OK;
    }

    int wait(uint64_t t, int* status, double* queued_s, double* latency_s) {
        std::unique_lock<std::mutex> lk(mu);
        if (reqs.find(t) == reqs.end()) return TC_ERR_ARG;
        cv_done.wait(lk, [&] { return reqs[t].done; });
        const Request& r = reqs[t];
        if (status) *status = r.status;
        if (queued_s) *queued_s = std::chrono::duration<double>(r.started - r.submitted).count();
        if (latency_s) *latency_s = std::chrono::duration<double>(r.finished - r.submitted).count();
        reqs.erase(t);
        return TC_OK;
    }
};

extern "C" {

uint64_t tc_job_footprint(const tc_job* j) {
    if (!j || j->n <= 0 || j->m < 2 || j->k < 1) return 0;
    const uint64_t n = (uint64_t)j->n, m = (uint64_t)j->m, k = (uint64_t)j->k;
    const uint64_t F = (uint64_t)tc::fft_size(j->m, j->mode);
    const uint64_t ld = (m + 3) & ~3ull;
    const uint64_t Pp = std::max<uint64_t>((n + 63 * k + 63) / 64 * 64, 64);
    uint64_t b = 0;
    b += n * m * 4;                        // normalised series
    b += n * m * 4;                        // members in cluster order
    b += n * 4 * 5;                        // labels, old labels, shifts, distances, permutation
    b += k * m * 4 + k * (F / 2 + 1) * 8;  // centroids, spectra
    b += 10 * k * m * ld * 4;              // Gram matrices, their K-share partials (<= 8), squares
    b += (k * m + k) * 8 + 3 * k * m * 4;  // row sums, power-iteration vectors
    b += k * 8 * 4;                        // counts, offsets, padded offsets, gates
    const uint64_t esize = j->precision == TC_PREC_BF16 ? 2 : 4;
    const uint64_t planes = j->precision == TC_PREC_FP32 ? 2 : 1;
    const uint64_t mp64 = (m + 63) / 64 * 64;
    const uint64_t Psq = std::max<uint64_t>((k * mp64 + 63 * k + 63) / 64 * 64, 64);
    b += std::max(m * Pp * esize * planes, m * Psq * 8);  // Gram operand (members, or the squared matrices)
    const bool screened = j->precision == TC_PREC_FP32 && tc::screen_supported(j->m, (int)F, j->k);
    if ((j->precision != TC_PREC_FP32 && tc::tc_assign_supported(j->m, (int)F, j->k, j->precision)) || screened) {
        const uint64_t mp = (m + 63) / 64 * 64;
        b += n * mp * 2 + n * 4;           // BF16 series and norms
        b += k * (F / 8) * (mp + 56) * 2 + k * 4;  // shifted centroid buffers
    }
    if (screened) b += n * (tc::SCREEN_CAP + 1) * 4;  // candidates
    const bool bounded = k >= 2 && k <= 64 &&
                         (screened || (j->precision != TC_PREC_FP32 &&
                                       tc::tc_assign_supported(j->m, (int)F, j->k, j->precision)));
    if (bounded) {
        const uint64_t mp = (m + 63) / 64 * 64;
        b += k * n * 4 + (k * m + k) * 4 + n * 12 + (n + 2 * k * k) * 4;  // bounds, best bounds, grouping
        b += n * mp * 2 + n * 4 + ((n + 127) / 128) * 8;                  // grouped BF16 copy, tile masks
        if (screened) b += n * 8 + k * m * 4 + k;                          // FP32 labels, distances, centroids
    }
    b += n * 4 + 3 * k * m * 4 + 3 * k + 64;  // extraction memo
    b += ((n + 4095) / 4096) * k * 4;      // segment chunk counts
    return b + (1u << 20);
}

int tc_pool_create(int device, const tc_pool_opts* opts, tc_pool** out) {
    if (!out) return TC_ERR_ARG;
    *out = nullptr;
    const int workers = opts && opts->workers > 0 ? opts->workers : 8;
    if (workers > 256) return TC_ERR_ARG;
    if (cudaSetDevice(device) != cudaSuccess) {
        cudaGetLastError();
        return TC_ERR_CUDA;
    }
    tc_pool* p = new (std::nothrow) tc_pool();
    if (!p) return TC_ERR_NOMEM;
    p->device = device;
    if (const char* hw = std::getenv("TIMESC_POOL_HEAD_WAIT_S")) p->head_wait_s = std::atof(hw);
    if (opts && opts->hbm_budget_bytes > 0) {
        p->budget = opts->hbm_budget_bytes;
    } else {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            cudaGetLastError();
            delete p;
            return TC_ERR_CUDA;
        }
        p->budget = (uint64_t)(0.8 * (double)fr);
    }
    for (int w = 0; w < workers; ++w) {
        tc_ctx* c = nullptr;
        const int st = tc_create(device, &c);
        if (st != TC_OK) {
            for (tc_ctx* q : p->ctx) tc_destroy(q);
            delete p;
            return st;
        }
        p->ctx.push_back(c);
    }
    p->held.assign(workers, 0);
    p->resv.assign(workers, 0);
    p->busy.assign(workers, false);
    for (int w = 0; w < workers; ++w) p->threads.emplace_back([p, w] { p->worker(w); });
    *out = p;
    return TC_OK;
}

int tc_pool_destroy(tc_pool* p) {
    if (!p) return TC_ERR_ARG;
    {
        std::unique_lock<std::mutex> lk(p->mu);
        p->cv_done.wait(lk, [&] { return p->queue.empty() && p->running == 0; });
        p->stopping = true;
    }
    p->cv_work.notify_all();
    for (auto& t : p->threads) t.join();
    for (tc_ctx* c : p->ctx) tc_destroy(c);
    delete p;
    return TC_OK;
}

int tc_pool_submit(tc_pool* p, const tc_job* job, tc_result* result, uint64_t* ticket) {
    if (!p || !job || !result || !ticket) return TC_ERR_ARG;
    return p->submit(job, result, ticket);
}

int tc_pool_wait(tc_pool* p, uint64_t ticket, int* status, double* queued_s, double* latency_s) {
    if (!p) return TC_ERR_ARG;
    return p->wait(ticket, status, queued_s, latency_s);
}

int tc_pool_stats(tc_pool* p, int* running, int* queued, uint64_t* held_bytes) {
    if (!p) return TC_ERR_ARG;
    std::lock_guard<std::mutex> lk(p->mu);
    if (running) *running = p->running;
    if (queued) *queued = (int)p->queue.size();
    if (held_bytes) *held_bytes = p->held_total();
    return TC_OK;
}

int tc_pool_run_batch(tc_pool* p, const tc_job* jobs, int njobs, tc_result* results, int* statuses) {
    if (!p || njobs < 0 || (njobs > 0 && (!jobs || !results))) return TC_ERR_ARG;
    std::vector<int> order(njobs);
    for (int i = 0; i < njobs; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return job_work(jobs[a]) > job_work(jobs[b]); });
    std::vector<uint64_t> tickets(njobs, 0);
    std::vector<int> st(njobs, TC_OK);
    for (int i : order) st[i] = p->submit(&jobs[i], &results[i], &tickets[i]);
    int first = TC_OK;
    for (int i = 0; i < njobs; ++i) {
        if (st[i] == TC_OK) p->wait(tickets[i], &st[i], nullptr, nullptr);
        if (statuses) statuses[i] = st[i];
        if (first == TC_OK && st[i] != TC_OK) first = st[i];
    }
    return first;
}

}  // extern "C"
