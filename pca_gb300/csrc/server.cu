/*
 * server.cu -- pcagb_server: continuous solve serving on one GPU.
 *
 * The reference solves one task per process run (tools/enumerate.c,
 * gpu/hybrid.cu:631-836) and has no serving loop. This server takes solve
 * requests of any input count, test count and depth as they arrive:
 *
 *   - Admission by free HBM. One device pool is allocated at creation; a
 *     solve reserves an arena slice from it (first fit, coalescing on
 *     release) and a queued request is admitted as soon as a worker is idle
 *     and the pool holds its slice, not when an earlier batch ends. Requests
 *     are admitted in arrival order; when the pool cannot hold the next
 *     one, it waits until a running solve releases memory.
 *   - Concurrent solves. Each worker thread drives one engine on its own
 *     CUDA stream, so the kernels of different solves overlap on the device;
 *     a worker that finds several requests queued takes the head request and
 *     up to max_batch - 1 more of the same test width (16 or 32) in arrival
 *     order into one batched solve (shared launches, one arena).
 *   - Per-request delivery. A request's answer is stored as soon as its own
 *     task is decided, before its batch ends, and pcagb_server_next hands
 *     out completions in the order they happen.
 *   - No device-side waits. Every wait here is a host condition variable
 *     with a timeout; kernels never poll host memory, so no request can leave
 *     a kernel spinning on the GPU.
 *
 * Every answer is the one the task gets alone: a solve's levels, OEP tables
 * and test order live in its own arena and are keyed by task, and
 * first-only answers (the proven optimal depth and the DFS-first program)
 * do not depend on the batch or the split the autotuner picks.
 */
#include <cuda_runtime.h>

#include <chrono>
#include <condition_variable>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/pca_gb300.h"

extern "C" int pcagb_internal_engine_create_bare(int device, pcagb_engine_t **out);
extern "C" int pcagb_internal_solve_batch_arena(pcagb_engine_t *e, void *arena, size_t bytes,
                                                const task_spec_t *tasks, const int *max_depths,
                                                int ntasks, const pcagb_opts_t *opts,
                                                pcagb_result_t *results, uint16_t *sol_progs,
                                                int *sol_lens, int cap, pcagb_done_cb on_done,
                                                void *user);

namespace {

thread_local char t_srv_err[256];

void srv_err(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_srv_err, sizeof t_srv_err, fmt, ap);
    va_end(ap);
}

struct Req {
    uint64_t id = 0;
    task_spec_t task{};
    int max_depth = 4;
    double t_submit = 0, t_admit = -1, t_done = -1;
    int batch = 0;
    bool done = false;
    int rc = 0;
    pcagb_result_t res{};
    std::vector<uint16_t> progs;
    std::vector<int> lens;
};

/* First-fit allocator over [0, size) of the device pool. */
struct Pool {
    char *base = nullptr;
    size_t size = 0, used = 0, peak = 0;
    std::map<size_t, size_t> free_;   /* offset -> length */

    bool alloc(size_t n, size_t *off)
    {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < n) continue;
            *off = it->first;
            const size_t rest = it->second - n;
            const size_t at = it->first + n;
            free_.erase(it);
            if (rest) free_[at] = rest;
            used += n;
            if (used > peak) peak = used;
            return true;
        }
        return false;
    }
    void release(size_t off, size_t n)
    {
        used -= n;
        auto it = free_.emplace(off, n).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t largest() const
    {
        size_t m = 0;
        for (const auto &f : free_) m = f.second > m ? f.second : m;
        return m;
    }
};

}  // namespace

struct pcagb_server {
    pcagb_server_config_t cfg{};
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<Req>> queue;
    std::unordered_map<uint64_t, std::shared_ptr<Req>> reqs;
    std::deque<uint64_t> completed;   /* done, not yet handed out by next() */
    Pool pool;
    int running = 0;
    bool stop = false;
    uint64_t next_id = 1, admitted = 0, finished = 0, batches = 0;
    int max_running = 0;
    std::vector<std::thread> workers;
    std::vector<pcagb_engine_t *> engines;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();

    double now() const
    {
        return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
    void worker(int w);
};

namespace {

struct BatchCtx {
    pcagb_server *s;
    std::vector<std::shared_ptr<Req>> *batch;
    std::vector<uint16_t> *progs;
    std::vector<int> *lens;
    int cap;
};

/* Called by the engine as soon as task i of the batch is decided. */
void on_task_done(int i, const pcagb_result_t *r, void *user)
{
    BatchCtx &c = *(BatchCtx *)user;
    std::lock_guard<std::mutex> lk(c.s->mu);
    Req &q = *(*c.batch)[i];
    q.res = *r;
    const int n = r->stored < c.cap ? r->stored : c.cap;
    q.progs.assign(c.progs->begin() + (size_t)i * c.cap * 16,
                   c.progs->begin() + ((size_t)i * c.cap + n) * 16);
    q.lens.assign(c.lens->begin() + (size_t)i * c.cap, c.lens->begin() + (size_t)i * c.cap + n);
    q.t_done = c.s->now();
    q.done = true;
    c.s->finished++;
    c.s->completed.push_back(q.id);
    c.s->cv_done.notify_all();
}

}  // namespace

void pcagb_server::worker(int w)
{
    pcagb_engine_t *eng = engines[w];
    const size_t per = cfg.arena_bytes;
    for (;;) {
        std::vector<std::shared_ptr<Req>> batch;
        size_t off = 0, bytes = 0;
        {
            std::unique_lock<std::mutex> lk(mu);
            for (;;) {
                if (queue.empty()) {
                    if (stop) return;
                    cv_work.wait_for(lk, std::chrono::milliseconds(200));
                    continue;
                }
                /* the head request's slice, or a batch's: the queued requests
                   up to max_batch share one solve and one arena of up to four
                   slices (their levels hold all their tasks) */
                const size_t k = queue.size() < (size_t)cfg.max_batch ? queue.size()
                                                                      : (size_t)cfg.max_batch;
                const size_t want = per * (k < 4 ? k : 4);
                if (pool.alloc(want, &off)) {
                    bytes = want;
                } else if (pool.alloc(per, &off)) {
                    bytes = per;
                } else if (running == 0) {
                    /* nothing will release memory: the pool cannot hold one */
                    std::shared_ptr<Req> r = queue.front();
                    queue.pop_front();
                    r->rc = PCAGB_ENOMEM;
                    r->done = true;
                    r->t_done = now();
                    finished++;
                    completed.push_back(r->id);
                    cv_done.notify_all();
                    continue;
                } else {
                    cv_work.wait_for(lk, std::chrono::milliseconds(200));
                    continue;
                }
                /* the head request, then (with room for a batch) the queued
                   requests of its test width in arrival order: a batch's
                   states hold the width of its widest task, so a 16-test task
                   in a 32-wide batch would do twice its work */
                const size_t take = bytes == per ? 1 : k;
                const bool wide = queue.front()->task.num_tests > 16;
                batch.push_back(queue.front());
                queue.pop_front();
                for (auto it = queue.begin(); it != queue.end() && batch.size() < take;) {
                    if (((*it)->task.num_tests > 16) == wide) {
                        batch.push_back(*it);
                        it = queue.erase(it);
                    } else {
                        ++it;
                    }
                }
                break;
            }
            const double t = now();
            for (auto &r : batch) {
                r->t_admit = t;
                r->batch = (int)batch.size();
            }
            admitted += batch.size();
            batches++;
            running++;
            if (running > max_running) max_running = running;
        }
        const int n = (int)batch.size();
        const int cap = cfg.sol_cap > 0 ? cfg.sol_cap : 1;
        std::vector<task_spec_t> tasks(n);
        std::vector<int> depths(n);
        for (int i = 0; i < n; i++) {
            tasks[i] = batch[i]->task;
            depths[i] = batch[i]->max_depth;
        }
        std::vector<pcagb_result_t> results(n);
        std::vector<uint16_t> progs((size_t)n * cap * 16, 0);
        std::vector<int> lens((size_t)n * cap, 0);
        BatchCtx ctx{this, &batch, &progs, &lens, cap};
        const int rc = pcagb_internal_solve_batch_arena(
            eng, pool.base + off, bytes, tasks.data(), depths.data(), n, &cfg.opts,
            results.data(), progs.data(), lens.data(), cap, on_task_done, &ctx);
        {
            std::lock_guard<std::mutex> lk(mu);
            /* a failed solve answers every request it leaves open */
            for (auto &r : batch) {
                if (r->done) continue;
                r->rc = rc ? rc : PCAGB_ELIMIT;
                r->done = true;
                r->t_done = now();
                finished++;
                completed.push_back(r->id);
            }
            pool.release(off, bytes);
            running--;
        }
        cv_done.notify_all();
        cv_work.notify_all();
    }
}

extern "C" {

const char *pcagb_server_last_error(void) { return t_srv_err; }

void pcagb_server_default_config(pcagb_server_config_t *c)
{
    memset(c, 0, sizeof *c);
    c->device = 0;
    c->pool_bytes = 0;
    c->arena_bytes = 1ull << 30;
    c->workers = 8;
    c->max_batch = 64;
    c->sol_cap = 16;
    pcagb_default_opts(&c->opts);
    c->opts.first_only = 1;
}

int pcagb_server_create(const pcagb_server_config_t *cfg, pcagb_server_t **out)
{
    t_srv_err[0] = 0;
    if (!cfg || !out) { srv_err("null argument"); return PCAGB_EINVAL; }
    *out = nullptr;
    if (cfg->workers < 1 || cfg->workers > 64 || cfg->max_batch < 1 || cfg->max_batch > 8192 ||
        cfg->arena_bytes < (16u << 20)) {
        srv_err("bad server config (workers 1..64, max_batch 1..8192, arena_bytes >= 16 MiB)");
        return PCAGB_EINVAL;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || cfg->device < 0 || cfg->device >= ndev) {
        cudaGetLastError();
        srv_err("no CUDA device %d: the PCA-16 engine runs only on the GPU", cfg->device);
        return PCAGB_ENODEV;
    }
    pcagb_server *s = new pcagb_server();
    s->cfg = *cfg;
    /* several workers run their solves at once: none of them times its
       stages alone */
    if (cfg->workers > 1) s->cfg.opts.shared_gpu = 1;
    if (cudaSetDevice(cfg->device) != cudaSuccess) {
        srv_err("cudaSetDevice(%d) failed", cfg->device);
        delete s;
        return PCAGB_ECUDA;
    }
    for (int w = 0; w < cfg->workers; w++) {
        pcagb_engine_t *e = nullptr;
        const int rc = pcagb_internal_engine_create_bare(cfg->device, &e);
        if (rc) {
            srv_err("engine for worker %d: %s", w, pcagb_last_error());
            for (pcagb_engine_t *x : s->engines) pcagb_engine_destroy(x);
            delete s;
            return rc;
        }
        s->engines.push_back(e);
    }
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    size_t pool = cfg->pool_bytes ? cfg->pool_bytes : (size_t)(free_b * 0.8);
    if (pool > free_b) pool = free_b;
    pool &= ~size_t(4095);
    if (pool < cfg->arena_bytes || cudaMalloc(&s->pool.base, pool) != cudaSuccess) {
        cudaGetLastError();
        srv_err("device pool of %zu bytes unavailable (arena %zu bytes)", pool,
                (size_t)cfg->arena_bytes);
        for (pcagb_engine_t *x : s->engines) pcagb_engine_destroy(x);
        delete s;
        return PCAGB_ENOMEM;
    }
    s->pool.size = pool;
    s->pool.free_[0] = pool;
    s->cfg.pool_bytes = pool;
    for (int w = 0; w < cfg->workers; w++)
        s->workers.emplace_back([s, w, dev = cfg->device] {
            cudaSetDevice(dev);
            s->worker(w);
        });
    *out = s;
    return PCAGB_OK;
}

int pcagb_server_submit(pcagb_server_t *s, const task_spec_t *task, int max_depth, uint64_t *id)
{
    if (!s || !task || !id) { srv_err("null argument"); return PCAGB_EINVAL; }
    auto r = std::make_shared<Req>();
    r->task = *task;
    r->max_depth = max_depth;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) { srv_err("the server is closed"); return PCAGB_EINVAL; }
        r->id = s->next_id++;
        r->t_submit = s->now();
        s->reqs[r->id] = r;
        s->queue.push_back(r);
        *id = r->id;
    }
    s->cv_work.notify_one();
    return PCAGB_OK;
}

int pcagb_server_next(pcagb_server_t *s, double timeout_s, uint64_t *id)
{
    if (!s || !id) { srv_err("null argument"); return PCAGB_EINVAL; }
    std::unique_lock<std::mutex> lk(s->mu);
    const auto until = std::chrono::steady_clock::now() +
                       std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                           std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0));
    while (s->completed.empty()) {
        if (s->cv_done.wait_until(lk, until) == std::cv_status::timeout && s->completed.empty())
            return 0;
    }
    *id = s->completed.front();
    s->completed.pop_front();
    return 1;
}

int pcagb_server_collect(pcagb_server_t *s, uint64_t id, pcagb_result_t *res, uint16_t *progs,
                         int *lens, int cap, double *times)
{
    if (!s) { srv_err("null argument"); return PCAGB_EINVAL; }
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(id);
    if (it == s->reqs.end() || !it->second->done) {
        srv_err("request %llu is unknown, already collected or not done",
                (unsigned long long)id);
        return PCAGB_EINVAL;
    }
    Req &r = *it->second;
    if (res) *res = r.res;
    const int n = (int)r.lens.size() < cap ? (int)r.lens.size() : cap;
    if (progs && n > 0) memcpy(progs, r.progs.data(), (size_t)n * 16 * sizeof(uint16_t));
    if (lens && n > 0) memcpy(lens, r.lens.data(), (size_t)n * sizeof(int));
    if (res) res->stored = n;
    if (times) {
        times[0] = r.t_submit;
        times[1] = r.t_admit;
        times[2] = r.t_done;
        times[3] = (double)r.batch;
    }
    const int rc = r.rc;
    if (rc) srv_err("request %llu failed (%d)", (unsigned long long)id, rc);
    s->reqs.erase(it);
    return rc;
}

int pcagb_server_stats(pcagb_server_t *s, pcagb_server_stats_t *st)
{
    if (!s || !st) { srv_err("null argument"); return PCAGB_EINVAL; }
    std::lock_guard<std::mutex> lk(s->mu);
    st->queued = s->queue.size();
    st->running_solves = s->running;
    st->max_running_solves = s->max_running;
    st->admitted = s->admitted;
    st->finished = s->finished;
    st->batches = s->batches;
    st->pool_bytes = s->pool.size;
    st->pool_used = s->pool.used;
    st->pool_peak = s->pool.peak;
    st->pool_largest_free = s->pool.largest();
    return PCAGB_OK;
}

void pcagb_server_destroy(pcagb_server_t *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &t : s->workers) t.join();
    for (pcagb_engine_t *e : s->engines) pcagb_engine_destroy(e);
    if (s->pool.base) cudaFree(s->pool.base);
    delete s;
}

}  // extern "C"
