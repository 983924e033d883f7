// crgpu_server.cu - a solve server: continuous batching of independent solve requests.
//
// The reference answers one (graph, k, p) per process run.  A server keeps one process and one
// GPU busy with a stream of such requests: requests are queued as they arrive; a pool of
// worker threads, each with its own CUDA stream, takes the first queued request whose device
// footprint (cr_solver_footprint) fits in what the memory budget has left, solves it on its
// stream while the other workers' solves run on theirs, and leaves the finished table
// resident on the device until the client releases it.  A request that arrives while others
// are on the GPU starts as soon as a worker and enough memory are free; nothing waits for a
// batch to fill.  Each result records its queueing, run and total latency.
//
// Small full-visibility requests could also be folded into the batch kernel; the server keeps
// one solver per request so every result is produced by the same code path as cr_solve.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <new>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/crgpu.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr double kMaxOvertakeMs = 2000.0;  // longest a queued request can be overtaken

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

uint64_t mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

enum class State { Queued, Running, Done, Failed };

struct Request {
    uint64_t id = 0;
    int32_t n = 0, k = 0, p = 0, rules = 0;
    std::vector<uint32_t> row_ptr;
    std::vector<uint16_t> col;
    uint64_t footprint = 0;
    State state = State::Queued;
    Clock::time_point t_submit, t_start, t_done;
    cr_request_result res{};
    cr_solver* solver = nullptr;  // resident table until released
    cr_context* owner = nullptr;  // the worker context the solver lives on
    const void* table = nullptr;  // its device table (taken by the worker once the solve is done)
    size_t table_bytes = 0;
    int readers = 0;              // client read-backs in flight; release waits for them
    std::string err;
};

}  // namespace

struct cr_server {
    int device = 0;
    // budget = what requests may hold; reserve = what the workers' contexts may keep of freed
    // solver buffers for reuse (their block caches), set aside from the caller's budget
    uint64_t budget = 0, reserve = 0, in_use = 0, peak_in_use = 0;
    cudaStream_t copy_stream = nullptr;   // client read-backs, apart from the workers' streams
    std::mutex copy_mu;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<std::thread> workers;
    std::vector<cr_context*> contexts;
    uint64_t next_id = 1;
    bool stopping = false;
    uint64_t completed = 0, failed = 0, states_done = 0, running = 0, max_running = 0;
    Clock::time_point t_first_submit, t_last_done;
    bool any_submit = false;
    std::string err;
};

namespace {

// Solve one request on the worker's context (the same phases as cr_solve).
void run_request(cr_server* srv, cr_context* ctx, Request* r) {
    cr_graph g{r->n, r->row_ptr.data(), r->col.data()};
    cr_solver* s = nullptr;
    int rc = cr_solver_create(ctx, &g, r->k, r->p, r->rules, &s);
    uint64_t caps = 0;
    std::vector<uint64_t> counts(1 << 12);
    int32_t passes = 0;
    cr_verdict v{};
    uint64_t digest = 0;
    cr_table_sizes sz{};
    if (!rc) rc = cr_solver_init(s, &caps);
    if (!rc) rc = cr_solver_run(s, counts.data(), (int32_t)counts.size(), &passes);
    if (!rc) rc = cr_solver_verdict(s, &v);
    if (!rc) rc = cr_solver_digest(s, &digest);
    if (!rc) rc = cr_solver_sizes(s, &sz);
    void* table = nullptr;
    size_t table_bytes = 0;
    if (!rc) rc = cr_solver_device_states(s, &table, &table_bytes);
    std::lock_guard<std::mutex> lock(srv->mu);
    r->t_done = Clock::now();
    srv->t_last_done = r->t_done;
    srv->running--;
    r->res.status = rc;
    r->res.queue_ms = ms_between(r->t_submit, r->t_start);
    r->res.run_ms = ms_between(r->t_start, r->t_done);
    r->res.latency_ms = ms_between(r->t_submit, r->t_done);
    if (rc) {
        r->err = cr_context_last_error(ctx);
        r->state = State::Failed;
        srv->failed++;
        if (s) cr_solver_destroy(s);
        srv->in_use -= r->footprint;
    } else {
        r->solver = s;
        r->owner = ctx;
        r->table = table;
        r->table_bytes = table_bytes;
        r->res.win = v.win;
        r->res.capture_plies = v.capture_plies;
        r->res.best_config = v.best_config;
        r->res.passes = passes;
        r->res.base_captures = caps;
        r->res.states = sz.num_states;
        r->res.digest = digest;
        uint64_t h = 0;
        for (int i = 0; i < passes; ++i) h += mix64(counts[i] ^ ((uint64_t)(i + 1) * 0xD1B54A32D192ED03ull));
        r->res.pass_hash = h;
        r->state = State::Done;
        srv->completed++;
        srv->states_done += sz.num_states;
    }
    srv->cv_done.notify_all();
    srv->cv_work.notify_all();  // memory may have been returned
}

void worker_main(cr_server* srv, cr_context* ctx) {
    cudaSetDevice(srv->device);
    for (;;) {
        Request* r = nullptr;
        {
            std::unique_lock<std::mutex> lock(srv->mu);
            for (;;) {
                if (srv->stopping) return;
                // the first queued request that fits in the memory left; earlier ones that do
                // not fit yet keep their place, and once the oldest has waited kMaxOvertakeMs
                // nothing overtakes it any more (so a large request cannot starve)
                const bool head_only = !srv->queue.empty() &&
                    ms_between(srv->queue.front()->t_submit, Clock::now()) > kMaxOvertakeMs;
                for (auto it = srv->queue.begin(); it != srv->queue.end(); ++it) {
                    if (srv->in_use + (*it)->footprint <= srv->budget) {
                        r = *it;
                        srv->queue.erase(it);
                        break;
                    }
                    if (head_only) break;
                }
                if (r) break;
                srv->cv_work.wait_for(lock, std::chrono::milliseconds(50));
            }
            srv->in_use += r->footprint;
            if (srv->in_use > srv->peak_in_use) srv->peak_in_use = srv->in_use;
            srv->running++;
            if (srv->running > srv->max_running) srv->max_running = srv->running;
            r->state = State::Running;
            r->t_start = Clock::now();
        }
        run_request(srv, ctx, r);
    }
}

}  // namespace

extern "C" {

int cr_server_create(int32_t device, uint64_t memory_budget, int32_t workers, cr_server** out) {
    if (!out || workers <= 0 || workers > 256) return CR_ERR_INVALID;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return CR_ERR_CUDA;
    auto* srv = new (std::nothrow) cr_server();
    if (!srv) return CR_ERR_NOMEM;
    srv->device = device;
    if (memory_budget == 0) {
        size_t free_b = 0, total_b = 0;
        cudaMemGetInfo(&free_b, &total_b);
        memory_budget = (uint64_t)(free_b * 0.8);
    }
    // each worker context keeps up to `keep` bytes of freed solver buffers, so that requests of
    // a size it has seen allocate nothing; that memory is set aside from the budget
    const uint64_t keep = std::min<uint64_t>(1ull << 30, memory_budget / (8 * (uint64_t)workers));
    srv->reserve = keep * (uint64_t)workers;
    srv->budget = memory_budget - srv->reserve;
    if (cudaStreamCreateWithFlags(&srv->copy_stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete srv;
        return CR_ERR_CUDA;
    }
    for (int i = 0; i < workers; ++i) {
        cr_context* c = nullptr;
        if (cr_context_create(device, nullptr, &c) != CR_OK || cr_context_set_cache_limit(c, keep) != CR_OK) {
            if (c) cr_context_destroy(c);
            for (cr_context* q : srv->contexts) cr_context_destroy(q);
            cudaStreamDestroy(srv->copy_stream);
            delete srv;
            return CR_ERR_CUDA;
        }
        srv->contexts.push_back(c);
    }
    for (int i = 0; i < workers; ++i) srv->workers.emplace_back(worker_main, srv, srv->contexts[i]);
    *out = srv;
    return CR_OK;
}

int cr_server_submit(cr_server* srv, const cr_graph* g, int32_t k, int32_t p, int32_t rules,
                     uint64_t* request_id) {
    if (!srv || !g || !request_id || g->n <= 0 || !g->row_ptr) return CR_ERR_INVALID;
    auto r = std::make_unique<Request>();
    r->n = g->n;
    r->k = k;
    r->p = p;
    r->rules = rules;
    r->row_ptr.assign(g->row_ptr, g->row_ptr + g->n + 1);
    const uint32_t nnz = g->row_ptr[g->n];
    if (nnz && !g->col_idx) return CR_ERR_INVALID;
    r->col.assign(g->col_idx, g->col_idx + nnz);
    if (r->col.empty()) r->col.push_back(0);
    r->footprint = cr_solver_footprint(g->n, k, p, rules);
    if (r->footprint == 0) return CR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(srv->mu);
    if (r->footprint > srv->budget) {
        srv->err = "request footprint exceeds the server's memory budget";
        return CR_ERR_NOMEM;
    }
    r->id = srv->next_id++;
    r->t_submit = Clock::now();
    if (!srv->any_submit) {
        srv->any_submit = true;
        srv->t_first_submit = r->t_submit;
    }
    *request_id = r->id;
    srv->queue.push_back(r.get());
    srv->reqs.emplace(r->id, std::move(r));
    srv->cv_work.notify_one();
    return CR_OK;
}

int cr_server_poll(cr_server* srv, uint64_t id, int32_t wait_ms, cr_request_result* out) {
    if (!srv || !out) return CR_ERR_INVALID;
    std::unique_lock<std::mutex> lock(srv->mu);
    auto it = srv->reqs.find(id);
    if (it == srv->reqs.end()) return CR_ERR_INVALID;
    Request* r = it->second.get();
    const auto deadline = Clock::now() + std::chrono::milliseconds(wait_ms > 0 ? wait_ms : 0);
    while ((r->state == State::Queued || r->state == State::Running) && wait_ms != 0) {
        if (wait_ms > 0) {
            if (srv->cv_done.wait_until(lock, deadline) == std::cv_status::timeout) break;
        } else {
            srv->cv_done.wait(lock);
        }
    }
    if (r->state == State::Queued || r->state == State::Running) return CR_ERR_STATE;
    *out = r->res;
    if (r->state == State::Failed) {
        srv->err = r->err;
        return r->res.status ? r->res.status : CR_ERR_INTERNAL;
    }
    return CR_OK;
}

// The copy runs on the server's own stream from the client's thread: it touches neither the
// worker's stream (which may be solving the next request) nor its context's error text, and the
// request cannot be released while it runs (release waits for its readers).
int cr_server_read_states(cr_server* srv, uint64_t id, uint8_t* dst, size_t bytes) {
    if (!srv || !dst) return CR_ERR_INVALID;
    Request* r = nullptr;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        auto it = srv->reqs.find(id);
        if (it == srv->reqs.end() || it->second->state != State::Done || !it->second->table)
            return CR_ERR_STATE;
        r = it->second.get();
        if (bytes < r->table_bytes) {
            srv->err = "states buffer smaller than the table";
            return CR_ERR_INVALID;
        }
        r->readers++;
    }
    cudaError_t e;
    {
        std::lock_guard<std::mutex> copy(srv->copy_mu);
        e = cudaSetDevice(srv->device);
        if (e == cudaSuccess) e = cudaMemcpyAsync(dst, r->table, r->table_bytes, cudaMemcpyDeviceToHost, srv->copy_stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(srv->copy_stream);
    }
    std::lock_guard<std::mutex> lock(srv->mu);
    r->readers--;
    srv->cv_done.notify_all();
    if (e != cudaSuccess) {
        srv->err = std::string("table read-back failed: ") + cudaGetErrorString(e);
        return CR_ERR_CUDA;
    }
    return CR_OK;
}

int cr_server_release(cr_server* srv, uint64_t id) {
    if (!srv) return CR_ERR_INVALID;
    std::unique_ptr<Request> r;
    {
        std::unique_lock<std::mutex> lock(srv->mu);
        auto it = srv->reqs.find(id);
        if (it == srv->reqs.end()) return CR_ERR_INVALID;
        if (it->second->state == State::Queued || it->second->state == State::Running) return CR_ERR_STATE;
        Request* q = it->second.get();
        srv->cv_done.wait(lock, [q] { return q->readers == 0; });   // a read-back in flight finishes first
        it = srv->reqs.find(id);
        if (it == srv->reqs.end()) return CR_ERR_INVALID;   // released by another thread meanwhile
        r = std::move(it->second);
        srv->reqs.erase(it);
        if (r->state == State::Done) srv->in_use -= r->footprint;
    }
    if (r->solver) cr_solver_destroy(r->solver);
    std::lock_guard<std::mutex> lock(srv->mu);
    srv->cv_work.notify_all();
    return CR_OK;
}

int cr_server_stats(cr_server* srv, cr_server_report* out) {
    if (!srv || !out) return CR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(srv->mu);
    memset(out, 0, sizeof(*out));
    out->completed = srv->completed;
    out->failed = srv->failed;
    out->queued = srv->queue.size();
    out->running = srv->running;
    out->max_running = srv->max_running;
    out->memory_budget = srv->budget + srv->reserve;
    out->memory_in_use = srv->in_use;
    out->peak_memory_in_use = srv->peak_in_use;
    out->states_done = srv->states_done;
    out->busy_ms = srv->any_submit ? ms_between(srv->t_first_submit, srv->t_last_done) : 0.0;
    return CR_OK;
}

const char* cr_server_last_error(const cr_server* srv) { return srv ? srv->err.c_str() : ""; }

int cr_server_destroy(cr_server* srv) {
    if (!srv) return CR_OK;
    {
        std::lock_guard<std::mutex> lock(srv->mu);
        srv->stopping = true;
    }
    srv->cv_work.notify_all();
    for (auto& t : srv->workers) t.join();
    for (auto& kv : srv->reqs)
        if (kv.second->solver) cr_solver_destroy(kv.second->solver);
    srv->reqs.clear();
    for (cr_context* c : srv->contexts) cr_context_destroy(c);
    if (srv->copy_stream) cudaStreamDestroy(srv->copy_stream);
    delete srv;
    return CR_OK;
}

}  // extern "C"
