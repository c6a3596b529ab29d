// tsg_serve.cpp -- the serving loop (tsg_server_*): continuous batching of
// SpGEMM requests on one GPU, built on the public C ABI.
//
// No counterpart in the reference, which computes one product per process.
//
// Requests enter a pending queue.  Admission moves them to a worker when the
// device memory they may need fits the budget: operands plus an upper bound
// of C taken from the intermediate-product count (every product creates at
// most one entry, 12 bytes each) plus the tile structure.  Each worker owns
// a context (its own CUDA stream and memory pool), so admitted requests of
// different workers run concurrently on the device.  A worker takes up to
// max_batch of its requests at once:
//   - a request with a pattern key whose plan the worker holds runs only the
//     numeric step (tsg_plan_execute);
//   - a keyed request without a plan builds one (tsg_plan_create), keeps it
//     in the worker's plan cache (LRU, bounded by plan_cache_bytes), runs it;
//   - keyless requests of one op are computed together as one batched
//     product (tsg_spgemm_batched).
// Keyed requests go to the worker hash(key) % workers, so repeats find their
// plan.  Results are host CSRs (pinned), returned by tsg_server_wait.
#include "tilespgemm.h"

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <list>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace tsg {
void set_last_error(const char *msg);
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int64_t id = 0;
    tsg_op op = TSG_OP_AA;
    tsg_csr A{}, B{};
    bool hasB = false;
    uint64_t key = 0;
    int64_t est_bytes = 0;
    int worker = -1;
    Clock::time_point t_submit, t_start, t_done;
    tsg_csr C{};
    tsg_status status = TSG_OK;
    std::string err;
    bool done = false;
    bool claimed = false;    // a tsg_server_wait is waiting for it (wait_any skips it)
    int numeric_only = 0;
    int batched_with = 1;
};

struct PlanEntry {
    tsg_plan *plan = nullptr;
    int64_t bytes = 0;
    uint64_t fp = 0;                     // fingerprint of the pattern the plan was built for
    std::list<uint64_t>::iterator lru;
};

struct Worker {
    tsg_ctx *ctx = nullptr;
    std::deque<Request *> q;
    std::unordered_map<uint64_t, PlanEntry> plans;
    std::list<uint64_t> lru;   // most recent first
    int64_t plan_bytes = 0;
    std::thread th;
};

int64_t rowptr_at(const tsg_csr &M, int64_t i)
{
    return M.rowptr_bits == 64 ? ((const int64_t *)M.row_ptr)[i] : ((const int32_t *)M.row_ptr)[i];
}

// Fingerprint of a request's pattern: op, shapes, entry counts, the whole
// row pointer and 64 evenly spaced column indices of each operand (FNV-1a).
// A keyed request whose fingerprint differs from its key's plan rebuilds
// the plan instead of running another pattern's numeric step.
uint64_t fingerprint(tsg_op op, const tsg_csr &A, const tsg_csr *B)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&](uint64_t v) { for (int b = 0; b < 8; ++b) { h ^= (v >> (8 * b)) & 0xff; h *= 1099511628211ull; } };
    auto one = [&](const tsg_csr &M) {
        mix((uint64_t)M.m); mix((uint64_t)M.n); mix((uint64_t)M.nnz);
        for (int64_t i = 0; i <= M.m; ++i) mix((uint64_t)rowptr_at(M, i));
        if (M.nnz > 0)
            for (int t = 0; t < 64; ++t) mix((uint64_t)(uint32_t)M.col[(M.nnz - 1) * t / 63]);
    };
    mix((uint64_t)op);
    one(A);
    if (B) one(*B);
    return h;
}

// Device bytes a request may need: operands, C's upper bound (per row, the
// row's intermediate-product count capped by C's column count; 12 bytes per
// entry), tiles.
int64_t estimate_bytes(tsg_op op, const tsg_csr &A, const tsg_csr *B)
{
    const int64_t n = (op == TSG_OP_AB && B) ? B->n : (op == TSG_OP_AA ? A.n : A.m);
    int64_t cmax = 0;
    std::vector<int32_t> colcnt;
    if (op == TSG_OP_AAT) {
        // B = A^T: B row k has as many entries as A column k
        colcnt.assign((size_t)(A.n > 0 ? A.n : 1), 0);
        for (int64_t p = 0; p < A.nnz; ++p) {
            const int c = A.col[p];
            if ((unsigned)c < (unsigned)A.n) colcnt[(size_t)c]++;
        }
    }
    const tsg_csr &Bm = (op == TSG_OP_AB && B) ? *B : A;
    for (int i = 0; i < A.m; ++i) {
        int64_t row = 0;
        for (int64_t p = rowptr_at(A, i); p < rowptr_at(A, i + 1); ++p) {
            const int c = A.col[p];
            if (op == TSG_OP_AAT) {
                if ((unsigned)c < (unsigned)A.n) row += colcnt[(size_t)c];
            } else if ((unsigned)c < (unsigned)Bm.m) {
                row += rowptr_at(Bm, c + 1) - rowptr_at(Bm, c);
            }
        }
        cmax += row < n ? row : n;
    }
    const int64_t opnd = 24 * (A.nnz + ((op == TSG_OP_AB && B) ? B->nnz : A.nnz)) + 32ll * (A.m + A.n + 2);
    return opnd + 12 * cmax + 48 * cmax / 8 + 16ll * (A.m + 1) + (1 << 20);
}

}  // namespace

struct tsg_server {
    tsg_server_opts opts{};
    std::vector<Worker> workers;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Request *> pending;
    std::unordered_map<int64_t, Request *> reqs;
    std::deque<int64_t> finished;      // completed request ids, in completion order
    int64_t unclaimed = 0;             // outstanding requests no waiter has claimed
    int64_t inflight_bytes = 0;
    int64_t next_id = 1;
    int rr = 0;
    bool stop = false;
};

namespace {

// move pending requests to workers while the budget allows (mu held)
void admit(tsg_server *s)
{
    while (!s->pending.empty()) {
        Request *r = s->pending.front();
        if (s->inflight_bytes > 0 && s->inflight_bytes + r->est_bytes > s->opts.budget_bytes) break;
        s->pending.pop_front();
        s->inflight_bytes += r->est_bytes;
        int w;
        if (r->key) {
            w = (int)(r->key % (uint64_t)s->workers.size());
        } else {
            // least loaded worker
            w = 0;
            for (int k = 1; k < (int)s->workers.size(); ++k)
                if (s->workers[k].q.size() < s->workers[w].q.size()) w = k;
        }
        r->worker = w;
        s->workers[w].q.push_back(r);
    }
    s->cv_work.notify_all();
}

void evict_plans(Worker &W, int64_t limit)
{
    while (W.plan_bytes > limit && !W.lru.empty()) {
        const uint64_t k = W.lru.back();
        W.lru.pop_back();
        auto it = W.plans.find(k);
        if (it != W.plans.end()) {
            W.plan_bytes -= it->second.bytes;
            tsg_plan_destroy(W.ctx, it->second.plan);
            W.plans.erase(it);
        }
    }
}

void run_keyed(tsg_server *s, Worker &W, Request *r)
{
    const uint64_t fp = fingerprint(r->op, r->A, r->hasB ? &r->B : nullptr);
    auto it = W.plans.find(r->key);
    if (it != W.plans.end() && it->second.fp != fp) {   // the key now names another pattern
        W.lru.erase(it->second.lru);
        W.plan_bytes -= it->second.bytes;
        tsg_plan_destroy(W.ctx, it->second.plan);
        W.plans.erase(it);
        it = W.plans.end();
    }
    tsg_plan *plan = nullptr;
    if (it != W.plans.end()) {
        plan = it->second.plan;
        W.lru.erase(it->second.lru);
        W.lru.push_front(r->key);
        it->second.lru = W.lru.begin();
        r->numeric_only = 1;
    } else {
        r->status = tsg_plan_create(W.ctx, r->op, &r->A, r->hasB ? &r->B : nullptr, &plan, nullptr);
        if (r->status != TSG_OK) { r->err = tsg_last_error(); return; }
        PlanEntry e;
        e.plan = plan;
        e.bytes = tsg_plan_device_bytes(plan);
        e.fp = fp;
        W.lru.push_front(r->key);
        e.lru = W.lru.begin();
        W.plans[r->key] = e;
        W.plan_bytes += e.bytes;
    }
    r->C.where = TSG_MEM_HOST;
    r->status = tsg_plan_execute(W.ctx, plan, r->A.val, r->hasB ? r->B.val : nullptr, r->A.where, &r->C, nullptr);
    if (r->status != TSG_OK) r->err = tsg_last_error();
    evict_plans(W, s->opts.plan_cache_bytes);
}

void run_batch(Worker &W, std::vector<Request *> &grp)
{
    const int n = (int)grp.size();
    std::vector<tsg_csr> A(n), B(n), C(n);
    for (int i = 0; i < n; ++i) {
        A[i] = grp[i]->A;
        if (grp[i]->hasB) B[i] = grp[i]->B;
        C[i] = tsg_csr{};
    }
    C[0].where = TSG_MEM_HOST;
    tsg_status st;
    if (n == 1) st = tsg_spgemm(W.ctx, grp[0]->op, &A[0], grp[0]->hasB ? &B[0] : nullptr, &C[0], nullptr);
    else st = tsg_spgemm_batched(W.ctx, grp[0]->op, n, A.data(), grp[0]->op == TSG_OP_AB ? B.data() : nullptr,
                                 C.data(), nullptr);
    const char *msg = st == TSG_OK ? "" : tsg_last_error();
    for (int i = 0; i < n; ++i) {
        grp[i]->status = st;
        grp[i]->err = msg;
        grp[i]->batched_with = n;
        if (st == TSG_OK) grp[i]->C = C[i];
    }
}

void worker_main(tsg_server *s, int w)
{
    Worker &W = s->workers[w];
    for (;;) {
        std::vector<Request *> take;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !W.q.empty(); });
            if (s->stop && W.q.empty()) return;
            while (!W.q.empty() && (int)take.size() < s->opts.max_batch) {
                take.push_back(W.q.front());
                W.q.pop_front();
            }
        }
        const auto t0 = Clock::now();
        for (Request *r : take) r->t_start = t0;
        // keyed requests one by one (plan hit = numeric only); keyless grouped by op
        std::vector<Request *> groups[3];
        for (Request *r : take) {
            if (r->key) run_keyed(s, W, r);
            else groups[(int)r->op].push_back(r);
        }
        for (auto &g : groups)
            if (!g.empty()) run_batch(W, g);
        const auto t1 = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            for (Request *r : take) {
                r->t_done = t1;
                r->done = true;
                s->inflight_bytes -= r->est_bytes;
                s->finished.push_back(r->id);
            }
            admit(s);
        }
        s->cv_done.notify_all();
    }
}

}  // namespace

extern "C" {

void tsg_server_opts_default(tsg_server_opts *o)
{
    if (!o) return;
    o->device = 0;
    o->workers = 4;
    o->max_batch = 32;
    o->budget_bytes = 64ll << 30;
    o->plan_cache_bytes = 8ll << 30;
}

tsg_status tsg_server_create(const tsg_server_opts *opts, tsg_server **out)
{
    if (!out) { tsg::set_last_error("out is NULL"); return TSG_ERR_INVALID_ARG; }
    *out = nullptr;
    tsg_server *s = new tsg_server();
    tsg_server_opts_default(&s->opts);
    if (opts) s->opts = *opts;
    if (s->opts.workers < 1) s->opts.workers = 1;
    if (s->opts.max_batch < 1) s->opts.max_batch = 1;
    s->workers = std::vector<Worker>((size_t)s->opts.workers);
    for (auto &W : s->workers) {
        tsg_status st = tsg_create(&W.ctx, s->opts.device, nullptr);
        if (st != TSG_OK) {
            for (auto &X : s->workers) if (X.ctx) tsg_destroy(X.ctx);
            delete s;
            return st;
        }
    }
    for (int w = 0; w < (int)s->workers.size(); ++w) s->workers[w].th = std::thread(worker_main, s, w);
    *out = s;
    return TSG_OK;
}

tsg_status tsg_server_submit(tsg_server *s, tsg_op op, const tsg_csr *A, const tsg_csr *B, uint64_t pattern_key,
                             int64_t *request_id)
{
    if (!s || !A || !request_id) { tsg::set_last_error("server/A/request_id is NULL"); return TSG_ERR_INVALID_ARG; }
    if (A->where != TSG_MEM_HOST || (B && B->where != TSG_MEM_HOST)) {
        tsg::set_last_error("served requests take host operands");
        return TSG_ERR_INVALID_ARG;
    }
    if (op == TSG_OP_AB && !B) { tsg::set_last_error("B is NULL for A*B"); return TSG_ERR_INVALID_ARG; }
    Request *r = new Request();
    r->op = op;
    r->A = *A;
    r->A.owner = nullptr;
    r->hasB = op == TSG_OP_AB;
    if (r->hasB) { r->B = *B; r->B.owner = nullptr; }
    r->key = pattern_key;
    r->est_bytes = estimate_bytes(op, *A, r->hasB ? B : nullptr);
    if (r->est_bytes > s->opts.budget_bytes) {
        delete r;
        tsg::set_last_error("request needs more device memory than the server's budget");
        return TSG_ERR_BUDGET;
    }
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        r->id = s->next_id++;
        s->reqs[r->id] = r;
        ++s->unclaimed;
        s->pending.push_back(r);
        admit(s);
    }
    *request_id = r->id;
    return TSG_OK;
}

}  // extern "C"

namespace {

// hand a completed request (already removed from s->reqs) to the caller
tsg_status finish_wait(Request *r, tsg_csr *C, tsg_server_result *info)
{
    const tsg_status st = r->status;
    if (info) {
        info->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        info->queue_ms = std::chrono::duration<double, std::milli>(r->t_start - r->t_submit).count();
        info->run_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_start).count();
        info->numeric_only = r->numeric_only;
        info->batched_with = r->batched_with;
        info->worker = r->worker;
    }
    if (st == TSG_OK) *C = r->C;
    else tsg::set_last_error(r->err.c_str());
    delete r;
    return st;
}

}  // namespace

extern "C" {

tsg_status tsg_server_wait(tsg_server *s, int64_t request_id, tsg_csr *C, tsg_server_result *info)
{
    if (!s || !C) { tsg::set_last_error("server/C is NULL"); return TSG_ERR_INVALID_ARG; }
    Request *r = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        auto it = s->reqs.find(request_id);
        if (it == s->reqs.end()) { tsg::set_last_error("unknown request id"); return TSG_ERR_INVALID_ARG; }
        r = it->second;
        if (r->claimed) { tsg::set_last_error("another thread is waiting for this request"); return TSG_ERR_INVALID_ARG; }
        // claimed: no other waiter takes it, so r stays valid while this one sleeps
        r->claimed = true;
        --s->unclaimed;
        s->cv_done.wait(lk, [&] { return r->done; });
        s->reqs.erase(request_id);
    }
    return finish_wait(r, C, info);
}

tsg_status tsg_server_wait_any(tsg_server *s, int64_t *request_id, tsg_csr *C, tsg_server_result *info)
{
    if (!s || !C || !request_id) { tsg::set_last_error("server/C/request_id is NULL"); return TSG_ERR_INVALID_ARG; }
    Request *r = nullptr;
    {
        std::unique_lock<std::mutex> lk(s->mu);
        for (;;) {
            // ids returned by tsg_server_wait, or claimed by a waiting one, are skipped
            while (!s->finished.empty()) {
                auto f = s->reqs.find(s->finished.front());
                if (f != s->reqs.end() && !f->second->claimed) break;
                s->finished.pop_front();
            }
            if (!s->finished.empty()) break;
            if (s->unclaimed == 0) { tsg::set_last_error("no outstanding requests"); return TSG_ERR_INVALID_ARG; }
            s->cv_done.wait(lk);
        }
        const int64_t id = s->finished.front();
        s->finished.pop_front();
        auto it = s->reqs.find(id);
        r = it->second;
        s->reqs.erase(it);
        --s->unclaimed;
        *request_id = id;
    }
    return finish_wait(r, C, info);
}

tsg_status tsg_server_destroy(tsg_server *s)
{
    if (!s) return TSG_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto &W : s->workers)
        if (W.th.joinable()) W.th.join();
    for (auto &kv : s->reqs) {
        if (kv.second->done && kv.second->status == TSG_OK) tsg_csr_free(nullptr, &kv.second->C);
        delete kv.second;
    }
    for (auto &W : s->workers) {
        for (auto &kv : W.plans) tsg_plan_destroy(W.ctx, kv.second.plan);
        tsg_destroy(W.ctx);
    }
    delete s;
    return TSG_OK;
}

}  // extern "C"
