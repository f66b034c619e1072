/*
 * grns_gb300 -- serving: a stream of vector-op requests with continuous
 * batching over device-resident operands.
 *
 * No counterpart in the reference (a header-only library with no runtime).
 * Clients put arrays into server-owned device memory once (handles) and
 * submit requests that name them; outputs become new resident handles, and an
 * eval request's output is remembered as that array's evaluation so later
 * comparisons read 32-byte intervals instead of the residues.  A scheduler
 * thread:
 *   - gives each free launch slot (stream) the moduli set of the oldest
 *     pending request that can run, and packs every pending request of that
 *     set whose HBM footprint (output arrays) fits the budget into ONE launch
 *     of the persistent batched kernel, allocating outputs from the server's
 *     memory pool (stream-ordered, no device-wide synchronisation).  A
 *     request that does not fit is passed by later ones that do, until it has
 *     waited kPassCapUs: then nothing is admitted past it, so freed memory
 *     goes to it.  With several slots, requests arriving while launches are
 *     in flight are admitted and launched alongside them, so their work
 *     overlaps on the device.  With direct_min_count set (off by default),
 *     requests of that many numbers or more (eval, cmp, div, scale2pow,
 *     mp_int add/sub/mul) run in the same launch round through the per-op
 *     kernels instead, after the packed kernel on the same stream: lower
 *     latency for the small requests under load, less throughput;
 *   - marks requests done from a host callback at the end of each launch and
 *     records submit-to-completion latency (p50/p99 in grns_server_stats).
 * Each array counts the unfinished requests that read it (counted at
 * submission, and for a cached evaluation when a launch uses it); freeing an
 * array waits until that count is zero.  A finished request's status and
 * output handles stay readable for kKeepFinishedUs after it finishes and are
 * then dropped (at most kKeepFinishedMax finished requests are kept).
 * Every per-element computation is independent of its neighbours, so a
 * result does not depend on what else shares its launch.
 */
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace {

using Clock = std::chrono::steady_clock;

constexpr double kPassCapUs = 50e3;          // after this wait for memory, later requests stop passing one
constexpr double kKeepFinishedUs = 60e6;     // finished requests stay readable this long
constexpr size_t kKeepFinishedMax = 1 << 16; // and at most this many of them
/* default of grns_server_options.direct_min_count: off.  On the served stream
 * of the benchmark (64 requests of 10^3..10^7 numbers) packing everything ran
 * 1.41-1.43 G numbers/s and 2^18 as the threshold 1.11-1.20 (lower p50 under
 * Poisson load, higher p99): one persistent launch balances the large
 * requests across the SMs better than their own kernels queued per slot */
constexpr int32_t kDirectMinDefault = -1;

double now_us() {
    return std::chrono::duration<double, std::micro>(Clock::now().time_since_epoch()).count();
}

struct Array {
    void *p = nullptr;
    int ctx = 0;
    int kind = 0;
    int64_t count = 0;
    int layout = GRNS_LAYOUT_SOA;
    size_t bytes = 0;
    uint64_t eval = 0;      // handle of this array's evaluation (RNS arrays), 0 if none
    uint64_t producer = 0;  // request that writes it (0: put by the client)
    int readers = 0;        // unfinished requests that read it
};

struct Req {
    grns_request r{};
    int state = 0;  // 0 pending, 1 in flight, 2 done
    int32_t status = GRNS_OK;
    uint64_t out0 = 0, out1 = 0;
    size_t footprint = 0;
    int64_t count = 0;
    bool direct = false;  // runs through the per-op kernels (direct_min_count)
    double t_submit = 0, t_done = 0;
    uint64_t reads[4] = {0, 0, 0, 0};  // arrays whose reader count this request holds
};

struct Slot {
    cudaStream_t s = nullptr;
    void *staging = nullptr;  // pinned job-table staging
    bool busy = false;
    std::vector<uint64_t> reqs;
    std::atomic<int> done{0};
    double t_done = 0;
    struct grns_server *srv = nullptr;
};

size_t elem_bytes(int kind, int n) {
    switch (kind) {
        case GRNS_ARRAY_RNS: return 4 * (size_t)n;
        case GRNS_ARRAY_U32: return 4;
        case GRNS_ARRAY_MPINT: return GRNS_MPINT_BYTES(n);
        case GRNS_ARRAY_INTERVAL: return sizeof(interval_t);
        default: return 0;
    }
}

}  // namespace

struct grns_server {
    grns_server_options opt{};
    std::vector<grns_ctx *> ctxs;
    std::mutex mu;
    std::condition_variable cv;
    std::unordered_map<uint64_t, Array> arrays;
    std::unordered_map<uint64_t, Req> reqs;
    std::deque<uint64_t> pending;
    std::deque<std::pair<uint64_t, double>> finished;  // (request, completion time), oldest first
    std::vector<Slot *> slots;
    uint64_t next_handle = 1, next_req = 1;
    size_t in_use = 0;
    size_t allocated = 0;  // bytes of live arrays (alloc_cap_bytes applies to it)
    cudaMemPool_t pool = nullptr;
    cudaStream_t copy = nullptr;
    int device = 0;
    bool stop = false;
    std::thread worker;
    // stats
    std::vector<double> lat;
    uint64_t completed = 0, rejected = 0, cancelled = 0, launches = 0, jobs_launched = 0;
    double numbers = 0, t_first = 0, t_last = 0;
    double t_last_submit = 0;  // submission time of the newest request (the gathering window)
};

namespace {

/* Runs on CUDA's callback thread after a launch.  It must not take the
 * server mutex: the scheduler holds that mutex across stream-ordered CUDA
 * calls, and a call that waits for stream work (which includes this callback)
 * would deadlock.  So: atomic flag, timestamp, notify without the lock (the
 * scheduler and waiters also wake on a short timeout). */
void CUDART_CB on_launch_done(void *arg) {
    Slot *sl = (Slot *)arg;
    sl->t_done = now_us();
    sl->done.store(1, std::memory_order_release);
    sl->srv->cv.notify_all();
}

/* true when request `id` has finished (or has been dropped after finishing) */
bool req_finished(const grns_server *sv, uint64_t id) {
    auto it = sv->reqs.find(id);
    return it == sv->reqs.end() || it->second.state == 2;
}

/* the request holds a reader count on array h until it finishes */
void hold_read(grns_server *sv, Req &q, uint64_t h) {
    auto it = h ? sv->arrays.find(h) : sv->arrays.end();
    if (it == sv->arrays.end()) return;
    for (uint64_t &slot : q.reads)
        if (!slot) {
            slot = h;
            it->second.readers++;
            return;
        }
}

/* marks a request finished: status, time, reader counts released */
void finish(grns_server *sv, uint64_t id, Req &q, int32_t status, double t) {
    q.state = 2;
    q.status = status;
    q.t_done = t;
    for (uint64_t &h : q.reads) {
        auto it = h ? sv->arrays.find(h) : sv->arrays.end();
        if (it != sv->arrays.end() && it->second.readers > 0) it->second.readers--;
        h = 0;
    }
    sv->finished.emplace_back(id, t);
    sv->cv.notify_all();
}

grns_status alloc_array(grns_server *sv, cudaStream_t s, int ctx, int kind, int64_t count, int layout, Array &a) {
    const grns_ctx *c = sv->ctxs[ctx];
    size_t bytes = elem_bytes(kind, c->n) * (size_t)count;
    if (kind == GRNS_ARRAY_MAXOUT) bytes = ((4 * (size_t)c->n + 7) / 8) * 8 + 8;
    if (sv->opt.alloc_cap_bytes && sv->allocated + bytes > sv->opt.alloc_cap_bytes) return GRNS_ERR_OUT_OF_MEMORY;
    cudaError_t e = cudaMallocFromPoolAsync(&a.p, bytes ? bytes : 16, sv->pool, s);
    if (e != cudaSuccess) return grns::cuda_status(e);
    sv->allocated += bytes;
    a.ctx = ctx;
    a.kind = kind;
    a.count = count;
    a.layout = layout;
    a.bytes = bytes;
    return GRNS_OK;
}

/* output arrays of a request plus its launch scratch (division records):
 * sizes only (for admission) */
size_t footprint_of(const grns_server *sv, const Req &q) {
    const grns_ctx *c = sv->ctxs[q.r.ctx_index];
    const int n = c->n;
    const int64_t k = q.count;
    switch (q.r.op) {
        case GRNS_OP_EVAL: return sizeof(interval_t) * k;
        case GRNS_OP_CMP: return 4 * (size_t)k;
        case GRNS_OP_DIV: return 2 * 4 * (size_t)n * k + (12 * (size_t)k);  // + the batched kernel's records
        case GRNS_OP_SCALE2POW: return (4 * (size_t)n + 12) * k;
        case GRNS_OP_MAX: return ((4 * (size_t)n + 7) / 8) * 8 + 8;
        case GRNS_OP_MPINT_DIV:  // + the batched kernel's records, remainder digits and flags
            return (GRNS_MPINT_BYTES(n) + 12 + 4 * (size_t)n + 1) * k;
        default: return GRNS_MPINT_BYTES(n) * (size_t)k;
    }
}

/* whether a request runs through the per-op kernels: large enough, and
 * shaped as they take it (one leading dimension for inputs and outputs) */
bool direct_request(const grns_server *sv, const Req &q) {
    const int32_t thr = sv->opt.direct_min_count == 0 ? kDirectMinDefault : sv->opt.direct_min_count;
    if (thr < 0 || q.count < thr) return false;
    switch (q.r.op) {
        case GRNS_OP_EVAL:
        case GRNS_OP_CMP:
        case GRNS_OP_DIV:
        case GRNS_OP_SCALE2POW:
        case GRNS_OP_MPINT_ADD:
        case GRNS_OP_MPINT_SUB:
        case GRNS_OP_MPINT_MUL: return true;
        default: return false;
    }
}

/* device scratch of a request run through the per-op kernels */
size_t direct_scratch(const grns_server *sv, const Req &q) {
    const grns_ctx *c = sv->ctxs[q.r.ctx_index];
    switch (q.r.op) {
        case GRNS_OP_DIV: return grns::div_scratch_bytes(c, q.count);
        case GRNS_OP_SCALE2POW: return q.r.b ? 4 * (size_t)q.count : 0;  // the longest-first order
        default: return 256;                                                 // the evaluation's claim counter
    }
}

/* one request through the per-op kernels on stream s (the plain calls'
 * launches); SoA outputs are dense (leading dimension count) like the
 * packed kernel's */
grns_status run_direct(const grns_ctx *c, const grns_job &j, cudaStream_t s) {
    const uint32_t *a = (const uint32_t *)j.a, *b = (const uint32_t *)j.b;
    const bool soa = j.layout == GRNS_LAYOUT_SOA;
    const int64_t ld = soa ? j.ld : 0, ldo = soa ? j.count : 0;
    switch (j.op) {
        case GRNS_OP_EVAL: return grns::launch_eval(c, a, ld, j.count, (interval_t *)j.out0, nullptr, s);
        case GRNS_OP_CMP: return grns::launch_cmp(c, a, b, ld, j.count, (int32_t *)j.out0, nullptr, s);
        case GRNS_OP_DIV:
            return grns::launch_div(c, a, b, ld, j.count, (uint32_t *)j.out0, (uint32_t *)j.out1, nullptr, s, 0, ldo);
        case GRNS_OP_SCALE2POW:
            return grns::launch_scale2pow(c, a, b, j.D_uniform, ld, j.count, (uint32_t *)j.out0, nullptr, s, 0, ldo);
        default: return grns::launch_mpint(c, j.op - GRNS_OP_MPINT_ADD, j.a, j.b, j.count, j.out0, nullptr, s);
    }
}

/* scheduler: completions, admission, packing, launch (caller holds mu) */
void schedule_locked(grns_server *sv) {
    for (Slot *sl : sv->slots) {
        if (!sl->busy || !sl->done.load(std::memory_order_acquire)) continue;
        for (uint64_t id : sl->reqs) {
            auto it = sv->reqs.find(id);
            if (it == sv->reqs.end()) continue;
            Req &q = it->second;
            finish(sv, id, q, q.status, sl->t_done);
            sv->lat.push_back(q.t_done - q.t_submit);
            sv->completed++;
            sv->numbers += (double)q.count;
            sv->t_last = std::max(sv->t_last, q.t_done);
        }
        sl->reqs.clear();
        sl->busy = false;
        sl->done.store(0);
    }
    const double now = now_us();
    /* finished requests past their retention */
    while (!sv->finished.empty() &&
           (now - sv->finished.front().second > kKeepFinishedUs || sv->finished.size() > kKeepFinishedMax)) {
        auto it = sv->reqs.find(sv->finished.front().first);
        if (it != sv->reqs.end() && it->second.state == 2) sv->reqs.erase(it);
        sv->finished.pop_front();
    }
    /* requests that waited too long for memory */
    for (auto it = sv->pending.begin(); it != sv->pending.end();) {
        Req &q = sv->reqs.at(*it);
        if (now - q.t_submit < 1e3 * sv->opt.admission_timeout_ms) {
            ++it;
            continue;
        }
        finish(sv, *it, q, GRNS_ERR_REJECTED, now);
        sv->rejected++;
        it = sv->pending.erase(it);
    }
    /* gathering: while requests keep arriving, free slots wait for more */
    if (sv->opt.gather_us > 0 && !sv->pending.empty() &&
        (int)sv->pending.size() < sv->opt.max_jobs_per_launch) {
        const double oldest = sv->reqs.at(sv->pending.front()).t_submit;
        if (now - sv->t_last_submit < sv->opt.gather_us && now - oldest < 4.0 * sv->opt.gather_us) return;
    }
    for (Slot *sl : sv->slots) {
        if (sl->busy || sv->pending.empty()) continue;
        int ctx = -1;  // the moduli set of this launch: that of the oldest request admitted
        std::vector<grns_job> jobs, direct;  // packed into the batched kernel / through the per-op kernels
        for (auto it = sv->pending.begin();
             it != sv->pending.end() && (int)(jobs.size() + direct.size()) < sv->opt.max_jobs_per_launch;) {
            const uint64_t id = *it;
            Req &q = sv->reqs.at(id);
            if (ctx >= 0 && q.r.ctx_index != ctx) {
                ++it;
                continue;
            }
            {  /* operands written by requests still in flight: not runnable yet */
                auto busy = [&](uint64_t h) {
                    auto a = sv->arrays.find(h);
                    return a != sv->arrays.end() && a->second.producer && !req_finished(sv, a->second.producer);
                };
                if (busy(q.r.a) || (q.r.b && busy(q.r.b))) {
                    ++it;
                    continue;
                }
            }
            if (sv->arrays.find(q.r.a) == sv->arrays.end() || (q.r.b && sv->arrays.find(q.r.b) == sv->arrays.end())) {
                /* a defensive guard: freeing an array waits for the requests that read it, so an
                 * operand of a pending request is never gone; counted as a rejection */
                finish(sv, id, q, GRNS_ERR_INVALID_ARGUMENT, now_us());
                sv->rejected++;
                it = sv->pending.erase(it);
                continue;
            }
            if (sv->in_use + q.footprint > sv->opt.hbm_budget_bytes) {
                if (now - q.t_submit > kPassCapUs) break;  // no later request passes it any more
                ++it;                                      // later requests that fit go first
                continue;
            }
            ctx = q.r.ctx_index;
            const grns_ctx *c = sv->ctxs[ctx];
            const Array A = sv->arrays[q.r.a];  /* copies: inserting outputs below may rehash the map */
            Array Bv;
            const Array *B = nullptr;
            if (q.r.b) {
                Bv = sv->arrays[q.r.b];
                B = &Bv;
            }
            Array o0, o1;
            grns_status st = GRNS_OK;
            switch (q.r.op) {
                case GRNS_OP_EVAL: st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_INTERVAL, q.count, 0, o0); break;
                case GRNS_OP_CMP: st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_U32, q.count, 0, o0); break;
                case GRNS_OP_DIV:
                    st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_RNS, q.count, GRNS_LAYOUT_SOA, o0);
                    if (st == GRNS_OK) st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_RNS, q.count, GRNS_LAYOUT_SOA, o1);
                    break;
                case GRNS_OP_SCALE2POW: st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_RNS, q.count, A.layout, o0); break;
                case GRNS_OP_MAX: st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_MAXOUT, 1, 0, o0); break;
                default: st = alloc_array(sv, sl->s, ctx, GRNS_ARRAY_MPINT, q.count, 0, o0); break;
            }
            it = sv->pending.erase(it);
            if (st != GRNS_OK) {
                if (o0.p) {
                    cudaFreeAsync(o0.p, sl->s);
                    sv->allocated -= std::min(sv->allocated, o0.bytes);
                }
                finish(sv, id, q, st, now_us());
                continue;
            }
            sv->in_use += q.footprint;
            o0.producer = id;
            q.out0 = sv->next_handle++;
            sv->arrays[q.out0] = o0;
            if (o1.p) {
                o1.producer = id;
                q.out1 = sv->next_handle++;
                sv->arrays[q.out1] = o1;
            }
            grns_job j{};
            j.op = q.r.op;
            j.layout = A.layout;
            j.count = q.count;
            j.ld = A.layout == GRNS_LAYOUT_SOA ? A.count : 0;
            j.a = A.p;
            j.b = B ? B->p : nullptr;
            j.out0 = o0.p;
            j.D_uniform = q.r.D_uniform;
            if (q.r.op == GRNS_OP_DIV) {
                j.out1 = o1.p;
                j.layout = GRNS_LAYOUT_SOA;
            } else if (q.r.op == GRNS_OP_MAX) {
                j.out1 = (char *)o0.p + ((4 * (size_t)c->n + 7) / 8) * 8;
            } else if (q.r.op == GRNS_OP_CMP && A.eval && B && B->eval) {  /* finished evaluations only */
                auto ea = sv->arrays.find(A.eval), eb = sv->arrays.find(B->eval);
                if (ea != sv->arrays.end() && eb != sv->arrays.end() && ea->second.count >= q.count &&
                    eb->second.count >= q.count && req_finished(sv, ea->second.producer) &&
                    req_finished(sv, eb->second.producer)) {
                    j.eval_a = (const interval_t *)ea->second.p;
                    j.eval_b = (const interval_t *)eb->second.p;
                    hold_read(sv, q, A.eval);  // freeing them now waits for this launch
                    hold_read(sv, q, B->eval);
                }
            }
            if (q.r.op == GRNS_OP_EVAL && q.count == A.count) sv->arrays[q.r.a].eval = q.out0;
            q.state = 1;
            sl->reqs.push_back(id);
            if (q.direct && !j.eval_a) direct.push_back(j);  // cached evaluations: the packed kernel reads them
            else jobs.push_back(j);
        }
        if (jobs.empty() && direct.empty()) continue;
        grns::NvtxRange range("grns_server launch");
        grns_status st = GRNS_OK;
        if (!jobs.empty())
            st = grns::batch_run_async(sv->ctxs[ctx], jobs.data(), (int)jobs.size(), sl->staging, sl->s);
        for (const grns_job &j : direct)
            if (st == GRNS_OK) st = run_direct(sv->ctxs[ctx], j, sl->s);
        if (st == GRNS_OK) st = grns::cuda_status(cudaLaunchHostFunc(sl->s, on_launch_done, sl));
        if (st != GRNS_OK) {
            for (uint64_t id : sl->reqs) finish(sv, id, sv->reqs.at(id), st, now_us());
            sl->reqs.clear();
            continue;
        }
        sl->busy = true;
        sv->launches++;
        sv->jobs_launched += jobs.size() + direct.size();
    }
}

void worker_main(grns_server *sv) {
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    while (!sv->stop) {
        schedule_locked(sv);
        sv->cv.wait_for(lk, std::chrono::microseconds(200));
    }
}

/* waits (bounded) for a request; the short wait slices also cover notifications
 * that raced ahead of the wait */
bool wait_done(grns_server *sv, std::unique_lock<std::mutex> &lk, uint64_t id, int64_t timeout_us) {
    const int64_t cap = (int64_t)600 * 1000 * 1000;  // 10 minutes
    auto until = Clock::now() + std::chrono::microseconds(timeout_us < 0 || timeout_us > cap ? cap : timeout_us);
    while (!req_finished(sv, id)) {
        const auto now = Clock::now();
        if (now >= until) return false;
        /* wake at least every millisecond (completions notify without the lock), never past the deadline */
        sv->cv.wait_until(lk, std::min(until, now + std::chrono::milliseconds(1)));
    }
    return true;
}

/* waits (bounded) until no unfinished request reads array h; false on timeout */
bool wait_unread(grns_server *sv, std::unique_lock<std::mutex> &lk, uint64_t h) {
    auto until = Clock::now() + std::chrono::minutes(10);
    for (;;) {
        auto it = sv->arrays.find(h);
        if (it == sv->arrays.end() || it->second.readers == 0) return true;
        if (Clock::now() >= until) return false;
        sv->cv.wait_for(lk, std::chrono::milliseconds(1));
    }
}

}  // namespace

extern "C" {

grns_status grns_server_create(const grns_server_options *opt, grns_server **out) {
    if (!out) return GRNS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    grns_server *sv = new (std::nothrow) grns_server();
    if (!sv) return GRNS_ERR_OUT_OF_MEMORY;
    if (opt) sv->opt = *opt;
    if (sv->opt.launch_slots <= 0) sv->opt.launch_slots = 4;
    if (sv->opt.max_jobs_per_launch <= 0) sv->opt.max_jobs_per_launch = 256;
    if (sv->opt.admission_timeout_ms <= 0) sv->opt.admission_timeout_ms = 10000;
    cudaError_t e = cudaGetDevice(&sv->device);
    size_t fr = 0, tot = 0;
    if (e == cudaSuccess) e = cudaMemGetInfo(&fr, &tot);
    if (e == cudaSuccess && sv->opt.hbm_budget_bytes == 0) sv->opt.hbm_budget_bytes = (size_t)(0.8 * (double)fr);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = sv->device;
    if (e == cudaSuccess) e = cudaMemPoolCreate(&sv->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = ~0ull;  // keep freed memory in the pool
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->copy, cudaStreamNonBlocking);
    for (int i = 0; e == cudaSuccess && i < sv->opt.launch_slots; i++) {
        Slot *sl = new Slot();
        sl->srv = sv;
        e = cudaStreamCreateWithFlags(&sl->s, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaMallocHost(&sl->staging, grns::batch_staging_bytes(sv->opt.max_jobs_per_launch));
        sv->slots.push_back(sl);
    }
    if (e != cudaSuccess) {
        grns_server_destroy(sv);
        return grns::cuda_status(e);
    }
    sv->worker = std::thread(worker_main, sv);
    *out = sv;
    return GRNS_OK;
}

grns_status grns_server_destroy(grns_server *sv) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> g(sv->mu);
        sv->stop = true;
        sv->cv.notify_all();
    }
    if (sv->worker.joinable()) sv->worker.join();
    for (Slot *sl : sv->slots) {
        if (sl->s) cudaStreamSynchronize(sl->s);
    }
    for (auto &kv : sv->arrays)
        if (kv.second.p) cudaFreeAsync(kv.second.p, sv->copy ? sv->copy : nullptr);
    if (sv->copy) cudaStreamSynchronize(sv->copy);
    for (Slot *sl : sv->slots) {
        if (sl->staging) cudaFreeHost(sl->staging);
        if (sl->s) cudaStreamDestroy(sl->s);
        delete sl;
    }
    if (sv->copy) cudaStreamDestroy(sv->copy);
    if (sv->pool) cudaMemPoolDestroy(sv->pool);
    delete sv;
    return GRNS_OK;
}

grns_status grns_server_add_context(grns_server *sv, grns_ctx *c, int *index) {
    if (!sv || !c || !index) return GRNS_ERR_INVALID_ARGUMENT;
    if (c->n > grns::kBatchMaxModuli) return GRNS_ERR_UNSUPPORTED;  // requests run in the batched kernel
    std::lock_guard<std::mutex> g(sv->mu);
    sv->ctxs.push_back(c);
    *index = (int)sv->ctxs.size() - 1;
    return GRNS_OK;
}

grns_status grns_server_put(grns_server *sv, int ctx, int kind, const void *src, int src_on_device, int64_t count,
                            int layout, uint64_t *handle) {
    if (!sv || !handle || count < 0 || (count > 0 && !src)) return GRNS_ERR_INVALID_ARGUMENT;
    if (kind != GRNS_ARRAY_RNS && kind != GRNS_ARRAY_U32 && kind != GRNS_ARRAY_MPINT) return GRNS_ERR_INVALID_ARGUMENT;
    if (layout != GRNS_LAYOUT_SOA && layout != GRNS_LAYOUT_AOS) return GRNS_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (ctx < 0 || ctx >= (int)sv->ctxs.size()) return GRNS_ERR_INVALID_ARGUMENT;
    const size_t bytes = elem_bytes(kind, sv->ctxs[ctx]->n) * (size_t)count;
    if (sv->in_use + bytes > sv->opt.hbm_budget_bytes) return GRNS_ERR_REJECTED;
    Array a;
    grns_status st = alloc_array(sv, sv->copy, ctx, kind, count, layout, a);
    if (st != GRNS_OK) return st;
    sv->in_use += bytes;
    lk.unlock();
    cudaError_t e = cudaSuccess;
    if (bytes)
        e = cudaMemcpyAsync(a.p, src, bytes, src_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, sv->copy);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sv->copy);
    lk.lock();
    if (e != cudaSuccess) {
        cudaFreeAsync(a.p, sv->copy);
        sv->in_use -= bytes;
        sv->allocated -= std::min(sv->allocated, a.bytes);
        return grns::cuda_status(e);
    }
    *handle = sv->next_handle++;
    sv->arrays[*handle] = a;
    return GRNS_OK;
}

grns_status grns_server_array_info(grns_server *sv, uint64_t h, int64_t *count, size_t *bytes, void **device_ptr) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    auto it = sv->arrays.find(h);
    if (it == sv->arrays.end()) return GRNS_ERR_INVALID_ARGUMENT;
    if (count) *count = it->second.count;
    if (bytes) *bytes = it->second.bytes;
    if (device_ptr) *device_ptr = it->second.p;
    return GRNS_OK;
}

grns_status grns_server_get(grns_server *sv, uint64_t h, void *host_dst, size_t bytes) {
    if (!sv || !host_dst) return GRNS_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->arrays.find(h);
    if (it == sv->arrays.end() || bytes > it->second.bytes) return GRNS_ERR_INVALID_ARGUMENT;
    const uint64_t prod = it->second.producer;
    if (prod && !wait_done(sv, lk, prod, -1)) return GRNS_ERR_TIMEOUT;
    void *p = sv->arrays[h].p;
    lk.unlock();
    cudaError_t e = cudaMemcpyAsync(host_dst, p, bytes, cudaMemcpyDeviceToHost, sv->copy);
    if (e == cudaSuccess) e = cudaStreamSynchronize(sv->copy);
    return grns::cuda_status(e);
}

grns_status grns_server_free(grns_server *sv, uint64_t h) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->arrays.find(h);
    if (it == sv->arrays.end()) return GRNS_ERR_INVALID_ARGUMENT;
    const uint64_t prod = it->second.producer;
    if (prod && !wait_done(sv, lk, prod, -1)) return GRNS_ERR_TIMEOUT;
    /* unfinished requests that read this array (as an operand, or a launch
     * reading it as a cached evaluation): wait for them, so no launch reads
     * freed memory */
    if (!wait_unread(sv, lk, h)) return GRNS_ERR_TIMEOUT;
    it = sv->arrays.find(h);
    if (it == sv->arrays.end()) return GRNS_ERR_INVALID_ARGUMENT;
    cudaFreeAsync(it->second.p, sv->copy);
    sv->in_use -= std::min(sv->in_use, it->second.bytes);
    sv->allocated -= std::min(sv->allocated, it->second.bytes);
    for (auto &kv : sv->arrays)
        if (kv.second.eval == h) kv.second.eval = 0;
    sv->arrays.erase(it);
    sv->cv.notify_all();
    return GRNS_OK;
}

grns_status grns_server_submit(grns_server *sv, const grns_request *r, uint64_t *request_id) {
    if (!sv || !r || !request_id) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    if (r->ctx_index < 0 || r->ctx_index >= (int)sv->ctxs.size()) return GRNS_ERR_INVALID_ARGUMENT;
    if (r->op < GRNS_OP_EVAL || r->op > GRNS_OP_MPINT_DIV) return GRNS_ERR_INVALID_ARGUMENT;
    auto ia = sv->arrays.find(r->a);
    if (ia == sv->arrays.end() || ia->second.ctx != r->ctx_index) return GRNS_ERR_INVALID_ARGUMENT;
    const bool mp = r->op >= GRNS_OP_MPINT_ADD;
    if ((mp ? GRNS_ARRAY_MPINT : GRNS_ARRAY_RNS) != ia->second.kind) return GRNS_ERR_INVALID_ARGUMENT;
    const int64_t count = r->count > 0 ? r->count : ia->second.count;
    if (count > ia->second.count) return GRNS_ERR_INVALID_ARGUMENT;
    const bool needs_b = r->op == GRNS_OP_CMP || r->op == GRNS_OP_DIV || mp;
    if (needs_b || r->b) {
        auto ib = sv->arrays.find(r->b);
        if (ib == sv->arrays.end() || ib->second.count < count) return GRNS_ERR_INVALID_ARGUMENT;
        const int want = r->op == GRNS_OP_SCALE2POW ? GRNS_ARRAY_U32 : (mp ? GRNS_ARRAY_MPINT : GRNS_ARRAY_RNS);
        if (ib->second.kind != want) return GRNS_ERR_INVALID_ARGUMENT;
        if (want == GRNS_ARRAY_RNS && (ib->second.layout != ia->second.layout || ib->second.count != ia->second.count))
            return GRNS_ERR_INVALID_ARGUMENT;  // one leading dimension per job
    }
    if (r->op == GRNS_OP_DIV && ia->second.layout != GRNS_LAYOUT_SOA) return GRNS_ERR_INVALID_ARGUMENT;
    const uint64_t id = sv->next_req++;
    Req &q = sv->reqs[id];
    q.r = *r;
    q.count = count;
    q.footprint = footprint_of(sv, q);
    q.direct = direct_request(sv, q);
    if (q.direct) q.footprint += direct_scratch(sv, q);
    q.t_submit = now_us();
    if (sv->t_first == 0) sv->t_first = q.t_submit;
    *request_id = id;
    hold_read(sv, q, r->a);
    if (r->b) hold_read(sv, q, r->b);
    if (q.footprint > sv->opt.hbm_budget_bytes) {  // can never be admitted
        finish(sv, id, q, GRNS_ERR_REJECTED, q.t_submit);
        sv->rejected++;
        return GRNS_OK;
    }
    sv->pending.push_back(id);
    sv->t_last_submit = q.t_submit;
    sv->cv.notify_all();
    return GRNS_OK;
}

grns_status grns_server_poll(grns_server *sv, uint64_t id, int *done, int32_t *status, uint64_t *out0, uint64_t *out1) {
    if (!sv || !done) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return GRNS_ERR_INVALID_ARGUMENT;
    *done = it->second.state == 2;
    if (status) *status = it->second.status;
    if (out0) *out0 = it->second.out0;
    if (out1) *out1 = it->second.out1;
    return GRNS_OK;
}

grns_status grns_server_wait(grns_server *sv, uint64_t id, int64_t timeout_us, int32_t *status, uint64_t *out0,
                             uint64_t *out1) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(sv->mu);
    if (sv->reqs.find(id) == sv->reqs.end()) return GRNS_ERR_INVALID_ARGUMENT;
    if (!wait_done(sv, lk, id, timeout_us)) return GRNS_ERR_TIMEOUT;
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return GRNS_ERR_INVALID_ARGUMENT;  // dropped after its retention
    const Req &q = it->second;
    if (status) *status = q.status;
    if (out0) *out0 = q.out0;
    if (out1) *out1 = q.out1;
    return GRNS_OK;
}

grns_status grns_server_cancel(grns_server *sv, uint64_t id) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    auto it = sv->reqs.find(id);
    if (it == sv->reqs.end()) return GRNS_ERR_INVALID_ARGUMENT;
    Req &q = it->second;
    if (q.state == 1) return GRNS_ERR_BUSY;
    if (q.state == 2) return GRNS_OK;
    auto pos = std::find(sv->pending.begin(), sv->pending.end(), id);
    if (pos != sv->pending.end()) sv->pending.erase(pos);
    finish(sv, id, q, GRNS_ERR_CANCELLED, now_us());
    sv->cancelled++;
    return GRNS_OK;
}

grns_status grns_server_stats_get(grns_server *sv, grns_server_stats *st) {
    if (!sv || !st) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    *st = grns_server_stats{};
    st->completed = sv->completed;
    st->rejected = sv->rejected;
    st->pending = sv->pending.size();
    for (const Slot *sl : sv->slots) st->inflight += sl->reqs.size();
    st->launches = sv->launches;
    st->mean_jobs_per_launch = sv->launches ? (double)sv->jobs_launched / (double)sv->launches : 0.0;
    st->bytes_in_use = sv->in_use;
    st->budget = sv->opt.hbm_budget_bytes;
    if (!sv->lat.empty()) {
        std::vector<double> v(sv->lat);
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5))]; };
        st->p50_us = pct(0.50);
        st->p99_us = pct(0.99);
        double s = 0;
        for (double x : v) s += x;
        st->mean_us = s / (double)v.size();
    }
    if (sv->t_last > sv->t_first) st->numbers_per_s = sv->numbers / ((sv->t_last - sv->t_first) * 1e-6);
    return GRNS_OK;
}

grns_status grns_server_set_gather_us(grns_server *sv, int32_t gather_us) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    sv->opt.gather_us = gather_us;
    sv->cv.notify_all();
    return GRNS_OK;
}

grns_status grns_server_reset_stats(grns_server *sv) {
    if (!sv) return GRNS_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> g(sv->mu);
    sv->lat.clear();
    sv->completed = sv->rejected = sv->launches = sv->jobs_launched = 0;
    sv->numbers = 0;
    sv->t_first = sv->t_last = 0;
    return GRNS_OK;
}

}  // extern "C"
