/*
 * grns_gb300 -- autotuner for the batched kernel's per-op schedule.
 *
 * For one op and moduli set it times each candidate (serial vs n-threaded
 * lane groups for cmp and max; chunk length for all) in a single-job batch on
 * synthetic inputs generated on the device, keeps the fastest in the context,
 * and appends "gpu|n|op|log2(count)|coop|chunk|ms" to a plain-text cache that
 * grns_autotune_load re-applies on the same GPU model.
 */
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "internal.h"

namespace {

std::string gpu_name(int device) {
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return "unknown";
    std::string s = p.name;
    for (char &ch : s)
        if (ch == ' ' || ch == '|') ch = '_';
    return s;
}

struct DevBuf {
    void *p = nullptr;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t alloc(size_t bytes) { return cudaMalloc(&p, bytes ? bytes : 16); }
};

}  // namespace

extern "C" {

grns_status grns_autotune(grns_ctx *c, int op, int64_t count, const char *cache_path, grns_schedule *chosen,
                          double *best_ms) {
    if (!c || op < GRNS_OP_EVAL || op > GRNS_OP_MPINT_MUL || count <= 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (c->n > grns::kBatchMaxModuli) return GRNS_ERR_UNSUPPORTED;
    const int n = c->n;
    const bool mp = op >= GRNS_OP_MPINT_ADD;
    const size_t num_bytes = mp ? GRNS_MPINT_BYTES(n) : (size_t)n * 4;
    DevBuf a, b, o0, o1;
    cudaError_t e = a.alloc(num_bytes * count);
    if (e == cudaSuccess) e = b.alloc(num_bytes * count);
    if (e == cudaSuccess) e = o0.alloc(op == GRNS_OP_EVAL ? 32 * count : num_bytes * count);
    if (e == cudaSuccess) e = o1.alloc(num_bytes * count);
    if (e != cudaSuccess) return grns::cuda_status(e);
    cudaStream_t s = nullptr;
    if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return grns::cuda_status(e);
    grns_status st = GRNS_OK;
    if (mp) {
        e = cudaMemsetAsync(a.p, 0, num_bytes * count, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(b.p, 0, num_bytes * count, s);
        st = grns::cuda_status(e);
    } else {
        st = grns_gen_uniform(c, 12345, 1, count, GRNS_LAYOUT_SOA, (int32_t *)a.p, s);
        if (st == GRNS_OK) {
            if (op == GRNS_OP_DIV) st = grns_gen_divisors(c, 12345, count, GRNS_LAYOUT_SOA, (int32_t *)b.p, s);
            else if (op == GRNS_OP_SCALE2POW) st = grns_gen_shifts(12345, count, 900, (uint32_t *)b.p, s);
            else st = grns_gen_uniform(c, 12345, 2, count, GRNS_LAYOUT_SOA, (int32_t *)b.p, s);
        }
    }
    if (st != GRNS_OK) {
        cudaStreamDestroy(s);
        return st;
    }
    grns_job job{};
    job.op = op;
    job.layout = GRNS_LAYOUT_SOA;
    job.count = count;
    job.a = a.p;
    job.b = (op == GRNS_OP_EVAL || op == GRNS_OP_MAX) ? nullptr : b.p;
    job.out0 = o0.p;
    job.out1 = (op == GRNS_OP_DIV || op == GRNS_OP_MAX) ? o1.p : nullptr;

    std::vector<grns::Sched> cands;
    /* division and scaling chunks are refilled lane by lane inside a warp,
     * so longer chunks trade tail length against balance; the memory-bound
     * ops want long chunks */
    const int chunks_cheap[] = {256, 1024, 4096}, chunks_div[] = {64, 256, 1024}, chunks_scale[] = {64, 256, 1024};
    const int *chunks = op == GRNS_OP_DIV ? chunks_div : op == GRNS_OP_SCALE2POW ? chunks_scale : chunks_cheap;
    for (int coop = 0; coop <= ((op == GRNS_OP_CMP || op == GRNS_OP_MAX) ? 1 : 0); coop++)
        for (int t = 0; t < 3; t++) cands.push_back(grns::Sched{coop, chunks[t]});

    const grns::Sched saved = c->sched[op];
    grns::Sched best = saved;
    double best_t = 1e30;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (const auto &cand : cands) {
        c->sched[op] = cand;
        grns_batch *bt = nullptr;
        st = grns_batch_create(c, &job, 1, 0, &bt);
        if (st != GRNS_OK) break;
        st = grns_batch_launch(bt, s);  // warm-up
        float ms = 1e30f;
        for (int rep = 0; rep < 3 && st == GRNS_OK; rep++) {
            cudaEventRecord(e0, s);
            st = grns_batch_launch(bt, s);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            float t = 0;
            cudaEventElapsedTime(&t, e0, e1);
            if (t < ms) ms = t;
        }
        grns_batch_destroy(bt);
        if (st != GRNS_OK) break;
        if (ms < best_t) {
            best_t = ms;
            best = cand;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaStreamDestroy(s);
    c->sched[op] = st == GRNS_OK ? best : saved;
    if (st != GRNS_OK) return st;
    if (chosen) *chosen = grns_schedule{best.coop, best.chunk};
    if (best_ms) *best_ms = best_t;
    if (cache_path) {
        FILE *f = std::fopen(cache_path, "a");
        if (f) {
            std::fprintf(f, "%s|%d|%d|%d|%d|%d|%.6f\n", gpu_name(c->device).c_str(), n, op,
                         (int)std::lround(std::log2((double)count)), best.coop, best.chunk, best_t);
            std::fclose(f);
        }
    }
    return GRNS_OK;
}

grns_status grns_autotune_load(grns_ctx *c, const char *cache_path, int *applied) {
    if (!c || !cache_path) return GRNS_ERR_INVALID_ARGUMENT;
    FILE *f = std::fopen(cache_path, "r");
    if (applied) *applied = 0;
    if (!f) return GRNS_OK;
    const std::string me = gpu_name(c->device);
    char line[512];
    int count = 0;
    while (std::fgets(line, sizeof line, f)) {
        char name[256];
        int n, op, lg, coop, chunk;
        double ms;
        if (std::sscanf(line, "%255[^|]|%d|%d|%d|%d|%d|%lf", name, &n, &op, &lg, &coop, &chunk, &ms) != 7) continue;
        if (me != name || n != c->n || op < 0 || op > 7) continue;
        grns_schedule sc{coop, chunk};
        if (grns_ctx_set_schedule(c, op, &sc) == GRNS_OK) count++;  // later lines win
    }
    std::fclose(f);
    if (applied) *applied = count;
    return GRNS_OK;
}

}  // extern "C"
