/*
 * The reference library's n-threaded device functions (kisupov/grns
 * src/rnseval.cuh:332 rns_eval_compute_parallel, src/rnscmp.cuh:87
 * rns_cmp_parallel, src/rnsdiv.cuh:244/:301 rns_div_parallel /
 * rns_div_parallel_fast, src/mrc.cuh:121 mrc_pipeline) executed on the CPU
 * as one thread block: RNS_MODULI_SIZE host threads, one per CUDA thread,
 * with the block semantics of oracle/ref/shim/cuda_host_shim.h
 * (ORACLE_BLOCK_EMULATION).  A checker of the oracle's restatement of the
 * n-threaded summation order (oracle/grns_oracle_n.h eval_dpar) -- test
 * infrastructure only, built by oracle/ref/build_ref.py into oracle/_ref/.
 *
 * Only blocks of whole warps (RNS_MODULI_SIZE a multiple of 32) are defined
 * here: with fewer threads the reference's full-mask shuffles read lanes
 * that do not exist, which CUDA leaves undefined.
 */
#include <condition_variable>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

/* CUDA gives a __shared__ local one instance per block: here a static.  The
 * one header that writes `static __shared__` (pairwise.cuh) reaches this unit
 * through the recipe's standard input with those two words as `__shared__`
 * (oracle/ref/build_ref.py), ahead of this file; the rest are read as they
 * lie in the reference checkout */
#undef __shared__
#define __shared__ static
#include "rnseval.cuh"
#include "rnscmp.cuh"
#include "rnsdiv.cuh"
#include "rnsscal.cuh"
#include "mpint.cuh"
#undef __shared__
#define __shared__

#define N_ RNS_MODULI_SIZE
static_assert(N_ % 32 == 0, "block emulation needs whole warps");

thread_local oracle_shim_dim3 threadIdx;
oracle_shim_dim3 blockIdx, blockDim, gridDim;

namespace {

class Barrier {
  public:
    explicit Barrier(int n) : n_(n) {}
    void wait() {
        std::unique_lock<std::mutex> lk(mu_);
        const unsigned g = gen_;
        if (++count_ == n_) {
            count_ = 0;
            gen_++;
            cv_.notify_all();
        } else {
            cv_.wait(lk, [&] { return gen_ != g; });
        }
    }

  private:
    std::mutex mu_;
    std::condition_variable cv_;
    int n_, count_ = 0;
    unsigned gen_ = 0;
};

Barrier *g_block = nullptr;
std::vector<Barrier *> g_warp;
double g_lane[N_];  // shuffle exchange: lane values of every warp

/* body(t) on N_ threads as one block (threadIdx.x = t) */
template <class F>
void run_block(F body) {
    Barrier block(N_);
    std::vector<std::unique_ptr<Barrier>> warps;
    for (int w = 0; w < N_ / 32; w++) warps.emplace_back(new Barrier(32));
    g_block = &block;
    g_warp.clear();
    for (auto &w : warps) g_warp.push_back(w.get());
    blockDim = {N_, 1, 1};
    gridDim = {1, 1, 1};
    blockIdx = {0, 0, 0};
    std::vector<std::thread> th;
    for (int t = 0; t < N_; t++)
        th.emplace_back([&, t] {
            threadIdx = {(unsigned)t, 0, 0};
            body(t);
        });
    for (auto &x : th) x.join();
    g_block = nullptr;
}

}  // namespace

void oracle_block_sync() { g_block->wait(); }

double oracle_warp_shfl_down(double v, int delta) {
    const int t = (int)threadIdx.x, lane = t % 32;
    Barrier *b = g_warp[t / 32];
    g_lane[t] = v;
    b->wait();
    const double r = lane + delta < 32 ? g_lane[t + delta] : v;  // beyond the warp: the caller's own value
    b->wait();
    return r;
}

extern "C" {

int ref_block_n() { return N_; }

}  // extern "C"

/* the block's copies of the current number(s), block-wide like __shared__ */
static int g_x[N_], g_y[N_], g_q[N_], g_r[N_];

extern "C" {

void ref_block_init() {
    rns_const_init();
    mpint_const_init();
}

/* x: count numbers, AoS; every number evaluated by one block run */
void ref_block_eval(const int *x, long count, interval_t *out) {
    int *xs = g_x;
    run_block([&](int t) {
        for (long k = 0; k < count; k++) {
            xs[t] = x[k * N_ + t];
            __syncthreads();
            cuda::rns_eval_compute_parallel(&out[k].low, &out[k].upp, xs);
            __syncthreads();
        }
    });
}

void ref_block_cmp(const int *x, const int *y, long count, int *out) {
    int *xs = g_x, *ys = g_y;
    run_block([&](int t) {
        for (long k = 0; k < count; k++) {
            xs[t] = x[k * N_ + t];
            ys[t] = y[k * N_ + t];
            __syncthreads();
            const int c = cuda::rns_cmp_parallel(xs, ys);
            if (t == 0) out[k] = c;
            __syncthreads();
        }
    });
}

/* fast = 0: rns_div_parallel, 1: rns_div_parallel_fast */
void ref_block_div(const int *x, const int *d, long count, int *q, int *r, int fast) {
    int *xs = g_x, *ds = g_y, *qs = g_q, *rs = g_r;
    run_block([&](int t) {
        for (long k = 0; k < count; k++) {
            xs[t] = x[k * N_ + t];
            ds[t] = d[k * N_ + t];
            __syncthreads();
            if (fast) cuda::rns_div_parallel_fast(qs, rs, xs, ds);
            else cuda::rns_div_parallel(qs, rs, xs, ds);
            __syncthreads();
            q[k * N_ + t] = qs[t];
            r[k * N_ + t] = rs[t];
            __syncthreads();
        }
    });
}

void ref_block_mrc(const int *x, long count, int *mr) {
    int *xs = g_x, *ms = g_q;
    run_block([&](int t) {
        for (long k = 0; k < count; k++) {
            xs[t] = x[k * N_ + t];
            __syncthreads();
            cuda::mrc_pipeline(ms, xs);
            __syncthreads();
            mr[k * N_ + t] = ms[t];
            __syncthreads();
        }
    });
}

}  // extern "C"
