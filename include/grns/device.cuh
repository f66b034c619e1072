/*
 * grns_gb300 -- source-level drop-in for the reference's per-number device
 * functions (kisupov/grns, namespace cuda), for user kernels that call them
 * one number per thread.
 *
 * Usage, as with the reference: define the moduli set with the params.h
 * convention (RNS_MODULI_SIZE, RNS_MODULI_VALUES -- e.g. include your
 * params.h), include this header in the .cu file that holds your kernels,
 * call rns_const_init() (and mpint_const_init()) on the host before the first
 * launch, then call inside kernels:
 *
 *   cuda::rns_eval_compute(er_float_ptr low, er_float_ptr upp, int *x)   src/rnseval.cuh:182
 *   cuda::rns_eval_compute_fast(low, upp, x)                             src/rnseval.cuh:266
 *   int cuda::rns_cmp(int *x, int *y)                                    src/rnscmp.cuh:55
 *   cuda::rns_div(int *q, int *r, int *x, int *d)                        src/rnsdiv.cuh:128
 *   cuda::rns_scale2pow(int *result, int *x, unsigned D)                 src/rnsscal.cuh:207
 *   cuda::mpint_add / mpint_sub / mpint_mul / mpint_div(mp_int_ptr r, mp_int_ptr x, mp_int_ptr y)
 *                                                                        src/mpint.cuh:336/407/478/511
 *   cuda::rns_div_fast(q, r, x, d)                                       src/rnsdiv.cuh:180
 *   cuda::mrc(int *mr, int *x), int cuda::mrc_compare_rns(int *x, int *y) src/mrc.cuh:101/:162
 *
 * and the n-threaded forms, called by all RNS_MODULI_SIZE threads of a block
 * of exactly that many threads, thread i on residue i (as the reference):
 *
 *   cuda::rns_eval_compute_parallel(low, upp, x)                         src/rnseval.cuh:332
 *   int cuda::rns_cmp_parallel(x, y)                                     src/rnscmp.cuh:87
 *   cuda::rns_div_parallel / rns_div_parallel_fast(q, r, x, d)           src/rnsdiv.cuh:244/:301
 *   cuda::mrc_pipeline(mr, x), int cuda::mrc_pipeline_msd(x),
 *   int cuda::mrc_pipeline_compare_rns(x, y)                             src/mrc.cuh:121/:142/:175
 *
 * Results: the interval of rns_eval_compute bit for bit (the reference's
 * device path); the integer results of rns_cmp, rns_div, rns_scale2pow,
 * mrc and the mp_int operations exactly (computed with this library's
 * integer-pipe algorithms, which return the same integers).
 * rns_eval_compute_parallel sums in the reference's n-threaded order (lane l
 * adds lane l + 16, then l + 8, ..., then the warp sums), which gives bounds
 * of its own, bit for bit for n a multiple of 32; for n < 32 the reference's
 * shuffles read lanes that do not exist, so its bounds are undefined, and
 * here the absent lanes are skipped.  The n-threaded integer operations give
 * the serial results (thread 0 computes them, every thread receives them);
 * unlike the reference's refinement loop, no shared value is rewritten before
 * every thread has read it.  Like the reference's, the
 * constants live in per-translation-unit device memory (a __constant__
 * block plus one table allocation kept until exit), so the kernels that use
 * them belong in the translation unit that calls rns_const_init().  The
 * integer-heavy functions (rns_div, rns_scale2pow, mrc, mrc_compare_rns,
 * mpint_div) are compiled once per translation unit and called, not inlined:
 * a kernel that inlined mpint_div, rns_div_fast and mrc_compare_rns together
 * returned wrong mixed-radix digits from the inlined mrc.  For
 * whole arrays, prefer the C ABI (grns.h): it is faster than one call per
 * thread.  rns_const_init() returns nothing, as the reference's does; it
 * leaves the constants zeroed when CUDA fails, and grns_device_init_status()
 * reports the error.
 */
#ifndef GRNS_GB300_DEVICE_CUH
#define GRNS_GB300_DEVICE_CUH

#if !defined(RNS_MODULI_SIZE) || !defined(RNS_MODULI_VALUES)
#error "define RNS_MODULI_SIZE and RNS_MODULI_VALUES (the params.h convention) before including grns/device.cuh"
#endif

#include <cuda_runtime.h>

#include <vector>

#include "../../grns_gb300/csrc/consts_host.h"
#include "../../grns_gb300/csrc/rns_device.cuh"
#include "../../grns_gb300/csrc/rns_fast.cuh"
#include "../../grns_gb300/csrc/rns_mpint.cuh"
#include "types.h"

typedef er_float_t *er_float_ptr;
typedef interval_t *interval_ptr;
typedef struct {  // the reference's mp_int_t for this moduli set (src/types.cuh:45)
    int digits[RNS_MODULI_SIZE];
    int sign;
    er_float_t eval[2];
} mp_int_t;
typedef mp_int_t *mp_int_ptr;
static_assert(sizeof(mp_int_t) == sizeof(grns::MpInt<RNS_MODULI_SIZE>), "mp_int_t layout");

__constant__ grns::Consts<RNS_MODULI_SIZE> grns_dev_consts;

/* per-translation-unit state (internal linkage: several libraries built on
 * this header with different moduli sets can share a process) */
namespace grns_device_detail {
static inline cudaError_t &init_status() {
    static cudaError_t st = cudaErrorNotReady;
    return st;
}
static inline void *&tables() {
    static void *p = nullptr;
    return p;
}
/* mp_int_t <-> the library's record, member by member (no type punning) */
__device__ __forceinline__ grns::MpInt<RNS_MODULI_SIZE> load_mp(const mp_int_t *p) {
    grns::MpInt<RNS_MODULI_SIZE> m;
    for (int i = 0; i < RNS_MODULI_SIZE; i++) m.digits[i] = (uint32_t)p->digits[i];
    m.sign = p->sign;
    m.pad = 0;
    m.eval[0] = grns::Er{p->eval[0].frac, (int64_t)p->eval[0].exp};
    m.eval[1] = grns::Er{p->eval[1].frac, (int64_t)p->eval[1].exp};
    return m;
}
__device__ __forceinline__ void store_mp(mp_int_t *p, const grns::MpInt<RNS_MODULI_SIZE> &m) {
    for (int i = 0; i < RNS_MODULI_SIZE; i++) p->digits[i] = (int)m.digits[i];
    p->sign = m.sign;
    p->eval[0].frac = m.eval[0].frac;
    p->eval[0].exp = m.eval[0].exp;
    p->eval[1].frac = m.eval[1].frac;
    p->eval[1].exp = m.eval[1].exp;
}
}  // namespace grns_device_detail

/* builds the constant tables of the RNS_MODULI_VALUES set for the current
 * device (the reference's rns_const_init, src/rnsbase.cuh:324) */
static inline void rns_const_init() {
    static const int moduli[RNS_MODULI_SIZE] = RNS_MODULI_VALUES;
    grns::HostTables T;
    grns::build_tables(T, reinterpret_cast<const uint32_t *>(moduli), RNS_MODULI_SIZE);
    const std::vector<uint32_t> blob = grns::table_blob(T);
    void *&d = grns_device_detail::tables();
    cudaError_t e = cudaSuccess;
    if (!d) e = cudaMalloc(&d, blob.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d, blob.data(), blob.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        static grns::Consts<RNS_MODULI_SIZE> C;
        grns::fill_consts<RNS_MODULI_SIZE>(C, T, static_cast<const uint32_t *>(d));
        e = cudaMemcpyToSymbol(grns_dev_consts, &C, sizeof(C));
    }
    grns_device_detail::init_status() = e;
}
/* the reference's mpint_const_init (src/mpint.cuh:20): the mp_int operations
 * need no constants beyond rns_const_init's */
static inline void mpint_const_init() {}
/* cudaSuccess once rns_const_init() has built the tables */
static inline cudaError_t grns_device_init_status() { return grns_device_detail::init_status(); }

namespace cuda {

__device__ __forceinline__ void rns_eval_compute(er_float_ptr low, er_float_ptr upp, int *x) {
    grns::Er lo, up;
    uint32_t f = 0;
    grns::eval<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; }, lo, up, f);
    low->frac = lo.frac;
    low->exp = lo.exp;
    upp->frac = up.frac;
    upp->exp = up.exp;
}

/* for numbers "not too large" (below about M/2), as the reference's */
__device__ __forceinline__ void rns_eval_compute_fast(er_float_ptr low, er_float_ptr upp, int *x) {
    grns::Er lo, up;
    uint32_t f = 0;
    auto get = [&](int i) { return (uint32_t)x[i]; };
    grns::eval<RNS_MODULI_SIZE, decltype(get), true>(grns_dev_consts, get, lo, up, f);
    low->frac = lo.frac;
    low->exp = lo.exp;
    upp->frac = up.frac;
    upp->exp = up.exp;
}

__device__ __forceinline__ int rns_cmp(int *x, int *y) {
    return grns::cmp_fast<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; },
                                           [&](int i) { return (uint32_t)y[i]; });
}

__device__ __noinline__ void rns_div(int *q, int *r, int *x, int *d) {
    constexpr int N = RNS_MODULI_SIZE;
    uint32_t xx[N], dd[N], qq[N], rr[N], f = 0;
    for (int i = 0; i < N; i++) {
        xx[i] = (uint32_t)x[i];
        dd[i] = (uint32_t)d[i];
    }
    grns::div_fast<N>(grns_dev_consts, qq, rr, xx, dd, f);
    for (int i = 0; i < N; i++) {
        q[i] = (int)qq[i];
        r[i] = (int)rr[i];
    }
}

__device__ __noinline__ void rns_scale2pow(int *result, int *x, unsigned D) {
    constexpr int N = RNS_MODULI_SIZE;
    uint32_t xx[N], yy[N];
    for (int i = 0; i < N; i++) xx[i] = (uint32_t)x[i];
    grns::scale_fast<N>(grns_dev_consts, yy, xx, D);
    for (int i = 0; i < N; i++) result[i] = (int)yy[i];
}

__device__ __forceinline__ void mpint_add(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using namespace grns_device_detail;
    uint32_t f = 0;
    grns::MpInt<RNS_MODULI_SIZE> r;
    grns::mpint_addsub<RNS_MODULI_SIZE>(grns_dev_consts, r, load_mp(x), load_mp(y), false, f);
    store_mp(result, r);
}

__device__ __forceinline__ void mpint_sub(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using namespace grns_device_detail;
    uint32_t f = 0;
    grns::MpInt<RNS_MODULI_SIZE> r;
    grns::mpint_addsub<RNS_MODULI_SIZE>(grns_dev_consts, r, load_mp(x), load_mp(y), true, f);
    store_mp(result, r);
}

__device__ __forceinline__ void rns_div_fast(int *q, int *r, int *x, int *d) { rns_div(q, r, x, d); }

__device__ __noinline__ void mrc(int *mr, int *x) {
    constexpr int N = RNS_MODULI_SIZE;
    uint32_t a[N];
    grns::mrc_digits<N>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; }, a);
    for (int i = 0; i < N; i++) mr[i] = (int)a[i];
}

__device__ __noinline__ int mrc_compare_rns(int *x, int *y) {
    uint32_t a[RNS_MODULI_SIZE], b[RNS_MODULI_SIZE];
    grns::mrc_digits<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; }, a);
    grns::mrc_digits<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)y[i]; }, b);
    for (int i = RNS_MODULI_SIZE - 1; i >= 0; i--)
        if (a[i] != b[i]) return a[i] > b[i] ? 1 : -1;
    return 0;
}

__device__ __forceinline__ void mpint_mul(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using namespace grns_device_detail;
    uint32_t f = 0;
    grns::MpInt<RNS_MODULI_SIZE> r;
    grns::mpint_mul<RNS_MODULI_SIZE>(grns_dev_consts, r, load_mp(x), load_mp(y), f);
    store_mp(result, r);
}

/* Euclidean quotient (src/mpint.cuh:511): |x| div |y|, plus one for a negative
 * x with a nonzero remainder; sign x.sign ^ y.sign, 0 for a zero quotient */
__device__ __noinline__ void mpint_div(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    constexpr int N = RNS_MODULI_SIZE;
    uint32_t q[N], r[N], f = 0;
    uint32_t xd[N], yd[N];
    for (int i = 0; i < N; i++) {
        xd[i] = (uint32_t)x->digits[i];
        yd[i] = (uint32_t)y->digits[i];
    }
    grns::div_fast<N>(grns_dev_consts, q, r, xd, yd, f);
    bool rz = true, qz = true;
    for (int i = 0; i < N; i++) rz &= r[i] == 0;
    const int xs = x->sign, ys = y->sign;
    for (int i = 0; i < N; i++) {
        if (xs == 1 && !rz) q[i] = grns::addmod(q[i], 1u, grns_dev_consts.m[i]);
        qz &= q[i] == 0;
    }
    grns::MpInt<N> res;
    uint32_t ef = 0;
    grns::eval<N>(grns_dev_consts, [&](int i) { return q[i]; }, res.eval[0], res.eval[1], ef);
    for (int i = 0; i < N; i++) res.digits[i] = q[i];
    res.sign = qz ? 0 : (xs ^ ys);
    grns_device_detail::store_mp(result, res);
}

/* ---------------- n-threaded forms (a block of RNS_MODULI_SIZE threads) ---------------- */

}  // namespace cuda

namespace grns_device_detail {
/* the n-threaded schedule's sum: lane 0 of every warp reduces its warp by
 * shuffles down (offsets 16, 8, 4, 2, 1), then warp 0 the warp sums; thread 0
 * returns the total */
template <bool UP>
__device__ __forceinline__ double block_sum(double v) {
    constexpr int N = RNS_MODULI_SIZE;
    static_assert(N <= 32 || N % 32 == 0, "n-threaded forms: n <= 32 or a multiple of 32");
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr unsigned mask = N >= 32 ? 0xffffffffu : ((1u << N) - 1u);
    constexpr int lanes = N >= 32 ? 32 : N;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double o = __shfl_down_sync(mask, v, off);
        if (lane + off < lanes) v = UP ? __dadd_ru(v, o) : __dadd_rd(v, o);
    }
    if (N <= 32) return v;
    constexpr int W = N > 32 ? N / 32 : 1;
    __shared__ double part[W];
    if (lane == 0) part[wid] = v;
    __syncthreads();
    double w = lane < W ? part[lane] : 0.0;
    if (wid == 0) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            const double o = __shfl_down_sync(0xffffffffu, w, off);
            if (lane + off < W) w = UP ? __dadd_ru(w, o) : __dadd_rd(w, o);
        }
    }
    __syncthreads();  // part is free for the next sum
    return w;
}
/* thread 0's value, to every thread of the block */
template <class T>
__device__ __forceinline__ T broadcast(T v) {
    __shared__ T sh;
    if (threadIdx.x == 0) sh = v;
    __syncthreads();
    const T r = sh;
    __syncthreads();  // every thread has read sh before it is written again
    return r;
}
__device__ __forceinline__ void set_er(er_float_ptr p, const grns::Er &e) {
    p->frac = e.frac;
    p->exp = e.exp;
}
}  // namespace grns_device_detail

namespace cuda {

__device__ __forceinline__ void rns_eval_compute_parallel(er_float_ptr low, er_float_ptr upp, int *x) {
    using namespace grns_device_detail;
    constexpr int N = RNS_MODULI_SIZE;
    const grns::Consts<N> &C = grns_dev_consts;
    const int t = threadIdx.x;
    uint32_t s = grns::mulmod_shoup((uint32_t)x[t], C.w[t], C.w_sh[t], C.m[t]);
    double suml = broadcast(block_sum<false>(__dmul_rd(grns::u32_to_double(s), C.rrd[t])));
    double sumu = broadcast(block_sum<true>(__dmul_ru(grns::u32_to_double(s), C.rru[t])));
    if (suml == 0 && sumu == 0) {
        if (t == 0) {
            set_er(low, grns::Er{0.0, 0});
            set_er(upp, grns::Er{0.0, 0});
        }
        return;
    }
    const unsigned whl = __double2uint_rz(suml), whu = __double2uint_rz(sumu);
    suml = __dsub_rd(suml, grns::u32_to_double(whl));
    sumu = __dsub_ru(sumu, grns::u32_to_double(whu));
    if (t == 0) {
        set_er(low, grns::er_from_double(suml));
        set_er(upp, grns::er_from_double(sumu));
    }
    int mr = -1;
    if (whl != whu) {
        int msd = 0;
        if (t == 0) {
            uint32_t a[N];
            grns::mrc_digits<N>(C, [&](int i) { return (uint32_t)x[i]; }, a);
            msd = (int)a[N - 1];
        }
        mr = broadcast(msd);
    }
    if (mr > 0) {
        if (t == 0) set_er(upp, C.inv_unit_upp);
        return;
    }
    if (mr == 0 && t == 0) set_er(low, C.unit_low);
    if (sumu >= C.acc) return;
    int K = 0, guard = 0;
    const int cap = C.log2M / (C.ref_factor > 0 ? C.ref_factor : 1) + 8;
    while (sumu < C.acc && ++guard <= cap) {
        const double a = -(ceil(log2(sumu)) + 1);
        int k = (int)(a > (double)C.ref_factor ? a : (double)C.ref_factor);
        if (k < 0 || k > C.log2M) break;
        s = grns::mulmod_barrett(s, __ldg(C.pow2 + (int64_t)k * N + t), C.m[t], C.mu[t], C.b[t]);
        sumu = broadcast(block_sum<true>(__dmul_ru(grns::u32_to_double(s), C.rru[t])));
        sumu = __dsub_ru(sumu, grns::u32_to_double(__double2uint_rz(sumu)));
        K += k;
    }
    suml = block_sum<false>(__dmul_rd(grns::u32_to_double(s), C.rrd[t]));
    if (t == 0) {
        suml = __dsub_rd(suml, grns::u32_to_double(__double2uint_rz(suml)));
        grns::Er lo = grns::er_from_double(suml), up = grns::er_from_double(sumu);
        lo.exp -= K;
        up.exp -= K;
        set_er(low, lo);
        set_er(upp, up);
    }
}

__device__ __forceinline__ int rns_cmp_parallel(int *x, int *y) {
    return grns_device_detail::broadcast(threadIdx.x == 0 ? rns_cmp(x, y) : 0);
}

__device__ __forceinline__ void rns_div_parallel(int *q, int *r, int *x, int *d) {
    constexpr int N = RNS_MODULI_SIZE;
    __shared__ int sq[N], sr[N];
    __syncthreads();  // x and d complete; sq and sr free
    if (threadIdx.x == 0) rns_div(sq, sr, x, d);
    __syncthreads();
    q[threadIdx.x] = sq[threadIdx.x];
    r[threadIdx.x] = sr[threadIdx.x];
    __syncthreads();
}
__device__ __forceinline__ void rns_div_parallel_fast(int *q, int *r, int *x, int *d) { rns_div_parallel(q, r, x, d); }

__device__ __forceinline__ void mrc_pipeline(int *mr, int *x) {
    constexpr int N = RNS_MODULI_SIZE;
    __shared__ int sm[N];
    __syncthreads();
    if (threadIdx.x == 0) mrc(sm, x);
    __syncthreads();
    mr[threadIdx.x] = sm[threadIdx.x];
    __syncthreads();
}
/* the most significant mixed-radix digit on thread 0, 0 on the others (as the reference) */
__device__ __forceinline__ int mrc_pipeline_msd(int *x) {
    constexpr int N = RNS_MODULI_SIZE;
    int msd = 0;
    if (threadIdx.x == 0) {
        uint32_t a[N];
        grns::mrc_digits<N>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; }, a);
        msd = (int)a[N - 1];
    }
    __syncthreads();
    return msd;
}
__device__ __forceinline__ int mrc_pipeline_compare_rns(int *x, int *y) {
    return grns_device_detail::broadcast(threadIdx.x == 0 ? mrc_compare_rns(x, y) : 0);
}

}  // namespace cuda

#endif
