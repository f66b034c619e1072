/*
 * grns_gb300 -- multiple-precision integer kernels over arrays of mp_int_t
 * (reference layout, src/types.cuh:45): add / sub / mul with the interval
 * evaluation derived from the operands' evaluations, as cuda::mpint_add /
 * mpint_sub / mpint_mul (reference src/mpint.cuh:336/:407/:478).  Overflow
 * goes to the per-element flags (the reference prints from the device).
 *
 * mpint_div (src/mpint.cuh:511) runs in three launches: the digit columns of
 * both operands are gathered into residue-major scratch, the division driver
 * of grns_div computes |x| div |y| and the remainder, and a finishing kernel
 * applies the Euclidean step (a negative dividend with a nonzero remainder
 * takes one more), evaluates the quotient and sets the sign.
 */
#include "internal.h"
#include "rns_mpint.cuh"

namespace grns {

template <int N>
__global__ void __launch_bounds__(256) k_mpint(const __grid_constant__ Consts<N> C, int op,
                                               const MpInt<N> *__restrict__ x, const MpInt<N> *__restrict__ y,
                                               int64_t count, MpInt<N> *__restrict__ out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        MpInt<N> a = x[k], b = y[k], r;
        r.pad = 0;
        uint32_t f = 0;
        if (op == 2) mpint_mul<N>(C, r, a, b, f);
        else mpint_addsub<N>(C, r, a, b, op == 1, f);
        out[k] = r;
        if (flags) flags[k] = (uint8_t)f;
    }
}

/* residue-major columns of the operands' digits: xs[i * count + k] = x[k].digits[i] */
template <int N>
__global__ void __launch_bounds__(256) k_mpint_gather(const MpInt<N> *__restrict__ x, const MpInt<N> *__restrict__ y,
                                                      int64_t count, uint32_t *__restrict__ xs,
                                                      uint32_t *__restrict__ ys) {
    const int64_t total = count * N;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / N;
        const int i = (int)(t - k * N);
        xs[(int64_t)i * count + k] = __ldg(&x[k].digits[i]);
        ys[(int64_t)i * count + k] = __ldg(&y[k].digits[i]);
    }
}

/* Euclidean adjustment, evaluation and sign of mpint_div from the division's
 * quotient and remainder columns; flags holds the division's flags on entry.
 * A zero divisor or an invalid digit gives the zero record. */
template <int N>
__global__ void __launch_bounds__(128) k_mpint_div_finish(const __grid_constant__ Consts<N> C,
                                                          const MpInt<N> *__restrict__ x,
                                                          const MpInt<N> *__restrict__ y,
                                                          const uint32_t *__restrict__ q,
                                                          const uint32_t *__restrict__ r, int64_t count,
                                                          MpInt<N> *__restrict__ out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = flags[k];
        const bool bad = (f & (kFlagInvalidInput | kFlagDivByZero)) != 0;
        bool rz = true;
#pragma unroll 8
        for (int i = 0; i < N; i++) rz &= __ldg(r + (int64_t)i * count + k) == 0;
        const int xs = __ldg(&x[k].sign), ys = __ldg(&y[k].sign);
        const bool inc = xs == 1 && !rz && !bad;
        MpInt<N> res;
        bool qz = true;
#pragma unroll 8
        for (int i = 0; i < N; i++) {
            uint32_t v = bad ? 0u : __ldg(q + (int64_t)i * count + k);
            if (inc) v = addmod(v, 1u, C.m[i]);
            res.digits[i] = v;
            qz &= v == 0;
        }
        eval<N>(C, [&](int i) { return res.digits[i]; }, res.eval[0], res.eval[1], f);
        res.sign = qz ? 0 : (xs ^ ys);
        res.pad = 0;
        out[k] = res;
        flags[k] = (uint8_t)f;
    }
}

template <int N>
static grns_status run_mpint_div(const grns_ctx *c, const void *x, const void *y, int64_t count, void *out,
                                 uint8_t *flags, cudaStream_t s) {
    const size_t words = (size_t)N * count;
    void *scratch = nullptr;
    cudaError_t e = scratch_alloc(c, &scratch, words * 4 * sizeof(uint32_t) + (flags ? 0 : (size_t)count), s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t *xs = (uint32_t *)scratch, *ys = xs + words, *q = ys + words, *r = q + words;
    uint8_t *f = flags ? flags : (uint8_t *)(r + words);
    const MpInt<N> *xm = (const MpInt<N> *)x, *ym = (const MpInt<N> *)y;
    k_mpint_gather<N><<<grid_for(c, count * N, 256), 256, 0, s>>>(xm, ym, count, xs, ys);
    grns_status st = cuda_status(cudaGetLastError());
    if (st == GRNS_OK) st = launch_div(c, xs, ys, count, count, q, r, f, s);
    if (st == GRNS_OK) {
        k_mpint_div_finish<N><<<grid_for(c, count, 128), 128, 0, s>>>(consts_of<N>(c), xm, ym, q, r, count,
                                                                      (MpInt<N> *)out, f);
        st = cuda_status(cudaGetLastError());
    }
    scratch_free(scratch, s);
    return st;
}

template <int N>
static grns_status run_mpint(const grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                             uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    k_mpint<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), op, (const MpInt<N> *)x, (const MpInt<N> *)y,
                                                  count, (MpInt<N> *)out, flags);
    return cuda_status(cudaGetLastError());
}

grns_status launch_mpint(const grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                         uint8_t *flags, cudaStream_t s) {
#define C_(n) return op == 3 ? run_mpint_div<n>(c, x, y, count, out, flags, s) : run_mpint<n>(c, op, x, y, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
