/*
 * grns_gb300 -- division and power-of-two scaling kernels (reference-faithful
 * forms; one thread per number, operands gathered into registers/local
 * arrays, results written per modulus slice).
 *   k_div  : q = floor(X/D), r = X - qD      (reference src/rnsdiv.cuh:128)
 *   k_scale: floor(X / 2^D)                  (reference src/rnsscal.cuh:207)
 */
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

template <int N, bool FAST>
__global__ void __launch_bounds__(128) k_div(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> d,
                                             int64_t count, Output<N> q, Output<N> r, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], da[N], qa[N], ra[N], f = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            da[i] = d.load(k, i);
            f |= (xa[i] >= C.m[i] || da[i] >= C.m[i]) ? kFlagInvalidInput : 0u;
        }
        if (f) {
#pragma unroll
            for (int i = 0; i < N; i++) { qa[i] = 0; ra[i] = 0; }
        } else if (FAST) {
            div_fast<N>(C, qa, ra, xa, da, f);
        } else {
            div_ref<N>(C, qa, ra, xa, da, f);
        }
#pragma unroll
        for (int i = 0; i < N; i++) {
            q.store(k, i, qa[i]);
            r.store(k, i, ra[i]);
        }
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N, bool FAST>
__global__ void __launch_bounds__(128) k_scale(const __grid_constant__ Consts<N> C, Operand<N> x,
                                               const uint32_t *__restrict__ D, uint32_t D_uniform, int64_t count,
                                               Output<N> out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], ya[N], f = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            f |= xa[i] >= C.m[i] ? kFlagInvalidInput : 0u;
        }
        unsigned dk = D ? __ldg(D + k) : D_uniform;
        if (f) {
#pragma unroll
            for (int i = 0; i < N; i++) ya[i] = 0;
        } else if (FAST) {
            scale_fast<N>(C, ya, xa, dk);
        } else {
            scale2pow_ref<N>(C, ya, xa, dk);
        }
#pragma unroll
        for (int i = 0; i < N; i++) out.store(k, i, ya[i]);
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N>
static grns_status run_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                           uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE)
        k_div<N, false><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{d, ld},
                                                               count, Output<N>{q, ld}, Output<N>{r, ld}, flags);
    else
        k_div<N, true><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{d, ld},
                                                              count, Output<N>{q, ld}, Output<N>{r, ld}, flags);
    return cuda_status(cudaGetLastError());
}

template <int N>
static grns_status run_scale(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                             int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE)
        k_scale<N, false><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, count,
                                                                 Output<N>{out, ld}, flags);
    else
        k_scale<N, true><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, count,
                                                                Output<N>{out, ld}, flags);
    return cuda_status(cudaGetLastError());
}

grns_status launch_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                       uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_div<n>(c, x, d, ld, count, q, r, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_scale2pow(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                             int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_scale<n>(c, x, D, Du, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
