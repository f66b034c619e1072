/*
 * grns_gb300 -- multiple-precision integer kernels over arrays of mp_int_t
 * (reference layout, src/types.cuh:45): add / sub / mul with the interval
 * evaluation derived from the operands' evaluations, as cuda::mpint_add /
 * mpint_sub / mpint_mul (reference src/mpint.cuh:336/:407/:478).  Overflow
 * goes to the per-element flags (the reference prints from the device).
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
#define C_(n) return run_mpint<n>(c, op, x, y, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
