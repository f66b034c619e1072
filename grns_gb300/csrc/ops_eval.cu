/*
 * grns_gb300 -- interval evaluation and magnitude comparison kernels.
 *   k_eval: out[k] = rns_eval_compute(X_k)   (reference src/rnseval.cuh:182)
 *   k_cmp : out[k] = rns_cmp(X_k, Y_k)       (reference src/rnscmp.cuh:55),
 *           both evaluations fused in registers, never written back.
 * One thread per number, grid-stride, residues read per modulus slice.
 */
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

template <int N>
__global__ void __launch_bounds__(256) k_eval(const __grid_constant__ Consts<N> C, Operand<N> x, int64_t count,
                                              Er *__restrict__ out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        Er lo, up;
        eval<N>(C, [&](int i) { return x.load(k, i); }, lo, up, f);
        out[2 * k] = lo;
        out[2 * k + 1] = up;
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N>
__global__ void __launch_bounds__(256) k_cmp(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> y,
                                             int64_t count, int32_t *__restrict__ out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        Er xl, xu, yl, yu;
        auto gx = [&](int i) { return x.load(k, i); };
        auto gy = [&](int i) { return y.load(k, i); };
        eval<N>(C, gx, xl, xu, f);
        eval<N>(C, gy, yl, yu, f);
        int r = cmp_intervals<N>(xl, xu, yl, yu);
        if (r == 2) r = cmp_tie<N>(C, gx, gy);
        out[k] = f ? 0 : r;
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N>
__device__ __noinline__ int fast_tie_cmp(const Consts<N> &C, const Operand<N> x, const Operand<N> y, int64_t k) {
    return cmp_fx96_then_exact<N>(C, [&](int i) { return x.load(k, i); }, [&](int i) { return y.load(k, i); });
}

/* fast path: 64-bit fixed-point enclosures on the integer pipe, exact fallback */
template <int N>
__global__ void __launch_bounds__(256) k_cmp_fast(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> y,
                                                  int64_t count, int32_t *__restrict__ out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        auto gx = [&](int i) { return x.load(k, i); };
        auto gy = [&](int i) { return y.load(k, i); };
        uint64_t a = 0, b = 0;
        uint32_t bad = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            const uint32_t xi = gx(i), yi = gy(i);
            bad |= (uint32_t)(xi >= C.m[i]) | (uint32_t)(yi >= C.m[i]);
            const uint32_t sx = mulmod_shoup(xi, C.w[i], C.w_sh[i], C.m[i]);
            const uint32_t sy = mulmod_shoup(yi, C.w[i], C.w_sh[i], C.m[i]);
            a += (uint64_t)sx * C.c64l[i];
            a += (uint64_t)(uint32_t)(sx * C.c64h[i]) << 32;
            b += (uint64_t)sy * C.c64l[i];
            b += (uint64_t)(uint32_t)(sy * C.c64h[i]) << 32;
        }
        int r = fx64_order(a, b, C.E);
        if (r == 2 && !bad) r = fast_tie_cmp<N>(C, x, y, k);
        out[k] = bad ? 0 : r;
        if (flags) flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
    }
}

template <int N>
static grns_status run_eval(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                            uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    k_eval<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, (Er *)out, flags);
    return cuda_status(cudaGetLastError());
}

template <int N>
static grns_status run_cmp(const grns_ctx *c, const uint32_t *x, const uint32_t *y, int64_t ld, int64_t count,
                           int32_t *out, uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    if (c->path == GRNS_PATH_REFERENCE)
        k_cmp<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{y, ld}, count, out,
                                                    flags);
    else
        k_cmp_fast<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{y, ld}, count,
                                                         out, flags);
    return cuda_status(cudaGetLastError());
}

grns_status launch_eval(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                        uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_eval<n>(c, x, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_cmp(const grns_ctx *c, const uint32_t *x, const uint32_t *y, int64_t ld, int64_t count,
                       int32_t *out, uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_cmp<n>(c, x, y, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
