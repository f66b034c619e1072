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

constexpr int kMpTile = 64;      // records per tile of k_mpint_tile
constexpr int kMpParts = 4;      // threads per record
constexpr int kMpTileBlock = kMpTile * kMpParts;

/* copy `bytes` (a multiple of 8) from global to shared memory (or back) with
 * the block's threads: 16-byte words while both sides allow, 8-byte words for
 * the tail (the tiles start 16-byte aligned) */
__device__ __forceinline__ void tile_copy(void *dst, const void *src, int bytes) {
    const int n16 = bytes >> 4;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int t = threadIdx.x; t < n16; t += blockDim.x) d4[t] = s4[t];
    if ((bytes & 15) && threadIdx.x == 0)
        reinterpret_cast<uint2 *>(dst)[2 * n16] = reinterpret_cast<const uint2 *>(src)[2 * n16];
}

/* add / sub / mul over tiles: a block copies kMpTile records of x and y into
 * shared memory with coalesced 16-byte loads, kMpParts threads compute each
 * record there, and the block writes the output tile
 * back with 16-byte stores -- every HBM access a full coalesced line, where
 * a thread copying its own 296-byte records strides the warp's accesses */
template <int N>
__global__ void __launch_bounds__(kMpTileBlock, 2) k_mpint_tile(const __grid_constant__ Consts<N> C, int op,
                                                             const MpInt<N> *__restrict__ x,
                                                             const MpInt<N> *__restrict__ y, int64_t count,
                                                             MpInt<N> *__restrict__ out, uint8_t *__restrict__ flags) {
    extern __shared__ uint4 mp_smem[];
    MpInt<N> *sx = reinterpret_cast<MpInt<N> *>(mp_smem);
    MpInt<N> *sy = sx + kMpTile, *so = sy + kMpTile;
    for (int64_t k0 = (int64_t)blockIdx.x * kMpTile; k0 < count; k0 += (int64_t)gridDim.x * kMpTile) {
        const int nt = count - k0 < kMpTile ? (int)(count - k0) : kMpTile;
        const int bytes = nt * (int)sizeof(MpInt<N>);
        tile_copy(sx, x + k0, bytes);
        tile_copy(sy, y + k0, bytes);
        __syncthreads();
        {  /* kMpParts threads per record, each with every kMpParts-th residue; part 0
            * writes the sign, the evaluation and the flags */
            const int t = threadIdx.x / kMpParts, p = threadIdx.x % kMpParts;
            const bool act = t < nt;
            const MpInt<N> &a = sx[act ? t : 0], &b = sy[act ? t : 0];
            MpInt<N> &r = so[act ? t : 0];
            uint32_t f = 0;
            bool zero = true;
            Er lo{0, 0}, up{0, 0};
            bool minus = false;
            if (act) {
                if (op == 2) {
#pragma unroll 4
                    for (int i = p; i < N; i += kMpParts) {
                        const uint32_t m = C.m[i], u = a.digits[i], v = b.digits[i];
                        f |= (u >= m || v >= m) ? kFlagInvalidInput : 0u;
                        const uint32_t w = mulmod_barrett(u, v, m, C.mu[i], C.b[i]);
                        r.digits[i] = w;
                        zero &= w == 0;
                    }
                } else {
                    minus = mpint_addsub_eval(head_of(a), head_of(b), op == 1, lo, up);
                    const int s1 = a.sign, s2 = op == 1 ? (b.sign ^ 1) : b.sign;
#pragma unroll 4
                    for (int i = p; i < N; i += kMpParts)
                        r.digits[i] = mpint_addsub_digit(a.digits[i], b.digits[i], C.m[i], s1, s2, minus, f);
                }
            }
#pragma unroll
            for (int o = 1; o < kMpParts; o <<= 1) {  // the parts of a record are adjacent lanes
                f |= __shfl_xor_sync(0xffffffffu, f, o);
                zero &= __shfl_xor_sync(0xffffffffu, (int)zero, o) != 0;
            }
            if (act && p == 0) {
                r.pad = 0;
                if (op == 2) {
                    r.eval[0] = er_md<false>(a.eval[0], b.eval[0], C.unit_upp);
                    r.eval[1] = er_md<true>(a.eval[1], b.eval[1], C.unit_low);
                    r.sign = zero ? 0 : (a.sign ^ b.sign);
                } else {
                    r.sign = minus;
                    r.eval[0] = lo;
                    r.eval[1] = up;
                }
                f |= overflow_flags<N>(C, r.eval[0], r.eval[1]);
                if (flags) flags[k0 + t] = (uint8_t)f;
            }
        }
        __syncthreads();
        tile_copy(out + k0, so, bytes);
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
    if ((((uintptr_t)x | (uintptr_t)y | (uintptr_t)out) & 15) == 0) {  // tiles start 16-byte aligned
        constexpr size_t smem = 3 * kMpTile * sizeof(MpInt<N>);
        static std::atomic<int> occ[kOccDevices];  // resident blocks per SM, per device
        const int per_sm = resident_blocks(occ, c, k_mpint_tile<N>, kMpTileBlock, smem);
        k_mpint_tile<N><<<grid_for(c, (count + kMpTile - 1) / kMpTile, 1, per_sm), kMpTileBlock, smem, s>>>(
            consts_of<N>(c), op, (const MpInt<N> *)x, (const MpInt<N> *)y, count, (MpInt<N> *)out, flags);
        return cuda_status(cudaGetLastError());
    }
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
