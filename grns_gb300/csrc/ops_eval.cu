/*
 * grns_gb300 -- interval evaluation and magnitude comparison kernels.
 *   k_eval: out[k] = rns_eval_compute(X_k)   (reference src/rnseval.cuh:182)
 *   k_cmp : out[k] = rns_cmp(X_k, Y_k)       (reference src/rnscmp.cuh:55),
 *           both evaluations fused in registers, never written back.
 * One thread per number, grid-stride, residues read per modulus slice.
 * GRNS_SPLIT_BY_N: compiled as one unit per group of moduli counts.
 */
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

/* warps whose index mod 8 is below fp_eighths evaluate on the FP64 pipe
 * (eval_fp64), the others on the integer pipe (eval_int): the same bits.
 * The FP64 pipe is per scheduler and the warps of a 256-thread block go to
 * the four schedulers in turn, so 4 (warps 0-3 of every 8 on FP64) gives each
 * scheduler one warp of each kind -- the fastest setting measured (5.77 G
 * numbers/s at n = 32 against 4.83 all on the integer pipe, 3.82 all on
 * FP64).  A warp keeps one pipe: alternating per number ran at 3.8 G/s. */
__device__ __forceinline__ bool warp_on_fp64(int fp_eighths) {
    return (int)((((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) & 7) < fp_eighths;
}

/* one number's common-path evaluation on the chosen pipe, then the rare
 * branches (eval_full re-reads the residues through getm) */
template <int N, bool FAST, class Get, class GetM>
__device__ __forceinline__ void eval_split(const Consts<N> &C, bool fp, Get get, GetM getm, Er &lo, Er &up,
                                           uint32_t &f) {
    uint32_t bad = 0;
    const int st = fp ? eval_fp64<N, Get, FAST>(C, get, lo, up, bad) : eval_int<N, Get, FAST>(C, get, lo, up, bad);
    if (bad) {
        f = kFlagInvalidInput;
        lo = up = Er{0.0, 0};
    } else if (st == kEvalZero) {
        lo = up = Er{0.0, 0};
    } else if (st == kEvalRare) {
        eval_full<N, GetM, FAST>(C, getm, lo, up, f);
    }
}

template <int N, bool FAST = false>
__global__ void __launch_bounds__(256) k_eval(const __grid_constant__ CArg<N> CA, Operand<N> x, int64_t count,
                                              Er *__restrict__ out, uint8_t *__restrict__ flags, int fp_eighths) {
    const Consts<N> &C = CA.get();
    const bool fp = warp_on_fp64(fp_eighths);
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        Er lo, up;
        auto get = [&](int i) { return x.load(k, i); };
        eval_split<N, FAST>(C, fp, get, get, lo, up, f);
        out[2 * k] = lo;
        out[2 * k + 1] = up;
        if (flags) flags[k] = (uint8_t)f;
    }
}

/* the same, with the next number's residues loaded into registers while the
 * current one is evaluated (the common path is latency-bound on its loads
 * otherwise); the rare branch re-reads its residues from memory */
template <int N, bool FAST = false>
__global__ void __launch_bounds__(256, 2) k_eval_pipe(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                      int64_t count, Er *__restrict__ out,
                                                      uint8_t *__restrict__ flags, int fp_eighths) {
    const Consts<N> &C = CA.get();
    const bool fp = warp_on_fp64(fp_eighths);
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t cur[N];
    if (k < count) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) cur[i] = x.load(k, i);
    }
    for (; k < count; k += stride) {
        uint32_t nxt[N];
        const int64_t kn = k + stride;
        if (kn < count) {
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) nxt[i] = x.load(kn, i);
        }
        uint32_t f = 0;
        Er lo, up;
        auto getc = [&](int i) { return cur[i]; };
        const int64_t kk = k;
        auto getm = [&](int i) { return x.load(kk, i); };
        eval_split<N, FAST>(C, fp, getc, getm, lo, up, f);
        out[2 * k] = lo;
        out[2 * k + 1] = up;
        if (flags) flags[k] = (uint8_t)f;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) cur[i] = nxt[i];
    }
}

/* the same with the numbers claimed by warps from a counter, kEvalClaim
 * lanes' worth at a time, so the FP64-pipe and integer-pipe warps each take
 * work at their own rate until the array runs out (with a fixed grid-stride
 * share the faster kind idles at the end); the next number's residues load
 * while the current one is evaluated */
constexpr int kEvalClaim = 8;  // numbers per lane per claim

template <int N, bool FAST = false>
__global__ void __launch_bounds__(256, 2) k_eval_claim(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                       int64_t count, Er *__restrict__ out,
                                                       uint8_t *__restrict__ flags, int fp_eighths,
                                                       unsigned long long *__restrict__ ctr) {
    const Consts<N> &C = CA.get();
    const bool fp = warp_on_fp64(fp_eighths);
    const int lane = threadIdx.x & 31;
    auto claim = [&]() -> int64_t {
        unsigned long long b = 0;
        if (lane == 0) b = atomicAdd(ctr, 32ull * kEvalClaim);
        return (int64_t)__shfl_sync(0xffffffffu, b, 0);
    };
    int64_t base = claim();
    int j = 0;
    int64_t k = base + lane;
    uint32_t cur[N];
    if (k < count) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) cur[i] = x.load(k, i);
    }
    while (base < count) {  // warp-uniform
        int64_t nbase = base;
        int nj = j + 1;
        if (nj == kEvalClaim) {
            nbase = claim();
            nj = 0;
        }
        const int64_t kn = nbase + 32 * nj + lane;
        uint32_t nxt[N];
        if (kn < count) {
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) nxt[i] = x.load(kn, i);
        }
        if (k < count) {
            uint32_t f = 0;
            Er lo, up;
            auto getc = [&](int i) { return cur[i]; };
            const int64_t kk = k;
            auto getm = [&](int i) { return x.load(kk, i); };
            eval_split<N, FAST>(C, fp, getc, getm, lo, up, f);
            out[2 * k] = lo;
            out[2 * k + 1] = up;
            if (flags) flags[k] = (uint8_t)f;
        }
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) cur[i] = nxt[i];
        base = nbase;
        j = nj;
        k = kn;
    }
}

/* one-ulp enclosure where certified (rns_fast.cuh eval_tight), the
 * bit-exact evaluation otherwise (noinline: rare for uniform X) */
template <int N>
__device__ __noinline__ void eval_tight_fallback(const Consts<N> &C, const Operand<N> x, int64_t k, Er &lo, Er &up,
                                                 uint32_t &f) {
    eval<N>(C, [&](int i) { return x.load(k, i); }, lo, up, f);
}

template <int N>
__global__ void __launch_bounds__(256) k_eval_tight(const __grid_constant__ CArg<N> CA, Operand<N> x, int64_t count,
                                                    Er *__restrict__ out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0, bad = 0;
        Er lo, up;
        const bool ok = eval_tight<N>(C, [&](int i) { return x.load_cs(k, i); }, lo, up, bad);
        if (bad) {
            f = kFlagInvalidInput;
            lo = Er{0.0, 0};
            up = Er{0.0, 0};
        } else if (!ok) {
            eval_tight_fallback<N>(C, x, k, lo, up, f);
        }
        out[2 * k] = lo;
        out[2 * k + 1] = up;
        if (flags) flags[k] = (uint8_t)f;
    }
}

/* four consecutive numbers per thread with 16-byte loads of each modulus
 * slice (SoA, leading dimension a multiple of 4, 16-byte aligned base) */
template <int N>
__global__ void __launch_bounds__(256, 2) k_eval_tight_soa4(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                            int64_t count, Er *__restrict__ out,
                                                            uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    const int64_t quads = count / 4;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < quads; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = 4 * t;
        Fx128 f[4];
        uint32_t bad = 0;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            const uint4 v = __ldcs(reinterpret_cast<const uint4 *>(x.base + (int64_t)i * x.ld + k));
            const uint32_t m = C.m[i], c0 = C.c128w_0[i], c1 = C.c128w_1[i], c2 = C.c128w_2[i], c3 = C.c128w_3[i];
            bad |= (uint32_t)(v.x >= m) | (uint32_t)(v.y >= m) | (uint32_t)(v.z >= m) | (uint32_t)(v.w >= m);
            f[0].add(v.x, c0, c1, c2, c3);
            f[1].add(v.y, c0, c1, c2, c3);
            f[2].add(v.z, c0, c1, c2, c3);
            f[3].add(v.w, c0, c1, c2, c3);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            Er lo, up;
            uint32_t fl = 0;
            const bool ok = !bad && eval_tight_finish(f[j].value(), C.E, lo, up);
            if (!ok) eval_tight_fallback<N>(C, x, k + j, lo, up, fl);  // invalid residues are flagged there
            out[2 * (k + j)] = lo;
            out[2 * (k + j) + 1] = up;
            if (flags) flags[k + j] = (uint8_t)fl;
        }
    }
    const int64_t tail = 4 * quads + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tail < count) {
        uint32_t fl = 0, bad = 0;
        Er lo, up;
        const bool ok = eval_tight<N>(C, [&](int i) { return x.load(tail, i); }, lo, up, bad);
        if (bad || !ok) eval_tight_fallback<N>(C, x, tail, lo, up, fl);
        out[2 * tail] = lo;
        out[2 * tail + 1] = up;
        if (flags) flags[tail] = (uint8_t)fl;
    }
}

template <int N>
__global__ void __launch_bounds__(256) k_cmp(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> y,
                                             int64_t count, int32_t *__restrict__ out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
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

/* fast path: 64-bit fixed-point enclosures on the integer pipe, exact fallback.
 * SoA: each thread takes 4 consecutive numbers and reads every modulus slice
 * with one 128-bit load per operand; AoS: each thread reads its own number
 * with n/4 128-bit loads.  Register-capped so several blocks stay resident. */
__device__ __forceinline__ void fx64_acc(uint64_t &a, uint32_t x, uint32_t cl, uint32_t ch) {
    a += (uint64_t)x * cl;
    a += (uint64_t)(uint32_t)(x * ch) << 32;
}

template <int N>
__device__ __forceinline__ void cmp_finish(const Consts<N> &C, const Operand<N> &x, const Operand<N> &y, int64_t k,
                                           uint64_t a, uint64_t b, bool bad, int32_t *out, uint8_t *flags) {
    int r = fx64_order(a, b, C.E);
    if (r == 2 && !bad) r = fast_tie_cmp<N>(C, x, y, k);
    out[k] = bad ? 0 : r;
    if (flags) flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
}

template <int N>
__global__ void __launch_bounds__(256, 3) k_cmp_fast_soa4(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                          Operand<N> y, int64_t count, int32_t *__restrict__ out,
                                                          uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    const int64_t quads = count / 4;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < quads; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = 4 * t;
        uint64_t a[4] = {0, 0, 0, 0}, b[4] = {0, 0, 0, 0};
        uint32_t bad = 0;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            const uint4 xv = __ldcs(reinterpret_cast<const uint4 *>(x.base + (int64_t)i * x.ld + k));
            const uint4 yv = __ldcs(reinterpret_cast<const uint4 *>(y.base + (int64_t)i * y.ld + k));
            const uint32_t m = C.m[i], cl = C.c64l[i], ch = C.c64h[i];
            bad |= (uint32_t)(xv.x >= m) | (uint32_t)(xv.y >= m) | (uint32_t)(xv.z >= m) | (uint32_t)(xv.w >= m);
            bad |= ((uint32_t)(yv.x >= m) | (uint32_t)(yv.y >= m) | (uint32_t)(yv.z >= m) | (uint32_t)(yv.w >= m));
            fx64_acc(a[0], xv.x, cl, ch); fx64_acc(a[1], xv.y, cl, ch);
            fx64_acc(a[2], xv.z, cl, ch); fx64_acc(a[3], xv.w, cl, ch);
            fx64_acc(b[0], yv.x, cl, ch); fx64_acc(b[1], yv.y, cl, ch);
            fx64_acc(b[2], yv.z, cl, ch); fx64_acc(b[3], yv.w, cl, ch);
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            bool badj = false;
            if (bad) {  /* rare: find which of the four numbers is invalid */
#pragma unroll 1
                for (int i = 0; i < N; i++) badj |= x.load(k + j, i) >= C.m[i] || y.load(k + j, i) >= C.m[i];
            }
            cmp_finish<N>(C, x, y, k + j, a[j], b[j], badj, out, flags);
        }
    }
    /* tail: count % 4 numbers */
    const int64_t tail = 4 * quads + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (tail < count) {
        uint64_t a = 0, b = 0;
        bool bad = false;
#pragma unroll 1
        for (int i = 0; i < N; i++) {
            const uint32_t xi = x.load(tail, i), yi = y.load(tail, i);
            bad |= xi >= C.m[i] || yi >= C.m[i];
            fx64_acc(a, xi, C.c64l[i], C.c64h[i]);
            fx64_acc(b, yi, C.c64l[i], C.c64h[i]);
        }
        cmp_finish<N>(C, x, y, tail, a, b, bad, out, flags);
    }
}

template <int N>
__global__ void __launch_bounds__(256, 3) k_cmp_fast(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> y,
                                                     int64_t count, int32_t *__restrict__ out,
                                                     uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint64_t a = 0, b = 0;
        uint32_t bad = 0;
        if (x.ld == 0 && (N % 4) == 0) {  /* AoS: the number's residues are contiguous */
            const uint4 *px = reinterpret_cast<const uint4 *>(x.base + k * N);
            const uint4 *py = reinterpret_cast<const uint4 *>(y.base + k * N);
GRNS_UNROLL_TO(N / 4)
            for (int q = 0; q < N / 4; q++) {
                const uint4 xv = __ldcs(px + q), yv = __ldcs(py + q);
                const uint32_t xs[4] = {xv.x, xv.y, xv.z, xv.w}, ys[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = 4 * q + j;
                    bad |= (uint32_t)(xs[j] >= C.m[i]) | (uint32_t)(ys[j] >= C.m[i]);
                    fx64_acc(a, xs[j], C.c64l[i], C.c64h[i]);
                    fx64_acc(b, ys[j], C.c64l[i], C.c64h[i]);
                }
            }
        } else {
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) {
                const uint32_t xi = x.load_cs(k, i), yi = y.load_cs(k, i);
                bad |= (uint32_t)(xi >= C.m[i]) | (uint32_t)(yi >= C.m[i]);
                fx64_acc(a, xi, C.c64l[i], C.c64h[i]);
                fx64_acc(b, yi, C.c64l[i], C.c64h[i]);
            }
        }
        cmp_finish<N>(C, x, y, k, a, b, bad != 0, out, flags);
    }
}

constexpr int64_t kEvalClaimMin = 1 << 16;  // smaller arrays keep the fixed grid-stride share

template <int N, bool FAST>
grns_status run_eval(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                     uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    if constexpr (N > 32) {
        k_eval<N, FAST><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, (Er *)out,
                                                           flags, c->eval_fp64_eighths);
        return cuda_status(cudaGetLastError());
    }
    if (count >= kEvalClaimMin && c->eval_fp64_eighths > 0 && c->eval_fp64_eighths < 8) {
        /* both pipes in use: warps claim their numbers (a counter from the pool, zeroed in stream order) */
        void *ctr = nullptr;
        cudaError_t e = scratch_alloc(c, &ctr, sizeof(unsigned long long), s);
        if (e == cudaSuccess) e = cudaMemsetAsync(ctr, 0, sizeof(unsigned long long), s);
        if (e != cudaSuccess) return cuda_status(e);
        k_eval_claim<N, FAST><<<grid_for(c, count, B, 2), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count,
                                                                    (Er *)out, flags, c->eval_fp64_eighths,
                                                                    (unsigned long long *)ctr);
        e = cudaGetLastError();
        scratch_free(ctr, s);
        return cuda_status(e);
    }
    k_eval_pipe<N, FAST><<<grid_for(c, count, B, 2), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, (Er *)out,
                                                               flags, c->eval_fp64_eighths);
    return cuda_status(cudaGetLastError());
}

template <int N>
grns_status run_cmp(const grns_ctx *c, const uint32_t *x, const uint32_t *y, int64_t ld, int64_t count, int32_t *out,
                    uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    if (c->path == GRNS_PATH_REFERENCE)
        k_cmp<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{y, ld}, count, out,
                                                    flags);
    else if (ld != 0 && ld % 4 == 0 && ((uintptr_t)x % 16) == 0 && ((uintptr_t)y % 16) == 0)
        k_cmp_fast_soa4<N><<<grid_for(c, (count + 3) / 4, B, 3), B, 0, s>>>(
            consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{y, ld}, count, out, flags);
    else
        k_cmp_fast<N><<<grid_for(c, count, B, 3), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{y, ld},
                                                            count, out, flags);
    return cuda_status(cudaGetLastError());
}

template <int N>
grns_status run_eval_tight(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                           uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    if (ld != 0 && ld % 4 == 0 && ((uintptr_t)x % 16) == 0)
        k_eval_tight_soa4<N><<<grid_for(c, (count + 3) / 4, B, 2), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld},
                                                                             count, (Er *)out, flags);
    else
        k_eval_tight<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, (Er *)out,
                                                           flags);
    return cuda_status(cudaGetLastError());
}

/* the per-count entry points: extern here, instantiated for this unit's counts below */
#define GRNS_EVAL_ROOTS_(n, EXT)                                                                                    \
    EXT template grns_status run_eval<n, true>(const grns_ctx *, const uint32_t *, int64_t, int64_t, interval_t *,   \
                                               uint8_t *, cudaStream_t);                                            \
    EXT template grns_status run_eval<n, false>(const grns_ctx *, const uint32_t *, int64_t, int64_t, interval_t *,  \
                                                uint8_t *, cudaStream_t);                                           \
    EXT template grns_status run_cmp<n>(const grns_ctx *, const uint32_t *, const uint32_t *, int64_t, int64_t,      \
                                        int32_t *, uint8_t *, cudaStream_t);                                        \
    EXT template grns_status run_eval_tight<n>(const grns_ctx *, const uint32_t *, int64_t, int64_t, interval_t *,   \
                                               uint8_t *, cudaStream_t);
#define GRNS_EXTERN_(n) GRNS_EVAL_ROOTS_(n, extern)
#define GRNS_DEFINE_(n) GRNS_EVAL_ROOTS_(n, )
GRNS_FOR_EACH_N(GRNS_EXTERN_)
GRNS_PART_N(GRNS_DEFINE_)
#undef GRNS_EXTERN_
#undef GRNS_DEFINE_

#if GRNS_PART_MAIN
grns_status launch_eval_tight(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                              uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_eval_tight<n>(c, x, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_eval(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                        uint8_t *flags, cudaStream_t s, bool fast) {
#define C_(n) return fast ? run_eval<n, true>(c, x, ld, count, out, flags, s) : run_eval<n, false>(c, x, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_cmp(const grns_ctx *c, const uint32_t *x, const uint32_t *y, int64_t ld, int64_t count,
                       int32_t *out, uint8_t *flags, cudaStream_t s) {
#define C_(n) return run_cmp<n>(c, x, y, ld, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}
#endif  // GRNS_PART_MAIN

}  // namespace grns
