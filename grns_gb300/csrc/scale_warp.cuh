/*
 * grns_gb300 -- warp-level power-of-two scaling (integer fast path).
 *
 * floor(X / 2^D), the result of rns_scale2pow (reference src/rnsscal.cuh:207),
 * by exact steps of up to kScaleB = 52 bits (scale_fast, rns_fast.cuh).  A
 * warp scales a contiguous range of numbers, one number per lane; every trip
 * is one step (rank by 96-bit fixed point, X mod 2^j from the 64-bit CRT
 * weights, one Barrett reduction and one Shoup multiplication per residue),
 * so the residue loops run converged although numbers need 0 to ~38 steps.
 * Lanes whose number is done store it and take the next numbers of the range
 * together (kDivRefill), in decreasing step count (lpt_order) when the
 * exponents differ.  Residues live in this thread's shared-memory column and
 * the per-modulus constants in a per-block table, as in the division.
 */
#pragma once

#include "div_warp.cuh"

namespace grns {

/* per-modulus constants of the scaling loops: DivK-compatible words for
 * kred53 (a = m, mu, w, w_sh; c = fixed-point 2^96 / m words 0..2, 2^32 mod m;
 * s = b - 1, b + 1, 2^32 Shoup companion, b) and e = M_i mod 2^64 (lo, hi),
 * 2^-52 mod m and its Shoup companion */
struct ScK {
    DivK k;
    uint4 e;
};

template <int N>
__device__ __forceinline__ void sck_fill(const Consts<N> &C, ScK *K) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        ScK v;
        v.k.a = make_uint4(C.m[i], C.mu[i], C.w[i], C.w_sh[i]);
        v.k.c = make_uint4(C.c96_0[i], C.c96_1[i], C.c96_2[i], C.t32[i]);
        v.k.s = make_uint4(C.b[i] - 1, C.b[i] + 1, C.t32_sh[i], C.b[i]);
        v.e = make_uint4((uint32_t)C.mi64[i], (uint32_t)(C.mi64[i] >> 32), C.pow2neg[kScaleB * N + i],
                         C.pow2neg_sh[kScaleB * N + i]);
        K[i] = v;
    }
}

/* steps of floor(X / 2^D): exponents of log2 M + 1 or more give 0 at once */
template <int N>
__device__ __forceinline__ int scale_steps(const Consts<N> &C, unsigned D) {
    if (D > (unsigned)C.log2M) return 0;
    return (int)((D + kScaleB - 1) / kScaleB);
}

/* exact rank when the fixed point cannot tell (first step, X near M) */
template <int N>
__device__ __noinline__ uint32_t scale_rank_exact(const Consts<N> &C, const uint32_t *col, int stride, uint32_t kk) {
    uint32_t v[N], a[N];
    for (int i = 0; i < N; i++) v[i] = col[i * stride];
    mrc_hd<N>(C, [&](int i) { return v[i]; }, a);
    return a[N - 1] == 0 ? kk : kk - 1;
}

/* one warp's range [begin, end); col: this thread's N-word column; order:
 * per-number scratch for the longest-first order (unused when D == nullptr) */
template <int N>
__device__ __forceinline__ void scale_range(const ScK *K, const Consts<N> &C, const Operand<N> &x,
                                            const uint32_t *__restrict__ Darr, uint32_t Duni, const Output<N> &out,
                                            uint8_t *flags, int32_t *order, int64_t begin, int64_t end,
                                            uint32_t *col, int stride, uint32_t *hist) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    enum { Idle, Live, Done, Dead };
    uint32_t *__restrict__ X = col;
    if (Darr) lpt_order([&](int64_t e) { return scale_steps<N>(C, __ldg(Darr + e)); }, order, begin, end, hist);

    int ph = Idle, left = 0;
    bool small = false, zero = false;
    uint32_t f = 0;
    int64_t idx = 0, next = begin;
    for (;;) {
        const unsigned lv = __ballot_sync(FULL, ph == Live);
        const unsigned wt = __ballot_sync(FULL, ph == Done || ph == Idle);
        if (lv == 0 || __popc(wt) >= kDivRefill) {
            if (ph == Done) {
#pragma unroll 4
                for (int i = 0; i < N; i++) out.store(idx, i, zero ? 0u : X[i * stride]);
                if (flags) flags[idx] = (uint8_t)f;
                ph = Idle;
            }
            const unsigned need = __ballot_sync(FULL, ph == Idle);
            const int64_t my = next + __popc(need & lt);
            next += __popc(need);
            if (ph == Idle) {
                if (my < end) {
                    idx = Darr ? begin + order[my] : my;
                    const unsigned D = Darr ? __ldg(Darr + idx) : Duni;
                    uint32_t bad = 0;
#pragma unroll 4
                    for (int i = 0; i < N; i++) {
                        const uint32_t v = x.load(idx, i);
                        bad |= (uint32_t)(v >= K[i].k.a.x);
                        X[i * stride] = v;
                    }
                    f = bad ? kFlagInvalidInput : 0u;
                    zero = bad || D > (unsigned)C.log2M;  // invalid: 0 as the reference-faithful kernel; 2^D > X: 0
                    left = (int)D;
                    small = false;
                    ph = (zero || D == 0) ? Done : Live;
                } else {
                    ph = Dead;
                }
            }
            if (__ballot_sync(FULL, ph != Dead) == 0) break;
            if (__ballot_sync(FULL, ph == Live) == 0) continue;
        }

        /* one step on every live lane */
        const bool live = ph == Live;
        const int j = left < kScaleB ? left : kScaleB;
        uint64_t S0 = 0, S1 = 0, S2 = 0, acc = 0;
#pragma unroll 4
        for (int i = 0; i < N; i++) {
            const ScK k = K[i];
            const uint32_t c = mulmod_shoup(X[i * stride], k.k.a.z, k.k.a.w, k.k.a.x);
            const uint64_t p0 = (uint64_t)c * k.k.c.x;
            const uint64_t p1 = (uint64_t)c * k.k.c.y;
            const uint64_t p2 = (uint64_t)c * k.k.c.z;
            S0 += (uint32_t)p0;
            S1 += (p0 >> 32) + (uint32_t)p1;
            S2 += (p1 >> 32) + p2;
            acc += (uint64_t)c * (((uint64_t)k.e.y << 32) | k.e.x);
        }
        const u128 t = (u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64);
        uint32_t kk = (uint32_t)(t >> 96);
        if (live && !small && (t & kMask96) < (u128)C.E) kk = scale_rank_exact<N>(C, X, stride, kk);
        const uint64_t res = (acc - (uint64_t)kk * C.m64) & ((((uint64_t)1) << j) - 1);
        const uint32_t *inv = C.pow2neg + (int64_t)j * N, *inv_sh = C.pow2neg_sh + (int64_t)j * N;
        if (__any_sync(FULL, live)) {
#pragma unroll 4
            for (int i = 0; i < N; i++) {
                const ScK k = K[i];
                const uint32_t m = k.k.a.x;
                const uint32_t w = j == kScaleB ? k.e.z : __ldg(inv + i);
                const uint32_t ws = j == kScaleB ? k.e.w : __ldg(inv_sh + i);
                const uint32_t v = X[i * stride];
                const uint32_t y = mulmod_shoup(submod(v, kred53(res, k.k), m), w, ws, m);
                if (live) X[i * stride] = y;
            }
        }
        if (live) {
            left -= j;
            small = true;
            if (left == 0) ph = Done;
        }
    }
}

/* shared memory of a block of `threads` threads running scale_range */
template <int N>
constexpr size_t scale_smem_bytes(int threads) {
    return sizeof(ScK) * N + (size_t)(threads / 32) * kDivBins * 4 + (size_t)N * 4 * threads;
}

}  // namespace grns
