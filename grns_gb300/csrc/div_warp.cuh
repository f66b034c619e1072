/*
 * grns_gb300 -- warp-level division driver (integer fast path).
 *
 * A warp divides a contiguous range of numbers in the two passes of the
 * digit-recurrence division (rns_fast.cuh):
 *   pass A  every lane normalises one number at a time -- divisor, then
 *           dividend -- by fixed-point evaluations of values magnified by the
 *           uniform constant 2^48, and writes an 8-byte record {status, s, e};
 *   pass B  every lane runs one division's digit steps; a step is one
 *           certified 48-bit digit from scalars, then R <- 2^48 R - q D,
 *           Q <- 2^48 Q + q and the fixed-point evaluation of the new R, with
 *           the same constants for every lane.
 * In both passes a finished lane stores its result and the lanes take the
 * next numbers of the range together once kDivRefill of them wait (one
 * coalesced batch of loads instead of one divergent load per finishing lane).
 * The batched kernel runs the two passes over one warp's job chunk
 * (div_range); the plain call runs them over the whole call through
 * prepared rows, longest divisions first (div_row_build / divrow_range below).
 *
 * Memory layout: each thread owns a column of 3N words of shared memory
 * (R, D, Q rows, [row][stride], conflict-free), and the block holds one DivK
 * record of constants per modulus, read with broadcast 16-byte loads.  The
 * residue loops are therefore rolled: the whole driver is a few kilobytes of
 * code (fully unrolled register versions overflowed the instruction cache
 * and stalled on instruction fetch) and uses few registers.
 *
 * Results are those of rns_div (reference src/rnsdiv.cuh:128): q = floor(x/d),
 * r = x - q d; flags DIV_BY_ZERO (q = 0, r = x), INVALID_INPUT (q = r = 0).
 */
#pragma once

#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

#ifndef GRNS_DIV_REFILL
#define GRNS_DIV_REFILL 8
#endif
#ifndef GRNS_DIV_GROUP
#define GRNS_DIV_GROUP 4
#endif
constexpr int kDivRefill = GRNS_DIV_REFILL;
constexpr int kDivGroup = GRNS_DIV_GROUP;  // residues per load / arithmetic / store group of a digit step
constexpr int kDivPrefetch = 64;  // pass A prefetches the operands this many numbers ahead

/* per-modulus constants of the division loops (shared memory, one per modulus) */
struct DivK {
    uint4 a;  // m, mu, 2^48 mod m, Shoup companion
    uint4 c;  // w-folded ceil(2^96 w / m) words 0..2, 2^32 mod m
    uint4 s;  // b - 1, b + 1, Shoup companion of 2^32 mod m, b
};

/* block-wide: fill the DivK table (caller synchronises the block) */
template <int N>
__device__ __forceinline__ void divk_fill(const Consts<N> &C, DivK *K) {
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        DivK k;
        k.a = make_uint4(C.m[i], C.mu[i], C.b48[i], C.b48_sh[i]);
        k.c = make_uint4(C.c96w_0[i], C.c96w_1[i], C.c96w_2[i], C.t32[i]);
        k.s = make_uint4(C.b[i] - 1, C.b[i] + 1, C.t32_sh[i], C.b[i]);
        K[i] = k;
    }
}

/* bits [s, s + 32) of a 64-bit value for s <= 32 (one funnel shift) */
__device__ __forceinline__ uint32_t shr64(uint64_t v, uint32_t s) {
    return __funnelshift_rc((uint32_t)v, (uint32_t)(v >> 32), s);
}
__device__ __forceinline__ uint32_t kmulmod(uint32_t x, uint32_t y, const DivK &k) {  // Barrett x y mod m
    const uint64_t p = (uint64_t)x * y;
    const uint32_t t = shr64(p, k.s.x);                          // b - 1 <= 30
    const uint32_t q = shr64((uint64_t)t * k.a.y, k.s.y);        // b + 1 <= 32
    uint32_t r = (uint32_t)p - q * k.a.x;
    r = umin32(r, r - k.a.x);
    return umin32(r, r - k.a.x);
}
__device__ __forceinline__ uint32_t kmag(uint32_t x, const DivK &k) {  // x 2^48 mod m
    return mulmod_shoup(x, k.a.z, k.a.w, k.a.x);
}
__device__ __forceinline__ uint32_t kred32(uint32_t v, const DivK &k) {  // v mod m
    return k.s.w >= 16 ? kmulmod(v, 1u, k) : v % k.a.x;
}
__device__ __forceinline__ uint32_t kred53(uint64_t v, const DivK &k) {  // v mod m, v < 2^53
    if (k.s.w >= 27) {  // hi * (2^32 mod m) + lo < 2^54 <= 2^(2b): one Barrett step
        const uint64_t p = (uint64_t)(uint32_t)(v >> 32) * k.c.w + (uint32_t)v;
        const uint32_t t = shr64(p, k.s.x);
        const uint32_t q = shr64((uint64_t)t * k.a.y, k.s.y);
        uint32_t r = (uint32_t)p - q * k.a.x;
        r = umin32(r, r - k.a.x);
        return umin32(r, r - k.a.x);
    }
    const uint32_t hi = mulmod_shoup(kred32((uint32_t)(v >> 32), k), k.c.w, k.s.z, k.a.x);
    return addmod(hi, kred32((uint32_t)v, k), k.a.x);
}
/* fixed-point accumulation of one residue (fx96w) */
struct Fx96 {
    uint64_t S0 = 0, S1 = 0;
    uint32_t S2 = 0;
    __device__ __forceinline__ void add(uint32_t x, const DivK &k) {
        const uint64_t p0 = (uint64_t)x * k.c.x;
        const uint64_t p1 = (uint64_t)x * k.c.y;
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (uint32_t)(p1 >> 32) + x * k.c.z;
    }
    __device__ __forceinline__ u128 value() const {
        return ((u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64)) & kMask96;
    }
};

constexpr int kDivUnroll = 4;

/* c = floor(R / D) when the fixed-point comparison was too close to call:
 * R = j D exactly (dv_final_tie, from the residues in the shared-memory
 * columns), else the exact comparisons */
/* the same with R and D read through accessors */
template <int N, class GR, class GD>
__device__ __forceinline__ int div_final_tie_g(const Consts<N> &C, GR gr, GD gd, u128 UD) {
    const int j = dv_final_tie<N>(C, UD, gr, gd);
    if (j) return j;
    uint32_t a[N], b[N];
    for (int i = 0; i < N; i++) {
        a[i] = gr(i);
        b[i] = gd(i);
    }
    return dv_final_exact<N>(C, a, b);
}

template <int N>
__device__ __forceinline__ int div_final_tie(const DivK *K, const Consts<N> &C, const uint32_t *Rc, const uint32_t *Dc,
                                             int stride, u128 UD) {
    return div_final_tie_g<N>(C, [&](int i) { return Rc[i * stride]; }, [&](int i) { return Dc[i * stride]; }, UD);
}

/* pass A over the numbers claim() hands out below end: rec[k] = record of
 * number k.  Column rows: the working value in rows [0, N), the dividend in
 * rows [N, 2N). */
template <int N, class Claim, class Finish, class Op>
__device__ __forceinline__ void divnorm_range_f(const DivK *K, const Consts<N> &C, const Op &x, const Op &d,
                                                Finish finish, int64_t end, Claim claim, int64_t prefetch,
                                                uint32_t *col, int stride) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    enum { Idle, ChainD, ChainX, Done, Dead };
    uint32_t *__restrict__ W = col;
    uint32_t *__restrict__ X = col + N * stride;
    int ph = Idle, k = 0, guard = 0, s = 0;
    bool xz = false;
    int64_t idx = 0;
    uint2 out = make_uint2(0, 0);
    for (;;) {
        const unsigned lv = __ballot_sync(FULL, ph == ChainD || ph == ChainX);
        const unsigned wt = __ballot_sync(FULL, ph == Done || ph == Idle);
        if (lv == 0 || __popc(wt) >= kDivRefill) {
            if (ph == Done) {
                finish(idx, out, X);
                ph = Idle;
            }
            const unsigned need = __ballot_sync(FULL, ph == Idle);
            const int64_t my = claim(__popc(need)) + __popc(need & lt);
            if (ph == Idle) {
                if (my + prefetch < end) {  // numbers taken a little later, into L2
                    d.prefetch_l2(my + prefetch);
                    x.prefetch_l2(my + prefetch);
                }
                if (my < end) {
                    idx = my;
                    uint32_t bad = 0, dnz = 0, xnz = 0;
#pragma unroll 4
                    for (int i = 0; i < N; i++) {
                        const uint32_t dv = d.load(idx, i), xv = x.load(idx, i), m = K[i].a.x;
                        W[i * stride] = dv;
                        X[i * stride] = xv;
                        bad |= (uint32_t)(dv >= m) | (uint32_t)(xv >= m);
                        dnz |= dv;
                        xnz |= xv;
                    }
                    xz = xnz == 0;
                    k = 0;
                    guard = 0;
                    ph = ChainD;
                    if (bad) {
                        out = dv_pack(kDnBad, 0, 0, false);
                        ph = Done;
                    } else if (!dnz) {
                        out = dv_pack(kDnZero, 0, 0, false);
                        ph = Done;
                    }
                } else {
                    ph = Dead;
                }
            }
            if (__ballot_sync(FULL, ph != Dead) == 0) break;
            if (__ballot_sync(FULL, ph == ChainD || ph == ChainX) == 0) continue;
        }
        const bool live = ph == ChainD || ph == ChainX;
        Fx96 fx;
#pragma unroll 8
        for (int i = 0; i < N; i++) fx.add(W[i * stride], K[i]);
        const u128 U = fx.value();
        bool more = false, tox = false;
        if (live) {
            const int k0 = k;
            const int ns = dn_step<N>(C, U, k, guard);
            if (ns == kNormMore) {
                more = true;
            } else if (ph == ChainD) {
                if (ns == kNormOk) {
                    s = dv_shift(k0, bitlen128(U));
                    if (xz) {
                        out = dv_pack(kDnOk, s, s % kDivB - kDivB, false);
                        ph = Done;
                    } else {
                        tox = true;
                        k = 0;
                        guard = 0;
                        ph = ChainX;
                    }
                } else {
                    out = dv_pack(ns == kNormNear ? kDnNear : kDnCap, 0, 0, false);
                    ph = Done;
                }
            } else {
                if (ns == kNormOk) out = dv_pack(kDnOk, s, dv_skip(s, k0, bitlen128(U)), false);
                else if (ns == kNormNear) out = dv_pack(kDnOk, s, s % kDivB - kDivB, true);
                else out = dv_pack(kDnCap, 0, 0, false);
                ph = Done;
            }
        }
        /* magnify by 2^48 (lanes that go on), or start the dividend's chain */
        if (__any_sync(FULL, more || tox)) {
#pragma unroll 1
            for (int i0 = 0; i0 < N; i0 += 4) {  // groups of 4: loads, arithmetic, stores
                uint32_t w[4], xv[4];
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = (N % 4 == 0 || i0 + j < N) ? i0 + j : N - 1;  // past N: the last residue again
                    w[j] = W[i * stride];
                    xv[j] = X[i * stride];
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int i = (N % 4 == 0 || i0 + j < N) ? i0 + j : N - 1;
                    w[j] = tox ? xv[j] : (more ? kmag(w[j], K[i]) : w[j]);
                }
#pragma unroll
                for (int j = 0; j < 4; j++)
                    if (N % 4 == 0 || i0 + j < N) W[(i0 + j) * stride] = w[j];
            }
        }
    }
}

/* pass A writing records rec[k] (the batched kernel's per-warp form) */
template <int N, class Claim, class Op>
__device__ __forceinline__ void divnorm_range(const DivK *K, const Consts<N> &C, const Op &x, const Op &d, uint2 *rec,
                                              int64_t end, Claim claim, int64_t prefetch, uint32_t *col, int stride) {
    divnorm_range_f<N>(K, C, x, d, [&](int64_t idx, uint2 r, const uint32_t *) { rec[idx] = r; }, end, claim,
                       prefetch, col, stride);
}

/* pass B over [begin, end) with the records of pass A, numbers taken in the
 * order of div_order.  Column rows: R in [0, N), the scaled divisor D in
 * [N, 2N), the quotient Q in [2N, 3N). */
template <int N, class Claim, class Op, class OutQ, class OutR>
__device__ __forceinline__ void divloop_range(const DivK *K, const Consts<N> &C, const Op &x, const Op &d,
                                              const uint2 *rec, const int32_t *order, const OutQ &qo,
                                              const OutR &ro, uint8_t *flags, int64_t begin, int64_t end, Claim claim,
                                              uint32_t *col, int stride) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    enum { Idle, Iter, Final, Done, Dead };
    uint32_t *__restrict__ Rc = col;
    uint32_t *__restrict__ Dc = col + N * stride;
    uint32_t *__restrict__ Qc = col + 2 * N * stride;

    DivSt st;
    st.f = 0;
    st.left = 0;
    st.b = kDivB;
    u128 U = 0;
    int ph = Idle;
    int64_t idx = 0;

    for (;;) {
        const unsigned lv = __ballot_sync(FULL, ph == Iter);
        const unsigned wt = __ballot_sync(FULL, ph == Final || ph == Done || ph == Idle);
        if (lv == 0 || __popc(wt) >= kDivRefill) {
            if (ph == Final) {  // q = Q + c, r = x - q d
                int c = dv_final_fx(st, U, C.E);
                if (c < 0) c = div_final_tie<N>(K, C, Rc, Dc, stride, st.UD);
#pragma unroll 4
                for (int i = 0; i < N; i++) {
                    const DivK k = K[i];
                    const uint32_t m = k.a.x;
                    const uint32_t qi = addmod(Qc[i * stride], (uint32_t)c % m, m);
                    qo.store(idx, i, qi);
                    ro.store(idx, i, submod(x.load(idx, i), kmulmod(qi, d.load(idx, i), k), m));
                }
                if (flags) flags[idx] = (uint8_t)st.f;
                ph = Idle;
            } else if (ph == Done) {  // results already in the R and Q rows
#pragma unroll 4
                for (int i = 0; i < N; i++) {
                    qo.store(idx, i, Qc[i * stride]);
                    ro.store(idx, i, Rc[i * stride]);
                }
                if (flags) flags[idx] = (uint8_t)st.f;
                ph = Idle;
            }
            const unsigned need = __ballot_sync(FULL, ph == Idle);
            const int64_t my = claim(__popc(need)) + __popc(need & lt);
            if (ph == Idle) {
                if (my < end) {
                    idx = begin + order[my];
                    const uint2 r2 = rec[idx];
                    const uint32_t status = r2.x >> 16;
                    uint32_t bad = 0, xnz = 0;
#pragma unroll 4
                    for (int i = 0; i < N; i++) {
                        const uint32_t xv = x.load(idx, i);
                        bad |= (uint32_t)(xv >= K[i].a.x);
                        xnz |= xv;
                        Rc[i * stride] = xv;  // the remainder when the quotient is 0
                        Qc[i * stride] = 0u;
                    }
                    st.f = 0;
                    ph = Done;
                    if (bad || status == kDnBad) {
                        st.f = kFlagInvalidInput;
                        for (int i = 0; i < N; i++) Rc[i * stride] = 0;
                    } else if (status == kDnZero) {
                        st.f = kFlagDivByZero;
                    } else if (status == kDnCap) {
                        st.f = kFxIterCap;
                    } else if (!xnz) {
                        /* q = r = 0 */
                    } else if (status == kDnNear) {  // d > M (1 - E / 2^96): the quotient is 0 or 1
                        uint32_t a[N], b[N];
                        for (int i = 0; i < N; i++) {
                            a[i] = Rc[i * stride];
                            b[i] = d.load(idx, i);
                        }
                        if (dv_cmp_vec<N>(C, a, b) >= 0) {
                            for (int i = 0; i < N; i++) {
                                Qc[i * stride] = 1u;
                                Rc[i * stride] = submod(a[i], b[i], C.m[i]);
                            }
                        }
                    } else {
                        const int s = (int)(r2.x & 0xffffu), e = dv_rec_e(r2);
                        const uint32_t *ps = C.pow2 + (int64_t)s * N, *pss = C.pow2_sh + (int64_t)s * N;
                        const uint32_t *pe = e < 0 ? C.pow2neg + (int64_t)(-e) * N : C.pow2 + (int64_t)e * N;
                        const uint32_t *pes =
                            e < 0 ? C.pow2neg_sh + (int64_t)(-e) * N : C.pow2_sh + (int64_t)e * N;
                        Fx96 fd, fxx, fr;
#pragma unroll 4
                        for (int i = 0; i < N; i++) {
                            const DivK k = K[i];
                            const uint32_t Dv = mulmod_shoup(d.load(idx, i), __ldg(ps + i), __ldg(pss + i), k.a.x);
                            const uint32_t xv = Rc[i * stride];
                            const uint32_t Rv = mulmod_shoup(xv, __ldg(pe + i), __ldg(pes + i), k.a.x);
                            Dc[i * stride] = Dv;
                            Rc[i * stride] = Rv;
                            fd.add(Dv, k);
                            fxx.add(xv, k);
                            fr.add(Rv, k);
                        }
                        dv_setup(st, fd.value(), s, e);
                        U = (r2.y >> 31) ? (((u128)1) << 96) : (e < 0 ? fxx.value() : fr.value());
                        ph = Iter;
                    }
                } else {
                    ph = Dead;
                }
            }
            if (__ballot_sync(FULL, ph != Dead) == 0) break;
            if (__ballot_sync(FULL, ph == Iter) == 0) continue;
        }

        /* one step: digit, residue update, evaluation of the new remainder */
        const bool live = ph == Iter;
        const uint64_t qd = live ? dv_digit(st, U, C.E, st.f) : 0;
        Fx96 fx;
        /* groups of G residues; N not a multiple of G: the slots past N repeat
         * the last residue and neither store nor enter the evaluation */
        constexpr int G = N % kDivGroup == 0 ? kDivGroup : 4;
        constexpr bool ragged = N % G != 0;
#pragma unroll 1
        for (int i0 = 0; i0 < N; i0 += G) {  // groups: loads, arithmetic, stores
            uint32_t rv[G], dv[G], qv[G];
#pragma unroll
            for (int j = 0; j < G; j++) {
                const int i = (!ragged || i0 + j < N) ? i0 + j : N - 1;
                rv[j] = Rc[i * stride];
                dv[j] = Dc[i * stride];
                qv[j] = Qc[i * stride];
            }
#pragma unroll
            for (int j = 0; j < G; j++) {
                const DivK k = K[(!ragged || i0 + j < N) ? i0 + j : N - 1];
                const uint32_t m = k.a.x;
                const uint32_t qi = kred53(qd, k);
                const uint32_t rn = submod(kmag(rv[j], k), kmulmod(qi, dv[j], k), m);
                rv[j] = live ? rn : rv[j];
                qv[j] = addmod(kmag(qv[j], k), qi, m);
                if (!ragged || i0 + j < N) fx.add(rv[j], k);
            }
#pragma unroll
            for (int j = 0; j < G; j++) {
                if (ragged && i0 + j >= N) continue;
                Rc[(i0 + j) * stride] = rv[j];
                if (live) Qc[(i0 + j) * stride] = qv[j];
            }
        }
        if (live) {
            U = fx.value();
            st.b = kDivB;
            if (--st.left == 0) ph = Final;
        }
    }
}

/* ---------------- the plain call's division through prepared rows ----------------
 * (rns_fast.cuh: div_row_setup / div_row_final are the one-number forms)
 *
 * Pass A (divnorm_range) writes each number's 8-byte record; a kernel over
 * the numbers in index order (div_row_build, every lane busy) turns records
 * and operands into rows: the digit steps' starting state, or q and r at
 * once.  A global counting sort by step count (k_div_place, ops_div.cu) orders all
 * numbers longest first; pass B (divrow_range) takes positions of that order
 * from a grid-wide counter, reads each row with 16-byte loads, runs the
 * steps and writes q and r back into the row; a last kernel moves them to
 * the caller's layout.  The schedule is longest-processing-time first over
 * the whole call (the grid ends on its shortest divisions), while every
 * access to a number's data stays one contiguous row. */

constexpr int kDivRowBins = 256;  // step counts 0..255 (a division takes at most (log2M + 49) / 48 + 1)

/* the row of one division from its pass-A record (the device form of
 * div_row_setup; getters xg(i), dg(i) read the operands; row: the number's
 * row in global memory, written with 16-byte stores).  Returns the digit
 * steps (0: q and r written, flags set in f). */
template <int N, class GX, class GD>
__device__ __forceinline__ int div_row_build(const DivK *K, const Consts<N> &C, uint2 rec, GX xg, GD dg,
                                             uint32_t *row, uint32_t &f) {
    constexpr int P = kRowPad<N>();
    const uint32_t status = rec.x >> 16;
    uint32_t xnz = 0;
#pragma unroll 8
    for (int i = 0; i < N; i++) xnz |= xg(i);
    if (status != kDnOk || !xnz) {  // no digit step: q = 0, r = x unless stated below
        bool one = false;
        if (status == kDnBad) f |= kFlagInvalidInput;  // q = r = 0
        else if (status == kDnZero) f |= kFlagDivByZero;
        else if (status == kDnCap) f |= kFxIterCap;
        else if (status == kDnNear && xnz) {  // d > M (1 - E / 2^96): the quotient is 0 or 1
            uint32_t a[N], b[N];
            for (int i = 0; i < N; i++) {
                a[i] = xg(i);
                b[i] = dg(i);
            }
            one = dv_cmp_vec<N>(C, a, b) >= 0;
        }
#pragma unroll 1
        for (int i0 = 0; i0 < P; i0 += 4) {
            uint32_t qv[4], rv[4];
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = i0 + j;
                qv[j] = rv[j] = 0;
                if (N % 4 == 0 || i < N) {
                    const uint32_t xv = status == kDnBad ? 0u : xg(i);
                    qv[j] = one ? 1u : 0u;
                    rv[j] = one ? submod(xv, dg(i), K[i].a.x) : xv;
                }
            }
            *reinterpret_cast<uint4 *>(row + i0) = make_uint4(qv[0], qv[1], qv[2], qv[3]);
            *reinterpret_cast<uint4 *>(row + P + i0) = make_uint4(rv[0], rv[1], rv[2], rv[3]);
        }
        return 0;
    }
    const int s = (int)(rec.x & 0xffffu), e = dv_rec_e(rec);
    Fx96 fd, fu;  // the divisor's value; the first step's (x itself when e < 0, else R = x 2^e)
#pragma unroll 1
    for (int i0 = 0; i0 < P; i0 += 4) {
        uint32_t dv[4], rv[4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int i = i0 + j;
            dv[j] = rv[j] = 0;
            if (N % 4 == 0 || i < N) {
                const DivK k = K[i];
                const uint32_t xv = xg(i);
                dv[j] = mul_pow2<N>(C, i, dg(i), s);
                if (e < 0) {  // -e <= 48: one factor, 2^e = 2^-(-e)
                    const uint2 p = __ldg(C.p2nlo + i * 64 - e);
                    rv[j] = mulmod_shoup(xv, p.x, p.y, k.a.x);
                } else {
                    rv[j] = mul_pow2<N>(C, i, xv, e);
                }
                fd.add(dv[j], k);
                fu.add(e < 0 ? xv : rv[j], k);
            }
        }
        *reinterpret_cast<uint4 *>(row + i0) = make_uint4(dv[0], dv[1], dv[2], dv[3]);
        *reinterpret_cast<uint4 *>(row + P + i0) = make_uint4(rv[0], rv[1], rv[2], rv[3]);
    }
    DivSt st;
    dv_setup(st, fd.value(), s, e);
    const u128 U = (rec.y >> 31) ? (((u128)1) << 96) : fu.value();
    uint32_t h[kRowHdr];
    div_hdr_put(h, st, U, s);
    uint4 *hp = reinterpret_cast<uint4 *>(row + 2 * P);
#pragma unroll
    for (int j = 0; j < kRowHdr / 4; j++) hp[j] = make_uint4(h[4 * j], h[4 * j + 1], h[4 * j + 2], h[4 * j + 3]);
    return st.left;
}

/* pass B over positions [0, end) of `order` (numbers with digit steps,
 * longest first) claimed with claim(); rows: kRowWords(N) words per number.
 * Column rows: R in [0, N), Q in [N, 2N); D stays in the row (16-byte loads
 * through the read-only path each step), which keeps the block's shared
 * memory at 2n words a thread. */
template <int N, class Claim>
__device__ __forceinline__ void divrow_range(const DivK *K, const Consts<N> &C, uint32_t *rows,
                                             const int32_t *order, uint8_t *flags, int64_t end, Claim claim,
                                             uint32_t *col, int stride) {
    constexpr int P = kRowPad<N>();
    constexpr int RW = kRowWords<N>();
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    enum { Idle, Iter, Final, Dead };
    uint32_t *__restrict__ Rc = col;
    uint32_t *__restrict__ Qc = col + N * stride;
    DivSt st;
    st.f = 0;
    st.left = 0;
    st.b = kDivB;
    u128 U = 0;
    int s = 0, ph = Idle;
    uint32_t *row = rows;  // this lane's row: D stays there (read through the read-only path) until q replaces it
    int64_t idx = 0;
    for (;;) {
        const unsigned lv = __ballot_sync(FULL, ph == Iter);
        const unsigned wt = __ballot_sync(FULL, ph == Final || ph == Idle);
        if (lv == 0 || __popc(wt) >= kDivRefill) {
            if (ph == Final) {  // q = Q + c, r = (R - c D) 2^-s, into the row
                int c = dv_final_fx(st, U, C.E);
                if (c < 0)
                    c = div_final_tie_g<N>(C, [&](int i) { return Rc[i * stride]; }, [&](int i) { return row[i]; },
                                           st.UD);
#pragma unroll 1
                for (int i0 = 0; i0 < P; i0 += 4) {
                    uint32_t qv[4], rv[4];
                    const uint4 d4 = *reinterpret_cast<const uint4 *>(row + i0);  // before q overwrites it
                    const uint32_t dw[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        const int i = i0 + j;
                        qv[j] = rv[j] = 0;
                        if (N % 4 == 0 || i < N) {
                            const DivK k = K[i];
                            const uint32_t m = k.a.x, cm = (uint32_t)c % m;
                            const uint32_t v = submod(Rc[i * stride], kmulmod(cm, dw[j], k), m);
                            qv[j] = addmod(Qc[i * stride], cm, m);
                            rv[j] = mul_pow2neg<N>(C, i, v, s);
                        }
                    }
                    *reinterpret_cast<uint4 *>(row + i0) = make_uint4(qv[0], qv[1], qv[2], qv[3]);
                    *reinterpret_cast<uint4 *>(row + P + i0) = make_uint4(rv[0], rv[1], rv[2], rv[3]);
                }
                if (flags) flags[idx] = (uint8_t)st.f;
                ph = Idle;
            }
            const unsigned need = __ballot_sync(FULL, ph == Idle);
            const int64_t my = claim(__popc(need)) + __popc(need & lt);
            if (ph == Idle) {
                if (my < end) {
                    idx = order[my];
                    row = rows + idx * RW;
                    const uint4 *hp = reinterpret_cast<const uint4 *>(row + 2 * P);
                    uint32_t h[kRowHdr];
#pragma unroll
                    for (int j = 0; j < kRowHdr / 4; j++) {
                        const uint4 v = hp[j];
                        h[4 * j] = v.x;
                        h[4 * j + 1] = v.y;
                        h[4 * j + 2] = v.z;
                        h[4 * j + 3] = v.w;
                    }
                    div_hdr_get(h, st, U, s);
#pragma unroll 2
                    for (int i0 = 0; i0 < P; i0 += 4) {
                        const uint4 rv = *reinterpret_cast<const uint4 *>(row + P + i0);
                        const uint32_t r4[4] = {rv.x, rv.y, rv.z, rv.w};
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const int i = i0 + j;
                            if (N % 4 == 0 || i < N) {
                                Rc[i * stride] = r4[j];
                                Qc[i * stride] = 0u;
                            }
                        }
                    }
                    ph = Iter;
                } else {
                    ph = Dead;
                }
            }
            if (__ballot_sync(FULL, ph != Dead) == 0) break;
            if (__ballot_sync(FULL, ph == Iter) == 0) continue;
        }

        /* one step: digit, residue update, evaluation of the new remainder */
        const bool live = ph == Iter;
        const uint64_t qd = live ? dv_digit(st, U, C.E, st.f) : 0;
        Fx96 fx;
#pragma unroll 1
        for (int i0 = 0; i0 < N; i0 += 4) {  // groups of 4: loads, arithmetic, stores
            uint32_t rv[4], qv[4];
            const uint4 d4 = __ldg(reinterpret_cast<const uint4 *>(row + i0));  // D (zeros past N)
            const uint32_t dv[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = i0 + j < N ? i0 + j : N - 1;  // N not a multiple of 4: the last residue again
                rv[j] = Rc[i * stride];
                qv[j] = Qc[i * stride];
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const int i = i0 + j < N ? i0 + j : N - 1;
                const DivK k = K[i];
                const uint32_t m = k.a.x;
                const uint32_t qi = kred53(qd, k);
                const uint32_t rn = submod(kmag(rv[j], k), kmulmod(qi, dv[j], k), m);
                rv[j] = live ? rn : rv[j];
                qv[j] = addmod(kmag(qv[j], k), qi, m);
                if (N % 4 == 0 || i0 + j < N) fx.add(rv[j], k);
            }
#pragma unroll
            for (int j = 0; j < 4; j++) {
                if (N % 4 == 0 || i0 + j < N) {
                    const int i = i0 + j;
                    Rc[i * stride] = rv[j];
                    if (live) Qc[i * stride] = qv[j];
                }
            }
        }
        if (live) {
            U = fx.value();
            st.b = kDivB;
            if (--st.left == 0) ph = Final;
        }
    }
}

/* shared memory of pass A: the DivK table, then two column rows per residue */
template <int N>
constexpr size_t divprep_smem_bytes(int threads) {
    return sizeof(DivK) * N + (size_t)2 * N * 4 * threads;
}
/* shared memory of pass B with rows: the DivK table, then the R and Q
 * columns (D is read from the row) */
template <int N>
constexpr size_t divrow_smem_bytes(int threads) {
    return sizeof(DivK) * N + (size_t)2 * N * 4 * threads;
}

/* digit steps of a division from its record (0: no step loop) */
__device__ __forceinline__ int dv_rec_steps(const uint2 &r) {
    if ((r.x >> 16) != kDnOk) return 0;
    const int s = (int)(r.x & 0xffffu), e = dv_rec_e(r);
    const int t = s % kDivB, a = s / kDivB;
    return a + 1 - (e < 0 ? 0 : (e - t) / kDivB + 1);
}

constexpr int kDivBins = 64;  // step-count bins of a warp's ordering (> log2(M) / 48 + 1 up to 64 moduli)

/* order[begin + p] (p = 0..) = offsets of the range's numbers by decreasing
 * step count steps_of(k) (a counting sort over kDivBins bins, counts of 63 or
 * more sharing the last -- 128 and 256 moduli reach ~170 steps; hist: this
 * warp's kDivBins shared counters), so a warp's last numbers are its
 * cheapest and the drain at the end of the range is short */
template <class StepsOf>
__device__ __forceinline__ void lpt_order(StepsOf steps_of, int32_t *order, int64_t begin, int64_t end,
                                          uint32_t *hist) {
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    hist[lane] = 0;
    hist[lane + 32] = 0;
    __syncwarp();
    auto bin = [&](int64_t e) { return min(kDivBins - 1, (int)steps_of(e)); };
    for (int64_t e = begin + lane; e < end; e += 32) atomicAdd(&hist[bin(e)], 1u);
    __syncwarp();
    /* exclusive prefix over bins in decreasing order: lane l holds bins 63 - l and 31 - l */
    const uint32_t h0 = hist[63 - lane], h1 = hist[31 - lane];
    uint32_t s0 = h0, s1 = h1;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t a0 = __shfl_up_sync(FULL, s0, o), a1 = __shfl_up_sync(FULL, s1, o);
        if (lane >= o) {
            s0 += a0;
            s1 += a1;
        }
    }
    s1 += __shfl_sync(FULL, s0, 31);
    __syncwarp();
    hist[63 - lane] = s0 - h0;
    hist[31 - lane] = s1 - h1;
    __syncwarp();
    for (int64_t e = begin + lane; e < end; e += 32) {
        const uint32_t p = atomicAdd(&hist[bin(e)], 1u);
        order[begin + p] = (int32_t)(e - begin);
    }
    __syncwarp();  // the order written by one lane is read by another
}

__device__ __forceinline__ void div_order(const uint2 *rec, int32_t *order, int64_t begin, int64_t end,
                                          uint32_t *hist) {
    lpt_order([&](int64_t e) { return dv_rec_steps(rec[e]); }, order, begin, end, hist);
}

/* both passes for one warp's range; rec / order hold one entry per number of
 * the range's index space (index k in [begin, end)); col: this thread's
 * 3N-word shared-memory column (row stride `stride` words); hist: this
 * warp's kDivBins shared counters */
template <int N, class Op, class OutQ, class OutR>
__device__ __forceinline__ void div_range(const DivK *K, const Consts<N> &C, const Op &x, const Op &d, uint2 *rec,
                                          int32_t *order, const OutQ &qo, const OutR &ro, uint8_t *flags,
                                          int64_t begin, int64_t end, uint32_t *col, int stride, uint32_t *hist) {
    int64_t next = begin;
    divnorm_range<N>(K, C, x, d, rec, end, [&](int c) { const int64_t b = next; next += c; return b; }, kDivPrefetch,
                     col, stride);
    __syncwarp();  // records written by one lane are read by another
    div_order(rec, order, begin, end, hist);
    int64_t pos = 0;  // order holds offsets from begin at positions begin..end-1
    divloop_range<N>(K, C, x, d, rec, order + begin, qo, ro, flags, begin, end - begin,
                     [&](int c) { const int64_t b = pos; pos += c; return b; }, col, stride);
}

/* a warp's claim of c consecutive positions from a grid-wide counter (all
 * lanes call it with the same c; lane 0 does the atomic) */
__device__ __forceinline__ int64_t warp_claim(unsigned long long *ctr, int c) {
    unsigned long long b = 0;
    if ((threadIdx.x & 31) == 0 && c > 0) b = atomicAdd(ctr, (unsigned long long)c);
    return (int64_t)__shfl_sync(0xffffffffu, b, 0);
}


/* scratch bytes per number of the global pass-A records and the order */
constexpr size_t kDivScratchPerNumber = sizeof(uint2) + sizeof(int32_t);

}  // namespace grns
