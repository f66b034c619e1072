/*
 * grns_gb300 -- integer-pipe algorithms for the non-modular operations.
 *
 * Comparison, division, power-of-two scaling and the maximum have exact
 * integer results, so the enclosure of X/M they use internally is free to
 * differ from the reference's FP64 one (src/rnseval.cuh:182) as long as it
 * is certified.  GB300's FP64 pipe is ~1/40 of its integer pipe, so these
 * paths evaluate X/M as a fixed-point sum on the integer pipe:
 *
 *     X/M = frac( sum_i s_i / m_i ),   s_i = x_i * w_i mod m_i
 *     T   = sum_i s_i * ceil(2^P / m_i)        (P = 64 or 96)
 *     2^P * frac(X/M) lies in [U - E, U] where U = T mod 2^P,
 *     E = sum_i (m_i - 1), whenever U >= E (no wrap); otherwise X is within
 *     E/2^P of 0 or of M and the exact mixed-radix digits decide.
 *
 * P = 64 costs two IMADs per residue (an IMAD.WIDE accumulating mod 2^64);
 * P = 96 keeps three 64-bit column sums.  Small values are magnified by
 * powers of two (X * 2^k mod M = X * 2^k when no wrap can occur), the
 * integer-pipe counterpart of the reference's refinement loop (:234-244).
 *
 * Everything here is host+device so the CPU tests can run the same code.
 */
#pragma once

#include <cmath>

#include "rns_common.cuh"
#include "rns_convert.cuh"

namespace grns {

typedef unsigned __int128 u128;

GRNS_HD uint32_t ldg_u32(const uint32_t *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}
GRNS_HD uint2 ldg_u2(const uint2 *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}

/* v 2^s mod m_i and v 2^-s mod m_i for 0 <= s < 64 p2rows: two Shoup products
 * with (value, companion) pairs of the residue-major tables, so the lanes of a
 * warp looking up different shifts for one residue read a few cache lines */
template <int N>
GRNS_HD uint32_t mul_pow2(const Consts<N> &C, int i, uint32_t v, int s) {
    const uint32_t m = C.m[i];
    const uint2 a = ldg_u2(C.p2lo + i * 64 + (s & 63)), b = ldg_u2(C.p2hi + (int64_t)i * C.p2rows + (s >> 6));
    return mulmod_shoup(mulmod_shoup(v, a.x, a.y, m), b.x, b.y, m);
}
template <int N>
GRNS_HD uint32_t mul_pow2neg(const Consts<N> &C, int i, uint32_t v, int s) {
    const uint32_t m = C.m[i];
    const uint2 a = ldg_u2(C.p2nlo + i * 64 + (s & 63)), b = ldg_u2(C.p2nhi + (int64_t)i * C.p2rows + (s >> 6));
    return mulmod_shoup(mulmod_shoup(v, a.x, a.y, m), b.x, b.y, m);
}

GRNS_HD int clz32(uint32_t x) {
#ifdef __CUDA_ARCH__
    return __clz(x);
#else
    return x ? __builtin_clz(x) : 32;
#endif
}
GRNS_HD int clz64(uint64_t x) {
#ifdef __CUDA_ARCH__
    return __clzll(x);
#else
    return x ? __builtin_clzll(x) : 64;
#endif
}
GRNS_HD int bitlen32(uint32_t x) { return 32 - clz32(x); }
GRNS_HD int bitlen64(uint64_t x) { return 64 - clz64(x); }
GRNS_HD int bitlen128(u128 v) {
    uint64_t hi = (uint64_t)(v >> 64);
    return hi ? 128 - clz64(hi) : 64 - clz64((uint64_t)v);
}

constexpr u128 kMask96 = (((u128)1) << 96) - 1;

/* v mod m for v < 2^32 */
template <int N>
GRNS_HD uint32_t reduce32(const Consts<N> &C, int i, uint32_t v) {
    return C.b[i] >= 16 ? mulmod_barrett(v, 1u, C.m[i], C.mu[i], C.b[i]) : v % C.m[i];
}
/* v mod m for v < 2^64 */
template <int N>
GRNS_HD uint32_t reduce64(const Consts<N> &C, int i, uint64_t v) {
    uint32_t hi = mulmod_shoup(reduce32<N>(C, i, (uint32_t)(v >> 32)), C.t32[i], C.t32_sh[i], C.m[i]);
    return addmod(hi, reduce32<N>(C, i, (uint32_t)v), C.m[i]);
}

/* ---------------- fixed-point sums ---------------- */

/* sum_i x_i * ceil(2^64 w_i / m_i) mod 2^64: within E above 2^64 * frac(X/M)
 * (frac(x w / m) = s / m, so folding w_i into the constant needs no modular
 * multiplication; the truncation error is below sum x_i <= E) */
template <int N, class Get>
GRNS_HD uint64_t fx64(const Consts<N> &C, Get get) {
    uint64_t a = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t x = get(i);
        a += (uint64_t)x * C.c64l[i];
        a += (uint64_t)(uint32_t)(x * C.c64h[i]) << 32;
    }
    return a;
}

/* sum_i s_i * ceil(2^96/m_i) exactly (no wrap; integer part in bits 96..);
 * s_i = gets(i) given directly -- used where the integer part is needed */
template <int N, class GetS>
GRNS_HD u128 fx96_s(const Consts<N> &C, GetS gets) {
    uint64_t S0 = 0, S1 = 0, S2 = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        uint32_t s = gets(i);
        uint64_t p0 = (uint64_t)s * C.c96_0[i];
        uint64_t p1 = (uint64_t)s * C.c96_1[i];
        uint64_t p2 = (uint64_t)s * C.c96_2[i];
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (p1 >> 32) + p2;
    }
    return (u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64);
}

/* sum_i x_i * c96k[k][i] mod 2^96: within E above 2^96 * frac(X 2^k / M) */
template <int N, class Get>
GRNS_HD u128 fx96_k(const Consts<N> &C, Get get, int k) {
    const uint4 *row = C.c96k + (int64_t)k * N;
    uint64_t S0 = 0, S1 = 0;
    uint32_t S2 = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t x = get(i);
#ifdef __CUDA_ARCH__
        const uint4 c = __ldg(row + i);
#else
        const uint4 c = row[i];
#endif
        uint64_t p0 = (uint64_t)x * c.x;
        uint64_t p1 = (uint64_t)x * c.y;
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (uint32_t)(p1 >> 32) + x * c.z;
    }
    return ((u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64)) & kMask96;
}

/* sum_i x_i * ceil(2^96 w_i / m_i) mod 2^96 with the constants of the
 * parameter block (fx96_k at k = 0 without the table) */
template <int N, class Get>
GRNS_HD u128 fx96w(const Consts<N> &C, Get get) {
    uint64_t S0 = 0, S1 = 0;
    uint32_t S2 = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t x = get(i);
        const uint64_t p0 = (uint64_t)x * C.c96w_0[i];
        const uint64_t p1 = (uint64_t)x * C.c96w_1[i];
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (uint32_t)(p1 >> 32) + x * C.c96w_2[i];
    }
    return ((u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64)) & kMask96;
}

template <int N, class Get>
GRNS_HD u128 fx96(const Consts<N> &C, Get get) {
    return fx96w<N>(C, get);
}

/* ---------------- interval evaluation on the integer pipe (bit-exact) ----------------
 *
 * The common path of rns_eval_compute (src/rnseval.cuh:182-215) multiplies
 * s_i = x_i w_i mod m_i by RNS_MODULI_RECIP_RD / _RU with rounding down / up
 * and adds the products pairwise with rounding down / up.  Every value on it
 * is 0 or a double in [2^-31, n) with 53 significant bits, i.e. an integer
 * multiple of 2^17 at scale 2^100 below 2^108 (n <= 256).  So each operation is computed
 * exactly as a 128-bit integer and rounded to 53 significant bits by masking
 * (a nonzero value is >= 2^69 at this scale, so its bit length is 64 +
 * bitlen(hi) and the rounding position 11 + bitlen(hi) lies in the low word):
 * the same doubles as the FP64 directed-rounding instructions, at integer-pipe
 * speed (GB300's FP64 rate is a small fraction of its integer rate).
 */
struct Fx100 {
    uint64_t lo, hi;
};

GRNS_HD Fx100 fx100_round(Fx100 v, bool up) {
    const int t = 11 + bitlen64(v.hi);
    const uint64_t mask = (((uint64_t)1) << t) - 1;
    if (up) {
        if (v.lo & mask) {
            v.lo = (v.lo | mask) + 1;
            v.hi += v.lo == 0 ? 1 : 0;
        }
    } else {
        v.lo &= ~mask;
    }
    return v;
}
GRNS_HD Fx100 fx100_add(Fx100 a, Fx100 b) {
    Fx100 r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
    return r;
}
/* s * c for c = clo + chi 2^64 with the product below 2^106 */
GRNS_HD Fx100 fx100_mul(uint32_t s, uint64_t clo, uint64_t chi) {
    const uint64_t p0 = (uint64_t)s * (uint32_t)clo;
    const uint64_t p1 = (uint64_t)s * (uint32_t)(clo >> 32);
    Fx100 r;
    r.lo = p0 + (p1 << 32);
    r.hi = (p1 >> 32) + (uint64_t)s * chi + (r.lo < p0 ? 1 : 0);
    return r;
}
GRNS_HD bool fx100_less(const Fx100 &a, uint64_t blo, uint64_t bhi) {
    return a.hi < bhi || (a.hi == bhi && a.lo < blo);
}
/* er_set_d of the double a (a = value * 2^100) */
GRNS_HD Er er_from_fx100(const Fx100 &a) {
    if (!a.hi && !a.lo) return Er{0.0, 0};
    const int L = a.hi ? 64 + bitlen64(a.hi) : bitlen64(a.lo);
    const u128 v = ((u128)a.hi << 64) | a.lo;
    const uint64_t mant = (uint64_t)(L > 53 ? (v >> (L - 53)) : (v << (53 - L)));  // exact: 53 bits
    const uint64_t bits = (mant & ((((uint64_t)1) << 52) - 1)) | (((uint64_t)1023) << 52);
    return Er{bitsd(bits), (int64_t)(L - 101)};
}

/* the reference's pairwise tree (psum_rd / psum_ru, src/pairwise.cuh) as a
 * streaming binary counter, on exact integers */
template <int N, bool UP>
struct Fx100Tree {
    static constexpr int L = ilog2c(N) + 1;
    Fx100 lv[L];
    GRNS_HD void push(int i, Fx100 v) {
#pragma unroll
        for (int k = 0; k < L; k++) {
            if (!((i >> k) & 1)) {
                lv[k] = v;
                return;
            }
            v = fx100_round(fx100_add(lv[k], v), UP);
        }
    }
    GRNS_HD Fx100 total() const {
        Fx100 acc{0, 0};
        bool have = false;
#pragma unroll
        for (int k = 0; k < L; k++) {
            if ((N >> k) & 1) {
                acc = have ? fx100_round(fx100_add(lv[k], acc), UP) : lv[k];
                have = true;
            }
        }
        return acc;
    }
};

enum : int { kEvalOk = 0, kEvalRare = 1, kEvalZero = 2 };

/* Common path of rns_eval_compute: kEvalOk with low / upp set, kEvalZero for
 * X = 0, kEvalRare when the integer parts of the two sums differ or the upper
 * fraction is below RNS_EVAL_ACCURACY (the reference's mixed-radix and
 * refinement branches decide then).  bad collects residues >= m_i. */
template <int N, class Get, bool FAST = false>
GRNS_HD int eval_int(const Consts<N> &C, Get get, Er &low, Er &upp, uint32_t &bad) {
    Fx100Tree<N, false> tl;
    Fx100Tree<N, true> tu;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t xi = get(i);
        bad |= (uint32_t)(xi >= C.m[i]);
        const uint32_t s = mulmod_shoup(xi, C.w[i], C.w_sh[i], C.m[i]);
        tl.push(i, fx100_round(fx100_mul(s, C.evl_lo[i], C.evl_hi[i]), false));
        tu.push(i, fx100_round(fx100_mul(s, C.evu_lo[i], C.evu_hi[i]), true));
    }
    Fx100 sl = tl.total(), su = tu.total();
    if (!sl.hi && !sl.lo && !su.hi && !su.lo) return kEvalZero;
    const uint64_t whl = sl.hi >> 36, whu = su.hi >> 36;  // integer parts (scale 2^100 = 2^(64+36))
    sl.hi &= (((uint64_t)1) << 36) - 1;
    su.hi &= (((uint64_t)1) << 36) - 1;
    /* rns_eval_compute_fast (src/rnseval.cuh:266) keeps the fractions when the
     * integer parts differ; rns_eval_compute resolves that case by mixed radix */
    if ((!FAST && whl != whu) || fx100_less(su, C.acc_lo, C.acc_hi)) return kEvalRare;
    low = er_from_fx100(sl);
    upp = er_from_fx100(su);
    return kEvalOk;
}

/* ---------------- directed-rounding product and quotient on the integer pipe ----------------
 * out = (a * b) / c with both operations rounded down (up = false) or up,
 * as __ddiv_rd(__dmul_rd(a, b), c) / __ddiv_ru(__dmul_ru(a, b), c): the
 * 53-bit mantissas multiplied exactly (106 bits) and rounded, then an exact
 * 128 / 64-bit division rounded.  Returns false -- the caller then uses the
 * FP64 instructions -- unless a and b are normal or zero, c is normal, and
 * both results are normal or zero. */
/* floor(2^116 / mc) for the 53-bit mantissa mc of a normal c: the quotient
 * below then needs one multiplication and at most two corrections */
GRNS_HD uint64_t dmuldiv_recip(double c) {
    const uint64_t mc = (dbits(c) & ((((uint64_t)1) << 52) - 1)) | (((uint64_t)1) << 52);
    return (uint64_t)((((u128)1) << 116) / mc);
}

GRNS_HD bool dmuldiv_dir_i(double a, double b, double c, bool up, double &out, uint64_t rcp = 0) {
    const uint64_t ua = dbits(a), ub = dbits(b), uc = dbits(c);
    const int ea = (int)((ua >> 52) & 0x7ff), eb = (int)((ub >> 52) & 0x7ff), ec = (int)((uc >> 52) & 0x7ff);
    const uint64_t fm = (((uint64_t)1) << 52) - 1;
    const bool za = !(ua << 1), zb = !(ub << 1);
    if ((ea == 0 && !za) || (eb == 0 && !zb) || ea == 0x7ff || eb == 0x7ff || ec == 0 || ec == 0x7ff) return false;
    const uint64_t sp = (ua ^ ub) >> 63, sq = sp ^ (uc >> 63);  // signs of the product and the quotient
    if (za || zb) {  // (+-0) / c
        out = bitsd(sq << 63);
        return true;
    }
    /* the product, rounded to 53 bits toward -inf (down) or +inf (up) */
    const u128 P = (u128)((ua & fm) | (fm + 1)) * (u128)((ub & fm) | (fm + 1));
    int sh = bitlen128(P) - 53;  // 52 or 53
    uint64_t pm = (uint64_t)(P >> sh);
    if ((P & ((((u128)1) << sh) - 1)) != 0 && (up != (sp != 0))) {  // inexact, magnitude rounded away from 0
        if (++pm == (((uint64_t)1) << 53)) {
            pm >>= 1;
            sh++;
        }
    }
    const int ep = ea + eb - 1023 + (sh - 52);  // biased exponent of the rounded product
    if (ep < 1 || ep > 2046) return false;
    /* the quotient pm 2^64 / mc, rounded the same way */
    const uint64_t mc = (uc & fm) | (fm + 1);
    const u128 N = ((u128)pm) << 64;
    u128 Q;
    if (rcp) {  // rcp = floor(2^116 / mc): Q <= floor(N / mc), short by at most 2
        Q = ((u128)pm * rcp) >> 52;
        u128 R = N - Q * mc;
        while (R >= mc) {
            R -= mc;
            Q++;
        }
    } else {
        Q = N / mc;
    }
    const bool rem = (N - Q * mc) != 0;
    const int qs = bitlen128(Q) - 53;  // 11 or 12
    uint64_t qm = (uint64_t)(Q >> qs);
    if ((rem || (Q & ((((u128)1) << qs) - 1)) != 0) && (up != (sq != 0))) {
        if (++qm == (((uint64_t)1) << 53)) {
            qm >>= 1;
            return false;  // a carry into the next binade: left to the FP64 form
        }
    }
    const int eq = ep - ec + qs + 1011;  // biased exponent of the quotient: qm 2^(qs - 64) 2^(ep - ec)
    if (eq < 1 || eq > 2046) return false;
    out = bitsd((sq << 63) | ((uint64_t)eq << 52) | (qm & fm));
    return true;
}

/* ---------------- one-ulp interval evaluation ----------------
 *
 * T = sum_i x_i ceil(2^128 w_i / m_i) mod 2^128 exceeds 2^128 frac(X/M) by
 * less than sum_i x_i <= E = sum_i (m_i - 1) (frac(x w / m) = s / m), so when
 * T > E, X/M lies in ((T - E) / 2^128, T / 2^128] -- width < 2^-90.
 * Rounded outward to 53-bit er_float bounds it is at most one unit in the last
 * place wide whenever both ends round down to the same double.  X/M (M odd,
 * X != 0) is never a dyadic rational, so no double enclosure of it -- the
 * reference's included -- is narrower than one ulp: this interval is never
 * wider than rns_eval_compute's (src/rnseval.cuh:182).  Otherwise (T < E: X
 * near 0 or M; the ends in different ulps) the caller falls back to the
 * bit-exact evaluation.
 */
/* one residue's term of the 128-bit sum (S3 keeps bits 96..127) */
struct Fx128 {
    uint64_t S0 = 0, S1 = 0, S2 = 0;
    uint32_t S3 = 0;
    GRNS_HD void add(uint32_t x, uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3) {
        const uint64_t p0 = (uint64_t)x * c0;
        const uint64_t p1 = (uint64_t)x * c1;
        const uint64_t p2 = (uint64_t)x * c2;
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (p1 >> 32) + (uint32_t)p2;
        S3 += (uint32_t)(p2 >> 32) + x * c3;
    }
    GRNS_HD u128 value() const {
        return (u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64) + ((u128)S3 << 96);
    }
};

/* er_float of v / 2^128 rounded to 53 bits (down, or up), for v > 0; also
 * the rounded-down mantissa and bit length (to compare two values' ulps) */
GRNS_HD Er er_fx128(u128 v, bool up, uint64_t &mant, int &L) {
    L = bitlen128(v);
    uint64_t m;
    if (L > 53) {
        m = (uint64_t)(v >> (L - 53));
        const bool inexact = (v & ((((u128)1) << (L - 53)) - 1)) != 0;
        mant = m;
        if (up && inexact && ++m == (((uint64_t)1) << 53)) {
            m >>= 1;
            return Er{bitsd(((m & ((((uint64_t)1) << 52) - 1)) | (((uint64_t)1023) << 52))), (int64_t)(L - 128)};
        }
    } else {
        m = (uint64_t)v << (53 - L);
        mant = m;
    }
    return Er{bitsd((m & ((((uint64_t)1) << 52) - 1)) | (((uint64_t)1023) << 52)), (int64_t)(L - 129)};
}

/* the one-ulp interval of X/M from T = the 128-bit sum (true when certified) */
GRNS_HD bool eval_tight_finish(u128 T, uint64_t E, Er &low, Er &upp) {
    if (T <= (u128)E) return false;  // X near 0 or M (or X = 0)
    uint64_t ml, mu;
    int Ll, Lu;
    low = er_fx128(T - E, false, ml, Ll);
    upp = er_fx128(T, true, mu, Lu);
    return Ll == Lu && ml == mu;
}

/* one number: the one-ulp interval when certified (returns true), else
 * false; bad collects residues >= m_i */
template <int N, class Get>
GRNS_HD bool eval_tight(const Consts<N> &C, Get get, Er &low, Er &upp, uint32_t &bad) {
    Fx128 f;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t x = get(i);
        bad |= (uint32_t)(x >= C.m[i]);
        f.add(x, C.c128w_0[i], C.c128w_1[i], C.c128w_2[i], C.c128w_3[i]);
    }
    return eval_tight_finish(f.value(), C.E, low, upp);
}

/* ---------------- mixed-radix conversion (exact) ---------------- */
/* digits a_0..a_{N-1} with X = sum a_t * m_0...m_{t-1}; canonical (src/mrc.cuh:101) */
template <int N, class Get>
GRNS_HD void mrc_hd(const Consts<N> &C, Get get, uint32_t *mr) {
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        uint32_t v = get(i), m = C.m[i];
#pragma unroll 1
        for (int j = 0; j < i; j++) {
            uint32_t aj = mr[j] < m ? mr[j] : mr[j] % m;
            v = submod(v, aj, m);
            v = mulmod_shoup(v, ldg_u32(C.mrc_inv + j * N + i), ldg_u32(C.mrc_inv_sh + j * N + i), m);
        }
        mr[i] = v;
    }
}

template <int N, class GetX, class GetY>
GRNS_HD int cmp_exact(const Consts<N> &C, GetX gx, GetY gy) {
    bool eq = true;
#pragma unroll 1
    for (int i = 0; i < N; i++) eq &= gx(i) == gy(i);
    if (eq) return 0;
    uint32_t a[N], b[N];
    mrc_hd<N>(C, gx, a);
    mrc_hd<N>(C, gy, b);
#pragma unroll 1
    for (int i = N - 1; i >= 0; i--) {
        if (a[i] != b[i]) return a[i] > b[i] ? 1 : -1;
    }
    return 0;
}

/* ---------------- comparison ---------------- */
/* decision from two 64-bit fixed-point fractions: 1 / -1, or 2 when undecided */
GRNS_HD int fx64_order(uint64_t a, uint64_t b, uint64_t E) {
    if (a >= E && b >= E) {
        if (a - E > b) return 1;
        if (b - E > a) return -1;
    }
    return 2;
}

template <int N, class GetX, class GetY>
GRNS_HD int cmp_fx96_then_exact(const Consts<N> &C, GetX gx, GetY gy) {
    u128 tx = fx96<N>(C, gx), ty = fx96<N>(C, gy);
    const u128 E = C.E;
    if (tx >= E && ty >= E) {
        if (tx - E > ty) return 1;
        if (ty - E > tx) return -1;
    }
    return cmp_exact<N>(C, gx, gy);
}

/* sign(X - Y), the result of rns_cmp (src/rnscmp.cuh:55) */
template <int N, class GetX, class GetY>
GRNS_HD int cmp_fast(const Consts<N> &C, GetX gx, GetY gy) {
    int r = fx64_order(fx64<N>(C, gx), fx64<N>(C, gy), C.E);
    if (r != 2) return r;
    return cmp_fx96_then_exact<N>(C, gx, gy);
}

enum : uint32_t { kFxIterCap = 1u << 2 };

/* ---------------- directed-rounding helpers for the quotient estimate ---------------- */

/* double >= v */
GRNS_HD double u128_to_double_ru(u128 v) {
    int bl = bitlen128(v);
    if (bl <= 53) return (double)(uint64_t)v;
    uint64_t top = (uint64_t)(v >> (bl - 53));
    bool inexact = (v & ((((u128)1) << (bl - 53)) - 1)) != 0;
    return std::ldexp((double)(top + (inexact ? 1 : 0)), bl - 53);
}
/* a / b rounded toward -inf (a, b > 0) */
GRNS_HD double ddiv_rd_hd(double a, double b) {
#ifdef __CUDA_ARCH__
    return __ddiv_rd(a, b);
#else
    double q = a / b, r = std::fma(-q, b, a);
    return r < 0.0 ? std::nextafter(q, -INFINITY) : q;
#endif
}

/* ---------------- division: scaled-remainder digit recurrence ----------------
 *
 * q = floor(x / d), r = x - q d (the results of rns_div, src/rnsdiv.cuh:128).
 *
 * Pass A (dv_record) normalises, by fixed-point evaluations at k = 0 of
 * values magnified by the uniform constant 2^48 (dn_normalize):
 *   - the divisor: a shift s with D = d 2^s in [M/16 (1 - 2^-8), M/8 (1 + 2^-8))
 *     (s = 0 when d >= M/8 already);
 *   - the dividend: its magnitude, to skip the leading quotient digits that
 *     are certainly zero, and whether it lies within E / 2^96 of M.
 * Pass B computes floor(x 2^s / D) = q digit by digit, kDivB = 48 bits per
 * step; s = 48 a + t with 0 <= t < 48, k leading steps skipped (0 <= k <= a):
 *     k = 0:  R = x 2^(t-48) mod M, first step magnifies by 2^48 with the
 *             digit estimated from x itself (b = t);
 *     k >= 1: R = x 2^e with e = t + 48 (k - 1) (x 2^e < D certain: the
 *             skipped digits are 0), every step b = 48;
 *     step:   q_j = certified lower bound of floor(2^b R / D),
 *             R <- 2^48 R - q_j D,  Q <- 2^48 Q + q_j;
 * after a + 1 - k steps R = 2^s (x - Q d).  Every q_j is within 3 of the true
 * digit, which keeps 0 <= R < 4D < M/2: the residues of R (computed mod M)
 * are exact although 2^48 R itself wraps.  A final certified correction
 * c = floor(R / D) in {0..3} gives q = Q + c, and r = x - q d.
 *
 * Every residue operation of a step uses the same constants for all numbers
 * (2^48 mod m_i and the fixed-point reciprocals of the kernel parameter
 * block); the per-number tables (2^s, 2^e) are read once per division.  The
 * digit estimate is integer-only: the divisor's 63-bit upper mantissa Dm gets
 * a 53-bit reciprocal Rm <= 2^126 / Dm once (the single FP64 division), each
 * step takes the high word of At * Rm, At the top 64 bits of the remainder's
 * lower bound.  Digit error < 1.3 per step (ratio R / D < 4), < 2.3 on a
 * k = 0 first step (ratio x / D < 16.1).
 */
enum : uint32_t { kDnOk = 0, kDnNear = 1, kDnZero = 2, kDnBad = 3, kDnCap = 4 };

#ifdef __CUDACC__
#define GRNS_HD_RARE __host__ __device__ __noinline__
#else
#define GRNS_HD_RARE __attribute__((noinline))
#endif

GRNS_HD uint64_t umulhi64(uint64_t a, uint64_t b) {
#ifdef __CUDA_ARCH__
    return __umul64hi(a, b);
#else
    return (uint64_t)(((u128)a * b) >> 64);
#endif
}

/* floor(2^126 / Dm) rounded down to 53 bits, for 2^62 < Dm <= 2^63 */
GRNS_HD uint64_t dv_recip(uint64_t Dm) {
#ifdef __CUDA_ARCH__
    return __double2ull_rz(__ddiv_rd(0x1p126, __ull2double_ru(Dm)));
#else
    return (uint64_t)ddiv_rd_hd(std::ldexp(1.0, 126), u128_to_double_ru((u128)Dm));
#endif
}

/* v mod m_i for v < 2^53 (one Barrett step when b_i >= 27) */
template <int N>
GRNS_HD uint32_t reduce53(const Consts<N> &C, int i, uint64_t v) {
    if (C.b[i] >= 27) {  // hi * (2^32 mod m) + lo < 2^54 <= 2^(2b)
        const uint64_t p = (uint64_t)(uint32_t)(v >> 32) * C.t32[i] + (uint32_t)v;
        const uint32_t t = (uint32_t)(p >> (C.b[i] - 1));
        const uint32_t q = (uint32_t)(((uint64_t)t * C.mu[i]) >> (C.b[i] + 1));
        uint32_t r = (uint32_t)p - q * C.m[i];
        r = umin32(r, r - C.m[i]);
        return umin32(r, r - C.m[i]);
    }
    return reduce64<N>(C, i, v);
}

template <int N>
GRNS_HD_RARE int dv_cmp_vec(const Consts<N> &C, const uint32_t *a, const uint32_t *b) {
    return cmp_exact<N>(C, [&](int i) { return a[i]; }, [&](int i) { return b[i]; });
}

enum : int { kNormMore = 0, kNormOk = 1, kNormNear = 2, kNormCap = 3 };
/* normalisation steps of 48 bits a nonzero value can need (M below 2^(32 kMaxModuli)) */
constexpr int kNormMaxSteps = 32 * kMaxModuli / kDivB + 2;

/* One normalisation step of a nonzero Z: U = fx96w(Z 2^k).  U >= 2^43 fixes
 * the magnitude: Z 2^k / M in [U - E, U] / 2^96, U >= 2^43.  Below that Z 2^k
 * < 2^-53 M, so 2^48 more cannot wrap (the caller then magnifies its residues
 * and k grows by 48) -- unless k = 0 and U < E, where Z may instead be within
 * E / 2^96 of M; a magnification tells them apart: a small value then has
 * U < 2^91 + E, a value near M U > 2^96 (1 - 2^-13) (or it wraps again and
 * the next magnification decides). */
template <int N>
GRNS_HD int dn_step(const Consts<N> &C, u128 U, int &k, int &guard) {
    if (U >= (((u128)1) << 43)) {
        if (k > 0 && U >= (((u128)1) << 95)) return kNormNear;
        return kNormOk;
    }
    k += kDivB;
    if (++guard > kNormMaxSteps || k > C.log2M) return kNormCap;
    return kNormMore;
}

/* divisor shift s from the normalised divisor (magnification k, bit length bl of U) */
GRNS_HD int dv_shift(int k, int bl) {
    const int s = k + 93 - bl;
    return s < 0 ? 0 : s;
}

/* first kept quotient step: returns e (x is replaced by x 2^e), e < 0 when no
 * step is skipped; kx, blx describe the normalised dividend */
GRNS_HD int dv_skip(int s, int kx, int blx) {
    const int t = s % kDivB, a = s / kDivB;
    const int num = 91 + kx - blx - t;  // x 2^e < D certain for e <= num
    int k = num < 0 ? 0 : num / kDivB + 1;
    if (k > a) k = a;
    return t + kDivB * (k - 1);
}

/* pass-A record: x = status << 16 | s, y = xnear << 31 | (e & 0xffff) */
GRNS_HD uint2 dv_pack(uint32_t status, int s, int e, bool xnear) {
    uint2 r;
    r.x = (status << 16) | (uint32_t)s;
    r.y = (xnear ? 0x80000000u : 0u) | ((uint32_t)e & 0xffffu);
    return r;
}
GRNS_HD int dv_rec_e(const uint2 &r) { return (int)(int16_t)(uint16_t)(r.y & 0xffffu); }

template <int N>
GRNS_HD int dn_normalize(const Consts<N> &C, const uint32_t *z, int &k, int &bl) {
    uint32_t w[N];
    for (int i = 0; i < N; i++) w[i] = z[i];
    k = 0;
    int guard = 0;
    for (;;) {
        const int k0 = k;
        const u128 U = fx96w<N>(C, [&](int i) { return w[i]; });
        const int ns = dn_step<N>(C, U, k, guard);
        if (ns == kNormOk) {
            bl = bitlen128(U);
            k = k0;
        }
        if (ns != kNormMore) return ns;
        for (int i = 0; i < N; i++) w[i] = mulmod_shoup(w[i], C.b48[i], C.b48_sh[i], C.m[i]);
    }
}

/* pass A for one number (x, d canonical) */
template <int N>
GRNS_HD uint2 dv_record(const Consts<N> &C, const uint32_t *x, const uint32_t *d) {
    bool dz = true, xz = true;
    for (int i = 0; i < N; i++) {
        dz &= d[i] == 0;
        xz &= x[i] == 0;
    }
    if (dz) return dv_pack(kDnZero, 0, 0, false);
    int kd, bld;
    const int nd = dn_normalize<N>(C, d, kd, bld);
    if (nd == kNormNear) return dv_pack(kDnNear, 0, 0, false);
    if (nd == kNormCap) return dv_pack(kDnCap, 0, 0, false);
    const int s = dv_shift(kd, bld);
    if (xz) return dv_pack(kDnOk, s, s % kDivB - kDivB, false);
    int kx, blx;
    const int nx = dn_normalize<N>(C, x, kx, blx);
    if (nx == kNormCap) return dv_pack(kDnCap, 0, 0, false);
    if (nx == kNormNear) return dv_pack(kDnOk, s, s % kDivB - kDivB, true);
    return dv_pack(kDnOk, s, dv_skip(s, kx, blx), false);
}

/* pass B state of one division */
struct DivSt {
    u128 UD;      // D / M * 2^96 in [UD - E, UD]
    uint64_t Rm;  // <= 2^126 / Dm,  Dm = floor(UD / 2^sd) + 1
    int sd;
    int b;        // magnification of the next step's digit
    int left;     // steps still to run
    uint32_t f;
};

GRNS_HD void dv_setup(DivSt &st, u128 UD, int s, int e) {
    st.UD = UD;
    st.sd = bitlen128(UD) - 63;
    st.Rm = dv_recip((uint64_t)(UD >> st.sd) + 1);
    const int t = s % kDivB, a = s / kDivB;
    const int k = e < 0 ? 0 : (e - t) / kDivB + 1;
    st.b = e < 0 ? t : kDivB;
    st.left = a + 1 - k;
    st.f = 0;
}

/* lower bound of floor(2^b R / D) from U = fx96w(R) (U = 2^96 stands for R
 * within E / 2^96 of M) */
GRNS_HD uint64_t dv_digit(const DivSt &st, u128 U, uint64_t E, uint32_t &flags) {
    if (U <= (u128)E) return 0;
    const u128 A = U - E;
    const int L = bitlen128(A);
    const uint64_t At = L >= 64 ? (uint64_t)(A >> (L - 64)) : (uint64_t)A << (64 - L);
    const uint64_t qt = umulhi64(At, st.Rm);
    /* 2^b R / D >= 2^b A / UD >= qt 2^(b + (L - 64) - sd - 62) */
    const int sh = st.b + (L - 64) - st.sd - 62;
    if (sh >= 0) {  // a digit >= 2^62: not a reachable state
        flags |= kFxIterCap;
        return 0;
    }
    return -sh >= 64 ? 0 : qt >> (-sh);
}

/* c = floor(R / D) for 0 <= R < 4D from the fixed-point values; -1 when a
 * comparison is too close to call (the exact path decides).  UR < E is
 * ambiguous once 4D may reach M (1 - E / 2^96): R is then either tiny or
 * within E M / 2^96 of M, where the evaluation wraps past 2^96 to below E. */
GRNS_HD int dv_final_fx(const DivSt &st, u128 UR, uint64_t Eu) {
    const u128 E = Eu;
    if (UR < E && 4 * st.UD + E > (((u128)1) << 96)) return -1;
    int c = 0;
    for (int j = 1; j <= 3; j++) {
        const u128 jD = (u128)j * st.UD, jDl = (u128)j * (st.UD - E);
        if (UR >= E && UR - E >= jD) {
            c = j;  // R >= j D certain
        } else if (UR < jDl) {
            return c;  // R < j D certain
        } else {
            return -1;
        }
    }
    return c;
}

/* R = j D for some j in 1..3, read from the residues; valid when 3D < M
 * (then equal residues mean equal values), i.e. for UD < 2^94 (D < M / 4).
 * Returns j, or 0.  This is the usual way the fixed-point comparisons end
 * too close to call: after the steps R = 2^s (x - Q d), so R - j D is a
 * multiple of 2^s, which the fixed-point band (width ~ 2^-60 M) can only
 * contain as 0 when d < 2^48 -- a divisor that divides the dividend. */
template <int N, class GR, class GD>
GRNS_HD int dv_final_tie(const Consts<N> &C, u128 UD, GR rg, GD dg) {
    if (UD >= (((u128)1) << 94)) return 0;
    bool e1 = true, e2 = true, e3 = true;
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i], r = rg(i), d1 = dg(i), d2 = addmod(d1, d1, m);
        e1 &= r == d1;
        e2 &= r == d2;
        e3 &= r == addmod(d2, d1, m);
    }
    return e1 ? 1 : (e2 ? 2 : (e3 ? 3 : 0));
}

/* exact c = floor(R / D) (R < 4D): repeated exact comparison and subtraction */
template <int N>
GRNS_HD_RARE int dv_final_exact(const Consts<N> &C, const uint32_t *R, const uint32_t *D) {
    uint32_t a[N];
    for (int i = 0; i < N; i++) a[i] = R[i];
    int c = 0;
    while (c < 3 && dv_cmp_vec<N>(C, a, D) >= 0) {
        for (int i = 0; i < N; i++) a[i] = submod(a[i], D[i], C.m[i]);
        c++;
    }
    return c;
}

/* q, r of one division (both passes, one number); q, r, x, d: N canonical
 * residues each */
template <int N>
GRNS_HD void div_fast(const Consts<N> &C, uint32_t *q, uint32_t *r, const uint32_t *x, const uint32_t *d,
                      uint32_t &flags) {
    bool xz = true;
    for (int i = 0; i < N; i++) {
        q[i] = 0;
        r[i] = x[i];
        xz &= x[i] == 0;
    }
    const uint2 rec = dv_record<N>(C, x, d);
    const uint32_t status = rec.x >> 16;
    if (status == kDnZero) {
        flags |= 1u << 1;  // division by zero
        return;
    }
    if (status == kDnCap) {
        flags |= kFxIterCap;
        return;
    }
    if (xz) return;
    if (status == kDnNear) {  // d > M (1 - E / 2^96): the quotient is 0 or 1
        if (dv_cmp_vec<N>(C, x, d) >= 0) {
            for (int i = 0; i < N; i++) {
                q[i] = 1;
                r[i] = submod(r[i], d[i], C.m[i]);
            }
        }
        return;
    }
    const int s = (int)(rec.x & 0xffffu), e = dv_rec_e(rec);
    uint32_t D[N], R[N], Q[N];
    const uint32_t *ps = C.pow2 + (int64_t)s * N, *pss = C.pow2_sh + (int64_t)s * N;
    for (int i = 0; i < N; i++) D[i] = mulmod_shoup(d[i], ldg_u32(ps + i), ldg_u32(pss + i), C.m[i]);
    DivSt st;
    dv_setup(st, fx96w<N>(C, [&](int i) { return D[i]; }), s, e);
    const uint32_t *pe = e < 0 ? C.pow2neg + (int64_t)(-e) * N : C.pow2 + (int64_t)e * N;
    const uint32_t *pes = e < 0 ? C.pow2neg_sh + (int64_t)(-e) * N : C.pow2_sh + (int64_t)e * N;
    for (int i = 0; i < N; i++) {
        R[i] = mulmod_shoup(x[i], ldg_u32(pe + i), ldg_u32(pes + i), C.m[i]);
        Q[i] = 0;
    }
    u128 U = (rec.y >> 31) ? (((u128)1) << 96) : fx96w<N>(C, [&](int i) { return e < 0 ? x[i] : R[i]; });
    for (; st.left > 0; st.left--) {
        const uint64_t qd = dv_digit(st, U, C.E, st.f);
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i];
            const uint32_t qi = reduce53<N>(C, i, qd);
            R[i] = submod(mulmod_shoup(R[i], C.b48[i], C.b48_sh[i], m), mulmod_barrett(qi, D[i], m, C.mu[i], C.b[i]), m);
            Q[i] = addmod(mulmod_shoup(Q[i], C.b48[i], C.b48_sh[i], m), qi, m);
        }
        U = fx96w<N>(C, [&](int i) { return R[i]; });
        st.b = kDivB;
    }
    int c = dv_final_fx(st, U, C.E);
    if (c < 0) {
        c = dv_final_tie<N>(C, st.UD, [&](int i) { return R[i]; }, [&](int i) { return D[i]; });
        if (c == 0) c = dv_final_exact<N>(C, R, D);
    }
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i];
        q[i] = addmod(Q[i], (uint32_t)c % m, m);
        r[i] = submod(x[i], mulmod_barrett(q[i], d[i], m, C.mu[i], C.b[i]), m);
    }
    flags |= st.f;
}

/* ---------------- division through prepared rows ----------------
 *
 * The plain call's form of the same division.  Pass A leaves, per number, a
 * row of kRowWords(N) words: the scaled divisor D = d 2^s (N residues at
 * offset 0), the starting remainder R (N residues at offset kRowPad(N), N
 * rounded up to a multiple of 4) and a 16-word header with the digit
 * loop's state (dv_setup's UD, reciprocal, shift and step count, and the
 * first step's fixed-point value), or -- for a division with no digit step
 * (invalid input, zero divisor, zero dividend, divisor within E / 2^96 of M,
 * normalisation cap) -- its final q and r.  Pass B runs the digit steps from
 * the row alone, in any order, and leaves q and r in the row's first 2N
 * words, so the numbers can be scheduled longest first across the whole call
 * while every access to a number's data is one contiguous row.
 *
 * The remainder comes from the final R without x and d: after the steps
 * R = 2^s (x - Q d) with 0 <= R < 4D, so for c = floor(R / D)
 *     q = Q + c,   r = x - q d = (R - c D) 2^-s,
 * and 2^-s mod m_i exists for the odd moduli (2^-s = 2^-(s mod 64) 2^-(64 floor(s / 64)),
 * two table rows; s <= log2M + 49).
 */
constexpr int kRowHdr = 16;  // header words of a row
template <int N>
constexpr int kRowPad() {  // residue block of a row: N words rounded up to a multiple of 4
    return (N + 3) & ~3;
}
template <int N>
constexpr int kRowWords() {  // D (or q) at 0, R (or r) at kRowPad, the header at 2 kRowPad: 16-byte vectors
    return 2 * kRowPad<N>() + kRowHdr;
}
/* header word offsets (after the 2N residues) */
enum : int { kHdrUD = 0, kHdrU = 4, kHdrRm = 8, kHdrS = 10, kHdrSd = 11, kHdrB = 12, kHdrLeft = 13, kHdrFlags = 14 };

GRNS_HD void u128_put(uint32_t *w, u128 v) {
    w[0] = (uint32_t)v;
    w[1] = (uint32_t)(v >> 32);
    w[2] = (uint32_t)(v >> 64);
    w[3] = (uint32_t)(v >> 96);
}
GRNS_HD u128 u128_get(const uint32_t *w) {
    return (u128)w[0] | ((u128)w[1] << 32) | ((u128)w[2] << 64) | ((u128)w[3] << 96);
}

/* header of a division with digit steps (st after dv_setup, U the first step's value) */
GRNS_HD void div_hdr_put(uint32_t *h, const DivSt &st, u128 U, int s) {
    u128_put(h + kHdrUD, st.UD);
    u128_put(h + kHdrU, U);
    h[kHdrRm] = (uint32_t)st.Rm;
    h[kHdrRm + 1] = (uint32_t)(st.Rm >> 32);
    h[kHdrS] = (uint32_t)s;
    h[kHdrSd] = (uint32_t)st.sd;
    h[kHdrB] = (uint32_t)st.b;
    h[kHdrLeft] = (uint32_t)st.left;
    h[kHdrFlags] = 0;
    h[kHdrFlags + 1] = 0;
}
GRNS_HD void div_hdr_get(const uint32_t *h, DivSt &st, u128 &U, int &s) {
    st.UD = u128_get(h + kHdrUD);
    U = u128_get(h + kHdrU);
    st.Rm = (uint64_t)h[kHdrRm] | ((uint64_t)h[kHdrRm + 1] << 32);
    s = (int)h[kHdrS];
    st.sd = (int)h[kHdrSd];
    st.b = (int)h[kHdrB];
    st.left = (int)h[kHdrLeft];
    st.f = 0;
}

/* pass A's row of one division from its record (dv_record) and the operands
 * (x, d canonical; getters xg(i), dg(i)); returns the digit steps (0: the
 * row already holds q and r, flags set) */
template <int N, class GX, class GD>
GRNS_HD int div_row_setup(const Consts<N> &C, uint2 rec, GX xg, GD dg, uint32_t *row, uint32_t &flags) {
    const uint32_t status = rec.x >> 16;
    bool xz = true;
    for (int i = 0; i < N; i++) xz &= xg(i) == 0;
    if (status != kDnOk || xz) {  // q = 0, r = x unless stated below
        bool one = false;
        if (status == kDnBad) flags |= 1u;  // INVALID_INPUT: q = r = 0
        else if (status == kDnZero) flags |= 1u << 1;  // division by zero
        else if (status == kDnCap) flags |= kFxIterCap;
        else if (status == kDnNear && !xz) {  // d > M (1 - E / 2^96): the quotient is 0 or 1
            uint32_t a[N], b[N];
            for (int i = 0; i < N; i++) {
                a[i] = xg(i);
                b[i] = dg(i);
            }
            one = dv_cmp_vec<N>(C, a, b) >= 0;
        }
        for (int i = 0; i < N; i++) {
            const uint32_t xv = status == kDnBad ? 0u : xg(i);
            row[i] = one ? 1u : 0u;
            row[kRowPad<N>() + i] = one ? submod(xv, dg(i), C.m[i]) : xv;
        }
        return 0;
    }
    const int s = (int)(rec.x & 0xffffu), e = dv_rec_e(rec);
    constexpr int P = kRowPad<N>();
    for (int i = 0; i < N; i++) {
        row[i] = mul_pow2<N>(C, i, dg(i), s);
        row[P + i] = e < 0 ? mul_pow2neg<N>(C, i, xg(i), -e) : mul_pow2<N>(C, i, xg(i), e);
    }
    DivSt st;
    dv_setup(st, fx96w<N>(C, [&](int i) { return row[i]; }), s, e);
    const u128 U = (rec.y >> 31) ? (((u128)1) << 96)
                                 : (e < 0 ? fx96w<N>(C, xg) : fx96w<N>(C, [&](int i) { return row[P + i]; }));
    div_hdr_put(row + 2 * P, st, U, s);
    return st.left;
}

/* q and r of a division whose digit steps are done: R (the remainder rows),
 * D, Q residues, U = fx96w(R), st its state, s its shift; c from the
 * fixed-point values, exact comparisons when too close to call */
template <int N>
GRNS_HD void div_row_final(const Consts<N> &C, const uint32_t *R, const uint32_t *D, const uint32_t *Q, u128 U,
                           const DivSt &st, int s, uint32_t *q, uint32_t *r) {
    int c = dv_final_fx(st, U, C.E);
    if (c < 0) {
        c = dv_final_tie<N>(C, st.UD, [&](int i) { return R[i]; }, [&](int i) { return D[i]; });
        if (c == 0) c = dv_final_exact<N>(C, R, D);
    }
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i], cm = (uint32_t)c % m;  // c <= 3, m >= 3
        const uint32_t cd = mulmod_barrett(cm, D[i], m, C.mu[i], C.b[i]);
        q[i] = addmod(Q[i], cm, m);
        r[i] = mul_pow2neg<N>(C, i, submod(R[i], cd, m), s);
    }
}

/* the digit steps of one row (host form of pass B, for checks): q and r
 * replace the row's first 2N words */
template <int N>
GRNS_HD void div_row_run(const Consts<N> &C, uint32_t *row, uint32_t &flags) {
    constexpr int P = kRowPad<N>();
    DivSt st;
    u128 U;
    int s;
    div_hdr_get(row + 2 * P, st, U, s);
    uint32_t R[N], D[N], Q[N];
    for (int i = 0; i < N; i++) {
        D[i] = row[i];
        R[i] = row[P + i];
        Q[i] = 0;
    }
    for (; st.left > 0; st.left--) {
        const uint64_t qd = dv_digit(st, U, C.E, st.f);
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i];
            const uint32_t qi = reduce53<N>(C, i, qd);
            R[i] = submod(mulmod_shoup(R[i], C.b48[i], C.b48_sh[i], m), mulmod_barrett(qi, D[i], m, C.mu[i], C.b[i]), m);
            Q[i] = addmod(mulmod_shoup(Q[i], C.b48[i], C.b48_sh[i], m), qi, m);
        }
        U = fx96w<N>(C, [&](int i) { return R[i]; });
        st.b = kDivB;
    }
    div_row_final<N>(C, R, D, Q, U, st, s, row, row + P);
    flags |= st.f;
}

/* q, r of one division through a row (the plain call's three passes for one
 * number; checked against div_fast and exact arithmetic on the CPU) */
template <int N>
GRNS_HD void div_rows(const Consts<N> &C, uint32_t *q, uint32_t *r, const uint32_t *x, const uint32_t *d,
                      uint32_t &flags) {
    uint32_t row[kRowWords<N>()];
    bool bad = false;
    for (int i = 0; i < N; i++) bad |= x[i] >= C.m[i] || d[i] >= C.m[i];
    const uint2 rec = bad ? dv_pack(kDnBad, 0, 0, false) : dv_record<N>(C, x, d);
    if (div_row_setup<N>(C, rec, [&](int i) { return x[i]; }, [&](int i) { return d[i]; }, row, flags) > 0)
        div_row_run<N>(C, row, flags);
    for (int i = 0; i < N; i++) {
        q[i] = row[i];
        r[i] = row[kRowPad<N>() + i];
    }
}

/* ---------------- power-of-two scaling (results of rns_scale2pow, src/rnsscal.cuh:93) ---------------- */

/* k with X = sum_i M_i c_i - k M (rns_rank_compute, :134); `small` when X < M/2^30 is known */
template <int N>
GRNS_HD uint32_t rank_fast(const Consts<N> &C, const uint32_t *x, const uint32_t *c, bool small) {
    u128 t = fx96_s<N>(C, [&](int i) { return c[i]; });
    u128 U = t & kMask96;
    uint32_t kk = (uint32_t)(t >> 96);
    if (U >= (u128)C.E || small) return kk;
    uint32_t a[N];
    mrc_hd<N>(C, [&](int i) { return x[i]; }, a);
    return a[N - 1] == 0 ? kk : kk - 1;
}

/* One exact scaling step (the role of make_scaling_step, :181, with steps of
 * up to kScaleB = 52 bits instead of RNS_P2_SCALING_THRESHOLD = 30):
 * y = (x - (X mod 2^j)) 2^-j, with X mod 2^j = (sum_i c_i M_i - k M) mod 2^j
 * computed in 64-bit wrap-around arithmetic (c_i = x_i w_i mod m_i, k the
 * rank) and reduced once per modulus (X mod 2^j < 2^52). */
template <int N>
GRNS_HD void scaling_step_big(const Consts<N> &C, uint32_t *y, uint32_t k, int j, const uint32_t *x,
                              const uint32_t *c) {
    uint64_t acc = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) acc += (uint64_t)c[i] * C.mi64[i];
    const uint64_t res = (acc - (uint64_t)k * C.m64) & ((((uint64_t)1) << j) - 1);
    const uint32_t *inv = C.pow2neg + (int64_t)j * N, *inv_sh = C.pow2neg_sh + (int64_t)j * N;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i];
        y[i] = mulmod_shoup(submod(x[i], reduce53<N>(C, i, res), m), ldg_u32(inv + i), ldg_u32(inv_sh + i), m);
    }
}

/* floor(X / 2^D) (the result of rns_scale2pow, src/rnsscal.cuh:207): steps of
 * kScaleB bits; the first step's rank is checked (X arbitrary), later ones
 * act on X < M / 2 */
template <int N>
GRNS_HD void scale_fast(const Consts<N> &C, uint32_t *res, const uint32_t *x, unsigned D) {
    uint32_t cur[N], c[N];
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) cur[i] = x[i];
    bool small = false;
    if (D > (unsigned)C.log2M) D = 0, small = true;  // X < M < 2^(log2M + 1): the result is 0
    if (small) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) res[i] = 0;
        return;
    }
#pragma unroll 1
    for (unsigned left = D; left > 0;) {
        const int j = left < (unsigned)kScaleB ? (int)left : kScaleB;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) c[i] = mulmod_shoup(cur[i], C.w[i], C.w_sh[i], C.m[i]);
        const uint32_t k = rank_fast<N>(C, cur, c, small);
        scaling_step_big<N>(C, cur, k, j, cur, c);
        left -= (unsigned)j;
        small = true;
    }
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) res[i] = cur[i];
}

/* ---------------- power-of-two scaling in one pass ----------------
 *
 * floor(X / 2^D) = (X - (X mod 2^D)) 2^-D mod M (M odd).  With the exact rank
 * k, X = sum_i s_i M_i - k M (s_i = x_i w_i mod m_i), so the low D bits of X
 * are the low 26-bit chunks of that sum (the CRT weights M_i and M in 26-bit
 * chunks, the binary conversion's tables), carried chunk by chunk; each chunk
 * r_c of X mod 2^D enters every residue as r_c (2^(26 c) mod m_i).  Work
 * grows with D / 26 (two n-term sums per chunk) instead of one rank and two
 * passes over the residues per 52-bit step. */

/* exact rank of X (the fixed-point estimate, decided by mixed radix when
 * the fraction lies within E of an integer) */
template <int N, class GetS, class GetX>
GRNS_HD uint32_t scale_bin_rank(const Consts<N> &C, GetS gs, GetX gx) {
    const u128 t = fx96_s<N>(C, gs);
    const uint32_t kk = (uint32_t)(t >> 96);
    if ((t & kMask96) >= (u128)C.E) return kk;
    uint32_t a[N];
    mrc_hd<N>(C, gx, a);
    return a[N - 1] == 0 ? kk : kk - 1;
}

/* (x_i - r_i) 2^-D mod m_i from r_i = (X mod 2^D) mod m_i */
template <int N>
GRNS_HD uint32_t scale_bin_finish(const Consts<N> &C, int i, uint32_t x, uint32_t r, unsigned D) {
    const uint32_t m = C.m[i];
    const uint2 lo = ldg_u2(C.p2nlo + (int64_t)i * 64 + (D & 63u));
    const uint2 hi = ldg_u2(C.p2nhi + (int64_t)i * C.p2rows + (D >> 6));
    return mulmod_shoup(mulmod_shoup(submod(x, r, m), lo.x, lo.y, m), hi.x, hi.y, m);
}

template <int N>
GRNS_HD void scale_bin(const Consts<N> &C, uint32_t *res, const uint32_t *x, unsigned D) {
    if (D > (unsigned)C.log2M || D == 0) {  // X < M < 2^(log2M + 1): 0; D = 0: X
        for (int i = 0; i < N; i++) res[i] = D ? 0u : x[i];
        return;
    }
    uint32_t s[N];
    uint64_t acc[N];
    for (int i = 0; i < N; i++) {
        s[i] = mulmod_shoup(x[i], C.w[i], C.w_sh[i], C.m[i]);
        acc[i] = 0;
    }
    const uint32_t kk = scale_bin_rank<N>(C, [&](int i) { return s[i]; }, [&](int i) { return x[i]; });
    const int chunks = (int)((D + kBinChunk - 1) / kBinChunk);
    int64_t carry = 0;
    for (int c = 0; c < chunks; c++) {
        uint64_t a = 0;
        const uint32_t *mi = C.bin_mi26 + (size_t)c * bin_ld(N);
        for (int i = 0; i < N; i++) a += (uint64_t)s[i] * mi[i];
        const int64_t v = (int64_t)a - (int64_t)kk * C.bin_m26[c] + carry;
        carry = v >> kBinChunk;  // floor division (arithmetic shift)
        uint32_t r = (uint32_t)v & kBinMask;
        if (c == chunks - 1 && D % kBinChunk) r &= (1u << (D % kBinChunk)) - 1u;
        const uint32_t *p = C.bin_p26 + (size_t)c * bin_ld(N);
        for (int i = 0; i < N; i++) acc[i] += (uint64_t)r * p[i];
    }
    for (int i = 0; i < N; i++) res[i] = scale_bin_finish<N>(C, i, x[i], bin_mod64<N>(C, i, acc[i]), D);
}

}  // namespace grns
