/*
 * grns_gb300 -- device algorithms of the RNS interval-evaluation path.
 *
 * Semantics follow the reference's GPU functions (kisupov/grns, namespace
 * cuda) bit for bit; each function cites the one it matches.  The structure
 * is GB300-first rather than a translation:
 *   - one thread per number ("serial" schedule) over structure-of-arrays
 *     residues, so every modulus slice is a coalesced load;
 *   - the fixed pairwise summation tree of the reference (psum_rd/psum_ru,
 *     src/pairwise.cuh:837-918) is evaluated as a streaming binary counter
 *     over the residues (log2 n partial sums live, no n-element arrays);
 *   - x_i * w_i mod m_i on the integer pipe (Shoup), no 64-bit remainder;
 *   - the rare branches (MRC ambiguity, refinement loop, MRC tie-breaks)
 *     live in non-inlined functions that reload the operands, keeping the
 *     common path small;
 *   - every data-dependent loop has an iteration cap that raises a status
 *     flag instead of spinning.
 */
#pragma once

#include "rns_common.cuh"
#include "rns_fast.cuh"

namespace grns {

/* status flag bits written by kernels (per element) */
enum : uint32_t {
    kFlagInvalidInput = 1u << 0,   // residue >= modulus
    kFlagDivByZero = 1u << 1,      // rns_div with d == 0
    kFlagIterCap = 1u << 2,        // a data-dependent loop hit its cap
    kFlagOverflow = 1u << 3,       // mp_int result overflowed (mpint_check_overflow, "has occurred")
    kFlagMayOverflow = 1u << 4,    // mp_int result may have overflowed ("needs to be clarified")
};

/* ---------------- operand access ---------------- */

/* residue i of number k: SoA (x[i * ld + k]) or AoS (x[k * N + i]) */
template <int N>
struct Operand {
    const uint32_t *base;
    int64_t ld;   // SoA leading dimension (elements); AoS when ld == 0
    __device__ __forceinline__ uint32_t load(int64_t k, int i) const {
        return ld ? __ldg(base + (int64_t)i * ld + k) : __ldg(base + k * N + i);
    }
    __device__ __forceinline__ uint32_t load_cs(int64_t k, int i) const {  // streaming, evict-first
        return ld ? __ldcs(base + (int64_t)i * ld + k) : __ldcs(base + k * N + i);
    }
    /* bring number k's residues into L2 ahead of their loads */
    __device__ __forceinline__ void prefetch_l2(int64_t k) const {
        if (ld) {
#pragma unroll 4
            for (int i = 0; i < N; i++) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + (int64_t)i * ld + k));
        } else {
GRNS_UNROLL_N
            for (int i = 0; i < N; i += 32) asm volatile("prefetch.global.L2 [%0];" ::"l"(base + k * N + i));
        }
    }
};

template <int N>
struct Output {
    uint32_t *base;
    int64_t ld;
    __device__ __forceinline__ void store(int64_t k, int i, uint32_t v) const {
        if (ld) base[(int64_t)i * ld + k] = v; else base[k * N + i] = v;
    }
};

/* ---------------- the reference's pairwise tree as a streaming counter ---------------- */


template <int N, bool UP>
struct PTree {
    static constexpr int L = ilog2c(N) + 1;
    double lv[L];
    __device__ __forceinline__ static double add(double a, double b) { return UP ? __dadd_ru(a, b) : __dadd_rd(a, b); }
    /* push leaf `i` (compile-time after unrolling) */
    __device__ __forceinline__ void push(int i, double v) {
#pragma unroll
        for (int k = 0; k < L; k++) {
            if (!((i >> k) & 1)) { lv[k] = v; return; }
            v = add(lv[k], v);
        }
    }
    /* tree total after the N leaves: zero-padded complete tree (adding an
     * exact zero is exact in directed rounding) */
    __device__ __forceinline__ double total() const {
        double acc = 0.0;
        bool have = false;
#pragma unroll
        for (int k = 0; k < L; k++) {
            if ((N >> k) & 1) {
                acc = have ? add(lv[k], acc) : lv[k];
                have = true;
            }
        }
        return acc;
    }
};

/* ---------------- mixed-radix conversion (src/mrc.cuh:101) ---------------- */
/* Szabo-Tanaka digits, canonical in [0, m_i). */
template <int N, class Get>
__device__ __forceinline__ void mrc_digits(const Consts<N> &C, Get get, uint32_t *mr) {
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        uint32_t v = get(i), m = C.m[i];
#pragma unroll 1
        for (int j = 0; j < i; j++) {
            v = submod(v, mr[j] % m, m);
            v = mulmod_shoup(v, C.mrc_inv[j * N + i], C.mrc_inv_sh[j * N + i], m);
        }
        mr[i] = v;
    }
}

/* ---------------- interval evaluation (src/rnseval.cuh:182-256) ---------------- */

/* Full reference algorithm with arrays; used for the rare branches. */
template <int N, class Get, bool FAST = false>
__device__ __noinline__ void eval_full(const Consts<N> &C, Get get, Er &low, Er &upp, uint32_t &flags) {
    uint32_t s[N];
    PTree<N, false> tl;
    PTree<N, true> tu;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        s[i] = mulmod_shoup(get(i), C.w[i], C.w_sh[i], C.m[i]);
        double d = u32_to_double(s[i]);
        tl.push(i, __dmul_rd(d, C.rrd[i]));
        tu.push(i, __dmul_ru(d, C.rru[i]));
    }
    double suml = tl.total(), sumu = tu.total();
    if (suml == 0 && sumu == 0) {
        low = Er{0.0, 0};
        upp = Er{0.0, 0};
        return;
    }
    unsigned whl = __double2uint_rz(suml), whu = __double2uint_rz(sumu);
    suml = __dsub_rd(suml, u32_to_double(whl));
    sumu = __dsub_ru(sumu, u32_to_double(whu));
    low = er_from_double(suml);
    upp = er_from_double(sumu);
    int mr = -1;
    if (!FAST && whl != whu) {  // rns_eval_compute_fast skips the ambiguity step
        uint32_t d[N];
        mrc_digits<N>(C, get, d);
        mr = (int)d[N - 1];
    }
    if (mr > 0) {
        upp = C.inv_unit_upp;
        return;
    }
    if (mr == 0) low = C.unit_low;
    if (sumu >= C.acc) return;
    int K = 0, guard = 0;
    const int cap = C.log2M / (C.ref_factor > 0 ? C.ref_factor : 1) + 8;
#pragma unroll 1
    while (sumu < C.acc) {
        if (++guard > cap) { flags |= kFlagIterCap; break; }
        double a = -(ceil(log2(sumu)) + 1);
        int k = (int)(a > (double)C.ref_factor ? a : (double)C.ref_factor);
        if (k < 0 || k > C.log2M) { flags |= kFlagIterCap; break; }
        const uint32_t *p2 = C.pow2 + (int64_t)k * N;
        PTree<N, true> t2;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            s[i] = mulmod_barrett(s[i], __ldg(p2 + i), C.m[i], C.mu[i], C.b[i]);
            t2.push(i, __dmul_ru(u32_to_double(s[i]), C.rru[i]));
        }
        sumu = t2.total();
        sumu = __dsub_ru(sumu, u32_to_double(__double2uint_rz(sumu)));
        K += k;
    }
    PTree<N, false> t3;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) t3.push(i, __dmul_rd(u32_to_double(s[i]), C.rrd[i]));
    suml = t3.total();
    suml = __dsub_rd(suml, u32_to_double(__double2uint_rz(suml)));
    low = er_from_double(suml);
    upp = er_from_double(sumu);
    low.exp -= K;
    upp.exp -= K;
}

/* Common path on the FP64 pipe: the reference's own directed-rounding
 * products and pairwise sums (src/rnseval.cuh:194-215), with eval_int's
 * outcomes -- kEvalOk (low / upp set), kEvalZero, or kEvalRare for an
 * ambiguous integer part or a fraction below RNS_EVAL_ACCURACY (eval_full
 * decides those).  The same doubles as eval_int, which emulates exactly
 * these operations on the integer pipe; a kernel can give some of its warps
 * this form so the FP64 and integer pipes work at once. */
template <int N, class Get, bool FAST = false>
__device__ __forceinline__ int eval_fp64(const Consts<N> &C, Get get, Er &low, Er &upp, uint32_t &bad) {
    PTree<N, false> tl;
    PTree<N, true> tu;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t xi = get(i);
        bad |= (uint32_t)(xi >= C.m[i]);
        const double d = u32_to_double(mulmod_shoup(xi, C.w[i], C.w_sh[i], C.m[i]));
        tl.push(i, __dmul_rd(d, C.rrd[i]));
        tu.push(i, __dmul_ru(d, C.rru[i]));
    }
    double suml = tl.total(), sumu = tu.total();
    if (suml == 0 && sumu == 0) return kEvalZero;
    const unsigned whl = __double2uint_rz(suml), whu = __double2uint_rz(sumu);
    if (!FAST && whl != whu) return kEvalRare;
    suml = __dsub_rd(suml, u32_to_double(whl));
    sumu = __dsub_ru(sumu, u32_to_double(whu));
    if (sumu < C.acc) return kEvalRare;
    low = er_from_double(suml);
    upp = er_from_double(sumu);
    return kEvalOk;
}

/* Common path on the integer pipe (eval_int, rns_fast.cuh: the same doubles as
 * the FP64 directed-rounding trees, computed exactly); falls back to eval_full
 * for ambiguous integer parts or small values (rare for uniform X). */
template <int N, class Get, bool FAST = false>
__device__ __forceinline__ void eval(const Consts<N> &C, Get get, Er &low, Er &upp, uint32_t &flags) {
    uint32_t bad = 0;
    const int st = eval_int<N, Get, FAST>(C, get, low, upp, bad);
    if (bad) {
        flags |= kFlagInvalidInput;
        low = Er{0.0, 0};
        upp = Er{0.0, 0};
        return;
    }
    if (st == kEvalZero) {
        low = Er{0.0, 0};
        upp = Er{0.0, 0};
        return;
    }
    if (st == kEvalRare) eval_full<N, Get, FAST>(C, get, low, upp, flags);
}

/* ---------------- comparison (src/rnscmp.cuh:55-74) ---------------- */
template <int N, class GetX, class GetY>
__device__ __noinline__ int cmp_tie(const Consts<N> &C, GetX gx, GetY gy) {
    bool eq = true;
#pragma unroll 1
    for (int i = 0; i < N; i++) eq &= gx(i) == gy(i);
    if (eq) return 0;
    uint32_t a[N], b[N];
    mrc_digits<N>(C, gx, a);
    mrc_digits<N>(C, gy, b);
#pragma unroll 1
    for (int i = N - 1; i >= 0; i--) {
        if (a[i] > b[i]) return 1;
        if (b[i] > a[i]) return -1;
    }
    return 0;
}

template <int N>
__device__ __forceinline__ int cmp_intervals(const Er &xl, const Er &xu, const Er &yl, const Er &yu) {
    if (er_ucmp(xl, yu) > 0) return 1;
    if (er_ucmp(yl, xu) > 0) return -1;
    return 2;  // undecided
}


/* ---------------- division (src/rnsdiv.cuh:128-174) ---------------- */
/* Reference-faithful cuda::rns_div on per-thread arrays: one power of two of
 * the quotient estimate per iteration, a full evaluation of the remainder
 * each time, MRC-based final correction.  Loop capped (kFlagIterCap). */
template <int N>
__device__ __noinline__ void div_ref(const Consts<N> &C, uint32_t *q, uint32_t *r, const uint32_t *x,
                                     const uint32_t *d, uint32_t &flags) {
    bool dz = true;
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        q[i] = 0;
        r[i] = x[i];
        dz &= d[i] == 0;
    }
    if (dz) { flags |= kFlagDivByZero; return; }
    Er dl, du, rl, ru;
    eval<N>(C, [&](int i) { return d[i]; }, dl, du, flags);
    eval<N>(C, [&](int i) { return r[i]; }, rl, ru, flags);
    const int cap = 2 * C.log2M + 64;
    int it = 0;
#pragma unroll 1
    while (er_ucmp(rl, du) >= 0) {
        if (++it > cap) { flags |= kFlagIterCap; return; }
        Er flq;
        flq.exp = rl.exp - du.exp;
        flq.frac = __ddiv_rd(rl.frac, du.frac);
        er_adjust(flq);
        if (flq.exp < 0 || flq.exp > C.log2M) { flags |= kFlagIterCap; return; }
        const uint32_t *pq = C.pow2 + (int64_t)flq.exp * N;
#pragma unroll 1
        for (int i = 0; i < N; i++) {
            uint32_t p = __ldg(pq + i), m = C.m[i];
            q[i] = addmod(q[i], p, m);
            r[i] = submod(r[i], mulmod_barrett(p, d[i], m, C.mu[i], C.b[i]), m);
        }
        eval<N>(C, [&](int i) { return r[i]; }, rl, ru, flags);
    }
    if (er_ucmp(ru, dl) >= 0) {
        uint32_t dmr[N], rmr[N];
        mrc_digits<N>(C, [&](int i) { return d[i]; }, dmr);
        mrc_digits<N>(C, [&](int i) { return r[i]; }, rmr);
        bool rged = true;
#pragma unroll 1
        for (int i = N - 1; i >= 0; i--) {
            if (rmr[i] < dmr[i]) { rged = false; break; }
            if (rmr[i] > dmr[i]) break;
        }
        if (rged) {
#pragma unroll 1
            for (int i = 0; i < N; i++) {
                q[i] = addmod(q[i], 1, C.m[i]);
                r[i] = submod(r[i], d[i], C.m[i]);
            }
        }
    }
}

/* ---------------- power-of-two scaling (src/rnsscal.cuh:134-235) ---------------- */
/* rns_rank_compute (checked=true, :134) / rns_rank_compute_fast (:168):
 * k with X = sum_i M_i c_i - k M, c_i = x_i w_i mod m_i. */
template <int N>
__device__ __forceinline__ uint32_t rank_ref(const Consts<N> &C, const uint32_t *x, const uint32_t *c, bool checked) {
    PTree<N, true> tu;
    PTree<N, false> tl;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        double dd = u32_to_double(c[i]);
        tu.push(i, __dmul_ru(dd, C.rru[i]));
        if (checked) tl.push(i, __dmul_rd(dd, C.rrd[i]));
    }
    double sumu = tu.total();
    if (!checked) return (uint32_t)__double2int_rz(sumu);
    double suml = tl.total();
    unsigned whl = __double2uint_rz(suml), whu = __double2uint_rz(sumu);
    if (whl == whu) return whl;
    uint32_t mr[N];
    mrc_digits<N>(C, [&](int i) { return x[i]; }, mr);
    return mr[N - 1] == 0 ? whu : whl;
}

/* make_scaling_step (:181): y = (x - (X mod 2^j)) * (2^j)^-1 */
template <int N>
__device__ __forceinline__ void scaling_step(const Consts<N> &C, uint32_t *y, uint32_t k, unsigned j,
                                             const uint32_t *x, const uint32_t *c) {
    const uint32_t mask = (j >= 32) ? 0xffffffffu : ((1u << j) - 1u);
    const uint32_t *hrow = C.mi_pow2 + (int64_t)(j - 1) * N;
    uint64_t acc = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) acc += (uint64_t)((__ldg(hrow + i) * c[i]) & mask);
    uint32_t res = (uint32_t)((acc - (uint64_t)k * __ldg(C.m_pow2 + j - 1)) & mask);
    const uint32_t *inv = C.pow2_inv + (int64_t)(j - 1) * N;
    const uint32_t *inv_sh = C.pow2_inv_sh + (int64_t)(j - 1) * N;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        uint32_t m = C.m[i];
        uint32_t rm = res % m;
        y[i] = mulmod_shoup(submod(x[i], rm, m), __ldg(inv + i), __ldg(inv_sh + i), m);
    }
}

/* rns_scale2pow with the host's rank choice in the last step (src/rnsscal.cuh:116):
 * the checked rank whenever that step acts on the unscaled input, which the
 * device twin (:232) inverts; this keeps results equal to floor(X / 2^D). */
template <int N>
__device__ __noinline__ void scale2pow_ref(const Consts<N> &C, uint32_t *res, const uint32_t *x, unsigned D) {
    uint32_t c[N], cur[N];
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) cur[i] = x[i];
    unsigned t = D / kScaleStep;
    bool first = true;
#pragma unroll 1
    while (t > 0) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) c[i] = mulmod_shoup(cur[i], C.w[i], C.w_sh[i], C.m[i]);
        uint32_t k = rank_ref<N>(C, cur, c, first);
        scaling_step<N>(C, cur, k, kScaleStep, cur, c);
        first = false;
        t--;
    }
    unsigned dr = D % kScaleStep;
    if (dr > 0) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) c[i] = mulmod_shoup(cur[i], C.w[i], C.w_sh[i], C.m[i]);
        uint32_t k = rank_ref<N>(C, cur, c, first);
        scaling_step<N>(C, cur, k, dr, cur, c);
    }
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) res[i] = cur[i];
}

/* ---------------- multiple-precision integers (src/mpint.cuh:318-503) ---------------- */

/* er_add_rd / er_add_ru (src/extrange.cuh:403/:423) */
template <bool UP>
__device__ __forceinline__ Er er_add_dir(Er x, Er y) {
    x.exp *= (x.frac != 0);
    y.exp *= (y.frac != 0);
    int dexp = (int)((x.exp - y.exp) * (x.frac != 0) * (y.frac != 0));
    Er r;
    double a, b;
    if (dexp > 0) {
        r.exp = x.exp; a = x.frac; b = scalbn(y.frac, -dexp);
    } else if (dexp < 0) {
        r.exp = y.exp; a = y.frac; b = scalbn(x.frac, dexp);
    } else {
        r.exp = (x.exp == 0) ? y.exp : x.exp; a = x.frac; b = y.frac;
    }
    r.frac = UP ? __dadd_ru(a, b) : __dadd_rd(a, b);
    er_adjust(r);
    return r;
}

/* ---- the same operations with the bit handling on the integer pipe ----
 * Sign tests, sign flips, the exponent renormalisation of er_adjust and
 * scalbn of a normal result are exact bit operations on the IEEE encoding;
 * on GB300 the FP64 pipe (a few operations per clock per SM) would otherwise
 * bound the mp_int kernels.  Only the directed-rounding addition itself stays
 * an FP64 instruction.  Results are bit-identical to the FP64 forms above. */
__device__ __forceinline__ bool dneg_i(double v) {  // v < 0 (false for -0)
    const uint64_t u = dbits(v);
    return (u >> 63) && (u << 1);
}
__device__ __forceinline__ bool dnz_i(double v) { return (dbits(v) << 1) != 0; }  // v != 0
__device__ __forceinline__ double dflip_i(double v, bool neg) {                   // neg ? -v : v
    return bitsd(dbits(v) ^ ((uint64_t)neg << 63));
}
/* scalbn(v, -d) for d >= 0: exact exponent arithmetic while the result stays
 * normal, the library call otherwise (a subnormal or zero result) */
__device__ __forceinline__ double scalbn_down_i(double v, int d) {
    const uint64_t u = dbits(v);
    const int e = (int)((u >> 52) & 0x7ff);
    if (e == 0x7ff || (e == 0 && !(u << 1))) return v;  // infinities, NaN, +-0 are unchanged
    if (e - d >= 1) return bitsd(u - ((uint64_t)d << 52));
    return scalbn(v, -d);  // a subnormal argument or result
}
/* er_adjust (src/extrange.cuh:366) on the integer pipe: the frac of a zero
 * keeps its sign, as the reference's multiplication by 0.0 does */
__device__ __forceinline__ void er_adjust_i(Er &x) {
    const uint64_t u = dbits(x.frac);
    if (u << 1) {
        x.exp = x.exp + (int64_t)((u & 0x7fffffffffffffffull) >> 52) - 1023;
        x.frac = bitsd((u & 0x800fffffffffffffull) | 0x3ff0000000000000ull);
    } else {
        x.exp = 0;
        x.frac = bitsd(u & 0x8000000000000000ull);
    }
}
template <bool UP>
__device__ __forceinline__ Er er_add_dir_i(Er x, Er y) {
    const bool xz = !dnz_i(x.frac), yz = !dnz_i(y.frac);
    if (xz) x.exp = 0;
    if (yz) y.exp = 0;
    const int dexp = (xz || yz) ? 0 : (int)(x.exp - y.exp);
    Er r;
    double a, b;
    if (dexp > 0) {
        r.exp = x.exp; a = x.frac; b = scalbn_down_i(y.frac, dexp);
    } else if (dexp < 0) {
        r.exp = y.exp; a = y.frac; b = scalbn_down_i(x.frac, -dexp);
    } else {
        r.exp = (x.exp == 0) ? y.exp : x.exp; a = x.frac; b = y.frac;
    }
    r.frac = UP ? __dadd_ru(a, b) : __dadd_rd(a, b);
    er_adjust_i(r);
    return r;
}
/* total order of doubles (not NaN) as unsigned keys */
__device__ __forceinline__ uint64_t dkey_i(double v) {
    const uint64_t u = dbits(v);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}
/* er_ucmp (src/extrange.cuh:597) with the double comparisons as key comparisons
 * (-0 and +0 compare equal there, as in the FP64 form) */
__device__ __forceinline__ int er_ucmp_i(const Er &x, const Er &y) {
    const uint64_t kx = dnz_i(x.frac) ? dkey_i(x.frac) : dkey_i(0.0), ky = dnz_i(y.frac) ? dkey_i(y.frac) : dkey_i(0.0);
    const int diff = (int)(x.exp - y.exp);
    if (diff == 0) return kx == ky ? 0 : (kx > ky ? 1 : -1);
    return (dnz_i(x.frac) && (diff > 0 || (diff < 0 && !dnz_i(y.frac)))) ? 1 : -1;
}
template <int N>
__device__ __forceinline__ uint32_t overflow_flags_i(const Consts<N> &C, const Er &low, const Er &upp) {
    if (upp.exp < -1 || er_ucmp_i(upp, C.inv_unit_low) <= 0) return 0;
    if (er_ucmp_i(low, C.inv_unit_upp) == 1) return kFlagOverflow;
    return kFlagMayOverflow;
}

/* er_md_rd / er_md_ru (src/extrange.cuh:557/:566) */
template <bool UP>
__device__ __forceinline__ Er er_md(const Er &x, const Er &y, const Er &z) {
    Er r;
    r.exp = x.exp + y.exp - z.exp;
    r.frac = UP ? __ddiv_ru(__dmul_ru(x.frac, y.frac), z.frac) : __ddiv_rd(__dmul_rd(x.frac, y.frac), z.frac);
    er_adjust(r);
    return r;
}

/* mpint_check_overflow (src/mpint.cuh:318) as flag bits */
template <int N>
__device__ __forceinline__ uint32_t overflow_flags(const Consts<N> &C, const Er &low, const Er &upp) {
    if (upp.exp < -1 || er_ucmp(upp, C.inv_unit_low) <= 0) return 0;
    if (er_ucmp(low, C.inv_unit_upp) == 1) return kFlagOverflow;
    return kFlagMayOverflow;
}

}  // namespace grns
