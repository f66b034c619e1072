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

namespace grns {

typedef unsigned __int128 u128;

GRNS_HD uint32_t ldg_u32(const uint32_t *p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
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
#pragma unroll
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
#pragma unroll
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
#pragma unroll
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

template <int N, class Get>
GRNS_HD u128 fx96(const Consts<N> &C, Get get) {
    return fx96_k<N>(C, get, 0);
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

/* ---------------- normalised evaluation (for division) ---------------- */
struct Norm {
    u128 U;  // Z * 2^k / M * 2^96 lies in [U - E, U]; U >= 2^85 when kind == 0
    int k;
    int kind;  // 0 normal, 1 Z == 0, 2 Z > M (1 - E/2^96) (then U = 2^96, k = 0)
};

enum : uint32_t { kFxIterCap = 1u << 2 };

/* Certified enclosure of Z * 2^k / M with relative width < 2^-47, starting
 * from a magnification k0 known not to wrap (Z * 2^k0 < M). */
template <int N, class Get>
GRNS_HD Norm norm96(const Consts<N> &C, Get get, int k0, uint32_t &flags) {
    const u128 lower = ((u128)1) << 85;
    const u128 E = C.E;
    const int eb = bitlen64(C.E);
    int k = k0;
#pragma unroll 1
    for (int guard = 0; guard < 64; guard++) {
        if (k < 0 || k > C.log2M) break;
        u128 U = fx96_k<N>(C, get, k);
        if (U >= lower) return Norm{U, k, 0};
        if (U >= E) {
            k += 89 - bitlen128(U);
        } else if (k > 0) {
            k += 89 - eb;
        } else {
            uint32_t a[N];
            mrc_hd<N>(C, get, a);
            int t = N - 1;
            while (t >= 0 && a[t] == 0) t--;
            if (t < 0) return Norm{0, 0, 1};
            if (t == N - 1) return Norm{((u128)1) << 96, 0, 2};
            int bz = bitlen32(a[t] + 1) + (int)C.mrbits[t];
            k = C.log2M - bz - 7;
            if (k < 1) k = 1;
        }
    }
    flags |= kFxIterCap;
    return Norm{0, 0, 1};
}

/* ---------------- directed-rounding helpers for the quotient estimate ---------------- */

/* double <= v (v < 2^128), exact when v has <= 53 significant bits */
GRNS_HD double u128_to_double_rd(u128 v) {
    int bl = bitlen128(v);
    if (bl <= 53) return (double)(uint64_t)v;
    uint64_t top = (uint64_t)(v >> (bl - 53));
    return std::ldexp((double)top, bl - 53);
}
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

/* ---------------- division (exact q, r; the results of rns_div, src/rnsdiv.cuh:128) ---------------- */

/* 0: r < d certain, 1: r >= d certain, 2: undecided */
GRNS_HD int norm_order(const Norm &r, const Norm &d, uint64_t Eu) {
    const u128 E = Eu;
    const int sh = d.k - r.k;  // r/d = (Ur / Ud) * 2^sh
    if (sh >= 13) return 1;    // Ur - E >= 2^84 and Ud <= 2^96
    if (sh <= -13) return 0;
    u128 rl = r.U - E, ru = r.U, dl = d.U - E, du = d.U;
    if (sh >= 0) {
        rl <<= sh;
        ru <<= sh;
    } else {
        dl <<= -sh;
        du <<= -sh;
    }
    if (rl >= du) return 1;
    if (ru < dl) return 0;
    return 2;
}

/* pq residues of floor(F * 2^s) for a 53-bit F */
template <int N>
GRNS_HD bool floor_scaled_residues(const Consts<N> &C, uint64_t F, int s, uint32_t *pq, int &bits) {
    uint64_t base = F;
    int e = 0;
    if (s < 0) {
        base = (-s) >= 64 ? 0 : (F >> (-s));
    } else {
        e = s;
    }
    bits = base ? bitlen64(base) + e : 0;
    if (e > C.log2M) return false;  // cannot happen for a certified lower bound of r/d < M
    const uint32_t *p2 = C.pow2 + (int64_t)e * N;
    const uint32_t *p2s = C.pow2_sh + (int64_t)e * N;
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        uint32_t v;
        if (C.b[i] >= 27) {  /* base < 2^53: hi * (2^32 mod m) + lo < 2^54 <= 2^(2b), one Barrett step */
            uint64_t p = (uint64_t)(uint32_t)(base >> 32) * C.t32[i] + (uint32_t)base;
            uint32_t t = (uint32_t)(p >> (C.b[i] - 1));
            uint32_t q = (uint32_t)(((uint64_t)t * C.mu[i]) >> (C.b[i] + 1));
            uint32_t r = (uint32_t)p - q * C.m[i];
            r = umin32(r, r - C.m[i]);
            v = umin32(r, r - C.m[i]);
        } else {
            v = reduce64<N>(C, i, base);
        }
        pq[i] = e ? mulmod_shoup(v, ldg_u32(p2 + i), ldg_u32(p2s + i), C.m[i]) : v;
    }
    return true;
}

template <int N>
GRNS_HD void div_fast(const Consts<N> &C, uint32_t *q, uint32_t *r, const uint32_t *x, const uint32_t *d,
                      uint32_t &flags) {
    bool dz = true;
#pragma unroll 1
    for (int i = 0; i < N; i++) {
        q[i] = 0;
        r[i] = x[i];
        dz &= d[i] == 0;
    }
    if (dz) {
        flags |= 1u << 1;  // division by zero
        return;
    }
    auto gd = [&](int i) { return d[i]; };
    auto gr = [&](int i) { return r[i]; };
    Norm nd = norm96<N>(C, gd, 0, flags);
    if (nd.kind == 2) {  // d > M (1 - 2^-59): the quotient is 0 or 1
        if (cmp_exact<N>(C, gr, gd) >= 0) {
#pragma unroll 1
            for (int i = 0; i < N; i++) {
                q[i] = 1;
                r[i] = submod(r[i], d[i], C.m[i]);
            }
        }
        return;
    }
    const int bud = bitlen128(nd.U);
    int kr = 0;
    const int cap = C.log2M / 40 + 12;
    uint32_t pq[N];
#pragma unroll 1
    for (int it = 0;; it++) {
        if (it > cap) {
            flags |= kFxIterCap;
            return;
        }
        bool rz = true;
#pragma unroll 1
        for (int i = 0; i < N; i++) rz &= r[i] == 0;
        if (rz) return;
        Norm nr = norm96<N>(C, gr, kr, flags);
        if (nr.kind == 1) return;
        int ord = norm_order(nr, nd, C.E);
        if (ord == 0) return;
        int g;
        if (ord == 2) {
            if (cmp_exact<N>(C, gr, gd) < 0) return;
#pragma unroll 1
            for (int i = 0; i < N; i++) pq[i] = 1;
            g = 1;
        } else {
            double a = u128_to_double_rd(nr.U - (u128)C.E);
            double b = u128_to_double_ru(nd.U);
            double ratio = ddiv_rd_hd(a, b);  // <= (Ur - E) / Ud
            int ex;
            double fr = std::frexp(ratio, &ex);  // ratio = fr * 2^ex, fr in [0.5, 1)
            uint64_t F = (uint64_t)std::ldexp(fr, 53);
            int bits;
            if (!floor_scaled_residues<N>(C, F, ex - 53 + (nd.k - nr.k), pq, bits)) {
                flags |= kFxIterCap;
                return;
            }
            if (bits == 0) {
#pragma unroll 1
                for (int i = 0; i < N; i++) pq[i] = 1;
                bits = 1;
            }
            g = (bits > 44 ? bits - 44 : 0) + 1;
        }
#pragma unroll 1
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i];
            q[i] = addmod(q[i], pq[i], m);
            r[i] = submod(r[i], mulmod_barrett(pq[i], d[i], m, C.mu[i], C.b[i]), m);
        }
        kr = nd.k + 89 - g - bud;
        if (kr < 0) kr = 0;
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

/* one step of make_scaling_step (:181): y = (x - (X mod 2^j)) * (2^j)^-1 */
template <int N>
GRNS_HD void scaling_step_hd(const Consts<N> &C, uint32_t *y, uint32_t k, unsigned j, const uint32_t *x,
                             const uint32_t *c) {
    const uint32_t mask = (1u << j) - 1u;
    const uint32_t *hrow = C.mi_pow2 + (int64_t)(j - 1) * N;
    uint64_t acc = 0;
#pragma unroll
    for (int i = 0; i < N; i++) acc += (uint64_t)((ldg_u32(hrow + i) * c[i]) & mask);
    uint32_t res = (uint32_t)((acc - (uint64_t)k * ldg_u32(C.m_pow2 + j - 1)) & mask);
    const uint32_t *inv = C.pow2_inv + (int64_t)(j - 1) * N;
    const uint32_t *inv_sh = C.pow2_inv_sh + (int64_t)(j - 1) * N;
#pragma unroll
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i];
        uint32_t rm = reduce32<N>(C, i, res);
        y[i] = mulmod_shoup(submod(x[i], rm, m), ldg_u32(inv + i), ldg_u32(inv_sh + i), m);
    }
}

template <int N>
GRNS_HD void scale_fast(const Consts<N> &C, uint32_t *res, const uint32_t *x, unsigned D) {
    uint32_t cur[N], c[N];
#pragma unroll
    for (int i = 0; i < N; i++) cur[i] = x[i];
    unsigned t = D / kScaleStep, dr = D % kScaleStep;
    bool small = false;
#pragma unroll 1
    for (unsigned step = 0; step < t + (dr ? 1u : 0u); step++) {
        const unsigned j = step < t ? (unsigned)kScaleStep : dr;
#pragma unroll
        for (int i = 0; i < N; i++) c[i] = mulmod_shoup(cur[i], C.w[i], C.w_sh[i], C.m[i]);
        uint32_t k = rank_fast<N>(C, cur, c, small);
        scaling_step_hd<N>(C, cur, k, j, cur, c);
        small = true;
    }
#pragma unroll
    for (int i = 0; i < N; i++) res[i] = cur[i];
}

}  // namespace grns
