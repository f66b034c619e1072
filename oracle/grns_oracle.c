/*
 * ORACLE -- test infrastructure only.  A CPU restatement of the reference
 * library kisupov/grns (header-only CUDA C++).  It serves two purposes:
 *   1. the checker for the GPU product (tests, smoke, bench parity), and
 *   2. the timed CPU baseline: the reference's HOST path (rns_eval_compute,
 *      rns_cmp, rns_div, rns_scale2pow, mpint_add/sub/mul) restated
 *      operation by operation, multithreaded with OpenMP.
 * The product never links or calls it.  It is pinned against the unmodified
 * reference compiled for the CPU (oracle/_ref, see oracle/ref/build_ref.py)
 * and against the golden vectors under tests/golden/.
 *
 * Constants follow rns_const_init (reference src/rnsbase.cuh:324-451)
 * without GMP/MPFR: M is only needed as its bit length and its top 53 bits
 * (MPFR rounds M down to 53 bits before computing 1/M), and every other table
 * is a product or an inverse modulo a 31-bit modulus or a power of two.
 */
#include <stdlib.h>
#include <stdio.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include "grns_oracle_common.h"

#define ON 4
#include "grns_oracle_n.h"
#undef ON
#define ON 5
#include "grns_oracle_n.h"
#undef ON
#define ON 6
#include "grns_oracle_n.h"
#undef ON
#define ON 7
#include "grns_oracle_n.h"
#undef ON
#define ON 8
#include "grns_oracle_n.h"
#undef ON
#define ON 9
#include "grns_oracle_n.h"
#undef ON
#define ON 10
#include "grns_oracle_n.h"
#undef ON
#define ON 11
#include "grns_oracle_n.h"
#undef ON
#define ON 12
#include "grns_oracle_n.h"
#undef ON
#define ON 13
#include "grns_oracle_n.h"
#undef ON
#define ON 14
#include "grns_oracle_n.h"
#undef ON
#define ON 15
#include "grns_oracle_n.h"
#undef ON
#define ON 16
#include "grns_oracle_n.h"
#undef ON
#define ON 32
#include "grns_oracle_n.h"
#undef ON
#define ON 64
#include "grns_oracle_n.h"
#undef ON
#define ON 128
#include "grns_oracle_n.h"
#undef ON
#define ON 256
#include "grns_oracle_n.h"
#undef ON

#define OR_SUPPORTED(n) (((n) >= 4 && (n) <= 16) || (n) == 32 || (n) == 64 || (n) == 128 || (n) == 256)

/* mod_inverse semantics (src/rnsbase.cuh:121/:156): the inverse in [0, m). */
static long or_inverse(long x, long m) {
    long a = ((x % m) + m) % m, b = m, x0 = 1, x1 = 0;
    while (b) {
        long q = a / b, t = a - q * b;
        a = b; b = t;
        t = x0 - q * x1; x0 = x1; x1 = t;
    }
    return ((x0 % m) + m) % m;
}

static long or_gcd(long a, long b) { while (b) { long t = a % b; a = b; b = t; } return a; }

/* Directed rounding of a rational 0 < p/q <= 1 (p, q < 2^54) to 53 bits,
 * returned the way mpfr_get_d_2exp reports it: frac in [0.5, 1) and exp. */
static void or_round_ratio(uint64_t p, uint64_t q, int up, double *frac, long *exp) {
    const unsigned __int128 lo = (unsigned __int128)1 << 52;
    int s = 0;
    while (((unsigned __int128)p << s) / q < lo) s++;
    unsigned __int128 num = (unsigned __int128)p << s;
    unsigned __int128 mant = num / q, rem = num % q;
    if (up && rem) mant += 1;
    if (mant == ((unsigned __int128)1 << 53)) { mant >>= 1; s -= 1; }
    *frac = ldexp((double)(uint64_t)mant, -53);
    *exp = 53 - s;
}

or_ctx *oracle_ctx_create(const int *moduli, int n) {
    if (!OR_SUPPORTED(n)) return NULL;
    for (int i = 0; i < n; i++) {
        if (moduli[i] < 3) return NULL;
        for (int j = 0; j < i; j++) if (or_gcd(moduli[i], moduli[j]) != 1) return NULL;
    }
    or_ctx *c = (or_ctx *)calloc(1, sizeof(or_ctx));
    c->n = n;
    for (int i = 0; i < n; i++) c->m[i] = moduli[i];
    /* M as little-endian 32-bit limbs */
    uint32_t M[OR_MAXN + 2];
    int len = 1;
    M[0] = 1;
    for (int i = 0; i < n; i++) {
        uint64_t carry = 0;
        for (int k = 0; k < len; k++) {
            uint64_t t = (uint64_t)M[k] * (uint32_t)moduli[i] + carry;
            M[k] = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) M[len++] = (uint32_t)carry;
    }
    int bitlen = 32 * (len - 1);
    for (uint32_t top = M[len - 1]; top; top >>= 1) bitlen++;
    c->log2M = bitlen - 1;
    /* top 53 bits of M (MPFR default precision, RNDD): T * 2^E */
    long E = bitlen > 53 ? bitlen - 53 : 0;
    uint64_t T = 0;
    for (int b = bitlen - 1; b >= (int)E; b--) T = (T << 1) | ((M[b / 32] >> (b % 32)) & 1u);
    for (int i = 0; i < n; i++) {
        c->one[i] = 1;
        /* M_i mod m_i and w_i = (M_i)^-1 mod m_i */
        long mi = 1;
        for (int j = 0; j < n; j++) if (j != i) mi = (mi * (moduli[j] % moduli[i])) % moduli[i];
        c->w[i] = (int)or_inverse(mi, moduli[i]);
        /* RNS_MODULI_RECIP_RD/RU = ddiv_rd/ru(1.0, m_i) with host (Rump) rounding */
        c->recip_rd[i] = h_div_rd(1.0, (double)moduli[i]);
        c->recip_ru[i] = h_div_ru(1.0, (double)moduli[i]);
    }
    /* RNS_EVAL_ACCURACY / RNS_EVAL_REF_FACTOR (src/rnsbase.cuh:389-391), same operation order */
    c->acc = 4 * pow(2.0, 1 - 53) * n * log2((double)n) * (1 + 0.0000001 / 2) / 0.0000001;
    c->ref_factor = (int)floor(log2(1 / (2 * c->acc)));
    /* RNS_EVAL_UNIT = [RD, RU](1/M53); RNS_EVAL_INV_UNIT = [RD, RU](1 - 1/M53) */
    or_round_ratio(1, T, 0, &c->unit.low.frac, &c->unit.low.exp);
    or_round_ratio(1, T, 1, &c->unit.upp.frac, &c->unit.upp.exp);
    c->unit.low.exp -= E;
    c->unit.upp.exp -= E;
    if (E == 0) {
        or_round_ratio(T - 1, T, 0, &c->inv_unit.low.frac, &c->inv_unit.low.exp);
        or_round_ratio(T - 1, T, 1, &c->inv_unit.upp.frac, &c->inv_unit.upp.exp);
    } else if (E == 1 && T == ((uint64_t)1 << 52)) { /* 1/M53 = 2^-53 exactly */
        c->inv_unit.low.frac = c->inv_unit.upp.frac = 1.0 - 0x1p-53;
        c->inv_unit.low.exp = c->inv_unit.upp.exp = 0;
    } else { /* 0 < 1/M53 < 2^-53 */
        c->inv_unit.low.frac = 1.0 - 0x1p-53; c->inv_unit.low.exp = 0;
        c->inv_unit.upp.frac = 0.5; c->inv_unit.upp.exp = 1;
    }
    /* RNS_POW2 */
    c->pow2 = (int *)malloc(sizeof(int) * (size_t)(c->log2M + 1) * n);
    for (int j = 0; j < n; j++) {
        long v = 1;
        for (int i = 0; i <= c->log2M; i++) {
            c->pow2[(long)i * n + j] = (int)v;
            v = (v * 2) % moduli[j];
        }
    }
    /* scaling tables (src/rnsbase.cuh:364-387) */
    for (int t = 0; t < OR_T; t++) {
        uint64_t mask = ((uint64_t)1 << (t + 1)) - 1, mm = 1;
        for (int i = 0; i < n; i++) mm = (mm * (uint64_t)moduli[i]) & mask;
        c->m_pow2_res[t] = (int)mm;
        for (int i = 0; i < n; i++) {
            uint64_t v = 1;
            for (int j = 0; j < n; j++) if (j != i) v = (v * (uint64_t)moduli[j]) & mask;
            c->mi_pow2_res[t][i] = (int)v;
            long p2 = 1;
            for (int k = 0; k <= t; k++) p2 = (p2 * 2) % moduli[i];
            c->pow2_inv[t][i] = (int)or_inverse(p2, moduli[i]);
        }
    }
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) c->mrc_inv[i][j] = j > i ? (int)or_inverse(moduli[i], moduli[j]) : 0;
    return c;
}

void oracle_ctx_destroy(or_ctx *c) {
    if (!c) return;
    free(c->pow2);
    free(c);
}

int oracle_n(const or_ctx *c) { return c->n; }
int oracle_log2(const or_ctx *c) { return c->log2M; }
int oracle_mpint_bytes(int n) { return ((4 * n + 4 + 7) / 8) * 8 + 32; }

void oracle_consts(const or_ctx *c, int *w, double *recip_rd, double *recip_ru, double *acc, int *ref_factor,
                   or_iv *unit, or_iv *inv_unit, int *mrc_inv, int *pow2, int *m_pow2_res, int *mi_pow2_res,
                   int *pow2_inv) {
    int n = c->n;
    memcpy(w, c->w, sizeof(int) * n);
    memcpy(recip_rd, c->recip_rd, sizeof(double) * n);
    memcpy(recip_ru, c->recip_ru, sizeof(double) * n);
    *acc = c->acc;
    *ref_factor = c->ref_factor;
    *unit = c->unit;
    *inv_unit = c->inv_unit;
    for (int i = 0; i < n; i++) for (int j = 0; j < n; j++) mrc_inv[i * n + j] = c->mrc_inv[i][j];
    memcpy(pow2, c->pow2, sizeof(int) * (size_t)(c->log2M + 1) * n);
    memcpy(m_pow2_res, c->m_pow2_res, sizeof(int) * OR_T);
    for (int t = 0; t < OR_T; t++) for (int i = 0; i < n; i++) {
        mi_pow2_res[t * n + i] = c->mi_pow2_res[t][i];
        pow2_inv[t * n + i] = c->pow2_inv[t][i];
    }
}

int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

#define OR_DISPATCH(c, CALL)                 \
    switch ((c)->n) {                        \
        case 4: CALL(4); break;          \
        case 5: CALL(5); break;          \
        case 6: CALL(6); break;          \
        case 7: CALL(7); break;          \
        case 8: CALL(8); break;          \
        case 9: CALL(9); break;          \
        case 10: CALL(10); break;        \
        case 11: CALL(11); break;        \
        case 12: CALL(12); break;        \
        case 13: CALL(13); break;        \
        case 14: CALL(14); break;        \
        case 15: CALL(15); break;        \
        case 16: CALL(16); break;        \
        case 32: CALL(32); break;        \
        case 64: CALL(64); break;        \
        case 128: CALL(128); break;      \
        case 256: CALL(256); break;      \
        default: break;                      \
    }

/* path: 0 = reference host path, 1 = reference device path (2 = host _fast, eval only) */
void oracle_eval(const or_ctx *c, const int *x, long N, or_iv *out, int path, int threads) {
#define C_(n) batch_eval_n##n(c, x, N, out, path, threads)
    OR_DISPATCH(c, C_)
#undef C_
}
void oracle_cmp(const or_ctx *c, const int *x, const int *y, long N, int *out, int path, int threads) {
#define C_(n) batch_cmp_n##n(c, x, y, N, out, path, threads)
    OR_DISPATCH(c, C_)
#undef C_
}
void oracle_div(const or_ctx *c, const int *x, const int *d, long N, int *q, int *r, int path, int fast, int threads) {
#define C_(n) batch_div_n##n(c, x, d, N, q, r, path, fast, threads)
    OR_DISPATCH(c, C_)
#undef C_
}
void oracle_scale2pow(const or_ctx *c, const int *x, const unsigned *D, long N, int *out, int path, int gpu_quirk, int threads) {
#define C_(n) batch_scale_n##n(c, x, D, N, out, path, gpu_quirk, threads)
    OR_DISPATCH(c, C_)
#undef C_
}
void oracle_mrc(const or_ctx *c, const int *x, long N, int *mr, int path) {
#define C_(n) batch_mrc_n##n(c, x, N, mr, path)
    OR_DISPATCH(c, C_)
#undef C_
}
void oracle_mpint(const or_ctx *c, int op, const void *x, const void *y, long N, void *out, int *flags, int path, int threads) {
#define C_(n) batch_mpint_n##n(c, op, x, y, N, out, flags, path, threads)
    OR_DISPATCH(c, C_)
#undef C_
}
long oracle_max(const or_ctx *c, const int *x, long N) {
    long r = -1;
#define C_(n) r = max_exact_n##n(c, x, N)
    OR_DISPATCH(c, C_)
#undef C_
    return r;
}

/* scalar directed-rounding primitives, exposed so tests can pin them */
double oracle_d_op(int op, double a, double b) {
    switch (op) {
        case 0: return d_add_rd(a, b);
        case 1: return d_add_ru(a, b);
        case 2: return d_mul_rd(a, b);
        case 3: return d_mul_ru(a, b);
        case 4: return d_div_rd(a, b);
        case 5: return d_div_ru(a, b);
        case 6: return d_sub_rd(a, b);
        default: return d_sub_ru(a, b);
    }
}

/* ceil(log2 x) override support for the device path (see or_ceil_log2_dev) */
void oracle_log2_record(double *buf, long cap) { or_l2_rec = buf; or_l2_rec_cap = cap; or_l2_rec_n = 0; }
long oracle_log2_recorded(void) { long n = or_l2_rec_n; or_l2_rec = 0; or_l2_rec_cap = 0; or_l2_rec_n = 0; return n; }
void oracle_log2_table(const double *xs, const int *cs, long n) { or_l2_tab_x = xs; or_l2_tab_c = cs; or_l2_tab_n = n; }
