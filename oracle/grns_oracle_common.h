/*
 * ORACLE -- test infrastructure only.  CPU restatement of the reference
 * library (kisupov/grns) used as the checker for the GPU product and as the
 * timed CPU baseline.  Nothing in the product may link or call this code.
 *
 * Shared scalar primitives for the restatement:
 *   h_*  the reference HOST arithmetic: directed rounding simulated in
 *        round-to-nearest after Rump et al. "BoundNear1"
 *        (reference src/dinterval.cuh:25-136), no FMA contraction.
 *   d_*  the reference DEVICE arithmetic: the CUDA intrinsics __dadd_rd,
 *        __dmul_ru, __ddiv_rd ... are IEEE-754 correctly rounded operations
 *        in a fixed direction.  They are reproduced exactly in round-to-
 *        nearest with error-free transformations (TwoSum, FMA-based
 *        TwoProduct and division remainder) plus one nextafter step.
 * Build with -ffp-contract=off (aarch64 gcc would otherwise fuse x*y+z).
 */
#ifndef GRNS_ORACLE_COMMON_H
#define GRNS_ORACLE_COMMON_H

#include <math.h>
#include <stdint.h>
#include <string.h>

#define OR_MAXN 256
#define OR_T 30 /* RNS_P2_SCALING_THRESHOLD, reference src/params.h:22 */

typedef struct { double frac; long exp; } or_er;          /* er_float_t, src/types.cuh:13 */
typedef struct { or_er low, upp; } or_iv;                  /* interval_t, src/types.cuh:25 */

typedef struct {
    int n;
    int log2M;                 /* floor(log2 M): RNS_MODULI_PRODUCT_LOG2 convention */
    int m[OR_MAXN];            /* RNS_MODULI */
    int w[OR_MAXN];            /* RNS_PART_MODULI_PRODUCT_INVERSE: (M/m_i)^-1 mod m_i */
    double recip_rd[OR_MAXN];  /* RNS_MODULI_RECIP_RD = ddiv_rd(1, m_i), host rounding */
    double recip_ru[OR_MAXN];
    double acc;                /* RNS_EVAL_ACCURACY */
    int ref_factor;            /* RNS_EVAL_REF_FACTOR */
    or_iv unit, inv_unit;      /* RNS_EVAL_UNIT ~ 1/M, RNS_EVAL_INV_UNIT ~ 1-1/M */
    int *pow2;                 /* RNS_POW2[log2M+1][n] */
    int mrc_inv[OR_MAXN][OR_MAXN]; /* MRC_MULT_INV[i][j] = m_i^-1 mod m_j, j>i */
    int m_pow2_res[OR_T];      /* RNS_MODULI_PRODUCT_POW2_RESIDUES: M mod 2^(j+1) */
    int mi_pow2_res[OR_T][OR_MAXN]; /* RNS_PART_MODULI_PRODUCT_POW2_RESIDUES */
    int pow2_inv[OR_T][OR_MAXN];    /* RNS_POW2_INVERSE: (2^(j+1))^-1 mod m_i */
    int one[OR_MAXN];
} or_ctx;

/* ---------------- host (Rump BoundNear1) arithmetic ---------------- */
/* DBL_PHI1 = 2^-53 (1 + 2^-52), DBL_ETA = 2^-1074: src/bitwise.cuh:16-28 */
#define OR_PHI1 (0x1p-53 * (1.0 + 2.0 * 0x1p-53))
#define OR_ETA 0x1p-1074

static inline double h_fmac(double x, double y, double z) { return x * y + z; }
static inline double h_add_rd(double a, double b) { double c = a + b; return c - h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_add_ru(double a, double b) { double c = a + b; return c + h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_sub_rd(double a, double b) { double c = a - b; return c - h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_sub_ru(double a, double b) { double c = a - b; return c + h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_mul_rd(double a, double b) { double c = a * b; return c - h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_mul_ru(double a, double b) { double c = a * b; return c + h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_div_rd(double a, double b) { double c = a / b; return c - h_fmac(OR_PHI1, fabs(c), OR_ETA); }
static inline double h_div_ru(double a, double b) { double c = a / b; return c + h_fmac(OR_PHI1, fabs(c), OR_ETA); }

/* ---------------- device (IEEE directed) arithmetic, exact ---------------- */
static inline double d_add_rd(double a, double b) {
    double s = a + b, bb = s - a, e = (a - (s - bb)) + (b - bb);
    if (s == 0.0 && e == 0.0) return (a == 0.0 && b == 0.0 && !signbit(a) && !signbit(b)) ? 0.0 : -0.0;
    return e < 0.0 ? nextafter(s, -INFINITY) : s;
}
static inline double d_add_ru(double a, double b) {
    double s = a + b, bb = s - a, e = (a - (s - bb)) + (b - bb);
    if (s == 0.0 && e == 0.0) return (a == 0.0 && b == 0.0 && signbit(a) && signbit(b)) ? -0.0 : 0.0;
    return e > 0.0 ? nextafter(s, INFINITY) : s;
}
static inline double d_sub_rd(double a, double b) { return d_add_rd(a, -b); }
static inline double d_sub_ru(double a, double b) { return d_add_ru(a, -b); }
static inline double d_mul_rd(double a, double b) {
    double p = a * b, e = fma(a, b, -p);
    return e < 0.0 ? nextafter(p, -INFINITY) : p;
}
static inline double d_mul_ru(double a, double b) {
    double p = a * b, e = fma(a, b, -p);
    return e > 0.0 ? nextafter(p, INFINITY) : p;
}
static inline double d_div_rd(double a, double b) {
    double q = a / b, r = fma(-q, b, a);
    double s = (b > 0.0) ? r : -r; /* sign of (a/b - q) */
    return s < 0.0 ? nextafter(q, -INFINITY) : q;
}
static inline double d_div_ru(double a, double b) {
    double q = a / b, r = fma(-q, b, a);
    double s = (b > 0.0) ? r : -r;
    return s > 0.0 ? nextafter(q, INFINITY) : q;
}

/* ---------------- bit-level helpers, src/bitwise.cuh / src/extrange.cuh ---------------- */
static inline uint64_t or_bits(double x) { uint64_t u; memcpy(&u, &x, 8); return u; }
static inline double or_dbl(uint64_t u) { double x; memcpy(&x, &u, 8); return x; }

/* fast_scalbn, src/bitwise.cuh:75 */
static inline double or_fast_scalbn(double x, int n) {
    uint64_t u = or_bits(x) + ((uint64_t)(int64_t)n << 52);
    return or_dbl(u) * (double)(x != 0 && n >= -1023);
}

/* er_set_d, src/extrange.cuh:29 / :75 (identical on both paths) */
static inline void or_er_set_d(or_er *r, double x) {
    uint64_t u = or_bits(x);
    if (x != 0) {
        r->exp = (long)((u & ~((uint64_t)1 << 63)) >> 52) - 1023;
        u = (u & ((((uint64_t)1 << 52) - 1) | ((uint64_t)1 << 63))) | ((uint64_t)1023 << 52);
        r->frac = or_dbl(u);
    } else {
        r->exp = 0;
        r->frac = 0;
    }
}

/* er_adjust, src/extrange.cuh:116 / :366 */
static inline void or_er_adjust(or_er *x) {
    uint64_t u = or_bits(x->frac);
    x->exp = (x->exp + (long)((u & ~((uint64_t)1 << 63)) >> 52) - 1023) * (long)(x->frac != 0);
    u = (u & ((((uint64_t)1 << 52) - 1) | ((uint64_t)1 << 63))) | ((uint64_t)1023 << 52);
    x->frac = or_dbl(u) * (double)(x->frac != 0);
}

/* er_ucmp, src/extrange.cuh:347 / :597 */
static inline int or_er_ucmp(const or_er *x, const or_er *y) {
    int diff = (int)(x->exp - y->exp);
    if (diff == 0) return x->frac == y->frac ? 0 : (x->frac > y->frac ? 1 : -1);
    return (x->frac != 0 && (diff > 0 || (diff < 0 && y->frac == 0))) ? 1 : -1;
}

/* er_cmp, src/extrange.cuh:327 / :577 */
static inline int or_er_cmp(const or_er *x, const or_er *y) {
    int diff = (int)(x->exp - y->exp);
    if (diff == 0) return x->frac == y->frac ? 0 : (x->frac > y->frac ? 1 : -1);
    if (x->frac == 0) return y->frac > 0 ? -1 : 1;
    if (y->frac == 0) return x->frac > 0 ? 1 : -1;
    return ((diff > 0 && x->frac > 0) || (diff < 0 && y->frac < 0)) ? 1 : -1;
}

/* ---------------- ceil(log2 x) of the device refinement loop ----------------
 * The reference's GPU refinement (src/rnseval.cuh:236) evaluates
 * ceil(log2(sumu)) with CUDA's device log2, which is not exact at every power
 * of two.  The oracle uses the C library's log2 unless the caller supplies the
 * device's values for the exact inputs met (record mode collects them; the
 * override table, sorted by x, replays them).  Record/override use is
 * single-threaded. */
static double *or_l2_rec = 0;
static long or_l2_rec_n = 0, or_l2_rec_cap = 0;
static const double *or_l2_tab_x = 0;
static const int *or_l2_tab_c = 0;
static long or_l2_tab_n = 0;

static inline double or_ceil_log2_dev(double x) {
    if (or_l2_rec_cap && or_l2_rec_n < or_l2_rec_cap) or_l2_rec[or_l2_rec_n++] = x;
    if (or_l2_tab_n) {
        long lo = 0, hi = or_l2_tab_n - 1;
        while (lo <= hi) {
            long mid = (lo + hi) / 2;
            if (or_l2_tab_x[mid] == x) return (double)or_l2_tab_c[mid];
            if (or_l2_tab_x[mid] < x) lo = mid + 1; else hi = mid - 1;
        }
    }
    return ceil(log2(x));
}

/* ---------------- modular helpers ---------------- */
/* host mod_mul(x,y,m,d): FP reciprocal trick, may be non-canonical (src/modular.cuh:74) */
static inline int h_modmul_d(int x, int y, int m) {
    long r = (long)x * (long)y;
    double q = (double)r * (1.0 / m);
    int i = (int)q;
    return (int)(r - (long)i * (long)m);
}
/* host mod_add(x,y,m,d) (src/modular.cuh:29) */
static inline int h_modadd_d(int x, int y, int m) {
    long r = (long)x + (long)y;
    double q = (double)r * (1.0 / m);
    int i = (int)q;
    return (int)(r - (long)i * (long)m);
}
/* mod_psub (src/modular.cuh:52 / :112) and exact mod_mul (:62 / :122) */
static inline int or_modpsub(int x, int y, int m) { return (int)(((long)x - (long)y + (long)m) % (long)m); }
static inline int or_modmul(int x, int y, int m) { return (int)(((long)x * (long)y) % (long)m); }
static inline int or_modadd(int x, int y, int m) { return (int)(((long)x + (long)y) % (long)m); }

/* (unsigned int) of a double as gcc/x86-64 converts it (through a 64-bit
 * integer); only differs from saturating conversion for negative sums. */
static inline unsigned or_u32(double x) { return (unsigned)(long)x; }

/* mpint_check_overflow, src/mpint.cuh:142 / :318: 0 none, 1 "may have", 2 "has occurred" */
static int or_overflow(const or_ctx *c, const or_er *low, const or_er *upp) {
    if (upp->exp < -1 || or_er_ucmp(upp, &c->inv_unit.low) <= 0) return 0;
    if (or_er_ucmp(low, &c->inv_unit.upp) == 1) return 2;
    return 1;
}

/* er_md_rd/ru: host src/extrange.cuh:307/:316, device :557/:566 */
static void or_er_md(or_er *r, const or_er *x, const or_er *y, const or_er *z, int dev, int up) {
    r->exp = x->exp + y->exp - z->exp;
    if (dev) r->frac = up ? d_div_ru(d_mul_ru(x->frac, y->frac), z->frac) : d_div_rd(d_mul_rd(x->frac, y->frac), z->frac);
    else r->frac = up ? h_div_ru(h_mul_ru(x->frac, y->frac), z->frac) : h_div_rd(h_mul_rd(x->frac, y->frac), z->frac);
    or_er_adjust(r);
}

#endif
