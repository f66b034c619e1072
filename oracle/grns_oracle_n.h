/*
 * ORACLE -- test infrastructure only (see grns_oracle_common.h).
 * Per-moduli-count core, included once per supported n with ON defined, so
 * loops have compile-time trip counts like the reference's template-unrolled
 * code.  Every function cites the reference function it restates
 * (paths relative to the kisupov/grns checkout).
 */
#define OR_CAT2(a, b) a##_n##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OFN(name) OR_CAT(name, ON)

/* Fixed pairwise tree of the reference: psum_rd/psum_ru dispatch
 * (src/pairwise.cuh:384-468 host, :837-918 device).  For L >= 4 the tree
 * spans K = 2*2^floor(log2 L) leaves; absent right subtrees contribute a
 * literal 0 through one more addition (which widens the bound on the host,
 * and is exact on the device).  L == 3 is summed sequentially. */
#define OR_DEFINE_TREE(NAME, ADD)                                                   \
    static inline double NAME(const double *x) {                                    \
        const int L = ON;                                                           \
        if (L == 1) return x[0];                                                    \
        if (L == 2) return ADD(x[0], x[1]);                                         \
        if (L == 3) return ADD(ADD(x[0], x[1]), x[2]);                              \
        int K = 8;                                                                  \
        while (K <= L) K <<= 1;                                                     \
        double v[ON];                                                               \
        int live = 0;                                                               \
        for (int j = 0; 2 * j < L; j++) {                                           \
            v[j] = ADD(x[2 * j], (2 * j + 1 < L) ? x[2 * j + 1] : 0.0);             \
            live++;                                                                 \
        }                                                                           \
        for (int nodes = K / 2; nodes > 1; nodes >>= 1) {                           \
            int nlive = 0;                                                          \
            for (int j = 0; 2 * j < live; j++) {                                    \
                v[j] = ADD(v[2 * j], (2 * j + 1 < live) ? v[2 * j + 1] : 0.0);      \
                nlive++;                                                            \
            }                                                                       \
            live = nlive;                                                           \
        }                                                                           \
        return v[0];                                                                \
    }

OR_DEFINE_TREE(OFN(tree_h_rd), h_add_rd)
OR_DEFINE_TREE(OFN(tree_h_ru), h_add_ru)
OR_DEFINE_TREE(OFN(tree_d_rd), d_add_rd)
OR_DEFINE_TREE(OFN(tree_d_ru), d_add_ru)

/* The n-threaded schedule's sums (cuda::block_reduce_sum_rd/ru,
 * src/pairwise.cuh:969/:984, over warp_reduce_sum_rd/ru :932/:939): inside a
 * warp, lane l adds lane l + 16, then l + 8, 4, 2, 1 (shuffles down), so lane 0
 * holds ((v0 + v16) + (v8 + v24)) + ...; with n = 64 the two warp sums are
 * then reduced the same way with zeros in the other lanes, which is s0 + s1.
 * For n < 32 the reference's shuffles read lanes that do not exist
 * (undefined); here, as in the device header, absent lanes are skipped. */
static double OFN(warp_tree)(const double *v, int lanes, int up) {
    double a[32], b[32];
    for (int l = 0; l < 32; l++) a[l] = l < lanes ? v[l] : 0.0;
    for (int off = 16; off > 0; off >>= 1) {
        for (int l = 0; l < 32; l++)
            b[l] = (l + off < lanes) ? (up ? d_add_ru(a[l], a[l + off]) : d_add_rd(a[l], a[l + off])) : a[l];
        for (int l = 0; l < 32; l++) a[l] = b[l];
    }
    return a[0];
}
static double OFN(ptree_d)(const double *v, int up) {
    if (ON <= 32) return OFN(warp_tree)(v, ON, up);
    double w[32];
    const int warps = ON / 32;
    for (int j = 0; j < warps; j++) w[j] = OFN(warp_tree)(v + 32 * j, 32, up);
    return OFN(warp_tree)(w, warps, up);
}

/* ---------------- mixed-radix conversion, src/mrc.cuh:31 (host) / :101 (device) ---------------- */
static inline void OFN(mrc_h)(const or_ctx *c, int *mr, const int *x) {
    for (int i = 0; i < ON; i++) {
        mr[i] = x[i];
        for (int j = 0; j < i; j++) {
            if (mr[i] < mr[j]) mr[i] = (int)((long)c->m[i] - (long)mr[j] + (long)mr[i]);
            else mr[i] = mr[i] - mr[j];
            mr[i] = or_modmul(mr[i], c->mrc_inv[j][i], c->m[i]);
        }
    }
}
static inline void OFN(mrc_d)(const or_ctx *c, int *mr, const int *x) {
    for (int i = 0; i < ON; i++) {
        mr[i] = x[i];
        for (int j = 0; j < i; j++) {
            if (mr[i] < mr[j]) mr[i] = or_modpsub(mr[i], mr[j], c->m[i]);
            else mr[i] = mr[i] - mr[j];
            mr[i] = or_modmul(mr[i], c->mrc_inv[j][i], c->m[i]);
        }
    }
}
/* mrs_cmp, src/mrc.cuh:13 / :83 */
static inline int OFN(mrs_cmp)(const int *a, const int *b) {
    for (int i = ON - 1; i >= 0; i--) {
        if (a[i] > b[i]) return 1;
        if (b[i] > a[i]) return -1;
    }
    return 0;
}

/* ---------------- interval evaluation ---------------- */
/* host rns_eval_compute, src/rnseval.cuh:29-102 */
static void OFN(eval_h)(const or_ctx *c, or_iv *out, const int *x) {
    int s[ON], mrd[ON], mr = -1;
    double fl[ON], fu[ON];
    int zero = 1;
    for (int i = 0; i < ON; i++) zero &= (x[i] == 0);
    if (zero) { out->low.frac = out->upp.frac = 0; out->low.exp = out->upp.exp = 0; return; }
    for (int i = 0; i < ON; i++) s[i] = h_modmul_d(x[i], c->w[i], c->m[i]);
    for (int i = 0; i < ON; i++) {
        fl[i] = h_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = h_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_h_rd)(fl), sumu = OFN(tree_h_ru)(fu);
    unsigned whl = or_u32(suml), whu = or_u32(sumu);
    suml = suml - whl;
    sumu = sumu - whu;
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    if (whl != whu) { OFN(mrc_h)(c, mrd, x); mr = mrd[ON - 1]; }
    if (mr > 0) { out->upp = c->inv_unit.upp; return; }
    if (mr == 0) out->low = c->unit.low;
    if (sumu >= c->acc) return;
    int K = 0;
    while (sumu < c->acc) {
        double a = -(ceil(log2(sumu)) + 1);
        int k = (int)(a > c->ref_factor ? a : (double)c->ref_factor);
        const int *p2 = c->pow2 + (long)k * ON;
        for (int i = 0; i < ON; i++) s[i] = h_modmul_d(s[i], p2[i], c->m[i]);
        for (int i = 0; i < ON; i++) fu[i] = h_div_ru((double)s[i], (double)c->m[i]);
        sumu = OFN(tree_h_ru)(fu);
        sumu -= or_u32(sumu);
        K += k;
    }
    for (int i = 0; i < ON; i++) fl[i] = h_div_rd((double)s[i], (double)c->m[i]);
    suml = OFN(tree_h_rd)(fl);
    suml -= or_u32(suml);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    out->low.exp -= K;
    out->upp.exp -= K;
}

/* host rns_eval_compute_fast, src/rnseval.cuh:112-167 */
static void OFN(eval_fast_h)(const or_ctx *c, or_iv *out, const int *x) {
    int s[ON];
    double fl[ON], fu[ON];
    int zero = 1;
    for (int i = 0; i < ON; i++) zero &= (x[i] == 0);
    if (zero) { out->low.frac = out->upp.frac = 0; out->low.exp = out->upp.exp = 0; return; }
    for (int i = 0; i < ON; i++) s[i] = h_modmul_d(x[i], c->w[i], c->m[i]);
    for (int i = 0; i < ON; i++) {
        fl[i] = h_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = h_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_h_rd)(fl), sumu = OFN(tree_h_ru)(fu);
    suml -= or_u32(suml);
    sumu -= or_u32(sumu);
    if (sumu >= c->acc) { or_er_set_d(&out->low, suml); or_er_set_d(&out->upp, sumu); return; }
    int K = 0;
    while (sumu < c->acc) {
        double a = -(ceil(log2(sumu)) + 1);
        int k = (int)(a > c->ref_factor ? a : (double)c->ref_factor);
        const int *p2 = c->pow2 + (long)k * ON;
        for (int i = 0; i < ON; i++) s[i] = h_modmul_d(s[i], p2[i], c->m[i]);
        for (int i = 0; i < ON; i++) fu[i] = h_div_ru((double)s[i], (double)c->m[i]);
        sumu = OFN(tree_h_ru)(fu);
        sumu -= or_u32(sumu);
        K += k;
    }
    for (int i = 0; i < ON; i++) fl[i] = h_div_rd((double)s[i], (double)c->m[i]);
    suml = OFN(tree_h_rd)(fl);
    suml -= or_u32(suml);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    out->low.exp -= K;
    out->upp.exp -= K;
}

/* device cuda::rns_eval_compute, src/rnseval.cuh:182-256 */
static void OFN(eval_d)(const or_ctx *c, or_iv *out, const int *x) {
    int s[ON], mrd[ON], mr = -1;
    double fl[ON], fu[ON];
    for (int i = 0; i < ON; i++) s[i] = or_modmul(x[i], c->w[i], c->m[i]);
    for (int i = 0; i < ON; i++) {
        fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_d_rd)(fl), sumu = OFN(tree_d_ru)(fu);
    if (suml == 0 && sumu == 0) { out->low.frac = out->upp.frac = 0; out->low.exp = out->upp.exp = 0; return; }
    unsigned whl = (unsigned)suml, whu = (unsigned)sumu;
    suml = d_sub_rd(suml, (double)whl);
    sumu = d_sub_ru(sumu, (double)whu);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    if (whl != whu) { OFN(mrc_d)(c, mrd, x); mr = mrd[ON - 1]; }
    if (mr > 0) { out->upp = c->inv_unit.upp; return; }
    if (mr == 0) out->low = c->unit.low;
    if (sumu >= c->acc) return;
    int K = 0;
    while (sumu < c->acc) {
        double a = -(or_ceil_log2_dev(sumu) + 1);
        int k = (int)(a > c->ref_factor ? a : (double)c->ref_factor);
        const int *p2 = c->pow2 + (long)k * ON;
        for (int i = 0; i < ON; i++) s[i] = or_modmul(s[i], p2[i], c->m[i]);
        for (int i = 0; i < ON; i++) fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
        sumu = OFN(tree_d_ru)(fu);
        sumu = d_sub_ru(sumu, (double)(unsigned)sumu);
        K += k;
    }
    for (int i = 0; i < ON; i++) fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
    suml = OFN(tree_d_rd)(fl);
    suml = d_sub_rd(suml, (double)(unsigned)suml);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    out->low.exp -= K;
    out->upp.exp -= K;
}

/* device cuda::rns_eval_compute_fast, src/rnseval.cuh:266-322: the device
 * algorithm without the mixed-radix ambiguity step */
static void OFN(eval_fast_d)(const or_ctx *c, or_iv *out, const int *x) {
    int s[ON];
    double fl[ON], fu[ON];
    for (int i = 0; i < ON; i++) s[i] = or_modmul(x[i], c->w[i], c->m[i]);
    for (int i = 0; i < ON; i++) {
        fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_d_rd)(fl), sumu = OFN(tree_d_ru)(fu);
    if (suml == 0 && sumu == 0) { out->low.frac = out->upp.frac = 0; out->low.exp = out->upp.exp = 0; return; }
    suml = d_sub_rd(suml, (double)(unsigned)suml);
    sumu = d_sub_ru(sumu, (double)(unsigned)sumu);
    if (sumu >= c->acc) { or_er_set_d(&out->low, suml); or_er_set_d(&out->upp, sumu); return; }
    int K = 0;
    while (sumu < c->acc) {
        double a = -(or_ceil_log2_dev(sumu) + 1);
        int k = (int)(a > c->ref_factor ? a : (double)c->ref_factor);
        const int *p2 = c->pow2 + (long)k * ON;
        for (int i = 0; i < ON; i++) s[i] = or_modmul(s[i], p2[i], c->m[i]);
        for (int i = 0; i < ON; i++) fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
        sumu = OFN(tree_d_ru)(fu);
        sumu = d_sub_ru(sumu, (double)(unsigned)sumu);
        K += k;
    }
    for (int i = 0; i < ON; i++) fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
    suml = OFN(tree_d_rd)(fl);
    suml = d_sub_rd(suml, (double)(unsigned)suml);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    out->low.exp -= K;
    out->upp.exp -= K;
}

/* device cuda::rns_eval_compute_parallel, src/rnseval.cuh:332-418: the
 * serial algorithm with the n-threaded schedule's sums (ptree_d) */
static void OFN(eval_dpar)(const or_ctx *c, or_iv *out, const int *x) {
    int s[ON], mrd[ON], mr = -1;
    double fl[ON], fu[ON];
    for (int i = 0; i < ON; i++) s[i] = or_modmul(x[i], c->w[i], c->m[i]);
    for (int i = 0; i < ON; i++) {
        fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(ptree_d)(fl, 0), sumu = OFN(ptree_d)(fu, 1);
    if (suml == 0 && sumu == 0) { out->low.frac = out->upp.frac = 0; out->low.exp = out->upp.exp = 0; return; }
    unsigned whl = (unsigned)suml, whu = (unsigned)sumu;
    suml = d_sub_rd(suml, (double)whl);
    sumu = d_sub_ru(sumu, (double)whu);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    if (whl != whu) { OFN(mrc_d)(c, mrd, x); mr = mrd[ON - 1]; }
    if (mr > 0) { out->upp = c->inv_unit.upp; return; }
    if (mr == 0) out->low = c->unit.low;
    if (sumu >= c->acc) return;
    int K = 0;
    while (sumu < c->acc) {
        double a = -(or_ceil_log2_dev(sumu) + 1);
        int k = (int)(a > c->ref_factor ? a : (double)c->ref_factor);
        const int *p2 = c->pow2 + (long)k * ON;
        for (int i = 0; i < ON; i++) s[i] = or_modmul(s[i], p2[i], c->m[i]);
        for (int i = 0; i < ON; i++) fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
        sumu = OFN(ptree_d)(fu, 1);
        sumu = d_sub_ru(sumu, (double)(unsigned)sumu);
        K += k;
    }
    for (int i = 0; i < ON; i++) fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
    suml = OFN(ptree_d)(fl, 0);
    suml = d_sub_rd(suml, (double)(unsigned)suml);
    or_er_set_d(&out->low, suml);
    or_er_set_d(&out->upp, sumu);
    out->low.exp -= K;
    out->upp.exp -= K;
}

/* ---------------- comparison ---------------- */
static int OFN(equal)(const int *x, const int *y) {
    for (int i = 0; i < ON; i++) if (x[i] != y[i]) return 0;
    return 1;
}
/* host rns_cmp, src/rnscmp.cuh:20-39 */
static int OFN(cmp_h)(const or_ctx *c, const int *x, const int *y) {
    or_iv ex, ey;
    OFN(eval_h)(c, &ex, x);
    OFN(eval_h)(c, &ey, y);
    if (or_er_ucmp(&ex.low, &ey.upp) > 0) return 1;
    if (or_er_ucmp(&ey.low, &ex.upp) > 0) return -1;
    if (OFN(equal)(x, y)) return 0;
    int mx[ON], my[ON];
    OFN(mrc_h)(c, mx, x);
    OFN(mrc_h)(c, my, y);
    return OFN(mrs_cmp)(mx, my);
}
/* device cuda::rns_cmp, src/rnscmp.cuh:55-74 */
static int OFN(cmp_d)(const or_ctx *c, const int *x, const int *y) {
    or_iv ex, ey;
    OFN(eval_d)(c, &ex, x);
    OFN(eval_d)(c, &ey, y);
    if (or_er_ucmp(&ex.low, &ey.upp) > 0) return 1;
    if (or_er_ucmp(&ey.low, &ex.upp) > 0) return -1;
    if (OFN(equal)(x, y)) return 0;
    int mx[ON], my[ON];
    OFN(mrc_d)(c, mx, x);
    OFN(mrc_d)(c, my, y);
    return OFN(mrs_cmp)(mx, my);
}

/* ---------------- division ---------------- */
/* host rns_div (fast=0, src/rnsdiv.cuh:19-61) and rns_div_fast (fast=1, :67-114) */
static void OFN(div_h)(const or_ctx *c, int *q, int *r, const int *x, const int *d, int fast) {
    int pq[ON];
    or_er flq;
    or_iv dev_, rev;
    for (int i = 0; i < ON; i++) { q[i] = 0; r[i] = x[i]; }
    OFN(eval_h)(c, &dev_, d);
    OFN(eval_h)(c, &rev, r);
    while (or_er_ucmp(&rev.low, &dev_.upp) >= 0) {
        flq.exp = rev.low.exp - dev_.upp.exp;
        flq.frac = h_div_rd(rev.low.frac, dev_.upp.frac);
        or_er_adjust(&flq);
        if (!fast) {
            /* the reference reads RNS_POW2[flq.exp]; exp < 0 would read outside the table */
            if (flq.exp < 0 || flq.exp > c->log2M) return;
            memcpy(pq, c->pow2 + (long)flq.exp * ON, sizeof(pq));
        } else {
            for (int i = 0; i < ON; i++) pq[i] = 0;
            while (flq.exp >= 0 && flq.frac > 0) {
                if (flq.exp > c->log2M) return;
                const int *p2 = c->pow2 + (long)flq.exp * ON;
                for (int i = 0; i < ON; i++) pq[i] = h_modadd_d(pq[i], p2[i], c->m[i]);
                flq.frac = h_sub_rd(flq.frac, 1.0);
                or_er_adjust(&flq);
            }
        }
        for (int i = 0; i < ON; i++) q[i] = h_modadd_d(q[i], pq[i], c->m[i]);
        for (int i = 0; i < ON; i++) pq[i] = h_modmul_d(pq[i], d[i], c->m[i]);
        for (int i = 0; i < ON; i++) r[i] = or_modpsub(r[i], pq[i], c->m[i]);
        OFN(eval_h)(c, &rev, r);
    }
    if (or_er_ucmp(&rev.upp, &dev_.low) >= 0) {
        int dmr[ON], rged = 1;
        OFN(mrc_h)(c, dmr, d);
        OFN(mrc_h)(c, pq, r);
        for (int i = ON - 1; i >= 0; i--) {
            if (pq[i] < dmr[i]) { rged = 0; break; }
            else if (pq[i] > dmr[i]) break;
        }
        if (rged) {
            for (int i = 0; i < ON; i++) q[i] = h_modadd_d(q[i], 1, c->m[i]);
            for (int i = 0; i < ON; i++) r[i] = or_modpsub(r[i], d[i], c->m[i]);
        }
    }
}

/* device cuda::rns_div (fast=0, src/rnsdiv.cuh:128-174) / rns_div_fast (fast=1, :180-233) */
static void OFN(div_d)(const or_ctx *c, int *q, int *r, const int *x, const int *d, int fast) {
    int pq[ON];
    or_er flq;
    or_iv dev_, rev;
    for (int i = 0; i < ON; i++) { q[i] = 0; r[i] = x[i]; }
    OFN(eval_d)(c, &dev_, d);
    OFN(eval_d)(c, &rev, r);
    while (or_er_ucmp(&rev.low, &dev_.upp) >= 0) {
        flq.exp = rev.low.exp - dev_.upp.exp;
        flq.frac = d_div_rd(rev.low.frac, dev_.upp.frac);
        or_er_adjust(&flq);
        if (!fast) {
            if (flq.exp < 0 || flq.exp > c->log2M) return;
            memcpy(pq, c->pow2 + (long)flq.exp * ON, sizeof(pq));
        } else {
            for (int i = 0; i < ON; i++) pq[i] = 0;
            while (flq.exp >= 0 && flq.frac > 0) {
                if (flq.exp > c->log2M) return;
                const int *p2 = c->pow2 + (long)flq.exp * ON;
                for (int i = 0; i < ON; i++) pq[i] = or_modadd(pq[i], p2[i], c->m[i]);
                flq.frac = d_sub_rd(flq.frac, 1.0);
                or_er_adjust(&flq);
            }
        }
        for (int i = 0; i < ON; i++) q[i] = or_modadd(q[i], pq[i], c->m[i]);
        for (int i = 0; i < ON; i++) pq[i] = or_modmul(pq[i], d[i], c->m[i]);
        for (int i = 0; i < ON; i++) r[i] = or_modpsub(r[i], pq[i], c->m[i]);
        OFN(eval_d)(c, &rev, r);
    }
    if (or_er_ucmp(&rev.upp, &dev_.low) >= 0) {
        int dmr[ON], rged = 1;
        OFN(mrc_d)(c, dmr, d);
        OFN(mrc_d)(c, pq, r);
        for (int i = ON - 1; i >= 0; i--) {
            if (pq[i] < dmr[i]) { rged = 0; break; }
            else if (pq[i] > dmr[i]) break;
        }
        if (rged) {
            for (int i = 0; i < ON; i++) {
                q[i] = or_modadd(q[i], 1, c->m[i]);
                r[i] = or_modpsub(r[i], d[i], c->m[i]);
            }
        }
    }
}

/* ---------------- power-of-two scaling ---------------- */
/* rns_rank_compute, src/rnsscal.cuh:17 (host) / :134 (device) */
static int OFN(rank_h)(const or_ctx *c, const int *x, const int *s) {
    double fl[ON], fu[ON];
    for (int i = 0; i < ON; i++) {
        fl[i] = h_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = h_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_h_rd)(fl), sumu = OFN(tree_h_ru)(fu);
    unsigned whl = or_u32(suml), whu = or_u32(sumu);
    if (whl == whu) return (int)whl;
    int mrd[ON];
    OFN(mrc_h)(c, mrd, x);
    return mrd[ON - 1] == 0 ? (int)whu : (int)whl;
}
static int OFN(rank_d)(const or_ctx *c, const int *x, const int *s) {
    double fl[ON], fu[ON];
    for (int i = 0; i < ON; i++) {
        fl[i] = d_mul_rd((double)s[i], c->recip_rd[i]);
        fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
    }
    double suml = OFN(tree_d_rd)(fl), sumu = OFN(tree_d_ru)(fu);
    unsigned whl = (unsigned)suml, whu = (unsigned)sumu;
    if (whl == whu) return (int)whl;
    int mrd[ON];
    OFN(mrc_d)(c, mrd, x);
    return mrd[ON - 1] == 0 ? (int)whu : (int)whl;
}
/* rns_rank_compute_fast, src/rnsscal.cuh:53 / :168 */
static int OFN(rank_fast_h)(const or_ctx *c, const int *s) {
    double fu[ON];
    for (int i = 0; i < ON; i++) fu[i] = h_mul_ru((double)s[i], c->recip_ru[i]);
    return (int)OFN(tree_h_ru)(fu);
}
static int OFN(rank_fast_d)(const or_ctx *c, const int *s) {
    double fu[ON];
    for (int i = 0; i < ON; i++) fu[i] = d_mul_ru((double)s[i], c->recip_ru[i]);
    return (int)OFN(tree_d_ru)(fu);
}
/* make_scaling_step, src/rnsscal.cuh:67 (host) / :181 (device); dev selects
 * the device's exact mod_mul in the final multiplication */
static void OFN(scaling_step)(const or_ctx *c, int *y, int k, unsigned j, int pow2j, const int *x, const int *cc, int dev) {
    long residue = 0;
    int mult[ON];
    for (int i = 0; i < ON; i++) residue += (long)or_modmul(c->mi_pow2_res[j - 1][i], cc[i], pow2j);
    long temp = (long)k * (long)c->m_pow2_res[j - 1];
    residue = (residue - temp) % pow2j;
    if (residue < 0) residue += pow2j;
    for (int i = 0; i < ON; i++) mult[i] = (int)(residue % c->m[i]);
    for (int i = 0; i < ON; i++) mult[i] = or_modpsub(x[i], mult[i], c->m[i]);
    for (int i = 0; i < ON; i++)
        y[i] = dev ? or_modmul(mult[i], c->pow2_inv[j - 1][i], c->m[i]) : h_modmul_d(mult[i], c->pow2_inv[j - 1][i], c->m[i]);
}
/* rns_scale2pow, host src/rnsscal.cuh:93-119.  The device twin
 * (src/rnsscal.cuh:207-235) differs only in the last step's rank choice:
 * gpu_quirk=1 reproduces it (checked rank when d < D, fast rank when d == D). */
static void OFN(scale2pow)(const or_ctx *c, int *res, const int *x, unsigned D, int dev, int gpu_quirk) {
    int cc[ON];
    for (int i = 0; i < ON; i++) res[i] = x[i];
    int t = (int)(D / OR_T), k;
    if (t > 0) {
        for (int i = 0; i < ON; i++) cc[i] = dev ? or_modmul(x[i], c->w[i], c->m[i]) : h_modmul_d(x[i], c->w[i], c->m[i]);
        k = dev ? OFN(rank_d)(c, x, cc) : OFN(rank_h)(c, x, cc);
        OFN(scaling_step)(c, res, k, OR_T, 1 << OR_T, x, cc, dev);
        t -= 1;
    }
    while (t > 0) {
        for (int i = 0; i < ON; i++) cc[i] = dev ? or_modmul(res[i], c->w[i], c->m[i]) : h_modmul_d(res[i], c->w[i], c->m[i]);
        k = dev ? OFN(rank_fast_d)(c, cc) : OFN(rank_fast_h)(c, cc);
        int tmp[ON];
        memcpy(tmp, res, sizeof(tmp));
        OFN(scaling_step)(c, res, k, OR_T, 1 << OR_T, tmp, cc, dev);
        t -= 1;
    }
    unsigned d = D % OR_T;
    if (d > 0) {
        for (int i = 0; i < ON; i++) cc[i] = dev ? or_modmul(res[i], c->w[i], c->m[i]) : h_modmul_d(res[i], c->w[i], c->m[i]);
        int checked = gpu_quirk ? (d < D) : !(d < D);
        if (dev) k = checked ? OFN(rank_d)(c, res, cc) : OFN(rank_fast_d)(c, cc);
        else k = checked ? OFN(rank_h)(c, res, cc) : OFN(rank_fast_h)(c, cc);
        int tmp[ON];
        memcpy(tmp, res, sizeof(tmp));
        OFN(scaling_step)(c, res, k, d, 1 << d, tmp, cc, dev);
    }
}

/* ---------------- multiple-precision integers (src/mpint.cuh) ---------------- */
typedef struct {
    int digits[ON];
    int sign;
    or_er eval[2];
} OFN(or_mpint);

/* er_add_rd / er_add_ru: host src/extrange.cuh:153/:173 (fast_scalbn, Rump),
 * device :403/:423 (scalbn, IEEE directed). */
static void OFN(er_add_dir)(or_er *r, or_er *x, or_er *y, int dev, int up) {
    x->exp *= (x->frac != 0);
    y->exp *= (y->frac != 0);
    int dexp = (int)((x->exp - y->exp) * (x->frac != 0) * (y->frac != 0));
    double a, b;
    if (dexp > 0) {
        r->exp = x->exp;
        a = x->frac;
        b = dev ? scalbn(y->frac, -dexp) : or_fast_scalbn(y->frac, -dexp);
    } else if (dexp < 0) {
        r->exp = y->exp;
        a = y->frac;
        b = dev ? scalbn(x->frac, dexp) : or_fast_scalbn(x->frac, dexp);
    } else {
        r->exp = (x->exp == 0) ? y->exp : x->exp;
        a = x->frac;
        b = y->frac;
    }
    if (dev) r->frac = up ? d_add_ru(a, b) : d_add_rd(a, b);
    else r->frac = up ? h_add_ru(a, b) : h_add_rd(a, b);
    or_er_adjust(r);
}

/* mpint_add (sub=0) / mpint_sub (sub=1): host src/mpint.cuh:160/:215, device :336/:407 */
static int OFN(mpint_addsub)(const or_ctx *c, OFN(or_mpint) *res, const OFN(or_mpint) *x, const OFN(or_mpint) *y, int sub, int dev) {
    int sx = x->sign, sy = sub ? (y->sign ^ 1) : y->sign;
    or_er evx[2] = {x->eval[0], x->eval[1]}, evy[2] = {y->eval[0], y->eval[1]};
    int alpha = 1 - 2 * sx, beta = 1 - 2 * sy;
    int dig[ON];
    for (int i = 0; i < ON; i++) {
        int m = c->m[i], rsd;
        if (dev) rsd = or_modadd(alpha * x->digits[i], beta * y->digits[i], m);
        else rsd = h_modadd_d(alpha * x->digits[i], beta * y->digits[i], m);
        dig[i] = rsd < 0 ? rsd + m : rsd;
    }
    evx[0].frac *= alpha; evx[1].frac *= alpha;
    evy[0].frac *= beta; evy[1].frac *= beta;
    OFN(er_add_dir)(&res->eval[0], &evx[sx], &evy[sy], dev, 0);
    OFN(er_add_dir)(&res->eval[1], &evx[1 - sx], &evy[1 - sy], dev, 1);
    int minus = res->eval[0].frac < 0 && res->eval[1].frac < 0;
    res->sign = minus;
    if (minus) {
        for (int i = 0; i < ON; i++) dig[i] = dig[i] == 0 ? 0 : c->m[i] - dig[i];
        or_er tmp = res->eval[0];
        res->eval[0].frac = -1 * res->eval[1].frac;
        res->eval[0].exp = res->eval[1].exp;
        res->eval[1].frac = -1 * tmp.frac;
        res->eval[1].exp = tmp.exp;
    }
    for (int i = 0; i < ON; i++) res->digits[i] = dig[i];
    return or_overflow(c, &res->eval[0], &res->eval[1]);
}

/* mpint_mul: host src/mpint.cuh:270, device :478 */
static int OFN(mpint_mul)(const or_ctx *c, OFN(or_mpint) *res, const OFN(or_mpint) *x, const OFN(or_mpint) *y, int dev) {
    or_er_md(&res->eval[0], &x->eval[0], &y->eval[0], &c->unit.upp, dev, 0);
    or_er_md(&res->eval[1], &x->eval[1], &y->eval[1], &c->unit.low, dev, 1);
    int zero = 1;
    for (int i = 0; i < ON; i++) {
        res->digits[i] = dev ? or_modmul(x->digits[i], y->digits[i], c->m[i]) : h_modmul_d(x->digits[i], y->digits[i], c->m[i]);
        zero &= res->digits[i] == 0;
    }
    res->sign = zero ? 0 : (x->sign ^ y->sign);
    return or_overflow(c, &res->eval[0], &res->eval[1]);
}

/* mpint_div (Euclidean quotient): host src/mpint.cuh:286 (rns_div_fast + host
 * evaluation), device :511 (cuda::rns_div + device evaluation).  A negative
 * dividend with a nonzero remainder takes |q| + 1, so x = q*y + r, 0 <= r < |y|;
 * the reference checks no overflow here. */
static int OFN(mpint_div)(const or_ctx *c, OFN(or_mpint) *res, const OFN(or_mpint) *x, const OFN(or_mpint) *y, int dev) {
    int q[ON], r[ON], rz = 1, qz = 1;
    if (dev) OFN(div_d)(c, q, r, x->digits, y->digits, 0);
    else OFN(div_h)(c, q, r, x->digits, y->digits, 1);
    for (int i = 0; i < ON; i++) rz &= r[i] == 0;
    if (x->sign == 1 && !rz)
        for (int i = 0; i < ON; i++) q[i] = (q[i] + 1) % c->m[i];
    or_iv ev;
    if (dev) OFN(eval_d)(c, &ev, q);
    else OFN(eval_h)(c, &ev, q);
    for (int i = 0; i < ON; i++) { res->digits[i] = q[i]; qz &= q[i] == 0; }
    res->eval[0] = ev.low;
    res->eval[1] = ev.upp;
    res->sign = qz ? 0 : (x->sign ^ y->sign);
    return 0;
}

/* ---------------- batch drivers (AoS arrays, reference layout) ---------------- */
static void OFN(batch_eval)(const or_ctx *c, const int *x, long N, or_iv *out, int path, int threads) {
    #pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (threads > 1)
    for (long k = 0; k < N; k++) {
        if (path == 0) OFN(eval_h)(c, out + k, x + k * ON);
        else if (path == 1) OFN(eval_d)(c, out + k, x + k * ON);
        else if (path == 3) OFN(eval_dpar)(c, out + k, x + k * ON);
        else if (path == 4) OFN(eval_fast_d)(c, out + k, x + k * ON);
        else OFN(eval_fast_h)(c, out + k, x + k * ON);
    }
}
static void OFN(batch_cmp)(const or_ctx *c, const int *x, const int *y, long N, int *out, int path, int threads) {
    #pragma omp parallel for schedule(dynamic, 256) num_threads(threads) if (threads > 1)
    for (long k = 0; k < N; k++)
        out[k] = path ? OFN(cmp_d)(c, x + k * ON, y + k * ON) : OFN(cmp_h)(c, x + k * ON, y + k * ON);
}
static void OFN(batch_div)(const or_ctx *c, const int *x, const int *d, long N, int *q, int *r, int path, int fast, int threads) {
    #pragma omp parallel for schedule(dynamic, 16) num_threads(threads) if (threads > 1)
    for (long k = 0; k < N; k++) {
        if (path) OFN(div_d)(c, q + k * ON, r + k * ON, x + k * ON, d + k * ON, fast);
        else OFN(div_h)(c, q + k * ON, r + k * ON, x + k * ON, d + k * ON, fast);
    }
}
static void OFN(batch_scale)(const or_ctx *c, const int *x, const unsigned *D, long N, int *out, int path, int gpu_quirk, int threads) {
    #pragma omp parallel for schedule(dynamic, 64) num_threads(threads) if (threads > 1)
    for (long k = 0; k < N; k++) OFN(scale2pow)(c, out + k * ON, x + k * ON, D[k], path, gpu_quirk);
}
static void OFN(batch_mrc)(const or_ctx *c, const int *x, long N, int *mr, int path) {
    for (long k = 0; k < N; k++) {
        if (path) OFN(mrc_d)(c, mr + k * ON, x + k * ON);
        else OFN(mrc_h)(c, mr + k * ON, x + k * ON);
    }
}
/* op: 0 add, 1 sub, 2 mul, 3 div; flags (optional) receives the overflow status per element */
static void OFN(batch_mpint)(const or_ctx *c, int op, const void *xs, const void *ys, long N, void *outs, int *flags, int path, int threads) {
    const OFN(or_mpint) *x = (const OFN(or_mpint) *)xs, *y = (const OFN(or_mpint) *)ys;
    OFN(or_mpint) *o = (OFN(or_mpint) *)outs;
    #pragma omp parallel for schedule(dynamic, 16) num_threads(threads) if (threads > 1)
    for (long k = 0; k < N; k++) {
        OFN(or_mpint) r;
        memset(&r, 0, sizeof(r));
        int f = op == 3   ? OFN(mpint_div)(c, &r, x + k, y + k, path)
                : op == 2 ? OFN(mpint_mul)(c, &r, x + k, y + k, path)
                          : OFN(mpint_addsub)(c, &r, x + k, y + k, op, path);
        o[k] = r;
        if (flags) flags[k] = f;
    }
}
/* Exact maximum of an RNS array (value as the reference's cuda::rns_max,
 * src/dpp/rnsmax.cuh:129, returns it); ties resolve to the smallest index.
 * Compares mixed-radix digits (device MRC), which is exact for canonical
 * residues. */
static long OFN(max_exact)(const or_ctx *c, const int *x, long N) {
    if (N <= 0) return -1;
    int best[ON], cur[ON];
    long bi = 0;
    OFN(mrc_d)(c, best, x);
    for (long k = 1; k < N; k++) {
        OFN(mrc_d)(c, cur, x + k * ON);
        if (OFN(mrs_cmp)(cur, best) > 0) { memcpy(best, cur, sizeof(best)); bi = k; }
    }
    return bi;
}

#undef OR_CAT2
#undef OR_CAT
#undef OFN
