// CPU build of the product's integer fast-path algorithms (grns_gb300/csrc/rns_fast.cuh)
// for exhaustive and randomised checks against exact integer arithmetic.
// Driven by tests/test_fast_paths.py; arrays are AoS [count][n].
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../grns_gb300/csrc/consts_host.h"
#include "../../grns_gb300/csrc/rns_fast.cuh"
#include "../../grns_gb300/csrc/rns_convert.cuh"

using namespace grns;

struct Box {
    int n;
    HostTables T;
    std::vector<uint32_t> blob;
    alignas(16) unsigned char consts[sizeof(Consts<kMaxModuli>)];
};

template <int N>
static const Consts<N> &K(const Box *b) { return *reinterpret_cast<const Consts<N> *>(b->consts); }

#define FC_CASE_(n) case n: C_(n); break;  // C_: the caller's macro
#define DISPATCH(n, CALL) switch (n) { GRNS_FOR_EACH_N(FC_CASE_) default: return -1; }

extern "C" {

void *fc_create(const uint32_t *m, int n) {
    Box *b = new Box();
    b->n = n;
    build_tables(b->T, m, n);
    b->blob = table_blob(b->T);
#define F_(N) fill_consts<N>(*reinterpret_cast<Consts<N> *>(b->consts), b->T, b->blob.data())
#define FC_FILL_(n) case n: F_(n); break;
    switch (n) { GRNS_FOR_EACH_N(FC_FILL_) default: delete b; return nullptr; }
#undef FC_FILL_
#undef F_
    return b;
}
void fc_destroy(void *p) { delete (Box *)p; }

int fc_cmp(void *p, const uint32_t *x, const uint32_t *y, long cnt, int32_t *out) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) out[k] = cmp_fast<N>(K<N>(b), [&](int i) { return x[k * N + i]; }, \
                                                                [&](int i) { return y[k * N + i]; })
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

int fc_div(void *p, const uint32_t *x, const uint32_t *d, long cnt, uint32_t *q, uint32_t *r, uint32_t *flags) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { uint32_t f = 0; div_fast<N>(K<N>(b), q + k * N, r + k * N, x + k * N, \
                                                                           d + k * N, f); flags[k] = f; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* the same divisions through prepared rows (the plain call's pass A / pass B split) */
int fc_div_rows(void *p, const uint32_t *x, const uint32_t *d, long cnt, uint32_t *q, uint32_t *r, uint32_t *flags) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { uint32_t f = 0; div_rows<N>(K<N>(b), q + k * N, r + k * N, x + k * N, \
                                                                           d + k * N, f); flags[k] = f; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

int fc_scale(void *p, const uint32_t *x, const uint32_t *D, long cnt, uint32_t *out) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) scale_fast<N>(K<N>(b), out + k * N, x + k * N, D[k])
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

int fc_scale_bin(void *p, const uint32_t *x, const uint32_t *D, long cnt, uint32_t *out) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) scale_bin<N>(K<N>(b), out + k * N, x + k * N, D[k])
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* fixed-point sums for direct checks: frac64 = fx64, and the 128-bit fx96 total */
int fc_fx(void *p, const uint32_t *x, long cnt, uint64_t *f64, uint64_t *f96lo, uint64_t *f96hi) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { auto g = [&](int i) { return x[k * N + i]; }; \
        f64[k] = fx64<N>(K<N>(b), g); u128 t = fx96<N>(K<N>(b), g); f96lo[k] = (uint64_t)t; f96hi[k] = (uint64_t)(t >> 64); }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* integer-pipe interval evaluation: status per number (kEvalOk / kEvalRare /
 * kEvalZero, 8 for an invalid residue) and, for kEvalOk, the interval */
int fc_eval(void *p, const uint32_t *x, long cnt, int32_t *status, Er *iv) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { uint32_t bad = 0; Er lo{0, 0}, up{0, 0}; \
        int st = eval_int<N>(K<N>(b), [&](int i) { return x[k * N + i]; }, lo, up, bad); \
        status[k] = bad ? 8 : st; iv[2 * k] = lo; iv[2 * k + 1] = up; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* the same for rns_eval_compute_fast (no mixed-radix step) */
int fc_eval_fast(void *p, const uint32_t *x, long cnt, int32_t *status, Er *iv) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { uint32_t bad = 0; Er lo{0, 0}, up{0, 0}; \
        auto g = [&](int i) { return x[k * N + i]; }; \
        int st = eval_int<N, decltype(g), true>(K<N>(b), g, lo, up, bad); \
        status[k] = bad ? 8 : st; iv[2 * k] = lo; iv[2 * k + 1] = up; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* one-ulp evaluation: 1 where certified (interval written), 0 where the
 * bit-exact evaluation would be used */
int fc_eval_tight(void *p, const uint32_t *x, long cnt, int32_t *ok, Er *iv) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) { uint32_t bad = 0; Er lo{0, 0}, up{0, 0}; \
        ok[k] = eval_tight<N>(K<N>(b), [&](int i) { return x[k * N + i]; }, lo, up, bad) ? 1 : 0; \
        iv[2 * k] = lo; iv[2 * k + 1] = up; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* binary -> RNS: words[k * limbs ..] little-endian 32-bit limbs */
int fc_from_binary(void *p, const uint32_t *words, int limbs, long cnt, uint32_t *out) {
    Box *b = (Box *)p;
#define C_(N) for (long k = 0; k < cnt; k++) from_binary<N>(K<N>(b), words + k * limbs, limbs, out + k * N)
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* RNS -> binary: out[k * bin_limbs ..]; ok[k] = 0 for an invalid residue */
int fc_to_binary(void *p, const uint32_t *x, long cnt, uint32_t *out, int32_t *ok) {
    Box *b = (Box *)p;
    std::vector<uint32_t> d(b->T.bin_chunks);
    const int L = b->T.bin_limbs;
#define C_(N) for (long k = 0; k < cnt; k++) { \
        ok[k] = to_binary<N>(K<N>(b), [&](int i) { return x[k * N + i]; }, d.data(), 1) ? 1 : 0; \
        for (int l = 0; l < L; l++) out[k * L + l] = d[l]; }
    DISPATCH(b->n, C_)
#undef C_
    return 0;
}

/* (a b) / c with directed rounding on the integer pipe; ok[k] = 0 where it defers to FP64 */
int fc_dmuldiv(const double *a, const double *b, const double *c, long cnt, int up, double *out, int32_t *ok) {
    for (long k = 0; k < cnt; k++) {
        double r = 0;
        ok[k] = dmuldiv_dir_i(a[k], b[k], c[k], up != 0, r) ? 1 : 0;
        double r2 = 0;  /* with the precomputed reciprocal: the same answer */
        if (dmuldiv_dir_i(a[k], b[k], c[k], up != 0, r2, dmuldiv_recip(c[k])) != (ok[k] != 0) ||
            dbits(r2) != dbits(r))
            ok[k] = -1;
        out[k] = r;
    }
    return 0;
}

int fc_binary_limbs(void *p) { return ((Box *)p)->T.bin_limbs; }

uint64_t fc_E(void *p) { return ((Box *)p)->T.E; }

/* table `which` as grns_ctx_get_table returns it: bytes copied to dst, or -1 */
long fc_table(void *p, int which, void *dst, long cap) {
    const std::vector<uint8_t> t = table_bytes(((Box *)p)->T, which);
    if (t.empty() || (long)t.size() > cap) return -1;
    memcpy(dst, t.data(), t.size());
    return (long)t.size();
}

}
