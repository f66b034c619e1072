/*
 * C-ABI driver around the UNMODIFIED reference library (kisupov/grns src/),
 * compiled for the CPU by oracle/ref/build_ref.py into oracle/_ref/.  It is
 * a checker: it pins the C restatement in oracle/grns_oracle.c and generates
 * the golden vectors under tests/golden/.  Nothing in the product links it.
 *
 * Each build fixes one moduli set through a params header pre-included ahead
 * of the reference's own src/params.h (whose include guard then skips it).
 * Both reference paths are exported:
 *   ref_host_*  -> the global-namespace host functions (Rump-style rounding)
 *   ref_dev_*   -> the `namespace cuda` device functions, run on the CPU with
 *                  exact emulation of the directed-rounding intrinsics.
 * Arrays of RNS numbers use the reference AoS layout [x1..xn][x1..xn]...
 */
#include "rnseval.cuh"
#include "rnscmp.cuh"
#include "rnsdiv.cuh"
#include "rnsscal.cuh"
#include "mpint.cuh"

oracle_shim_dim3 threadIdx, blockIdx, blockDim, gridDim;

#define N_ RNS_MODULI_SIZE

extern "C" {

int ref_n() { return RNS_MODULI_SIZE; }
int ref_log2() { return RNS_MODULI_PRODUCT_LOG2; }
int ref_sizeof_mpint() { return (int)sizeof(mp_int_t); }

void ref_init() {
    rns_const_init();
    mpint_const_init();
}

/* Constants as rns_const_init leaves them in the `cuda::` tables (the ones the
 * GPU path reads) plus the host-only reciprocal set. */
void ref_consts(int *w, double *recip_rd, double *recip_ru, double *acc, int *ref_factor,
                interval_t *unit, interval_t *inv_unit, int *mrc_inv, int *pow2,
                int *m_pow2_res, int *mi_pow2_res, int *pow2_inv) {
    memcpy(w, cuda::RNS_PART_MODULI_PRODUCT_INVERSE, sizeof(int) * N_);
    memcpy(recip_rd, cuda::RNS_MODULI_RECIP_RD, sizeof(double) * N_);
    memcpy(recip_ru, cuda::RNS_MODULI_RECIP_RU, sizeof(double) * N_);
    *acc = cuda::RNS_EVAL_ACCURACY;
    *ref_factor = cuda::RNS_EVAL_REF_FACTOR;
    *unit = cuda::RNS_EVAL_UNIT;
    *inv_unit = cuda::RNS_EVAL_INV_UNIT;
    memcpy(mrc_inv, cuda::MRC_MULT_INV, sizeof(int) * N_ * N_);
    memcpy(pow2, cuda::RNS_POW2, sizeof(int) * (RNS_MODULI_PRODUCT_LOG2 + 1) * N_);
    memcpy(m_pow2_res, cuda::RNS_MODULI_PRODUCT_POW2_RESIDUES, sizeof(int) * RNS_P2_SCALING_THRESHOLD);
    memcpy(mi_pow2_res, cuda::RNS_PART_MODULI_PRODUCT_POW2_RESIDUES, sizeof(int) * RNS_P2_SCALING_THRESHOLD * N_);
    memcpy(pow2_inv, cuda::RNS_POW2_INVERSE, sizeof(int) * RNS_P2_SCALING_THRESHOLD * N_);
}

void ref_host_eval(const int *x, long N, interval_t *out) {
    int t[N_];
    for (long k = 0; k < N; k++) { memcpy(t, x + k * N_, sizeof(t)); rns_eval_compute(&out[k].low, &out[k].upp, t); }
}
void ref_host_eval_fast(const int *x, long N, interval_t *out) {
    int t[N_];
    for (long k = 0; k < N; k++) { memcpy(t, x + k * N_, sizeof(t)); rns_eval_compute_fast(&out[k].low, &out[k].upp, t); }
}
void ref_dev_eval(const int *x, long N, interval_t *out) {
    int t[N_];
    for (long k = 0; k < N; k++) { memcpy(t, x + k * N_, sizeof(t)); cuda::rns_eval_compute(&out[k].low, &out[k].upp, t); }
}
void ref_dev_eval_fast(const int *x, long N, interval_t *out) {
    int t[N_];
    for (long k = 0; k < N; k++) { memcpy(t, x + k * N_, sizeof(t)); cuda::rns_eval_compute_fast(&out[k].low, &out[k].upp, t); }
}

void ref_host_cmp(const int *x, const int *y, long N, int *out) {
    int a[N_], b[N_];
    for (long k = 0; k < N; k++) {
        memcpy(a, x + k * N_, sizeof(a)); memcpy(b, y + k * N_, sizeof(b));
        out[k] = rns_cmp(a, b);
    }
}
void ref_dev_cmp(const int *x, const int *y, long N, int *out) {
    int a[N_], b[N_];
    for (long k = 0; k < N; k++) {
        memcpy(a, x + k * N_, sizeof(a)); memcpy(b, y + k * N_, sizeof(b));
        out[k] = cuda::rns_cmp(a, b);
    }
}

/* variant: 0 = rns_div, 1 = rns_div_fast */
void ref_host_div(const int *x, const int *d, long N, int variant, int *q, int *r) {
    int a[N_], b[N_];
    for (long k = 0; k < N; k++) {
        memcpy(a, x + k * N_, sizeof(a)); memcpy(b, d + k * N_, sizeof(b));
        if (variant) rns_div_fast(q + k * N_, r + k * N_, a, b); else rns_div(q + k * N_, r + k * N_, a, b);
    }
}
void ref_dev_div(const int *x, const int *d, long N, int variant, int *q, int *r) {
    int a[N_], b[N_];
    for (long k = 0; k < N; k++) {
        memcpy(a, x + k * N_, sizeof(a)); memcpy(b, d + k * N_, sizeof(b));
        if (variant) cuda::rns_div_fast(q + k * N_, r + k * N_, a, b); else cuda::rns_div(q + k * N_, r + k * N_, a, b);
    }
}

void ref_host_scale2pow(const int *x, const unsigned *D, long N, int *out) {
    int a[N_];
    for (long k = 0; k < N; k++) { memcpy(a, x + k * N_, sizeof(a)); rns_scale2pow(out + k * N_, a, D[k]); }
}
void ref_dev_scale2pow(const int *x, const unsigned *D, long N, int *out) {
    int a[N_];
    for (long k = 0; k < N; k++) { memcpy(a, x + k * N_, sizeof(a)); cuda::rns_scale2pow(out + k * N_, a, D[k]); }
}

void ref_host_mrc(const int *x, long N, int *mr) {
    int a[N_];
    for (long k = 0; k < N; k++) { memcpy(a, x + k * N_, sizeof(a)); mrc(mr + k * N_, a); }
}
void ref_dev_mrc(const int *x, long N, int *mr) {
    int a[N_];
    for (long k = 0; k < N; k++) { memcpy(a, x + k * N_, sizeof(a)); cuda::mrc(mr + k * N_, a); }
}

/* op: 0 add, 1 sub, 2 mul, 3 div */
void ref_host_mpint(int op, const mp_int_t *x, const mp_int_t *y, long N, mp_int_t *out) {
    for (long k = 0; k < N; k++) {
        mp_int_t a = x[k], b = y[k], z;
        memset(&z, 0, sizeof(z));
        switch (op) {
            case 0: mpint_add(&z, &a, &b); break;
            case 1: mpint_sub(&z, &a, &b); break;
            case 2: mpint_mul(&z, &a, &b); break;
            default: mpint_div(&z, &a, &b); break;
        }
        out[k] = z;
    }
}
void ref_dev_mpint(int op, const mp_int_t *x, const mp_int_t *y, long N, mp_int_t *out) {
    for (long k = 0; k < N; k++) {
        mp_int_t a = x[k], b = y[k], z;
        memset(&z, 0, sizeof(z));
        switch (op) {
            case 0: cuda::mpint_add(&z, &a, &b); break;
            case 1: cuda::mpint_sub(&z, &a, &b); break;
            case 2: cuda::mpint_mul(&z, &a, &b); break;
            default: cuda::mpint_div(&z, &a, &b); break;
        }
        out[k] = z;
    }
}

/* mp_int from a decimal string via the reference's mpint_set_mpz (host eval). */
void ref_mpint_from_str(const char *dec, mp_int_t *out) {
    mpz_t v;
    mpz_init(v);
    mpz_set_str(v, dec, 10);
    mpint_set_mpz(out, v);
    mpz_clear(v);
}
void ref_mpint_set_i(int v, mp_int_t *out) { mpint_set_i(out, v); }

/* rns_from_binary (src/rnsbase.cuh:253) of the integer in a decimal string */
void ref_rns_from_str(const char *dec, int *out) {
    mpz_t v;
    mpz_init(v);
    mpz_set_str(v, dec, 10);
    rns_from_binary(out, v);
    mpz_clear(v);
}
/* rns_to_binary (src/rnsbase.cuh:277) as a decimal string; buf holds 2048 chars */
void ref_rns_to_str(const int *x, char *buf) {
    mpz_t v;
    mpz_init(v);
    int t[N_];
    memcpy(t, x, sizeof(t));
    rns_to_binary(v, t);
    mpz_get_str(buf, 10, v);
    mpz_clear(v);
}
/* mpint_get_mpz (src/mpint.cuh:100) as a decimal string; buf holds 2048 chars */
void ref_mpint_to_str(const mp_int_t *x, char *buf) {
    mpz_t v;
    mpz_init(v);
    mp_int_t t = *x;
    mpint_get_mpz(v, &t);
    mpz_get_str(buf, 10, v);
    mpz_clear(v);
}

/* extended-range ops for the reference's er_* known-answer checks.
 * op: 0 add, 1 add_rd, 2 add_ru, 3 sub, 4 sub_rd, 5 sub_ru, 6 mul, 7 mul_rd,
 *     8 mul_ru, 9 div, 10 div_rd, 11 div_ru, 12 md_rd(x,y,z), 13 md_ru(x,y,z),
 *     14 cmp, 15 ucmp, 16 set_d (x->frac holds the double)
 * dev selects the `cuda::` twin. Returns the comparison for 14/15. */
int ref_er(int op, int dev, const er_float_t *x, const er_float_t *y, const er_float_t *z, er_float_t *out) {
    er_float_t a = *x, b = *y, c = *z;
    if (!dev) {
        switch (op) {
            case 0: er_add(out, &a, &b); break;
            case 1: er_add_rd(out, &a, &b); break;
            case 2: er_add_ru(out, &a, &b); break;
            case 3: er_sub(out, &a, &b); break;
            case 4: er_sub_rd(out, &a, &b); break;
            case 5: er_sub_ru(out, &a, &b); break;
            case 6: er_mul(out, &a, &b); break;
            case 7: er_mul_rd(out, &a, &b); break;
            case 8: er_mul_ru(out, &a, &b); break;
            case 9: er_div(out, &a, &b); break;
            case 10: er_div_rd(out, &a, &b); break;
            case 11: er_div_ru(out, &a, &b); break;
            case 12: er_md_rd(out, &a, &b, &c); break;
            case 13: er_md_ru(out, &a, &b, &c); break;
            case 14: return er_cmp(&a, &b);
            case 15: return er_ucmp(&a, &b);
            default: er_set_d(out, a.frac); break;
        }
    } else {
        switch (op) {
            case 0: cuda::er_add(out, &a, &b); break;
            case 1: cuda::er_add_rd(out, &a, &b); break;
            case 2: cuda::er_add_ru(out, &a, &b); break;
            case 3: cuda::er_sub(out, &a, &b); break;
            case 4: cuda::er_sub_rd(out, &a, &b); break;
            case 5: cuda::er_sub_ru(out, &a, &b); break;
            case 6: cuda::er_mul(out, &a, &b); break;
            case 7: cuda::er_mul_rd(out, &a, &b); break;
            case 8: cuda::er_mul_ru(out, &a, &b); break;
            case 9: cuda::er_div(out, &a, &b); break;
            case 10: cuda::er_div_rd(out, &a, &b); break;
            case 11: cuda::er_div_ru(out, &a, &b); break;
            case 12: cuda::er_md_rd(out, &a, &b, &c); break;
            case 13: cuda::er_md_ru(out, &a, &b, &c); break;
            case 14: return cuda::er_cmp(&a, &b);
            case 15: return cuda::er_ucmp(&a, &b);
            default: cuda::er_set_d(out, a.frac); break;
        }
    }
    return 0;
}

}  // extern "C"
