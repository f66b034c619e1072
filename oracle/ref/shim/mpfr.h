/*
 * Minimal MPFR prototype shim used ONLY to compile the reference library as
 * a CPU checker under oracle/_ref (libmpfr.so.6 is installed without its
 * header).  Hand-written declarations of the calls the reference makes; the
 * struct matches MPFR 4.x with the default 64-bit precision/exponent formats.
 */
#ifndef ORACLE_SHIM_MPFR_H
#define ORACLE_SHIM_MPFR_H
#include "gmp.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef long mpfr_prec_t;
typedef int mpfr_sign_t;
typedef long mpfr_exp_t;
typedef struct { mpfr_prec_t _mpfr_prec; mpfr_sign_t _mpfr_sign; mpfr_exp_t _mpfr_exp; mp_limb_t *_mpfr_d; } __mpfr_struct;
typedef __mpfr_struct mpfr_t[1];
typedef __mpfr_struct *mpfr_ptr;
typedef const __mpfr_struct *mpfr_srcptr;
typedef enum { MPFR_RNDN = 0, MPFR_RNDZ, MPFR_RNDU, MPFR_RNDD, MPFR_RNDA, MPFR_RNDF, MPFR_RNDNA = -1 } mpfr_rnd_t;

void mpfr_init(mpfr_ptr);
void mpfr_init2(mpfr_ptr, mpfr_prec_t);
void mpfr_clear(mpfr_ptr);
int mpfr_set_z(mpfr_ptr, mpz_srcptr, mpfr_rnd_t);
int mpfr_set_ui(mpfr_ptr, unsigned long, mpfr_rnd_t);
int mpfr_set_d(mpfr_ptr, double, mpfr_rnd_t);
int mpfr_div(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_sub(mpfr_ptr, mpfr_srcptr, mpfr_srcptr, mpfr_rnd_t);
int mpfr_log2(mpfr_ptr, mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d(mpfr_srcptr, mpfr_rnd_t);
double mpfr_get_d_2exp(long *, mpfr_srcptr, mpfr_rnd_t);
#ifdef __cplusplus
}
#endif
#endif
