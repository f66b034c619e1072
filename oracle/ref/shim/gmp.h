/*
 * Minimal GMP prototype shim used ONLY to compile the reference library
 * (kisupov/grns) as a CPU checker under oracle/_ref.  The system ships
 * libgmp.so.10 without its header; these hand-written declarations cover
 * exactly the entry points the reference's src/ headers call.  The ABI
 * (mpz struct, limb type) is the LP64 Linux one used by libgmp 6.x on both
 * x86_64 and aarch64.
 */
#ifndef ORACLE_SHIM_GMP_H
#define ORACLE_SHIM_GMP_H
#ifdef __cplusplus
extern "C" {
#endif
typedef unsigned long mp_limb_t;
typedef struct { int _mp_alloc; int _mp_size; mp_limb_t *_mp_d; } __mpz_struct;
typedef __mpz_struct mpz_t[1];
typedef __mpz_struct *mpz_ptr;
typedef const __mpz_struct *mpz_srcptr;

void __gmpz_init(mpz_ptr);
void __gmpz_clear(mpz_ptr);
void __gmpz_set(mpz_ptr, mpz_srcptr);
void __gmpz_set_ui(mpz_ptr, unsigned long);
void __gmpz_set_si(mpz_ptr, long);
int __gmpz_set_str(mpz_ptr, const char *, int);
void __gmpz_add(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_add_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_sub(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul(mpz_ptr, mpz_srcptr, mpz_srcptr);
void __gmpz_mul_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mul_si(mpz_ptr, mpz_srcptr, long);
void __gmpz_fdiv_q(mpz_ptr, mpz_srcptr, mpz_srcptr);
unsigned long __gmpz_fdiv_q_ui(mpz_ptr, mpz_srcptr, unsigned long);
unsigned long __gmpz_fdiv_r_ui(mpz_ptr, mpz_srcptr, unsigned long);
void __gmpz_mod(mpz_ptr, mpz_srcptr, mpz_srcptr);
int __gmpz_cmp_ui(mpz_srcptr, unsigned long);
unsigned long __gmpz_get_ui(mpz_srcptr);
long __gmpz_get_si(mpz_srcptr);
double __gmpz_get_d(mpz_srcptr);
char *__gmpz_get_str(char *, int, mpz_srcptr);
void __gmpz_abs(mpz_ptr, mpz_srcptr);

#define mpz_init __gmpz_init
#define mpz_clear __gmpz_clear
#define mpz_set __gmpz_set
#define mpz_set_ui __gmpz_set_ui
#define mpz_set_si __gmpz_set_si
#define mpz_set_str __gmpz_set_str
#define mpz_add __gmpz_add
#define mpz_add_ui __gmpz_add_ui
#define mpz_sub __gmpz_sub
#define mpz_mul __gmpz_mul
#define mpz_mul_ui __gmpz_mul_ui
#define mpz_mul_si __gmpz_mul_si
#define mpz_fdiv_q __gmpz_fdiv_q
#define mpz_div_ui __gmpz_fdiv_q_ui
#define mpz_mod_ui __gmpz_fdiv_r_ui
#define mpz_mod __gmpz_mod
#define mpz_cmp_ui __gmpz_cmp_ui
#define mpz_get_ui __gmpz_get_ui
#define mpz_get_si __gmpz_get_si
#define mpz_get_d __gmpz_get_d
#define mpz_get_str __gmpz_get_str
#define mpz_abs __gmpz_abs
#ifdef __cplusplus
}
#endif
#endif
