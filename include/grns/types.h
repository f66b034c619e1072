/*
 * Public data layouts of grns_gb300, byte-identical to the reference
 * library kisupov/grns (src/types.cuh:13-49) so buffers written by code
 * that uses the reference can be passed straight in.
 */
#ifndef GRNS_GB300_TYPES_H
#define GRNS_GB300_TYPES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Extended-range float f * 2^exp, |f| in [1, 2) or 0 (src/types.cuh:13-16). 16 bytes. */
typedef struct {
    double frac;
    int64_t exp;
} er_float_t;

/* Interval evaluation [low, upp] that encloses X/M (src/types.cuh:25-28). 32 bytes. */
typedef struct {
    er_float_t low;
    er_float_t upp;
} interval_t;

/* Interval evaluation plus an integer tag, e.g. an array index (src/types.cuh:36-40). 40 bytes. */
typedef struct {
    er_float_t low;
    er_float_t upp;
    int32_t idx;
} xinterval_t;

/*
 * mp_int_t (src/types.cuh:45-49) is `struct { int digits[n]; int sign;
 * er_float_t eval[2]; }` with n fixed per moduli set, so its size depends on n:
 * digits at offset 0, sign at 4n, eval at GRNS_MPINT_EVAL_OFFSET(n).
 * n = 8 -> 72 bytes, n = 32 -> 168, n = 64 -> 296.
 */
#define GRNS_MPINT_EVAL_OFFSET(n) ((((size_t)(n) * 4 + 4 + 7) / 8) * 8)
#define GRNS_MPINT_BYTES(n) (GRNS_MPINT_EVAL_OFFSET(n) + 2 * sizeof(er_float_t))

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(er_float_t) == 16, "er_float_t layout");
static_assert(sizeof(interval_t) == 32, "interval_t layout");
static_assert(sizeof(xinterval_t) == 40, "xinterval_t layout");
static_assert(GRNS_MPINT_BYTES(8) == 72 && GRNS_MPINT_BYTES(32) == 168 && GRNS_MPINT_BYTES(64) == 296,
              "mp_int_t layout");
#endif

#endif
