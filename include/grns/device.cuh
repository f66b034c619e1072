/*
 * grns_gb300 -- source-level drop-in for the reference's per-number device
 * functions (kisupov/grns, namespace cuda), for user kernels that call them
 * one number per thread.
 *
 * Usage, as with the reference: define the moduli set with the params.h
 * convention (RNS_MODULI_SIZE, RNS_MODULI_VALUES -- e.g. include your
 * params.h), include this header in the .cu file that holds your kernels,
 * call rns_const_init() (and mpint_const_init()) on the host before the first
 * launch, then call inside kernels:
 *
 *   cuda::rns_eval_compute(er_float_ptr low, er_float_ptr upp, int *x)   src/rnseval.cuh:182
 *   int cuda::rns_cmp(int *x, int *y)                                    src/rnscmp.cuh:55
 *   cuda::rns_div(int *q, int *r, int *x, int *d)                        src/rnsdiv.cuh:128
 *   cuda::rns_scale2pow(int *result, int *x, unsigned D)                 src/rnsscal.cuh:207
 *   cuda::mpint_add / mpint_sub / mpint_mul(mp_int_ptr r, mp_int_ptr x, mp_int_ptr y)
 *                                                                        src/mpint.cuh:336/407/478
 *
 * Results: the interval of rns_eval_compute bit for bit (the reference's
 * device path); the integer results of rns_cmp, rns_div, rns_scale2pow and
 * the mp_int operations exactly (computed with this library's integer-pipe
 * algorithms, which return the same integers).  Like the reference's, the
 * constants live in per-translation-unit device memory (a __constant__
 * block plus one table allocation kept until exit), so the kernels that use
 * them belong in the translation unit that calls rns_const_init().  For
 * whole arrays, prefer the C ABI (grns.h): it is faster than one call per
 * thread.  rns_const_init() returns nothing, as the reference's does; it
 * leaves the constants zeroed when CUDA fails, and grns_device_init_status()
 * reports the error.
 */
#ifndef GRNS_GB300_DEVICE_CUH
#define GRNS_GB300_DEVICE_CUH

#if !defined(RNS_MODULI_SIZE) || !defined(RNS_MODULI_VALUES)
#error "define RNS_MODULI_SIZE and RNS_MODULI_VALUES (the params.h convention) before including grns/device.cuh"
#endif

#include <cuda_runtime.h>

#include <vector>

#include "../../grns_gb300/csrc/consts_host.h"
#include "../../grns_gb300/csrc/rns_device.cuh"
#include "../../grns_gb300/csrc/rns_fast.cuh"
#include "../../grns_gb300/csrc/rns_mpint.cuh"
#include "types.h"

typedef er_float_t *er_float_ptr;
typedef interval_t *interval_ptr;
typedef struct {  // the reference's mp_int_t for this moduli set (src/types.cuh:45)
    int digits[RNS_MODULI_SIZE];
    int sign;
    er_float_t eval[2];
} mp_int_t;
typedef mp_int_t *mp_int_ptr;
static_assert(sizeof(mp_int_t) == sizeof(grns::MpInt<RNS_MODULI_SIZE>), "mp_int_t layout");

__constant__ grns::Consts<RNS_MODULI_SIZE> grns_dev_consts;

namespace grns_device_detail {
inline cudaError_t &init_status() {
    static cudaError_t st = cudaErrorNotReady;
    return st;
}
inline void *&tables() {
    static void *p = nullptr;
    return p;
}
}  // namespace grns_device_detail

/* builds the constant tables of the RNS_MODULI_VALUES set for the current
 * device (the reference's rns_const_init, src/rnsbase.cuh:324) */
inline void rns_const_init() {
    static const int moduli[RNS_MODULI_SIZE] = RNS_MODULI_VALUES;
    grns::HostTables T;
    grns::build_tables(T, reinterpret_cast<const uint32_t *>(moduli), RNS_MODULI_SIZE);
    const std::vector<uint32_t> blob = grns::table_blob(T);
    void *&d = grns_device_detail::tables();
    cudaError_t e = cudaSuccess;
    if (!d) e = cudaMalloc(&d, blob.size() * sizeof(uint32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d, blob.data(), blob.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        static grns::Consts<RNS_MODULI_SIZE> C;
        grns::fill_consts<RNS_MODULI_SIZE>(C, T, static_cast<const uint32_t *>(d));
        e = cudaMemcpyToSymbol(grns_dev_consts, &C, sizeof(C));
    }
    grns_device_detail::init_status() = e;
}
/* the reference's mpint_const_init (src/mpint.cuh:20): the mp_int operations
 * need no constants beyond rns_const_init's */
inline void mpint_const_init() {}
/* cudaSuccess once rns_const_init() has built the tables */
inline cudaError_t grns_device_init_status() { return grns_device_detail::init_status(); }

namespace cuda {

__device__ __forceinline__ void rns_eval_compute(er_float_ptr low, er_float_ptr upp, int *x) {
    grns::Er lo, up;
    uint32_t f = 0;
    grns::eval<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; }, lo, up, f);
    low->frac = lo.frac;
    low->exp = lo.exp;
    upp->frac = up.frac;
    upp->exp = up.exp;
}

__device__ __forceinline__ int rns_cmp(int *x, int *y) {
    return grns::cmp_fast<RNS_MODULI_SIZE>(grns_dev_consts, [&](int i) { return (uint32_t)x[i]; },
                                           [&](int i) { return (uint32_t)y[i]; });
}

__device__ __forceinline__ void rns_div(int *q, int *r, int *x, int *d) {
    uint32_t f = 0;
    grns::div_fast<RNS_MODULI_SIZE>(grns_dev_consts, reinterpret_cast<uint32_t *>(q), reinterpret_cast<uint32_t *>(r),
                                    reinterpret_cast<const uint32_t *>(x), reinterpret_cast<const uint32_t *>(d), f);
}

__device__ __forceinline__ void rns_scale2pow(int *result, int *x, unsigned D) {
    grns::scale_fast<RNS_MODULI_SIZE>(grns_dev_consts, reinterpret_cast<uint32_t *>(result),
                                      reinterpret_cast<const uint32_t *>(x), D);
}

__device__ __forceinline__ void mpint_add(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using M = grns::MpInt<RNS_MODULI_SIZE>;
    uint32_t f = 0;
    M r;
    r.pad = 0;
    grns::mpint_addsub<RNS_MODULI_SIZE>(grns_dev_consts, r, *reinterpret_cast<const M *>(x),
                                        *reinterpret_cast<const M *>(y), false, f);
    *reinterpret_cast<M *>(result) = r;
}

__device__ __forceinline__ void mpint_sub(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using M = grns::MpInt<RNS_MODULI_SIZE>;
    uint32_t f = 0;
    M r;
    r.pad = 0;
    grns::mpint_addsub<RNS_MODULI_SIZE>(grns_dev_consts, r, *reinterpret_cast<const M *>(x),
                                        *reinterpret_cast<const M *>(y), true, f);
    *reinterpret_cast<M *>(result) = r;
}

__device__ __forceinline__ void mpint_mul(mp_int_ptr result, mp_int_ptr x, mp_int_ptr y) {
    using M = grns::MpInt<RNS_MODULI_SIZE>;
    uint32_t f = 0;
    M r;
    r.pad = 0;
    grns::mpint_mul<RNS_MODULI_SIZE>(grns_dev_consts, r, *reinterpret_cast<const M *>(x),
                                     *reinterpret_cast<const M *>(y), f);
    *reinterpret_cast<M *>(result) = r;
}

}  // namespace cuda

#endif
