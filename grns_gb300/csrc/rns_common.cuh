/*
 * grns_gb300 -- shared host/device building blocks.
 *
 *   * per-moduli-set constant block passed to every kernel by value (so the
 *     per-modulus constants sit in the kernel-parameter constant bank and are
 *     read with compile-time offsets from fully unrolled loops); above 64
 *     moduli the block is passed by the address of its device copy (CArg);
 *   * modular arithmetic on the integer pipe: Shoup multiplication by a
 *     constant, Barrett multiplication of two residues, branch-free add/sub;
 *   * extended-range float (er_float_t) helpers with the reference's exact
 *     semantics (src/extrange.cuh:366-603).
 *
 * Residues are canonical uint32 in [0, m) with m odd and 3 <= m <= 1431655765
 * (3m fits in 32 bits, which the Barrett step below relies on).
 */
#pragma once

#include <cstddef>
#include <cstdint>
#include <type_traits>

#ifdef __CUDACC__
#define GRNS_HD __host__ __device__ __forceinline__
#else
#define GRNS_HD inline
#endif

/* Loops over the moduli are unrolled fully up to 64 moduli.  For 128 and 256
 * they stay rolled: their per-number arrays live in local memory either way,
 * and full unrolling there costs minutes of compile time per kernel.
 * GRNS_UNROLL_TO(B) is for a loop of at most B trips in a template on N. */
#define GRNS_PRAGMA_(x) _Pragma(#x)
#define GRNS_UNROLL_TO(B) GRNS_PRAGMA_(unroll((N) > 64 ? 1 : (B)))
#define GRNS_UNROLL_N GRNS_UNROLL_TO(N)

#ifndef __CUDACC__
struct uint4 { uint32_t x, y, z, w; };
struct uint2 { uint32_t x, y; };
#endif

namespace grns {

constexpr int kMaxModuli = 256;
constexpr int kScaleStep = 30;  // RNS_P2_SCALING_THRESHOLD (reference src/params.h:22)
constexpr int kDivB = 48;       // quotient bits per step of the integer division
constexpr int kScaleB = 52;     // bits per step of the integer power-of-two scaling
constexpr int kPow2NegRows = 64;  // rows j = 0..63 of the 2^-j mod m_i table
/* rows a = 0.. of the 2^(64 a) and 2^-(64 a) mod m_i tables: every division shift s <= log2M + 64 */
constexpr int pow2_hi_rows(int log2M) { return (log2M + 64) / 64 + 1; }
/* binary <-> RNS conversion: integers as 32-bit little-endian limbs, worked
 * on in 26-bit chunks (26 + 30.42 bits per product: up to 158 products, or
 * 64 moduli, sum below 2^64; longer sums fold every kBinFold products or, for
 * more than 64 moduli, add in 128 bits) */
constexpr int kBinChunk = 26;
constexpr int kBinMaxLimbs = 256;                                   // 8192-bit inputs
constexpr int kBinMaxChunks = (32 * kBinMaxLimbs + kBinChunk - 1) / kBinChunk;  // 316
constexpr int kBinFold = 128;

/* levels of the pairwise summation tree over n leaves */
constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c((n + 1) / 2); }

struct Er {  // er_float_t
    double frac;
    int64_t exp;
};

/* Constant block of one moduli set, specialised on the moduli count N. */
/* the moduli counts kernels are built for: every n from 4 to 16, 32, 64, 128
 * and 256 (the sizes of the reference's params catalogue) */
#define GRNS_FOR_EACH_N(X) \
    X(4) X(5) X(6) X(7) X(8) X(9) X(10) X(11) X(12) X(13) X(14) X(15) X(16) X(32) X(64) X(128) X(256)
GRNS_HD constexpr bool supported_n(int n) {
    return (n >= 4 && n <= 16) || n == 32 || n == 64 || n == 128 || n == 256;
}

/* words per row of the binary conversion tables: n rounded up to a multiple of 4 */
GRNS_HD constexpr int bin_ld(int n) { return (n + 3) / 4 * 4; }

template <int N>
struct Consts {
    uint32_t m[N];        // moduli
    uint32_t w[N];        // (M/m_i)^-1 mod m_i          RNS_PART_MODULI_PRODUCT_INVERSE
    uint32_t w_sh[N];     // floor(w_i * 2^32 / m_i)     Shoup companion of w_i
    uint32_t mu[N];       // floor(2^(2 b_i) / m_i)      Barrett constant, b_i = bit length of m_i
    uint32_t b[N];        // b_i
    double rrd[N];        // RNS_MODULI_RECIP_RD
    double rru[N];        // RNS_MODULI_RECIP_RU
    double acc;           // RNS_EVAL_ACCURACY
    int ref_factor;       // RNS_EVAL_REF_FACTOR
    int log2M;            // floor(log2 M), the RNS_MODULI_PRODUCT_LOG2 convention
    Er unit_low, unit_upp, inv_unit_low, inv_unit_upp;  // RNS_EVAL_UNIT, RNS_EVAL_INV_UNIT
    uint64_t unit_rcp_low, unit_rcp_upp;  // floor(2^116 / mantissa) of unit_low.frac, unit_upp.frac
    uint32_t m_pow2_res30;                // M mod 2^30
    /* integer fast path: fixed-point reciprocals.  "w-folded" constants give
     * frac(x_i w_i / m_i) directly from the residue x_i (frac(x w / m) = s / m). */
    uint32_t c64l[N], c64h[N];            // ceil(2^64 w_i / m_i) mod 2^64 (w-folded)
    uint32_t c96_0[N], c96_1[N], c96_2[N];  // ceil(2^96 / m_i), 32-bit words (applied to s_i)
    uint32_t c96w_0[N], c96w_1[N], c96w_2[N];  // ceil(2^96 w_i / m_i) mod 2^96 (w-folded, applied to x_i)
    uint32_t b48[N], b48_sh[N];           // 2^kDivB mod m_i, Shoup companion
    /* integer-pipe interval evaluation: RNS_MODULI_RECIP_RD / _RU times 2^100
     * (exact integers below 2^100) and ceil(RNS_EVAL_ACCURACY * 2^100) */
    uint64_t evl_lo[N], evl_hi[N], evu_lo[N], evu_hi[N];
    uint64_t acc_lo, acc_hi;
    /* scaling: M_i mod 2^64, M mod 2^64 (binary low words of the CRT weights) */
    uint64_t mi64[N];
    uint64_t m64;
    /* one-ulp evaluation: ceil(2^128 w_i / m_i) mod 2^128, 32-bit words (w-folded) */
    uint32_t c128w_0[N], c128w_1[N], c128w_2[N], c128w_3[N];
    uint32_t t32[N], t32_sh[N];           // 2^32 mod m_i, Shoup companion
    uint32_t mrbits[N];                   // bit length of m_0 * ... * m_{t-1}
    uint64_t E;                           // sum_i (m_i - 1): fixed-point truncation error bound
    const uint32_t *pow2;       // [(log2M + 1) * N]  2^j mod m_i        (RNS_POW2)
    const uint32_t *pow2_sh;    // [(log2M + 1) * N]  Shoup companions
    const uint4 *c96k;          // [(log2M + 1) * N]  ceil(2^96 (2^k w_i mod m_i) / m_i) mod 2^96 (w-folded, x 2^k)
    const uint32_t *mrc_inv;    // [N * N]  [j * N + i] = m_j^-1 mod m_i (MRC_MULT_INV)
    const uint32_t *mrc_inv_sh; // [N * N]  Shoup companions
    const uint32_t *mi_pow2;    // [30 * N] M_i mod 2^(j+1)             (RNS_PART_MODULI_PRODUCT_POW2_RESIDUES)
    const uint32_t *m_pow2;     // [30]     M mod 2^(j+1)               (RNS_MODULI_PRODUCT_POW2_RESIDUES)
    const uint32_t *pow2_inv;   // [30 * N] (2^(j+1))^-1 mod m_i        (RNS_POW2_INVERSE)
    const uint32_t *pow2_inv_sh;// [30 * N]
    const uint32_t *pow2neg;    // [kPow2NegRows * N]  2^-j mod m_i
    const uint32_t *pow2neg_sh; // [kPow2NegRows * N]
    /* division: (value, Shoup companion) pairs, residue-major -- [i * 64 + j]: 2^j (p2lo),
     * 2^-j (p2nlo); [i * p2rows + a]: 2^(64 a) (p2hi), 2^-(64 a) (p2nhi) mod m_i */
    const uint2 *p2lo, *p2hi, *p2nlo, *p2nhi;
    int p2rows;
    /* binary conversion (16-byte aligned rows of bin_ld(N) words, zeros past N) */
    const uint32_t *bin_p26;    // [kBinMaxChunks * bin_ld(N)]  2^(26 c) mod m_i
    const uint32_t *bin_mi26;   // [bin_chunks * bin_ld(N)]     26-bit chunk c of M_i = M / m_i
    const uint32_t *bin_m26;    // [bin_chunks]         26-bit chunk c of M
    int bin_chunks;             // ceil(bits(M) / 26)
    int bin_limbs;              // ceil(bits(M) / 32): 32-bit limbs of an integer below M
    const void *self;           // device copy of this block (set where kernels take it by address)
    GRNS_HD const Consts &get() const { return *this; }
};

/* A kernel's constant-block parameter: the block itself up to 64 moduli, else
 * the address of its device copy -- the 256-moduli block (about 37 KB)
 * exceeds the 32 KB kernel parameter space, and kernels that spread a
 * number's residues over a warp's lanes read 32 different entries at once,
 * which the constant bank serves one address at a time and L1 in one
 * request.  In the kernel: const Consts<N> &C = CA.get(). */
template <int N>
struct ConstsRef {
    const Consts<N> *p;
    GRNS_HD ConstsRef(const Consts<N> &c) : p(static_cast<const Consts<N> *>(c.self)) {}
    GRNS_HD const Consts<N> &get() const { return *p; }
};
template <int N>
using CArg = typename std::conditional<(N > 64), ConstsRef<N>, Consts<N>>::type;
template <int N>
constexpr bool consts_by_address() { return N > 64; }

/* ---------------- modular arithmetic ---------------- */

/* x * w mod m for a constant w with Shoup companion ws = floor(w 2^32 / m); x < 2^32. */
GRNS_HD uint32_t mulmod_shoup(uint32_t x, uint32_t w, uint32_t ws, uint32_t m) {
#ifdef __CUDA_ARCH__
    uint32_t q = __umulhi(x, ws);
#else
    uint32_t q = (uint32_t)(((uint64_t)x * ws) >> 32);
#endif
    uint32_t r = x * w - q * m;  // true value in [0, 2m)
    return r >= m ? r - m : r;
}

GRNS_HD uint32_t umin32(uint32_t a, uint32_t b) { return a < b ? a : b; }

/* x * y mod m for canonical x, y (Barrett, HAC 14.42 in radix 2: quotient
 * estimate within 2 of the true quotient, so r < 3m < 2^32). */
GRNS_HD uint32_t mulmod_barrett(uint32_t x, uint32_t y, uint32_t m, uint32_t mu, uint32_t b) {
    uint64_t p = (uint64_t)x * y;
    uint32_t t = (uint32_t)(p >> (b - 1));
    uint32_t q = (uint32_t)(((uint64_t)t * mu) >> (b + 1));
    uint32_t r = (uint32_t)p - q * m;
    r = umin32(r, r - m);
    return umin32(r, r - m);
}

GRNS_HD uint32_t addmod(uint32_t x, uint32_t y, uint32_t m) {
    uint32_t r = x + y;
    return umin32(r, r - m);
}
GRNS_HD uint32_t submod(uint32_t x, uint32_t y, uint32_t m) {
    uint32_t r = x - y;
    return umin32(r, r + m);
}

/* ---------------- er_float_t (reference src/extrange.cuh) ---------------- */

GRNS_HD uint64_t dbits(double x) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(x);
#else
    uint64_t u;
    __builtin_memcpy(&u, &x, 8);
    return u;
#endif
}
GRNS_HD double bitsd(uint64_t u) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)u);
#else
    double x;
    __builtin_memcpy(&x, &u, 8);
    return x;
#endif
}

/* er_set_d (src/extrange.cuh:75) */
GRNS_HD Er er_from_double(double x) {
    Er r;
    uint64_t u = dbits(x);
    if (x != 0) {
        r.exp = (int64_t)((u & 0x7fffffffffffffffull) >> 52) - 1023;
        r.frac = bitsd((u & 0x800fffffffffffffull) | 0x3ff0000000000000ull);
    } else {
        r.exp = 0;
        r.frac = 0;
    }
    return r;
}

/* er_adjust (src/extrange.cuh:366) */
GRNS_HD void er_adjust(Er &x) {
    uint64_t u = dbits(x.frac);
    int64_t nz = x.frac != 0;
    x.exp = (x.exp + (int64_t)((u & 0x7fffffffffffffffull) >> 52) - 1023) * nz;
    x.frac = bitsd((u & 0x800fffffffffffffull) | 0x3ff0000000000000ull) * (double)nz;
}

/* er_ucmp (src/extrange.cuh:597) */
GRNS_HD int er_ucmp(const Er &x, const Er &y) {
    int diff = (int)(x.exp - y.exp);
    if (diff == 0) return x.frac == y.frac ? 0 : (x.frac > y.frac ? 1 : -1);
    return (x.frac != 0 && (diff > 0 || (diff < 0 && y.frac == 0))) ? 1 : -1;
}

/* exact double of a uint32 built on the integer pipe (avoids the slow
 * I2F.F64 conversion); equals (double)s */
GRNS_HD double u32_to_double(uint32_t s) {
#ifdef __CUDA_ARCH__
    if (s == 0) return 0.0;
    int lz = __clz(s);
    uint64_t bits = ((uint64_t)(1053 - lz) << 52) + ((uint64_t)s << (lz + 21));
    return bitsd(bits);
#else
    return (double)s;
#endif
}

}  // namespace grns
