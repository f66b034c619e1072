/*
 * grns_gb300 -- multiple-precision integers (mp_int_t, reference layout
 * src/types.cuh:45): add / sub / mul with the interval evaluation derived
 * from the operands' evaluations, as cuda::mpint_add / mpint_sub /
 * mpint_mul (reference src/mpint.cuh:336/:407/:478).  Overflow becomes flag
 * bits (the reference prints from the device).
 */
#pragma once

#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

/* byte layout of the reference mp_int_t for n = N: digits, sign, then the
 * 8-byte aligned evaluation -- 4 bytes of padding after the sign for even N,
 * none for odd N */
template <int N, bool EVEN = (N % 2 == 0)>
struct MpIntT;
template <int N>
struct MpIntT<N, true> {
    uint32_t digits[N];
    int32_t sign;
    int32_t pad;  // written as 0
    Er eval[2];
};
template <int N>
struct MpIntT<N, false> {
    uint32_t digits[N];
    int32_t sign;
    Er eval[2];
};
template <int N>
using MpInt = MpIntT<N>;
template <int N>
__host__ __device__ __forceinline__ void clear_pad(MpIntT<N, true> &r) {
    r.pad = 0;
}
template <int N>
__host__ __device__ __forceinline__ void clear_pad(MpIntT<N, false> &) {}
static_assert(sizeof(MpInt<8>) == 72 && sizeof(MpInt<32>) == 168 && sizeof(MpInt<64>) == 296 &&
                  sizeof(MpInt<5>) == 56 && sizeof(MpInt<15>) == 96,
              "mp_int_t layout");

__device__ __forceinline__ double neg_if(double v, bool neg) { return neg ? -v : v; }

/* the digits of an array of mp_int_t records as an operand / output of the
 * warp division driver (digit i of record k) */
template <int N>
struct MpDigitsIn {
    const uint32_t *base;  // record 0
    static constexpr int RW = (int)(sizeof(MpInt<N>) / 4);
    __device__ __forceinline__ uint32_t load(int64_t k, int i) const { return __ldg(base + k * RW + i); }
    __device__ __forceinline__ void prefetch_l2(int64_t k) const {
        asm volatile("prefetch.global.L2 [%0];" ::"l"(base + k * RW));
    }
};
template <int N>
struct MpDigitsOut {
    uint32_t *base;
    static constexpr int RW = (int)(sizeof(MpInt<N>) / 4);
    __device__ __forceinline__ void store(int64_t k, int i, uint32_t v) const { base[k * RW + i] = v; }
};

/* mpint_div's last step (reference src/mpint.cuh:511): from the division of
 * the magnitudes (quotient digits q(i), remainder digits r(i), its flags f),
 * the Euclidean quotient -- one more when the dividend is negative and the
 * remainder nonzero, so that x = q y + r with 0 <= r < |y| -- its
 * evaluation and sign; an invalid digit or a zero divisor gives the zero
 * record.  res: digits, sign, evaluation and padding written. */
template <int N, class GQ, class GR>
__device__ __forceinline__ void mpint_div_finish(const Consts<N> &C, int xs, int ys, GQ q, GR r, uint32_t &f,
                                                 MpInt<N> &res) {
    const bool bad = (f & (kFlagInvalidInput | kFlagDivByZero)) != 0;
    bool rz = true;
#pragma unroll 8
    for (int i = 0; i < N; i++) rz &= r(i) == 0;
    const bool inc = xs == 1 && !rz && !bad;
    bool qz = true;
#pragma unroll 8
    for (int i = 0; i < N; i++) {
        uint32_t v = bad ? 0u : q(i);
        if (inc) v = addmod(v, 1u, C.m[i]);
        res.digits[i] = v;
        qz &= v == 0;
    }
    eval<N>(C, [&](int i) { return res.digits[i]; }, res.eval[0], res.eval[1], f);
    res.sign = qz ? 0 : (xs ^ ys);
    clear_pad(res);
}

/* er_md_rd / er_md_ru (src/extrange.cuh:557/:566) with the product and the
 * quotient on the integer pipe (dmuldiv_dir_i; z_rcp = dmuldiv_recip(z.frac)),
 * the FP64 instructions where it defers; the same bits as er_md */
template <bool UP>
__device__ __forceinline__ Er er_md_i(const Er &x, const Er &y, const Er &z, uint64_t z_rcp) {
    Er r;
    r.exp = x.exp + y.exp - z.exp;
    double q;
    if (!dmuldiv_dir_i(x.frac, y.frac, z.frac, UP, q, z_rcp))
        q = UP ? __ddiv_ru(__dmul_ru(x.frac, y.frac), z.frac) : __ddiv_rd(__dmul_rd(x.frac, y.frac), z.frac);
    r.frac = q;
    er_adjust_i(r);
    return r;
}

/* the sign and evaluation of an mp_int (the part of the record besides the digits) */
struct MpIntHead {
    int32_t sign;
    Er eval[2];
};
template <int N>
__device__ __forceinline__ MpIntHead head_of(const MpInt<N> &x) {
    return MpIntHead{x.sign, {x.eval[0], x.eval[1]}};
}

/* the interval of x + y (sub: x - y) by interval addition of the signed
 * evaluations, and whether the result is negative (both bounds below 0, the
 * reference's rule, src/mpint.cuh:381); lo / up are the result's bounds
 * after the sign is taken out */
__device__ __forceinline__ bool mpint_addsub_eval(const MpIntHead &x, const MpIntHead &y, bool sub, Er &lo, Er &up) {
    const int sx = x.sign, sy = sub ? (y.sign ^ 1) : y.sign;
    Er evx[2] = {x.eval[0], x.eval[1]}, evy[2] = {y.eval[0], y.eval[1]};
    evx[0].frac = dflip_i(evx[0].frac, sx);
    evx[1].frac = dflip_i(evx[1].frac, sx);
    evy[0].frac = dflip_i(evy[0].frac, sy);
    evy[1].frac = dflip_i(evy[1].frac, sy);
    lo = er_add_dir_i<false>(evx[sx], evy[sy]);
    up = er_add_dir_i<true>(evx[1 - sx], evy[1 - sy]);
    const bool minus = dneg_i(lo.frac) && dneg_i(up.frac);
    if (minus) {
        const Er t = lo;
        lo = Er{dflip_i(up.frac, true), up.exp};
        up = Er{dflip_i(t.frac, true), t.exp};
    }
    return minus;
}

/* digit i of x + y (sub: x - y) for a result of sign `minus` */
__device__ __forceinline__ uint32_t mpint_addsub_digit(uint32_t a, uint32_t b, uint32_t m, int sx, int sy, bool minus,
                                                       uint32_t &flags) {
    flags |= (a >= m || b >= m) ? kFlagInvalidInput : 0u;
    const uint32_t sa = sx ? submod(0u, a, m) : a;
    const uint32_t sb = sy ? submod(0u, b, m) : b;
    const uint32_t d = addmod(sa, sb, m);
    return minus ? (d ? m - d : 0u) : d;
}

template <int N>
__device__ __forceinline__ void mpint_addsub(const Consts<N> &C, MpInt<N> &res, const MpInt<N> &x, const MpInt<N> &y,
                                             bool sub, uint32_t &flags) {
    Er lo, up;
    const bool minus = mpint_addsub_eval(head_of(x), head_of(y), sub, lo, up);
    const int sx = x.sign, sy = sub ? (y.sign ^ 1) : y.sign;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) res.digits[i] = mpint_addsub_digit(x.digits[i], y.digits[i], C.m[i], sx, sy, minus, flags);
    res.sign = minus;
    res.eval[0] = lo;
    res.eval[1] = up;
    flags |= overflow_flags_i<N>(C, lo, up);
}

template <int N>
__device__ __forceinline__ void mpint_mul(const Consts<N> &C, MpInt<N> &res, const MpInt<N> &x, const MpInt<N> &y,
                                          uint32_t &flags) {
    res.eval[0] = er_md_i<false>(x.eval[0], y.eval[0], C.unit_upp, C.unit_rcp_upp);
    res.eval[1] = er_md_i<true>(x.eval[1], y.eval[1], C.unit_low, C.unit_rcp_low);
    bool zero = true;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t m = C.m[i], a = x.digits[i], b = y.digits[i];
        flags |= (a >= m || b >= m) ? kFlagInvalidInput : 0u;
        uint32_t v = mulmod_barrett(a, b, m, C.mu[i], C.b[i]);
        res.digits[i] = v;
        zero &= v == 0;
    }
    res.sign = zero ? 0 : (x.sign ^ y.sign);
    flags |= overflow_flags_i<N>(C, res.eval[0], res.eval[1]);
}

}  // namespace grns
