/*
 * grns_gb300 -- one division (and one power-of-two scaling) per warp, for the
 * 128- and 256-moduli sets.
 *
 * The n-threaded schedule of the reference's division (src/rnsdiv.cuh:244
 * and :301 run one number per block of n threads): here a warp holds one
 * number, lane l the residues i = l + 32 j (j < n / 32), and runs the same
 * digit recurrence as div_fast (rns_fast.cuh) step for step.  The residue
 * work of a step is spread over the lanes; the fixed-point sums fx96w are
 * summed across the warp with butterfly shuffles.  They are integer sums
 * taken mod 2^96 (each lane's partial value, added mod 2^128 and masked), so
 * every lane holds the serial form's value bit for bit and all control flow
 * stays uniform across the warp.  The rare exact comparisons (mixed radix)
 * gather the residues into the warp's shared-memory scratch and run on lane
 * 0, which broadcasts the answer.
 *
 * With one number per thread these sets keep 5.7 to 11 KB of residue arrays
 * a thread in local memory, which lives in L2; here a lane holds 4 or 8
 * residues of each array in registers, and the per-modulus constants come
 * from the block's DivK table in shared memory (a lane reads the same n / 32
 * records for every number).
 *
 * The scaling (scale_warp_coop) runs scale_fast's 52-bit steps the same way:
 * per step the rank's fixed-point sum (exact in 128 bits) and the low bits
 * of X (a sum mod 2^64) are warp sums, the rest is per residue.
 */
#pragma once

#include "div_warp.cuh"

namespace grns {

constexpr unsigned kWarpFull = 0xffffffffu;

/* the sum over the warp of v mod 2^128, in every lane */
__device__ __forceinline__ u128 warp_sum_u128(u128 v) {
    uint64_t lo = (uint64_t)v, hi = (uint64_t)(v >> 64);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const uint64_t l2 = __shfl_xor_sync(kWarpFull, lo, o), h2 = __shfl_xor_sync(kWarpFull, hi, o);
        const uint64_t s = lo + l2;
        hi = hi + h2 + (s < lo ? 1u : 0u);
        lo = s;
    }
    return ((u128)hi << 64) | lo;
}

/* the sum over the warp of v mod 2^64, in every lane */
__device__ __forceinline__ uint64_t warp_sum_u64(uint64_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kWarpFull, v, o);
    return v;
}

/* fx96w over a number spread over the warp (v[j]: residue lane + 32 j) */
template <int N>
__device__ __forceinline__ u128 fx96w_warp(const DivK *K, const uint32_t (&v)[N / 32], int lane) {
    uint64_t S0 = 0, S1 = 0;
    uint32_t S2 = 0;
#pragma unroll
    for (int j = 0; j < N / 32; j++) {
        const uint4 c = K[lane + 32 * j].c;  // c96w_0, c96w_1, c96w_2
        const uint32_t x = v[j];
        const uint64_t p0 = (uint64_t)x * c.x;
        const uint64_t p1 = (uint64_t)x * c.y;
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (uint32_t)(p1 >> 32) + x * c.z;
    }
    return warp_sum_u128((u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64)) & kMask96;
}

/* the warp's residues of two numbers into scratch (a at [0, N), b at [N, 2N)) */
template <int N>
__device__ __forceinline__ void warp_gather2(uint32_t *scratch, const uint32_t (&a)[N / 32], const uint32_t (&b)[N / 32],
                                             int lane) {
    __syncwarp();
#pragma unroll
    for (int j = 0; j < N / 32; j++) {
        scratch[lane + 32 * j] = a[j];
        scratch[N + lane + 32 * j] = b[j];
    }
    __syncwarp();
}

/* dn_normalize for a number spread over the warp */
template <int N>
__device__ __forceinline__ int dn_normalize_warp(const DivK *K, const Consts<N> &C, const uint32_t (&z)[N / 32],
                                                 int lane, int &k, int &bl) {
    uint32_t w[N / 32];
#pragma unroll
    for (int j = 0; j < N / 32; j++) w[j] = z[j];
    k = 0;
    int guard = 0;
    for (;;) {
        const int k0 = k;
        const u128 U = fx96w_warp<N>(K, w, lane);
        const int ns = dn_step<N>(C, U, k, guard);
        if (ns == kNormOk) {
            bl = bitlen128(U);
            k = k0;
        }
        if (ns != kNormMore) return ns;
#pragma unroll
        for (int j = 0; j < N / 32; j++) w[j] = kmag(w[j], K[lane + 32 * j]);
    }
}

/* dv_record for a number pair spread over the warp */
template <int N>
__device__ __forceinline__ uint2 dv_record_warp(const DivK *K, const Consts<N> &C, const uint32_t (&x)[N / 32],
                                                const uint32_t (&d)[N / 32], int lane) {
    bool dz = true, xz = true;
#pragma unroll
    for (int j = 0; j < N / 32; j++) {
        dz &= d[j] == 0;
        xz &= x[j] == 0;
    }
    dz = __all_sync(kWarpFull, dz);
    xz = __all_sync(kWarpFull, xz);
    if (dz) return dv_pack(kDnZero, 0, 0, false);
    int kd, bld;
    const int nd = dn_normalize_warp<N>(K, C, d, lane, kd, bld);
    if (nd == kNormNear) return dv_pack(kDnNear, 0, 0, false);
    if (nd == kNormCap) return dv_pack(kDnCap, 0, 0, false);
    const int s = dv_shift(kd, bld);
    if (xz) return dv_pack(kDnOk, s, s % kDivB - kDivB, false);
    int kx, blx;
    const int nx = dn_normalize_warp<N>(K, C, x, lane, kx, blx);
    if (nx == kNormCap) return dv_pack(kDnCap, 0, 0, false);
    if (nx == kNormNear) return dv_pack(kDnOk, s, s % kDivB - kDivB, true);
    return dv_pack(kDnOk, s, dv_skip(s, kx, blx), false);
}

/* div_fast for one number pair spread over the warp (x, d canonical; q, r
 * this lane's residues of the results); K: the block's DivK table; scratch:
 * 2N words of shared memory for this warp */
template <int N>
__device__ __forceinline__ void div_warp_coop(const DivK *K, const Consts<N> &C, uint32_t (&q)[N / 32],
                                              uint32_t (&r)[N / 32],
                                              const uint32_t (&x)[N / 32], const uint32_t (&d)[N / 32],
                                              uint32_t &flags, int lane, uint32_t *scratch) {
    static_assert(N % 32 == 0, "one warp per number needs n a multiple of 32");
    constexpr int J = N / 32;
    bool xz = true;
#pragma unroll
    for (int j = 0; j < J; j++) {
        q[j] = 0;
        r[j] = x[j];
        xz &= x[j] == 0;
    }
    xz = __all_sync(kWarpFull, xz);
    const uint2 rec = dv_record_warp<N>(K, C, x, d, lane);
    const uint32_t status = rec.x >> 16;
    if (status == kDnZero) {
        flags |= 1u << 1;  // division by zero
        return;
    }
    if (status == kDnCap) {
        flags |= kFxIterCap;
        return;
    }
    if (xz) return;
    if (status == kDnNear) {  // d > M (1 - E / 2^96): the quotient is 0 or 1
        warp_gather2<N>(scratch, x, d, lane);
        int ge = 0;
        if (lane == 0) ge = dv_cmp_vec<N>(C, scratch, scratch + N) >= 0;
        if (__shfl_sync(kWarpFull, ge, 0)) {
#pragma unroll
            for (int j = 0; j < J; j++) {
                q[j] = 1;
                r[j] = submod(r[j], d[j], K[lane + 32 * j].a.x);
            }
        }
        return;
    }
    const int s = (int)(rec.x & 0xffffu), e = dv_rec_e(rec);
    uint32_t D[J], R[J], Q[J];
    const uint32_t *ps = C.pow2 + (int64_t)s * N, *pss = C.pow2_sh + (int64_t)s * N;
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        D[j] = mulmod_shoup(d[j], ldg_u32(ps + i), ldg_u32(pss + i), K[i].a.x);
    }
    DivSt st;
    dv_setup(st, fx96w_warp<N>(K, D, lane), s, e);
    const uint32_t *pe = e < 0 ? C.pow2neg + (int64_t)(-e) * N : C.pow2 + (int64_t)e * N;
    const uint32_t *pes = e < 0 ? C.pow2neg_sh + (int64_t)(-e) * N : C.pow2_sh + (int64_t)e * N;
#pragma unroll
    for (int j = 0; j < J; j++) {
        const int i = lane + 32 * j;
        R[j] = mulmod_shoup(x[j], ldg_u32(pe + i), ldg_u32(pes + i), K[i].a.x);
        Q[j] = 0;
    }
    u128 U = (rec.y >> 31) ? (((u128)1) << 96) : (e < 0 ? fx96w_warp<N>(K, x, lane) : fx96w_warp<N>(K, R, lane));
    for (; st.left > 0; st.left--) {
        const uint64_t qd = dv_digit(st, U, C.E, st.f);
#pragma unroll
        for (int j = 0; j < J; j++) {
            const DivK k = K[lane + 32 * j];
            const uint32_t qi = kred53(qd, k);
            R[j] = submod(kmag(R[j], k), kmulmod(qi, D[j], k), k.a.x);
            Q[j] = addmod(kmag(Q[j], k), qi, k.a.x);
        }
        U = fx96w_warp<N>(K, R, lane);
        st.b = kDivB;
    }
    int c = dv_final_fx(st, U, C.E);
    if (c < 0) {  // dv_final_tie over the warp, then the exact comparisons on lane 0
        c = 0;
        if (st.UD < (((u128)1) << 94)) {
            bool e1 = true, e2 = true, e3 = true;
#pragma unroll
            for (int j = 0; j < J; j++) {
                const uint32_t m = K[lane + 32 * j].a.x, d1 = D[j], d2 = addmod(d1, d1, m);
                e1 &= R[j] == d1;
                e2 &= R[j] == d2;
                e3 &= R[j] == addmod(d2, d1, m);
            }
            e1 = __all_sync(kWarpFull, e1);
            e2 = __all_sync(kWarpFull, e2);
            e3 = __all_sync(kWarpFull, e3);
            c = e1 ? 1 : (e2 ? 2 : (e3 ? 3 : 0));
        }
        if (c == 0) {
            warp_gather2<N>(scratch, R, D, lane);
            if (lane == 0) c = dv_final_exact<N>(C, scratch, scratch + N);
            c = __shfl_sync(kWarpFull, c, 0);
        }
    }
#pragma unroll
    for (int j = 0; j < J; j++) {
        const DivK k = K[lane + 32 * j];
        const uint32_t m = k.a.x;
        q[j] = addmod(Q[j], (uint32_t)c % m, m);
        r[j] = submod(x[j], kmulmod(q[j], d[j], k), m);
    }
    flags |= st.f;
}

/* the top mixed-radix digit of the number in v[0, N) (the rank's tie-break) */
template <int N>
__device__ __noinline__ uint32_t mrc_top_digit(const Consts<N> &C, const uint32_t *v) {
    uint32_t a[N];
    mrc_hd<N>(C, [&](int i) { return v[i]; }, a);
    return a[N - 1];
}

/* rank_fast for a number spread over the warp (c[j] = x w mod m of residue
 * lane + 32 j); scratch: N words of shared memory for this warp */
template <int N>
__device__ __forceinline__ uint32_t rank_warp(const Consts<N> &C, const uint32_t (&x)[N / 32],
                                              const uint32_t (&c)[N / 32], bool small, int lane, uint32_t *scratch) {
    uint64_t S0 = 0, S1 = 0, S2 = 0;
#pragma unroll
    for (int j = 0; j < N / 32; j++) {
        const int i = lane + 32 * j;
        const uint32_t sv = c[j];
        const uint64_t p0 = (uint64_t)sv * C.c96_0[i];
        const uint64_t p1 = (uint64_t)sv * C.c96_1[i];
        const uint64_t p2 = (uint64_t)sv * C.c96_2[i];
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (p1 >> 32) + p2;
    }
    const u128 t = warp_sum_u128((u128)S0 + ((u128)S1 << 32) + ((u128)S2 << 64));
    const uint32_t kk = (uint32_t)(t >> 96);
    if ((t & kMask96) >= (u128)C.E || small) return kk;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < N / 32; j++) scratch[lane + 32 * j] = x[j];
    __syncwarp();
    uint32_t top = 0;
    if (lane == 0) top = mrc_top_digit<N>(C, scratch);
    top = __shfl_sync(kWarpFull, top, 0);
    return top == 0 ? kk : kk - 1;
}

/* scale_fast for a number spread over the warp (x canonical; res this lane's
 * residues of floor(X / 2^D)); scratch: N words of shared memory for this warp */
template <int N>
__device__ __forceinline__ void scale_warp_coop(const Consts<N> &C, uint32_t (&res)[N / 32],
                                                const uint32_t (&x)[N / 32], unsigned D, int lane,
                                                uint32_t *scratch) {
    constexpr int J = N / 32;
    uint32_t cur[J], c[J];
#pragma unroll
    for (int j = 0; j < J; j++) cur[j] = x[j];
    if (D > (unsigned)C.log2M) {  // X < M < 2^(log2M + 1): the result is 0
#pragma unroll
        for (int j = 0; j < J; j++) res[j] = 0;
        return;
    }
    bool small = false;
#pragma unroll 1
    for (unsigned left = D; left > 0;) {
        const int step = left < (unsigned)kScaleB ? (int)left : kScaleB;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = lane + 32 * j;
            c[j] = mulmod_shoup(cur[j], C.w[i], C.w_sh[i], C.m[i]);
        }
        const uint32_t k = rank_warp<N>(C, cur, c, small, lane, scratch);
        /* scaling_step_big: X mod 2^step from the CRT sum in 64-bit wrap-around arithmetic */
        uint64_t acc = 0;
#pragma unroll
        for (int j = 0; j < J; j++) acc += (uint64_t)c[j] * C.mi64[lane + 32 * j];
        acc = warp_sum_u64(acc);
        const uint64_t low = (acc - (uint64_t)k * C.m64) & ((((uint64_t)1) << step) - 1);
        const uint32_t *inv = C.pow2neg + (int64_t)step * N, *inv_sh = C.pow2neg_sh + (int64_t)step * N;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = lane + 32 * j;
            const uint32_t m = C.m[i];
            cur[j] = mulmod_shoup(submod(cur[j], reduce53<N>(C, i, low), m), ldg_u32(inv + i), ldg_u32(inv_sh + i), m);
        }
        left -= (unsigned)step;
        small = true;
    }
#pragma unroll
    for (int j = 0; j < J; j++) res[j] = cur[j];
}

}  // namespace grns
