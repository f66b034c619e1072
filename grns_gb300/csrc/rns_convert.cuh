/*
 * grns_gb300 -- binary <-> RNS conversion, host+device arithmetic.
 *
 * Integers travel as little-endian 32-bit limbs.  Both directions work on
 * 26-bit chunks so that every sum of products fits one 64-bit word (up to
 * 64 moduli and kBinSumMax chunks; longer chunk sums are reduced every
 * kBinFold products, and more than 64 moduli sum in 128 bits):
 *
 *   from binary (rns_from_binary, reference src/rnsbase.cuh:253, which takes
 *   mpz_mod_ui per modulus): x_i = sum_c chunk_c * (2^(26 c) mod m_i) mod m_i,
 *   one 64-bit accumulator per residue, one reduction at the end;
 *
 *   to binary (rns_to_binary, src/rnsbase.cuh:277: sum_i x_i B_i mod M with
 *   the orthogonal bases B_i = M_i w_i): with s_i = x_i w_i mod m_i,
 *   X = sum_i s_i M_i - k M where k = floor(sum_i s_i / m_i).  k comes from the
 *   96-bit fixed-point sum with ceil(2^96 / m_i), which exceeds the true sum
 *   by less than sum_i (m_i - 1) / 2^96 < 1, so it is k or k + 1.  The chunks
 *   of sum_i s_i M_i - k M are formed with a signed carry; a negative final
 *   carry means the estimate was k + 1, and adding M back fixes it.  No mixed-
 *   radix fallback is needed, and the work is the same for every input.
 */
#pragma once

#include "rns_common.cuh"

namespace grns {

constexpr uint32_t kBinMask = (1u << kBinChunk) - 1u;
/* products of a 26-bit chunk and a residue below 2^30.42 whose sum stays below 2^64 */
constexpr int kBinSumMax = 158;

/* the CRT chunk sums: 64-bit up to 64 moduli, 128-bit above (n products of 56.42 bits) */
template <int N>
using BinAcc = typename std::conditional<(N > 64), unsigned __int128, uint64_t>::type;
template <int N>
using BinSAcc = typename std::conditional<(N > 64), __int128, int64_t>::type;

/* chunk c (bits [26 c, 26 c + 26)) of the little-endian limbs row[0..nlimbs) */
GRNS_HD uint32_t bin_chunk(const uint32_t *row, int nlimbs, int c) {
    const int bit = kBinChunk * c, j = bit >> 5, off = bit & 31;
    const uint64_t lo = j < nlimbs ? row[j] : 0u;
    const uint64_t hi = j + 1 < nlimbs ? row[j + 1] : 0u;
    return (uint32_t)(((hi << 32) | lo) >> off) & kBinMask;
}

/* v mod m for any 64-bit v: the high word by Barrett (b >= 16) and 2^32 mod m */
template <int N>
GRNS_HD uint32_t bin_mod64(const Consts<N> &C, int i, uint64_t v) {
    const uint32_t m = C.m[i];
    if (C.b[i] < 16) return (uint32_t)(v % m);
    const uint32_t h = mulmod_barrett((uint32_t)(v >> 32), 1u, m, C.mu[i], C.b[i]);
    const uint32_t l = mulmod_barrett((uint32_t)v, 1u, m, C.mu[i], C.b[i]);
    return addmod(mulmod_shoup(h, C.t32[i], C.t32_sh[i], m), l, m);
}

/* residues of the integer in row[0..nlimbs) (nlimbs <= kBinMaxLimbs) */
template <int N>
GRNS_HD void from_binary(const Consts<N> &C, const uint32_t *row, int nlimbs, uint32_t *res) {
    const int chunks = (32 * nlimbs + kBinChunk - 1) / kBinChunk;
    for (int i = 0; i < N; i++) {
        uint64_t acc = 0;
        for (int c = 0; c < chunks; c++) {
            acc += (uint64_t)bin_chunk(row, nlimbs, c) * C.bin_p26[c * bin_ld(N) + i];
            if (chunks > kBinSumMax && c % kBinFold == kBinFold - 1) acc = bin_mod64<N>(C, i, acc);
        }
        res[i] = bin_mod64<N>(C, i, acc);
    }
}

/* k or k + 1 for k = floor(sum_i s_i / m_i) */
template <int N>
GRNS_HD uint32_t bin_rank(const Consts<N> &C, const uint32_t *s) {
    uint64_t S0 = 0, S1 = 0, S2 = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint64_t p0 = (uint64_t)s[i] * C.c96_0[i];
        const uint64_t p1 = (uint64_t)s[i] * C.c96_1[i];
        const uint64_t p2 = (uint64_t)s[i] * C.c96_2[i];
        S0 += (uint32_t)p0;
        S1 += (p0 >> 32) + (uint32_t)p1;
        S2 += (p1 >> 32) + p2;
    }
    const unsigned __int128 t = (unsigned __int128)S0 + ((unsigned __int128)S1 << 32) + ((unsigned __int128)S2 << 64);
    return (uint32_t)(t >> 96);
}

/* one chunk of sum_i s_i M_i - kk M plus the signed carry */
template <int N>
GRNS_HD uint32_t bin_crt_chunk(const Consts<N> &C, const uint32_t *s, uint32_t kk, int c, int64_t &carry) {
    BinAcc<N> acc = 0;
    const uint32_t *row = C.bin_mi26 + (size_t)c * bin_ld(N);
    for (int i = 0; i < N; i++) acc += (BinAcc<N>)s[i] * row[i];
    const BinSAcc<N> v = (BinSAcc<N>)acc - (BinSAcc<N>)kk * C.bin_m26[c] + carry;
    carry = (int64_t)(v >> kBinChunk);  // floor division (arithmetic shift)
    return (uint32_t)v & kBinMask;
}

/* adds M to the chunks d[0..chunks) (the estimate of k was one too high) */
template <int N>
GRNS_HD void bin_add_m(const Consts<N> &C, uint32_t *d, int stride) {
    uint32_t carry = 0;
    for (int c = 0; c < C.bin_chunks; c++) {
        const uint32_t v = d[c * stride] + C.bin_m26[c] + carry;
        d[c * stride] = v & kBinMask;
        carry = v >> kBinChunk;
    }
}

/* packs 26-bit chunks d[0..chunks) into 32-bit limbs d[0..limbs) in place
 * (limb l reads chunks floor(32 l / 26) .. + 2, never below l) */
GRNS_HD void bin_pack(uint32_t *d, int stride, int chunks, int limbs) {
    for (int l = 0; l < limbs; l++) {
        const int bit = 32 * l, c = bit / kBinChunk, off = bit - c * kBinChunk;
        uint64_t w = c < chunks ? (uint64_t)(d[c * stride] >> off) : 0u;
        if (c + 1 < chunks) w |= (uint64_t)d[(c + 1) * stride] << (kBinChunk - off);
        if (c + 2 < chunks) w |= (uint64_t)d[(c + 2) * stride] << (2 * kBinChunk - off);
        d[l * stride] = (uint32_t)w;
    }
}

/* X in [0, M) as C.bin_limbs limbs in d[0..], d holding C.bin_chunks words;
 * returns false (and zeros) for a residue >= its modulus */
template <int N, class Get>
GRNS_HD bool to_binary(const Consts<N> &C, Get x, uint32_t *d, int stride) {
    uint32_t s[N];
    bool bad = false;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        const uint32_t v = x(i);
        bad |= v >= C.m[i];
        s[i] = mulmod_shoup(v, C.w[i], C.w_sh[i], C.m[i]);
    }
    if (bad) {
        for (int c = 0; c < C.bin_chunks; c++) d[c * stride] = 0;
        return false;
    }
    const uint32_t kk = bin_rank<N>(C, s);
    int64_t carry = 0;
    for (int c = 0; c < C.bin_chunks; c++) d[c * stride] = bin_crt_chunk<N>(C, s, kk, c, carry);
    if (carry < 0) bin_add_m<N>(C, d, stride);
    bin_pack(d, stride, C.bin_chunks, C.bin_limbs);
    return true;
}

}  // namespace grns
