/*
 * grns_gb300 -- host computation of a moduli set's constant tables (plain
 * C++, no CUDA), shared by the device context (ctx.cu) and the CPU checks of
 * the integer algorithms.
 *
 * Reference tables (rns_const_init, kisupov/grns src/rnsbase.cuh:324-451)
 * reproduced bit for bit without GMP/MPFR: M is only needed as its bit
 * length and its top 53 bits (MPFR rounds M down to 53 bits before 1/M is
 * taken), everything else is a product, power or inverse modulo a 31-bit
 * modulus or a power of two.  Plus the tables of the integer fast path:
 * fixed-point reciprocals ceil(2^64/m_i), ceil(2^96/m_i), 2^32 mod m_i,
 * Shoup companions, and the bit lengths of the mixed-radix weights.
 */
#pragma once

#include <cmath>
#include <cstdint>
#include <vector>

#include "rns_common.cuh"

namespace grns {

struct HostTables {
    int n = 0, log2M = 0;
    std::vector<uint32_t> m, w, w_sh, mu, bits;
    std::vector<double> rrd, rru;
    double acc = 0;
    int ref_factor = 0;
    Er unit_low{}, unit_upp{}, inv_unit_low{}, inv_unit_upp{};
    std::vector<uint32_t> pow2, pow2_sh;          // (log2M+1) x n
    std::vector<uint32_t> mrc_inv, mrc_inv_sh;    // n x n, [j*n+i] = m_j^-1 mod m_i (j < i)
    std::vector<uint32_t> mi_pow2, m_pow2, pow2_inv, pow2_inv_sh;  // 30 x n, 30, 30 x n, 30 x n
    std::vector<uint32_t> c64l, c64h, c96_0, c96_1, c96_2, t32, t32_sh, mrbits;
    std::vector<uint32_t> c96k;  // (log2M+1) x n x 4 words: ceil(2^96 (2^k w_i mod m_i)/m_i) mod 2^96, 0
    std::vector<uint32_t> b48, b48_sh;           // 2^kDivB mod m_i
    std::vector<uint64_t> evl_lo, evl_hi, evu_lo, evu_hi;  // recip_rd / recip_ru * 2^100
    uint64_t acc_lo = 0, acc_hi = 0;             // ceil(acc * 2^100)
    std::vector<uint32_t> c128w;                 // n x 4 words: ceil(2^128 w_i / m_i) mod 2^128
    std::vector<uint32_t> pow2neg, pow2neg_sh;   // kPow2NegRows x n: 2^-j mod m_i
    /* division, residue-major (a lane's row lookups for one residue stay within a few cache
     * lines): pairs (2^j mod m_i, Shoup companion), [i * 64 + j] for j < 64 and
     * [i * pow2_hi_rows + a] for 2^(64 a); the same for 2^-j and 2^-(64 a) */
    std::vector<uint32_t> p2lo, p2hi, p2nlo, p2nhi;
    std::vector<uint64_t> mi64;                  // M_i mod 2^64
    uint64_t m64 = 0;                            // M mod 2^64
    uint64_t E = 0;  // sum_i (m_i - 1)
    std::vector<uint32_t> bin_p26;               // kBinMaxChunks x bin_ld(n): 2^(26 c) mod m_i
    std::vector<uint32_t> bin_mi26;              // bin_chunks x bin_ld(n): 26-bit chunks of M_i
    std::vector<uint32_t> bin_m26;               // bin_chunks, padded to a multiple of 4: chunks of M
    int bin_chunks = 0, bin_limbs = 0;
};

namespace hostdetail {

inline int64_t inverse_mod(int64_t x, int64_t m) {
    int64_t a = ((x % m) + m) % m, b = m, x0 = 1, x1 = 0;
    while (b) {
        int64_t q = a / b, t = a - q * b;
        a = b;
        b = t;
        t = x0 - q * x1;
        x0 = x1;
        x1 = t;
    }
    return ((x0 % m) + m) % m;
}

/* ddiv_rd/ddiv_ru(1, m) with the reference's host rounding (src/dinterval.cuh:124-136):
 * the round-to-nearest quotient moved by PHI1*|c| + ETA; volatile keeps the
 * multiply and add unfused. */
inline double recip_host(double m, bool up) {
    volatile double c = 1.0 / m;
    volatile double phi1 = 0x1p-53 * (1.0 + 2.0 * 0x1p-53);
    volatile double t = phi1 * std::fabs(c);
    volatile double e = t + 0x1p-1074;
    return up ? c + e : c - e;
}

/* directed rounding of 0 < p/q <= 1 to 53 bits, as mpfr_get_d_2exp reports
 * it: frac in [0.5, 1), value = frac * 2^exp */
inline void round_ratio(uint64_t p, uint64_t q, bool up, double &frac, int64_t &exp) {
    const unsigned __int128 lo = (unsigned __int128)1 << 52;
    int s = 0;
    while (((unsigned __int128)p << s) / q < lo) s++;
    unsigned __int128 num = (unsigned __int128)p << s;
    unsigned __int128 mant = num / q, rem = num % q;
    if (up && rem) mant += 1;
    if (mant == ((unsigned __int128)1 << 53)) {
        mant >>= 1;
        s -= 1;
    }
    frac = std::ldexp((double)(uint64_t)mant, -53);
    exp = 53 - s;
}

inline uint32_t shoup(uint32_t v, uint32_t m) { return (uint32_t)(((uint64_t)v << 32) / m); }

/* v * 2^100 for a positive double v, rounded up when not an integer */
inline void fx100_of(double v, uint64_t &lo, uint64_t &hi) {
    int e;
    const double f = std::frexp(v, &e);  // v = f 2^e, f in [0.5, 1)
    const uint64_t M = (uint64_t)std::ldexp(f, 53);
    const int sh = e + 47;               // v 2^100 = M 2^(e + 47)
    unsigned __int128 r;
    if (sh >= 0) {
        r = (unsigned __int128)M << sh;
    } else {
        r = (unsigned __int128)M >> (-sh);
        if (M & ((((uint64_t)1) << (-sh)) - 1)) r += 1;
    }
    lo = (uint64_t)r;
    hi = (uint64_t)(r >> 64);
}

}  // namespace hostdetail

/* Fills every table for the moduli m[0..n-1] (odd, pairwise coprime, validated by the caller). */
inline void build_tables(HostTables &T, const uint32_t *mod, int n) {
    using namespace hostdetail;
    T.n = n;
    T.m.assign(mod, mod + n);
    const std::vector<uint32_t> &m = T.m;
    std::vector<uint32_t> M(1, 1u);
    for (int i = 0; i < n; i++) {
        uint64_t carry = 0;
        for (auto &limb : M) {
            uint64_t t = (uint64_t)limb * m[i] + carry;
            limb = (uint32_t)t;
            carry = t >> 32;
        }
        if (carry) M.push_back((uint32_t)carry);
    }
    int bitlen = 32 * (int)(M.size() - 1);
    for (uint32_t top = M.back(); top; top >>= 1) bitlen++;
    T.log2M = bitlen - 1;
    const int Eb = bitlen > 53 ? bitlen - 53 : 0;
    uint64_t Top = 0;
    for (int bit = bitlen - 1; bit >= Eb; bit--) Top = (Top << 1) | ((M[bit / 32] >> (bit % 32)) & 1u);

    T.w.resize(n); T.w_sh.resize(n); T.mu.resize(n); T.bits.resize(n); T.rrd.resize(n); T.rru.resize(n);
    T.c64l.resize(n); T.c64h.resize(n); T.c96_0.resize(n); T.c96_1.resize(n); T.c96_2.resize(n);
    T.t32.resize(n); T.t32_sh.resize(n); T.mrbits.resize(n);
    T.evl_lo.resize(n); T.evl_hi.resize(n); T.evu_lo.resize(n); T.evu_hi.resize(n);
    T.E = 0;
    for (int i = 0; i < n; i++) {
        int64_t mi = 1;
        for (int j = 0; j < n; j++)
            if (j != i) mi = (mi * (m[j] % m[i])) % m[i];
        T.w[i] = (uint32_t)inverse_mod(mi, m[i]);
        T.w_sh[i] = shoup(T.w[i], m[i]);
        uint32_t b = 0;
        for (uint32_t v = m[i]; v; v >>= 1) b++;
        T.bits[i] = b;
        T.mu[i] = (uint32_t)(((unsigned __int128)1 << (2 * b)) / m[i]);
        T.rrd[i] = recip_host((double)m[i], false);
        T.rru[i] = recip_host((double)m[i], true);
        fx100_of(T.rrd[i], T.evl_lo[i], T.evl_hi[i]);
        fx100_of(T.rru[i], T.evu_lo[i], T.evu_hi[i]);
        unsigned __int128 c64 = ((((unsigned __int128)T.w[i]) << 64) + m[i] - 1) / m[i];  /* w-folded */
        T.c64l[i] = (uint32_t)c64;
        T.c64h[i] = (uint32_t)(c64 >> 32);
        unsigned __int128 two96 = ((unsigned __int128)1) << 96;
        unsigned __int128 c96 = (two96 + m[i] - 1) / m[i];
        T.c96_0[i] = (uint32_t)c96;
        T.c96_1[i] = (uint32_t)(c96 >> 32);
        T.c96_2[i] = (uint32_t)(c96 >> 64);
        T.t32[i] = (uint32_t)((((uint64_t)1) << 32) % m[i]);
        T.t32_sh[i] = shoup(T.t32[i], m[i]);
        T.E += m[i] - 1;
    }
    /* ceil(2^128 w_i / m_i) by long division in 32-bit steps (w_i < m_i) */
    T.c128w.assign((size_t)n * 4, 0);
    for (int i = 0; i < n; i++) {
        uint64_t r = T.w[i];
        uint32_t q[4];
        for (int j = 3; j >= 0; j--) {
            const uint64_t v = r << 32;
            q[j] = (uint32_t)(v / m[i]);
            r = v % m[i];
        }
        if (r) {  // round up, carrying through the words (mod 2^128)
            for (int j = 0; j < 4; j++)
                if (++q[j] != 0) break;
        }
        for (int j = 0; j < 4; j++) T.c128w[(size_t)i * 4 + j] = q[j];
    }
    /* bit length of P_t = m_0 * ... * m_{t-1} */
    {
        std::vector<uint32_t> P(1, 1u);
        for (int t = 0; t < n; t++) {
            int bl = 32 * (int)(P.size() - 1);
            for (uint32_t top = P.back(); top; top >>= 1) bl++;
            T.mrbits[t] = (uint32_t)bl;
            uint64_t carry = 0;
            for (auto &limb : P) {
                uint64_t v = (uint64_t)limb * m[t] + carry;
                limb = (uint32_t)v;
                carry = v >> 32;
            }
            if (carry) P.push_back((uint32_t)carry);
        }
    }
    /* RNS_EVAL_ACCURACY, RNS_EVAL_REF_FACTOR (src/rnsbase.cuh:389-391), same operation order */
    volatile double acc = 4 * std::pow(2.0, 1 - 53);
    acc = acc * n;
    acc = acc * std::log2((double)n);
    acc = acc * (1 + 0.0000001 / 2);
    acc = acc / 0.0000001;
    T.acc = acc;
    fx100_of(T.acc, T.acc_lo, T.acc_hi);
    T.ref_factor = (int)std::floor(std::log2(1 / (2 * T.acc)));
    /* RNS_EVAL_UNIT ~ 1/M53 and RNS_EVAL_INV_UNIT ~ 1 - 1/M53 (src/rnsbase.cuh:393-411) */
    round_ratio(1, Top, false, T.unit_low.frac, T.unit_low.exp);
    round_ratio(1, Top, true, T.unit_upp.frac, T.unit_upp.exp);
    T.unit_low.exp -= Eb;
    T.unit_upp.exp -= Eb;
    if (Eb == 0) {
        round_ratio(Top - 1, Top, false, T.inv_unit_low.frac, T.inv_unit_low.exp);
        round_ratio(Top - 1, Top, true, T.inv_unit_upp.frac, T.inv_unit_upp.exp);
    } else if (Eb == 1 && Top == ((uint64_t)1 << 52)) {
        T.inv_unit_low = T.inv_unit_upp = Er{1.0 - 0x1p-53, 0};
    } else {
        T.inv_unit_low = Er{1.0 - 0x1p-53, 0};
        T.inv_unit_upp = Er{0.5, 1};
    }
    /* RNS_POW2[j][i] = 2^j mod m_i, with Shoup companions */
    T.pow2.resize((size_t)(T.log2M + 1) * n);
    T.pow2_sh.resize(T.pow2.size());
    for (int i = 0; i < n; i++) {
        uint64_t v = 1;
        for (int j = 0; j <= T.log2M; j++) {
            T.pow2[(size_t)j * n + i] = (uint32_t)v;
            T.pow2_sh[(size_t)j * n + i] = shoup((uint32_t)v, m[i]);
            v = (v * 2) % m[i];
        }
    }
    /* magnification rows: ceil(2^96 u / m_i) mod 2^96 with u = 2^k w_i mod m_i */
    T.c96k.assign((size_t)(T.log2M + 1) * n * 4, 0);
    for (int i = 0; i < n; i++) {
        for (int k = 0; k <= T.log2M; k++) {
            uint64_t u = ((uint64_t)T.pow2[(size_t)k * n + i] * T.w[i]) % m[i];
            unsigned __int128 c = ((((unsigned __int128)u) << 96) + m[i] - 1) / m[i];
            uint32_t *row = &T.c96k[((size_t)k * n + i) * 4];
            row[0] = (uint32_t)c;
            row[1] = (uint32_t)(c >> 32);
            row[2] = (uint32_t)(c >> 64);
        }
    }
    /* division and scaling: 2^kDivB mod m_i and 2^-j mod m_i for j < kPow2NegRows */
    T.b48.resize(n);
    T.b48_sh.resize(n);
    T.pow2neg.resize((size_t)kPow2NegRows * n);
    T.pow2neg_sh.resize(T.pow2neg.size());
    for (int i = 0; i < n; i++) {
        uint64_t v = 1;
        for (int j = 0; j < kDivB; j++) v = (v * 2) % m[i];
        T.b48[i] = (uint32_t)v;
        T.b48_sh[i] = shoup((uint32_t)v, m[i]);
        const uint64_t half = (m[i] + 1) / 2;  // 2^-1 mod m_i (m_i odd)
        uint64_t u = 1;
        for (int j = 0; j < kPow2NegRows; j++) {
            T.pow2neg[(size_t)j * n + i] = (uint32_t)u;
            T.pow2neg_sh[(size_t)j * n + i] = shoup((uint32_t)u, m[i]);
            u = (u * half) % m[i];
        }
    }
    /* division: 2^s = 2^(s mod 64) 2^(64 floor(s / 64)) and 2^-s likewise, for every shift s < 64 rows */
    const int rows = pow2_hi_rows(T.log2M);
    T.p2lo.assign((size_t)n * 64 * 2, 0);
    T.p2nlo.assign((size_t)n * 64 * 2, 0);
    T.p2hi.assign((size_t)n * rows * 2, 0);
    T.p2nhi.assign((size_t)n * rows * 2, 0);
    for (int i = 0; i < n; i++) {
        const uint64_t half = (m[i] + 1) / 2;  // 2^-1 mod m_i
        uint64_t up = 1, dn = 1;
        for (int j = 0; j < 64; j++) {
            T.p2lo[((size_t)i * 64 + j) * 2] = (uint32_t)up;
            T.p2lo[((size_t)i * 64 + j) * 2 + 1] = shoup((uint32_t)up, m[i]);
            T.p2nlo[((size_t)i * 64 + j) * 2] = (uint32_t)dn;
            T.p2nlo[((size_t)i * 64 + j) * 2 + 1] = shoup((uint32_t)dn, m[i]);
            up = (up * 2) % m[i];
            dn = (dn * half) % m[i];
        }
        const uint64_t up64 = up, dn64 = dn;  // 2^64 and 2^-64 mod m_i
        up = dn = 1;
        for (int a = 0; a < rows; a++) {
            T.p2hi[((size_t)i * rows + a) * 2] = (uint32_t)up;
            T.p2hi[((size_t)i * rows + a) * 2 + 1] = shoup((uint32_t)up, m[i]);
            T.p2nhi[((size_t)i * rows + a) * 2] = (uint32_t)dn;
            T.p2nhi[((size_t)i * rows + a) * 2 + 1] = shoup((uint32_t)dn, m[i]);
            up = (up * up64) % m[i];
            dn = (dn * dn64) % m[i];
        }
    }
    /* scaling: M_i mod 2^64 and M mod 2^64 */
    T.mi64.assign(n, 0);
    T.m64 = 1;
    for (int i = 0; i < n; i++) T.m64 *= m[i];
    for (int i = 0; i < n; i++) {
        uint64_t v = 1;
        for (int j = 0; j < n; j++)
            if (j != i) v *= m[j];
        T.mi64[i] = v;
    }
    /* MRC_MULT_INV as [j*n + i] = m_j^-1 mod m_i for j < i */
    T.mrc_inv.assign((size_t)n * n, 0);
    T.mrc_inv_sh.assign((size_t)n * n, 0);
    for (int j = 0; j < n; j++)
        for (int i = j + 1; i < n; i++) {
            uint32_t v = (uint32_t)inverse_mod(m[j], m[i]);
            T.mrc_inv[(size_t)j * n + i] = v;
            T.mrc_inv_sh[(size_t)j * n + i] = shoup(v, m[i]);
        }
    /* binary conversion: 26-bit chunks of M and of M_i = M / m_i, 2^(26 c) mod m_i */
    {
        auto chunks26 = [](const std::vector<uint32_t> &v, int count, uint32_t *dst, size_t stride) {
            for (int c = 0; c < count; c++) {
                const int bit = kBinChunk * c, j = bit / 32, off = bit % 32;
                uint64_t w = j < (int)v.size() ? v[j] : 0;
                if (j + 1 < (int)v.size()) w |= (uint64_t)v[j + 1] << 32;
                dst[(size_t)c * stride] = (uint32_t)(w >> off) & ((1u << kBinChunk) - 1);
            }
        };
        T.bin_limbs = (int)M.size();
        T.bin_chunks = (bitlen + kBinChunk - 1) / kBinChunk;
        T.bin_m26.assign((size_t)((T.bin_chunks + 3) / 4) * 4, 0);
        chunks26(M, T.bin_chunks, T.bin_m26.data(), 1);
        const int ld = bin_ld(n);
        T.bin_mi26.assign((size_t)T.bin_chunks * ld, 0);
        for (int i = 0; i < n; i++) {
            std::vector<uint32_t> q(M.size(), 0);  // M / m_i by long division
            uint64_t r = 0;
            for (int j = (int)M.size() - 1; j >= 0; j--) {
                const uint64_t v = (r << 32) | M[j];
                q[j] = (uint32_t)(v / m[i]);
                r = v % m[i];
            }
            chunks26(q, T.bin_chunks, &T.bin_mi26[i], (size_t)ld);
        }
        T.bin_p26.assign((size_t)kBinMaxChunks * ld, 0);
        for (int i = 0; i < n; i++) {
            const uint64_t step = (((uint64_t)1) << kBinChunk) % m[i];
            uint64_t v = 1 % m[i];
            for (int c = 0; c < kBinMaxChunks; c++) {
                T.bin_p26[(size_t)c * ld + i] = (uint32_t)v;
                v = (v * step) % m[i];
            }
        }
    }
    /* scaling tables (src/rnsbase.cuh:364-387) */
    T.mi_pow2.resize((size_t)30 * n);
    T.m_pow2.resize(30);
    T.pow2_inv.resize((size_t)30 * n);
    T.pow2_inv_sh.resize((size_t)30 * n);
    for (int t = 0; t < 30; t++) {
        uint64_t mask = ((uint64_t)1 << (t + 1)) - 1, mm = 1;
        for (int i = 0; i < n; i++) mm = (mm * m[i]) & mask;
        T.m_pow2[t] = (uint32_t)mm;
        for (int i = 0; i < n; i++) {
            uint64_t v = 1;
            for (int j = 0; j < n; j++)
                if (j != i) v = (v * m[j]) & mask;
            T.mi_pow2[(size_t)t * n + i] = (uint32_t)v;
            uint64_t p2 = ((uint64_t)1 << (t + 1)) % m[i];
            uint32_t inv = (uint32_t)inverse_mod((int64_t)p2, m[i]);
            T.pow2_inv[(size_t)t * n + i] = inv;
            T.pow2_inv_sh[(size_t)t * n + i] = shoup(inv, m[i]);
        }
    }
}

/* The precomputed table `which` in the layout of the reference's device
 * globals (rns_const_init, src/rnsbase.cuh:324-451), as bytes; empty for an
 * unknown index.  0 RNS_ORTHOGONAL_BASE weights (int32[n]); 1/2 reciprocals of
 * the moduli rounded down/up (double[n]); 3 RNS_EVAL_ACCURACY (double); 4
 * RNS_EVAL_REF_FACTOR (int32); 5 RNS_EVAL_UNIT and 6 RNS_EVAL_INV_UNIT
 * (interval_t); 7 MRC inverses (int32[n][n]); 8 powers of two (int32[log2+1][n]);
 * 9 M mod 2^j, 10 M_i mod 2^j and 11 2^-j mod m_i (j < 30). */
inline std::vector<uint8_t> table_bytes(const HostTables &T, int which) {
    auto raw = [](const void *p, size_t bytes) {
        const uint8_t *b = static_cast<const uint8_t *>(p);
        return std::vector<uint8_t>(b, b + bytes);
    };
    const size_t n = (size_t)T.n;
    switch (which) {
        case 0: return raw(T.w.data(), 4 * n);
        case 1: return raw(T.rrd.data(), 8 * n);
        case 2: return raw(T.rru.data(), 8 * n);
        case 3: return raw(&T.acc, 8);
        case 4: return raw(&T.ref_factor, 4);
        case 5:
        case 6: {
            const Er iv[2] = {which == 5 ? T.unit_low : T.inv_unit_low, which == 5 ? T.unit_upp : T.inv_unit_upp};
            return raw(iv, sizeof(iv));
        }
        case 7: return raw(T.mrc_inv.data(), 4 * T.mrc_inv.size());
        case 8: return raw(T.pow2.data(), 4 * T.pow2.size());
        case 9: return raw(T.m_pow2.data(), 4 * 30);
        case 10: return raw(T.mi_pow2.data(), 4 * T.mi_pow2.size());
        case 11: return raw(T.pow2_inv.data(), 4 * T.pow2_inv.size());
        default: return {};
    }
}

/* The device-table blob (one allocation) and the pointer layout inside it. */
inline std::vector<uint32_t> table_blob(const HostTables &T) {
    std::vector<uint32_t> blob(T.c96k);  /* first: 16-byte aligned rows (every size below the
                                            conversion tables is a multiple of 4 words) */
    for (const auto *v : {&T.bin_p26, &T.bin_mi26, &T.bin_m26, &T.pow2, &T.pow2_sh, &T.mrc_inv, &T.mrc_inv_sh, &T.mi_pow2, &T.m_pow2, &T.pow2_inv,
                          &T.pow2_inv_sh, &T.pow2neg, &T.pow2neg_sh})
        blob.insert(blob.end(), v->begin(), v->end());
    blob.resize((blob.size() + 3) & ~(size_t)3, 0u);  // the pair tables start 16-byte aligned
    for (const auto *v : {&T.p2lo, &T.p2hi, &T.p2nlo, &T.p2nhi}) blob.insert(blob.end(), v->begin(), v->end());
    return blob;
}

/* Fills a Consts<N> whose table pointers address `blob` (device or host copy). */
template <int N>
inline void fill_consts(Consts<N> &C, const HostTables &T, const uint32_t *blob) {
    for (int i = 0; i < N; i++) {
        C.m[i] = T.m[i];
        C.w[i] = T.w[i];
        C.w_sh[i] = T.w_sh[i];
        C.mu[i] = T.mu[i];
        C.b[i] = T.bits[i];
        C.rrd[i] = T.rrd[i];
        C.rru[i] = T.rru[i];
        C.c64l[i] = T.c64l[i];
        C.c64h[i] = T.c64h[i];
        C.c96_0[i] = T.c96_0[i];
        C.c96_1[i] = T.c96_1[i];
        C.c96_2[i] = T.c96_2[i];
        C.c96w_0[i] = T.c96k[(size_t)i * 4 + 0];  // row k = 0 of the magnification table
        C.c96w_1[i] = T.c96k[(size_t)i * 4 + 1];
        C.c96w_2[i] = T.c96k[(size_t)i * 4 + 2];
        C.b48[i] = T.b48[i];
        C.b48_sh[i] = T.b48_sh[i];
        C.mi64[i] = T.mi64[i];
        C.c128w_0[i] = T.c128w[(size_t)i * 4 + 0];
        C.c128w_1[i] = T.c128w[(size_t)i * 4 + 1];
        C.c128w_2[i] = T.c128w[(size_t)i * 4 + 2];
        C.c128w_3[i] = T.c128w[(size_t)i * 4 + 3];
        C.evl_lo[i] = T.evl_lo[i];
        C.evl_hi[i] = T.evl_hi[i];
        C.evu_lo[i] = T.evu_lo[i];
        C.evu_hi[i] = T.evu_hi[i];
        C.t32[i] = T.t32[i];
        C.t32_sh[i] = T.t32_sh[i];
        C.mrbits[i] = T.mrbits[i];
    }
    C.acc = T.acc;
    C.acc_lo = T.acc_lo;
    C.m64 = T.m64;
    C.acc_hi = T.acc_hi;
    C.ref_factor = T.ref_factor;
    C.log2M = T.log2M;
    C.unit_low = T.unit_low;
    C.unit_upp = T.unit_upp;
    C.inv_unit_low = T.inv_unit_low;
    C.inv_unit_upp = T.inv_unit_upp;
    C.unit_rcp_low = (uint64_t)((((unsigned __int128)1) << 116) / ((dbits(T.unit_low.frac) & ((1ull << 52) - 1)) | (1ull << 52)));
    C.unit_rcp_upp = (uint64_t)((((unsigned __int128)1) << 116) / ((dbits(T.unit_upp.frac) & ((1ull << 52) - 1)) | (1ull << 52)));
    C.m_pow2_res30 = T.m_pow2[29];
    C.E = T.E;
    C.c96k = reinterpret_cast<const uint4 *>(blob);
    size_t off = T.c96k.size();
    C.bin_p26 = blob + off;     off += T.bin_p26.size();
    C.bin_mi26 = blob + off;    off += T.bin_mi26.size();
    C.bin_m26 = blob + off;     off += T.bin_m26.size();
    C.bin_chunks = T.bin_chunks;
    C.bin_limbs = T.bin_limbs;
    C.pow2 = blob + off;        off += T.pow2.size();
    C.pow2_sh = blob + off;     off += T.pow2_sh.size();
    C.mrc_inv = blob + off;     off += T.mrc_inv.size();
    C.mrc_inv_sh = blob + off;  off += T.mrc_inv_sh.size();
    C.mi_pow2 = blob + off;     off += T.mi_pow2.size();
    C.m_pow2 = blob + off;      off += T.m_pow2.size();
    C.pow2_inv = blob + off;    off += T.pow2_inv.size();
    C.pow2_inv_sh = blob + off; off += T.pow2_inv_sh.size();
    C.pow2neg = blob + off;     off += T.pow2neg.size();
    C.pow2neg_sh = blob + off;  off += T.pow2neg_sh.size();
    off = (off + 3) & ~(size_t)3;
    C.p2lo = reinterpret_cast<const uint2 *>(blob + off);   off += T.p2lo.size();
    C.p2hi = reinterpret_cast<const uint2 *>(blob + off);   off += T.p2hi.size();
    C.p2nlo = reinterpret_cast<const uint2 *>(blob + off);  off += T.p2nlo.size();
    C.p2nhi = reinterpret_cast<const uint2 *>(blob + off);
    C.p2rows = pow2_hi_rows(T.log2M);
}

}  // namespace grns
