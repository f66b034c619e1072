/*
 * grns_gb300 -- moduli-set contexts: the constant tables of the reference's
 * rns_const_init (kisupov/grns src/rnsbase.cuh:324-451) computed on the host
 * without GMP/MPFR, uploaded once per context.
 *
 * Only two properties of the big product M are needed: its bit length
 * (floor(log2 M), the RNS_MODULI_PRODUCT_LOG2 convention) and its top 53
 * bits, because the reference converts M to a 53-bit MPFR number rounded
 * down (mpfr_init default precision + MPFR_RNDD, :326/:336) before it
 * computes 1/M and 1-1/M.  Everything else is a product, power or inverse
 * modulo a 31-bit modulus or a power of two.
 */
#include <cmath>
#include <cstring>
#include <new>

#include "internal.h"

namespace {

int64_t inverse_mod(int64_t x, int64_t m) {  // x^-1 mod m in [0, m), gcd(x, m) = 1
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

int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

/* ddiv_rd/ddiv_ru(1, m) with the reference's host rounding: the round-to-
 * nearest quotient moved by PHI1*|c| + ETA (src/dinterval.cuh:124-136).
 * volatile keeps the compiler from fusing the multiply-add. */
double recip_host(double m, bool up) {
    volatile double c = 1.0 / m;
    volatile double phi1 = 0x1p-53 * (1.0 + 2.0 * 0x1p-53);
    volatile double t = phi1 * std::fabs(c);
    volatile double e = t + 0x1p-1074;
    return up ? c + e : c - e;
}

/* directed rounding of 0 < p/q <= 1 to 53 bits, reported as mpfr_get_d_2exp
 * does: frac in [0.5, 1), value = frac * 2^exp */
void round_ratio(uint64_t p, uint64_t q, bool up, double &frac, int64_t &exp) {
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

template <int N>
void fill_consts(grns_ctx *c, const uint32_t *d) {
    grns::Consts<N> &C = *reinterpret_cast<grns::Consts<N> *>(c->consts);
    for (int i = 0; i < N; i++) {
        C.m[i] = c->moduli[i];
        C.w[i] = c->w[i];
        C.w_sh[i] = c->w_sh[i];
        C.mu[i] = c->mu[i];
        C.b[i] = c->bits[i];
        C.rrd[i] = c->rrd[i];
        C.rru[i] = c->rru[i];
    }
    C.acc = c->acc;
    C.ref_factor = c->ref_factor;
    C.log2M = c->log2M;
    C.unit_low = c->unit_low;
    C.unit_upp = c->unit_upp;
    C.inv_unit_low = c->inv_unit_low;
    C.inv_unit_upp = c->inv_unit_upp;
    C.m_pow2_res30 = c->m_pow2[29];
    size_t off = 0;
    C.pow2 = d + off;        off += c->pow2.size();
    C.mrc_inv = d + off;     off += c->mrc_inv.size();
    C.mrc_inv_sh = d + off;  off += c->mrc_inv_sh.size();
    C.mi_pow2 = d + off;     off += c->mi_pow2.size();
    C.m_pow2 = d + off;      off += c->m_pow2.size();
    C.pow2_inv = d + off;    off += c->pow2_inv.size();
    C.pow2_inv_sh = d + off;
}

grns_status build(grns_ctx *c) {
    const int n = c->n;
    const std::vector<uint32_t> &m = c->moduli;
    /* M as 32-bit limbs: bit length and top 53 bits */
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
    c->log2M = bitlen - 1;
    const int E = bitlen > 53 ? bitlen - 53 : 0;
    uint64_t T = 0;
    for (int bit = bitlen - 1; bit >= E; bit--) T = (T << 1) | ((M[bit / 32] >> (bit % 32)) & 1u);

    c->w.resize(n); c->w_sh.resize(n); c->mu.resize(n); c->bits.resize(n);
    c->rrd.resize(n); c->rru.resize(n);
    for (int i = 0; i < n; i++) {
        int64_t mi = 1;
        for (int j = 0; j < n; j++)
            if (j != i) mi = (mi * (m[j] % m[i])) % m[i];
        c->w[i] = (uint32_t)inverse_mod(mi, m[i]);
        c->w_sh[i] = (uint32_t)(((uint64_t)c->w[i] << 32) / m[i]);
        uint32_t b = 0;
        for (uint32_t v = m[i]; v; v >>= 1) b++;
        c->bits[i] = b;
        c->mu[i] = (uint32_t)(((unsigned __int128)1 << (2 * b)) / m[i]);
        c->rrd[i] = recip_host((double)m[i], false);
        c->rru[i] = recip_host((double)m[i], true);
    }
    /* RNS_EVAL_ACCURACY and RNS_EVAL_REF_FACTOR (src/rnsbase.cuh:389-391), same operation order */
    volatile double acc = 4 * std::pow(2.0, 1 - 53);
    acc = acc * n;
    acc = acc * std::log2((double)n);
    acc = acc * (1 + 0.0000001 / 2);
    acc = acc / 0.0000001;
    c->acc = acc;
    c->ref_factor = (int)std::floor(std::log2(1 / (2 * c->acc)));
    /* RNS_EVAL_UNIT ~ 1/M53 and RNS_EVAL_INV_UNIT ~ 1 - 1/M53 (src/rnsbase.cuh:393-411) */
    round_ratio(1, T, false, c->unit_low.frac, c->unit_low.exp);
    round_ratio(1, T, true, c->unit_upp.frac, c->unit_upp.exp);
    c->unit_low.exp -= E;
    c->unit_upp.exp -= E;
    if (E == 0) {
        round_ratio(T - 1, T, false, c->inv_unit_low.frac, c->inv_unit_low.exp);
        round_ratio(T - 1, T, true, c->inv_unit_upp.frac, c->inv_unit_upp.exp);
    } else if (E == 1 && T == ((uint64_t)1 << 52)) {
        c->inv_unit_low = c->inv_unit_upp = grns::Er{1.0 - 0x1p-53, 0};
    } else {
        c->inv_unit_low = grns::Er{1.0 - 0x1p-53, 0};
        c->inv_unit_upp = grns::Er{0.5, 1};
    }
    /* RNS_POW2[j][i] = 2^j mod m_i */
    c->pow2.resize((size_t)(c->log2M + 1) * n);
    for (int i = 0; i < n; i++) {
        uint64_t v = 1;
        for (int j = 0; j <= c->log2M; j++) {
            c->pow2[(size_t)j * n + i] = (uint32_t)v;
            v = (v * 2) % m[i];
        }
    }
    /* MRC_MULT_INV, stored transposed for the device as [j*n + i] = m_j^-1 mod m_i */
    c->mrc_inv.assign((size_t)n * n, 0);
    c->mrc_inv_sh.assign((size_t)n * n, 0);
    for (int j = 0; j < n; j++)
        for (int i = j + 1; i < n; i++) {
            uint32_t v = (uint32_t)inverse_mod(m[j], m[i]);
            c->mrc_inv[(size_t)j * n + i] = v;
            c->mrc_inv_sh[(size_t)j * n + i] = (uint32_t)(((uint64_t)v << 32) / m[i]);
        }
    /* scaling tables (src/rnsbase.cuh:364-387) */
    c->mi_pow2.resize((size_t)30 * n);
    c->m_pow2.resize(30);
    c->pow2_inv.resize((size_t)30 * n);
    c->pow2_inv_sh.resize((size_t)30 * n);
    for (int t = 0; t < 30; t++) {
        uint64_t mask = ((uint64_t)1 << (t + 1)) - 1, mm = 1;
        for (int i = 0; i < n; i++) mm = (mm * m[i]) & mask;
        c->m_pow2[t] = (uint32_t)mm;
        for (int i = 0; i < n; i++) {
            uint64_t v = 1;
            for (int j = 0; j < n; j++)
                if (j != i) v = (v * m[j]) & mask;
            c->mi_pow2[(size_t)t * n + i] = (uint32_t)v;
            uint64_t p2 = ((uint64_t)1 << (t + 1)) % m[i];
            uint32_t inv = (uint32_t)inverse_mod((int64_t)p2, m[i]);
            c->pow2_inv[(size_t)t * n + i] = inv;
            c->pow2_inv_sh[(size_t)t * n + i] = (uint32_t)(((uint64_t)inv << 32) / m[i]);
        }
    }
    /* upload */
    std::vector<uint32_t> blob;
    for (auto *v : {&c->pow2, &c->mrc_inv, &c->mrc_inv_sh, &c->mi_pow2, &c->m_pow2, &c->pow2_inv, &c->pow2_inv_sh})
        blob.insert(blob.end(), v->begin(), v->end());
    cudaError_t e = cudaMalloc(&c->d_tables, blob.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return grns::cuda_status(e);
    e = cudaMemcpy(c->d_tables, blob.data(), blob.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return grns::cuda_status(e);
    const uint32_t *d = (const uint32_t *)c->d_tables;
    switch (n) {
        case 4: fill_consts<4>(c, d); break;
        case 8: fill_consts<8>(c, d); break;
        case 12: fill_consts<12>(c, d); break;
        case 16: fill_consts<16>(c, d); break;
        case 32: fill_consts<32>(c, d); break;
        case 64: fill_consts<64>(c, d); break;
        default: return GRNS_ERR_UNSUPPORTED;
    }
    return GRNS_OK;
}

}  // namespace

extern "C" {

const char *grns_status_string(grns_status s) {
    switch (s) {
        case GRNS_OK: return "ok";
        case GRNS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GRNS_ERR_UNSUPPORTED: return "unsupported moduli set";
        case GRNS_ERR_CUDA: return "CUDA error";
        case GRNS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case GRNS_ERR_TIMEOUT: return "timed out";
        case GRNS_ERR_REJECTED: return "rejected by admission control";
        case GRNS_ERR_BUSY: return "busy";
    }
    return "unknown status";
}

const char *grns_version(void) { return "grns_gb300 0.1 (sm_103a)"; }

grns_status grns_ctx_create(const int32_t *moduli, int n, grns_ctx **out) {
    if (!moduli || !out) return GRNS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!(n == 4 || n == 8 || n == 12 || n == 16 || n == 32 || n == 64)) return GRNS_ERR_UNSUPPORTED;
    for (int i = 0; i < n; i++) {
        if (moduli[i] < 3 || moduli[i] > 1431655765 || (moduli[i] & 1) == 0) return GRNS_ERR_UNSUPPORTED;
        for (int j = 0; j < i; j++)
            if (gcd64(moduli[i], moduli[j]) != 1) return GRNS_ERR_INVALID_ARGUMENT;
    }
    grns_ctx *c = new (std::nothrow) grns_ctx();
    if (!c) return GRNS_ERR_OUT_OF_MEMORY;
    c->n = n;
    c->moduli.assign(moduli, moduli + n);
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) {
        delete c;
        return grns::cuda_status(e);
    }
    grns_status st = build(c);
    if (st != GRNS_OK) {
        grns_ctx_destroy(c);
        return st;
    }
    *out = c;
    return GRNS_OK;
}

grns_status grns_ctx_destroy(grns_ctx *c) {
    if (!c) return GRNS_ERR_INVALID_ARGUMENT;
    if (c->d_tables) cudaFree(c->d_tables);
    if (c->d_scratch) cudaFree(c->d_scratch);
    delete c;
    return GRNS_OK;
}

int grns_ctx_n(const grns_ctx *c) { return c ? c->n : 0; }
int grns_ctx_log2(const grns_ctx *c) { return c ? c->log2M : 0; }

grns_status grns_ctx_get_table(const grns_ctx *c, int which, void *dst, size_t bytes) {
    if (!c || !dst) return GRNS_ERR_INVALID_ARGUMENT;
    const int n = c->n;
    std::vector<int32_t> tmp;
    const void *src = nullptr;
    size_t size = 0;
    interval_t iv;
    switch (which) {
        case 0: src = c->w.data(); size = 4 * n; break;
        case 1: src = c->rrd.data(); size = 8 * n; break;
        case 2: src = c->rru.data(); size = 8 * n; break;
        case 3: src = &c->acc; size = 8; break;
        case 4: src = &c->ref_factor; size = 4; break;
        case 5:
            iv.low = er_float_t{c->unit_low.frac, c->unit_low.exp};
            iv.upp = er_float_t{c->unit_upp.frac, c->unit_upp.exp};
            src = &iv; size = sizeof(iv); break;
        case 6:
            iv.low = er_float_t{c->inv_unit_low.frac, c->inv_unit_low.exp};
            iv.upp = er_float_t{c->inv_unit_upp.frac, c->inv_unit_upp.exp};
            src = &iv; size = sizeof(iv); break;
        case 7:  /* back to the reference orientation [i][j] = m_i^-1 mod m_j */
            tmp.assign((size_t)n * n, 0);
            for (int i = 0; i < n; i++)
                for (int j = i + 1; j < n; j++) tmp[(size_t)i * n + j] = (int32_t)c->mrc_inv[(size_t)i * n + j];
            src = tmp.data(); size = 4 * tmp.size(); break;
        case 8: src = c->pow2.data(); size = 4 * c->pow2.size(); break;
        case 9: src = c->m_pow2.data(); size = 4 * 30; break;
        case 10: src = c->mi_pow2.data(); size = 4 * c->mi_pow2.size(); break;
        case 11: src = c->pow2_inv.data(); size = 4 * c->pow2_inv.size(); break;
        default: return GRNS_ERR_INVALID_ARGUMENT;
    }
    if (bytes != size) return GRNS_ERR_INVALID_ARGUMENT;
    std::memcpy(dst, src, size);
    return GRNS_OK;
}

}  // extern "C"
