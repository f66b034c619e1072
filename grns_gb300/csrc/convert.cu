/*
 * grns_gb300 -- binary <-> RNS conversion kernels (rns_from_binary /
 * rns_to_binary, reference src/rnsbase.cuh:253/:277; mpint_set_mpz /
 * mpint_get_mpz, src/mpint.cuh:74/:100), arithmetic in rns_convert.cuh.
 *
 * A block handles tiles of 128 numbers.  Binary integers are number-major
 * rows of 32-bit limbs, so a tile's limbs are one contiguous range: the block
 * moves it between global and shared memory with coalesced accesses, and
 * each thread works on its own shared-memory row (odd row stride: no bank
 * conflicts).  The chunk tables sit in shared memory and are read as 16-byte
 * broadcasts.
 */
#include "internal.h"
#include "rns_convert.cuh"
#include "rns_device.cuh"
#include "rns_mpint.cuh"

namespace grns {

constexpr int kConvBlock = 128;

/* the chunk tables are staged in shared memory up to 64 moduli (at most
 * 316 x 64 words); above, a block holds only its rows */
template <int N>
constexpr bool conv_tables_shared() {
    return N <= 64;
}

__host__ __device__ constexpr int odd_at_least(int v) { return v | 1; }

/* ---------------- binary -> RNS ---------------- */

/* out[k * ks + i * is] = (integer k) mod m_i; nonzero[k] (optional) = integer k != 0 */
template <int N>
__global__ void __launch_bounds__(kConvBlock) k_from_binary(const __grid_constant__ CArg<N> CA,
                                                            const uint32_t *__restrict__ words, int nlimbs,
                                                            int64_t count, uint32_t *__restrict__ out, int64_t ks,
                                                            int64_t is, uint8_t *__restrict__ nonzero) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 conv_smem[];
    const int chunks = (32 * nlimbs + kBinChunk - 1) / kBinChunk;
    const int rs = odd_at_least(nlimbs + 1);  // row stride: limbs, one zero word, odd
    constexpr int L4 = bin_ld(N) / 4;         // 16-byte words per table row
    constexpr bool kShared = conv_tables_shared<N>();
    /* [chunks][L4]: staged in shared memory up to 64 moduli, else read through L1 / L2 */
    const uint4 *T4 = kShared ? conv_smem : reinterpret_cast<const uint4 *>(C.bin_p26);
    uint32_t *rows = reinterpret_cast<uint32_t *>(conv_smem + (kShared ? chunks * L4 : 0));
    if (kShared)
        for (int w = threadIdx.x; w < chunks * L4; w += blockDim.x)
            conv_smem[w] = reinterpret_cast<const uint4 *>(C.bin_p26)[w];
    const bool fold = chunks > kBinSumMax;
    uint32_t *row = rows + threadIdx.x * rs;
    for (int j = nlimbs; j < rs; j++) row[j] = 0;
    constexpr int G = (N % 8 == 0) ? 8 : 4;
    for (int64_t k0 = (int64_t)blockIdx.x * kConvBlock; k0 < count; k0 += (int64_t)gridDim.x * kConvBlock) {
        const int tile = count - k0 < kConvBlock ? (int)(count - k0) : kConvBlock;
        __syncthreads();
        const uint32_t *src = words + k0 * nlimbs;
        for (int w = threadIdx.x; w < tile * nlimbs; w += blockDim.x) {
            const int t = w / nlimbs, l = w - t * nlimbs;
            rows[t * rs + l] = __ldcs(src + w);
        }
        __syncthreads();
        if ((int)threadIdx.x >= tile) continue;
        const int64_t k = k0 + threadIdx.x;
        if (nonzero) {
            uint32_t any = 0;
            for (int j = 0; j < nlimbs; j++) any |= row[j];
            nonzero[k] = any != 0;
        }
        for (int g = 0; g < N; g += G) {
            uint64_t acc[G];
#pragma unroll
            for (int u = 0; u < G; u++) acc[u] = 0;
            for (int c = 0; c < chunks; c++) {
                const int bit = kBinChunk * c, j = bit >> 5;
                const uint32_t ch = __funnelshift_r(row[j], row[j + 1], bit & 31) & kBinMask;
                const uint4 *t = T4 + c * L4 + g / 4;
#pragma unroll
                for (int u = 0; u < G; u += 4) {
                    const uint4 v = t[u / 4];
                    acc[u] += (uint64_t)ch * v.x;
                    acc[u + 1] += (uint64_t)ch * v.y;
                    acc[u + 2] += (uint64_t)ch * v.z;
                    acc[u + 3] += (uint64_t)ch * v.w;
                }
                if (fold && c % kBinFold == kBinFold - 1) {
#pragma unroll
                    for (int u = 0; u < G; u++)
                        if (N % G == 0 || g + u < N) acc[u] = bin_mod64<N>(C, g + u, acc[u]);
                }
            }
#pragma unroll
            for (int u = 0; u < G; u++)
                if (N % G == 0 || g + u < N) out[k * ks + (int64_t)(g + u) * is] = bin_mod64<N>(C, g + u, acc[u]);
        }
    }
}

template <int N>
constexpr size_t from_binary_smem(int nlimbs) {
    return (conv_tables_shared<N>() ? (size_t)((32 * nlimbs + kBinChunk - 1) / kBinChunk) * bin_ld(N) * 4 : 0) +
           (size_t)kConvBlock * odd_at_least(nlimbs + 1) * 4;
}

/* ---------------- RNS -> binary ---------------- */

/* words[k * nout + l] = limb l of X_k in [0, M) (zeros above the value);
 * x_k's residue i at x[k * ks + i * is].  sign_in (optional, stride ss words)
 * and sign_out: sign_out[k] = sign_in == 1 and X_k != 0 (mpint_get_mpz's
 * sign).  An invalid residue flags the number and gives zero. */
template <int N>
__global__ void __launch_bounds__(kConvBlock) k_to_binary(const __grid_constant__ CArg<N> CA,
                                                          const uint32_t *__restrict__ x, int64_t ks, int64_t is,
                                                          int64_t count, uint32_t *__restrict__ words, int nout,
                                                          const int32_t *__restrict__ sign_in, int64_t ss,
                                                          int32_t *__restrict__ sign_out,
                                                          uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 conv_smem[];
    const int chunks = C.bin_chunks;
    const int m4 = (chunks + 3) / 4;
    const int rs = odd_at_least(chunks);
    constexpr int L = bin_ld(N);            // table row: N words and zeros up to a multiple of 4
    constexpr bool kShared = conv_tables_shared<N>();
    /* [chunks][L / 4] and [m4 * 4]: staged in shared memory up to 64 moduli, else read through L1 / L2 */
    uint4 *Mi4s = conv_smem;
    uint32_t *M26s = reinterpret_cast<uint32_t *>(Mi4s + chunks * (L / 4));
    const uint4 *Mi4 = kShared ? Mi4s : reinterpret_cast<const uint4 *>(C.bin_mi26);
    const uint32_t *M26 = kShared ? M26s : C.bin_m26;
    uint32_t *rows = kShared ? M26s + m4 * 4 : reinterpret_cast<uint32_t *>(conv_smem);
    if (kShared) {
        for (int w = threadIdx.x; w < chunks * (L / 4); w += blockDim.x)
            Mi4s[w] = reinterpret_cast<const uint4 *>(C.bin_mi26)[w];
        for (int w = threadIdx.x; w < m4 * 4; w += blockDim.x) M26s[w] = C.bin_m26[w];
    }
    uint32_t *row = rows + threadIdx.x * rs;
    for (int64_t k0 = (int64_t)blockIdx.x * kConvBlock; k0 < count; k0 += (int64_t)gridDim.x * kConvBlock) {
        const int tile = count - k0 < kConvBlock ? (int)(count - k0) : kConvBlock;
        __syncthreads();
        if ((int)threadIdx.x < tile) {
            const int64_t k = k0 + threadIdx.x;
            uint32_t s[L];
            uint32_t bad = 0, any = 0;
GRNS_UNROLL_TO(L)
            for (int i = N; i < L; i++) s[i] = 0;
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) {
                const uint32_t v = __ldg(x + k * ks + (int64_t)i * is);
                bad |= (uint32_t)(v >= C.m[i]);
                any |= v;
                s[i] = mulmod_shoup(v, C.w[i], C.w_sh[i], C.m[i]);
            }
            if (bad) {
                for (int c = 0; c < chunks; c++) row[c] = 0;
            } else {
                const uint32_t kk = bin_rank<N>(C, s);
                int64_t carry = 0;
                for (int c = 0; c < chunks; c++) {
                    const uint4 *t = Mi4 + c * (L / 4);
                    BinAcc<N> a0 = 0, a1 = 0, a2 = 0, a3 = 0;
GRNS_UNROLL_TO(L)
                    for (int i = 0; i < L; i += 4) {
                        const uint4 v = t[i / 4];
                        a0 += (uint64_t)s[i] * v.x;
                        a1 += (uint64_t)s[i + 1] * v.y;
                        a2 += (uint64_t)s[i + 2] * v.z;
                        a3 += (uint64_t)s[i + 3] * v.w;
                    }
                    const BinSAcc<N> v = (BinSAcc<N>)((a0 + a1) + (a2 + a3)) - (BinSAcc<N>)kk * M26[c] + carry;
                    carry = (int64_t)(v >> kBinChunk);
                    row[c] = (uint32_t)v & kBinMask;
                }
                if (carry < 0) {
                    uint32_t cy = 0;
                    for (int c = 0; c < chunks; c++) {
                        const uint32_t v = row[c] + M26[c] + cy;
                        row[c] = v & kBinMask;
                        cy = v >> kBinChunk;
                    }
                }
                bin_pack(row, 1, chunks, C.bin_limbs);
            }
            if (flags) flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
            if (sign_out) sign_out[k] = (sign_in && !bad && any && __ldg(sign_in + k * ss) == 1) ? 1 : 0;
        }
        __syncthreads();
        uint32_t *dst = words + k0 * nout;
        for (int w = threadIdx.x; w < tile * nout; w += blockDim.x) {
            const int t = w / nout, l = w - t * nout;
            __stcs(dst + w, l < C.bin_limbs ? rows[t * rs + l] : 0u);
        }
    }
}

template <int N>
size_t to_binary_smem(const Consts<N> &C) {
    return (conv_tables_shared<N>() ? (size_t)C.bin_chunks * bin_ld(N) * 4 + (size_t)((C.bin_chunks + 3) / 4) * 16
                                    : 0) +
           (size_t)kConvBlock * odd_at_least(C.bin_chunks) * 4;
}

/* ---------------- mp_int records from residue columns ---------------- */

/* mpint_set_mpz's record: digits from residue-major columns (ld = count), the
 * sign of a nonzero integer, the evaluation of the digits */
template <int N>
__global__ void __launch_bounds__(128) k_mpint_pack(const __grid_constant__ CArg<N> CA,
                                                    const uint32_t *__restrict__ res, const int32_t *__restrict__ signs,
                                                    const uint8_t *__restrict__ nonzero, int64_t count,
                                                    MpInt<N> *__restrict__ out) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        MpInt<N> r;
        uint32_t f = 0;
#pragma unroll 8
        for (int i = 0; i < N; i++) r.digits[i] = __ldg(res + (int64_t)i * count + k);
        eval<N>(C, [&](int i) { return r.digits[i]; }, r.eval[0], r.eval[1], f);
        r.sign = (signs && __ldg(signs + k) != 0 && nonzero[k]) ? 1 : 0;
        clear_pad(r);
        out[k] = r;
    }
}

/* ---------------- launchers ---------------- */

template <class K>
static int conv_grid(const grns_ctx *c, K kernel, size_t smem, int64_t count) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kConvBlock, smem) != cudaSuccess || nb < 1) nb = 1;
    const int64_t tiles = (count + kConvBlock - 1) / kConvBlock;
    const int64_t cap = (int64_t)c->sm_count * nb;
    return (int)(tiles < cap ? tiles : cap);
}

template <int N>
static grns_status run_from_binary(const grns_ctx *c, const uint32_t *words, int nlimbs, int64_t count,
                                   uint32_t *out, int64_t ks, int64_t is, uint8_t *nonzero, cudaStream_t s) {
    const size_t smem = from_binary_smem<N>(nlimbs);
    const int grid = conv_grid(c, k_from_binary<N>, smem, count);
    k_from_binary<N><<<grid, kConvBlock, smem, s>>>(consts_of<N>(c), words, nlimbs, count, out, ks, is, nonzero);
    return cuda_status(cudaGetLastError());
}

template <int N>
static grns_status run_to_binary(const grns_ctx *c, const uint32_t *x, int64_t ks, int64_t is, int64_t count,
                                 uint32_t *words, int nout, const int32_t *sign_in, int64_t ss, int32_t *sign_out,
                                 uint8_t *flags, cudaStream_t s) {
    const size_t smem = to_binary_smem<N>(consts_of<N>(c));
    const int grid = conv_grid(c, k_to_binary<N>, smem, count);
    k_to_binary<N><<<grid, kConvBlock, smem, s>>>(consts_of<N>(c), x, ks, is, count, words, nout, sign_in, ss,
                                                  sign_out, flags);
    return cuda_status(cudaGetLastError());
}

template <int N>
static grns_status run_mpint_from_binary(const grns_ctx *c, const uint32_t *words, int nlimbs, const int32_t *signs,
                                         int64_t count, void *out, cudaStream_t s) {
    void *scratch = nullptr;
    cudaError_t e = scratch_alloc(c, &scratch, (size_t)count * (4 * N + 1), s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t *res = (uint32_t *)scratch;
    uint8_t *nz = (uint8_t *)(res + (size_t)N * count);
    grns_status st = run_from_binary<N>(c, words, nlimbs, count, res, 1, count, nz, s);
    if (st == GRNS_OK) {
        k_mpint_pack<N><<<grid_for(c, count, 128), 128, 0, s>>>(consts_of<N>(c), res, signs, nz, count,
                                                                (MpInt<N> *)out);
        st = cuda_status(cudaGetLastError());
    }
    scratch_free(scratch, s);
    return st;
}

}  // namespace grns

using grns::kBinMaxLimbs;

extern "C" {

int grns_ctx_binary_limbs(const grns_ctx *c) { return c ? c->T.bin_limbs : 0; }

grns_status grns_from_binary(grns_ctx *c, const uint32_t *words, int limbs, int64_t count, int layout, int32_t *out,
                             void *stream) {
    if (!c || count < 0 || limbs < 1 || limbs > kBinMaxLimbs ||
        (layout != GRNS_LAYOUT_SOA && layout != GRNS_LAYOUT_AOS))
        return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!words || !out) return GRNS_ERR_INVALID_ARGUMENT;
    const int64_t ks = layout == GRNS_LAYOUT_SOA ? 1 : c->n, is = layout == GRNS_LAYOUT_SOA ? count : 1;
#define C_(n) return grns::run_from_binary<n>(c, words, limbs, count, (uint32_t *)out, ks, is, nullptr, (cudaStream_t)stream)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_to_binary(grns_ctx *c, const int32_t *x, int64_t count, int layout, uint32_t *words, int limbs,
                           uint8_t *flags, void *stream) {
    if (!c || count < 0 || limbs < c->T.bin_limbs || limbs > kBinMaxLimbs ||
        (layout != GRNS_LAYOUT_SOA && layout != GRNS_LAYOUT_AOS))
        return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !words) return GRNS_ERR_INVALID_ARGUMENT;
    const int64_t ks = layout == GRNS_LAYOUT_SOA ? 1 : c->n, is = layout == GRNS_LAYOUT_SOA ? count : 1;
#define C_(n)                                                                                              \
    return grns::run_to_binary<n>(c, (const uint32_t *)x, ks, is, count, words, limbs, nullptr, 0, nullptr, \
                                  flags, (cudaStream_t)stream)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_mpint_from_binary(grns_ctx *c, const uint32_t *words, int limbs, const int32_t *signs,
                                   int64_t count, void *out, void *stream) {
    if (!c || count < 0 || limbs < 1 || limbs > kBinMaxLimbs) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!words || !out) return GRNS_ERR_INVALID_ARGUMENT;
#define C_(n) return grns::run_mpint_from_binary<n>(c, words, limbs, signs, count, out, (cudaStream_t)stream)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_mpint_to_binary(grns_ctx *c, const void *x, int64_t count, uint32_t *words, int limbs,
                                 int32_t *signs, uint8_t *flags, void *stream) {
    if (!c || count < 0 || limbs < c->T.bin_limbs || limbs > kBinMaxLimbs) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !words) return GRNS_ERR_INVALID_ARGUMENT;
#define C_(n)                                                                                                    \
    {                                                                                                            \
        const int64_t W = (int64_t)(sizeof(grns::MpInt<n>) / 4);                                                 \
        const uint32_t *base = (const uint32_t *)x;                                                              \
        return grns::run_to_binary<n>(c, base, W, 1, count, words, limbs, (const int32_t *)(base + n), W, signs, \
                                      flags, (cudaStream_t)stream);                                              \
    }
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // extern "C"
