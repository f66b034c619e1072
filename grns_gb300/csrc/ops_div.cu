/*
 * grns_gb300 -- division and power-of-two scaling kernels.
 *   k_div      : q = floor(X/D), r = X - qD (reference src/rnsdiv.cuh:128),
 *                reference-faithful FP64 form, one thread per number
 *   k_div_a, k_div_rows, k_div_place, k_div_b, k_div_out : the same
 *                results on the integer fast path (div_warp.cuh): pass A
 *                writing one record per number, one row per number, a
 *                counting sort of all numbers by step count,
 *                pass B over the rows longest first (numbers claimed from
 *                grid-wide counters), the rows to the caller's layout
 *   k_scale    : floor(X / 2^D)             (reference src/rnsscal.cuh:207)
 * GRNS_SPLIT_BY_N: compiled as one unit per group of moduli counts.
 */
#include <algorithm>

#include "div_warp.cuh"
#include "scale_warp.cuh"
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"
#include "div_coop.cuh"

namespace grns {

/* the reference's division (div_ref, one quotient bit a step), one number per thread */
template <int N>
__global__ void __launch_bounds__(128) k_div(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> d,
                                             int64_t count, Output<N> q, Output<N> r, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], da[N], qa[N], ra[N], f = 0;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            da[i] = d.load(k, i);
            f |= (xa[i] >= C.m[i] || da[i] >= C.m[i]) ? kFlagInvalidInput : 0u;
        }
        if (f) {
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) { qa[i] = 0; ra[i] = 0; }
        } else {
            div_ref<N>(C, qa, ra, xa, da, f);
        }
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            q.store(k, i, qa[i]);
            r.store(k, i, ra[i]);
        }
        if (flags) flags[k] = (uint8_t)f;
    }
}

constexpr int kDivBlock = 128;

/* one division per warp (div_coop.cuh), for the 128- and 256-moduli sets:
 * lane l holds residues l + 32 j; scratch for the rare exact comparisons */
constexpr int kDivCoopBlock = 128;
template <int N>
__global__ void __launch_bounds__(kDivCoopBlock)
    k_div_coop(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> d, int64_t count, Output<N> q,
               Output<N> r, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    constexpr int J = N / 32;
    __shared__ DivK K[N];
    __shared__ uint32_t scratch[kDivCoopBlock / 32][2 * N];
    divk_fill<N>(C, K);
    __syncthreads();
    const int lane = threadIdx.x & 31;
    uint32_t *sc = scratch[threadIdx.x >> 5];
    const int64_t warps = ((int64_t)gridDim.x * kDivCoopBlock) >> 5;
    for (int64_t k = ((int64_t)blockIdx.x * kDivCoopBlock + threadIdx.x) >> 5; k < count; k += warps) {
        uint32_t xa[J], da[J], qa[J], ra[J];
        bool bad = false;
#pragma unroll
        for (int j = 0; j < J; j++) {
            const int i = lane + 32 * j;
            xa[j] = x.load(k, i);
            da[j] = d.load(k, i);
            bad |= xa[j] >= C.m[i] || da[j] >= C.m[i];
        }
        uint32_t f = __any_sync(kWarpFull, bad) ? kFlagInvalidInput : 0u;
        if (f) {
#pragma unroll
            for (int j = 0; j < J; j++) qa[j] = ra[j] = 0;
        } else {
            div_warp_coop<N>(K, C, qa, ra, xa, da, f, lane, sc);
        }
#pragma unroll
        for (int j = 0; j < J; j++) {
            q.store(k, lane + 32 * j, qa[j]);
            r.store(k, lane + 32 * j, ra[j]);
        }
        if (flags && lane == 0) flags[k] = (uint8_t)f;
    }
}

/* resident 128-thread blocks per SM the register budget must allow: shared
 * memory (3N words per thread) allows 4 at n <= 32 and 2 at n = 64 */
#ifndef GRNS_DIV_MIN_BLOCKS
#define GRNS_DIV_MIN_BLOCKS 5
#endif
template <int N>
constexpr int div_min_blocks() {
    return N > 32 ? 2 : GRNS_DIV_MIN_BLOCKS;
}

/* the division's scratch per chunk of numbers stays below this (the context's
 * pool keeps kPoolKeepBytes across synchronisations) */
constexpr size_t kDivScratchBytes = 192ull << 20;

/* grid-wide state of one division call (one memset clears it) */
struct DivRowsG {
    unsigned long long ctr_a, ctr_b;  // pass A / pass B claim counters
    uint32_t hist[kDivRowBins];       // numbers per digit-step count
    uint32_t cursor[kDivRowBins];     // positions handed out per step count
};

/* pass A: numbers claimed from G->ctr_a in index order; per number its
 * 8-byte record (div_warp.cuh, divnorm_range) */
template <int N>
__global__ void __launch_bounds__(kDivBlock, N > 32 ? 3 : 6)
    k_div_a(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> d, uint2 *__restrict__ rec,
            DivRowsG *__restrict__ G, int64_t count) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 div_smem[];
    DivK *K = reinterpret_cast<DivK *>(div_smem);
    uint32_t *cols = reinterpret_cast<uint32_t *>(K + N);  // layout of divprep_smem_bytes
    divk_fill<N>(C, K);
    __syncthreads();
    /* prefetch distance: one number per lane of the grid ahead, about what the
     * grid claims while a number is normalised */
    const int64_t lanes = (int64_t)gridDim.x * blockDim.x;
    divnorm_range<N>(K, C, x, d, rec, count, [&](int c) { return warp_claim(&G->ctr_a, c); }, lanes,
                     cols + threadIdx.x, blockDim.x);
}

/* rows: one thread per number in index order (coalesced operand loads, every
 * lane busy); per number its row, its step count and (no digit step) its
 * flags; the step-count histogram */
template <int N>
__global__ void __launch_bounds__(256) k_div_rows(const __grid_constant__ CArg<N> CA, Operand<N> x, Operand<N> d,
                                                  const uint2 *__restrict__ rec, uint32_t *__restrict__ rows,
                                                  uint8_t *__restrict__ steps, uint8_t *__restrict__ flags,
                                                  DivRowsG *__restrict__ G, int64_t count) {
    const Consts<N> &C = CA.get();
    __shared__ DivK K[N];
    __shared__ uint32_t hist[kDivRowBins];
    divk_fill<N>(C, K);
    for (int i = threadIdx.x; i < kDivRowBins; i += blockDim.x) hist[i] = 0;
    __syncthreads();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        const int st = div_row_build<N>(K, C, rec[k], [&](int i) { return x.load(k, i); },
                                        [&](int i) { return d.load(k, i); }, rows + k * kRowWords<N>(), f);
        steps[k] = (uint8_t)st;
        atomicAdd(&hist[st], 1u);
        if (flags && st == 0) flags[k] = (uint8_t)f;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kDivRowBins; i += blockDim.x)
        if (hist[i]) atomicAdd(&G->hist[i], hist[i]);
}

constexpr int kDivPlaceChunk = 2048;  // numbers per block step of the placement

/* order: the numbers by decreasing step count over the whole call (a
 * counting sort: positions of step count b start after every number with
 * more steps; each block reserves its range per count with one atomic) */
static __global__ void __launch_bounds__(256) k_div_place(const uint8_t *__restrict__ steps, DivRowsG *__restrict__ G,
                                                          int32_t *__restrict__ order, int64_t count) {
    __shared__ uint32_t loc[kDivRowBins], base[kDivRowBins], tot[kDivRowBins];
    for (int i = threadIdx.x; i < kDivRowBins; i += blockDim.x) tot[i] = G->hist[i];
    for (int64_t b0 = (int64_t)blockIdx.x * kDivPlaceChunk; b0 < count; b0 += (int64_t)gridDim.x * kDivPlaceChunk) {
        const int64_t b1 = b0 + kDivPlaceChunk < count ? b0 + kDivPlaceChunk : count;
        for (int i = threadIdx.x; i < kDivRowBins; i += blockDim.x) loc[i] = 0;
        __syncthreads();
        for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) atomicAdd(&loc[steps[k]], 1u);
        __syncthreads();
        for (int t = threadIdx.x; t < kDivRowBins; t += blockDim.x) {
            uint32_t start = 0;  // numbers with more steps than t
            for (int u = t + 1; u < kDivRowBins; u++) start += tot[u];
            base[t] = start + (loc[t] ? atomicAdd(&G->cursor[t], loc[t]) : 0u);
            loc[t] = 0;
        }
        __syncthreads();
        for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
            const uint32_t bin = steps[k];
            order[base[bin] + atomicAdd(&loc[bin], 1u)] = (int32_t)k;
        }
        __syncthreads();
    }
}

/* pass B: positions of the order claimed from G->ctr_b, longest divisions
 * first; the numbers without digit steps (the last G->hist[0] positions) are
 * done already */
template <int N>
__global__ void __launch_bounds__(kDivBlock, div_min_blocks<N>())
    k_div_b(const __grid_constant__ CArg<N> CA, uint32_t *__restrict__ rows, const int32_t *__restrict__ order,
            uint8_t *__restrict__ flags, DivRowsG *__restrict__ G, int64_t count) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 div_smem[];
    DivK *K = reinterpret_cast<DivK *>(div_smem);
    uint32_t *cols = reinterpret_cast<uint32_t *>(K + N);  // layout of divrow_smem_bytes
    divk_fill<N>(C, K);
    __syncthreads();
    const int64_t end = count - (int64_t)G->hist[0];
    divrow_range<N>(K, C, rows, order, flags, end, [&](int c) { return warp_claim(&G->ctr_b, c); },
                    cols + threadIdx.x, blockDim.x);
}

constexpr int kDivOutTile = 64;  // numbers per tile of the output kernel

/* q and r from the rows into the caller's layout: a tile of rows read with
 * coalesced 16-byte loads into shared memory, written residue-major (SoA)
 * or number-major (AoS) */
template <int N>
__global__ void __launch_bounds__(256) k_div_out(const uint32_t *__restrict__ rows, int64_t count, Output<N> q,
                                                 Output<N> r) {
    constexpr int P = kRowPad<N>(), RW = kRowWords<N>(), W = 2 * P + 1;  // tile row: q, r, one word of padding
    constexpr int V = 2 * P / 4;                                         // 16-byte words of q and r per row
    __shared__ uint32_t tile[kDivOutTile * W];
    for (int64_t k0 = (int64_t)blockIdx.x * kDivOutTile; k0 < count; k0 += (int64_t)gridDim.x * kDivOutTile) {
        const int nk = count - k0 < kDivOutTile ? (int)(count - k0) : kDivOutTile;
        for (int t = threadIdx.x; t < nk * V; t += blockDim.x) {
            const int k = t / V, w = t - k * V;
            const uint4 v = __ldcs(reinterpret_cast<const uint4 *>(rows + (k0 + k) * RW) + w);
            uint32_t *dst = tile + k * W + 4 * w;
            dst[0] = v.x;
            dst[1] = v.y;
            dst[2] = v.z;
            dst[3] = v.w;
        }
        __syncthreads();
        if (q.ld) {  // residue-major: a warp writes 32 consecutive numbers of one residue
            for (int t = threadIdx.x; t < N * kDivOutTile; t += blockDim.x) {
                const int i = t / kDivOutTile, k = t - i * kDivOutTile;
                if (k < nk) {
                    q.store(k0 + k, i, tile[k * W + i]);
                    r.store(k0 + k, i, tile[k * W + P + i]);
                }
            }
        } else {
            for (int t = threadIdx.x; t < nk * N; t += blockDim.x) {
                const int k = t / N, i = t - k * N;
                q.store(k0 + k, i, tile[k * W + i]);
                r.store(k0 + k, i, tile[k * W + P + i]);
            }
        }
        __syncthreads();
    }
}

template <int N>
__global__ void __launch_bounds__(kDivBlock, N > 32 ? 4 : 6)
    k_scale_warp(const __grid_constant__ CArg<N> CA, Operand<N> x, const uint32_t *__restrict__ D,
                 uint32_t D_uniform, int32_t *__restrict__ order, int64_t count, int64_t per_warp, Output<N> out,
                 uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 scale_smem[];
    ScK *K = reinterpret_cast<ScK *>(scale_smem);
    uint32_t *hist = reinterpret_cast<uint32_t *>(K + N);
    uint32_t *cols = hist + (blockDim.x / 32) * kDivBins;
    sck_fill<N>(C, K);
    __syncthreads();
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t b = w * per_warp;
    if (b >= count) return;  // whole warp
    const int64_t e = b + per_warp < count ? b + per_warp : count;
    scale_range<N>(K, C, x, D, D_uniform, out, flags, order, b, e, cols + threadIdx.x, blockDim.x,
                   hist + (threadIdx.x / 32) * kDivBins);
}

/* floor(X / 2^D) in one pass (scale_bin, rns_fast.cuh) for n <= 32: a warp
 * takes a contiguous range of numbers, orders it by chunk count (longest
 * first, so the 32 lanes of a group run similar loops) and scales 32 numbers
 * at a time, one per lane.  The chunk tables (M_i and 2^(26 c) mod m_i in
 * 26-bit chunks, rows of bin_ld(N) words) sit in shared memory and are read
 * as 16-byte broadcasts; the residues' products s_i and the n 64-bit
 * accumulators stay in registers. */
constexpr int kScaleBinBlock = 128;

template <int N>
__device__ __forceinline__ int scale_bin_chunks(const Consts<N> &C, unsigned D) {
    return D > (unsigned)C.log2M ? 0 : (int)((D + kBinChunk - 1) / kBinChunk);
}

template <int N>
size_t scale_bin_smem(const Consts<N> &C) {
    return (size_t)C.bin_chunks * bin_ld(N) * 4 * 2 + (size_t)((C.bin_chunks + 3) / 4) * 16 +
           (size_t)(kScaleBinBlock / 32) * kDivBins * 4;
}

template <int N>
__global__ void __launch_bounds__(kScaleBinBlock, 3) k_scale_bin(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                              const uint32_t *__restrict__ Darr, uint32_t D_uniform,
                                                              int32_t *__restrict__ order, int64_t count,
                                                              int64_t per_warp, Output<N> out,
                                                              uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 sb_smem[];
    constexpr int L4 = bin_ld(N) / 4;
    const int chunks = C.bin_chunks, m4 = (chunks + 3) / 4;
    uint4 *MI4 = sb_smem;             // [chunks][L4]  26-bit chunk c of M_i
    uint4 *P4 = MI4 + chunks * L4;    // [chunks][L4]  2^(26 c) mod m_i
    uint32_t *M26 = reinterpret_cast<uint32_t *>(P4 + chunks * L4);  // [m4 * 4] chunks of M
    uint32_t *hist = M26 + m4 * 4;
    for (int w = threadIdx.x; w < chunks * L4; w += blockDim.x) {
        MI4[w] = reinterpret_cast<const uint4 *>(C.bin_mi26)[w];
        P4[w] = reinterpret_cast<const uint4 *>(C.bin_p26)[w];
    }
    for (int w = threadIdx.x; w < m4 * 4; w += blockDim.x) M26[w] = C.bin_m26[w];
    __syncthreads();
    const int64_t wi = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t b = wi * per_warp;
    if (b >= count) return;  // whole warp
    const int64_t e = b + per_warp < count ? b + per_warp : count;
    if (Darr) {
        lpt_order([&](int64_t k) { return min(kDivBins - 1, scale_bin_chunks<N>(C, __ldg(Darr + k))); }, order, b, e,
                  hist + (threadIdx.x / 32) * kDivBins);
    }
    const int lane = threadIdx.x & 31;
    for (int64_t p = b + lane; p < e; p += 32) {
        const int64_t idx = Darr ? b + order[p] : p;
        const unsigned D = Darr ? __ldg(Darr + idx) : D_uniform;
        uint32_t s[4 * L4], bad = 0;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            const uint32_t v = x.load(idx, i);
            bad |= (uint32_t)(v >= C.m[i]);
            s[i] = mulmod_shoup(v, C.w[i], C.w_sh[i], C.m[i]);
        }
GRNS_UNROLL_TO(4 * L4)
        for (int i = N; i < 4 * L4; i++) s[i] = 0;
        if (flags) flags[idx] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
        if (bad || D > (unsigned)C.log2M || D == 0) {  // invalid or 2^D > X: 0; D = 0: X
#pragma unroll 4
            for (int i = 0; i < N; i++) out.store(idx, i, (bad || D) ? 0u : x.load(idx, i));
            continue;
        }
        const uint32_t kk = scale_bin_rank<N>(C, [&](int i) { return s[i]; }, [&](int i) { return x.load(idx, i); });
        const int nch = (int)((D + kBinChunk - 1) / kBinChunk);
        const uint32_t top = D % kBinChunk ? (1u << (D % kBinChunk)) - 1u : kBinMask;
        uint64_t acc[4 * L4];
GRNS_UNROLL_TO(4 * L4)
        for (int i = 0; i < 4 * L4; i++) acc[i] = 0;
        int64_t carry = 0;
#pragma unroll 1
        for (int c = 0; c < nch; c++) {
            const uint4 *t = MI4 + c * L4;
            uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
GRNS_UNROLL_TO(L4)
            for (int q = 0; q < L4; q++) {
                const uint4 v = t[q];
                a0 += (uint64_t)s[4 * q] * v.x;
                a1 += (uint64_t)s[4 * q + 1] * v.y;
                a2 += (uint64_t)s[4 * q + 2] * v.z;
                a3 += (uint64_t)s[4 * q + 3] * v.w;
            }
            const int64_t v = (int64_t)((a0 + a1) + (a2 + a3)) - (int64_t)kk * M26[c] + carry;
            carry = v >> kBinChunk;  // floor division (arithmetic shift)
            const uint32_t r = (uint32_t)v & (c == nch - 1 ? top : kBinMask);
            const uint4 *pp = P4 + c * L4;
GRNS_UNROLL_TO(L4)
            for (int q = 0; q < L4; q++) {
                const uint4 w = pp[q];
                acc[4 * q] += (uint64_t)r * w.x;
                acc[4 * q + 1] += (uint64_t)r * w.y;
                acc[4 * q + 2] += (uint64_t)r * w.z;
                acc[4 * q + 3] += (uint64_t)r * w.w;
            }
        }
GRNS_UNROLL_N
        for (int i = 0; i < N; i++)
            out.store(idx, i, scale_bin_finish<N>(C, i, x.load(idx, i), bin_mod64<N>(C, i, acc[i]), D));
    }
}

/* one power-of-two scaling per warp (div_coop.cuh), for the 128- and
 * 256-moduli sets */
template <int N>
__global__ void __launch_bounds__(kDivCoopBlock)
    k_scale_coop(const __grid_constant__ CArg<N> CA, Operand<N> x, const uint32_t *__restrict__ D,
                 uint32_t D_uniform, int64_t count, Output<N> out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    constexpr int J = N / 32;
    __shared__ uint32_t scratch[kDivCoopBlock / 32][N];
    const int lane = threadIdx.x & 31;
    uint32_t *sc = scratch[threadIdx.x >> 5];
    const int64_t warps = ((int64_t)gridDim.x * kDivCoopBlock) >> 5;
    for (int64_t k = ((int64_t)blockIdx.x * kDivCoopBlock + threadIdx.x) >> 5; k < count; k += warps) {
        uint32_t xa[J], ya[J];
        bool bad = false;
#pragma unroll
        for (int j = 0; j < J; j++) {
            xa[j] = x.load(k, lane + 32 * j);
            bad |= xa[j] >= C.m[lane + 32 * j];
        }
        const uint32_t f = __any_sync(kWarpFull, bad) ? kFlagInvalidInput : 0u;
        const unsigned dk = D ? __ldg(D + k) : D_uniform;
        if (f) {
#pragma unroll
            for (int j = 0; j < J; j++) ya[j] = 0;
        } else {
            scale_warp_coop<N>(C, ya, xa, dk, lane, sc);
        }
#pragma unroll
        for (int j = 0; j < J; j++) out.store(k, lane + 32 * j, ya[j]);
        if (flags && lane == 0) flags[k] = (uint8_t)f;
    }
}

/* the reference's power-of-two scaling (scale2pow_ref), one number per thread */
template <int N>
__global__ void __launch_bounds__(128) k_scale(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                               const uint32_t *__restrict__ D, uint32_t D_uniform, int64_t count,
                                               Output<N> out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], ya[N], f = 0;
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            f |= xa[i] >= C.m[i] ? kFlagInvalidInput : 0u;
        }
        unsigned dk = D ? __ldg(D + k) : D_uniform;
        if (f) {
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) ya[i] = 0;
        } else {
            scale2pow_ref<N>(C, ya, xa, dk);
        }
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) out.store(k, i, ya[i]);
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N>
grns_status run_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count, uint32_t *q,
                    uint32_t *r, uint8_t *flags, cudaStream_t s, int min_per_warp, int64_t ldo) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE) {
        k_div<N><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{d, ld},
                                                               count, Output<N>{q, ldo}, Output<N>{r, ldo}, flags);
        return cuda_status(cudaGetLastError());
    }
    if constexpr (N > 64) {
        /* one division per warp: the warp passes' shared-memory columns (2n
         * words a thread) do not fit, and one number per thread keeps its
         * residue arrays in local memory */
        k_div_coop<N><<<grid_for(c, count * 32, kDivCoopBlock, 16), kDivCoopBlock, 0, s>>>(
            consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{d, ld}, count, Output<N>{q, ldo}, Output<N>{r, ldo}, flags);
        (void)min_per_warp;
        return cuda_status(cudaGetLastError());
    } else {
    /* fast path (div_warp.cuh): pass A writing records, the rows, the longest-first order
     * over the whole call, pass B over the rows, the rows to the caller's
     * layout -- in chunks whose scratch stays below kDivScratchBytes */
    constexpr size_t RB = (size_t)kRowWords<N>() * 4;
    const size_t smem_a = divprep_smem_bytes<N>(kDivBlock), smem_b = divrow_smem_bytes<N>(kDivBlock);
    static std::atomic<int> occ_a[kOccDevices], occ_b[kOccDevices], occ_r[kOccDevices];  // resident blocks per SM
    const int occ[3] = {resident_blocks(occ_a, c, k_div_a<N>, kDivBlock, smem_a),
                        resident_blocks(occ_b, c, k_div_b<N>, kDivBlock, smem_b),
                        resident_blocks(occ_r, c, k_div_rows<N>, 256, 0)};
    const int64_t chunk_max = (int64_t)std::max<size_t>(4096, (kDivScratchBytes / (RB + 13)) & ~(size_t)4095);
    const int64_t chunk = count < chunk_max ? count : chunk_max;
    /* warps: every resident one, fewer when a warp would get under min_per_warp
     * numbers (or one per lane's worth) */
    auto grid_of = [&](int o, int64_t n) {
        int64_t warps = (n + 31) / 32;
        if (min_per_warp > 0 && warps > (n + min_per_warp - 1) / min_per_warp)
            warps = (n + min_per_warp - 1) / min_per_warp;
        const int64_t cap = (int64_t)c->sm_count * o * (kDivBlock / 32);
        if (warps > cap) warps = cap;
        if (warps < 1) warps = 1;
        return (unsigned)((warps * 32 + kDivBlock - 1) / kDivBlock);
    };
    /* scratch: rows, records, the order, the step counts, the grid-wide state */
    const size_t rows_bytes = (size_t)chunk * RB, rec_bytes = (size_t)chunk * 8;
    const size_t ord_bytes = ((size_t)chunk * 4 + 15) & ~(size_t)15;
    const size_t steps_bytes = ((size_t)chunk + 15) & ~(size_t)15;  // every part 16-byte aligned
    void *scratch = nullptr;
    cudaError_t e =
        scratch_alloc(c, &scratch, rows_bytes + rec_bytes + ord_bytes + steps_bytes + sizeof(DivRowsG), s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t *rows = (uint32_t *)scratch;
    uint2 *rec = (uint2 *)((char *)scratch + rows_bytes);
    int32_t *order = (int32_t *)((char *)scratch + rows_bytes + rec_bytes);
    uint8_t *steps = (uint8_t *)scratch + rows_bytes + rec_bytes + ord_bytes;
    DivRowsG *G = (DivRowsG *)((char *)scratch + rows_bytes + rec_bytes + ord_bytes + steps_bytes);
    for (int64_t c0 = 0; c0 < count && e == cudaSuccess; c0 += chunk) {
        const int64_t n = count - c0 < chunk ? count - c0 : chunk;
        const int64_t off = ld ? c0 : c0 * N;  // first number of the chunk (SoA columns keep the leading dimension)
        const int64_t offo = ldo ? c0 : c0 * N;
        const Operand<N> X{x + off, ld}, Dv{d + off, ld};
        uint8_t *fl = flags ? flags + c0 : nullptr;
        e = cudaMemsetAsync(G, 0, sizeof(DivRowsG), s);
        if (e == cudaSuccess) {
            k_div_a<N><<<grid_of(occ[0], n), kDivBlock, smem_a, s>>>(consts_of<N>(c), X, Dv, rec, G, n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            k_div_rows<N><<<grid_for(c, n, 256, occ[2]), 256, 0, s>>>(consts_of<N>(c), X, Dv, rec, rows, steps, fl, G,
                                                                     n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            k_div_place<<<grid_for(c, (n + kDivPlaceChunk - 1) / kDivPlaceChunk, 1, 8), 256, 0, s>>>(steps, G, order,
                                                                                                   n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            k_div_b<N><<<grid_of(occ[1], n), kDivBlock, smem_b, s>>>(consts_of<N>(c), rows, order, fl, G, n);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) {
            k_div_out<N><<<grid_for(c, (n + kDivOutTile - 1) / kDivOutTile, 1, 8), 256, 0, s>>>(
                rows, n, Output<N>{q + offo, ldo}, Output<N>{r + offo, ldo});
            e = cudaGetLastError();
        }
    }
    scratch_free(scratch, s);
    return cuda_status(e);
    }
}

template <int N>
grns_status run_scale_steps(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                            int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp,
                            int64_t ldo);

template <int N>
grns_status run_scale(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld, int64_t count,
                      uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp, int64_t ldo) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE) {
        k_scale<N><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, count,
                                                                 Output<N>{out, ldo}, flags);
        return cuda_status(cudaGetLastError());
    }
    if constexpr (N <= 32) {  /* one pass over the chunks of X mod 2^D */
        const size_t smem = scale_bin_smem<N>(consts_of<N>(c));
        static std::atomic<int> per_sm_bin[kOccDevices];
        const int occ = resident_blocks(per_sm_bin, c, k_scale_bin<N>, kScaleBinBlock, smem);
        const int64_t warps_cap = (int64_t)c->sm_count * occ * (kScaleBinBlock / 32);
        int64_t warps = (count + 63) / 64;  // ranges of 64 numbers or more: two lane groups to order
        if (min_per_warp > 0 && warps > (count + min_per_warp - 1) / min_per_warp)
            warps = (count + min_per_warp - 1) / min_per_warp;
        if (warps > warps_cap) warps = warps_cap;
        if (warps < 1) warps = 1;
        const int64_t per_warp = (count + warps - 1) / warps;
        const unsigned grid = (unsigned)((warps * 32 + kScaleBinBlock - 1) / kScaleBinBlock);
        int32_t *order = nullptr;
        cudaError_t e = cudaSuccess;
        if (D) e = scratch_alloc(c, (void **)&order, (size_t)count * sizeof(int32_t), s);
        if (e != cudaSuccess) return cuda_status(e);
        k_scale_bin<N><<<grid, kScaleBinBlock, smem, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, order, count,
                                                         per_warp > 0 ? per_warp : 1, Output<N>{out, ldo}, flags);
        e = cudaGetLastError();
        if (order) scratch_free(order, s);
        return cuda_status(e);
    } else if constexpr (N <= 64) {
        return run_scale_steps<N>(c, x, D, Du, ld, count, out, flags, s, min_per_warp, ldo);
    } else {  // exact 52-bit steps, one number per warp
        k_scale_coop<N><<<grid_for(c, count * 32, kDivCoopBlock, 16), kDivCoopBlock, 0, s>>>(
            consts_of<N>(c), Operand<N>{x, ld}, D, Du, count, Output<N>{out, ldo}, flags);
        return cuda_status(cudaGetLastError());
    }
}

/* n = 64: exact 52-bit steps, warps over contiguous ranges (scale_warp.cuh) */
template <int N>
grns_status run_scale_steps(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                            int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp,
                            int64_t ldo) {
    const size_t smem = scale_smem_bytes<N>(kDivBlock);
    static std::atomic<int> per_sm[kOccDevices];  // resident blocks per SM, per device
    const int occ = resident_blocks(per_sm, c, k_scale_warp<N>, kDivBlock, smem);
    const int64_t warps_cap = (int64_t)c->sm_count * occ * (kDivBlock / 32);
    int64_t warps = (count + 31) / 32;
    if (min_per_warp > 0 && warps > (count + min_per_warp - 1) / min_per_warp)
        warps = (count + min_per_warp - 1) / min_per_warp;
    if (warps > warps_cap) warps = warps_cap;
    if (warps < 1) warps = 1;
    const int64_t per_warp = (count + warps - 1) / warps;
    const unsigned grid = (unsigned)((warps * 32 + kDivBlock - 1) / kDivBlock);
    int32_t *order = nullptr;  // longest-first order scratch (per-number exponents only)
    cudaError_t e = cudaSuccess;
    if (D) e = scratch_alloc(c, (void **)&order, (size_t)count * sizeof(int32_t), s);
    if (e != cudaSuccess) return cuda_status(e);
    k_scale_warp<N><<<grid, kDivBlock, smem, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, order, count,
                                                  per_warp > 0 ? per_warp : 1, Output<N>{out, ldo}, flags);
    e = cudaGetLastError();
    if (order) scratch_free(order, s);
    return cuda_status(e);
}

template <int N>
size_t div_scratch_of(int64_t count) {
    constexpr size_t RB = (size_t)kRowWords<N>() * 4;
    const int64_t chunk_max = (int64_t)std::max<size_t>(4096, (kDivScratchBytes / (RB + 13)) & ~(size_t)4095);
    const int64_t chunk = count < chunk_max ? count : chunk_max;
    return (size_t)chunk * (RB + 8) + (((size_t)chunk * 4 + 15) & ~(size_t)15) + (((size_t)chunk + 15) & ~(size_t)15) +
           sizeof(DivRowsG);
}

/* the per-count entry points: extern here, instantiated for this unit's counts */
#define GRNS_DIV_ROOTS_(n, EXT)                                                                                      \
    EXT template grns_status run_div<n>(const grns_ctx *, const uint32_t *, const uint32_t *, int64_t, int64_t,        \
                                        uint32_t *, uint32_t *, uint8_t *, cudaStream_t, int, int64_t);              \
    EXT template grns_status run_scale<n>(const grns_ctx *, const uint32_t *, const uint32_t *, uint32_t, int64_t,     \
                                          int64_t, uint32_t *, uint8_t *, cudaStream_t, int, int64_t);               \
    EXT template size_t div_scratch_of<n>(int64_t);
#define GRNS_EXTERN_(n) GRNS_DIV_ROOTS_(n, extern)
#define GRNS_DEFINE_(n) GRNS_DIV_ROOTS_(n, )
GRNS_FOR_EACH_N(GRNS_EXTERN_)
GRNS_PART_N(GRNS_DEFINE_)
#undef GRNS_EXTERN_
#undef GRNS_DEFINE_

#if GRNS_PART_MAIN
size_t div_scratch_bytes(const grns_ctx *c, int64_t count) {
#define C_(n) return div_scratch_of<n>(count)
    GRNS_SWITCH_N(c->n, return 0)
#undef C_
}

grns_status launch_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                       uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s, int min_per_warp, int64_t ld_out) {
    const int64_t ldo = ld_out < 0 ? ld : ld_out;
#define C_(n) return run_div<n>(c, x, d, ld, count, q, r, flags, s, min_per_warp, ldo)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_scale2pow(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                             int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp,
                             int64_t ld_out) {
    const int64_t ldo = ld_out < 0 ? ld : ld_out;
#define C_(n) return run_scale<n>(c, x, D, Du, ld, count, out, flags, s, min_per_warp, ldo)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

#endif  // GRNS_PART_MAIN

}  // namespace grns
