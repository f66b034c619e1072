/*
 * grns_gb300 -- division and power-of-two scaling kernels.
 *   k_div      : q = floor(X/D), r = X - qD (reference src/rnsdiv.cuh:128),
 *                reference-faithful FP64 form, one thread per number
 *   k_div_a, k_div_sort, k_div_b : the same results on the integer fast
 *                path (div_warp.cuh): pass A over the whole grid, a counting
 *                sort by step count inside segments of consecutive numbers,
 *                pass B segment by segment, longest first, numbers claimed
 *                from grid-wide counters
 *   k_scale    : floor(X / 2^D)             (reference src/rnsscal.cuh:207)
 */
#include "div_warp.cuh"
#include "scale_warp.cuh"
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

template <int N, bool FAST>
__global__ void __launch_bounds__(128) k_div(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> d,
                                             int64_t count, Output<N> q, Output<N> r, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], da[N], qa[N], ra[N], f = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            da[i] = d.load(k, i);
            f |= (xa[i] >= C.m[i] || da[i] >= C.m[i]) ? kFlagInvalidInput : 0u;
        }
        if (f) {
#pragma unroll
            for (int i = 0; i < N; i++) { qa[i] = 0; ra[i] = 0; }
        } else if (FAST) {
            div_fast<N>(C, qa, ra, xa, da, f);
        } else {
            div_ref<N>(C, qa, ra, xa, da, f);
        }
#pragma unroll
        for (int i = 0; i < N; i++) {
            q.store(k, i, qa[i]);
            r.store(k, i, ra[i]);
        }
        if (flags) flags[k] = (uint8_t)f;
    }
}

constexpr int kDivBlock = 128;

/* resident 128-thread blocks per SM the register budget must allow: shared
 * memory (3N words per thread) allows 4 at n <= 32 and 2 at n = 64 */
#ifndef GRNS_DIV_MIN_BLOCKS
#define GRNS_DIV_MIN_BLOCKS 4
#endif
template <int N>
constexpr int div_min_blocks() {
    return N > 32 ? 2 : GRNS_DIV_MIN_BLOCKS;
}

/* pass A of the grid-wide division: numbers claimed from G->ctr_a, records
 * into rec */
template <int N>
__global__ void __launch_bounds__(kDivBlock, N > 32 ? 3 : 6)
    k_div_a(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> d, uint2 *__restrict__ rec,
            DivGlobal *__restrict__ G, int64_t count) {
    extern __shared__ uint4 div_smem[];
    DivK *K = reinterpret_cast<DivK *>(div_smem);
    uint32_t *cols = reinterpret_cast<uint32_t *>(K + N) + (blockDim.x / 32) * kDivBins;  // layout of div_smem_bytes
    divk_fill<N>(C, K);
    __syncthreads();
    /* prefetch distance: one number per lane of the grid ahead, about what the
     * grid claims while a number is normalised */
    const int64_t lanes = (int64_t)gridDim.x * blockDim.x;
    divnorm_range<N>(K, C, x, d, rec, count, [&](int c) { return warp_claim(&G->ctr_a, c); }, lanes,
                     cols + threadIdx.x, blockDim.x);
}

constexpr int kDivSegment = 4096;  // numbers sorted together: contiguous, so pass B's loads stay L2-local

/* order: within each segment of kDivSegment consecutive numbers, the numbers
 * by decreasing step count (one block per segment, a counting sort in shared
 * memory).  Pass B claims positions in order, so the grid works through the
 * segments one after another, longest divisions first inside each, and the
 * operands it touches at any time span a few segments (L2-resident). */
__global__ void __launch_bounds__(256) k_div_sort(const uint2 *__restrict__ rec, int32_t *__restrict__ order,
                                                  int64_t count) {
    __shared__ uint32_t h[kDivBins];
    for (int64_t b0 = (int64_t)blockIdx.x * kDivSegment; b0 < count; b0 += (int64_t)gridDim.x * kDivSegment) {
        const int64_t b1 = b0 + kDivSegment < count ? b0 + kDivSegment : count;
        for (int i = threadIdx.x; i < kDivBins; i += blockDim.x) h[i] = 0;
        __syncthreads();
        for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) atomicAdd(&h[dv_rec_steps(rec[k])], 1u);
        __syncthreads();
        if (threadIdx.x < 32) {  /* exclusive prefix over bins in decreasing order (lane l: bins 63 - l, 31 - l) */
            const int lane = threadIdx.x;
            const uint32_t h0 = h[63 - lane], h1 = h[31 - lane];
            uint32_t s0 = h0, s1 = h1;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t a0 = __shfl_up_sync(0xffffffffu, s0, o), a1 = __shfl_up_sync(0xffffffffu, s1, o);
                if (lane >= o) {
                    s0 += a0;
                    s1 += a1;
                }
            }
            s1 += __shfl_sync(0xffffffffu, s0, 31);
            h[63 - lane] = s0 - h0;
            h[31 - lane] = s1 - h1;
        }
        __syncthreads();
        for (int64_t k = b0 + threadIdx.x; k < b1; k += blockDim.x) {
            const uint32_t p = atomicAdd(&h[dv_rec_steps(rec[k])], 1u);
            order[b0 + p] = (int32_t)k;
        }
        __syncthreads();
    }
}

/* pass B of the grid-wide division: positions of the sorted order claimed
 * from G->ctr_b, longest divisions first */
template <int N>
__global__ void __launch_bounds__(kDivBlock, div_min_blocks<N>())
    k_div_b(const __grid_constant__ Consts<N> C, Operand<N> x, Operand<N> d, const uint2 *__restrict__ rec,
            const int32_t *__restrict__ order, DivGlobal *__restrict__ G, int64_t count, Output<N> q, Output<N> r,
            uint8_t *__restrict__ flags) {
    extern __shared__ uint4 div_smem[];
    DivK *K = reinterpret_cast<DivK *>(div_smem);
    uint32_t *cols = reinterpret_cast<uint32_t *>(K + N) + (blockDim.x / 32) * kDivBins;
    divk_fill<N>(C, K);
    __syncthreads();
    divloop_range<N>(K, C, x, d, rec, order, q, r, flags, 0, count,
                     [&](int c) { return warp_claim(&G->ctr_b, c); }, cols + threadIdx.x, blockDim.x);
}

template <int N>
__global__ void __launch_bounds__(kDivBlock, N > 32 ? 4 : 6)
    k_scale_warp(const __grid_constant__ Consts<N> C, Operand<N> x, const uint32_t *__restrict__ D,
                 uint32_t D_uniform, int32_t *__restrict__ order, int64_t count, int64_t per_warp, Output<N> out,
                 uint8_t *__restrict__ flags) {
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

template <int N, bool FAST>
__global__ void __launch_bounds__(128) k_scale(const __grid_constant__ Consts<N> C, Operand<N> x,
                                               const uint32_t *__restrict__ D, uint32_t D_uniform, int64_t count,
                                               Output<N> out, uint8_t *__restrict__ flags) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t xa[N], ya[N], f = 0;
#pragma unroll
        for (int i = 0; i < N; i++) {
            xa[i] = x.load(k, i);
            f |= xa[i] >= C.m[i] ? kFlagInvalidInput : 0u;
        }
        unsigned dk = D ? __ldg(D + k) : D_uniform;
        if (f) {
#pragma unroll
            for (int i = 0; i < N; i++) ya[i] = 0;
        } else if (FAST) {
            scale_fast<N>(C, ya, xa, dk);
        } else {
            scale2pow_ref<N>(C, ya, xa, dk);
        }
#pragma unroll
        for (int i = 0; i < N; i++) out.store(k, i, ya[i]);
        if (flags) flags[k] = (uint8_t)f;
    }
}

template <int N>
static grns_status run_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                           uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s, int min_per_warp) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE) {
        k_div<N, false><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, Operand<N>{d, ld},
                                                               count, Output<N>{q, ld}, Output<N>{r, ld}, flags);
        return cuda_status(cudaGetLastError());
    }
    /* fast path: pass A, a counting sort by step count, pass B (div_warp.cuh),
     * each over the whole grid with numbers claimed from counters */
    const size_t smem = div_smem_bytes<N>(kDivBlock), smem_a = divnorm_smem_bytes<N>(kDivBlock);
    static std::atomic<int> occ_a[kOccDevices], occ_b[kOccDevices];  // resident blocks per SM, per device
    const int occ[2] = {resident_blocks(occ_a, c, k_div_a<N>, kDivBlock, smem_a),
                        resident_blocks(occ_b, c, k_div_b<N>, kDivBlock, smem)};
    /* warps: every resident one, fewer when a warp would get under min_per_warp
     * numbers (or one per lane's worth) */
    auto grid_of = [&](int o) {
        int64_t warps = (count + 31) / 32;
        if (min_per_warp > 0 && warps > (count + min_per_warp - 1) / min_per_warp)
            warps = (count + min_per_warp - 1) / min_per_warp;
        const int64_t cap = (int64_t)c->sm_count * o * (kDivBlock / 32);
        if (warps > cap) warps = cap;
        if (warps < 1) warps = 1;
        return (unsigned)((warps * 32 + kDivBlock - 1) / kDivBlock);
    };
    /* scratch: records, order, the grid-wide counters */
    void *scratch = nullptr;
    const size_t rec_bytes = (size_t)count * sizeof(uint2), ord_bytes = ((size_t)count * 4 + 15) & ~(size_t)15;
    cudaError_t e = scratch_alloc(c, &scratch, rec_bytes + ord_bytes + sizeof(DivGlobal), s);
    if (e != cudaSuccess) return cuda_status(e);
    uint2 *rec = (uint2 *)scratch;
    int32_t *order = (int32_t *)((char *)scratch + rec_bytes);
    DivGlobal *G = (DivGlobal *)((char *)scratch + rec_bytes + ord_bytes);
    e = cudaMemsetAsync(G, 0, sizeof(DivGlobal), s);
    const Operand<N> X{x, ld}, Dv{d, ld};
    if (e == cudaSuccess) {
        k_div_a<N><<<grid_of(occ[0]), kDivBlock, smem_a, s>>>(consts_of<N>(c), X, Dv, rec, G, count);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_div_sort<<<grid_for(c, (count + kDivSegment - 1) / kDivSegment, 1, 8), 256, 0, s>>>(rec, order, count);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_div_b<N><<<grid_of(occ[1]), kDivBlock, smem, s>>>(consts_of<N>(c), X, Dv, rec, order, G, count,
                                                             Output<N>{q, ld}, Output<N>{r, ld}, flags);
        e = cudaGetLastError();
    }
    scratch_free(scratch, s);
    return cuda_status(e);
}

template <int N>
static grns_status run_scale(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                             int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp) {
    const int B = 128;
    if (c->path == GRNS_PATH_REFERENCE) {
        k_scale<N, false><<<grid_for(c, count, B, 16), B, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, D, Du, count,
                                                                 Output<N>{out, ld}, flags);
        return cuda_status(cudaGetLastError());
    }
    /* fast path: warps over contiguous ranges (scale_warp.cuh) */
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
                                                  per_warp > 0 ? per_warp : 1, Output<N>{out, ld}, flags);
    e = cudaGetLastError();
    if (order) scratch_free(order, s);
    return cuda_status(e);
}

grns_status launch_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                       uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s, int min_per_warp) {
#define C_(n) return run_div<n>(c, x, d, ld, count, q, r, flags, s, min_per_warp)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status launch_scale2pow(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t Du, int64_t ld,
                             int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s, int min_per_warp) {
#define C_(n) return run_scale<n>(c, x, D, Du, ld, count, out, flags, s, min_per_warp)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
