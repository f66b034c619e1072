/*
 * grns_gb300 -- maximum of an RNS array in ONE launch.
 *
 * Replaces cuda::rns_max (reference src/dpp/rnsmax.cuh:129-138), which runs
 * an evaluation kernel writing N xinterval_t to a buffer, two tree kernels
 * and a copy kernel, then synchronises the device.  Here each thread
 * evaluates its numbers in registers and keeps its best candidate
 * (interval, index); candidates are reduced by warp shuffles, then across
 * warps in shared memory, then across blocks by the last block to finish
 * (one atomic ticket per block).  Comparisons follow rns_max_cmp
 * (:24-48): interval test first, exact mixed-radix comparison only when
 * the intervals overlap.  Equal values resolve to the smallest index.
 */
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"

namespace grns {

struct Cand {
    Er lo, up;
    int64_t idx;  // < 0: empty
};

/* exact comparison of elements ia, ib (rare: overlapping intervals) */
template <int N>
__device__ __noinline__ int ref_tie(const Consts<N> &C, const Operand<N> x, int64_t ia, int64_t ib) {
    return cmp_tie<N>(C, [&](int i) { return x.load(ia, i); }, [&](int i) { return x.load(ib, i); });
}

template <int N>
__device__ __forceinline__ bool better(const Consts<N> &C, const Operand<N> &x, const Cand &a, const Cand &b) {
    if (b.idx < 0) return a.idx >= 0;
    if (a.idx < 0) return false;
    int r = cmp_intervals<N>(a.lo, a.up, b.lo, b.up);
    if (r == 2) r = ref_tie<N>(C, x, a.idx, b.idx);
    if (r != 0) return r > 0;
    return a.idx < b.idx;
}

__device__ __forceinline__ Cand shfl_cand(const Cand &c, int src_lane_xor) {
    Cand o;
    o.lo.frac = __shfl_xor_sync(0xffffffffu, c.lo.frac, src_lane_xor);
    o.lo.exp = __shfl_xor_sync(0xffffffffu, c.lo.exp, src_lane_xor);
    o.up.frac = __shfl_xor_sync(0xffffffffu, c.up.frac, src_lane_xor);
    o.up.exp = __shfl_xor_sync(0xffffffffu, c.up.exp, src_lane_xor);
    o.idx = __shfl_xor_sync(0xffffffffu, c.idx, src_lane_xor);
    return o;
}

template <int N>
__device__ __forceinline__ Cand block_reduce(const Consts<N> &C, const Operand<N> &x, Cand best, Cand *sm) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Cand o = shfl_cand(best, off);
        if (better<N>(C, x, o, best)) best = o;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) sm[wid] = best;
    __syncthreads();
    if (wid == 0) {
        best = lane < nw ? sm[lane] : Cand{{0.0, 0}, {0.0, 0}, -1};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            Cand o = shfl_cand(best, off);
            if (better<N>(C, x, o, best)) best = o;
        }
    }
    return best;  // valid in thread 0
}

template <int N>
__global__ void __launch_bounds__(256) k_max(const __grid_constant__ CArg<N> CA, Operand<N> x, int64_t count,
                                             uint32_t *__restrict__ out_value, int64_t *__restrict__ out_index,
                                             unsigned *__restrict__ ticket, Cand *__restrict__ partial) {
    const Consts<N> &C = CA.get();
    __shared__ Cand sm[32];
    __shared__ bool last;
    Cand best{{0.0, 0}, {0.0, 0}, -1};
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = 0;
        Cand c;
        c.idx = k;
        eval<N>(C, [&](int i) { return x.load(k, i); }, c.lo, c.up, f);
        if (better<N>(C, x, c, best)) best = c;
    }
    best = block_reduce<N>(C, x, best, sm);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = best;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    best = Cand{{0.0, 0}, {0.0, 0}, -1};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const Cand *p = partial + b;  /* written by other blocks: read through L2 */
        Cand c;
        c.lo.frac = __ldcg(&p->lo.frac);
        c.lo.exp = __ldcg((const long long *)&p->lo.exp);
        c.up.frac = __ldcg(&p->up.frac);
        c.up.exp = __ldcg((const long long *)&p->up.exp);
        c.idx = __ldcg((const long long *)&p->idx);
        if (better<N>(C, x, c, best)) best = c;
    }
    __syncthreads();
    best = block_reduce<N>(C, x, best, sm);
    if (threadIdx.x == 0) sm[0] = best;
    __syncthreads();
    const int64_t bi = sm[0].idx;
    if (threadIdx.x == 0 && out_index) *out_index = bi;
    for (int i = threadIdx.x; i < N; i += blockDim.x) out_value[i] = bi >= 0 ? x.load(bi, i) : 0u;
}

/* ---- fast path: candidates are (64-bit fixed-point fraction, index) ---- */
struct FCand {
    uint64_t a;    // sum_i s_i ceil(2^64/m_i) mod 2^64 (>= X/M * 2^64, within E)
    int64_t idx;   // < 0: empty
};

/* 96-bit then exact comparison of elements ip, iq (rare: fractions within E) */
template <int N>
__device__ __noinline__ int fast_tie(const Consts<N> &C, const Operand<N> x, int64_t ip, int64_t iq) {
    return cmp_fx96_then_exact<N>(C, [&](int i) { return x.load(ip, i); }, [&](int i) { return x.load(iq, i); });
}

template <int N>
__device__ __forceinline__ bool fbetter(const Consts<N> &C, const Operand<N> &x, const FCand &p, const FCand &q) {
    if (q.idx < 0) return p.idx >= 0;
    if (p.idx < 0) return false;
    int r = fx64_order(p.a, q.a, C.E);
    if (r == 2) r = fast_tie<N>(C, x, p.idx, q.idx);
    if (r != 0) return r > 0;
    return p.idx < q.idx;
}

template <int N>
__device__ __forceinline__ FCand fblock_reduce(const Consts<N> &C, const Operand<N> &x, FCand best, FCand *sm) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        FCand o{__shfl_xor_sync(0xffffffffu, best.a, off), __shfl_xor_sync(0xffffffffu, best.idx, off)};
        if (fbetter<N>(C, x, o, best)) best = o;
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (lane == 0) sm[wid] = best;
    __syncthreads();
    if (wid == 0) {
        best = lane < nw ? sm[lane] : FCand{0, -1};
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            FCand o{__shfl_xor_sync(0xffffffffu, best.a, off), __shfl_xor_sync(0xffffffffu, best.idx, off)};
            if (fbetter<N>(C, x, o, best)) best = o;
        }
    }
    return best;
}

template <int N>
__global__ void __launch_bounds__(256, 3) k_max_fast(const __grid_constant__ CArg<N> CA, Operand<N> x, int64_t count,
                                                  uint32_t *__restrict__ out_value, int64_t *__restrict__ out_index,
                                                  unsigned *__restrict__ ticket, FCand *__restrict__ partial) {
    const Consts<N> &C = CA.get();
    __shared__ FCand sm[32];
    __shared__ bool last;
    FCand best{0, -1};
    if (x.ld != 0 && x.ld % 4 == 0 && ((uintptr_t)x.base % 16) == 0) {
        /* SoA: 4 consecutive numbers per thread, one 128-bit load per modulus slice */
        const int64_t quads = count / 4;
        for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < quads;
             t += (int64_t)gridDim.x * blockDim.x) {
            const int64_t k = 4 * t;
            uint64_t a0 = 0, a1 = 0, a2 = 0, a3 = 0;
GRNS_UNROLL_N
            for (int i = 0; i < N; i++) {
                const uint4 v = __ldcs(reinterpret_cast<const uint4 *>(x.base + (int64_t)i * x.ld + k));
                const uint32_t cl = C.c64l[i], ch = C.c64h[i];
                a0 += (uint64_t)v.x * cl; a0 += (uint64_t)(uint32_t)(v.x * ch) << 32;
                a1 += (uint64_t)v.y * cl; a1 += (uint64_t)(uint32_t)(v.y * ch) << 32;
                a2 += (uint64_t)v.z * cl; a2 += (uint64_t)(uint32_t)(v.z * ch) << 32;
                a3 += (uint64_t)v.w * cl; a3 += (uint64_t)(uint32_t)(v.w * ch) << 32;
            }
            FCand c0{a0, k}, c1{a1, k + 1}, c2{a2, k + 2}, c3{a3, k + 3};
            if (fbetter<N>(C, x, c0, best)) best = c0;
            if (fbetter<N>(C, x, c1, best)) best = c1;
            if (fbetter<N>(C, x, c2, best)) best = c2;
            if (fbetter<N>(C, x, c3, best)) best = c3;
        }
        for (int64_t k = 4 * quads + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count;
             k += (int64_t)gridDim.x * blockDim.x) {
            FCand c{fx64<N>(C, [&](int i) { return x.load(k, i); }), k};
            if (fbetter<N>(C, x, c, best)) best = c;
        }
    } else {
        for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count;
             k += (int64_t)gridDim.x * blockDim.x) {
            FCand c{fx64<N>(C, [&](int i) { return x.load(k, i); }), k};
            if (fbetter<N>(C, x, c, best)) best = c;
        }
    }
    best = fblock_reduce<N>(C, x, best, sm);
    if (threadIdx.x == 0) {
        partial[blockIdx.x] = best;
        __threadfence();
        last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    best = FCand{0, -1};
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
        const FCand *p = partial + b;  /* written by other blocks: read through L2 */
        FCand c{(uint64_t)__ldcg((const unsigned long long *)&p->a), __ldcg((const long long *)&p->idx)};
        if (fbetter<N>(C, x, c, best)) best = c;
    }
    __syncthreads();
    best = fblock_reduce<N>(C, x, best, sm);
    if (threadIdx.x == 0) sm[0] = best;
    __syncthreads();
    const int64_t bi = sm[0].idx;
    if (threadIdx.x == 0 && out_index) *out_index = bi;
    for (int i = threadIdx.x; i < N; i += blockDim.x) out_value[i] = bi >= 0 ? x.load(bi, i) : 0u;
}

constexpr int kMaxBlock = 256;
constexpr int kMaxPerSm = 4;

static unsigned max_grid(const grns_ctx *c, int64_t count) { return grid_for(c, count, kMaxBlock, kMaxPerSm); }

size_t max_scratch_bytes(const grns_ctx *c, int64_t count) { return 64 + (size_t)max_grid(c, count) * sizeof(Cand); }

template <int N>
static grns_status run_max(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, uint32_t *out_value,
                           int64_t *out_index, void *scratch, cudaStream_t s) {
    unsigned G = max_grid(c, count);
    cudaError_t e = cudaMemsetAsync(scratch, 0, 64, s);
    if (e != cudaSuccess) return cuda_status(e);
    if (c->path == GRNS_PATH_REFERENCE)
        k_max<N><<<G, kMaxBlock, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, out_value, out_index,
                                         (unsigned *)scratch, (Cand *)((char *)scratch + 64));
    else
        k_max_fast<N><<<G, kMaxBlock, 0, s>>>(consts_of<N>(c), Operand<N>{x, ld}, count, out_value, out_index,
                                              (unsigned *)scratch, (FCand *)((char *)scratch + 64));
    return cuda_status(cudaGetLastError());
}

grns_status launch_max(grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, uint32_t *out_value,
                       int64_t *out_index, void *scratch, size_t scratch_bytes, cudaStream_t s) {
    if (count == 0) {
        if (out_index) return cuda_status(cudaMemsetAsync(out_index, 0xff, sizeof(int64_t), s));
        return GRNS_OK;
    }
    bool owned = false;
    if (!scratch) {  /* stream-ordered allocation: safe for concurrent calls on different streams */
        cudaError_t e = scratch_alloc(c, &scratch, max_scratch_bytes(c, count), s);
        if (e != cudaSuccess) return cuda_status(e);
        owned = true;
    }
    grns_status st;
#define C_(n) st = run_max<n>(c, x, ld, count, out_value, out_index, scratch, s); break
    GRNS_SWITCH_N(c->n, st = GRNS_ERR_UNSUPPORTED)
#undef C_
    if (owned) {
        cudaError_t e = scratch_free(scratch, s);
        if (st == GRNS_OK && e != cudaSuccess) st = cuda_status(e);
    }
    return st;
}

}  // namespace grns
