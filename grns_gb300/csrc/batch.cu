/*
 * grns_gb300 -- batched execution: many uneven-length arrays in ONE
 * persistent launch, captured in a CUDA graph.
 *
 * No counterpart in the reference (its callers launch one kernel per array,
 * e.g. tests/test_perf_rnscmp.cu:156).  Jobs (op, arrays, count) are split
 * into chunks; a persistent grid (SMs x resident blocks) pulls chunks with one
 * atomic per WARP, so uneven jobs and uneven per-element costs balance
 * dynamically and no block-wide barrier is ever needed.  Every op's interval
 * evaluation stays in registers (eval+cmp, div, scale2pow, max).  Jobs run
 * heaviest first (division, then scaling, ...) to shorten the tail.  Max jobs
 * leave one partial per chunk; the warp that completes a job's last chunk
 * reduces them and writes the value and index.
 *
 * Per-op schedule (a context setting, chosen by grns_autotune): "serial"
 * (one thread per number) or "coop" (n-threaded: the n residues of a number
 * spread over the lanes of a lane group, reduced by shuffles; cmp and max
 * only), and the chunk length.
 *
 * GRNS_SPLIT_BY_N: compiled as one unit per group of moduli counts.
 */
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "div_warp.cuh"
#include "scale_warp.cuh"
#include "internal.h"
#include "rns_device.cuh"
#include "rns_fast.cuh"
#include "rns_mpint.cuh"

namespace grns {

struct JobDev {
    int32_t op, layout;
    int64_t count;
    int64_t ld;  // SoA input leading dimension
    const uint32_t *a, *b;
    void *out0, *out1;
    uint8_t *flags;
    const Er *eval_a, *eval_b;  // cmp: optional cached evaluations (2 Er per number)
    uint2 *rec;                 // div: pass-A records (one per number; also reserved for scale jobs)
    int32_t *order;             // div, scale with per-number exponents: longest-first order
    uint32_t *rdig;             // mp_int div: remainder digits, N per number
    uint8_t *mflags;            // mp_int div: the division's flags per number
    uint32_t D_uniform;
    int32_t coop;
    int32_t vec;  // AoS operands 16-byte aligned, n a multiple of 4: a number's residues as 16-byte loads
    int64_t chunk_begin;   // first global chunk of this job
    int64_t partial_base;  // max jobs: first partial slot
    int32_t chunk_elems;
    int32_t nchunks;
};

struct Part {  // max: best of one chunk
    uint64_t a;
    int64_t idx;
};

/* block shape per moduli count: 256 threads x 2 blocks per SM, or 128 x 2 at
 * n = 64; division and scaling jobs keep their residues in shared-memory
 * columns (div_warp.cuh, scale_warp.cuh), allocated only when the batch holds
 * one: [DivK table][ScK table][warps' counters][columns of 3n words] */
template <int N>
struct BatchCfg {
    static constexpr int kBlock = N > 32 ? 128 : 256;
    static constexpr int kMinBlocks = 2;
    static constexpr size_t kTables = (sizeof(DivK) + sizeof(ScK)) * N;
    static constexpr size_t kHeavySmem = kTables + (size_t)(kBlock / 32) * kDivBins * 4 + (size_t)3 * N * 4 * kBlock;
};

__device__ __forceinline__ int find_job(const JobDev *jobs, int njobs, int64_t c) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (__ldg(&jobs[mid].chunk_begin) <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

template <int N>
__device__ __noinline__ int batch_tie(const Consts<N> &C, const Operand<N> x, int64_t ia, const Operand<N> y,
                                      int64_t ib) {
    return cmp_fx96_then_exact<N>(C, [&](int i) { return x.load(ia, i); }, [&](int i) { return y.load(ib, i); });
}

/* p better than q for the maximum (greater value, then smaller index) */
template <int N>
__device__ __forceinline__ bool part_better(const Consts<N> &C, const Operand<N> &x, const Part &p, const Part &q) {
    if (q.idx < 0) return p.idx >= 0;
    if (p.idx < 0) return false;
    int r = fx64_order(p.a, q.a, C.E);
    if (r == 2) r = batch_tie<N>(C, x, p.idx, x, q.idx);
    if (r != 0) return r > 0;
    return p.idx < q.idx;
}

template <int N>
__device__ __forceinline__ Part warp_best(const Consts<N> &C, const Operand<N> &x, Part best) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        Part o{__shfl_xor_sync(0xffffffffu, best.a, off), __shfl_xor_sync(0xffffffffu, best.idx, off)};
        if (part_better<N>(C, x, o, best)) best = o;
    }
    return best;
}

/* fx64 of number k, n-threaded: the lanes of a group of G = min(N, 32) lanes
 * share the residues; returns the full sum in every lane of the group */
template <int N>
__device__ __forceinline__ uint64_t fx64_coop(const Consts<N> &C, const Operand<N> &x, int64_t k, int gl,
                                              bool active, uint32_t &bad) {
    constexpr int G = N < 32 ? N : 32;
    uint64_t a = 0;
    uint32_t b = 0;
    if (active) {
GRNS_UNROLL_TO(N / G)
        for (int r = 0; r < N / G; r++) {
            const int i = gl + r * G;
            const uint32_t v = x.load_cs(k, i);
            b |= (uint32_t)(v >= C.m[i]);
            a += (uint64_t)v * C.c64l[i];
            a += (uint64_t)(uint32_t)(v * C.c64h[i]) << 32;
        }
    }
#pragma unroll
    for (int off = G / 2; off > 0; off >>= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, off);
        b |= __shfl_xor_sync(0xffffffffu, b, off);
    }
    bad |= b;
    return a;
}

/* a number's residues from an AoS array as 16-byte loads (N a multiple of 4,
 * the array 16-byte aligned) */
template <int N>
__device__ __forceinline__ void load_aos4(const uint32_t *base, int64_t k, uint32_t *v) {
    if constexpr (N % 4 == 0) {
        const uint4 *p = reinterpret_cast<const uint4 *>(base + k * N);
GRNS_UNROLL_TO(N / 4)
        for (int q = 0; q < N / 4; q++) {
            const uint4 w = __ldcs(p + q);
            v[4 * q] = w.x;
            v[4 * q + 1] = w.y;
            v[4 * q + 2] = w.z;
            v[4 * q + 3] = w.w;
        }
    }
}

/* the 64-bit fixed-point value of a number given as an array of residues */
template <int N>
__device__ __forceinline__ uint64_t fx64_arr(const Consts<N> &C, const uint32_t *v, uint32_t &bad) {
    uint64_t a = 0;
GRNS_UNROLL_N
    for (int i = 0; i < N; i++) {
        bad |= (uint32_t)(v[i] >= C.m[i]);
        a += (uint64_t)v[i] * C.c64l[i];
        a += (uint64_t)(uint32_t)(v[i] * C.c64h[i]) << 32;
    }
    return a;
}

template <int N>
__device__ __forceinline__ void run_chunk(const Consts<N> &C, const JobDev &J, int j, int64_t c, int lane,
                                          unsigned *done, Part *partials, uint32_t *smem) {
    const int64_t start = (c - J.chunk_begin) * (int64_t)J.chunk_elems;
    const int64_t end = min(start + (int64_t)J.chunk_elems, J.count);
    const int64_t ld = J.layout == GRNS_LAYOUT_SOA ? (J.count > 0 ? J.count : 1) : 0;   // outputs
    const int64_t ldi = J.layout == GRNS_LAYOUT_SOA ? J.ld : 0;                            // inputs
    const Operand<N> x{J.a, ldi}, y{J.b, ldi};
    switch (J.op) {
        case GRNS_OP_EVAL:
            for (int64_t k = start + lane; k < end; k += 32) {
                uint32_t f = 0;
                Er lo, up;
                if (J.vec) {
                    uint32_t v[N];
                    load_aos4<N>(J.a, k, v);
                    eval<N>(C, [&](int i) { return v[i]; }, lo, up, f);
                } else {
                    eval<N>(C, [&](int i) { return x.load_cs(k, i); }, lo, up, f);
                }
                ((Er *)J.out0)[2 * k] = lo;
                ((Er *)J.out0)[2 * k + 1] = up;
                if (J.flags) J.flags[k] = (uint8_t)f;
            }
            break;
        case GRNS_OP_CMP:
            if (J.coop) {
                constexpr int G = N < 32 ? N : 32;
                const int gl = lane % G, grp = lane / G;
                for (int64_t k0 = start; k0 < end; k0 += 32 / G) {
                    const int64_t k = k0 + grp;
                    const bool act = k < end;
                    uint32_t bad = 0;
                    const uint64_t a = fx64_coop<N>(C, x, k, gl, act, bad);
                    const uint64_t b = fx64_coop<N>(C, y, k, gl, act, bad);
                    if (act && gl == 0) {
                        int r = fx64_order(a, b, C.E);
                        if (r == 2 && !bad) r = batch_tie<N>(C, x, k, y, k);
                        ((int32_t *)J.out0)[k] = bad ? 0 : r;
                        if (J.flags) J.flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
                    }
                }
            } else {
                for (int64_t k = start + lane; k < end; k += 32) {
                    if (J.eval_a && J.eval_b) {  /* cached evaluations decide almost every pair */
                        const Er xl = J.eval_a[2 * k], xu = J.eval_a[2 * k + 1];
                        const Er yl = J.eval_b[2 * k], yu = J.eval_b[2 * k + 1];
                        const int r = cmp_intervals<N>(xl, xu, yl, yu);
                        if (r != 2) {
                            ((int32_t *)J.out0)[k] = r;
                            if (J.flags) J.flags[k] = 0;
                            continue;
                        }
                    }
                    uint64_t a = 0, b = 0;
                    uint32_t bad = 0;
                    if (J.vec) {
                        uint32_t v[N];
                        load_aos4<N>(J.a, k, v);
                        a = fx64_arr<N>(C, v, bad);
                        load_aos4<N>(J.b, k, v);
                        b = fx64_arr<N>(C, v, bad);
                    } else {
GRNS_UNROLL_N
                        for (int i = 0; i < N; i++) {
                            const uint32_t xi = x.load_cs(k, i), yi = y.load_cs(k, i);
                            bad |= (uint32_t)(xi >= C.m[i]) | (uint32_t)(yi >= C.m[i]);
                            a += (uint64_t)xi * C.c64l[i];
                            a += (uint64_t)(uint32_t)(xi * C.c64h[i]) << 32;
                            b += (uint64_t)yi * C.c64l[i];
                            b += (uint64_t)(uint32_t)(yi * C.c64h[i]) << 32;
                        }
                    }
                    int r = fx64_order(a, b, C.E);
                    if (r == 2 && !bad) r = batch_tie<N>(C, x, k, y, k);
                    ((int32_t *)J.out0)[k] = bad ? 0 : r;
                    if (J.flags) J.flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
                }
            }
            break;
        case GRNS_OP_DIV:
        {
            uint32_t *hist = smem + BatchCfg<N>::kTables / 4;
            uint32_t *cols = hist + (blockDim.x / 32) * kDivBins;
            div_range<N>(reinterpret_cast<const DivK *>(smem), C, x, y, J.rec, J.order,
                         Output<N>{(uint32_t *)J.out0, ld}, Output<N>{(uint32_t *)J.out1, ld}, J.flags, start, end,
                         cols + threadIdx.x, blockDim.x, hist + (threadIdx.x / 32) * kDivBins);
        }
            break;
        case GRNS_OP_MPINT_DIV: {  // mpint_div (src/mpint.cuh:511): the division of the digit fields in place,
                                   // then the Euclidean step, evaluation and sign of each number of the chunk
            uint32_t *hist = smem + BatchCfg<N>::kTables / 4;
            uint32_t *cols = hist + (blockDim.x / 32) * kDivBins;
            const MpInt<N> *px = (const MpInt<N> *)J.a, *py = (const MpInt<N> *)J.b;
            MpInt<N> *po = (MpInt<N> *)J.out0;
            div_range<N>(reinterpret_cast<const DivK *>(smem), C, MpDigitsIn<N>{J.a}, MpDigitsIn<N>{J.b}, J.rec,
                         J.order, MpDigitsOut<N>{(uint32_t *)J.out0}, Output<N>{J.rdig, 0}, J.mflags, start, end,
                         cols + threadIdx.x, blockDim.x, hist + (threadIdx.x / 32) * kDivBins);
            __syncwarp();  // the chunk's quotients and remainders, written by every lane
            for (int64_t k = start + lane; k < end; k += 32) {
                uint32_t f = J.mflags[k];
                const uint32_t *qd = po[k].digits, *rd = J.rdig + k * N;
                MpInt<N> res;
                mpint_div_finish<N>(C, __ldg(&px[k].sign), __ldg(&py[k].sign), [&](int i) { return qd[i]; },
                                    [&](int i) { return rd[i]; }, f, res);
                po[k] = res;
                if (J.flags) J.flags[k] = (uint8_t)f;
            }
            break;
        }
        case GRNS_OP_SCALE2POW: {
            uint32_t *hist = smem + BatchCfg<N>::kTables / 4;
            uint32_t *cols = hist + (blockDim.x / 32) * kDivBins;
            scale_range<N>(reinterpret_cast<const ScK *>(smem + sizeof(DivK) / 4 * N), C, x, J.b, J.D_uniform,
                           Output<N>{(uint32_t *)J.out0, ld}, J.flags, J.b ? J.order : nullptr, start, end,
                           cols + threadIdx.x, blockDim.x, hist + (threadIdx.x / 32) * kDivBins);
            break;
        }
        case GRNS_OP_MAX: {
            Part best{0, -1};
            if (J.coop) {
                constexpr int G = N < 32 ? N : 32;
                const int gl = lane % G, grp = lane / G;
                for (int64_t k0 = start; k0 < end; k0 += 32 / G) {
                    const int64_t k = k0 + grp;
                    const bool act = k < end;
                    uint32_t bad = 0;
                    const uint64_t a = fx64_coop<N>(C, x, k, gl, act, bad);
                    if (act) {
                        Part p{a, k};
                        if (part_better<N>(C, x, p, best)) best = p;
                    }
                }
            } else {
                for (int64_t k = start + lane; k < end; k += 32) {
                    uint64_t a;
                    if (J.vec) {
                        uint32_t v[N], bad = 0;
                        load_aos4<N>(J.a, k, v);
                        a = fx64_arr<N>(C, v, bad);
                    } else {
                        a = fx64<N>(C, [&](int i) { return x.load_cs(k, i); });
                    }
                    Part p{a, k};
                    if (part_better<N>(C, x, p, best)) best = p;
                }
            }
            best = warp_best<N>(C, x, best);
            const int64_t slot = J.partial_base + (c - J.chunk_begin);
            bool last = false;
            if (lane == 0) {
                partials[slot] = best;
                __threadfence();
                last = atomicAdd(&done[j], 1u) == (unsigned)J.nchunks - 1;
            }
            last = __shfl_sync(0xffffffffu, (int)last, 0);
            if (last) {
                __threadfence();
                Part b2{0, -1};
                for (int s = lane; s < J.nchunks; s += 32) {
                    const Part *pp = partials + J.partial_base + s;
                    Part p{(uint64_t)__ldcg((const unsigned long long *)&pp->a), __ldcg((const long long *)&pp->idx)};
                    if (part_better<N>(C, x, p, b2)) b2 = p;
                }
                b2 = warp_best<N>(C, x, b2);
                if (lane == 0 && J.out1) *(int64_t *)J.out1 = b2.idx;
                for (int i = lane; i < N; i += 32) ((uint32_t *)J.out0)[i] = b2.idx >= 0 ? x.load(b2.idx, i) : 0u;
            }
            break;
        }
        default: {  // mp_int add / sub / mul
            const MpInt<N> *px = (const MpInt<N> *)J.a, *py = (const MpInt<N> *)J.b;
            MpInt<N> *po = (MpInt<N> *)J.out0;
            for (int64_t k = start + lane; k < end; k += 32) {
                MpInt<N> a = px[k], b = py[k], r;
                clear_pad(r);
                uint32_t f = 0;
                if (J.op == GRNS_OP_MPINT_MUL) mpint_mul<N>(C, r, a, b, f);
                else mpint_addsub<N>(C, r, a, b, J.op == GRNS_OP_MPINT_SUB, f);
                po[k] = r;
                if (J.flags) J.flags[k] = (uint8_t)f;
            }
        }
    }
}

template <int N>
__global__ void __launch_bounds__(BatchCfg<N>::kBlock, BatchCfg<N>::kMinBlocks) k_batch(const __grid_constant__ CArg<N> CA,
                                                          const JobDev *__restrict__ jobs, int njobs,
                                                          int64_t total_chunks, unsigned long long *counter,
                                                          unsigned *done, Part *partials, int has_div) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 batch_smem4[];
    uint32_t *batch_smem = reinterpret_cast<uint32_t *>(batch_smem4);
    if (has_div) {  // division and scaling constants for every block
        divk_fill<N>(C, reinterpret_cast<DivK *>(batch_smem));
        sck_fill<N>(C, reinterpret_cast<ScK *>(batch_smem + sizeof(DivK) / 4 * N));
        __syncthreads();
    }
    const int lane = threadIdx.x & 31;
    for (;;) {
        unsigned long long c = 0;
        if (lane == 0) c = atomicAdd(counter, 1ull);
        c = __shfl_sync(0xffffffffu, c, 0);
        if ((int64_t)c >= total_chunks) break;
        const int j = find_job(jobs, njobs, (int64_t)c);
        const JobDev J = jobs[j];
        run_chunk<N>(C, J, j, (int64_t)c, lane, done, partials, batch_smem);
    }
}

}  // namespace grns

using namespace grns;

struct grns_batch {
    grns_ctx *ctx = nullptr;
    int njobs = 0;
    int64_t total_chunks = 0;
    int64_t nparts = 0;
    int64_t nrec = 0;                // division records
    int64_t nmp = 0;                 // numbers of mp_int division jobs (remainder digits and flags)
    uint2 *d_rec = nullptr;
    std::vector<JobDev> host_jobs;   // execution order
    std::vector<int> order;          // host_jobs[t] = user job order[t]
    JobDev *d_jobs = nullptr;
    unsigned long long *d_counter = nullptr;  // followed by the per-job done counters
    unsigned *d_done = nullptr;
    Part *d_parts = nullptr;
    size_t counters_bytes = 0;
    int grid = 0;
    size_t smem = 0;  // dynamic shared memory of the launch (division jobs present)
    std::vector<int64_t *> empty_max_index;  // count-0 max jobs: index written as -1
    bool use_graph = false;
    cudaGraphExec_t exec = nullptr;
    cudaStream_t graph_stream = nullptr;
};

namespace grns {

/* the kernel is built for up to kBatchMaxModuli moduli (batches of larger
 * sets are refused at creation) */
template <int N>
grns_status launch_batch_kernel(grns_batch *b, cudaStream_t s) {
    if constexpr (N > kBatchMaxModuli) {
        (void)b;
        (void)s;
        return GRNS_ERR_UNSUPPORTED;
    } else {
        k_batch<N><<<b->grid, BatchCfg<N>::kBlock, b->smem, s>>>(consts_of<N>(b->ctx), b->d_jobs, b->njobs,
                                                                 b->total_chunks, b->d_counter, b->d_done, b->d_parts,
                                                                 b->smem ? 1 : 0);
        return cuda_status(cudaGetLastError());
    }
}

template <int N>
int occupancy_blocks(size_t smem) {
    if constexpr (N > kBatchMaxModuli) {
        (void)smem;
        return 1;
    } else {
        if (BatchCfg<N>::kHeavySmem > 48 * 1024)  // per device: set on every shape computation
            cudaFuncSetAttribute(k_batch<N>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)BatchCfg<N>::kHeavySmem);
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_batch<N>, BatchCfg<N>::kBlock, smem);
        return nb > 0 ? nb : 1;
    }
}

/* the per-count entry points: extern here, instantiated for this unit's counts */
#define GRNS_BATCH_ROOTS_(n, EXT)                                                   \
    EXT template grns_status launch_batch_kernel<n>(grns_batch *, cudaStream_t);    \
    EXT template int occupancy_blocks<n>(size_t);
#define GRNS_EXTERN_(n) GRNS_BATCH_ROOTS_(n, extern)
#define GRNS_DEFINE_(n) GRNS_BATCH_ROOTS_(n, )
GRNS_FOR_EACH_N(GRNS_EXTERN_)
GRNS_PART_N(GRNS_DEFINE_)
#undef GRNS_EXTERN_
#undef GRNS_DEFINE_

}  // namespace grns

#if GRNS_PART_MAIN
namespace {

double op_cost(int op, int n) {
    switch (op) {
        case GRNS_OP_DIV:
        case GRNS_OP_MPINT_DIV: return 400.0 * n;
        case GRNS_OP_SCALE2POW: return 60.0 * n;
        case GRNS_OP_EVAL: return 8.0 * n;
        case GRNS_OP_MPINT_ADD:
        case GRNS_OP_MPINT_SUB:
        case GRNS_OP_MPINT_MUL: return 4.0 * n;
        default: return 1.0 * n;
    }
}

/* bytes of the division scratch: records and orders, mp_int remainder digits and flags */
size_t batch_rec_bytes(const grns_batch *b) {
    return kDivScratchPerNumber * (size_t)b->nrec + (4 * (size_t)b->ctx->n + 1) * (size_t)b->nmp;
}

bool job_ok(const grns_ctx *c, const grns_job &jb) {
    if (jb.op < GRNS_OP_EVAL || jb.op > GRNS_OP_MPINT_DIV || jb.count < 0) return false;
    if (jb.ld != 0 && jb.ld < jb.count) return false;
    if (jb.layout != GRNS_LAYOUT_SOA && jb.layout != GRNS_LAYOUT_AOS) return false;
    if (jb.count == 0) return jb.op != GRNS_OP_MAX || jb.out0;
    if (!jb.a || !jb.out0) return false;
    switch (jb.op) {
        case GRNS_OP_CMP:
        case GRNS_OP_MPINT_ADD:
        case GRNS_OP_MPINT_SUB:
        case GRNS_OP_MPINT_MUL: return jb.b != nullptr;
        case GRNS_OP_MPINT_DIV: {  // the quotient digits are written while the operands are still read
            const size_t bytes = (size_t)GRNS_MPINT_BYTES(c->n) * (size_t)jb.count;
            auto overlap = [&](const void *p) {
                return (const char *)p < (const char *)jb.out0 + bytes && (const char *)jb.out0 < (const char *)p + bytes;
            };
            return jb.b != nullptr && !overlap(jb.a) && !overlap(jb.b);
        }
        case GRNS_OP_DIV: return jb.b && jb.out1;
        default: return true;
    }
}

grns_status enqueue(grns_batch *b, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(b->d_counter, 0, b->counters_bytes, s);
    if (e != cudaSuccess) return cuda_status(e);
    for (int64_t *p : b->empty_max_index) {
        e = cudaMemsetAsync(p, 0xff, sizeof(int64_t), s);
        if (e != cudaSuccess) return cuda_status(e);
    }
    if (b->total_chunks == 0) return GRNS_OK;
#define C_(n) return launch_batch_kernel<n>(b, s)
    GRNS_DISPATCH_N(b->ctx->n, C_)
#undef C_
}

/* launch shape of a batch: grid (SMs x resident blocks) and shared memory */
void batch_shape(grns_batch *b) {
    bool has_div = false;
    for (const JobDev &J : b->host_jobs)
        has_div |= (J.op == GRNS_OP_DIV || J.op == GRNS_OP_MPINT_DIV || J.op == GRNS_OP_SCALE2POW) && J.count > 0;
    int per_sm = 1;
#define C_(n)                                                  \
    b->smem = has_div ? BatchCfg<n>::kHeavySmem : 0;           \
    per_sm = occupancy_blocks<n>(b->smem);                     \
    break
    GRNS_SWITCH_N(b->ctx->n, break)
#undef C_
    b->grid = b->ctx->sm_count * per_sm;
}

/* fill the device-side descriptors from user jobs (fixed order) */
grns_status fill_jobs(grns_batch *b, const grns_job *jobs) {
    const grns_ctx *c = b->ctx;
    int64_t chunk = 0, parts = 0, recs = 0, mps = 0;
    for (int t = 0; t < b->njobs; t++) {
        const grns_job &u = jobs[b->order[t]];
        JobDev &J = b->host_jobs[t];
        J.op = u.op;
        J.layout = u.layout;
        J.count = u.count;
        J.ld = u.ld > 0 ? u.ld : (u.count > 0 ? u.count : 1);
        J.eval_a = (const Er *)u.eval_a;
        J.eval_b = (const Er *)u.eval_b;
        J.a = (const uint32_t *)u.a;
        J.b = (const uint32_t *)u.b;
        J.out0 = u.out0;
        J.out1 = u.out1;
        J.flags = u.flags;
        J.D_uniform = u.D_uniform;
        J.rec = nullptr;
        J.order = nullptr;
        J.rdig = nullptr;
        J.mflags = nullptr;
        if (u.op == GRNS_OP_DIV || u.op == GRNS_OP_MPINT_DIV || (u.op == GRNS_OP_SCALE2POW && u.b)) {
            J.rec = b->d_rec ? b->d_rec + recs : nullptr;
            recs += u.count;
        }
        if (u.op == GRNS_OP_MPINT_DIV) {  // placed below, after the records and orders
            J.rdig = (uint32_t *)(uintptr_t)mps;
            mps += u.count;
        }
        const int op = u.op;
        const Sched &sc = c->sched[op];
        J.coop = (op == GRNS_OP_CMP || op == GRNS_OP_MAX) ? sc.coop : 0;
        J.vec = u.layout == GRNS_LAYOUT_AOS && c->n % 4 == 0 && ((uintptr_t)u.a & 15) == 0 &&
                ((uintptr_t)u.b & 15) == 0;
        J.chunk_elems = sc.chunk > 0 ? sc.chunk : 256;
        J.nchunks = (int32_t)((u.count + J.chunk_elems - 1) / J.chunk_elems);
        if (op == GRNS_OP_MAX && u.count == 0) J.nchunks = 0;
        J.chunk_begin = chunk;
        J.partial_base = parts;
        chunk += J.nchunks;
        if (op == GRNS_OP_MAX) parts += J.nchunks;
    }
    b->total_chunks = chunk;
    b->nparts = parts;
    b->nrec = recs;
    b->nmp = mps;
    /* one allocation: the records, the orders, then the mp_int divisions'
     * remainder digits and flags */
    for (int t = 0; t < b->njobs; t++) {
        JobDev &J = b->host_jobs[t];
        const int64_t mp_first = (int64_t)(uintptr_t)J.rdig;
        J.rdig = nullptr;
        if (!b->d_rec) continue;
        int32_t *ord = (int32_t *)(b->d_rec + recs);
        uint32_t *rd = (uint32_t *)(ord + recs);
        uint8_t *mf = (uint8_t *)(rd + (size_t)c->n * mps);
        if (J.rec) J.order = ord + (J.rec - b->d_rec);
        if (J.op == GRNS_OP_MPINT_DIV) {
            J.rdig = rd + (size_t)c->n * mp_first;
            J.mflags = mf + mp_first;
        }
    }
    b->empty_max_index.clear();
    for (int t = 0; t < b->njobs; t++) {
        const grns_job &u = jobs[b->order[t]];
        if (u.op == GRNS_OP_MAX && u.count == 0 && u.out1) b->empty_max_index.push_back((int64_t *)u.out1);
    }
    return GRNS_OK;
}

}  // namespace

namespace grns {

/* One-shot batch for the server: everything stream-ordered on `s`.  The
 * device job table is staged through `staging` (pinned, at least
 * batch_staging_bytes(njobs) bytes, not reused until the launch completes),
 * allocated from the context's stream-ordered pool and freed after the
 * kernel, so nothing here synchronises with other streams. */
size_t batch_staging_bytes(int njobs) { return sizeof(JobDev) * (size_t)(njobs > 0 ? njobs : 1); }

grns_status batch_run_async(grns_ctx *c, const grns_job *jobs, int njobs, void *staging, cudaStream_t s) {
    if (c->n > kBatchMaxModuli) return GRNS_ERR_UNSUPPORTED;
    NvtxRange range("grns batch_run");
    grns_batch b;
    b.ctx = c;
    b.njobs = njobs;
    b.order.resize(njobs);
    for (int t = 0; t < njobs; t++) b.order[t] = t;
    std::stable_sort(b.order.begin(), b.order.end(), [&](int p, int q) {
        return op_cost(jobs[p].op, c->n) * (double)jobs[p].count > op_cost(jobs[q].op, c->n) * (double)jobs[q].count;
    });
    b.host_jobs.resize(njobs);
    fill_jobs(&b, jobs);
    b.counters_bytes = sizeof(unsigned long long) + sizeof(unsigned) * (size_t)(njobs > 0 ? njobs : 1);
    cudaError_t e = cudaSuccess;
    if (b.nrec) {
        e = scratch_alloc(c, (void **)&b.d_rec, batch_rec_bytes(&b), s);
        if (e != cudaSuccess) return cuda_status(e);
        fill_jobs(&b, jobs);
    }
    std::memcpy(staging, b.host_jobs.data(), sizeof(JobDev) * njobs);
    e = scratch_alloc(c, (void **)&b.d_counter, b.counters_bytes, s);
    if (e == cudaSuccess) e = scratch_alloc(c, (void **)&b.d_jobs, sizeof(JobDev) * (njobs > 0 ? njobs : 1), s);
    if (e == cudaSuccess && b.nparts) e = scratch_alloc(c, (void **)&b.d_parts, sizeof(Part) * b.nparts, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.d_jobs, staging, sizeof(JobDev) * njobs, cudaMemcpyHostToDevice, s);
    grns_status st = cuda_status(e);
    if (st == GRNS_OK) {
        b.d_done = (unsigned *)(b.d_counter + 1);
        batch_shape(&b);
        st = enqueue(&b, s);
    }
    if (b.d_jobs) cudaFreeAsync(b.d_jobs, s);
    if (b.d_counter) cudaFreeAsync(b.d_counter, s);
    if (b.d_parts) cudaFreeAsync(b.d_parts, s);
    if (b.d_rec) cudaFreeAsync(b.d_rec, s);
    b.d_rec = nullptr;
    b.d_jobs = nullptr;
    b.d_counter = nullptr;
    b.d_parts = nullptr;
    return st;
}

}  // namespace grns

extern "C" {

grns_status grns_ctx_get_schedule(const grns_ctx *c, int op, grns_schedule *out) {
    if (!c || !out || op < GRNS_OP_EVAL || op > GRNS_OP_MPINT_MUL) return GRNS_ERR_INVALID_ARGUMENT;
    out->coop = c->sched[op].coop;
    out->chunk = c->sched[op].chunk;
    return GRNS_OK;
}

grns_status grns_ctx_set_schedule(grns_ctx *c, int op, const grns_schedule *s) {
    if (!c || !s || op < GRNS_OP_EVAL || op > GRNS_OP_MPINT_MUL) return GRNS_ERR_INVALID_ARGUMENT;
    if (s->chunk < 32 || s->chunk > (1 << 20) || (s->coop && op != GRNS_OP_CMP && op != GRNS_OP_MAX))
        return GRNS_ERR_INVALID_ARGUMENT;
    c->sched[op] = Sched{s->coop ? 1 : 0, s->chunk};
    return GRNS_OK;
}

grns_status grns_batch_create(grns_ctx *c, const grns_job *jobs, int njobs, int use_graph, grns_batch **out) {
    if (!c || !out || njobs < 0 || (njobs > 0 && !jobs)) return GRNS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (c->n > grns::kBatchMaxModuli) return GRNS_ERR_UNSUPPORTED;
    for (int t = 0; t < njobs; t++)
        if (!job_ok(c, jobs[t])) return GRNS_ERR_INVALID_ARGUMENT;
    grns_batch *b = new (std::nothrow) grns_batch();
    if (!b) return GRNS_ERR_OUT_OF_MEMORY;
    b->ctx = c;
    b->njobs = njobs;
    b->use_graph = use_graph != 0;
    b->order.resize(njobs);
    for (int t = 0; t < njobs; t++) b->order[t] = t;
    std::stable_sort(b->order.begin(), b->order.end(), [&](int p, int q) {
        return op_cost(jobs[p].op, c->n) * (double)jobs[p].count > op_cost(jobs[q].op, c->n) * (double)jobs[q].count;
    });
    b->host_jobs.resize(njobs);
    fill_jobs(b, jobs);
    b->counters_bytes = sizeof(unsigned long long) + sizeof(unsigned) * (size_t)(njobs > 0 ? njobs : 1);
    cudaError_t e = cudaMalloc(&b->d_counter, b->counters_bytes);
    if (e == cudaSuccess && njobs) e = cudaMalloc(&b->d_jobs, sizeof(JobDev) * njobs);
    if (e == cudaSuccess && b->nparts) e = cudaMalloc(&b->d_parts, sizeof(Part) * b->nparts);
    if (e == cudaSuccess && b->nrec) {
        e = cudaMalloc(&b->d_rec, batch_rec_bytes(b));
        if (e == cudaSuccess) fill_jobs(b, jobs);
    }
    if (e == cudaSuccess && njobs)
        e = cudaMemcpy(b->d_jobs, b->host_jobs.data(), sizeof(JobDev) * njobs, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        grns_batch_destroy(b);
        return cuda_status(e);
    }
    b->d_done = (unsigned *)(b->d_counter + 1);
    batch_shape(b);
    *out = b;
    return GRNS_OK;
}

grns_status grns_batch_update(grns_batch *b, const grns_job *jobs, int njobs) {
    if (!b || njobs != b->njobs || (njobs > 0 && !jobs)) return GRNS_ERR_INVALID_ARGUMENT;
    for (int t = 0; t < njobs; t++) {
        const grns_job &u = jobs[b->order[t]];
        const JobDev &J = b->host_jobs[t];
        if (!job_ok(b->ctx, u) || u.op != J.op || u.count != J.count || u.layout != J.layout)
            return GRNS_ERR_INVALID_ARGUMENT;
    }
    fill_jobs(b, jobs);
    cudaError_t e = njobs ? cudaMemcpy(b->d_jobs, b->host_jobs.data(), sizeof(JobDev) * njobs, cudaMemcpyHostToDevice)
                          : cudaSuccess;
    return cuda_status(e);
}

grns_status grns_batch_launch(grns_batch *b, void *stream) {
    grns::NvtxRange range("grns_batch_launch");
    if (!b) return GRNS_ERR_INVALID_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (!b->use_graph || s == nullptr) return enqueue(b, s);
    if (!b->exec) {
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_status(e);
        grns_status st = enqueue(b, s);
        e = cudaStreamEndCapture(s, &g);
        if (st != GRNS_OK) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return cuda_status(e);
        e = cudaGraphInstantiate(&b->exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_status(e);
    }
    return cuda_status(cudaGraphLaunch(b->exec, s));
}

grns_status grns_batch_destroy(grns_batch *b) {
    if (!b) return GRNS_ERR_INVALID_ARGUMENT;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->d_jobs) cudaFree(b->d_jobs);
    if (b->d_counter) cudaFree(b->d_counter);
    if (b->d_parts) cudaFree(b->d_parts);
    if (b->d_rec) cudaFree(b->d_rec);
    delete b;
    return GRNS_OK;
}

int64_t grns_batch_chunks(const grns_batch *b) { return b ? b->total_chunks : -1; }
int grns_batch_grid(const grns_batch *b) { return b ? b->grid : -1; }

}  // extern "C"
#endif  // GRNS_PART_MAIN
