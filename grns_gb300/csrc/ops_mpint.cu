/*
 * grns_gb300 -- multiple-precision integer kernels over arrays of mp_int_t
 * (reference layout, src/types.cuh:45): add / sub / mul with the interval
 * evaluation derived from the operands' evaluations, as cuda::mpint_add /
 * mpint_sub / mpint_mul (reference src/mpint.cuh:336/:407/:478).  Overflow
 * goes to the per-element flags (the reference prints from the device).
 *
 * mpint_div (src/mpint.cuh:511) runs in three launches: the digit columns of
 * both operands are gathered into residue-major scratch, the division driver
 * of grns_div computes |x| div |y| and the remainder, and a finishing kernel
 * applies the Euclidean step (a negative dividend with a nonzero remainder
 * takes one more), evaluates the quotient and sets the sign.
 */
#include "internal.h"
#include "rns_mpint.cuh"

namespace grns {

template <int N>
__global__ void __launch_bounds__(256) k_mpint(const __grid_constant__ CArg<N> CA, int op,
                                               const MpInt<N> *__restrict__ x, const MpInt<N> *__restrict__ y,
                                               int64_t count, MpInt<N> *__restrict__ out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        MpInt<N> a = x[k], b = y[k], r;
        clear_pad(r);
        uint32_t f = 0;
        if (op == 2) mpint_mul<N>(C, r, a, b, f);
        else mpint_addsub<N>(C, r, a, b, op == 1, f);
        out[k] = r;
        if (flags) flags[k] = (uint8_t)f;
    }
}

constexpr int kMpRecs = 8;   // records per warp chunk of k_mpint_bulk (8 records: a multiple of 16 bytes)
constexpr int kMpParts = 4;  // lanes per record

/* copy `bytes` (a multiple of 8) between global and shared memory with the
 * lanes of one warp: 16-byte words, 8-byte words for the tail (both sides
 * start 16-byte aligned) */
__device__ __forceinline__ void warp_copy(void *dst, const void *src, int bytes, int lane) {
    const int n16 = bytes >> 4;
    const uint4 *s4 = reinterpret_cast<const uint4 *>(src);
    uint4 *d4 = reinterpret_cast<uint4 *>(dst);
    for (int t = lane; t < n16; t += 32) d4[t] = s4[t];
    if ((bytes & 15) && lane == 0) reinterpret_cast<uint2 *>(dst)[2 * n16] = reinterpret_cast<const uint2 *>(src)[2 * n16];
}

/* ---- bulk-copy form: the same chunks moved by the copy engine, double-buffered per warp ----
 * cp.async.bulk (1-D, this GPU's own memory, no multicast): both addresses
 * 16-byte aligned and the size a multiple of 16 bytes -- a chunk of kMpRecs
 * records always is; a partial last chunk is copied by the lanes. */

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}
/* waits for phase `parity` of the barrier; false when it has not completed
 * after about 2^20 polls with back-off (the caller then stops) */
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_addr(bar);
    for (int it = 0; it < (1 << 20); it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (it > 64) __nanosleep(128);
    }
    return false;
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}
__device__ __forceinline__ void bulk_store(void *dst, const void *src, uint32_t bytes) {
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_addr(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

/* one chunk's arithmetic in place (the result replaces x's records): lanes
 * t * kMpParts .. + kMpParts - 1 take record t (every kMpParts-th residue);
 * lane p = 0 writes the sign, evaluation and flags */
template <int N>
__device__ __forceinline__ void mp_chunk(const Consts<N> &C, const uint4 *K, int op, MpInt<N> *sx, const MpInt<N> *sy,
                                         int nt, int64_t k0, uint8_t *flags, int lane) {
    const int t = lane / kMpParts, p = lane % kMpParts;
    const bool act = t < nt;
    MpInt<N> &a = sx[t];
    const MpInt<N> &b = sy[t];
    uint32_t f = 0;
    bool zero = true, minus = false;
    Er lo{0, 0}, up{0, 0};
    if (act && p == 0) {  // the record's interval, once
        if (op == 2) {
            lo = er_md_i<false>(a.eval[0], b.eval[0], C.unit_upp, C.unit_rcp_upp);
            up = er_md_i<true>(a.eval[1], b.eval[1], C.unit_low, C.unit_rcp_low);
        } else {
            minus = mpint_addsub_eval(head_of(a), head_of(b), op == 1, lo, up);
        }
    }
    minus = __shfl_sync(0xffffffffu, (int)minus, lane & ~(kMpParts - 1)) != 0;
    if (act) {
        if (op == 2) {
#pragma unroll 4
            for (int i = p; i < N; i += kMpParts) {
                const uint4 k = K[i];  // m, mu, b
                const uint32_t u = a.digits[i], v = b.digits[i];
                f |= (u >= k.x || v >= k.x) ? kFlagInvalidInput : 0u;
                const uint32_t w = mulmod_barrett(u, v, k.x, k.y, k.z);
                a.digits[i] = w;
                zero &= w == 0;
            }
        } else {
            const int s1 = a.sign, s2 = op == 1 ? (b.sign ^ 1) : b.sign;
#pragma unroll 4
            for (int i = p; i < N; i += kMpParts)
                a.digits[i] = mpint_addsub_digit(a.digits[i], b.digits[i], K[i].x, s1, s2, minus, f);
        }
    }
#pragma unroll
    for (int o = 1; o < kMpParts; o <<= 1) {  // the lanes of a record are adjacent
        f |= __shfl_xor_sync(0xffffffffu, f, o);
        zero &= __shfl_xor_sync(0xffffffffu, (int)zero, o) != 0;
    }
    const int sign = op == 2 ? (zero ? 0 : (a.sign ^ b.sign)) : (int)minus;
    __syncwarp();  // every lane of the record has read its sign and evaluation
    if (act && p == 0) {
        a.sign = sign;
        clear_pad(a);
        a.eval[0] = lo;
        a.eval[1] = up;
        f |= overflow_flags_i<N>(C, lo, up);
        if (flags) flags[k0 + t] = (uint8_t)f;
    }
    __syncwarp();
}

/* add / sub / mul with the chunks moved by bulk copies: per warp two stages
 * (x and y chunks each) and an mbarrier per stage; lane 0 loads chunk i + 1
 * while the warp computes chunk i in place and bulk-stores it.  A stage is
 * reloaded only after the store that read it has finished reading. */
template <int N>
__global__ void __launch_bounds__(256) k_mpint_bulk(const __grid_constant__ CArg<N> CA, int op,
                                                    const MpInt<N> *__restrict__ x, const MpInt<N> *__restrict__ y,
                                                    int64_t count, MpInt<N> *__restrict__ out,
                                                    uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint4 mp_smem[];
    __shared__ uint4 K[N];  // per modulus: m, mu, b (the lanes of a warp read different moduli at once)
    constexpr int RB = (int)sizeof(MpInt<N>);
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    for (int i = threadIdx.x; i < N; i += blockDim.x) K[i] = make_uint4(C.m[i], C.mu[i], C.b[i], 0u);
    __syncthreads();
    uint64_t *bars = reinterpret_cast<uint64_t *>(mp_smem) + wib * 2;  // [8 warps][2 stages]
    MpInt<N> *buf = reinterpret_cast<MpInt<N> *>(reinterpret_cast<char *>(mp_smem) + 16 * 8) + wib * 4 * kMpRecs;
    const int64_t W = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (lane == 0) {
        mbar_init(&bars[0]);
        mbar_init(&bars[1]);
        fence_async_smem();
    }
    __syncwarp();
    /* chunk c's records [c kMpRecs, ...) into stage s; returns whether the
     * copy engine moves it (else the lanes have copied it already) */
    auto load = [&](int64_t c, int st) -> bool {
        const int64_t k0 = c * kMpRecs;
        const int nt = count - k0 < kMpRecs ? (int)(count - k0) : kMpRecs;
        MpInt<N> *sx = buf + st * 2 * kMpRecs, *sy = sx + kMpRecs;
        if (nt == kMpRecs) {  // a full chunk: kMpRecs * RB bytes, a multiple of 16
            if (lane == 0) {
                fence_async_smem();
                mbar_expect_tx(&bars[st], 2u * kMpRecs * RB);
                bulk_load(sx, x + k0, kMpRecs * RB, &bars[st]);
                bulk_load(sy, y + k0, kMpRecs * RB, &bars[st]);
            }
            return true;
        }
        warp_copy(sx, x + k0, nt * RB, lane);
        warp_copy(sy, y + k0, nt * RB, lane);
        __syncwarp();
        return false;
    };
    bool bulk[2] = {false, false};
    uint32_t uses[2] = {0, 0};  // completed phases per stage
    if (w * kMpRecs < count) bulk[0] = load(w, 0);
    bool failed = false;
    for (int64_t i = 0;; i++) {
        const int64_t c = w + i * W;
        if (c * kMpRecs >= count) break;
        const int st = (int)(i & 1);
        const int64_t cn = c + W;
        if (cn * kMpRecs < count) {  // the next chunk into the other stage, once its last store has read it
            if (lane == 0) bulk_wait_read();
            __syncwarp();
            bulk[st ^ 1] = load(cn, st ^ 1);
        }
        if (bulk[st]) {
            if (!mbar_wait(&bars[st], uses[st] & 1)) {
                failed = true;
                break;
            }
            uses[st]++;
        }
        const int64_t k0 = c * kMpRecs;
        const int nt = count - k0 < kMpRecs ? (int)(count - k0) : kMpRecs;
        MpInt<N> *sx = buf + st * 2 * kMpRecs;
        mp_chunk<N>(C, K, op, sx, sx + kMpRecs, nt, k0, flags, lane);
        if (nt == kMpRecs) {
            fence_async_smem();  // the lanes' writes, before the copy engine reads them
            __syncwarp();
            if (lane == 0) bulk_store(out + k0, sx, kMpRecs * RB);
        } else {
            warp_copy(out + k0, sx, nt * RB, lane);
        }
        __syncwarp();
    }
    if (failed) {  // a copy that never arrived: flag this warp's remaining numbers and stop
        for (int64_t c = w; c * kMpRecs < count; c += W)
            for (int t = lane; t < kMpRecs && c * kMpRecs + t < count; t += 32)
                if (flags) flags[c * kMpRecs + t] |= (uint8_t)kFlagIterCap;
        for (int st = 0; st < 2; st++)  // let loads in flight land (bounded) before the block's memory goes
            if (bulk[st]) mbar_wait(&bars[st], uses[st] & 1);
    }
    if (lane == 0) bulk_wait_all();  // stores done before the shared memory goes
    __syncwarp();
}

/* residue-major columns of the operands' digits: xs[i * count + k] = x[k].digits[i] */
template <int N>
__global__ void __launch_bounds__(256) k_mpint_gather(const MpInt<N> *__restrict__ x, const MpInt<N> *__restrict__ y,
                                                      int64_t count, uint32_t *__restrict__ xs,
                                                      uint32_t *__restrict__ ys) {
    const int64_t total = count * N;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t k = t / N;
        const int i = (int)(t - k * N);
        xs[(int64_t)i * count + k] = __ldg(&x[k].digits[i]);
        ys[(int64_t)i * count + k] = __ldg(&y[k].digits[i]);
    }
}

/* Euclidean adjustment, evaluation and sign of mpint_div from the division's
 * quotient and remainder columns; flags holds the division's flags on entry.
 * A zero divisor or an invalid digit gives the zero record. */
template <int N>
__global__ void __launch_bounds__(128) k_mpint_div_finish(const __grid_constant__ CArg<N> CA,
                                                          const MpInt<N> *__restrict__ x,
                                                          const MpInt<N> *__restrict__ y,
                                                          const uint32_t *__restrict__ q,
                                                          const uint32_t *__restrict__ r, int64_t count,
                                                          MpInt<N> *__restrict__ out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t f = flags[k];
        MpInt<N> res;
        mpint_div_finish<N>(C, __ldg(&x[k].sign), __ldg(&y[k].sign),
                            [&](int i) { return __ldg(q + (int64_t)i * count + k); },
                            [&](int i) { return __ldg(r + (int64_t)i * count + k); }, f, res);
        out[k] = res;
        flags[k] = (uint8_t)f;
    }
}

template <int N>
static grns_status run_mpint_div(const grns_ctx *c, const void *x, const void *y, int64_t count, void *out,
                                 uint8_t *flags, cudaStream_t s) {
    const size_t words = (size_t)N * count;
    void *scratch = nullptr;
    cudaError_t e = scratch_alloc(c, &scratch, words * 4 * sizeof(uint32_t) + (flags ? 0 : (size_t)count), s);
    if (e != cudaSuccess) return cuda_status(e);
    uint32_t *xs = (uint32_t *)scratch, *ys = xs + words, *q = ys + words, *r = q + words;
    uint8_t *f = flags ? flags : (uint8_t *)(r + words);
    const MpInt<N> *xm = (const MpInt<N> *)x, *ym = (const MpInt<N> *)y;
    k_mpint_gather<N><<<grid_for(c, count * N, 256), 256, 0, s>>>(xm, ym, count, xs, ys);
    grns_status st = cuda_status(cudaGetLastError());
    if (st == GRNS_OK) st = launch_div(c, xs, ys, count, count, q, r, f, s);
    if (st == GRNS_OK) {
        k_mpint_div_finish<N><<<grid_for(c, count, 128), 128, 0, s>>>(consts_of<N>(c), xm, ym, q, r, count,
                                                                      (MpInt<N> *)out, f);
        st = cuda_status(cudaGetLastError());
    }
    scratch_free(scratch, s);
    return st;
}

template <int N>
static grns_status run_mpint(const grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                             uint8_t *flags, cudaStream_t s) {
    const int B = 256;
    /* staged chunks up to 64 moduli (above, 4 kMpRecs records a warp exceed shared memory) */
    if constexpr (N <= 64) {
        if ((((uintptr_t)x | (uintptr_t)y | (uintptr_t)out) & 15) == 0) {  // chunks start 16-byte aligned
            /* 8 warps: 2 mbarriers each, then 2 stages of x and y chunks each */
            constexpr size_t smem = 16 * 8 + (size_t)(B / 32) * 4 * kMpRecs * sizeof(MpInt<N>);
            static std::atomic<int> occ[kOccDevices];  // resident blocks per SM, per device
            const int per_sm = resident_blocks(occ, c, k_mpint_bulk<N>, B, smem);
            const int64_t chunks = (count + kMpRecs - 1) / kMpRecs;
            k_mpint_bulk<N><<<grid_for(c, chunks * 32, B, per_sm), B, smem, s>>>(
                consts_of<N>(c), op, (const MpInt<N> *)x, (const MpInt<N> *)y, count, (MpInt<N> *)out, flags);
            return cuda_status(cudaGetLastError());
        }
    }
    k_mpint<N><<<grid_for(c, count, B), B, 0, s>>>(consts_of<N>(c), op, (const MpInt<N> *)x, (const MpInt<N> *)y,
                                                  count, (MpInt<N> *)out, flags);
    return cuda_status(cudaGetLastError());
}

grns_status launch_mpint(const grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                         uint8_t *flags, cudaStream_t s) {
#define C_(n) return op == 3 ? run_mpint_div<n>(c, x, y, count, out, flags, s) : run_mpint<n>(c, op, x, y, count, out, flags, s)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

}  // namespace grns
