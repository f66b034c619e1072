/*
 * grns_gb300 -- mixed-radix conversion over arrays (cuda::mrc, reference
 * src/mrc.cuh:101; Szabo-Tanaka digits: X = a_0 + a_1 m_0 + a_2 m_0 m_1 + ...).
 *
 * One thread per number.  The digit loops are uniform across a warp (the
 * modulus i and the earlier digit j are the same on every lane), so the
 * constants m_j^-1 mod m_i with their Shoup companions sit in a per-block
 * shared table read as broadcasts, and each thread keeps its digits in a
 * shared-memory column; the loops stay rolled (n^2 / 2 steps would not fit
 * the instruction cache unrolled).  Digits are canonical (the reference's
 * mod_psub can return a negative digit for descending moduli, a case of
 * probability ~1e-13 on such sets).
 */
#include "internal.h"
#include "rns_device.cuh"

namespace grns {

constexpr int kMrcBlock = 128;

template <int N>
__global__ void __launch_bounds__(kMrcBlock) k_mrc(const __grid_constant__ CArg<N> CA, Operand<N> x, int64_t count,
                                                   Output<N> out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    extern __shared__ uint2 mrc_smem[];
    uint2 *inv = mrc_smem;  // [j * N + i] = (m_j^-1 mod m_i, Shoup companion), j < i
    uint32_t *col = reinterpret_cast<uint32_t *>(inv + N * N) + threadIdx.x;
    for (int w = threadIdx.x; w < N * N; w += blockDim.x) inv[w] = make_uint2(C.mrc_inv[w], C.mrc_inv_sh[w]);
    __syncthreads();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        uint32_t bad = 0;
#pragma unroll 1
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i], b = C.b[i], mu = C.mu[i];
            uint32_t v = x.load(k, i);
            bad |= (uint32_t)(v >= m);
#pragma unroll 4
            for (int j = 0; j < i; j++) {
                uint32_t t = col[j * kMrcBlock];
                if (C.m[j] > m) t = b >= 16 ? mulmod_barrett(t, 1u, m, mu, b) : t % m;  // digit j below m_j
                const uint2 c = inv[j * N + i];
                v = mulmod_shoup(submod(v, t, m), c.x, c.y, m);
            }
            col[i * kMrcBlock] = v;
        }
#pragma unroll 4
        for (int i = 0; i < N; i++) out.store(k, i, bad ? 0u : col[i * kMrcBlock]);
        if (flags) flags[k] = bad ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
    }
}

/* the 128- and 256-moduli sets, P = 512 / n numbers per warp (lane l holds
 * residues l + 32 j of each): column by column, digit j (residue j once
 * every earlier digit is applied) is broadcast from its lane and every later
 * residue i becomes (x_i - a_j) m_j^-1 mod m_i -- per residue the same
 * operations in the same order as k_mrc, so the same digits.  Each inverse
 * read from the n^2 table (512 KB at n = 256, through L2) serves the P
 * numbers. */
template <int N>
constexpr int mrc_warp_numbers() {
    return 512 / N;
}
template <int N>
__global__ void __launch_bounds__(kMrcBlock) k_mrc_warp(const __grid_constant__ CArg<N> CA, Operand<N> x,
                                                        int64_t count, Output<N> out, uint8_t *__restrict__ flags) {
    const Consts<N> &C = CA.get();
    constexpr int J = N / 32, P = mrc_warp_numbers<N>();
    const unsigned FULL = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    uint32_t m[J], b[J], mu[J];
#pragma unroll
    for (int j = 0; j < J; j++) {
        m[j] = C.m[lane + 32 * j];
        b[j] = C.b[lane + 32 * j];
        mu[j] = C.mu[lane + 32 * j];
    }
    const int64_t warps = ((int64_t)gridDim.x * kMrcBlock) >> 5;
    for (int64_t k0 = (((int64_t)blockIdx.x * kMrcBlock + threadIdx.x) >> 5) * P; k0 < count; k0 += warps * P) {
        uint32_t y[P][J];
        bool bad[P];
#pragma unroll
        for (int p = 0; p < P; p++) {
            bool bp = false;
#pragma unroll
            for (int j = 0; j < J; j++) {
                y[p][j] = k0 + p < count ? x.load(k0 + p, lane + 32 * j) : 0u;
                bp |= y[p][j] >= m[j];
            }
            bad[p] = __any_sync(FULL, bp);
        }
#pragma unroll
        for (int jj = 0; jj < J; jj++) {
#pragma unroll 1
            for (int l = 0; l < 32; l++) {
                const int j = 32 * jj + l;
                uint32_t a[P];
#pragma unroll
                for (int p = 0; p < P; p++) a[p] = __shfl_sync(FULL, y[p][jj], l);  // digit j of each number
                const uint32_t mj = C.m[j];
#pragma unroll
                for (int j2 = jj; j2 < J; j2++) {
                    const int i = lane + 32 * j2;
                    if (j2 > jj || lane > l) {
                        const uint32_t c = __ldg(C.mrc_inv + j * N + i), cs = __ldg(C.mrc_inv_sh + j * N + i);
#pragma unroll
                        for (int p = 0; p < P; p++) {
                            uint32_t t = a[p];
                            if (mj > m[j2]) t = b[j2] >= 16 ? mulmod_barrett(t, 1u, m[j2], mu[j2], b[j2]) : t % m[j2];
                            y[p][j2] = mulmod_shoup(submod(y[p][j2], t, m[j2]), c, cs, m[j2]);
                        }
                    }
                }
            }
        }
#pragma unroll
        for (int p = 0; p < P; p++) {
            if (k0 + p >= count) break;
#pragma unroll
            for (int j = 0; j < J; j++) out.store(k0 + p, lane + 32 * j, bad[p] ? 0u : y[p][j]);
            if (flags && lane == 0) flags[k0 + p] = bad[p] ? (uint8_t)kFlagInvalidInput : (uint8_t)0;
        }
    }
}

template <int N>
static grns_status run_mrc(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, uint32_t *out,
                           uint8_t *flags, cudaStream_t s) {
    if constexpr (N > 64) {
        constexpr int P = mrc_warp_numbers<N>();
        k_mrc_warp<N><<<grid_for(c, (count + P - 1) / P * 32, kMrcBlock, 16), kMrcBlock, 0, s>>>(
            consts_of<N>(c), Operand<N>{x, ld}, count, Output<N>{out, ld}, flags);
        return cuda_status(cudaGetLastError());
    } else {  // one number per thread, the inverses staged in shared memory (n^2 8-byte entries)
        const size_t smem = (size_t)N * N * sizeof(uint2) + (size_t)N * kMrcBlock * 4;
        static std::atomic<int> per_sm[kOccDevices];  // resident blocks per SM, per device
        const int occ = resident_blocks(per_sm, c, k_mrc<N>, kMrcBlock, smem);
        k_mrc<N><<<grid_for(c, count, kMrcBlock, occ), kMrcBlock, smem, s>>>(consts_of<N>(c), Operand<N>{x, ld},
                                                                              count, Output<N>{out, ld}, flags);
        return cuda_status(cudaGetLastError());
    }
}

}  // namespace grns

extern "C" grns_status grns_mrc(grns_ctx *c, const int32_t *x, int64_t count, int layout, int32_t *out,
                                uint8_t *flags, void *stream) {
    if (!c || count < 0 || (layout != GRNS_LAYOUT_SOA && layout != GRNS_LAYOUT_AOS)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    const int64_t ld = layout == GRNS_LAYOUT_SOA ? count : 0;
#define C_(n) return grns::run_mrc<n>(c, (const uint32_t *)x, ld, count, (uint32_t *)out, flags, (cudaStream_t)stream)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}
