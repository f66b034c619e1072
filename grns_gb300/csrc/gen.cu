/*
 * grns_gb300 -- seeded synthetic inputs generated in device memory.
 * No counterpart in the reference, whose tests draw operands from GMP's
 * Mersenne Twister seeded with time(NULL) (tests/tsthelper.cuh:33-60).
 * Definitions match grns_gb300/workload.py exactly (counter-based
 * splitmix64; Lemire rejection for uniform residues; L-bit divisors reduced
 * by Horner; exponents uniform in [1, dmax]).
 */
#include "internal.h"
#include "rns_device.cuh"
#include "rns_mpint.cuh"

namespace grns {

enum : uint32_t { S_X = 1, S_Y = 2, S_DLEN = 3, S_DLIMB = 4, S_SHIFT = 5, S_MAG = 6, S_SIGN = 7 };

__host__ __device__ __forceinline__ uint64_t splitmix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ uint64_t draw(uint64_t key, uint64_t ctr) { return splitmix64(key + ctr); }
inline uint64_t stream_key(uint64_t seed, uint32_t stream) { return splitmix64(seed ^ ((uint64_t)stream << 32)); }

template <int N>
__global__ void k_gen_uniform(const __grid_constant__ CArg<N> CA, uint64_t key, int64_t count, Output<N> out) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
GRNS_UNROLL_N
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i];
            const uint64_t thr = (0ull - (uint64_t)m) % m;
            uint64_t r = 0;
            for (int a = 0; a < 4; a++) {
                uint64_t u = draw(key, ((uint64_t)k * N + i) * 4 + a);
                r = __umul64hi(u, (uint64_t)m);
                if (u * (uint64_t)m >= thr) break;
            }
            out.store(k, i, (uint32_t)r);
        }
    }
}

template <int N>
__global__ void k_gen_divisors(const __grid_constant__ CArg<N> CA, uint64_t key_len, uint64_t key_limb, int log2M,
                               int64_t count, Output<N> out) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        const int L = (int)__umul64hi(draw(key_len, (uint64_t)k), (uint64_t)log2M) + 1;
        const int nl = (L + 31) / 32;
#pragma unroll 1
        for (int i = 0; i < N; i++) {
            const uint32_t m = C.m[i];
            const uint32_t t32 = (uint32_t)((1ull << 32) % m);
            uint32_t r = 0;
            for (int j = nl - 1; j >= 0; j--) {
                uint32_t w = (uint32_t)draw(key_limb, (uint64_t)k * 64 + j);
                if (j == nl - 1) {
                    const int top = L - 32 * (nl - 1);  // bits in the top limb, 1..32
                    if (top < 32) w &= (1u << top) - 1u;
                    w |= 1u << (top - 1);
                }
                r = addmod(mulmod_barrett(r, t32, m, C.mu[i], C.b[i]), w % m, m);
            }
            out.store(k, i, r);
        }
    }
}

/* mp_int_t records of signed integers with magnitude uniform in [0, 2^bits)
 * and a fair-coin sign (zero keeps sign 0), as workload.mpint_values: digits
 * (residues of the magnitude), sign, and the interval evaluation of the
 * digits by the device evaluation (the reference's mpint_set_mpz,
 * src/mpint.cuh:74, evaluates on the host) */
template <int N>
__global__ void k_gen_mpint(const __grid_constant__ CArg<N> CA, uint64_t key_mag, uint64_t key_sign, int bits,
                            int64_t count, MpInt<N> *out) {
    const Consts<N> &C = CA.get();
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x) {
        const int nl = (bits + 31) / 32;
        MpInt<N> v;
        uint32_t any = 0;
#pragma unroll 1
        for (int i = 0; i < N; i++) v.digits[i] = 0;
#pragma unroll 1
        for (int j = nl - 1; j >= 0; j--) {
            uint32_t w = (uint32_t)draw(key_mag, (uint64_t)k * 64 + j);
            if (j == nl - 1) {
                const int top = bits - 32 * (nl - 1);
                if (top < 32) w &= (1u << top) - 1u;
            }
            any |= w;
#pragma unroll 1
            for (int i = 0; i < N; i++) {
                const uint32_t m = C.m[i];
                const uint32_t t32 = (uint32_t)((1ull << 32) % m);
                v.digits[i] = addmod(mulmod_barrett(v.digits[i], t32, m, C.mu[i], C.b[i]), w % m, m);
            }
        }
        v.sign = (any && (draw(key_sign, (uint64_t)k) & 1u)) ? 1 : 0;
        clear_pad(v);
        uint32_t f = 0;
        eval<N>(C, [&](int i) { return v.digits[i]; }, v.eval[0], v.eval[1], f);
        out[k] = v;
    }
}

__global__ void k_gen_shifts(uint64_t key, int64_t count, uint32_t dmax, uint32_t *out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (uint32_t)__umul64hi(draw(key, (uint64_t)k), (uint64_t)dmax) + 1u;
}

}  // namespace grns

using namespace grns;

extern "C" {

grns_status grns_gen_uniform(grns_ctx *c, uint64_t seed, uint32_t stream, int64_t count, int layout, int32_t *out,
                             void *s) {
    if (!c || !out || count < 0 || (layout != 0 && layout != 1)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    const int64_t ld = layout == 0 ? count : 0;
    const uint64_t key = stream_key(seed, stream);
#define C_(n)                                                                                              \
    k_gen_uniform<n><<<grid_for(c, count, 256), 256, 0, (cudaStream_t)s>>>(consts_of<n>(c), key, count,     \
                                                                           Output<n>{(uint32_t *)out, ld}); \
    return cuda_status(cudaGetLastError())
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_gen_divisors(grns_ctx *c, uint64_t seed, int64_t count, int layout, int32_t *out, void *s) {
    if (!c || !out || count < 0 || (layout != 0 && layout != 1)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    const int64_t ld = layout == 0 ? count : 0;
    const uint64_t kl = stream_key(seed, S_DLEN), kw = stream_key(seed, S_DLIMB);
#define C_(n)                                                                                                  \
    k_gen_divisors<n><<<grid_for(c, count, 128), 128, 0, (cudaStream_t)s>>>(consts_of<n>(c), kl, kw, c->log2M, \
                                                                           count, Output<n>{(uint32_t *)out, ld}); \
    return cuda_status(cudaGetLastError())
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_gen_mpint(grns_ctx *c, uint64_t seed, int64_t count, int bits, void *out, void *s) {
    if (!c || !out || count < 0 || bits < 1 || bits > 32 * grns::kMaxModuli) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    const uint64_t km = stream_key(seed, S_MAG), ks = stream_key(seed, S_SIGN);
#define C_(n)                                                                                                   \
    k_gen_mpint<n><<<grid_for(c, count, 128), 128, 0, (cudaStream_t)s>>>(consts_of<n>(c), km, ks, bits, count,  \
                                                                        (MpInt<n> *)out);                       \
    return cuda_status(cudaGetLastError())
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

grns_status grns_gen_shifts(uint64_t seed, int64_t count, uint32_t dmax, uint32_t *out, void *s) {
    if (!out || count < 0 || dmax == 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    int64_t blocks = (count + 255) / 256;
    k_gen_shifts<<<(unsigned)(blocks < 4096 ? blocks : 4096), 256, 0, (cudaStream_t)s>>>(stream_key(seed, S_SHIFT), count,
                                                                                       dmax, out);
    return cuda_status(cudaGetLastError());
}

}  // extern "C"
