/*
 * Host-side stand-ins for the CUDA language features that the reference
 * library's headers (kisupov/grns src/*.cuh) use, so that g++ can compile
 * BOTH of its paths -- the host functions in the global namespace and the
 * device functions in `namespace cuda` -- into one CPU shared library that
 * serves as a checker (oracle/_ref).  Test infrastructure only.
 *
 *  - Execution-space qualifiers become nothing / plain `inline`.
 *  - The FP64 directed-rounding intrinsics (__dmul_rd, __dadd_ru, ...) are
 *    emulated exactly: the operation runs on the host FPU under the matching
 *    IEEE-754 dynamic rounding mode (fesetround).  IEEE-754 defines these
 *    operations as correctly rounded in the requested direction, which is
 *    what the CUDA intrinsics guarantee, so results are bit-identical.
 *    Operands go through volatiles so the compiler cannot move the
 *    arithmetic across the mode switch; build with -frounding-math.
 *  - cudaMemcpyToSymbol copies into the (now host) symbol, so the `cuda::`
 *    constant tables are filled exactly as rns_const_init fills them on a GPU.
 *  - Thread-index builtins exist only so the n-threaded variants compile;
 *    the serial checker never calls those variants.  With
 *    ORACLE_BLOCK_EMULATION defined (oracle/ref/ref_block.cpp) they run for
 *    real: one host thread per CUDA thread of a block, threadIdx per thread,
 *    __syncthreads a barrier of the block and __shfl_down_sync an exchange
 *    among the 32 lanes of a warp (the driver makes __shared__ locals
 *    block-wide statics around its include of the reference headers).
 */
#ifndef ORACLE_CUDA_HOST_SHIM_H
#define ORACLE_CUDA_HOST_SHIM_H

#include <cfenv>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#define __device__
#define __host__
#define __global__
#define __constant__
#define __shared__
#define __forceinline__ inline

typedef int cudaError_t;
#define cudaSuccess 0
inline const char *cudaGetErrorString(cudaError_t) { return "cuda host shim"; }
inline cudaError_t cudaGetLastError() { return 0; }
inline cudaError_t cudaDeviceSynchronize() { return 0; }
template <class T>
inline cudaError_t cudaMemcpyToSymbol(T &symbol, const void *src, size_t bytes) {
    std::memcpy((void *)&symbol, src, bytes);
    return 0;
}

struct oracle_shim_dim3 { unsigned x, y, z; };
static const int warpSize = 32;
#ifdef ORACLE_BLOCK_EMULATION
extern thread_local oracle_shim_dim3 threadIdx;
extern oracle_shim_dim3 blockIdx, blockDim, gridDim;
void oracle_block_sync();
double oracle_warp_shfl_down(double v, int delta);
inline void __syncthreads() { oracle_block_sync(); }
inline double __shfl_down_sync(unsigned, double v, int delta) { return oracle_warp_shfl_down(v, delta); }
#else
extern oracle_shim_dim3 threadIdx, blockIdx, blockDim, gridDim;
inline void __syncthreads() {}
inline double __shfl_down_sync(unsigned, double v, int) { return v; }
#endif

enum { ORACLE_OP_ADD, ORACLE_OP_SUB, ORACLE_OP_MUL, ORACLE_OP_DIV };

static inline double oracle_directed(int mode, int op, double a, double b) {
    volatile double va = a, vb = b;
    volatile double r;
    std::fesetround(mode);
    switch (op) {
        case ORACLE_OP_ADD: r = va + vb; break;
        case ORACLE_OP_SUB: r = va - vb; break;
        case ORACLE_OP_MUL: r = va * vb; break;
        default: r = va / vb; break;
    }
    std::fesetround(FE_TONEAREST);
    return r;
}

inline double __dadd_rd(double a, double b) { return oracle_directed(FE_DOWNWARD, ORACLE_OP_ADD, a, b); }
inline double __dadd_ru(double a, double b) { return oracle_directed(FE_UPWARD, ORACLE_OP_ADD, a, b); }
inline double __dsub_rd(double a, double b) { return oracle_directed(FE_DOWNWARD, ORACLE_OP_SUB, a, b); }
inline double __dsub_ru(double a, double b) { return oracle_directed(FE_UPWARD, ORACLE_OP_SUB, a, b); }
inline double __dmul_rd(double a, double b) { return oracle_directed(FE_DOWNWARD, ORACLE_OP_MUL, a, b); }
inline double __dmul_ru(double a, double b) { return oracle_directed(FE_UPWARD, ORACLE_OP_MUL, a, b); }
inline double __ddiv_rd(double a, double b) { return oracle_directed(FE_DOWNWARD, ORACLE_OP_DIV, a, b); }
inline double __ddiv_ru(double a, double b) { return oracle_directed(FE_UPWARD, ORACLE_OP_DIV, a, b); }

#endif
