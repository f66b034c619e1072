/*
 * grns_gb300 -- internal host-side declarations shared by the translation
 * units of libgrns_gb300.so.
 */
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/grns/grns.h"
#include "consts_host.h"
#include "rns_common.cuh"

namespace grns {
struct Sched {
    int coop;   // 0 serial (one thread per number), 1 n-threaded lane groups
    int chunk;  // numbers per warp claim in the batched kernel
};
}  // namespace grns

struct grns_ctx {
    int n = 0;
    int log2M = 0;
    int device = 0;
    int sm_count = 0;
    int path = 0;  // 0: integer fast path, 1: reference-faithful FP64 kernels (GRNS_PATH_*)
    /* eighths of the bit-identical evaluation's warps that compute on the FP64 pipe (the rest on
     * the integer pipe; the same bits either way) */
    int eval_fp64_eighths = 4;
    grns::HostTables T;  // host copies of all tables
    void *d_tables = nullptr;  // one device allocation holding the table blob
    void *d_consts = nullptr;  // device copy of the constant block, where kernels take it by address
    /* stream-ordered pool for per-call scratch (division records, scaling and
     * batch orders, max partials); keeps up to kPoolKeepBytes across
     * synchronisations so repeated calls do not map fresh memory */
    cudaMemPool_t pool = nullptr;
    /* batched-kernel schedule per grns_op (eval, cmp, div, scale2pow, max, mp_int add/sub/mul) */
    grns::Sched sched[8] = {{0, 256}, {0, 1024}, {0, 256}, {0, 256}, {0, 1024}, {0, 256}, {0, 256}, {0, 256}};
    /* idle stream sets of the host-buffer forms (copy in, copy out, one compute
     * stream per buffer slot), each with an event that completes once the
     * set's last call has ended */
    struct PipeStreams {
        cudaStream_t s[4];
        cudaEvent_t done;
    };
    std::mutex pipe_mu;
    std::vector<PipeStreams> pipe_idle;
    /* kernel constant block for this n (a grns::Consts<n>) */
    alignas(16) unsigned char consts[sizeof(grns::Consts<grns::kMaxModuli>)];
};

namespace grns {

template <int N>
inline const Consts<N> &consts_of(const grns_ctx *c) {
    return *reinterpret_cast<const Consts<N> *>(c->consts);
}

constexpr uint64_t kPoolKeepBytes = 256ull << 20;

/* the batched kernel (and so the server and the autotuner) serves moduli sets
 * of up to 64 moduli; the plain calls cover 128 and 256 */
constexpr int kBatchMaxModuli = 64;

/* an NVTX range over a host-side scope (batched launches, served launches,
 * host-buffer calls): visible in Nsight timelines, a no-op without a tool */
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

/* scratch from the context's pool (the device's default pool if it has none) */
inline cudaError_t scratch_alloc(const grns_ctx *c, void **p, size_t bytes, cudaStream_t s) {
    return c->pool ? cudaMallocFromPoolAsync(p, bytes, c->pool, s) : cudaMallocAsync(p, bytes, s);
}
inline cudaError_t scratch_free(void *p, cudaStream_t s) { return cudaFreeAsync(p, s); }

inline grns_status cuda_status(cudaError_t e) {
    if (e == cudaSuccess) return GRNS_OK;
    if (e == cudaErrorMemoryAllocation) return GRNS_ERR_OUT_OF_MEMORY;
    return GRNS_ERR_CUDA;
}

/* grid size for grid-stride kernels: enough blocks to cover `work`, capped
 * at `waves` resident blocks per SM */
inline unsigned grid_for(const grns_ctx *c, int64_t work, int block, int per_sm = 8) {
    int64_t need = (work + block - 1) / block;
    int64_t cap = (int64_t)c->sm_count * per_sm;
    if (need < 1) need = 1;
    return (unsigned)(need < cap ? need : cap);
}

/* resident blocks per SM of `kernel` at `block` threads and `smem` dynamic
 * bytes, with its shared-memory limit raised first; computed once per device
 * (`cache` holds one entry per device, a zero-initialised static array).  The
 * entry is published after the attribute is set, so a thread that reads a
 * nonzero entry may launch with that much shared memory at once; two threads
 * that both see zero both compute the same value. */
constexpr int kOccDevices = 16;
template <class K>
int resident_blocks(std::atomic<int> (&cache)[kOccDevices], const grns_ctx *c, K kernel, int block, size_t smem) {
    std::atomic<int> *slot = c->device >= 0 && c->device < kOccDevices ? &cache[c->device] : nullptr;
    if (slot) {
        const int v = slot->load(std::memory_order_acquire);
        if (v) return v;
    }
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, block, smem) != cudaSuccess || nb < 1) nb = 1;
    if (slot) slot->store(nb, std::memory_order_release);
    return nb;
}

/* launchers (one translation unit per op family) */
grns_status launch_eval_tight(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                              uint8_t *flags, cudaStream_t s);
grns_status launch_eval(const grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, interval_t *out,
                        uint8_t *flags, cudaStream_t s, bool fast = false);
grns_status launch_cmp(const grns_ctx *c, const uint32_t *x, const uint32_t *y, int64_t ld, int64_t count,
                       int32_t *out, uint8_t *flags, cudaStream_t s);
/* min_per_warp > 0 launches fewer warps when that gives each warp at least
 * min_per_warp numbers (better balance inside a warp's range; the kernel then
 * leaves SMs free for a concurrent launch); ld_out: the outputs' leading
 * dimension (SoA; -1: ld, 0 when the inputs are AoS) */
grns_status launch_div(const grns_ctx *c, const uint32_t *x, const uint32_t *d, int64_t ld, int64_t count,
                       uint32_t *q, uint32_t *r, uint8_t *flags, cudaStream_t s, int min_per_warp = 0,
                       int64_t ld_out = -1);
grns_status launch_scale2pow(const grns_ctx *c, const uint32_t *x, const uint32_t *D, uint32_t D_uniform,
                             int64_t ld, int64_t count, uint32_t *out, uint8_t *flags, cudaStream_t s,
                             int min_per_warp = 0, int64_t ld_out = -1);
grns_status launch_mpint(const grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                         uint8_t *flags, cudaStream_t s);
grns_status launch_max(grns_ctx *c, const uint32_t *x, int64_t ld, int64_t count, uint32_t *out_value,
                       int64_t *out_index, void *scratch, size_t scratch_bytes, cudaStream_t s);
size_t max_scratch_bytes(const grns_ctx *c, int64_t count);
size_t div_scratch_bytes(const grns_ctx *c, int64_t count);  // device scratch of one launch_div call
size_t batch_staging_bytes(int njobs);
grns_status batch_run_async(grns_ctx *c, const grns_job *jobs, int njobs, void *staging, cudaStream_t s);

}  // namespace grns

/* A source that names GRNS_SPLIT_BY_N in its header comment is compiled as
 * GRNS_N_PARTS units (-DGRNS_PART=0, 1, ...): unit k holds the explicit
 * instantiations of the file's per-count templates for the counts
 * GRNS_PART_N lists; unit 0 (GRNS_PART_MAIN) also holds the file's other
 * code, whose dispatch sees the templates through extern declarations.
 * Without GRNS_PART one unit holds everything.  The groups balance compile
 * time (n = 32 and n = 64 cost about as much as n = 4..16 together; 128 and
 * 256, whose loops over the moduli stay rolled, little). */
#define GRNS_N_PARTS 4
#define GRNS_N_PART0_(X) X(4) X(5) X(6) X(7) X(8) X(9) X(10)
#define GRNS_N_PART1_(X) X(11) X(12) X(13) X(14) X(15) X(16) X(128) X(256)
#define GRNS_N_PART2_(X) X(32)
#define GRNS_N_PART3_(X) X(64)
#if !defined(GRNS_PART)
#define GRNS_PART_MAIN 1
#define GRNS_PART_N(X) GRNS_FOR_EACH_N(X)
#elif GRNS_PART == 0
#define GRNS_PART_MAIN 1
#define GRNS_PART_N(X) GRNS_N_PART0_(X)
#elif GRNS_PART == 1
#define GRNS_PART_MAIN 0
#define GRNS_PART_N(X) GRNS_N_PART1_(X)
#elif GRNS_PART == 2
#define GRNS_PART_MAIN 0
#define GRNS_PART_N(X) GRNS_N_PART2_(X)
#elif GRNS_PART == 3
#define GRNS_PART_MAIN 0
#define GRNS_PART_N(X) GRNS_N_PART3_(X)
#else
#error "GRNS_PART out of range"
#endif

/* switch (n) over the supported counts; every case expands the caller's
 * macro C_(n) (which returns; C_NAME names it for the reader), other
 * counts return GRNS_ERR_UNSUPPORTED */
#define GRNS_DISPATCH_CASE_(n) \
    case n:                    \
        C_(n);
#define GRNS_DISPATCH_N(n, C_NAME)             \
    switch (n) {                               \
        GRNS_FOR_EACH_N(GRNS_DISPATCH_CASE_)   \
        default: return GRNS_ERR_UNSUPPORTED;  \
    }
/* the same with the caller's statement for other counts */
#define GRNS_SWITCH_N(n, DEFAULT)            \
    switch (n) {                             \
        GRNS_FOR_EACH_N(GRNS_DISPATCH_CASE_) \
        default: DEFAULT;                    \
    }
