/*
 * grns_gb300 -- maximum of an RNS array without any device allocation.
 *
 * grns_max needs a little scratch (a block counter and one partial result
 * per block).  It takes it from the caller or allocates it on the stream.
 * Some callers can do neither at call time: a process whose device memory is
 * entirely handed to another allocator (a framework's pool with a fixed
 * budget) must not create allocations outside it, and a latency-critical
 * caller cannot accept cudaMalloc/cudaFree, which may synchronise the whole
 * device.  For them this entry point uses a fixed scratch area compiled into
 * the library: one copy per GPU that loads the library, kept until the
 * process exits, GRNS_NOALLOC_SCRATCH_BYTES (32 KiB) large.
 *
 * The first call on a GPU looks the area's device address up
 * (cudaGetSymbolAddress) with that GPU current; that first call should come
 * before any stream capture.  All calls on one GPU share the area and it
 * keeps the previous call's contents: each call clears the block counter it
 * needs at zero (a stream-ordered memset, no allocation), and calls that
 * overlap on the GPU race on the area, so order them (same stream or events).
 */
#include <mutex>

#include "internal.h"

namespace {

static __device__ __align__(256) unsigned char g_max_scratch[GRNS_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::once_flag g_once[kMaxDevices];
void *g_addr[kMaxDevices];
cudaError_t g_status[kMaxDevices];

/* device address of g_max_scratch on the current GPU (set up once per GPU) */
grns_status scratch_address(int device, void **out) {
    if (device < 0 || device >= kMaxDevices) return GRNS_ERR_UNSUPPORTED;
    std::call_once(g_once[device], [device] {
        void *p = nullptr;
        g_status[device] = cudaGetSymbolAddress(&p, g_max_scratch);
        g_addr[device] = p;
    });
    if (g_status[device] != cudaSuccess) return grns::cuda_status(g_status[device]);
    *out = g_addr[device];
    return GRNS_OK;
}

}  // namespace

extern "C" grns_status grns_max_noalloc(grns_ctx *c, const int32_t *x, int64_t count, int layout, int32_t *out_value,
                                        int64_t *out_index, void *stream) {
    if (!c || count < 0 || (layout != GRNS_LAYOUT_SOA && layout != GRNS_LAYOUT_AOS)) return GRNS_ERR_INVALID_ARGUMENT;
    if (!out_value || (count > 0 && !x)) return GRNS_ERR_INVALID_ARGUMENT;
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return grns::cuda_status(e);
    if (device != c->device) return GRNS_ERR_INVALID_ARGUMENT;  // the context's tables live on c->device
    if (grns::max_scratch_bytes(c, count) > GRNS_NOALLOC_SCRATCH_BYTES) return GRNS_ERR_TOO_LARGE;
    void *scratch = nullptr;
    grns_status st = scratch_address(device, &scratch);
    if (st != GRNS_OK) return st;
    const int64_t ld = layout == GRNS_LAYOUT_SOA ? (count > 0 ? count : 1) : 0;
    return grns::launch_max(c, (const uint32_t *)x, ld, count, (uint32_t *)out_value, out_index, scratch,
                            GRNS_NOALLOC_SCRATCH_BYTES, (cudaStream_t)stream);
}
