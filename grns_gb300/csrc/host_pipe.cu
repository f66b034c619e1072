/*
 * grns_gb300 -- host-buffer entry points: the operation over arrays in host
 * memory, split into chunks so that the host->device copies of chunk j+1 and
 * the device->host copies of chunk j-1 overlap the kernels of chunk j.
 *
 * Internal streams per call: copy in, copy out (the two directions run at the
 * same time on the link) and one compute stream per device buffer slot (two
 * slots used in turn), with events between them; the caller's stream waits
 * for all of them.  Each chunk's kernel is launched with at least 64 numbers
 * per warp, which keeps the warps balanced on short chunks and leaves SMs to
 * the other slot's kernel.  The context keeps idle stream sets for later calls.
 * The call is stream-ordered like the device-pointer entry points: results are
 * in host memory once the caller's stream reaches that point.  Copies overlap
 * only for page-locked host buffers (cudaHostAlloc / cudaHostRegister); with
 * pageable memory they still give the right results.
 */
#include <vector>

#include "internal.h"

namespace grns {
namespace {

/* one host array of the operation: `rows` residue rows of `count` 4-byte
 * elements (SoA: row pitch count), or `count` records of `rec` bytes */
struct HostArr {
    void *host;
    bool soa;     // residue-major rows (pitch count elements)
    int rows;     // SoA rows
    size_t rec;   // bytes per element (AoS record or per-number scalar)
};

size_t chunk_bytes(const HostArr &a, int64_t len) { return a.soa ? (size_t)a.rows * len * 4 : a.rec * len; }

void copy_chunk(const HostArr &a, void *dev, int64_t count, int64_t k0, int64_t len, bool to_device,
                cudaStream_t s, cudaError_t &err) {
    if (err != cudaSuccess) return;
    if (a.soa) {
        char *h = (char *)a.host + k0 * 4;
        err = to_device ? cudaMemcpy2DAsync(dev, len * 4, h, count * 4, len * 4, a.rows, cudaMemcpyHostToDevice, s)
                        : cudaMemcpy2DAsync(h, count * 4, dev, len * 4, len * 4, a.rows, cudaMemcpyDeviceToHost, s);
    } else {
        char *h = (char *)a.host + k0 * a.rec;
        err = to_device ? cudaMemcpyAsync(dev, h, a.rec * len, cudaMemcpyHostToDevice, s)
                        : cudaMemcpyAsync(h, dev, a.rec * len, cudaMemcpyDeviceToHost, s);
    }
}

int auto_chunks(int64_t count, int64_t min_chunk) {
    int64_t c = count / min_chunk;
    return (int)(c < 1 ? 1 : c > 8 ? 8 : c);
}

/* launch(dev_in, dev_out, len, stream) runs the operation on one chunk whose
 * arrays are laid out as in the host arrays with `len` elements (SoA ld = len) */
template <class Launch>
grns_status pipeline(const grns_ctx *c, int64_t count, int chunks, const std::vector<HostArr> &in,
                     const std::vector<HostArr> &out, cudaStream_t user, Launch launch) {
    NvtxRange range("grns host-buffer call");
    constexpr int kSlots = 2;
    if (chunks < 1) chunks = 1;
    if (chunks > count) chunks = (int)count;
    const int64_t per = (count + chunks - 1) / chunks;
    chunks = (int)((count + per - 1) / per);
    size_t slot_bytes = 0;
    std::vector<size_t> off_in(in.size()), off_out(out.size());
    for (size_t a = 0; a < in.size(); a++) {
        off_in[a] = slot_bytes;
        slot_bytes += (chunk_bytes(in[a], per) + 255) & ~(size_t)255;
    }
    for (size_t a = 0; a < out.size(); a++) {
        off_out[a] = slot_bytes;
        slot_bytes += (chunk_bytes(out[a], per) + 255) & ~(size_t)255;
    }
    const int slots = chunks < kSlots ? chunks : kSlots;
    char *buf = nullptr;
    cudaError_t err = scratch_alloc(c, (void **)&buf, slot_bytes * slots, user);
    if (err != cudaSuccess) return cuda_status(err);

    /* a triple whose earlier calls have all ended (so concurrent calls on other
     * streams do not queue behind each other), else new streams */
    grns_ctx *cm = const_cast<grns_ctx *>(c);
    grns_ctx::PipeStreams ps = {{nullptr, nullptr, nullptr, nullptr}, nullptr};
    if (cudaPeekAtLastError() == cudaSuccess) {  // never hide an error the caller has not read
        std::lock_guard<std::mutex> lock(cm->pipe_mu);
        for (size_t k = 0; k < cm->pipe_idle.size(); k++) {
            if (cudaEventQuery(cm->pipe_idle[k].done) == cudaSuccess) {
                ps = cm->pipe_idle[k];
                cm->pipe_idle.erase(cm->pipe_idle.begin() + k);
                break;
            }
        }
        cudaGetLastError();  // a cudaErrorNotReady of the queries is not an error
    }
    cudaStream_t *st = ps.s;  // copy in, copy out, compute of slot 0, compute of slot 1
    for (int k = 0; k < 4; k++)
        if (!st[k] && err == cudaSuccess) err = cudaStreamCreateWithFlags(&st[k], cudaStreamNonBlocking);
    if (!ps.done && err == cudaSuccess) err = cudaEventCreateWithFlags(&ps.done, cudaEventDisableTiming);
    std::vector<cudaEvent_t> ev(3 * chunks + 1, nullptr);
    for (auto &e : ev)
        if (err == cudaSuccess) err = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    cudaEvent_t start = ev[3 * chunks];
    grns_status status = GRNS_OK;
    if (err == cudaSuccess) {
        err = cudaEventRecord(start, user);  // orders the scratch allocation before the copies
        for (int k = 0; k < 4; k++)
            if (err == cudaSuccess) err = cudaStreamWaitEvent(st[k], start, 0);
    }
    for (int j = 0; j < chunks && err == cudaSuccess && status == GRNS_OK; j++) {
        const int64_t k0 = (int64_t)j * per, len = count - k0 < per ? count - k0 : per;
        char *slot = buf + (size_t)(j % slots) * slot_bytes;
        cudaEvent_t e_in = ev[3 * j], e_comp = ev[3 * j + 1], e_out = ev[3 * j + 2];
        if (j >= slots) err = cudaStreamWaitEvent(st[0], ev[3 * (j - slots) + 1], 0);  // inputs consumed
        for (size_t a = 0; a < in.size(); a++) copy_chunk(in[a], slot + off_in[a], count, k0, len, true, st[0], err);
        cudaStream_t comp = st[2 + j % slots];  // chunks of the two slots may compute at the same time
        if (err == cudaSuccess) err = cudaEventRecord(e_in, st[0]);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(comp, e_in, 0);
        if (err == cudaSuccess && j >= slots) err = cudaStreamWaitEvent(comp, ev[3 * (j - slots) + 2], 0);  // outputs read
        if (err != cudaSuccess) break;
        std::vector<void *> din(in.size()), dout(out.size());
        for (size_t a = 0; a < in.size(); a++) din[a] = slot + off_in[a];
        for (size_t a = 0; a < out.size(); a++) dout[a] = slot + off_out[a];
        status = launch(din, dout, len, comp);
        if (status != GRNS_OK) break;
        err = cudaEventRecord(e_comp, comp);
        if (err == cudaSuccess) err = cudaStreamWaitEvent(st[1], e_comp, 0);
        for (size_t a = 0; a < out.size(); a++)
            copy_chunk(out[a], slot + off_out[a], count, k0, len, false, st[1], err);
        if (err == cudaSuccess) err = cudaEventRecord(e_out, st[1]);
    }
    /* join: the caller's stream waits for every internal stream, then frees the
     * slots; the streams go back to the context (work queued on them later
     * runs after this call's, which keeps the order without waiting here) */
    bool joined = ps.done != nullptr;
    for (int k = 0; k < 4; k++) {
        if (!st[k]) {
            joined = false;
            continue;
        }
        cudaEvent_t done = nullptr;
        bool waits = cudaEventCreateWithFlags(&done, cudaEventDisableTiming) == cudaSuccess;
        if (waits) {
            waits = cudaEventRecord(done, st[k]) == cudaSuccess && cudaStreamWaitEvent(user, done, 0) == cudaSuccess;
            cudaEventDestroy(done);
        }
        if (!waits) {  // the slots are freed on the caller's stream: this stream's copies end first
            cudaStreamSynchronize(st[k]);
            joined = false;
        }
    }
    if (joined) joined = cudaEventRecord(ps.done, user) == cudaSuccess;
    bool kept = false;
    if (joined) {
        std::lock_guard<std::mutex> lock(cm->pipe_mu);
        if (cm->pipe_idle.size() < 8) {
            cm->pipe_idle.push_back(ps);
            kept = true;
        }
    }
    if (!kept) {
        for (int k = 0; k < 4; k++)
            if (st[k]) cudaStreamDestroy(st[k]);  // released once its work completes
        if (ps.done) cudaEventDestroy(ps.done);
    }
    for (auto &e : ev)
        if (e) cudaEventDestroy(e);
    scratch_free(buf, user);
    if (status != GRNS_OK) return status;
    return cuda_status(err);
}

bool layout_ok(int layout) { return layout == GRNS_LAYOUT_SOA || layout == GRNS_LAYOUT_AOS; }

constexpr int kChunkPerWarp = 64;

}  // namespace
}  // namespace grns

extern "C" {

grns_status grns_div_host(grns_ctx *c, const int32_t *x, const int32_t *d, int64_t count, int layout, int32_t *q,
                          int32_t *r, uint8_t *flags, int chunks, void *stream) {
    using namespace grns;
    if (!c || count < 0 || !layout_ok(layout) || chunks < 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !d || !q || !r) return GRNS_ERR_INVALID_ARGUMENT;
    const bool soa = layout == GRNS_LAYOUT_SOA;
    const size_t rec = (size_t)4 * c->n;
    std::vector<HostArr> in = {{(void *)x, soa, c->n, rec}, {(void *)d, soa, c->n, rec}};
    std::vector<HostArr> out = {{(void *)q, soa, c->n, rec}, {(void *)r, soa, c->n, rec}};
    if (flags) out.push_back({(void *)flags, false, 1, 1});
    const bool has_flags = flags != nullptr;
    return pipeline(c, count, chunks ? chunks : auto_chunks(count, 1 << 17), in, out, (cudaStream_t)stream,
                    [&](const std::vector<void *> &di, const std::vector<void *> &dout, int64_t len, cudaStream_t s) {
                        return launch_div(c, (const uint32_t *)di[0], (const uint32_t *)di[1], soa ? len : 0, len,
                                          (uint32_t *)dout[0], (uint32_t *)dout[1],
                                          has_flags ? (uint8_t *)dout[2] : nullptr, s, kChunkPerWarp);
                    });
}

grns_status grns_scale2pow_host(grns_ctx *c, const int32_t *x, const uint32_t *D, uint32_t D_uniform, int64_t count,
                                int layout, int32_t *out, uint8_t *flags, int chunks, void *stream) {
    using namespace grns;
    if (!c || count < 0 || !layout_ok(layout) || chunks < 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    const bool soa = layout == GRNS_LAYOUT_SOA;
    const size_t rec = (size_t)4 * c->n;
    std::vector<HostArr> in = {{(void *)x, soa, c->n, rec}};
    if (D) in.push_back({(void *)D, false, 1, 4});
    std::vector<HostArr> outs = {{(void *)out, soa, c->n, rec}};
    if (flags) outs.push_back({(void *)flags, false, 1, 1});
    const bool has_D = D != nullptr, has_flags = flags != nullptr;
    return pipeline(c, count, chunks ? chunks : auto_chunks(count, 1 << 16), in, outs, (cudaStream_t)stream,
                    [&](const std::vector<void *> &di, const std::vector<void *> &dout, int64_t len, cudaStream_t s) {
                        return launch_scale2pow(c, (const uint32_t *)di[0], has_D ? (const uint32_t *)di[1] : nullptr,
                                                D_uniform, soa ? len : 0, len, (uint32_t *)dout[0],
                                                has_flags ? (uint8_t *)dout[1] : nullptr, s, kChunkPerWarp);
                    });
}

}  // extern "C"
