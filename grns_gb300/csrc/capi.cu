/*
 * grns_gb300 -- extern "C" entry points: argument validation, layout
 * resolution and dispatch to the per-op launchers.
 */
#include "internal.h"

namespace {

inline bool layout_ok(int layout) { return layout == GRNS_LAYOUT_SOA || layout == GRNS_LAYOUT_AOS; }
/* SoA leading dimension = count; 0 selects AoS addressing in the kernels */
inline int64_t ld_of(int layout, int64_t count) { return layout == GRNS_LAYOUT_SOA ? (count > 0 ? count : 1) : 0; }

}  // namespace

extern "C" {

grns_status grns_eval(grns_ctx *c, const int32_t *x, int64_t count, int layout, interval_t *out, uint8_t *flags,
                      void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_eval(c, (const uint32_t *)x, ld_of(layout, count), count, out, flags, (cudaStream_t)stream);
}

grns_status grns_eval_fast(grns_ctx *c, const int32_t *x, int64_t count, int layout, interval_t *out, uint8_t *flags,
                           void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_eval(c, (const uint32_t *)x, ld_of(layout, count), count, out, flags, (cudaStream_t)stream,
                             true);
}

grns_status grns_eval_tight(grns_ctx *c, const int32_t *x, int64_t count, int layout, interval_t *out, uint8_t *flags,
                            void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_eval_tight(c, (const uint32_t *)x, ld_of(layout, count), count, out, flags,
                                   (cudaStream_t)stream);
}

grns_status grns_cmp(grns_ctx *c, const int32_t *x, const int32_t *y, int64_t count, int layout, int32_t *out,
                     uint8_t *flags, void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !y || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_cmp(c, (const uint32_t *)x, (const uint32_t *)y, ld_of(layout, count), count, out, flags,
                            (cudaStream_t)stream);
}

grns_status grns_div(grns_ctx *c, const int32_t *x, const int32_t *d, int64_t count, int layout, int32_t *q,
                     int32_t *r, uint8_t *flags, void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !d || !q || !r) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_div(c, (const uint32_t *)x, (const uint32_t *)d, ld_of(layout, count), count, (uint32_t *)q,
                            (uint32_t *)r, flags, (cudaStream_t)stream);
}

grns_status grns_scale2pow(grns_ctx *c, const int32_t *x, const uint32_t *D, uint32_t D_uniform, int64_t count,
                           int layout, int32_t *out, uint8_t *flags, void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_scale2pow(c, (const uint32_t *)x, D, D_uniform, ld_of(layout, count), count, (uint32_t *)out,
                                  flags, (cudaStream_t)stream);
}

static grns_status mpint_op(grns_ctx *c, int op, const void *x, const void *y, int64_t count, void *out,
                            uint8_t *flags, void *stream) {
    if (!c || count < 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    if (!x || !y || !out) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_mpint(c, op, x, y, count, out, flags, (cudaStream_t)stream);
}
grns_status grns_mpint_add(grns_ctx *c, const void *x, const void *y, int64_t count, void *out, uint8_t *flags,
                           void *stream) {
    return mpint_op(c, 0, x, y, count, out, flags, stream);
}
grns_status grns_mpint_sub(grns_ctx *c, const void *x, const void *y, int64_t count, void *out, uint8_t *flags,
                           void *stream) {
    return mpint_op(c, 1, x, y, count, out, flags, stream);
}
grns_status grns_mpint_mul(grns_ctx *c, const void *x, const void *y, int64_t count, void *out, uint8_t *flags,
                           void *stream) {
    return mpint_op(c, 2, x, y, count, out, flags, stream);
}
grns_status grns_mpint_div(grns_ctx *c, const void *x, const void *y, int64_t count, void *out, uint8_t *flags,
                           void *stream) {
    return mpint_op(c, 3, x, y, count, out, flags, stream);
}

grns_status grns_max_scratch_size(const grns_ctx *c, int64_t count, size_t *bytes) {
    if (!c || !bytes || count < 0) return GRNS_ERR_INVALID_ARGUMENT;
    *bytes = grns::max_scratch_bytes(c, count);
    return GRNS_OK;
}

grns_status grns_max(grns_ctx *c, const int32_t *x, int64_t count, int layout, int32_t *out_value,
                     int64_t *out_index, void *scratch, size_t scratch_bytes, void *stream) {
    if (!c || count < 0 || !layout_ok(layout)) return GRNS_ERR_INVALID_ARGUMENT;
    if (!out_value || (count > 0 && !x)) return GRNS_ERR_INVALID_ARGUMENT;
    if (scratch && scratch_bytes < grns::max_scratch_bytes(c, count)) return GRNS_ERR_INVALID_ARGUMENT;
    return grns::launch_max(c, (const uint32_t *)x, ld_of(layout, count), count, (uint32_t *)out_value, out_index,
                            scratch, scratch_bytes, (cudaStream_t)stream);
}

}  // extern "C"
