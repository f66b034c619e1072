/*
 * grns_gb300 -- C ABI of the GB300-native RNS interval-evaluation path.
 *
 * Drop-in boundary for the data-parallel hot path of the reference library
 * kisupov/grns (header-only CUDA C++).  The reference exposes device
 * functions that user kernels call per number plus one host launcher
 * (cuda::rns_max).  This ABI replaces the per-number device calls by batched,
 * stream-ordered entry points over whole arrays, keeps the reference's data
 * layouts (types.h) and its moduli-set convention (params.h: a list of
 * pairwise-coprime moduli), and returns status codes instead of exiting.
 *
 * Conventions
 *  - All array pointers are DEVICE pointers unless stated otherwise.
 *  - RNS arrays: `layout` GRNS_LAYOUT_AOS is the reference layout
 *    [x1..xn][x1..xn]... (reference src/dpp/rnsmax.cuh:125); GRNS_LAYOUT_SOA
 *    stores residue i of all `count` numbers contiguously (x[i * count + k]),
 *    the native layout: every modulus slice is a coalesced load.
 *  - Residues are int32 in [0, m_i).  An out-of-range residue sets
 *    GRNS_FLAG_INVALID_INPUT in the element's flag and yields zeros.
 *  - `flags` (optional, may be NULL): one uint8 per element, bits GRNS_FLAG_*.
 *  - `stream` is a cudaStream_t (NULL = legacy default stream).  Calls only
 *    enqueue work; nothing synchronises the device implicitly.
 *  - A context is immutable after creation; it may be used from several host
 *    threads and streams at once.
 */
#ifndef GRNS_GB300_GRNS_H
#define GRNS_GB300_GRNS_H

#include <stddef.h>
#include <stdint.h>

#include "types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GRNS_OK = 0,
    GRNS_ERR_INVALID_ARGUMENT = 1,
    GRNS_ERR_UNSUPPORTED = 2,   /* moduli count or values outside the supported range */
    GRNS_ERR_CUDA = 3,          /* a CUDA runtime call or launch failed */
    GRNS_ERR_OUT_OF_MEMORY = 4,
    GRNS_ERR_TIMEOUT = 5,       /* a bounded wait ran out */
    GRNS_ERR_REJECTED = 6,      /* admission refused (serving) */
    GRNS_ERR_BUSY = 7,
    GRNS_ERR_TOO_LARGE = 8,     /* the request needs more than a fixed capacity */
    GRNS_ERR_CANCELLED = 9      /* serving: the request was cancelled before it ran */
} grns_status;

typedef enum { GRNS_LAYOUT_SOA = 0, GRNS_LAYOUT_AOS = 1 } grns_layout;

enum {
    GRNS_FLAG_INVALID_INPUT = 1u << 0,
    GRNS_FLAG_DIV_BY_ZERO = 1u << 1,
    GRNS_FLAG_ITER_CAP = 1u << 2,
    GRNS_FLAG_OVERFLOW = 1u << 3,      /* mp_int: "Overflow has occurred" (reference src/mpint.cuh:324) */
    GRNS_FLAG_MAY_OVERFLOW = 1u << 4   /* mp_int: "Overflow may occurred" (reference src/mpint.cuh:327) */
};

typedef struct grns_ctx grns_ctx;

const char *grns_status_string(grns_status s);
const char *grns_version(void);

/* ---- context: one moduli set resident on the current device ----
 * Replaces rns_const_init() (reference src/rnsbase.cuh:324) and
 * mpint_const_init() (src/mpint.cuh:20), which fill process-global tables;
 * here every moduli set is its own context, so several (e.g. n = 32 and
 * n = 64) can be resident together.  Supported n: every n from 4 to 16, 32,
 * 64, 128 and 256 (the sizes of the reference's params catalogue);
 * moduli odd, pairwise coprime, 3 <= m_i <= 1431655765.  Above 64 moduli the
 * division and scaling run one number per thread and the kernels' loops over
 * the moduli stay rolled (correct results, not tuned throughput). */
grns_status grns_ctx_create(const int32_t *moduli, int n, grns_ctx **out);
grns_status grns_ctx_destroy(grns_ctx *ctx);

/* Moduli sets in the reference's params.h format (src/params.h:11-39 and the
 * catalogue src/params/moduli-<range>/params.<n>m.<bits>b.h): the text of such a file, with
 * RNS_MODULI_SIZE and RNS_MODULI_VALUES; RNS_MODULI_PRODUCT_LOG2, when given,
 * must equal floor(log2 M), RNS_P2_SCALING_THRESHOLD 30 and
 * RNS_EVAL_RELATIVE_ERROR 1e-7 (the values of every shipped set; others return
 * GRNS_ERR_UNSUPPORTED).  grns_params_parse writes n (and the moduli when
 * `moduli` is not NULL and capacity >= n; log2_out gets the stated
 * RNS_MODULI_PRODUCT_LOG2 or -1); grns_ctx_create_from_params parses and
 * creates the context (grns_ctx_create's rules on n and the moduli apply). */
grns_status grns_params_parse(const char *text, int32_t *moduli, int capacity, int *n_out, int *log2_out);
grns_status grns_ctx_create_from_params(const char *text, grns_ctx **out);
/* the queries below answer 0 for a NULL context */
int grns_ctx_n(const grns_ctx *ctx);
/* floor(log2 M): the reference's RNS_MODULI_PRODUCT_LOG2 (src/params.h:16) */
int grns_ctx_log2(const grns_ctx *ctx);

/* Host copies of the constant tables rns_const_init computes, for checking.
 * which: 0 w_i (RNS_PART_MODULI_PRODUCT_INVERSE, int32[n]); 1 RNS_MODULI_RECIP_RD
 * (double[n]); 2 RNS_MODULI_RECIP_RU (double[n]); 3 RNS_EVAL_ACCURACY (double);
 * 4 RNS_EVAL_REF_FACTOR (int32); 5 RNS_EVAL_UNIT (interval_t); 6
 * RNS_EVAL_INV_UNIT (interval_t); 7 MRC_MULT_INV (int32[n][n], [i][j] = m_i^-1
 * mod m_j for j > i, else 0); 8 RNS_POW2 (int32[log2+1][n]); 9
 * RNS_MODULI_PRODUCT_POW2_RESIDUES (int32[30]); 10
 * RNS_PART_MODULI_PRODUCT_POW2_RESIDUES (int32[30][n]); 11 RNS_POW2_INVERSE
 * (int32[30][n]).  `bytes` must equal the table size. */
grns_status grns_ctx_get_table(const grns_ctx *ctx, int which, void *host_dst, size_t bytes);

/* Kernel family used by the comparison, division, scaling and maximum calls:
 * GRNS_PATH_FAST (default) -- integer-pipe fixed-point enclosures with exact
 * mixed-radix fallback; GRNS_PATH_REFERENCE -- the reference's own GPU
 * algorithms (FP64 interval evaluation inside cmp, one quotient bit per
 * division step as src/rnsdiv.cuh:128), one thread per number.  Both give
 * identical results; eval and mp_int ops are the same in both.  Not to be
 * changed while calls on the context are being enqueued from other threads. */
enum { GRNS_PATH_FAST = 0, GRNS_PATH_REFERENCE = 1 };
grns_status grns_ctx_set_path(grns_ctx *ctx, int path);

/* Share of grns_eval / grns_eval_fast work computed on the FP64 pipe, in
 * eighths of the kernel's warps (0..8): those warps run the reference's own
 * directed-rounding products and sums, the others the exact integer-pipe
 * emulation of the same operations, so both pipes work at once and the
 * intervals are the same bits for any setting.  No counterpart in the
 * reference (a tuning knob of this implementation); default 4, which gives
 * each SM scheduler one warp of each kind. */
grns_status grns_ctx_set_eval_split(grns_ctx *ctx, int fp64_eighths);
int grns_ctx_get_eval_split(const grns_ctx *ctx);

/* ceil(log2(x)) as the device computes it inside the evaluation's refinement
 * loop (src/rnseval.cuh:236 calls CUDA's log2, which is not exact at every
 * power of two).  Diagnostics for checking; x, out are device arrays. */
grns_status grns_device_ceil_log2(const double *x, int32_t *out, int64_t count, void *stream);

/* ---- interval evaluation ----
 * out[k] = [low, upp] enclosing X_k / M, bit-identical to
 * cuda::rns_eval_compute (reference src/rnseval.cuh:182). */
grns_status grns_eval(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, interval_t *out,
                      uint8_t *flags, void *stream);

/* out[k] = the narrowest enclosure of X_k / M with er_float bounds: one unit
 * in the last place wide wherever a 128-bit fixed-point evaluation certifies
 * it, and grns_eval's interval elsewhere (X near 0 or M, bounds straddling
 * two ulps).  Never wider than cuda::rns_eval_compute's interval (no double
 * interval around a nonzero X/M with odd M is narrower than one ulp), but not
 * bit-identical to it: the fast form of rns_eval_compute (reference
 * src/rnseval.cuh:182) for callers that need a certified enclosure. */
grns_status grns_eval_tight(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, interval_t *out,
                            uint8_t *flags, void *stream);

/* out[k] = cuda::rns_eval_compute_fast's interval (reference
 * src/rnseval.cuh:266) bit for bit: rns_eval_compute without the mixed-radix
 * step, for numbers "not too large" (below about M/2).  Near M, where the
 * reference's refinement reads outside its tables, the loop stops with
 * GRNS_FLAG_ITER_CAP. */
grns_status grns_eval_fast(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, interval_t *out,
                           uint8_t *flags, void *stream);

/* ---- magnitude comparison ----
 * out[k] = sign(X_k - Y_k) in {-1, 0, 1}, as cuda::rns_cmp
 * (reference src/rnscmp.cuh:55); the evaluations stay in registers. */
grns_status grns_cmp(grns_ctx *ctx, const int32_t *x, const int32_t *y, int64_t count, int layout,
                     int32_t *out, uint8_t *flags, void *stream);

/* ---- general integer division ----
 * q = floor(X / D), r = X - qD, as cuda::rns_div (reference
 * src/rnsdiv.cuh:128).  D = 0 sets GRNS_FLAG_DIV_BY_ZERO and yields q = 0, r = X. */
grns_status grns_div(grns_ctx *ctx, const int32_t *x, const int32_t *d, int64_t count, int layout,
                     int32_t *q, int32_t *r, uint8_t *flags, void *stream);

/* ---- power-of-two scaling ----
 * out = floor(X / 2^D), as rns_scale2pow (reference src/rnsscal.cuh:93/:207).
 * D is per element (device array `D`, uint32[count]); when D is NULL every
 * element uses `D_uniform`. */
grns_status grns_scale2pow(grns_ctx *ctx, const int32_t *x, const uint32_t *D, uint32_t D_uniform,
                           int64_t count, int layout, int32_t *out, uint8_t *flags, void *stream);

/* ---- host-buffer forms ----
 * grns_div / grns_scale2pow over arrays in HOST memory (same layouts, same
 * results): the arrays are split into `chunks` ranges (0: automatic) and the
 * host->device copies of one range, the kernels of the previous one and the
 * device->host copies of the one before run at the same time on internal
 * streams; the call is ordered on `stream` like the device-pointer forms (the
 * host outputs are complete when the stream reaches that point).  Copies
 * overlap for page-locked host memory.  Device scratch: two chunks' worth of
 * inputs and outputs from the context's pool. */
grns_status grns_div_host(grns_ctx *ctx, const int32_t *x, const int32_t *d, int64_t count, int layout, int32_t *q,
                          int32_t *r, uint8_t *flags, int chunks, void *stream);
grns_status grns_scale2pow_host(grns_ctx *ctx, const int32_t *x, const uint32_t *D, uint32_t D_uniform,
                                int64_t count, int layout, int32_t *out, uint8_t *flags, int chunks, void *stream);

/* ---- multiple-precision integers (mp_int_t arrays, reference layout) ----
 * result = x + y / x - y / x * y elementwise with the interval evaluation
 * derived as cuda::mpint_add / mpint_sub / mpint_mul (reference
 * src/mpint.cuh:336/:407/:478).  Overflow is reported through `flags`
 * (GRNS_FLAG_OVERFLOW / GRNS_FLAG_MAY_OVERFLOW) instead of printf. */
grns_status grns_mpint_add(grns_ctx *ctx, const void *x, const void *y, int64_t count, void *out,
                           uint8_t *flags, void *stream);
grns_status grns_mpint_sub(grns_ctx *ctx, const void *x, const void *y, int64_t count, void *out,
                           uint8_t *flags, void *stream);
grns_status grns_mpint_mul(grns_ctx *ctx, const void *x, const void *y, int64_t count, void *out,
                           uint8_t *flags, void *stream);
/* result = x / y with the Euclidean quotient, as cuda::mpint_div (reference
 * src/mpint.cuh:511; host mpint_div :286 returns the same digits): q = |x| div
 * |y|, plus one when x < 0 and the remainder is nonzero, so that x = q*y + r
 * with 0 <= r < |y|; sign x.sign ^ y.sign (0 for a zero quotient); the
 * evaluation is rns_eval_compute's of the quotient, bit for bit.  y = 0 sets
 * GRNS_FLAG_DIV_BY_ZERO and yields the zero record.  Runs the division of
 * grns_div on residue-major scratch of 16 * n bytes per element from the
 * context's pool; `out` must not overlap x or y. */
grns_status grns_mpint_div(grns_ctx *ctx, const void *x, const void *y, int64_t count, void *out,
                           uint8_t *flags, void *stream);

/* ---- mixed-radix conversion ----
 * out = the Szabo-Tanaka mixed-radix digits of each number (X = a_0 + a_1 m_0
 * + a_2 m_0 m_1 + ...), as cuda::mrc (reference src/mrc.cuh:101), in the
 * layout of x; digits canonical in [0, m_i).  A residue >= its modulus sets
 * GRNS_FLAG_INVALID_INPUT and gives zero digits. */
grns_status grns_mrc(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, int32_t *out, uint8_t *flags,
                     void *stream);

/* ---- binary <-> RNS conversion ----
 * Binary integers are number-major rows of `limbs` little-endian 32-bit
 * words (word l of number k at words[k * limbs + l]; GMP's
 * mpz_export(w, NULL, -1, 4, 0, 0, z) writes this form), limbs <= 256.
 *   grns_from_binary      : out = residues of each nonnegative integer, as
 *                           rns_from_binary (reference src/rnsbase.cuh:253);
 *                           integers of M or more give their residues mod M.
 *   grns_to_binary        : X in [0, M) of each RNS number, as rns_to_binary
 *                           (src/rnsbase.cuh:277); limbs >= grns_ctx_binary_limbs,
 *                           words above the value are zero.  A residue >= its
 *                           modulus sets GRNS_FLAG_INVALID_INPUT and gives 0.
 *   grns_mpint_from_binary: mp_int_t records of sign-magnitude integers, as
 *                           mpint_set_mpz (src/mpint.cuh:74): magnitudes in
 *                           `words`, signs[k] != 0 for a negative integer
 *                           (signs may be NULL: all nonnegative; zero gets
 *                           sign 0); the evaluation is cuda::rns_eval_compute's
 *                           of the digits (the host mpint_set_mpz uses the
 *                           host evaluation).
 *   grns_mpint_to_binary  : magnitudes and signs of mp_int_t records, as
 *                           mpint_get_mpz (src/mpint.cuh:100); signs may be
 *                           NULL; the sign of zero is 0. */
int grns_ctx_binary_limbs(const grns_ctx *ctx);  /* ceil(bits(M) / 32) */
grns_status grns_from_binary(grns_ctx *ctx, const uint32_t *words, int limbs, int64_t count, int layout,
                             int32_t *out, void *stream);
grns_status grns_to_binary(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, uint32_t *words, int limbs,
                           uint8_t *flags, void *stream);
grns_status grns_mpint_from_binary(grns_ctx *ctx, const uint32_t *words, int limbs, const int32_t *signs,
                                   int64_t count, void *out, void *stream);
grns_status grns_mpint_to_binary(grns_ctx *ctx, const void *x, int64_t count, uint32_t *words, int limbs,
                                 int32_t *signs, uint8_t *flags, void *stream);

/* ---- maximum of an RNS array ----
 * Replaces template cuda::rns_max<g1,b1,g2,b2>(out, in, N, buffer)
 * (reference src/dpp/rnsmax.cuh:129): one fused launch, evaluations kept in
 * registers.  out_value (device int32[n]) receives the maximum's residues,
 * out_index (device int64, may be NULL) its index; equal maxima resolve to
 * the smallest index.  count == 0 writes index -1 and leaves out_value as is.
 * scratch: device buffer of at least grns_max_scratch_size() bytes, or NULL
 * to let the call take a stream-ordered allocation (cudaMallocAsync /
 * cudaFreeAsync on `stream`).  The call clears the scratch's first 64 bytes
 * itself; calls that share one scratch buffer must be stream-ordered. */
grns_status grns_max_scratch_size(const grns_ctx *ctx, int64_t count, size_t *bytes);
grns_status grns_max(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, int32_t *out_value,
                     int64_t *out_index, void *scratch, size_t scratch_bytes, void *stream);

/* ---- maximum without allocating ----
 * No counterpart in the reference.  Same results as grns_max, for callers
 * that cannot allocate device memory at call time: processes whose device
 * memory belongs to another allocator with a fixed budget, and
 * latency-critical callers that cannot accept cudaMalloc/cudaFree (which may
 * synchronise the device).  The scratch is a fixed area inside the library,
 * GRNS_NOALLOC_SCRATCH_BYTES per GPU that loads it, held until the process
 * exits; counts whose launch would need more scratch than that return
 * GRNS_ERR_TOO_LARGE (on a 152-SM GB300 every count fits: the largest launch
 * needs 24,384 bytes).
 * The first call on a GPU looks the area up with that GPU current and should
 * come before any stream capture.  All calls on a GPU share the area: calls
 * that overlap on the GPU race, so order them on one stream.  The context's
 * device must be the current device. */
#define GRNS_NOALLOC_SCRATCH_BYTES 32768
grns_status grns_max_noalloc(grns_ctx *ctx, const int32_t *x, int64_t count, int layout, int32_t *out_value,
                             int64_t *out_index, void *stream);


/* ---- batching: many uneven-length arrays in one persistent launch ----
 * No counterpart in the reference, whose callers launch one kernel per array
 * (e.g. tests/test_perf_rnscmp.cu:156).  A batch fixes a list of jobs; each
 * launch runs all of them in ONE persistent kernel (warps pull chunks with an
 * atomic counter; evaluations stay in registers; heaviest jobs first),
 * optionally replayed from a CUDA graph captured on the first launch (needs a
 * non-NULL stream).  Per job: */
typedef enum {
    GRNS_OP_EVAL = 0,       /* a: x;  out0: interval_t[count] */
    GRNS_OP_CMP = 1,        /* a: x, b: y;  out0: int32[count] */
    GRNS_OP_DIV = 2,        /* a: x, b: d;  out0: q, out1: r */
    GRNS_OP_SCALE2POW = 3,  /* a: x, b: uint32 D[count] or NULL (D_uniform);  out0: result */
    GRNS_OP_MAX = 4,        /* a: x;  out0: int32[n] value, out1: int64 index (or NULL) */
    GRNS_OP_MPINT_ADD = 5,  /* a, b, out0: mp_int_t arrays */
    GRNS_OP_MPINT_SUB = 6,
    GRNS_OP_MPINT_MUL = 7,
    GRNS_OP_MPINT_DIV = 8   /* a, b, out0: mp_int_t arrays; the Euclidean quotient of grns_mpint_div
                               (cuda::mpint_div, src/mpint.cuh:511), the division fused in the batched kernel;
                               out0 must not overlap a or b */
} grns_op;

typedef struct {
    int32_t op;       /* grns_op */
    int32_t layout;   /* GRNS_LAYOUT_SOA / GRNS_LAYOUT_AOS for RNS arrays */
    int64_t count;
    int64_t ld;       /* SoA inputs: residue i of number k at a[i*ld + k]; 0 means count
                         (so a job can use the first `count` numbers of a longer array).
                         Outputs are always dense with leading dimension count. */
    const void *a, *b;
    void *out0, *out1;
    uint8_t *flags;   /* optional per-element flags */
    const interval_t *eval_a, *eval_b;  /* cmp: optional evaluations of a and b
                         (as grns_eval produced them); the intervals decide first */
    uint32_t D_uniform;
    uint32_t reserved;
} grns_job;

typedef struct grns_batch grns_batch;
/* contexts of up to 64 moduli (GRNS_ERR_UNSUPPORTED above; the plain calls
 * cover 128 and 256); the same holds for grns_autotune and
 * grns_server_add_context, whose requests run in this kernel */
grns_status grns_batch_create(grns_ctx *ctx, const grns_job *jobs, int njobs, int use_graph, grns_batch **out);
/* new pointers for the same job shapes (op, count, layout); keeps the graph.
 * The job table is copied synchronously from the host: call it once the
 * batch's earlier launches have completed (their stream synchronised or an
 * event after them waited on), since they read the table while they run. */
grns_status grns_batch_update(grns_batch *batch, const grns_job *jobs, int njobs);
grns_status grns_batch_launch(grns_batch *batch, void *stream);
grns_status grns_batch_destroy(grns_batch *batch);
int64_t grns_batch_chunks(const grns_batch *batch);
int grns_batch_grid(const grns_batch *batch);

/* Per-op schedule of the batched kernel: coop = 0 one thread per number
 * ("serial"), 1 the n residues of a number spread over a lane group
 * ("n-threaded", cmp and max only); chunk = numbers per warp claim. */
typedef struct {
    int32_t coop;
    int32_t chunk;
} grns_schedule;
grns_status grns_ctx_get_schedule(const grns_ctx *ctx, int op, grns_schedule *out);
grns_status grns_ctx_set_schedule(grns_ctx *ctx, int op, const grns_schedule *sched);

/* Autotuner: times the candidate schedules of `op` on `count` synthetic
 * numbers of this moduli set in a single-job batch, keeps the fastest in the
 * context and appends it to the text cache `cache_path` (may be NULL);
 * grns_autotune_load applies the cached choices for this GPU and moduli count. */
grns_status grns_autotune(grns_ctx *ctx, int op, int64_t count, const char *cache_path, grns_schedule *chosen,
                          double *best_ms);
grns_status grns_autotune_load(grns_ctx *ctx, const char *cache_path, int *applied);

/* ---- serving: a request stream with continuous batching ----
 * No counterpart in the reference.  Arrays live in server-owned device memory
 * (handles); requests name operand handles and get output handles.  A
 * scheduler thread gives each free launch slot the moduli set of the oldest
 * pending request that can run and packs every pending request of that set
 * whose output footprint fits the HBM budget into one launch of the batched
 * kernel; a request that does not fit is passed by later ones that do until
 * it has waited 50 ms, after which nothing is admitted past it.  It keeps
 * admitting and launching while earlier launches run.  A finished request's
 * status and output handles stay readable (poll, wait) for 60 s after it
 * finishes, for at most the 65,536 most recent ones; later calls naming it
 * return GRNS_ERR_INVALID_ARGUMENT.  An eval request's
 * output is remembered as its operand's evaluation; comparisons of two
 * evaluated arrays decide from the intervals first.  Latency = submit to
 * completion (host callback), summarised as p50 / p99. */
typedef struct grns_server grns_server;

enum {  /* array kinds */
    GRNS_ARRAY_RNS = 0,      /* int32 residues, n per number, SoA or AoS */
    GRNS_ARRAY_U32 = 1,      /* one 32-bit value per number (exponents, comparison results) */
    GRNS_ARRAY_MPINT = 2,    /* mp_int_t */
    GRNS_ARRAY_INTERVAL = 3, /* interval_t (outputs of eval) */
    GRNS_ARRAY_MAXOUT = 4    /* max output: int32[n] value, then int64 index at offset 8*ceil(n/2) */
};

typedef struct {
    size_t hbm_budget_bytes;     /* 0: 80 % of the free device memory at creation */
    int32_t launch_slots;        /* concurrent launches (streams); 0: 4 */
    int32_t max_jobs_per_launch; /* 0: 256 */
    int32_t admission_timeout_ms;/* a request not admitted within this time completes with
                                    GRNS_ERR_REJECTED (0: 10000) */
    int32_t direct_min_count;    /* requests of at least this many numbers run through the per-op
                                    kernels (the plain calls' launches, on the launch's stream)
                                    instead of inside the packed batched kernel: eval, cmp (unless
                                    both evaluations are cached), div, scale2pow, mp_int
                                    add/sub/mul.  0 or negative: never (the default: one packed
                                    launch balanced the benchmark's served stream best) */
    size_t alloc_cap_bytes;      /* hard cap on the device memory the server holds (0: none): a put
                                    beyond it returns, and an admitted request beyond it completes
                                    with, GRNS_ERR_OUT_OF_MEMORY; the server goes on */
    int32_t gather_us;           /* gathering window (0 or negative: off): while the newest pending
                                    request is younger than this, free launch slots wait for more
                                    requests, until the oldest pending one has waited 4 windows or
                                    the pending requests fill a launch.  More requests per launch
                                    for bursts, up to 4 windows more latency */
    int32_t reserved;            /* 0 */
} grns_server_options;

typedef struct {
    int32_t op;         /* grns_op */
    int32_t ctx_index;  /* from grns_server_add_context */
    int64_t count;      /* numbers to process from the start of a (0: all) */
    uint64_t a, b;      /* operand handles (b = 0 when unused; scale2pow: U32 exponents or 0) */
    uint32_t D_uniform;
    uint32_t reserved;
} grns_request;

typedef struct {
    uint64_t completed, rejected, pending, inflight, launches;
    double p50_us, p99_us, mean_us;
    double numbers_per_s;         /* numbers completed / (last completion - first submit) */
    double mean_jobs_per_launch;  /* requests packed per launch */
    size_t bytes_in_use, budget;
} grns_server_stats;

grns_status grns_server_create(const grns_server_options *opt, grns_server **out);
grns_status grns_server_destroy(grns_server *srv);
grns_status grns_server_add_context(grns_server *srv, grns_ctx *ctx, int *index);
/* copy an array in (host or device source); GRNS_ERR_REJECTED when over budget.
 * The copy has finished when the call returns.  It runs on the server's own
 * stream and does not wait for the caller's streams: a device source must
 * already hold its data (the work producing it finished). */
grns_status grns_server_put(grns_server *srv, int ctx_index, int kind, const void *src, int src_on_device,
                            int64_t count, int layout, uint64_t *handle);
/* copy an array out; waits for the request that produces it */
grns_status grns_server_get(grns_server *srv, uint64_t handle, void *host_dst, size_t bytes);
grns_status grns_server_array_info(grns_server *srv, uint64_t handle, int64_t *count, size_t *bytes, void **device_ptr);
/* release an array; waits for the request that produces it and for unfinished
 * requests that read it (directly or as a cached evaluation) */
grns_status grns_server_free(grns_server *srv, uint64_t handle);
/* non-blocking; a request whose footprint can never fit completes at once with GRNS_ERR_REJECTED */
grns_status grns_server_submit(grns_server *srv, const grns_request *req, uint64_t *request_id);
grns_status grns_server_poll(grns_server *srv, uint64_t request_id, int *done, int32_t *status, uint64_t *out0,
                             uint64_t *out1);
grns_status grns_server_wait(grns_server *srv, uint64_t request_id, int64_t timeout_us, int32_t *status,
                             uint64_t *out0, uint64_t *out1);
/* a request still waiting for admission completes with GRNS_ERR_CANCELLED;
 * one already launched runs to the end (GRNS_ERR_BUSY); a finished one is
 * left as it is (GRNS_OK) */
grns_status grns_server_cancel(grns_server *srv, uint64_t request_id);
grns_status grns_server_stats_get(grns_server *srv, grns_server_stats *stats);
grns_status grns_server_reset_stats(grns_server *srv);
/* the gathering window of grns_server_options.gather_us, changed on a live server */
grns_status grns_server_set_gather_us(grns_server *srv, int32_t gather_us);

/* ---- seeded synthetic inputs in device memory ----
 * No counterpart in the reference (its tests draw from GMP's Mersenne
 * Twister seeded with time(NULL), tests/tsthelper.cuh:33).  Counter-based
 * splitmix64 streams, identical to grns_gb300/workload.py:
 *   grns_gen_uniform : numbers uniform in [0, M) (independent uniform residues)
 *   grns_gen_divisors: divisors of bit length L, L uniform in [1, log2 M]
 *   grns_gen_shifts  : exponents uniform in [1, dmax]
 *   grns_gen_mpint   : mp_int_t records of signed integers, magnitude uniform in
 *                      [0, 2^bits) (1 <= bits <= 8192), fair-coin sign, interval
 *                      evaluation filled */
grns_status grns_gen_uniform(grns_ctx *ctx, uint64_t seed, uint32_t stream, int64_t count, int layout, int32_t *out,
                             void *cuda_stream);
grns_status grns_gen_divisors(grns_ctx *ctx, uint64_t seed, int64_t count, int layout, int32_t *out, void *cuda_stream);
grns_status grns_gen_shifts(uint64_t seed, int64_t count, uint32_t dmax, uint32_t *out, void *cuda_stream);
grns_status grns_gen_mpint(grns_ctx *ctx, uint64_t seed, int64_t count, int bits, void *out, void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif
