/*
 * grns_gb300 -- moduli-set contexts: the constant tables of the reference's
 * rns_const_init (kisupov/grns src/rnsbase.cuh:324-451) computed on the host
 * without GMP/MPFR, uploaded once per context.
 *
 * Only two properties of the big product M are needed: its bit length
 * (floor(log2 M), the RNS_MODULI_PRODUCT_LOG2 convention) and its top 53
 * bits, because the reference converts M to a 53-bit MPFR number rounded
 * down (mpfr_init default precision + MPFR_RNDD, :326/:336) before it
 * computes 1/M and 1-1/M.  Everything else is a product, power or inverse
 * modulo a 31-bit modulus or a power of two.
 */
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <new>
#include <string>

#include "internal.h"

namespace {

int64_t gcd64(int64_t a, int64_t b) {
    while (b) {
        int64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

/* the constant block on the host, and on the device where kernels take it by address */
template <int N>
grns_status finish_consts(grns_ctx *c, const uint32_t *d_tables) {
    grns::Consts<N> &C = *reinterpret_cast<grns::Consts<N> *>(c->consts);
    grns::fill_consts<N>(C, c->T, d_tables);
    C.self = nullptr;
    if (!grns::consts_by_address<N>()) return GRNS_OK;
    cudaError_t e = cudaMalloc(&c->d_consts, sizeof(C));
    if (e != cudaSuccess) return grns::cuda_status(e);
    C.self = c->d_consts;
    return grns::cuda_status(cudaMemcpy(c->d_consts, &C, sizeof(C), cudaMemcpyHostToDevice));
}

grns_status build(grns_ctx *c, const uint32_t *moduli) {
    grns::build_tables(c->T, moduli, c->n);
    c->log2M = c->T.log2M;
    std::vector<uint32_t> blob = grns::table_blob(c->T);
    cudaError_t e = cudaMalloc(&c->d_tables, blob.size() * sizeof(uint32_t));
    if (e != cudaSuccess) return grns::cuda_status(e);
    e = cudaMemcpy(c->d_tables, blob.data(), blob.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return grns::cuda_status(e);
    const uint32_t *d = (const uint32_t *)c->d_tables;
#define C_(n) return finish_consts<n>(c, d)
    GRNS_DISPATCH_N(c->n, C_)
#undef C_
}

/* ---- the reference's params.h format (src/params.h:11-39, src/params/...) ---- */

/* text with comments removed and backslash-newline continuations joined */
std::string params_clean(const char *text) {
    std::string out;
    for (const char *p = text; *p;) {
        if (p[0] == '/' && p[1] == '*') {
            const char *e = strstr(p + 2, "*/");
            p = e ? e + 2 : p + strlen(p);
            out += ' ';
        } else if (p[0] == '/' && p[1] == '/') {
            while (*p && *p != '\n') p++;
        } else if (p[0] == '\\' && p[1] == '\n') {
            p += 2;
            out += ' ';
        } else {
            out += *p++;
        }
    }
    return out;
}

/* the text after "#define NAME" up to the end of its line, or "" */
std::string params_define(const std::string &t, const char *name) {
    size_t pos = 0;
    const size_t nl = strlen(name);
    while ((pos = t.find("#define", pos)) != std::string::npos) {
        size_t q = pos + 7;
        while (q < t.size() && (t[q] == ' ' || t[q] == '\t')) q++;
        if (t.compare(q, nl, name) == 0 && q + nl < t.size() && !(isalnum((unsigned char)t[q + nl]) || t[q + nl] == '_')) {
            const size_t e = t.find('\n', q + nl);
            return t.substr(q + nl, e == std::string::npos ? std::string::npos : e - q - nl);
        }
        pos = q;
    }
    return "";
}

/* integers of a definition, ignoring parentheses, braces and commas; false on other text */
bool params_numbers(const std::string &v, std::vector<long long> &out, bool allow_fraction = false) {
    out.clear();
    for (size_t i = 0; i < v.size();) {
        const char ch = v[i];
        if (ch == ' ' || ch == '\t' || ch == '\r' || ch == '(' || ch == ')' || ch == '{' || ch == '}' || ch == ',') {
            i++;
        } else if (isdigit((unsigned char)ch) || (allow_fraction && ch == '.')) {
            size_t j = i;
            while (j < v.size() && (isdigit((unsigned char)v[j]) || (allow_fraction && (v[j] == '.' || v[j] == 'e' ||
                                                                                       v[j] == 'E' || v[j] == '-'))))
                j++;
            if (!allow_fraction) {
                if (j - i > 18) return false;  // beyond any size, modulus or exponent (and long long)
                out.push_back(strtoll(v.substr(i, j - i).c_str(), nullptr, 10));
            } else {
                out.push_back(0);
            }
            i = j;
        } else {
            return false;
        }
    }
    return true;
}

__global__ void k_ceil_log2(const double *x, int32_t *out, int64_t count) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < count; k += (int64_t)gridDim.x * blockDim.x)
        out[k] = (int32_t)ceil(log2(x[k]));
}

}  // namespace

extern "C" {

const char *grns_status_string(grns_status s) {
    switch (s) {
        case GRNS_OK: return "ok";
        case GRNS_ERR_INVALID_ARGUMENT: return "invalid argument";
        case GRNS_ERR_UNSUPPORTED: return "unsupported moduli set";
        case GRNS_ERR_CUDA: return "CUDA error";
        case GRNS_ERR_OUT_OF_MEMORY: return "out of device memory";
        case GRNS_ERR_TIMEOUT: return "timed out";
        case GRNS_ERR_REJECTED: return "rejected by admission control";
        case GRNS_ERR_BUSY: return "busy";
        case GRNS_ERR_TOO_LARGE: return "request exceeds a fixed capacity";
        case GRNS_ERR_CANCELLED: return "cancelled";
    }
    return "unknown status";
}

const char *grns_version(void) { return "grns_gb300 0.1 (sm_103a)"; }

grns_status grns_ctx_create(const int32_t *moduli, int n, grns_ctx **out) {
    if (!moduli || !out) return GRNS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    if (!grns::supported_n(n)) return GRNS_ERR_UNSUPPORTED;
    for (int i = 0; i < n; i++) {
        if (moduli[i] < 3 || moduli[i] > 1431655765 || (moduli[i] & 1) == 0) return GRNS_ERR_UNSUPPORTED;
        for (int j = 0; j < i; j++)
            if (gcd64(moduli[i], moduli[j]) != 1) return GRNS_ERR_INVALID_ARGUMENT;
    }
    grns_ctx *c = new (std::nothrow) grns_ctx();
    if (!c) return GRNS_ERR_OUT_OF_MEMORY;
    c->n = n;
    std::vector<uint32_t> mods(moduli, moduli + n);
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device);
    if (e != cudaSuccess) {
        delete c;
        return grns::cuda_status(e);
    }
    {  // scratch pool; without one, calls use the device's default pool
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = c->device;
        if (cudaMemPoolCreate(&c->pool, &props) == cudaSuccess) {
            uint64_t keep = grns::kPoolKeepBytes;
            cudaMemPoolSetAttribute(c->pool, cudaMemPoolAttrReleaseThreshold, &keep);
        } else {
            c->pool = nullptr;
            cudaGetLastError();
        }
    }
    grns_status st = build(c, mods.data());
    if (st != GRNS_OK) {
        grns_ctx_destroy(c);
        return st;
    }
    *out = c;
    return GRNS_OK;
}

grns_status grns_params_parse(const char *text, int32_t *moduli, int capacity, int *n_out, int *log2_out) {
    if (!text || !n_out) return GRNS_ERR_INVALID_ARGUMENT;
    const std::string t = params_clean(text);
    std::vector<long long> size, vals, lg, thr;
    if (!params_numbers(params_define(t, "RNS_MODULI_SIZE"), size) || size.size() != 1 ||
        !params_numbers(params_define(t, "RNS_MODULI_VALUES"), vals) || (long long)vals.size() != size[0])
        return GRNS_ERR_INVALID_ARGUMENT;
    const std::string l2 = params_define(t, "RNS_MODULI_PRODUCT_LOG2");
    if (!l2.empty() && (!params_numbers(l2, lg) || lg.size() != 1)) return GRNS_ERR_INVALID_ARGUMENT;
    /* the scaling threshold and the evaluation error bound are fixed at the
     * values every shipped set uses */
    const std::string th = params_define(t, "RNS_P2_SCALING_THRESHOLD");
    if (!th.empty() && (!params_numbers(th, thr) || thr.size() != 1 || thr[0] != grns::kScaleStep))
        return GRNS_ERR_UNSUPPORTED;
    const std::string re = params_define(t, "RNS_EVAL_RELATIVE_ERROR");
    if (!re.empty()) {
        const size_t at = re.find_first_not_of(" \t(");
        if (at == std::string::npos || std::fabs(strtod(re.c_str() + at, nullptr) - 0.0000001) > 1e-15)
            return GRNS_ERR_UNSUPPORTED;
    }
    for (long long v : vals)
        if (v < 1 || v > 0x7fffffffLL) return GRNS_ERR_INVALID_ARGUMENT;
    if (!lg.empty() && lg[0] > (1 << 20)) return GRNS_ERR_INVALID_ARGUMENT;
    *n_out = (int)size[0];
    if (log2_out) *log2_out = lg.empty() ? -1 : (int)lg[0];
    if (moduli) {
        if (capacity < (int)vals.size()) return GRNS_ERR_INVALID_ARGUMENT;
        for (size_t i = 0; i < vals.size(); i++) moduli[i] = (int32_t)vals[i];
    }
    return GRNS_OK;
}

grns_status grns_ctx_create_from_params(const char *text, grns_ctx **out) {
    if (!out) return GRNS_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0, lg = -1;
    grns_status st = grns_params_parse(text, nullptr, 0, &n, &lg);
    if (st != GRNS_OK) return st;
    std::vector<int32_t> mods(n > 0 ? n : 1);
    st = grns_params_parse(text, mods.data(), n, &n, &lg);
    if (st != GRNS_OK) return st;
    st = grns_ctx_create(mods.data(), n, out);
    if (st == GRNS_OK && lg >= 0 && lg != (*out)->log2M) {  // RNS_MODULI_PRODUCT_LOG2 must be floor(log2 M)
        grns_ctx_destroy(*out);
        *out = nullptr;
        return GRNS_ERR_INVALID_ARGUMENT;
    }
    return st;
}

grns_status grns_ctx_destroy(grns_ctx *c) {
    if (!c) return GRNS_ERR_INVALID_ARGUMENT;
    for (auto &p : c->pipe_idle) {
        for (cudaStream_t s : p.s) cudaStreamDestroy(s);
        cudaEventDestroy(p.done);
    }
    if (c->d_tables) cudaFree(c->d_tables);
    if (c->d_consts) cudaFree(c->d_consts);
    if (c->pool) cudaMemPoolDestroy(c->pool);  // released once outstanding scratch is freed
    delete c;
    return GRNS_OK;
}

int grns_ctx_n(const grns_ctx *c) { return c ? c->n : 0; }
int grns_ctx_log2(const grns_ctx *c) { return c ? c->log2M : 0; }

grns_status grns_ctx_get_table(const grns_ctx *c, int which, void *dst, size_t bytes) {
    if (!c || !dst) return GRNS_ERR_INVALID_ARGUMENT;
    static_assert(sizeof(interval_t) == 2 * sizeof(grns::Er), "interval_t is two er_float_t");
    const std::vector<uint8_t> t = grns::table_bytes(c->T, which);
    if (t.empty() || bytes != t.size()) return GRNS_ERR_INVALID_ARGUMENT;
    std::memcpy(dst, t.data(), t.size());
    return GRNS_OK;
}

grns_status grns_ctx_set_eval_split(grns_ctx *c, int fp64_eighths) {
    if (!c || fp64_eighths < 0 || fp64_eighths > 8) return GRNS_ERR_INVALID_ARGUMENT;
    c->eval_fp64_eighths = fp64_eighths;
    return GRNS_OK;
}

int grns_ctx_get_eval_split(const grns_ctx *c) { return c ? c->eval_fp64_eighths : -1; }

grns_status grns_ctx_set_path(grns_ctx *c, int path) {
    if (!c || (path != GRNS_PATH_FAST && path != GRNS_PATH_REFERENCE)) return GRNS_ERR_INVALID_ARGUMENT;
    c->path = path;
    return GRNS_OK;
}

grns_status grns_device_ceil_log2(const double *x, int32_t *out, int64_t count, void *stream) {
    if (!x || !out || count < 0) return GRNS_ERR_INVALID_ARGUMENT;
    if (count == 0) return GRNS_OK;
    int64_t blocks = (count + 255) / 256;
    k_ceil_log2<<<(unsigned)(blocks < 1024 ? blocks : 1024), 256, 0, (cudaStream_t)stream>>>(x, out, count);
    return grns::cuda_status(cudaGetLastError());
}

}  // extern "C"
