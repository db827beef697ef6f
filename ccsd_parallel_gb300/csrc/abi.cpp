// C ABI (include/ccsd_gb300.h): status codes, thread-local error text, and the
// handle that owns one Engine.  No C++ exception crosses this boundary.
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "batched.h"
#include "engine.h"

struct ccsd_handle {
    ccsd::Engine *engine = nullptr;
};

struct ccsd_batch {
    ccsd::Batch *batch = nullptr;
};

namespace {
thread_local std::string g_last_error;

int fail(int code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

template <class F>
int guarded(F &&f) {
    try {
        g_last_error.clear();
        f();
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        return fail(e.code, e.what());
    } catch (const std::bad_alloc &) {
        return fail(CCSD_ERR_OUT_OF_MEMORY, "host allocation failed");
    } catch (const std::exception &e) {
        return fail(CCSD_ERR_CUDA, e.what());
    } catch (...) {
        return fail(CCSD_ERR_CUDA, "unknown error");
    }
}
}  // namespace

namespace ccsd {
// Lets entry points defined in other files report through ccsd_last_error.
void set_last_error(const std::string &msg) { g_last_error = msg; }
}  // namespace ccsd

extern "C" {

int ccsd_default_options(ccsd_options *opts) {
    if (!opts) return fail(CCSD_ERR_INVALID_ARG, "opts is NULL");
    std::memset(opts, 0, sizeof(*opts));
    opts->energy_tol = 1e-10;
    opts->residual_tol = 0.0;
    opts->max_iter = 999;  // reference: iter starts at 1 and stops at 1000
    opts->fixed_iterations = 0;
    opts->diis_size = 0;
    opts->diis_start = 0;
    opts->precision = CCSD_PREC_FP64;
    opts->verbose = 0;
    opts->stream = nullptr;
    return CCSD_OK;
}

int ccsd_create(const ccsd_problem *problem, const ccsd_options *opts, ccsd_handle **out) {
    if (!problem || !out) return fail(CCSD_ERR_INVALID_ARG, "problem/out is NULL");
    *out = nullptr;
    ccsd_options o;
    if (opts)
        o = *opts;
    else
        ccsd_default_options(&o);
    return guarded([&] {
        ccsd::Engine *e = new ccsd::Engine(*problem, o);
        ccsd_handle *h = new (std::nothrow) ccsd_handle;
        if (!h) {
            delete e;
            throw std::bad_alloc();
        }
        h->engine = e;
        *out = h;
    });
}

int ccsd_solve(ccsd_handle *h, ccsd_result *res) {
    if (!h || !h->engine || !res) return fail(CCSD_ERR_INVALID_ARG, "handle/result is NULL");
    return guarded([&] { h->engine->solve(res); });
}

int ccsd_lambda_grad(ccsd_handle *h, const ccsd_problem *problem, ccsd_grad *grad) {
    if (!h || !h->engine || !problem || !grad) return fail(CCSD_ERR_INVALID_ARG, "handle/problem/grad is NULL");
    return guarded([&] { h->engine->lambda_grad(*problem, grad); });
}

int ccsd_set_options(ccsd_handle *h, const ccsd_options *opts) {
    if (!h || !h->engine || !opts) return fail(CCSD_ERR_INVALID_ARG, "handle/opts is NULL");
    return guarded([&] { h->engine->set_options(*opts); });
}

int ccsd_destroy(ccsd_handle *h) {
    if (!h) return CCSD_OK;
    int rc = guarded([&] { delete h->engine; });
    delete h;
    return rc;
}

int ccsd_batch_create(const ccsd_problem *const *problems, int32_t n, const ccsd_options *opts, ccsd_batch **out) {
    if (!problems || !out || n <= 0) return fail(CCSD_ERR_INVALID_ARG, "problems/out is NULL or n <= 0");
    *out = nullptr;
    ccsd_options o;
    if (opts)
        o = *opts;
    else
        ccsd_default_options(&o);
    return guarded([&] {
        ccsd::Batch *b = new ccsd::Batch(problems, n, o);
        ccsd_batch *h = new (std::nothrow) ccsd_batch;
        if (!h) {
            delete b;
            throw std::bad_alloc();
        }
        h->batch = b;
        *out = h;
    });
}

int ccsd_batch_solve(ccsd_batch *b, ccsd_result *results) {
    if (!b || !b->batch || !results) return fail(CCSD_ERR_INVALID_ARG, "batch/results is NULL");
    return guarded([&] { b->batch->solve(results); });
}

int ccsd_batch_report(ccsd_batch *b, char *buf, size_t len) {
    if (!b || !b->batch) return fail(CCSD_ERR_INVALID_ARG, "batch is NULL");
    std::string s;
    int rc = guarded([&] { s = b->batch->report(); });
    if (rc != CCSD_OK) return rc;
    if (buf && len > 0) {
        size_t c = std::min(len - 1, s.size());
        std::memcpy(buf, s.data(), c);
        buf[c] = '\0';
    }
    return (int)s.size();
}

int ccsd_batch_destroy(ccsd_batch *b) {
    if (!b) return CCSD_OK;
    int rc = guarded([&] { delete b->batch; });
    delete b;
    return rc;
}

int ccsd_solve_batched(const ccsd_problem *const *problems, int32_t n, const ccsd_options *opts,
                       ccsd_result *results) {
    if (!results) return fail(CCSD_ERR_INVALID_ARG, "results is NULL");
    ccsd_batch *b = nullptr;
    int rc = ccsd_batch_create(problems, n, opts, &b);
    if (rc != CCSD_OK) return rc;
    rc = ccsd_batch_solve(b, results);
    std::string keep = g_last_error;
    ccsd_batch_destroy(b);
    g_last_error = keep;
    return rc;
}

int ccsd_profile_report(ccsd_handle *h, char *buf, size_t len) {
    if (!h || !h->engine) return fail(CCSD_ERR_INVALID_ARG, "handle is NULL");
    std::string s;
    int rc = guarded([&] { s = h->engine->profile_json(); });
    if (rc != CCSD_OK) return rc;
    if (buf && len > 0) {
        size_t c = std::min(len - 1, s.size());
        std::memcpy(buf, s.data(), c);
        buf[c] = '\0';
    }
    return (int)s.size();
}

int ccsd_last_error(char *buf, size_t len) {
    const int n = (int)g_last_error.size();
    if (buf && len > 0) {
        size_t c = std::min(len - 1, g_last_error.size());
        std::memcpy(buf, g_last_error.data(), c);
        buf[c] = '\0';
    }
    return n;
}

int ccsd_gemm(int32_t precision, int32_t M, int32_t N, int32_t K, double alpha, const double *A, int64_t lda,
              const double *B, int64_t ldb, double beta, double *C, int64_t ldc, void *stream) {
    if (M < 0 || N < 0 || K < 0 || !A || !B || !C || lda < K || ldb < K || ldc < N)
        return fail(CCSD_ERR_INVALID_ARG, "ccsd_gemm: bad shape, leading dimension or NULL pointer");
    if (precision != CCSD_PREC_FP64 && precision != CCSD_PREC_SPLIT2 && precision != CCSD_PREC_SPLIT3 &&
        precision != CCSD_PREC_SPLIT4)
        return fail(CCSD_ERR_INVALID_ARG, "ccsd_gemm: unknown precision");
    return guarded([&] {
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw ccsd::Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
        }
        cudaStream_t st = (cudaStream_t)stream;
        ccsd::MatView a, b;
        a.p = A;
        a.row.s2 = lda;
        a.col.s2 = 1;
        b.p = B;
        b.row.s2 = ldb;
        b.col.s2 = 1;
        ccsd::OutView c;
        c.p = C;
        c.row.s2 = ldc;
        c.col.s2 = 1;
        if (M == 0 || N == 0) return;
        if (K == 0) {  // C = beta C, nothing to contract (alpha is not applied, as in BLAS)
            if (beta != 1.0) {
                ccsd::MatView cv;
                cv.p = C;
                cv.row = c.row;
                cv.col = c.col;
                ccsd::axpby_view(M, N, 0.0, cv, beta, c, st);
                CCSD_CUDA(cudaStreamSynchronize(st));
            }
            return;
        }
        if (precision == CCSD_PREC_FP64) {
            size_t ws_n = ccsd::gemm_f64_ws_elems(M, N, K);
            double *ws = nullptr;
            if (ws_n) CCSD_CUDA(cudaMalloc(&ws, ws_n * sizeof(double)));
            try {
                ccsd::gemm_f64(M, N, K, alpha, a, b, beta, c, ws, ws_n, st);
                CCSD_CUDA(cudaStreamSynchronize(st));
            } catch (...) {
                if (ws) cudaFree(ws);
                throw;
            }
            if (ws) cudaFree(ws);
        } else {
            ccsd::split_gemm_oneshot(precision, M, N, K, alpha, a, b, beta, c, st);
        }
    });
}

double ccsd_flops_per_update(int32_t nocc, int32_t nvir) {
    const double o = nocc, v = nvir;
    return 2.0 * o * o * v * v * v * v + 4.0 * o * o * o * o * v * v + 8.0 * o * o * o * v * v * v;
}

int ccsd_frozen_core_count(const double *Z, int32_t n_atoms) {
    if (n_atoms < 0 || (n_atoms > 0 && !Z)) return fail(CCSD_ERR_INVALID_ARG, "ccsd_frozen_core_count: n_atoms < 0 or Z is NULL");
    g_last_error.clear();
    int count = 0;
    for (int32_t a = 0; a < n_atoms; ++a)
        if (Z[a] > 2.0 && Z[a] < 11.0) ++count;
    return count;
}

}  // extern "C"
