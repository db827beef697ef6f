// C ABI (include/ccsd_gb300.h): status codes, thread-local error text, and the
// handle that owns one Engine.  No C++ exception crosses this boundary.
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "engine.h"

struct ccsd_handle {
    ccsd::Engine *engine = nullptr;
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

int ccsd_last_error(char *buf, size_t len) {
    const int n = (int)g_last_error.size();
    if (buf && len > 0) {
        size_t c = std::min(len - 1, g_last_error.size());
        std::memcpy(buf, g_last_error.data(), c);
        buf[c] = '\0';
    }
    return n;
}

double ccsd_flops_per_update(int32_t nocc, int32_t nvir) {
    const double o = nocc, v = nvir;
    return 2.0 * o * o * v * v * v * v + 4.0 * o * o * o * o * v * v + 8.0 * o * o * o * v * v * v;
}

}  // extern "C"
