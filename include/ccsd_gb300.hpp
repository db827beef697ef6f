// ccsd_gb300.hpp -- header-only C++ drop-in over the C ABI (ccsd_gb300.h).
//
// ccsd_gb300::CCSD_Memory_optimized mirrors the reference class of the same
// name (ccsd_memory_optimized.h:15-47) for its iterative part:
//
//   reference                                    here
//   -------------------------------------------------------------------------
//   CCSD_Memory_optimized(n_N, Z, R, basis,      CCSD_Memory_optimized(Problem, E_HF)
//     n_Elec, rank, size, HartFock*, frozen)      -- the inputs Prepear_AOs and
//                                                    Fill_FS produce are passed in;
//                                                    frozen = true is Problem.nfrozen =
//                                                    ccsd_frozen_core_count(Z, n_N)
//   n_Electrons (less 2 nr_freeze, .cpp:3520)    n_Electrons = 2 Problem.nocc (active)
//   double CCSD(double toler, bool print_stuff)  double CCSD(double toler, bool print_stuff)
//     returns E_HF + E_corr                        returns E_HF + E_corr
//   E_new, iter                                  E_new, iter (counter starts at 1)
//   T_1 (compact, V x o), t2 (compact field)     t1 [i][a], t2 [i][j][a][b] (spatial)
//
// As in the reference, CCSD() iterates plain Jacobi updates from the MP2
// guess until |E_new - E_old| < toler or iter reaches 1000.  By default it
// iterates the reference class's own map (CCSD_VARIANT_MEMORY_OPTIMIZED: F_mi
// contracted transposed in T2, ccsd_memory_optimized.cpp:2085-2086), so the
// energies and counters are the class's; CCSD_VARIANT_CCSD gives the CCSD
// equations of the reference's dense CCSD1.  Failures are
// reported with ccsd_gb300::Error (status code + message); the reference
// prints and keeps going instead.
#ifndef CCSD_GB300_HPP
#define CCSD_GB300_HPP

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "ccsd_gb300.h"

namespace ccsd_gb300 {

struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};

inline void check(int rc) {
    if (rc != CCSD_OK) {
        char buf[1024];
        ccsd_last_error(buf, sizeof buf);
        throw Error(rc, std::string("ccsd_gb300: ") + buf);
    }
}

class CCSD_Memory_optimized {
  public:
    // `problem` pointers must stay valid for the constructor only: the
    // integrals are copied to the device here.
    explicit CCSD_Memory_optimized(const ccsd_problem &problem, double E_HF = 0.0,
                                   int precision = CCSD_PREC_FP64,
                                   int variant = CCSD_VARIANT_MEMORY_OPTIMIZED)
        : E_HF_(E_HF), nocc_(problem.nocc), nvir_(problem.nvir) {
        ccsd_default_options(&opts_);
        opts_.precision = precision;
        opts_.variant = variant;
        check(ccsd_create(&problem, &opts_, &h_));
        n_Electrons = 2 * nocc_;
        unocc_orb = 2 * nvir_;
    }
    ~CCSD_Memory_optimized() {
        if (h_) ccsd_destroy(h_);
    }
    CCSD_Memory_optimized(const CCSD_Memory_optimized &) = delete;
    CCSD_Memory_optimized &operator=(const CCSD_Memory_optimized &) = delete;

    double CCSD(double toler, bool print_stuff) {
        opts_.energy_tol = toler;
        opts_.max_iter = 999;
        opts_.verbose = print_stuff ? 1 : 0;
        check(ccsd_set_options(h_, &opts_));
        const size_t o = nocc_, v = nvir_;
        t1.assign(o * v, 0.0);
        t2.assign(o * o * v * v, 0.0);
        energies.assign(1001, 0.0);
        ccsd_result r{};
        r.t1 = t1.data();
        r.t2 = t2.data();
        r.energy_history = energies.data();
        r.history_capacity = (int)energies.size();
        check(ccsd_solve(h_, &r));
        energies.resize(r.history_len);
        E_new = r.e_corr;
        iter = r.iterations + 1;
        if (print_stuff) std::printf("CCSD correction [au] = %.15e\n", E_new);
        return E_new + E_HF_;
    }

    ccsd_handle *handle() { return h_; }

    int n_Electrons = 0, unocc_orb = 0, iter = 1;
    double E_new = 0.0;
    std::vector<double> t1, t2, energies;

  private:
    ccsd_handle *h_ = nullptr;
    ccsd_options opts_{};
    double E_HF_;
    int nocc_, nvir_;
};

}  // namespace ccsd_gb300

#endif  // CCSD_GB300_HPP
