// Minimal C++ host program using the drop-in class: builds a seeded synthetic
// closed-shell system with the library generator and runs the reference's
// stopping rule (|dE| < toler) on the GPU engine.
//
//   g++ -std=c++17 -I<repo>/include dropin_synthetic.cpp \
//       -L<repo>/ccsd_parallel_gb300/_lib -lccsd_gb300 -Wl,-rpath,<repo>/ccsd_parallel_gb300/_lib
//   ./a.out <nocc> <nvir> <naux> <seed> <log10 tol> [fp64|split3]
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ccsd_gb300.hpp"

int main(int argc, char **argv) {
    const int o = argc > 1 ? std::atoi(argv[1]) : 4, v = argc > 2 ? std::atoi(argv[2]) : 12;
    const int naux = argc > 3 ? std::atoi(argv[3]) : 30;
    const unsigned long long seed = argc > 4 ? std::strtoull(argv[4], nullptr, 10) : 7;
    const double toler = std::pow(10.0, argc > 5 ? std::atof(argv[5]) : -10.0);
    const int prec = (argc > 6 && std::strcmp(argv[6], "split3") == 0) ? CCSD_PREC_SPLIT3 : CCSD_PREC_FP64;
    const int n = o + v;
    std::vector<double> fock((size_t)n * n), df((size_t)naux * n * n);
    ccsd_gb300::check(ccsd_make_synthetic(o, v, naux, seed, fock.data(), df.data()));
    ccsd_problem p{};
    p.nocc = o;
    p.nvir = v;
    p.integral_kind = CCSD_INTS_DF;
    p.naux = naux;
    p.fock = fock.data();
    p.df = df.data();
    try {
        ccsd_gb300::CCSD_Memory_optimized cc(p, /*E_HF=*/0.0, prec);
        const double e = cc.CCSD(toler, false);
        std::printf("iter %d ecorr %.17e etotal %.17e\n", cc.iter, cc.E_new, e);
    } catch (const ccsd_gb300::Error &err) {
        std::fprintf(stderr, "%s (code %d)\n", err.what(), err.code);
        return 1;
    }
    return 0;
}
