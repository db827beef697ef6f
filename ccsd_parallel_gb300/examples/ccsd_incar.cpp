// The reference's program entry (main.cpp: read INCAR, Initializer::Go) on the
// engine: reads an INCAR file and a Gaussian94 basis file and prints the energy.
//
//   g++ -std=c++17 -O2 -I include ccsd_parallel_gb300/examples/ccsd_incar.cpp \
//       -L ccsd_parallel_gb300/_lib -lccsd_gb300 -Wl,-rpath,<that directory> -o ccsd_incar
//   ./ccsd_incar INCAR [basis.g94] [split3]     (no basis file: the INCAR's Basis_File line)
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>

#include "ccsd_gb300.h"

static bool slurp(const char *path, std::string &out) {
    std::ifstream f(path);
    if (!f) return false;
    std::stringstream ss;
    ss << f.rdbuf();
    out = ss.str();
    return true;
}

int main(int argc, char **argv) {
    if (argc < 2) {
        std::fprintf(stderr, "usage: %s INCAR [basis.g94] [fp64|split2|split3|split4]\n", argv[0]);
        return 2;
    }
    int prec = CCSD_PREC_FP64, nargs = argc;
    const char *last = argv[argc - 1];
    if (argc > 2 && std::strncmp(last, "split", 5) == 0) {
        prec = std::strcmp(last, "split2") == 0 ? CCSD_PREC_SPLIT2
               : std::strcmp(last, "split4") == 0 ? CCSD_PREC_SPLIT4 : CCSD_PREC_SPLIT3;
        --nargs;
    } else if (argc > 2 && std::strcmp(last, "fp64") == 0) {
        --nargs;
    }
    std::string incar, basis;
    if (!slurp(argv[1], incar) || (nargs > 2 && !slurp(argv[2], basis))) {
        std::fprintf(stderr, "cannot read the INCAR or the basis file\n");
        return 2;
    }
    ccsd_incar_result r{};
    const int rc = ccsd_incar_run(incar.c_str(), basis.c_str(), prec, &r);
    if (rc != CCSD_OK) {
        char msg[1024];
        ccsd_last_error(msg, sizeof msg);
        std::fprintf(stderr, "error %d: %s\n", rc, msg);
        return 1;
    }
    std::printf("E_HF = %.12f  SCF steps %d\n", r.e_hf, r.scf_iterations);
    if (r.method >= 0) std::printf("E_corr = %.12f  iter %d\n", r.e_corr, r.cc_iter);
    std::printf("Energy = %.12f\n", r.energy);
    return 0;
}
