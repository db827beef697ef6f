// Driver that runs the reference's own CCSD (ccsd_memory_optimized.cpp,
// compiled unchanged) on a synthetic system (TEST INFRASTRUCTURE ONLY).
//
// The reference CCSD takes its inputs from a Hartree_Fock_Solver object
// (ccsd_memory_optimized.cpp:49-74): get_Energy, ReturnMatrixSize, ReturnC,
// return_eigval_F and Return_Field_Q(j, l), the (jl|rs) slice of the AO
// integrals for l <= j (hartree_fock_solver.cpp:1044-1210 leaves field_Q in
// that layout).  This file defines those members of the reference's
// (unchanged) class declaration for a system given directly in the MO basis:
// E_HF = 0, C = identity, orbital energies and chemist (pq|rs) read from a
// binary file, so Prepear_AOs passes the integrals through unchanged.
//
//   usage: ref_synthetic <input.bin> <log10 tolerance> [mo|ccsd1|ccsdt-<n>]
//     mo         CCSD_Memory_optimized::CCSD (the reference's "CCSD" method)
//     mo-print   the same with its own per-iteration output ("Energi: ... Time/iter: ...")
//     ccsd1      CCSDT::Calc_Energy(toler, -1), the dense spin-orbital CCSD ("CCSD1")
//     ccsdt-<n>  CCSDT::Calc_Energy(toler, n): 1 = CCSDT-1a, 2 = CCSDT-1b, 3 = CCSDT-2,
//                4 = CCSDT-3, 5 = CCSDT-4, 6 = CCSDT (initializer.cpp:98-128)
//   input: int32 n, int32 nocc, float64 eps[n], float64 eri[n^4] (p,q,r,s row-major)
//   prints: "iter <reference iter> ecorr <E_corr %.17e>"
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ccsd_memory_optimized.h"
#include "ccsdt.h"

namespace {
int g_n = 0, g_nocc = 0;
std::vector<double> g_eps, g_eri;
}  // namespace

Hartree_Fock_Solver::Hartree_Fock_Solver(int n_N, vec zz, mat rr, string B_s, int n_elec, bool pstf, int ran,
                                         int siz, bool frezcor) {
    n_Nuclei = n_N;
    Z = zz;
    R = rr;
    Basis_Set = B_s;
    n_Electrons = n_elec;
    print_stuff = pstf;
    rank = ran;
    size = siz;
    Freeze_Core = frezcor;
}

double Hartree_Fock_Solver::get_Energy(double, int) {
    Matrix_Size = g_n;
    C = zeros(g_n, g_n);
    for (int i = 0; i < g_n; ++i) C(i, i) = 1.0;
    eigenvalues_F = zeros(g_n);
    for (int i = 0; i < g_n; ++i) eigenvalues_F(i) = g_eps[i];
    return 0.0;
}

// unrestricted-reference accessors CCSDT references for Method_Nr == 7 only
mat Hartree_Fock_Solver::return_C_up() { return C; }
mat Hartree_Fock_Solver::return_C_down() { return C; }
void Hartree_Fock_Solver::Set_UP_DOWN(int, int) {}

int Hartree_Fock_Solver::ReturnMatrixSize() { return Matrix_Size; }
mat Hartree_Fock_Solver::ReturnC() { return C; }
mat Hartree_Fock_Solver::return_eigval_F() { return eigenvalues_F; }

mat Hartree_Fock_Solver::Return_Field_Q(int i, int j) {
    const size_t n = g_n;
    mat q = zeros(g_n, g_n);
    for (size_t r = 0; r < n; ++r)
        for (size_t s = 0; s < n; ++s) q(r, s) = g_eri[((i * n + j) * n + r) * n + s];
    return q;
}

int main(int argc, char **argv) {
    if (argc < 3) {
        std::fprintf(stderr, "usage: %s input.bin log10_tolerance\n", argv[0]);
        return 2;
    }
    FILE *f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    int hdr[2];
    if (std::fread(hdr, sizeof(int), 2, f) != 2) return 4;
    g_n = hdr[0];
    g_nocc = hdr[1];
    const size_t n = g_n;
    g_eps.resize(n);
    g_eri.resize(n * n * n * n);
    if (std::fread(g_eps.data(), sizeof(double), n, f) != n) return 5;
    if (std::fread(g_eri.data(), sizeof(double), g_eri.size(), f) != g_eri.size()) return 6;
    std::fclose(f);
    const double toler = std::pow(10.0, std::atof(argv[2]));

    MPI_Init(&argc, &argv);
    vec Z = zeros(1);
    mat R = zeros(1, 3);
    Hartree_Fock_Solver hf(1, Z, R, "synthetic", 2 * g_nocc, false, 0, 1, false);
    if (argc > 3 && (std::strcmp(argv[3], "ccsd1") == 0 || std::strncmp(argv[3], "ccsdt-", 6) == 0)) {
        const int method = std::strcmp(argv[3], "ccsd1") == 0 ? -1 : std::atoi(argv[3] + 6);
        CCSDT cc(1, Z, R, "synthetic", 2 * g_nocc, 0, 1, &hf, false);
        const double e = cc.Calc_Energy(toler, method);
        std::printf("iter %d ecorr %.17e etotal %.17e\n", cc.iter, e, e);
    } else {
        CCSD_Memory_optimized cc(1, Z, R, "synthetic", 2 * g_nocc, 0, 1, &hf, false);
        // "mo-print": the class prints its own per-iteration time (clock(), ccsd_memory_optimized.cpp:515-548)
        const bool print = argc > 3 && std::strcmp(argv[3], "mo-print") == 0;
        const double e = cc.CCSD(toler, print);
        std::printf("iter %d ecorr %.17e etotal %.17e\n", cc.iter, cc.E_new, e);
        if (argc > 4) {  // dump the final amplitudes in the class's compact layout
            FILE *o = std::fopen(argv[4], "wb");
            const int O = cc.n_Electrons, V = cc.unocc_orb;
            int hdr[2] = {O, V};
            std::fwrite(hdr, sizeof(int), 2, o);
            std::fwrite(cc.T_1.memptr(), sizeof(double), cc.T_1.n_elem, o);  // (V x O/2), column-major
            for (int a = 0; a < V; ++a)
                for (int i = 0; i < O; ++i) {
                    const mat &m = cc.t2(a, i);  // (V x O/2), column-major
                    std::fwrite(m.memptr(), sizeof(double), m.n_elem, o);
                }
            std::fclose(o);
        }
    }
    MPI_Finalize();
    return 0;
}
