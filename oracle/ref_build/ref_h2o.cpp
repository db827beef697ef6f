// Driver that runs the reference's RHF (hartree_fock_solver.cpp) and its CCSD
// (ccsd_memory_optimized.cpp), both compiled unchanged, on H2O and dumps the
// SCF outputs the CCSD consumed (TEST INFRASTRUCTURE ONLY).
//
//   usage: ref_h2o <basis> <geometry: config|incar> <log10 tolerance> <dump.bin>
//   geometry "config": O (0,0,0), H (+-1.4305, 1.1071, 0) bohr
//   geometry "incar":  the reference's INCAR~ sample (O 0 0 0; H 0 1.079252 1.474611;
//                      H 0 1.079252 -1.47611 bohr)
//   prints: "iter <reference iter> ecorr <E_corr> ehf <E_HF> etotal <E>"
//   dump:   int32 nao, int32 nocc, float64 C[nao][nao] (C[mu][p]), float64 eps[nao],
//           float64 ao_eri[nao^4] ((mu nu|la si), row-major), float64 E_HF
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "ccsd_memory_optimized.h"
#include "ccsdt.h"

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s basis config|incar log10_tol dump.bin\n", argv[0]);
        return 2;
    }
    const std::string basis = argv[1], geom = argv[2];
    const double toler = std::pow(10.0, std::atof(argv[3]));
    MPI_Init(&argc, &argv);
    vec Z = zeros(3);
    Z(0) = 8;
    Z(1) = 1;
    Z(2) = 1;
    mat R = zeros(3, 3);
    if (geom == "incar") {
        R(1, 1) = 1.079252;
        R(1, 2) = 1.474611;
        R(2, 1) = 1.079252;
        R(2, 2) = -1.47611;
    } else if (geom.rfind("yz:", 0) == 0) {  // yz:<y>,<z>  -> H (0, y, +-z)
        double y = 0, z = 0;
        std::sscanf(geom.c_str() + 3, "%lf,%lf", &y, &z);
        R(1, 1) = y;
        R(1, 2) = z;
        R(2, 1) = y;
        R(2, 2) = -z;
    } else {
        R(1, 0) = 1.4305;
        R(1, 1) = 1.1071;
        R(2, 0) = -1.4305;
        R(2, 1) = 1.1071;
    }
    const int n_elec = 10;
    Hartree_Fock_Solver hf(3, Z, R, basis, n_elec, false, 0, 1, false);
    CCSD_Memory_optimized cc(3, Z, R, basis, n_elec, 0, 1, &hf, false);
    const double e = cc.CCSD(toler, false);
    const double ehf = e - cc.E_new;
    std::printf("iter %d ecorr %.17e ehf %.17e etotal %.17e\n", cc.iter, cc.E_new, ehf, e);
    if (argc > 5 && (std::string(argv[5]) == "ccsd1" || std::string(argv[5]).rfind("ccsdt-", 0) == 0)) {
        // the reference's dense spin-orbital CCSD ("ccsd1", method -1) or CCSDT-n ("ccsdt-<n>")
        // on the same RHF (its SCF reruns to the same result)
        const std::string m = argv[5];
        const int method = m == "ccsd1" ? -1 : std::atoi(m.c_str() + 6);
        Hartree_Fock_Solver hf1(3, Z, R, basis, n_elec, false, 0, 1, false);
        CCSDT c1(3, Z, R, basis, n_elec, 0, 1, &hf1, false);
        const double e1 = c1.Calc_Energy(toler, method);
        std::printf("ccsd1_iter %d ccsd1_ecorr %.17e\n", c1.iter, e1 - ehf);
    }

    // SCF outputs that Prepear_AOs consumed: C, orbital energies, (pq|rs)
    const int n = hf.Matrix_Size;
    FILE *f = std::fopen(argv[4], "wb");
    if (!f) return 3;
    int hdr[2] = {n, n_elec / 2};
    std::fwrite(hdr, sizeof(int), 2, f);
    std::vector<double> buf((size_t)n * n);
    for (int mu = 0; mu < n; ++mu)
        for (int p = 0; p < n; ++p) buf[(size_t)mu * n + p] = hf.C(mu, p);
    std::fwrite(buf.data(), sizeof(double), buf.size(), f);
    std::vector<double> eps(n);
    for (int p = 0; p < n; ++p) eps[p] = hf.eigenvalues_F(p);
    std::fwrite(eps.data(), sizeof(double), n, f);
    std::vector<double> eri((size_t)n * n * n * n);
    for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) {
            mat m = hf.Return_Field_Q(p >= q ? p : q, p >= q ? q : p);  // (pq|rs), q <= p stored
            for (int r = 0; r < n; ++r)
                for (int s = 0; s < n; ++s) eri[(((size_t)p * n + q) * n + r) * n + s] = m(r, s);
        }
    std::fwrite(eri.data(), sizeof(double), eri.size(), f);
    std::fwrite(&ehf, sizeof(double), 1, f);
    std::fclose(f);
    MPI_Finalize();
    return 0;
}
