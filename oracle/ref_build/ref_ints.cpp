// Driver that runs the reference's RHF (hartree_fock_solver.cpp and
// hartree_integrals.cpp, compiled unchanged) on a molecule and dumps the basis
// description its integral engine received (Hartree_Integrals::Set_Input,
// hartree_integrals.cpp:8-21) with the integrals and the SCF result
// (TEST INFRASTRUCTURE ONLY).
//
//   usage: ref_ints <basis> <atoms "Z,x,y,z;Z,x,y,z;..." (bohr)> <n_electrons> <log10 tol> <dump.bin>
//          [uhf <n_up> <n_down>]   (then only "uhf <E_UHF> <steps>" is printed, nothing dumped)
//   dump (native endian):
//     int32 natoms, nbf, maxprim, nelec
//     float64 Z[natoms], R[natoms][3]
//     int32 atom_of_bf[nbf], nprim[nbf], powers[nbf][3]
//     float64 alpha[nbf][maxprim], c[nbf][maxprim]      (c after Normalize_small_c)
//     float64 S[nbf][nbf]                               (Overlap_Matrix)
//     float64 T[nbf][nbf]                               (Kinetic_Energy, as returned)
//     float64 Vne[nbf][nbf]                             (Nuclei_Electron_Interaction, as returned)
//     float64 eri[nbf^4]                                ((mu nu|la si), row-major)
//     float64 E_nuc, E_HF, eps[nbf], C[nbf][nbf]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "fill_alpha.h"
#include "fill_alpha2.h"
#include "hartree_fock_solver.h"
#include "matrix_size_setter.h"

int main(int argc, char **argv) {
    if (argc < 6) {
        std::fprintf(stderr, "usage: %s basis atoms n_electrons log10_tol dump.bin\n", argv[0]);
        return 2;
    }
    const std::string basis = argv[1], spec = argv[2];
    const int n_elec = std::atoi(argv[3]);
    const double toler = std::pow(10.0, std::atof(argv[4]));
    std::vector<double> zs, xyz;
    for (size_t pos = 0; pos < spec.size();) {
        size_t end = spec.find(';', pos);
        if (end == std::string::npos) end = spec.size();
        double z, x, y, w;
        if (std::sscanf(spec.substr(pos, end - pos).c_str(), "%lf,%lf,%lf,%lf", &z, &x, &y, &w) != 4) return 2;
        zs.push_back(z);
        xyz.insert(xyz.end(), {x, y, w});
        pos = end + 1;
    }
    const int na = (int)zs.size();
    MPI_Init(&argc, &argv);
    vec Z = zeros(na);
    mat R = zeros(na, 3);
    for (int a = 0; a < na; ++a) {
        Z(a) = zs[a];
        for (int d = 0; d < 3; ++d) R(a, d) = xyz[3 * a + d];
    }
    if (argc > 8 && std::string(argv[6]) == "uhf") {
        Hartree_Fock_Solver uhf(na, Z, R, basis, n_elec, false, 0, 1, false);
        uhf.Set_UP_DOWN(std::atoi(argv[7]), std::atoi(argv[8]));
        const double e = uhf.get_Energy(toler, 1);
        std::printf("uhf %.17e %d\n", e, uhf.steppp);
        MPI_Finalize();
        return 0;
    }
    Hartree_Fock_Solver hf(na, Z, R, basis, n_elec, false, 0, 1, false);
    const double ehf = hf.get_Energy(toler, 0);
    const int n = hf.Matrix_Size;
    // get_Energy clears its basis arrays and integral engine when it is done; a second
    // solver gets the same basis through get_Energy's own steps (Fill_Alpha /
    // fill_alpha2, Normalize_small_c) and a fresh engine its set-up (Set_Input,
    // Fill_E_ij, Set_Boys_Start)
    Hartree_Fock_Solver bs(na, Z, R, basis, n_elec, false, 0, 1, false);
    matrix_size_setter matset(Z, basis, na);
    if (matset.Set_Matrix_Size() != n) return 4;
    if (basis == "aug-cc-pVQZ" || basis == "aug-cc-pVTZ" || basis == "aug-cc-pVDZ") {
        fill_alpha2 fy(na, Z, basis, n, matset.Return_Max_Bas_Func());
        bs.alpha = fy.Fyll_Opp_Alpha();
        bs.c = fy.Fyll_Opp_c();
        bs.n_Basis = fy.Fyll_Opp_Nr_Basis_Functions();
        bs.Number_Of_Orbitals = fy.Fyll_Opp_Antall_Orbitaler();
        bs.Potenser = fy.Fyll_Opp_Potenser();
    } else {
        Fill_Alpha fy(na, Z, basis, n, matset.Return_Max_Bas_Func());
        bs.alpha = fy.Fyll_Opp_Alpha();
        bs.c = fy.Fyll_Opp_c();
        bs.n_Basis = fy.Fyll_Opp_Nr_Basis_Functions();
        bs.Number_Of_Orbitals = fy.Fyll_Opp_Antall_Orbitaler();
        bs.Potenser = fy.Fyll_Opp_Potenser();
    }
    bs.Normalize_small_c();
    int maxprim = 0;
    for (int i = 0; i < n; ++i) maxprim = std::max(maxprim, (int)bs.n_Basis(i));
    std::printf("nbf %d maxprim %d ehf %.17e\n", n, maxprim, ehf);
    std::fflush(stdout);
    Hartree_Integrals hi;
    hi.Set_Input(bs.alpha, n, bs.c, bs.Number_Of_Orbitals, bs.Potenser, bs.n_Basis, na, R, Z, n_elec);
    hi.Fill_E_ij();
    hi.Set_Boys_Start((max(max(bs.Potenser)) + 1) * 4);

    FILE *f = std::fopen(argv[5], "wb");
    if (!f) return 3;
    auto wi = [&](const std::vector<int> &v) { std::fwrite(v.data(), sizeof(int), v.size(), f); };
    auto wd = [&](const std::vector<double> &v) { std::fwrite(v.data(), sizeof(double), v.size(), f); };
    wi({na, n, maxprim, n_elec});
    wd(zs);
    wd(xyz);
    std::vector<int> atom(n), nprim(n), pw(3 * n);
    for (int a = 0, i = 0; a < na; ++a)
        for (int k = 0; k < (int)bs.Number_Of_Orbitals(a); ++k, ++i) atom[i] = a;
    std::vector<double> al((size_t)n * maxprim, 0.0), cc((size_t)n * maxprim, 0.0);
    for (int i = 0; i < n; ++i) {
        nprim[i] = (int)bs.n_Basis(i);
        for (int d = 0; d < 3; ++d) pw[3 * i + d] = (int)bs.Potenser(i, d);
        for (int k = 0; k < nprim[i]; ++k) {
            al[(size_t)i * maxprim + k] = bs.alpha(i, k);
            cc[(size_t)i * maxprim + k] = bs.c(i, k);
        }
    }
    wi(atom);
    wi(nprim);
    wi(pw);
    wd(al);
    wd(cc);
    auto wm = [&](const mat &m) {
        std::vector<double> b((size_t)n * n);
        for (int p = 0; p < n; ++p)
            for (int q = 0; q < n; ++q) b[(size_t)p * n + q] = m(p, q);
        wd(b);
    };
    wm(hi.Overlap_Matrix());
    wm(hi.Kinetic_Energy());
    wm(hi.Nuclei_Electron_Interaction());
    std::vector<double> eri((size_t)n * n * n * n);
    for (int p = 0; p < n; ++p)
        for (int q = 0; q < n; ++q) {
            mat m = hf.Return_Field_Q(p >= q ? p : q, p >= q ? q : p);  // (pq|rs), q <= p stored
            for (int r = 0; r < n; ++r)
                for (int s = 0; s < n; ++s) eri[(((size_t)p * n + q) * n + r) * n + s] = m(r, s);
        }
    wd(eri);
    std::vector<double> tail = {hf.Nuclei_Rep_Energy, ehf};
    for (int p = 0; p < n; ++p) tail.push_back(hf.eigenvalues_F(p));
    wd(tail);
    wm(hf.C);
    std::fclose(f);
    MPI_Finalize();
    return 0;
}
