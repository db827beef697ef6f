// Driver that applies the reference's memory-optimised CCSD update
// (CCSD_Memory_optimized, ccsd_memory_optimized.cpp compiled unchanged) to
// amplitudes chosen by the caller (TEST INFRASTRUCTURE ONLY).
//
// The class keeps its whole state in public members, so the update can be
// driven from outside: CCSD(huge tolerance) performs the set-up (integral
// transform Prepear_AOs, work maps, MP2 start) and one pass (:513-557); then
// T_1 and t2 are overwritten with the caller's amplitudes and the loop body of
// :513-537 is run again, member call by member call:
//   Fill_tau, Fill_F1, Fill_W1_and_W3, Distribute_Part1, Fill_F2, Fill_F3,
//   Fill_W4_MPI, Fill_W4, Fill_W5, Fill_t2_new, Map_T_new, T_1 = T_1_new / DEN_AI.
// The result is the reference's Jacobi map T -> T_new evaluated at any T.
//
// Storage of the class (spin orbitals interleaved: p -> spatial p/2, spin p%2,
// virtual indices counted from 0):
//   T_1(a/2 + (a%2)*Speed_Occ, i/2)        = t1[a][i]       for (a+i) even
//   t2(a,i)(b/2 + (b%2)*Speed_Occ, j/2)    = t2[a][b][i][j] for (a+i+b+j) even
//
//   usage: ref_probe <input.bin> <amps_in.bin> <amps_out.bin>
//   input.bin:    as ref_synthetic (int32 n, int32 nocc, float64 eps[n], float64 eri[n^4])
//   amps_in.bin:  int32 O, int32 V, float64 t1[V][O], float64 t2[V][V][O][O]
//   amps_out.bin: the same layout after one update, then float64 E_corr of the
//                 updated amplitudes (Fill_tau + Calc_Energy), then the Fock
//                 intermediates of the update, D1, D2, D3, each as int32 rows,
//                 int32 cols and float64 data in the class's (column-major) order
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "ccsd_memory_optimized.h"

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
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s input.bin amps_in.bin amps_out.bin\n", argv[0]);
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

    FILE *fa = std::fopen(argv[2], "rb");
    if (!fa) return 7;
    int dims[2];
    if (std::fread(dims, sizeof(int), 2, fa) != 2) return 8;
    const int O = dims[0], V = dims[1];
    if (O != 2 * g_nocc || V != 2 * (g_n - g_nocc)) return 9;
    std::vector<double> t1((size_t)V * O), t2((size_t)V * V * O * O);
    if (std::fread(t1.data(), sizeof(double), t1.size(), fa) != t1.size()) return 10;
    if (std::fread(t2.data(), sizeof(double), t2.size(), fa) != t2.size()) return 11;
    std::fclose(fa);

    MPI_Init(&argc, &argv);
    vec Z = zeros(1);
    mat R = zeros(1, 3);
    Hartree_Fock_Solver hf(1, Z, R, "synthetic", 2 * g_nocc, false, 0, 1, false);
    CCSD_Memory_optimized cc(1, Z, R, "synthetic", 2 * g_nocc, 0, 1, &hf, false);
    cc.CCSD(1e300, false);  // set-up and one pass; the tolerance stops the loop after it

    const int so = cc.Speed_Occ;
    auto T2 = [&](int a, int b, int i, int j) -> double & {
        return t2[(((size_t)a * V + b) * O + i) * O + j];
    };
    for (int a = 0; a < V; ++a)
        for (int i = 0; i < O; ++i)
            if ((a + i) % 2 == 0) cc.T_1(a / 2 + (a % 2) * so, i / 2) = t1[(size_t)a * O + i];
    for (int a = 0; a < V; ++a)
        for (int i = 0; i < O; ++i)
            for (int b = 0; b < V; ++b)
                for (int j = 0; j < O; ++j)
                    if ((a + i + b + j) % 2 == 0) cc.t2(a, i)(b / 2 + (b % 2) * so, j / 2) = T2(a, b, i, j);

    // the loop body of CCSD_Memory_optimized::CCSD (:517-537), after the Fill_tau that ends a pass (:536)
    cc.Fill_tau();
    cc.Fill_F1();
    cc.Fill_W1_and_W3();
    cc.Distribute_Part1();
    cc.Fill_F2();
    cc.Fill_F3();
    cc.Fill_W4_MPI();
    cc.Fill_W4();
    cc.Fill_W5();
    cc.Fill_t2_new();
    cc.Map_T_new();
    cc.T_1 = cc.T_1_new / cc.DEN_AI;
    cc.Fill_tau();
    const double e = cc.Calc_Energy();

    std::fill(t1.begin(), t1.end(), 0.0);
    std::fill(t2.begin(), t2.end(), 0.0);
    for (int a = 0; a < V; ++a)
        for (int i = 0; i < O; ++i)
            if ((a + i) % 2 == 0) t1[(size_t)a * O + i] = cc.T_1(a / 2 + (a % 2) * so, i / 2);
    for (int a = 0; a < V; ++a)
        for (int i = 0; i < O; ++i)
            for (int b = 0; b < V; ++b)
                for (int j = 0; j < O; ++j)
                    if ((a + i + b + j) % 2 == 0) T2(a, b, i, j) = cc.t2(a, i)(b / 2 + (b % 2) * so, j / 2);

    FILE *fo = std::fopen(argv[3], "wb");
    if (!fo) return 12;
    std::fwrite(dims, sizeof(int), 2, fo);
    std::fwrite(t1.data(), sizeof(double), t1.size(), fo);
    std::fwrite(t2.data(), sizeof(double), t2.size(), fo);
    std::fwrite(&e, sizeof(double), 1, fo);
    for (const mat *m : {&cc.D1, &cc.D2, &cc.D3}) {
        const int rc[2] = {(int)m->n_rows, (int)m->n_cols};
        std::fwrite(rc, sizeof(int), 2, fo);
        std::fwrite(m->memptr(), sizeof(double), m->n_elem, fo);
    }
    std::fclose(fo);
    MPI_Finalize();
    return 0;
}
