// Closed-shell Hartree-Fock (the reference's Hartree_Fock_Solver::get_Energy with
// do_uhf = 0, hartree_fock_solver.cpp:578-1229): the producer of the CCSD inputs.
//
// The integrals come from the GPU engine (ao_integrals) and stay on the device;
// each iteration's two O(n^4) contractions run there as matrix-vector products
// over views of the ERI tensor:
//   J[i][j] = sum_kl (ij|kl) P[l][k],   K[i][j] = sum_kl (il|kj) P[l][k]
//   F = h + J - K / 2                   (Make_Fock_Matrix, :490-569)
// The n x n algebra stays on the host in FP64, step for step as the reference:
//   - canonical orthogonalisation X = U diag(lambda^-1/2) from S (:686-690);
//   - P = 0 at the start, so the first F is h;
//   - DIIS over the last 3 Fock matrices with error F P S - S P F, from the second
//     Fock matrix on, extrapolating once 4 have been seen (DIIS, :1252-1311);
//   - eigenpairs of X^T F X ascending, C = X W, each column scaled to
//     c^T S c = 1 (Normalize, :1230-1245), P = 2 C_occ C_occ^T (Calc_Density);
//   - stop when |sum of occupied eps - previous sum| < tol or after 300 steps;
//   - E_HF = sum h*P + 1/2 sum F_prev*P - 1/2 sum h*P + E_nuc (Calc_Energy,
//     :482-488), F_prev the Fock matrix before DIIS and before the last step.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/ccsd_gb300.h"
#include "common.h"

namespace ccsd {
void set_last_error(const std::string &msg);

namespace {

using Mat = std::vector<double>;  // row-major n x n

// Eigenpairs of a symmetric matrix by cyclic Jacobi rotations (the rotation that
// zeroes a[p][q], applied to rows/columns p, q and accumulated into V), sorted
// ascending; V holds the eigenvectors as columns.
void jacobi_eigh(int n, Mat a, std::vector<double> &w, Mat &V) {
    V.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) V[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double & { return a[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += A(i, i) * A(i, i);
            for (int j = i + 1; j < n; ++j) off += A(i, j) * A(i, j);
        }
        if (off <= 1e-34 * std::max(diag, 1e-300)) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (apq == 0.0) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[(size_t)k * n + p], vkq = V[(size_t)k * n + q];
                    V[(size_t)k * n + p] = c * vkp - s * vkq;
                    V[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    std::vector<int> ord(n);
    for (int i = 0; i < n; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
    w.resize(n);
    Mat Vs((size_t)n * n);
    for (int c = 0; c < n; ++c) {
        w[c] = A(ord[c], ord[c]);
        for (int r = 0; r < n; ++r) Vs[(size_t)r * n + c] = V[(size_t)r * n + ord[c]];
    }
    V.swap(Vs);
}

// solve A x = b (m x m) by Gaussian elimination with partial pivoting
std::vector<double> solve_small(int m, Mat A, std::vector<double> b) {
    for (int c = 0; c < m; ++c) {
        int piv = c;
        for (int r = c + 1; r < m; ++r)
            if (std::fabs(A[(size_t)r * m + c]) > std::fabs(A[(size_t)piv * m + c])) piv = r;
        if (A[(size_t)piv * m + c] == 0.0) throw Error(CCSD_ERR_DIVERGED, "RHF: singular DIIS system");
        if (piv != c) {
            for (int k = 0; k < m; ++k) std::swap(A[(size_t)c * m + k], A[(size_t)piv * m + k]);
            std::swap(b[c], b[piv]);
        }
        for (int r = c + 1; r < m; ++r) {
            const double f = A[(size_t)r * m + c] / A[(size_t)c * m + c];
            for (int k = c; k < m; ++k) A[(size_t)r * m + k] -= f * A[(size_t)c * m + k];
            b[r] -= f * b[c];
        }
    }
    std::vector<double> x(m);
    for (int r = m - 1; r >= 0; --r) {
        double s = b[r];
        for (int k = r + 1; k < m; ++k) s -= A[(size_t)r * m + k] * x[k];
        x[r] = s / A[(size_t)r * m + r];
    }
    return x;
}

struct Dev {
    double *p = nullptr;
    ~Dev() {
        if (p) cudaFree(p);
    }
    void alloc(size_t n) { CCSD_CUDA(cudaMalloc(&p, sizeof(double) * std::max<size_t>(n, 1))); }
};

// What both SCF forms share: S, h = T + V and X = U diag(lambda^-1/2) on the host,
// the ERI tensor on the device, and the device contractions
//   G = aj J(Pj) + ak K(Pk),  J[i][j] = sum_kl (ij|kl) P[k][l],  K[i][j] = sum_kl (il|kj) P[l][k]
struct ScfSystem {
    int n;
    size_t nn;
    Mat S, h, X;
    double e_nuc = 0.0;
    Dev eri, P_d, G_d, ws;
    size_t ws_n = 1;
    cudaStream_t st;
    mutable Dev mA, mB, mC;  // operands of the n x n products on the device

    ScfSystem(const ccsd_basis &bs, cudaStream_t s) : n(bs.nbf), nn((size_t)bs.nbf * bs.nbf), st(s) {
        S.resize(nn);
        Mat T(nn), Vn(nn);
        eri.alloc(nn * nn);
        ao_integrals(bs, S.data(), T.data(), Vn.data(), nullptr, &e_nuc, false, st);
        ao_integrals(bs, nullptr, nullptr, nullptr, eri.p, nullptr, true, st);
        h.resize(nn);
        for (size_t k = 0; k < nn; ++k) h[k] = T[k] + Vn[k];
        P_d.alloc(2 * nn);
        G_d.alloc(nn);
        mA.alloc(nn);
        mB.alloc(nn);
        mC.alloc(nn);
        ws_n = std::max(gemm_f64_ws_elems((int)nn, 1, (int)nn), (size_t)1);
        ws.alloc(ws_n);
        std::vector<double> lam;
        Mat U;
        jacobi_eigh(n, S, lam, U);
        X.resize(nn);
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) X[(size_t)i * n + j] = U[(size_t)i * n + j] / std::sqrt(lam[j]);
    }

    void two_electron(const Mat &Pj, double aj, const Mat &Pk, double ak, Mat &G) {
        const int M = (int)nn;
        const int64_t N = n, N2 = N * N, N3 = N2 * N;
        CCSD_CUDA(cudaMemcpyAsync(P_d.p, Pj.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
        CCSD_CUDA(cudaMemcpyAsync(P_d.p + nn, Pk.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
        const OutView Gv{G_d.p, ix1(1), ix1(0)};
        gemm_f64(M, 1, M, aj, MatView{eri.p, ix1(N2), ix1(1)}, MatView{P_d.p, ix1(0), ix1(1)}, 0.0, Gv, ws.p,
                 ws_n, st);
        gemm_f64(M, 1, M, ak, MatView{eri.p, ix2((uint32_t)n, N3, 1), ix2((uint32_t)n, N2, N)},
                 MatView{P_d.p + nn, ix1(0), ix1(1)}, 1.0, Gv, ws.p, ws_n, st);
        G.resize(nn);
        CCSD_CUDA(cudaMemcpyAsync(G.data(), G_d.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
        CCSD_CUDA(cudaStreamSynchronize(st));
    }

    // op(a) b for n x n host matrices (op(a) = a^T with ta), k columns of op(a) (rows of b) summed,
    // as an FP64 contraction on the device: a product costs tens of microseconds there against
    // milliseconds of host loops at n = 150
    Mat dmm(const Mat &a, const Mat &b, bool ta = false, int k = -1) const {
        if (k < 0) k = n;
        CCSD_CUDA(cudaMemcpyAsync(mA.p, a.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
        CCSD_CUDA(cudaMemcpyAsync(mB.p, b.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, st));
        // C(i, j) = sum_l A(i, l) B(j, l) with A(i, l) = op(a)[i][l], B(j, l) = b[l][j]
        const MatView Av{mA.p, ta ? ix1(1) : ix1(n), ta ? ix1(n) : ix1(1)};
        const MatView Bv{mB.p, ix1(1), ix1(n)};
        gemm_f64(n, n, k, 1.0, Av, Bv, 0.0, OutView{mC.p, ix1(n), ix1(1)}, ws.p, ws_n, st);
        Mat c(nn);
        CCSD_CUDA(cudaMemcpyAsync(c.data(), mC.p, sizeof(double) * nn, cudaMemcpyDeviceToHost, st));
        CCSD_CUDA(cudaStreamSynchronize(st));
        return c;
    }

    // eigenpairs of X^T F X ascending, C = X W with every column at c^T S c = 1 (Normalize).
    // warm: the previous step's W of this spin; X^T F X is rotated into it first, where it
    // is nearly diagonal, so the Jacobi sweeps start close to the answer (then warm = W)
    void orbitals(const Mat &F, std::vector<double> &eps, Mat &C, Mat &warm) const {
        const Mat Fo = dmm(X, dmm(F, X), true);
        Mat W;
        if (warm.size() == nn) {
            Mat V;
            jacobi_eigh(n, dmm(warm, dmm(Fo, warm), true), eps, V);
            W = dmm(warm, V);
        } else {
            jacobi_eigh(n, Fo, eps, W);
        }
        warm = W;
        C = dmm(X, W);
        const Mat SC = dmm(S, C);  // c^T S c = sum_i C[i][c] (S C)[i][c]
        for (int c = 0; c < n; ++c) {
            double s = 0.0;
            for (int i = 0; i < n; ++i) s += C[(size_t)i * n + c] * SC[(size_t)i * n + c];
            const double f = 1.0 / std::sqrt(s);
            for (int i = 0; i < n; ++i) C[(size_t)i * n + c] *= f;
        }
    }

    // P = w C_occ C_occ^T over the first k columns
    Mat density(const Mat &C, int k, double w) const {
        Mat Ct(nn);  // C^T, so that the product sums over its first k rows
        for (int i = 0; i < n; ++i)
            for (int c = 0; c < n; ++c) Ct[(size_t)c * n + i] = C[(size_t)i * n + c];
        Mat P = dmm(C, Ct, false, k);
        for (double &x : P) x *= w;
        return P;
    }
};

void rhf(const ccsd_basis &bs, int nelec, double tol, int max_iter, ccsd_scf_result &res, cudaStream_t st) {
    const int n = bs.nbf;
    if (nelec <= 0 || nelec % 2 || nelec / 2 > n)
        throw Error(CCSD_ERR_INVALID_ARG, "RHF: n_electrons must be even, positive and at most 2 nbf");
    const int nocc = nelec / 2;
    const size_t nn = (size_t)n * n;
    ScfSystem sys(bs, st);
    const Mat &S = sys.S, &h = sys.h;
    const double e_nuc = sys.e_nuc;

    Mat P(nn, 0.0), F(nn), Fprev(nn), C(nn), warm;
    std::vector<double> eps;
    std::vector<Mat> errs, focks;
    const int ndiis = 3;
    double hf_new = 0.0, hf_old = 0.0;
    int step = 0;
    const int limit = max_iter > 0 ? max_iter : 300;
    bool converged = false;
    while (true) {
        hf_old = hf_new;
        // F = h + J - K/2 on the device
        sys.two_electron(P, 1.0, P, -0.5, F);
        for (size_t k = 0; k < nn; ++k) F[k] += h[k];
        Fprev = F;
        // DIIS (the reference's, with 3 vectors)
        if (step > 0) {
            Mat e = sys.dmm(sys.dmm(F, P), S);
            const Mat SPF = sys.dmm(S, sys.dmm(P, F));
            for (size_t k = 0; k < nn; ++k) e[k] -= SPF[k];
            errs.push_back(e);
            focks.push_back(F);
            if (step > ndiis) {
                errs.erase(errs.begin());
                focks.erase(focks.begin());
                Mat B((size_t)(ndiis + 1) * (ndiis + 1), 0.0);
                for (int i = 0; i < ndiis; ++i) {
                    for (int j = 0; j < ndiis; ++j) {
                        double tr = 0.0;
                        for (size_t k = 0; k < nn; ++k) tr += errs[i][k] * errs[j][k];
                        B[(size_t)i * (ndiis + 1) + j] = tr;
                    }
                    B[(size_t)i * (ndiis + 1) + ndiis] = B[(size_t)ndiis * (ndiis + 1) + i] = -1.0;
                }
                std::vector<double> z(ndiis + 1, 0.0);
                z[ndiis] = -1.0;
                const std::vector<double> c = solve_small(ndiis + 1, B, z);
                for (size_t k = 0; k < nn; ++k) {
                    double f = 0.0;
                    for (int i = 0; i < ndiis; ++i) f += c[i] * focks[i][k];
                    F[k] = f;
                }
            }
        }
        sys.orbitals(F, eps, C, warm);
        P = sys.density(C, nocc, 2.0);
        hf_new = 0.0;
        for (int i = 0; i < nocc; ++i) hf_new += eps[i];
        ++step;
        if (!std::isfinite(hf_new)) throw Error(CCSD_ERR_DIVERGED, "RHF diverged (NaN/Inf)");
        if (std::fabs(hf_new - hf_old) < tol) {
            converged = true;
            break;
        }
        if (step > limit) break;
    }
    double e1 = 0.0, e2 = 0.0;
    for (size_t k = 0; k < nn; ++k) {
        e1 += h[k] * P[k];
        e2 += Fprev[k] * P[k];
    }
    res.e_hf = e1 + 0.5 * e2 - 0.5 * e1 + e_nuc;
    res.e_nuc = e_nuc;
    res.iterations = step;
    res.converged = converged ? 1 : 0;
    if (res.eps) std::memcpy(res.eps, eps.data(), sizeof(double) * n);
    if (res.C) std::memcpy(res.C, C.data(), sizeof(double) * nn);
    if (res.eri) CCSD_CUDA(cudaMemcpy(res.eri, sys.eri.p, sizeof(double) * nn * nn, cudaMemcpyDeviceToHost));
}

// Unrestricted Hartree-Fock, step for step as get_Energy(toler, 1) (hartree_fock_solver.cpp:
// 959-1025, Unrestricted_Fock_Matrix :1359-1503, Unrestricted_P_Matrix :1505-1529,
// Unrestricted_Energy :1531-1537): F_up = h + J(P_up + P_down) - K(P_up), F_down likewise;
// no DIIS; stop when |eps_up[0] - previous| + |eps_down[0] - previous| < tol or after 300
// steps.  The reference starts from Armadillo's randn densities (Initialize_UHF); this
// starts from normal deviates of a seeded generator (symmetrised), so a run is repeatable.
void uhf(const ccsd_basis &bs, int n_up, int n_down, double tol, int max_iter, ccsd_uhf_result &res,
         cudaStream_t st) {
    const int n = bs.nbf;
    if (n_up < 0 || n_down < 0 || n_up + n_down == 0 || n_up > n || n_down > n)
        throw Error(CCSD_ERR_INVALID_ARG, "UHF: electron counts must be >= 0, not both 0, at most nbf each");
    const size_t nn = (size_t)n * n;
    ScfSystem sys(bs, st);
    // seeded normal deviates (xorshift64* and Box-Muller)
    uint64_t state = res.seed ? res.seed : 2024;
    auto uniform = [&]() {
        state ^= state >> 12;
        state ^= state << 25;
        state ^= state >> 27;
        return ((state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() {
        const double u1 = std::max(uniform(), 1e-300), u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * M_PI * u2);
    };
    Mat Pu(nn), Pd(nn);
    for (Mat *P : {&Pu, &Pd}) {
        for (size_t k = 0; k < nn; ++k) (*P)[k] = normal();
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < i; ++j) {
                const double m = 0.5 * ((*P)[(size_t)i * n + j] + (*P)[(size_t)j * n + i]);
                (*P)[(size_t)i * n + j] = (*P)[(size_t)j * n + i] = m;
            }
    }
    Mat Pt(nn), Fu, Fd, Cu, Cd, warm_u, warm_d;
    std::vector<double> eu, ed;
    double eu_old = 0.0, ed_old = 0.0;
    int step = 0;
    const int limit = max_iter > 0 ? max_iter : 300;
    bool converged = false;
    while (true) {
        for (size_t k = 0; k < nn; ++k) Pt[k] = Pu[k] + Pd[k];
        sys.two_electron(Pt, 1.0, Pu, -1.0, Fu);
        sys.two_electron(Pt, 1.0, Pd, -1.0, Fd);
        for (size_t k = 0; k < nn; ++k) {
            Fu[k] += sys.h[k];
            Fd[k] += sys.h[k];
        }
        sys.orbitals(Fu, eu, Cu, warm_u);
        sys.orbitals(Fd, ed, Cd, warm_d);
        Pu = sys.density(Cu, n_up, 1.0);
        Pd = sys.density(Cd, n_down, 1.0);
        const double check = std::fabs(eu[0] - eu_old) + std::fabs(ed[0] - ed_old);
        eu_old = eu[0];
        ed_old = ed[0];
        ++step;
        if (!std::isfinite(check)) throw Error(CCSD_ERR_DIVERGED, "UHF diverged (NaN/Inf)");
        if (check < tol) {
            converged = true;
            break;
        }
        if (step > limit) break;
    }
    double e1 = 0.0, e2 = 0.0;
    for (size_t k = 0; k < nn; ++k) {
        e1 += (Pu[k] + Pd[k]) * sys.h[k];
        e2 += Fu[k] * Pu[k] + Fd[k] * Pd[k];
    }
    res.e_uhf = e1 + 0.5 * e2 - 0.5 * e1 + sys.e_nuc;
    res.e_nuc = sys.e_nuc;
    res.iterations = step;
    res.converged = converged ? 1 : 0;
    if (res.eps_up) std::memcpy(res.eps_up, eu.data(), sizeof(double) * n);
    if (res.eps_down) std::memcpy(res.eps_down, ed.data(), sizeof(double) * n);
    if (res.C_up) std::memcpy(res.C_up, Cu.data(), sizeof(double) * nn);
    if (res.C_down) std::memcpy(res.C_down, Cd.data(), sizeof(double) * nn);
}

}  // namespace
}  // namespace ccsd

extern "C" int ccsd_rhf(const ccsd_basis *basis, int32_t n_electrons, double tol, int32_t max_iter,
                        ccsd_scf_result *res) {
    try {
        ccsd::set_last_error("");
        if (!basis || !res) throw ccsd::Error(CCSD_ERR_INVALID_ARG, "ccsd_rhf: basis or result is NULL");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw ccsd::Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
        }
        cudaStream_t st = (cudaStream_t)res->stream;
        ccsd::rhf(*basis, n_electrons, tol > 0.0 ? tol : 1e-10, max_iter, *res, st);
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        ccsd::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        ccsd::set_last_error(e.what());
        return CCSD_ERR_CUDA;
    }
}

extern "C" int ccsd_uhf(const ccsd_basis *basis, int32_t n_up, int32_t n_down, double tol, int32_t max_iter,
                        ccsd_uhf_result *res) {
    try {
        ccsd::set_last_error("");
        if (!basis || !res) throw ccsd::Error(CCSD_ERR_INVALID_ARG, "ccsd_uhf: basis or result is NULL");
        int ndev = 0;
        if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
            cudaGetLastError();
            throw ccsd::Error(CCSD_ERR_NO_DEVICE, "no CUDA device: this engine has no CPU path");
        }
        ccsd::uhf(*basis, n_up, n_down, tol > 0.0 ? tol : 1e-10, max_iter, *res, (cudaStream_t)res->stream);
        return CCSD_OK;
    } catch (const ccsd::Error &e) {
        ccsd::set_last_error(e.what());
        return e.code;
    } catch (const std::exception &e) {
        ccsd::set_last_error(e.what());
        return CCSD_ERR_CUDA;
    }
}
